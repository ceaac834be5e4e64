/*
 * Compatibility header with the reference's name (src/sfbessel.h):
 * sxs_sbessel is declared in fmftsaxs_gb300.h.
 */
#ifndef FMFTSAXS_GB300_COMPAT_SFBESSEL_H
#define FMFTSAXS_GB300_COMPAT_SFBESSEL_H
#include "common.h"
#include "fmftsaxs_gb300.h"
#endif
