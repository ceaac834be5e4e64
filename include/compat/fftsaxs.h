/*
 * Compatibility header with the reference's name (src/fftsaxs.h): its
 * declarations come from fmftsaxs_gb300_mol2.h (which includes libmol2's
 * headers and fmftsaxs_gb300.h), so that callers written against
 * libfmftsaxs compile unchanged against fmftsaxs-gb300.
 */
#ifndef FMFTSAXS_GB300_COMPAT_FFTSAXS_H
#define FMFTSAXS_GB300_COMPAT_FFTSAXS_H
#include "common.h"
#include "fmftsaxs_gb300_mol2.h"
#endif
