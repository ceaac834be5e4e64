/* Test-infrastructure shim: libmol2 transform header (no symbols used on the path). */
#ifndef SXS_SHIM_MOL2_TRANSFORM_H
#define SXS_SHIM_MOL2_TRANSFORM_H
#include "atom_group.h"
#include "matrix.h"
#include "vector.h"
#endif
