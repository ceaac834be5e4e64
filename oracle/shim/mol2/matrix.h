/* Test-infrastructure shim: libmol2's 3x3 matrix (src/saxs_utils.c:65-94). */
#ifndef SXS_SHIM_MOL2_MATRIX_H
#define SXS_SHIM_MOL2_MATRIX_H
struct mol_matrix3 { double m11, m12, m13, m21, m22, m23, m31, m32, m33; };
#endif
