/* Test-infrastructure shim: libmol2 matrix list (src/index.c:95-96). */
#ifndef SXS_SHIM_MOL2_LISTS_H
#define SXS_SHIM_MOL2_LISTS_H
#include <stddef.h>
#include "matrix.h"
struct mol_matrix3_list { size_t size; struct mol_matrix3 *members; };
struct mol_matrix3_list *mol_matrix3_list_from_file(const char *path);
#endif
