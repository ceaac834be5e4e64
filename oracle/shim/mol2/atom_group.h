/* Test-infrastructure shim: the fields of libmol2's mol_atom_group that the
 * reference reads (src/pdb2spf.c:36-66, src/saxs_utils.c:19-48,
 * src/form_factor_table.c:95-121) plus two libmol2 utilities it calls. */
#ifndef SXS_SHIM_MOL2_ATOM_GROUP_H
#define SXS_SHIM_MOL2_ATOM_GROUP_H
#include <stdbool.h>
#include <stddef.h>
#include "vector.h"
struct mol_atom_group {
	size_t natoms;
	struct mol_vector3 *coords;
	char **atom_name;
	char **residue_name;
	double *vdw_radius;
};
bool is_whitespace_line(const char *line);
void free_if_not_null(void *p);
#endif
