/*
 * Test stand-in for the parts of libmol2 that a correlate-style caller uses
 * besides the types of oracle/shim/mol2 (libmol2 itself is not available
 * here).  TEST INFRASTRUCTURE: implemented by tests/c/mol2_stub.c.
 */
#ifndef SXS_TEST_MOL2_PDB_H
#define SXS_TEST_MOL2_PDB_H
#include "mol2/atom_group.h"
#include "mol2/vector.h"

/* ATOM/HETATM records: atom name in columns 13-16 and residue name in
 * 18-21 kept as written (blanks included), then x, y, z as the three numbers
 * after column 30 (the test writes them at full precision) */
struct mol_atom_group *mol_read_pdb(const char *path);
void mol_atom_group_free(struct mol_atom_group *ag);
void centroid(struct mol_vector3 *center, const struct mol_atom_group *ag);
void center_of_extrema(struct mol_vector3 *center, const struct mol_atom_group *ag);
void mol_atom_group_translate(struct mol_atom_group *ag, const struct mol_vector3 *v);
#endif
