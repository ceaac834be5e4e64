/*
 * Test stand-in for libmol2's parameter files (see pdb.h).  Reads the
 * "atom <id> <residue> <atom> <type> <radius> ..." records of a parameter
 * file and sets each atom's van der Waals radius from its (residue, atom).
 */
#ifndef SXS_TEST_MOL2_PRMS_H
#define SXS_TEST_MOL2_PRMS_H
#include <stdbool.h>
#include "mol2/atom_group.h"

struct mol_prms;
struct mol_prms *mol_prms_read(const char *path);
void mol_prms_free(struct mol_prms *prms);
bool mol_atom_group_add_prms(struct mol_atom_group *ag, const struct mol_prms *prms);
#endif
