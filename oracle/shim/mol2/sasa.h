/* Test-infrastructure shim: libmol2 accs() (src/saxs_utils.c:38).  The checker
 * harness supplies per-atom accessible areas instead of computing them. */
#ifndef SXS_SHIM_MOL2_SASA_H
#define SXS_SHIM_MOL2_SASA_H
#include "atom_group.h"
void accs(double *as, const struct mol_atom_group *ag, double r_solv, short cont_acc);
#endif
