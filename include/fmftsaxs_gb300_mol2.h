/*
 * fmftsaxs-gb300: the reference's entry points whose arguments are libmol2
 * types (struct mol_atom_group, struct mol_matrix3_list).
 *
 * They are defined in libfmftsaxs_gb300/mol2/sxs_mol2.c, a small C file that
 * the caller compiles against its own libmol2 headers and links with
 * libmol2 and libfmftsaxs_gb300.so: the product library itself never sees a
 * libmol2 struct.  That file reads the atom group (coordinates, residue and
 * atom names, van der Waals radii), resolves form factors and accessible
 * areas the way the reference does (libmol2's own accs for the areas) and
 * hands flat arrays to the GPU expansion of fmftsaxs_gb300.h.
 *
 * Include this header where the reference's pdb2spf.h, form_factor_table.h,
 * saxs_utils.h or index.h were included; libmol2's include directory must
 * be on the include path, as it is for the reference.
 */
#ifndef FMFTSAXS_GB300_MOL2_H
#define FMFTSAXS_GB300_MOL2_H

#include <stdbool.h>
#include <stddef.h>

#include "mol2/atom_group.h"
#include "mol2/lists.h"
#include "mol2/matrix.h"
#include "mol2/sasa.h"
#include "mol2/vector.h"

#define SXS_HAVE_MOL2_TYPES
#include "fmftsaxs_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/form_factor_table.h:27-37: form-factor types (the index into
 * saxs_form_factor_table::factors). */
enum saxs_ff_type {
	H, He,
	Li, Be, B, C, N, O, F, Ne,
	Na, Mg, Al, Si, P, S, Cl, Ar,
	K, Ca, Cr, Mn, Fe, Co, Ni, Cu, Zn, Se, Br,
	Io, Ir, Pt, Au, Hg, SINGLE_ATOM_SIZE = 34,
	CH = 34, CH2 = 35, CH3 = 36, NH = 37, NH2 = 38, NH3 = 39, OH = 40, s_OH2 = 41, SH = 42, PO4 = 43,
	HEAVY_ATOM_SIZE = 43, s_UNK = 99
};

/* src/form_factor_table.h:40-56 */
struct saxs_form_factor_coeffs {
	double a[5];
	double b[5];
	double c;
	double excl_vol;
	bool valid;
};

struct saxs_form_factor {
	double zero_ff;
	double vacuum_ff;
	double dummy_ff;
	double *values;
};

/* src/form_factor_table.h:58-67.  Same layout; type_map holds this
 * library's (residue, atom) -> type map (sxsg_ff_map) where the reference
 * keeps a khash table.  The q-dependent coefficients are never filled: the
 * scoring path uses the zero-angle factors only. */
struct saxs_form_factor_table {
	struct saxs_form_factor factors[HEAVY_ATOM_SIZE];
	struct saxs_form_factor_coeffs coeffs[HEAVY_ATOM_SIZE];
	void *type_map;
	struct saxs_form_factor *water_ff;
};

/* src/form_factor_table.h:70.  Table of the default zero-angle form
 * factors with the (residue, atom) mapping read from type_mapping_file.
 * Like the reference, the first table built is returned by every later
 * call, whatever its path; a file that cannot be opened ends the process. */
struct saxs_form_factor_table *default_ff_table(const char *type_mapping_file);
/* src/form_factor_table.h:72.  Frees a table from default_ff_table (the
 * next default_ff_table call then builds a new one). */
void ff_table_destroy(struct saxs_form_factor_table *table);
/* src/form_factor_table.h:74 */
const char *ff_type_to_string(enum saxs_ff_type type);
/* src/form_factor_table.h:76-77.  Form factors of one atom; NULL (with the
 * reference's message) when its (residue, atom) pair has no mapping or
 * maps to an unknown type. */
const struct saxs_form_factor *get_ff(const struct saxs_form_factor_table *table,
                                      const struct mol_atom_group *ag, size_t atom_index);
/* src/form_factor_table.h:79-82 */
double dummy_ff(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag, size_t atom_index);
double vacuum_ff(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag, size_t atom_index);
/* src/form_factor_table.h:86-87 (declared there with the misspelt return
 * type enum sax_ff_type, i.e. an int) */
enum saxs_ff_type atom2ff_type(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag,
                               size_t atom_index);
/* src/form_factor_table.h:89-94: per-atom factors of a whole group */
void get_dummy_ff(double *dummy_ffs, const struct mol_atom_group *ag, const struct saxs_form_factor_table *table);
void get_vacuum_ff(double *vacuum_ffs, const struct mol_atom_group *ag, const struct saxs_form_factor_table *table);

/* src/pdb2spf.h:66-72.  A_lm(q) of one molecule, computed on the GPU
 * (sxsg_expand).  water = 1 adds the hydration shell with accessible
 * fractions from sxs_faccs (probe 1.4 A); the caller frees the result with
 * sxs_spf_full_free.  An atom without form factors ends the process. */
struct sxs_spf_full *atom_grp2spf(struct mol_atom_group *ag, struct saxs_form_factor_table *ff_table,
                                  double *qvals, int qnum, int L, int water);
/* src/pdb2spf.h:84-91.  Same into a caller-allocated spf_coefs (L, qnum as
 * created); saxs_sa: accessible fraction per atom, NULL for no shell. */
void atom_grp2spf_inplace(struct sxs_spf_full *spf_coefs, struct mol_atom_group *ag,
                          struct saxs_form_factor_table *ff_table, double *qvals, int qnum, int L,
                          double *saxs_sa);

/* src/saxs_utils.h:18-20 */
double mol_atom_group_max_dist(const struct mol_atom_group *ag);
double mol_atom_group_average_radius(const struct mol_atom_group *ag);
/* src/saxs_utils.h:47-52.  Accessible fraction per atom from libmol2's
 * accs (contact surface, probe r_solv) divided by 4 pi r^2; 0 for a zero
 * radius or a NaN area. */
void sxs_faccs(double *fractional_sa, const struct mol_atom_group *ag, double r_solv);

/* src/index.h:68.  Converts an FT file (id, translation, six more numbers
 * per line) with its rotation-matrix file (read by libmol2's
 * mol_matrix3_list_from_file) to the Euler file that correlate reads back:
 * "id z b1 g1 a2 b2 g2" in "% .3f". */
void sxs_ft_file2euler_file(const char *eu_path, const char *ft_path, const char *rm_path,
                            struct mol_vector3 *ref_lig);

#ifdef __cplusplus
}
#endif
#endif
