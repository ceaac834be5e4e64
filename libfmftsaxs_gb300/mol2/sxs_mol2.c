/*
 * The reference's libmol2-typed entry points (include/fmftsaxs_gb300_mol2.h)
 * over the flat C API of libfmftsaxs_gb300.so.
 *
 * Compile this file with the caller's libmol2 headers and link it with
 * libmol2 and libfmftsaxs_gb300.so:
 *     cc -std=c11 -c sxs_mol2.c -I<libmol2 include> -I<fmftsaxs-gb300 include>
 * It is the only code that reads libmol2 structs (struct mol_atom_group:
 * natoms, coords, residue_name, atom_name, vdw_radius) and the only caller of
 * libmol2 functions (accs, mol_matrix3_list_from_file); the expansion itself
 * runs on the GPU through sxsg_expand.
 *
 * Errors follow the reference's convention: a message and exit(EXIT_FAILURE).
 */
#define _XOPEN_SOURCE 700
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fmftsaxs_gb300_mol2.h"

/* the reference's pi under -std=c11 (src/define.h:14-16) */
#define SXS_MOL2_PI 3.14159265358

static void die(const char *func, const char *msg)
{
	fprintf(stderr, "[Error] fmftsaxs-gb300, function %s: %s\n", func, msg);
	exit(EXIT_FAILURE);
}

/* ------------------------------------------------------ form factors */

static struct saxs_form_factor_table *g_default_table = NULL;

struct saxs_form_factor_table *default_ff_table(const char *type_mapping_file)
{
	if (g_default_table) return g_default_table;
	sxsg_ff_map *map = sxsg_ff_map_load(type_mapping_file);
	if (!map) {
		fprintf(stderr, "%s\n", sxsg_last_error());
		exit(1);
	}
	struct saxs_form_factor_table *t = calloc(1, sizeof(*t));
	if (!t) die("default_ff_table", "out of memory");
	t->type_map = map;
	for (int i = 0; i < HEAVY_ATOM_SIZE; i++)
		sxsg_ff_constants(i, &t->factors[i].zero_ff, &t->factors[i].vacuum_ff, &t->factors[i].dummy_ff);
	g_default_table = t;
	return t;
}

void ff_table_destroy(struct saxs_form_factor_table *table)
{
	if (!table) return;
	sxsg_ff_map_free((sxsg_ff_map *)table->type_map);
	if (table == g_default_table) g_default_table = NULL;
	free(table);
}

const char *ff_type_to_string(enum saxs_ff_type type) { return sxsg_ff_name((int)type); }

/* the trimmed key get_ff prints (leading blanks skipped, up to the next
 * blank, at most 7 characters) */
static void key_part(const char *src, char *dst)
{
	int n = 0;
	while (*src == ' ') src++;
	while (*src && *src != ' ' && n < 7) dst[n++] = *src++;
	dst[n] = 0;
}

const struct saxs_form_factor *get_ff(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag,
                                      size_t atom_index)
{
	const char *res = ag->residue_name[atom_index], *atom = ag->atom_name[atom_index];
	int type = sxsg_ff_map_type((const sxsg_ff_map *)table->type_map, res, atom);
	if (type < 0 || type == SXSG_FF_UNKNOWN || type >= HEAVY_ATOM_SIZE) {
		char r[8], a[8];
		key_part(res, r);
		key_part(atom, a);
		if (type < 0) fprintf(stderr, "mapping for (%s, %s) not found\n", r, a);
		else printf("(%s, %s) maps to UNK\n", r, a);
		return NULL;
	}
	return &table->factors[type];
}

static const struct saxs_form_factor *need_ff(const struct saxs_form_factor_table *table,
                                              const struct mol_atom_group *ag, size_t i, const char *func)
{
	const struct saxs_form_factor *ff = get_ff(table, ag, i);
	if (!ff) die(func, "atom without form factors");
	return ff;
}

double dummy_ff(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag, size_t atom_index)
{
	return need_ff(table, ag, atom_index, "dummy_ff")->dummy_ff;
}

double vacuum_ff(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag, size_t atom_index)
{
	return need_ff(table, ag, atom_index, "vacuum_ff")->vacuum_ff;
}

enum saxs_ff_type atom2ff_type(const struct saxs_form_factor_table *table, const struct mol_atom_group *ag,
                               size_t atom_index)
{
	int type = sxsg_ff_map_type((const sxsg_ff_map *)table->type_map, ag->residue_name[atom_index],
	                            ag->atom_name[atom_index]);
	return type < 0 ? s_UNK : (enum saxs_ff_type)type;
}

void get_dummy_ff(double *dummy_ffs, const struct mol_atom_group *ag, const struct saxs_form_factor_table *table)
{
	for (size_t i = 0; i < ag->natoms; i++) dummy_ffs[i] = dummy_ff(table, ag, i);
}

void get_vacuum_ff(double *vacuum_ffs, const struct mol_atom_group *ag, const struct saxs_form_factor_table *table)
{
	for (size_t i = 0; i < ag->natoms; i++) vacuum_ffs[i] = vacuum_ff(table, ag, i);
}

/* ------------------------------------------------------- geometry, SASA */

double mol_atom_group_max_dist(const struct mol_atom_group *ag)
{
	double best = 0.0;
	for (size_t i = 0; i < ag->natoms; i++)
		for (size_t j = i + 1; j < ag->natoms; j++) {
			double dx = ag->coords[i].X - ag->coords[j].X, dy = ag->coords[i].Y - ag->coords[j].Y,
			       dz = ag->coords[i].Z - ag->coords[j].Z;
			best = fmax(best, dx * dx + dy * dy + dz * dz);
		}
	return sqrt(best);
}

/* src/saxs_utils.c:19-28: the radii summed in atom order, then divided */
double mol_atom_group_average_radius(const struct mol_atom_group *ag)
{
	double sum = 0.0;
	for (size_t i = 0; i < ag->natoms; i++) sum += ag->vdw_radius[i];
	return sum / ag->natoms;
}

/* src/saxs_utils.c:30-48 */
void sxs_faccs(double *fractional_sa, const struct mol_atom_group *ag, double r_solv)
{
	const double area_unit = 4 * SXS_MOL2_PI;
	accs(fractional_sa, ag, r_solv, 1);
	for (size_t i = 0; i < ag->natoms; i++) {
		double r = ag->vdw_radius[i];
		if (r == 0 || isnan(fractional_sa[i])) fractional_sa[i] = 0.0;
		else fractional_sa[i] = fractional_sa[i] / (area_unit * r * r);
	}
}

/* ------------------------------------------------------------ expansion */

void atom_grp2spf_inplace(struct sxs_spf_full *spf_coefs, struct mol_atom_group *ag,
                          struct saxs_form_factor_table *ff_table, double *qvals, int qnum, int L, double *saxs_sa)
{
	if (!spf_coefs || !ag || !ff_table || !qvals) die("atom_grp2spf_inplace", "null argument");
	if (spf_coefs->L != L || spf_coefs->qnum != qnum)
		die("atom_grp2spf_inplace", "spf_coefs was created for another L or qnum");
	size_t n = ag->natoms;
	size_t na = n ? n : 1;
	double *xyz = malloc(sizeof(double) * 3 * na), *vac = malloc(sizeof(double) * na),
	       *dum = malloc(sizeof(double) * na);
	size_t flat_n = (size_t)3 * qnum * (L + 1) * (L + 1) * 2;
	double *flat = malloc(sizeof(double) * flat_n);
	if (!xyz || !vac || !dum || !flat) die("atom_grp2spf_inplace", "out of memory");
	for (size_t i = 0; i < n; i++) {
		xyz[3 * i] = ag->coords[i].X;
		xyz[3 * i + 1] = ag->coords[i].Y;
		xyz[3 * i + 2] = ag->coords[i].Z;
		const struct saxs_form_factor *ff = need_ff(ff_table, ag, i, "atom_grp2spf_inplace");
		vac[i] = ff->vacuum_ff;
		dum[i] = ff->dummy_ff;
	}
	double water = ff_table->factors[s_OH2].zero_ff;
	if (sxsg_expand(xyz, vac, dum, saxs_sa, water, (int)n, qvals, qnum, L, flat))
		die("atom_grp2spf_inplace", sxsg_last_error());
	sxsg_spf_from_flat(spf_coefs, flat);
	spf_coefs->rm = mol_atom_group_average_radius(ag);
	free(xyz);
	free(vac);
	free(dum);
	free(flat);
}

struct sxs_spf_full *atom_grp2spf(struct mol_atom_group *ag, struct saxs_form_factor_table *ff_table, double *qvals,
                                  int qnum, int L, int water)
{
	struct sxs_spf_full *spf = sxs_spf_full_create(L, qnum);
	double *sa = NULL;
	if (water == 1) {
		sa = calloc(ag->natoms ? ag->natoms : 1, sizeof(double));
		if (!sa) die("atom_grp2spf", "out of memory");
		sxs_faccs(sa, ag, 1.4);
	}
	atom_grp2spf_inplace(spf, ag, ff_table, qvals, qnum, L, sa);
	free(sa);
	return spf;
}

/* ------------------------------------------------------- pose ingestion */

void sxs_ft_file2euler_file(const char *eu_path, const char *ft_path, const char *rm_path,
                            struct mol_vector3 *ref_lig)
{
	FILE *ft = fopen(ft_path, "r");
	if (!ft) die("sxs_ft_file2euler_file", "cannot open the FT file");
	FILE *eu = fopen(eu_path, "w");
	if (!eu) die("sxs_ft_file2euler_file", "cannot open the Euler file");
	struct mol_matrix3_list *rot = mol_matrix3_list_from_file(rm_path);
	if (!rot) die("sxs_ft_file2euler_file", "cannot read the rotation file");
	int id;
	double v[9];
	int nread;
	while ((nread = fscanf(ft, "%d %lf %lf %lf %lf %lf %lf %lf %lf %lf", &id, &v[0], &v[1], &v[2], &v[3], &v[4],
	                       &v[5], &v[6], &v[7], &v[8])) != EOF) {
		if (nread != 10) die("sxs_ft_file2euler_file", "Wrong input file format.");
		if (id < 0 || (size_t)id >= rot->size) die("sxs_ft_file2euler_file", "rotation id out of range");
		struct mol_vector3 t = {v[0], v[1], v[2]};
		struct sxs_euler e;
		sxs_ft2euler(&e, &t, &rot->members[id], ref_lig);
		fprintf(eu, "%d\t% .3f\t% .3f\t% .3f\t% .3f\t% .3f\t% .3f\n", id, e.z, e.b1, e.g1, e.a2, e.b2, e.g2);
	}
	fclose(eu);
	fclose(ft);
}
