/*
 * Test stand-in bodies for the libmol2 functions the drop-in callers and
 * libfmftsaxs_gb300/mol2/sxs_mol2.c need (declarations in tests/c/mol2 and
 * oracle/shim/mol2).  TEST INFRASTRUCTURE only.
 *
 * accs: the accessible areas come from the file named by the environment
 * variable SXS_TEST_ACCS (one area per line), read in sequence: each call
 * takes the next natoms values (a test writes the receptor's areas, then
 * the ligand's: the fixture's accessible fractions times 4 pi r^2).
 * mol_matrix3_list_from_file: one rotation per line, nine numbers row-major.
 */
#define _XOPEN_SOURCE 700
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mol2/atom_group.h"
#include "mol2/lists.h"
#include "mol2/pdb.h"
#include "mol2/prms.h"
#include "mol2/sasa.h"

static void fail(const char *what)
{
	fprintf(stderr, "mol2 stand-in: %s\n", what);
	exit(EXIT_FAILURE);
}

bool is_whitespace_line(const char *line)
{
	for (; *line; line++)
		if (!isspace((unsigned char)*line)) return false;
	return true;
}

void free_if_not_null(void *p)
{
	if (p) free(p);
}

static char *field(const char *line, int from, int to)
{
	char *s = calloc(8, 1);
	int n = 0;
	for (int c = from; c < to && line[c] && line[c] != '\n'; c++) s[n++] = line[c];
	return s;
}

struct mol_atom_group *mol_read_pdb(const char *path)
{
	FILE *f = fopen(path, "r");
	if (!f) fail("cannot open PDB file");
	struct mol_atom_group *ag = calloc(1, sizeof(*ag));
	size_t cap = 0;
	char line[512];
	while (fgets(line, sizeof(line), f)) {
		if (strncmp(line, "ATOM", 4) && strncmp(line, "HETATM", 6)) continue;
		if (ag->natoms == cap) {
			cap = cap ? 2 * cap : 1024;
			ag->coords = realloc(ag->coords, sizeof(*ag->coords) * cap);
			ag->atom_name = realloc(ag->atom_name, sizeof(char *) * cap);
			ag->residue_name = realloc(ag->residue_name, sizeof(char *) * cap);
		}
		size_t i = ag->natoms++;
		ag->atom_name[i] = field(line, 12, 16);
		ag->residue_name[i] = field(line, 17, 21);
		if (strlen(line) < 31 ||
		    sscanf(line + 30, "%lf %lf %lf", &ag->coords[i].X, &ag->coords[i].Y, &ag->coords[i].Z) != 3)
			fail("bad coordinates");
	}
	fclose(f);
	ag->vdw_radius = calloc(ag->natoms ? ag->natoms : 1, sizeof(double));
	return ag;
}

void mol_atom_group_free(struct mol_atom_group *ag)
{
	if (!ag) return;
	for (size_t i = 0; i < ag->natoms; i++) {
		free(ag->atom_name[i]);
		free(ag->residue_name[i]);
	}
	free(ag->atom_name);
	free(ag->residue_name);
	free(ag->coords);
	free(ag->vdw_radius);
	free(ag);
}

void centroid(struct mol_vector3 *c, const struct mol_atom_group *ag)
{
	c->X = c->Y = c->Z = 0.0;
	for (size_t i = 0; i < ag->natoms; i++) {
		c->X += ag->coords[i].X;
		c->Y += ag->coords[i].Y;
		c->Z += ag->coords[i].Z;
	}
	c->X /= ag->natoms;
	c->Y /= ag->natoms;
	c->Z /= ag->natoms;
}

void center_of_extrema(struct mol_vector3 *c, const struct mol_atom_group *ag)
{
	struct mol_vector3 lo = ag->coords[0], hi = ag->coords[0];
	for (size_t i = 1; i < ag->natoms; i++) {
		lo.X = fmin(lo.X, ag->coords[i].X); hi.X = fmax(hi.X, ag->coords[i].X);
		lo.Y = fmin(lo.Y, ag->coords[i].Y); hi.Y = fmax(hi.Y, ag->coords[i].Y);
		lo.Z = fmin(lo.Z, ag->coords[i].Z); hi.Z = fmax(hi.Z, ag->coords[i].Z);
	}
	c->X = 0.5 * (lo.X + hi.X);
	c->Y = 0.5 * (lo.Y + hi.Y);
	c->Z = 0.5 * (lo.Z + hi.Z);
}

void mol_atom_group_translate(struct mol_atom_group *ag, const struct mol_vector3 *v)
{
	for (size_t i = 0; i < ag->natoms; i++) {
		ag->coords[i].X += v->X;
		ag->coords[i].Y += v->Y;
		ag->coords[i].Z += v->Z;
	}
}

struct mol_prms {
	size_t n;
	char (*res)[8];
	char (*atom)[8];
	double *radius;
};

struct mol_prms *mol_prms_read(const char *path)
{
	FILE *f = fopen(path, "r");
	if (!f) fail("cannot open parameter file");
	struct mol_prms *p = calloc(1, sizeof(*p));
	size_t cap = 0;
	char line[512];
	while (fgets(line, sizeof(line), f)) {
		char kw[16], r[8], a[8], t[32];
		int id;
		double rad;
		if (sscanf(line, "%15s %d %7s %7s %31s %lf", kw, &id, r, a, t, &rad) != 6 || strcmp(kw, "atom")) continue;
		if (p->n == cap) {
			cap = cap ? 2 * cap : 256;
			p->res = realloc(p->res, sizeof(*p->res) * cap);
			p->atom = realloc(p->atom, sizeof(*p->atom) * cap);
			p->radius = realloc(p->radius, sizeof(double) * cap);
		}
		strcpy(p->res[p->n], r);
		strcpy(p->atom[p->n], a);
		p->radius[p->n++] = rad;
	}
	fclose(f);
	return p;
}

void mol_prms_free(struct mol_prms *p)
{
	if (!p) return;
	free(p->res);
	free(p->atom);
	free(p->radius);
	free(p);
}

static void trim(const char *s, char *d)
{
	int n = 0;
	while (*s == ' ') s++;
	while (*s && *s != ' ' && n < 7) d[n++] = *s++;
	d[n] = 0;
}

bool mol_atom_group_add_prms(struct mol_atom_group *ag, const struct mol_prms *p)
{
	for (size_t i = 0; i < ag->natoms; i++) {
		char r[8], a[8];
		trim(ag->residue_name[i], r);
		trim(ag->atom_name[i], a);
		size_t k = 0;
		while (k < p->n && (strcmp(p->res[k], r) || strcmp(p->atom[k], a))) k++;
		if (k == p->n) fail("atom without parameters");
		ag->vdw_radius[i] = p->radius[k];
	}
	return true;
}

void accs(double *as, const struct mol_atom_group *ag, double r_solv, short cont_acc)
{
	(void)r_solv;
	(void)cont_acc;
	static FILE *f = NULL;
	if (!f) {
		const char *path = getenv("SXS_TEST_ACCS");
		f = path ? fopen(path, "r") : NULL;
		if (!f) fail("accs: set SXS_TEST_ACCS to a file of accessible areas");
	}
	for (size_t i = 0; i < ag->natoms; i++)
		if (fscanf(f, "%lf", &as[i]) != 1) fail("accs: short area file");
}

struct mol_matrix3_list *mol_matrix3_list_from_file(const char *path)
{
	FILE *f = fopen(path, "r");
	if (!f) return NULL;
	struct mol_matrix3_list *l = calloc(1, sizeof(*l));
	size_t cap = 0;
	struct mol_matrix3 m;
	while (fscanf(f, "%lf %lf %lf %lf %lf %lf %lf %lf %lf", &m.m11, &m.m12, &m.m13, &m.m21, &m.m22, &m.m23, &m.m31,
	              &m.m32, &m.m33) == 9) {
		if (l->size == cap) {
			cap = cap ? 2 * cap : 1024;
			l->members = realloc(l->members, sizeof(m) * cap);
		}
		l->members[l->size++] = m;
	}
	fclose(f);
	return l;
}
