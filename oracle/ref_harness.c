/*
 * Checker harness around the reference's OWN sources (compiled unchanged from
 * the reference tree by oracle/Makefile.ref into oracle/_ref/libsxsref.so).
 * It exposes flat-array entry points so Python tests can run the reference
 * on the same inputs as the oracle restatement and the GPU path.
 *
 * Test infrastructure only: never linked into the product.
 *
 * Cross terms are captured by interposing sxs_fit_params, the external
 * symbol that sxs_compute_saxs_scores calls once per touched triple
 * (src/fftsaxs.c:909).  The reference's own definition is compiled under the
 * name sxs_fit_params_ref_impl (a -D rename on src/min_saxs.c only); the
 * wrapper below records the raw cross terms, calls it (peak rescale +
 * L-BFGS-B, src/min_saxs.c:153-194), then records the rescaled cross terms and
 * the reference's chi-square (point_score, src/min_saxs.c:391-448) at every
 * cell of a caller-given (c1, c2) grid.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftsaxs.h"
#include "min_saxs.h"
#include "pdb2spf.h"
#include "profile.h"
#include "index.h"
#include "borrowed.h"
#include "saxs_utils.h"
#include "form_factor_table.h"

void sxs_fit_params_ref_impl(struct sxs_profile **profiles, struct sxs_opt_params *params, int *mask, int n);
double point_score(struct sxs_profile *profile, struct sxs_opt_params *params, double c1, double c2);

/* ---------------------------------------------------------------- capture */
static struct {
	int active;
	int call;            /* how many triples fitted so far */
	int nout;
	int L;
	int qnum;
	const int *pose_triple;   /* [nout] order of the pose's triple among fitted triples */
	const int *pose_cell;     /* [nout] (a2*N+g1)*N+g2 */
	double *cross_raw;        /* [nout][6][qnum] */
	double *cross_scaled;     /* [nout][6][qnum] */
	double *grid;             /* [nout][n1*n2] */
	const double *c1g, *c2g;
	int n1, n2;
} cap;

static void copy_cross(double *dst, const struct sxs_profile *p, int qnum)
{
	const double *src[6] = {p->VV, p->VD, p->VW, p->DD, p->DW, p->WW};
	for (int c = 0; c < 6; c++)
		memcpy(dst + c * qnum, src[c], sizeof(double) * qnum);
}

void sxs_fit_params(struct sxs_profile **profiles, struct sxs_opt_params *params, int *mask, int n)
{
	if (cap.active) {
		for (int i = 0; i < cap.nout; i++)
			if (cap.pose_triple[i] == cap.call)
				copy_cross(cap.cross_raw + (size_t)i * 6 * cap.qnum, profiles[cap.pose_cell[i]], cap.qnum);
	}
	sxs_fit_params_ref_impl(profiles, params, mask, n);
	if (cap.active) {
		for (int i = 0; i < cap.nout; i++) {
			if (cap.pose_triple[i] != cap.call) continue;
			struct sxs_profile *p = profiles[cap.pose_cell[i]];
			copy_cross(cap.cross_scaled + (size_t)i * 6 * cap.qnum, p, cap.qnum);
			if (cap.grid)
				for (int a = 0; a < cap.n1; a++)
					for (int b = 0; b < cap.n2; b++)
						cap.grid[(size_t)i * cap.n1 * cap.n2 + a * cap.n2 + b] =
							point_score(p, params, cap.c1g[a], cap.c2g[b]);
		}
		cap.call++;
	}
}

/* ------------------------------------------------------------ conversions */
static struct sxs_spf_full *spf_from_flat(const double *flat, int L, int qnum, double rm)
{
	struct sxs_spf_full *s = sxs_spf_full_create(L, qnum);
	int K2 = (L + 1) * (L + 1);
	s->rm = rm;
	for (int ch = 0; ch < 3; ch++) {
		struct sxs_spf_sing **arr = ch == 0 ? s->V : (ch == 1 ? s->D : s->W);
		for (int q = 0; q < qnum; q++)
			for (int i = 0; i < K2; i++) {
				const double *v = flat + (((size_t)ch * qnum + q) * K2 + i) * 2;
				arr[q]->re[i] = v[0];
				arr[q]->im[i] = v[1];
			}
	}
	return s;
}

static void spf_to_flat(double *flat, const struct sxs_spf_full *s)
{
	int L = s->L, qnum = s->qnum, K2 = (L + 1) * (L + 1);
	for (int ch = 0; ch < 3; ch++) {
		struct sxs_spf_sing **arr = ch == 0 ? s->V : (ch == 1 ? s->D : s->W);
		for (int q = 0; q < qnum; q++)
			for (int i = 0; i < K2; i++) {
				double *v = flat + (((size_t)ch * qnum + q) * K2 + i) * 2;
				v[0] = arr[q]->re[i];
				v[1] = arr[q]->im[i];
			}
	}
}

static void spf_full_release(struct sxs_spf_full *s)
{
	sxs_spf_full_destroy(s);
	free(s->V); free(s->D); free(s->W);
	free(s);
}

/* Experimental profile with a +inf sentinel after the last point: the bin
 * loop in scoring_helper (src/min_saxs.c:369) does not bound j. */
static struct sxs_profile *exp_profile(const double *q, const double *in, const double *err, int n)
{
	double *qv = calloc(n + 1, sizeof(double));
	memcpy(qv, q, sizeof(double) * n);
	qv[n] = INFINITY;
	struct sxs_profile *p = sxs_profile_create(qv, n, 0);
	p->in = realloc(p->in, sizeof(double) * (n + 1));
	p->err = realloc(p->err, sizeof(double) * (n + 1));
	memcpy(p->in, in, sizeof(double) * n);
	memcpy(p->err, err, sizeof(double) * n);
	p->in[n] = 0.0; p->err[n] = 1.0;
	return p;
}

static void exp_profile_release(struct sxs_profile *p)
{
	double *qv = p->qvals;
	sxs_profile_free(p);
	free(qv);
}

/* ------------------------------------------------------------- exports */
double refh_sbessel(int l, double x) { return sxs_sbessel(l, x); }

void refh_mkarray(double b, double e, int n, double *out)
{
	double *q = sxs_mkarray(b, e, n);
	memcpy(out, q, sizeof(double) * n);
	free(q);
}

/* Wigner small-d table of src/borrowed.c:243-313, layout index_d_array. */
void refh_d_array(int L, double beta, double *out)
{
	struct d_array *d = generate_d_array(L, beta);
	memcpy(out, d->data, sizeof(double) * (L + 1) * (2 * L + 1) * (2 * L + 1));
	deallocate_d_array(d);
}

/* One 3j symbol through the reference's Racah evaluation (borrowed.c:86-222). */
double refh_w3j(int j1, int j2, int j3, int m1, int m2, int m3, int nfact)
{
	mpf_t *fact = generate_desc_fact_array_arb(nfact);
	mpf_t r;
	mpf_init(r);
	wigner_3j_symbol_arb(r, j1, j2, j3, m1, m2, m3, (const mpf_t *)fact);
	double v = mpf_get_d(r);
	free(fact);
	return v;
}

double refh_average_radius(const double *vdw, int n)
{
	struct mol_atom_group ag = {0};
	ag.natoms = n;
	ag.vdw_radius = (double *)vdw;
	return mol_atom_group_average_radius(&ag);
}

/* Look up (vacuum_ff, dummy_ff) for each atom through default_ff_table and
 * get_ff (form_factor_table.c:138-188, 294-339).  Names are 8-byte slots. */
int refh_ff_lookup(const char *map_path, const char *res, const char *atom, int n, double *vac, double *dum, double *h2o)
{
	struct saxs_form_factor_table *t = default_ff_table(map_path);
	struct mol_atom_group ag = {0};
	char **rn = calloc(n, sizeof(char *)), **an = calloc(n, sizeof(char *));
	for (int i = 0; i < n; i++) { rn[i] = (char *)res + 8 * i; an[i] = (char *)atom + 8 * i; }
	ag.natoms = n; ag.residue_name = rn; ag.atom_name = an;
	int bad = 0;
	for (int i = 0; i < n; i++) {
		const struct saxs_form_factor *f = get_ff(t, &ag, i);
		if (!f) { bad++; vac[i] = dum[i] = NAN; continue; }
		vac[i] = f->vacuum_ff;
		dum[i] = f->dummy_ff;
	}
	*h2o = t->factors[s_OH2].zero_ff;
	free(rn); free(an);
	return bad;
}

/* atom_grp2spf_inplace on caller arrays; sasa may be NULL (water = 0). */
int refh_expand(const double *xyz, const char *res, const char *atom, const double *vdw, const double *sasa,
                int n, const char *map_path, const double *q, int qnum, int L, double *out, double *rm)
{
	struct saxs_form_factor_table *t = default_ff_table(map_path);
	struct mol_atom_group ag = {0};
	ag.natoms = n;
	ag.coords = malloc(sizeof(struct mol_vector3) * n);
	ag.vdw_radius = (double *)vdw;
	char **rn = calloc(n, sizeof(char *)), **an = calloc(n, sizeof(char *));
	for (int i = 0; i < n; i++) {
		ag.coords[i].X = xyz[3 * i]; ag.coords[i].Y = xyz[3 * i + 1]; ag.coords[i].Z = xyz[3 * i + 2];
		rn[i] = (char *)res + 8 * i; an[i] = (char *)atom + 8 * i;
	}
	ag.residue_name = rn; ag.atom_name = an;
	struct sxs_spf_full *s = sxs_spf_full_create(L, qnum);
	atom_grp2spf_inplace(s, &ag, t, (double *)q, qnum, L, (double *)sasa);
	spf_to_flat(out, s);
	*rm = s->rm;
	spf_full_release(s);
	free(ag.coords); free(rn); free(an);
	return 0;
}

/* sxs_profile_from_spf (profile.c:186-233): I and err per q. */
void refh_profile_from_spf(const double *spf, int L, int qnum, double rm, const double *q, double c1, double c2,
                           double *in, double *err)
{
	struct sxs_spf_full *s = spf_from_flat(spf, L, qnum, rm);
	struct sxs_profile *p = sxs_profile_create((double *)q, qnum, 0);
	sxs_profile_from_spf(p, s, c1, c2);
	memcpy(in, p->in, sizeof(double) * qnum);
	memcpy(err, p->err, sizeof(double) * qnum);
	sxs_profile_free(p);
	spf_full_release(s);
}

/* scoring_helper + opt params (min_saxs.c:116-124, 353-389). */
void refh_opt_params(const double *eq, const double *ei, const double *ee, int ne, const double *q, int qnum,
                     double rm, double *a_out, double *mult, double *peak)
{
	struct sxs_profile *e = exp_profile(eq, ei, ee, ne);
	struct sxs_opt_params *p = sxs_opt_params_create(e, (double *)q, qnum, rm);
	memcpy(a_out, p->a, sizeof(double) * 6 * qnum);
	*mult = p->mult;
	*peak = p->peak;
	sxs_opt_params_free(p);
	exp_profile_release(e);
}

/* Fit one set of cross terms [6][qnum] exactly as sxs_fit_params does for a
 * masked pose: peak rescale, then L-BFGS-B (min_saxs.c:153-259).  Returns the
 * rescaled cross terms, chi, c1, c2, scale and the fitted intensity. */
void refh_fit_cross(const double *cross, const double *eq, const double *ei, const double *ee, int ne,
                    const double *q, int qnum, double rm, double *scaled, double *res5, double *in_out)
{
	struct sxs_profile *e = exp_profile(eq, ei, ee, ne);
	struct sxs_opt_params *par = sxs_opt_params_create(e, (double *)q, qnum, rm);
	struct sxs_profile *p = sxs_profile_create((double *)q, qnum, 1);
	double *dst[6] = {p->VV, p->VD, p->VW, p->DD, p->DW, p->WW};
	for (int c = 0; c < 6; c++) memcpy(dst[c], cross + c * qnum, sizeof(double) * qnum);
	int mask = 1;
	sxs_fit_params_ref_impl(&p, par, &mask, 1);
	copy_cross(scaled, p, qnum);
	res5[0] = p->score; res5[1] = p->c1; res5[2] = p->c2; res5[3] = p->scale;
	res5[4] = 0.0;
	memcpy(in_out, p->in, sizeof(double) * qnum);
	sxs_profile_free(p);
	sxs_opt_params_free(par);
	exp_profile_release(e);
}

/* point_score on given (already rescaled) cross terms. */
double refh_point_score(const double *cross, const double *eq, const double *ei, const double *ee, int ne,
                        const double *q, int qnum, double rm, double c1, double c2)
{
	struct sxs_profile *e = exp_profile(eq, ei, ee, ne);
	struct sxs_opt_params *par = sxs_opt_params_create(e, (double *)q, qnum, rm);
	struct sxs_profile *p = sxs_profile_create((double *)q, qnum, 1);
	double *dst[6] = {p->VV, p->VD, p->VW, p->DD, p->DW, p->WW};
	for (int c = 0; c < 6; c++) memcpy(dst[c], cross + c * qnum, sizeof(double) * qnum);
	double s = point_score(p, par, c1, c2);
	sxs_profile_free(p);
	sxs_opt_params_free(par);
	exp_profile_release(e);
	return s;
}

/* Full scoring call.  Poses must be in range (z < znum).  out_* may be NULL. */
int refh_score(const double *A, const double *B, double rmA, double rmB, double rm_mean,
               const double *eq, const double *ei, const double *ee, int ne,
               const double *q, int qnum, const double *z, int znum, int L,
               const int *index, int nout, int skip,
               const double *c1g, int n1, const double *c2g, int n2,
               double *chi, double *c1, double *c2,
               double *cross_raw, double *cross_scaled, double *grid, int *branch)
{
	int nb = L + 1, N = 2 * L + 1, N3 = N * N * N;
	struct sxs_spf_full *sA = spf_from_flat(A, L, qnum, rmA);
	struct sxs_spf_full *sB = spf_from_flat(B, L, qnum, rmB);
	struct sxs_profile *e = exp_profile(eq, ei, ee, ne);
	struct sxs_opt_params *par = sxs_opt_params_create(e, (double *)q, qnum, rm_mean);

	/* order in which the reference fits triples */
	int ntrip = znum * nb * nb;
	int *count = calloc(ntrip, sizeof(int));
	int *order = malloc(sizeof(int) * ntrip);
	int *ptrip = malloc(sizeof(int) * (nout > 0 ? nout : 1));
	int *pcell = malloc(sizeof(int) * (nout > 0 ? nout : 1));
	for (int i = 0; i < nout; i++) {
		struct sxs_index id;
		sxs_disassemble_index(&id, (size_t)(unsigned)index[i], nb, L);
		if (index[i] < 0 || id.z >= znum) { return -1; }
		count[(id.z * nb + id.b1) * nb + id.b2]++;
		pcell[i] = (id.a2 * N + id.g1) * N + id.g2;
		ptrip[i] = (id.z * nb + id.b1) * nb + id.b2;
	}
	int k = 0;
	for (int t = 0; t < ntrip; t++) order[t] = (skip == 1 && count[t] == 0) ? -1 : k++;
	for (int i = 0; i < nout; i++) {
		if (branch) branch[i] = (skip != 1 || count[ptrip[i]] >= 30) ? 1 : 0;
		ptrip[i] = order[ptrip[i]];
	}
	(void)N3;

	memset(&cap, 0, sizeof(cap));
	cap.active = 1;
	cap.nout = nout; cap.L = L; cap.qnum = qnum;
	cap.pose_triple = ptrip; cap.pose_cell = pcell;
	double *cr = cross_raw ? cross_raw : calloc((size_t)(nout > 0 ? nout : 1) * 6 * qnum, sizeof(double));
	double *cs = cross_scaled ? cross_scaled : calloc((size_t)(nout > 0 ? nout : 1) * 6 * qnum, sizeof(double));
	cap.cross_raw = cr; cap.cross_scaled = cs;
	cap.grid = grid; cap.c1g = c1g; cap.c2g = c2g; cap.n1 = n1; cap.n2 = n2;

	double *s = calloc(nout > 0 ? nout : 1, sizeof(double));
	double *a = calloc(nout > 0 ? nout : 1, sizeof(double));
	double *b = calloc(nout > 0 ? nout : 1, sizeof(double));
	sxs_compute_saxs_scores(s, a, b, (int *)index, nout, sA, sB, par, (double *)q, qnum, (double *)z, znum, L, skip);
	cap.active = 0;
	if (chi) memcpy(chi, s, sizeof(double) * nout);
	if (c1) memcpy(c1, a, sizeof(double) * nout);
	if (c2) memcpy(c2, b, sizeof(double) * nout);

	if (!cross_raw) free(cr);
	if (!cross_scaled) free(cs);
	free(s); free(a); free(b);
	free(count); free(order); free(ptrip); free(pcell);
	sxs_opt_params_free(par);
	exp_profile_release(e);
	spf_full_release(sA);
	spf_full_release(sB);
	return 0;
}

/* sxs_ft2euler (index.c:38-75) for pose generation. */
void refh_ft2euler(const double *tv, const double *rm9, const double *ref_lig, double *out6)
{
	struct sxs_euler eu;
	struct mol_vector3 t = {tv[0], tv[1], tv[2]}, r = {ref_lig[0], ref_lig[1], ref_lig[2]};
	struct mol_matrix3 m = {rm9[0], rm9[1], rm9[2], rm9[3], rm9[4], rm9[5], rm9[6], rm9[7], rm9[8]};
	sxs_ft2euler(&eu, &t, &m, &r);
	out6[0] = eu.z; out6[1] = eu.b1; out6[2] = eu.g1; out6[3] = eu.a2; out6[4] = eu.b2; out6[5] = eu.g2;
}
