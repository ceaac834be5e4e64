/*
 * Drop-in C API of the reference (containers, text I/O, fit helpers for
 * one profile, grid/index utilities, form-factor lookup) and the drop-in
 * scoring call.  Functions keep the reference's names, argument meanings,
 * ownership rules and exit-on-error behaviour; single-profile helpers that
 * are O(qnum) stay on the host, everything per pose runs on the GPU.
 */
#define _XOPEN_SOURCE 700
#include <ctype.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sxs_internal.h"

#define DIE(msg) sxs_die(__func__, (msg))
#define NEED(ptr) do { if ((ptr) == NULL) DIE("Null pointer"); } while (0)

/* Zeroed allocation for the drop-in functions, which exit on error like
 * the reference (n or size 0 still returns a distinct pointer). */
static void *xcalloc(const char *func, size_t n, size_t size)
{
	void *p = calloc(n ? n : 1, size ? size : 1);
	if (!p) sxs_die(func, "out of memory");
	return p;
}
#define XCALLOC(n, size) xcalloc(__func__, (n), (size))

/* ======================================================== containers */

/* src/pdb2spf.c:178-207 */
struct sxs_spf_sing *sxs_spf_sing_create(int L)
{
	struct sxs_spf_sing *s = XCALLOC(1, sizeof(*s));
	sxs_spf_sing_init(s, L);
	return s;
}

void sxs_spf_sing_init(struct sxs_spf_sing *s, int L)
{
	if (!s) return;
	s->L = L;
	s->re = XCALLOC((size_t)(L + 1) * (L + 1), sizeof(double));
	s->im = XCALLOC((size_t)(L + 1) * (L + 1), sizeof(double));
}

void sxs_spf_sing_destroy(struct sxs_spf_sing *s)
{
	if (!s) return;
	free(s->re);
	free(s->im);
	s->re = s->im = NULL;
}

void sxs_spf_sing_free(struct sxs_spf_sing *s)
{
	sxs_spf_sing_destroy(s);
	free(s);
}

/* src/pdb2spf.c:209-265.  destroy also releases the per-channel pointer
 * arrays, which the reference leaks (pdb2spf.c:241-250). */
struct sxs_spf_full *sxs_spf_full_create(int L, int qnum)
{
	struct sxs_spf_full *s = XCALLOC(1, sizeof(*s));
	sxs_spf_full_init(s, L, qnum);
	return s;
}

void sxs_spf_full_init(struct sxs_spf_full *s, int L, int qnum)
{
	if (!s) return;
	s->L = L;
	s->qnum = qnum;
	s->rm = 0.0;
	s->V = XCALLOC(qnum, sizeof(*s->V));
	s->D = XCALLOC(qnum, sizeof(*s->D));
	s->W = XCALLOC(qnum, sizeof(*s->W));
	for (int i = 0; i < qnum; i++) {
		s->V[i] = sxs_spf_sing_create(L);
		s->D[i] = sxs_spf_sing_create(L);
		s->W[i] = sxs_spf_sing_create(L);
	}
}

void sxs_spf_full_destroy(struct sxs_spf_full *s)
{
	if (!s) return;
	for (int i = 0; i < s->qnum; i++) {
		sxs_spf_sing_free(s->V[i]);
		sxs_spf_sing_free(s->D[i]);
		sxs_spf_sing_free(s->W[i]);
	}
	free(s->V); free(s->D); free(s->W);
	s->V = s->D = s->W = NULL;
	s->qnum = 0;
}

void sxs_spf_full_free(struct sxs_spf_full *s)
{
	sxs_spf_full_destroy(s);
	free(s);
}

void sxs_spf_full_reset(struct sxs_spf_full *s)
{
	size_t n = (size_t)(s->L + 1) * (s->L + 1);
	for (int i = 0; i < s->qnum; i++) {
		memset(s->V[i]->re, 0, n * sizeof(double)); memset(s->V[i]->im, 0, n * sizeof(double));
		memset(s->D[i]->re, 0, n * sizeof(double)); memset(s->D[i]->im, 0, n * sizeof(double));
		memset(s->W[i]->re, 0, n * sizeof(double)); memset(s->W[i]->im, 0, n * sizeof(double));
	}
}

/* SPF text format (src/pdb2spf.c:267-350): header "% i % i % .4f" (L, qnum,
 * rm), then per q and lm one line of six "% .4e" values V re/im, D re/im,
 * W re/im. */
void sxs_spf_full_write(char *path, struct sxs_spf_full *s)
{
	FILE *f = fopen(path, "w");
	if (!f) DIE("cannot open output file");
	fprintf(f, "% i % i % .4f\n", s->L, s->qnum, s->rm);
	int K2 = (s->L + 1) * (s->L + 1);
	for (int q = 0; q < s->qnum; q++)
		for (int i = 0; i < K2; i++)
			fprintf(f, "% .4e % .4e % .4e % .4e % .4e % .4e\n", s->V[q]->re[i], s->V[q]->im[i], s->D[q]->re[i],
			        s->D[q]->im[i], s->W[q]->re[i], s->W[q]->im[i]);
	fclose(f);
}

struct sxs_spf_full *sxs_spf_full_fread(FILE *f)
{
	if (!f) return NULL;
	int L, qnum;
	double rm;
	if (fscanf(f, "%i %i %lf\n", &L, &qnum, &rm) != 3) DIE("Wrong input file format.");
	if (L < 0 || qnum < 0) DIE("Wrong input file format.");
	struct sxs_spf_full *s = sxs_spf_full_create(L, qnum);
	s->rm = rm;
	int K2 = (L + 1) * (L + 1);
	for (int q = 0; q < qnum; q++)
		for (int i = 0; i < K2; i++)
			if (fscanf(f, "%lf %lf %lf %lf %lf %lf\n", &s->V[q]->re[i], &s->V[q]->im[i], &s->D[q]->re[i],
			           &s->D[q]->im[i], &s->W[q]->re[i], &s->W[q]->im[i]) != 6)
				DIE("Wrong input file format.");
	return s;
}

struct sxs_spf_full *sxs_spf_full_read(char *path)
{
	FILE *f = fopen(path, "r");
	if (!f) DIE("cannot open input file");
	struct sxs_spf_full *s = sxs_spf_full_fread(f);
	fclose(f);
	return s;
}

int sxsg_spf_to_flat(const struct sxs_spf_full *s, double *flat)
{
	if (!s || !flat) return sxs_fail(-2, "sxsg_spf_to_flat: null argument");
	int K2 = (s->L + 1) * (s->L + 1), Q = s->qnum;
	for (int ch = 0; ch < 3; ch++) {
		struct sxs_spf_sing **a = ch == 0 ? s->V : (ch == 1 ? s->D : s->W);
		for (int q = 0; q < Q; q++)
			for (int i = 0; i < K2; i++) {
				double *v = flat + (((size_t)ch * Q + q) * K2 + i) * 2;
				v[0] = a[q]->re[i];
				v[1] = a[q]->im[i];
			}
	}
	return 0;
}

int sxsg_spf_from_flat(struct sxs_spf_full *s, const double *flat)
{
	if (!s || !flat) return sxs_fail(-2, "sxsg_spf_from_flat: null argument");
	int K2 = (s->L + 1) * (s->L + 1), Q = s->qnum;
	for (int ch = 0; ch < 3; ch++) {
		struct sxs_spf_sing **a = ch == 0 ? s->V : (ch == 1 ? s->D : s->W);
		for (int q = 0; q < Q; q++)
			for (int i = 0; i < K2; i++) {
				const double *v = flat + (((size_t)ch * Q + q) * K2 + i) * 2;
				a[q]->re[i] = v[0];
				a[q]->im[i] = v[1];
			}
	}
	return 0;
}

/* ========================================================== profiles */

/* src/profile.c:3-67.  The profile borrows qvals; destroy clears the pointer
 * without freeing it. */
struct sxs_profile *sxs_profile_create(double *qvals, int qnum, int cross_terms_flag)
{
	struct sxs_profile *p = XCALLOC(1, sizeof(*p));
	sxs_profile_init(p, qvals, qnum, cross_terms_flag);
	return p;
}

void sxs_profile_init(struct sxs_profile *p, double *qvals, int qnum, int cross_terms_flag)
{
	if (!p) return;
	p->qnum = qnum;
	p->rerr = SXS_REL_ERR;
	p->qvals = qvals;
	p->in = XCALLOC(qnum, sizeof(double));
	p->err = XCALLOC(qnum, sizeof(double));
	p->score = INFINITY;
	p->c1 = SXS_C1_DEFAULT;
	p->c2 = SXS_C2_DEFAULT;
	p->scale = 1.0;
	if (cross_terms_flag == 1) sxs_profile_alloc_cross_terms(p, qnum);
	else p->VV = p->VD = p->VW = p->DD = p->DW = p->WW = NULL;
}

void sxs_profile_alloc_cross_terms(struct sxs_profile *p, int qnum)
{
	p->VV = XCALLOC(qnum, sizeof(double));
	p->VD = XCALLOC(qnum, sizeof(double));
	p->VW = XCALLOC(qnum, sizeof(double));
	p->DD = XCALLOC(qnum, sizeof(double));
	p->DW = XCALLOC(qnum, sizeof(double));
	p->WW = XCALLOC(qnum, sizeof(double));
}

void sxs_profile_destroy(struct sxs_profile *p)
{
	p->qvals = NULL;
	free(p->in); free(p->err);
	free(p->VV); free(p->VD); free(p->VW); free(p->DD); free(p->DW); free(p->WW);
	p->in = p->err = p->VV = p->VD = p->VW = p->DD = p->DW = p->WW = NULL;
}

void sxs_profile_free(struct sxs_profile *p)
{
	sxs_profile_destroy(p);
	free(p);
}

/* "%.4f %.4f %.4f" per q; a non-positive err is replaced by in * rerr
 * (src/profile.c:69-85). */
void sxs_profile_write(char *path, struct sxs_profile *p)
{
	FILE *f = fopen(path, "w");
	if (!f) {
		fprintf(stderr, "Unable to open %s\n", path);
		exit(EXIT_FAILURE);
	}
	for (int i = 0; i < p->qnum; i++) {
		double err = p->err[i] > 0.0 ? p->err[i] : p->in[i] * p->rerr;
		fprintf(f, "%.4f %.4f %.4f\n", p->qvals[i], p->in[i], err);
	}
	fclose(f);
}

/* Three whitespace-separated columns q, I, err; qvals is allocated here and
 * owned by the caller (src/profile.c:98-124). */
struct sxs_profile *sxs_profile_fread(FILE *f)
{
	if (!f) return NULL;
	int n = 0, c;
	double a, b, d;
	while ((c = fscanf(f, "%lf %lf %lf", &a, &b, &d)) != EOF) {
		if (c != 3) DIE("Wrong input file format.");
		n++;
	}
	rewind(f);
	double *qv = XCALLOC(n, sizeof(double));
	struct sxs_profile *p = sxs_profile_create(qv, n, 0);
	for (int i = 0; i < n; i++)
		if (fscanf(f, "%lf %lf %lf\n", &qv[i], &p->in[i], &p->err[i]) != 3) DIE("Wrong input file format.");
	return p;
}

struct sxs_profile *sxs_profile_read(char *path)
{
	FILE *f = fopen(path, "r");
	if (!f) DIE("cannot open input file");
	struct sxs_profile *p = sxs_profile_fread(f);
	fclose(f);
	return p;
}

static double g_mult(double rm)
{
	return pow(4.0 * SXS_PI / 3.0, 3.0 / 2.0) * rm * rm / (16.0 * SXS_PI);
}

/* I(q) = sum_lm |V - G D + c2 W|^2 with G from q[0] for every q, as the
 * reference evaluates it (src/profile.c:186-233). */
void sxs_profile_from_spf(struct sxs_profile *p, struct sxs_spf_full *s, double c1, double c2)
{
	NEED(p);
	NEED(s);
	if (p->qnum != s->qnum) DIE("profile and expansion have different qnum");
	int K2 = (s->L + 1) * (s->L + 1);
	double corr = -g_mult(s->rm) * (c1 * c1 - 1.0);
	for (int q = 0; q < p->qnum; q++) {
		double G = c1 * c1 * c1 * exp(corr * p->qvals[0] * p->qvals[0]);
		double in = 0.0;
		for (int i = 0; i < K2; i++) {
			double ar = s->V[q]->re[i] - G * s->D[q]->re[i] + c2 * s->W[q]->re[i];
			double ai = s->V[q]->im[i] - G * s->D[q]->im[i] + c2 * s->W[q]->im[i];
			in += ar * ar + ai * ai;
		}
		p->in[q] = in;
		p->err[q] = in * p->rerr;
	}
	p->c1 = c1;
	p->c2 = c2;
}

/* ============================================================ fitting */

/* Bins experimental points into model q-bins: bin i takes points with
 * q in [q_{i-1}, q_i] (bin 0: q == q_0), six 1/sigma^2-weighted moments,
 * divided by the number of points used (src/min_saxs.c:353-389).  The
 * reference does not stop at the last experimental point; here j is
 * bounded by exp->qnum. */
double *scoring_helper(struct sxs_profile *e, int qnum, double *qvals)
{
	double *a = XCALLOC((size_t)6 * qnum, sizeof(double));
	int j = 0;
	for (int i = 0; i < qnum; i++) {
		double lo = i > 0 ? qvals[i - 1] : qvals[0], hi = qvals[i];
		while (j < e->qnum && e->qvals[j] >= lo && e->qvals[j] <= hi) {
			a[i * 6 + 0] += e->in[j] * e->in[j] / (e->err[j] * e->err[j]);
			a[i * 6 + 1] += e->in[j] / (e->err[j] * e->err[j]);
			a[i * 6 + 2] += e->qvals[j] * e->in[j] / (e->err[j] * e->err[j]);
			a[i * 6 + 3] += 1.0 / (e->err[j] * e->err[j]);
			a[i * 6 + 4] += e->qvals[j] / (e->err[j] * e->err[j]);
			a[i * 6 + 5] += e->qvals[j] * e->qvals[j] / (e->err[j] * e->err[j]);
			j++;
		}
	}
	double norm = (double)j;
	for (int i = 0; i < 6 * qnum; i++) a[i] /= norm;
	return a;
}

/* src/min_saxs.c:108-150 */
struct sxs_opt_params *sxs_opt_params_create(struct sxs_profile *e, double *qvals, int qnum, double rm)
{
	struct sxs_opt_params *p = XCALLOC(1, sizeof(*p));
	sxs_opt_params_init(p, e, qvals, qnum, rm);
	return p;
}

void sxs_opt_params_init(struct sxs_opt_params *p, struct sxs_profile *e, double *qvals, int qnum, double rm)
{
	if (!p) return;
	p->a = scoring_helper(e, qnum, qvals);
	p->rm = rm;
	p->mult = pow(4.0 * SXS_PI / 3.0, 1.5) * rm * rm / (16.0 * SXS_PI);
	p->peak = e->in[0];
}

void sxs_opt_params_destroy(struct sxs_opt_params *p)
{
	if (!p) return;
	free(p->a);
	p->a = NULL;
}

void sxs_opt_params_free(struct sxs_opt_params *p)
{
	sxs_opt_params_destroy(p);
	free(p);
}

int sxsg_bin_experiment(const double *eq, const double *ei, const double *ee, int ne, const double *q, int qnum,
                        double rm, double *a, double *mult, double *peak)
{
	if (!eq || !ei || !ee || ne <= 0 || !q || qnum <= 0 || !a || !mult || !peak)
		return sxs_fail(-2, "sxsg_bin_experiment: bad arguments");
	struct sxs_profile e;
	memset(&e, 0, sizeof(e));
	e.qnum = ne;
	e.qvals = (double *)eq;
	e.in = (double *)ei;
	e.err = (double *)ee;
	double *t = scoring_helper(&e, qnum, (double *)q);
	memcpy(a, t, sizeof(double) * 6 * qnum);
	free(t);
	*mult = pow(4.0 * SXS_PI / 3.0, 1.5) * rm * rm / (16.0 * SXS_PI);
	*peak = ei[0];
	return 0;
}

static double model_in(const struct sxs_profile *p, int i, double G, double c2)
{
	return p->VV[i] - G * p->VD[i] + c2 * p->VW[i] + G * G * p->DD[i] - G * c2 * p->DW[i] + c2 * c2 * p->WW[i];
}

/* Optimal scale k = up/down of the piecewise-linear model against the binned
 * experiment (src/min_saxs.c:261-319). */
double sxs_best_scale(struct sxs_profile *p, struct sxs_opt_params *params, double c1, double c2)
{
	const double *q = p->qvals, *a = params->a;
	double corr = -params->mult * (c1 * c1 - 1.0);
	double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
	double in_prev = model_in(p, 0, G, c2);
	double c1c = c1 * c1 * c1, q_prev = -1.0, up = 0.0, down = 0.0;
	for (int i = 0; i < p->qnum; i++) {
		double qc = q[i];
		G = c1c * exp(corr * qc * qc);
		double in = model_in(p, i, G, c2);
		double tan = (in - in_prev) / (qc - q_prev);
		double buf = in - tan * qc;
		up += buf * a[i * 6 + 1] + tan * a[i * 6 + 2];
		down += buf * buf * a[i * 6 + 3] + 2.0 * tan * buf * a[i * 6 + 4] + tan * tan * a[i * 6 + 5];
		in_prev = in;
		q_prev = qc;
	}
	return up / down;
}

/* chi^2 at (c1, c2) with the best scale (src/min_saxs.c:391-448). */
double point_score(struct sxs_profile *p, struct sxs_opt_params *params, double c1, double c2)
{
	const double *q = p->qvals, *a = params->a;
	double corr = -params->mult * (c1 * c1 - 1.0);
	double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
	double in_prev = model_in(p, 0, G, c2);
	double k = sxs_best_scale(p, params, c1, c2);
	double c1c = c1 * c1 * c1, q_prev = -1.0, score = 0.0;
	for (int i = 0; i < p->qnum; i++) {
		double qc = q[i];
		G = c1c * exp(corr * qc * qc);
		double in = model_in(p, i, G, c2);
		double tan = (in - in_prev) / (qc - q_prev);
		double buf = in - tan * qc;
		score += a[i * 6] + k * (-2.0 * buf * a[i * 6 + 1] - 2.0 * tan * a[i * 6 + 2]
		                         + k * (buf * buf * a[i * 6 + 3] + 2.0 * buf * tan * a[i * 6 + 4] + tan * tan * a[i * 6 + 5]));
		in_prev = in;
		q_prev = qc;
	}
	return score;
}

double sxs_point_score(struct sxs_profile *p, struct sxs_opt_params *params, double c1, double c2)
{
	return point_score(p, params, c1, c2);
}

/* I(q) at (c1, c2) from the cross terms (src/min_saxs.c:321-350). */
void sxs_compile_intensity(struct sxs_profile *p, double rm, double c1, double c2)
{
	const double *q = p->qvals;
	double corr = -g_mult(rm) * (c1 * c1 - 1.0);
	for (int i = 0; i < p->qnum; i++) {
		double G = c1 * c1 * c1 * exp(corr * q[i] * q[i]);
		p->in[i] = model_in(p, i, G, c2);
		p->err[i] = p->rerr * p->in[i];
	}
}

/* Cross terms of a single molecule (src/min_saxs.c:450-505). */
void sxs_spf2cross_terms(struct sxs_profile *p, struct sxs_spf_full *s)
{
	int K2 = (s->L + 1) * (s->L + 1);
	for (int q = 0; q < p->qnum; q++) {
		double vv = 0, vd = 0, vw = 0, dd = 0, dw = 0, ww = 0;
		const double *Vr = s->V[q]->re, *Vi = s->V[q]->im, *Dr = s->D[q]->re, *Di = s->D[q]->im;
		const double *Wr = s->W[q]->re, *Wi = s->W[q]->im;
		for (int i = 0; i < K2; i++) {
			vv += Vr[i] * Vr[i] + Vi[i] * Vi[i];
			dd += Dr[i] * Dr[i] + Di[i] * Di[i];
			ww += Wr[i] * Wr[i] + Wi[i] * Wi[i];
			vd += Vr[i] * Dr[i] + Vi[i] * Di[i];
			vw += Vr[i] * Wr[i] + Vi[i] * Wi[i];
			dw += Dr[i] * Wr[i] + Di[i] * Wi[i];
		}
		p->VV[q] = vv; p->VD[q] = vd * 2.0; p->VW[q] = vw * 2.0;
		p->DD[q] = dd; p->DW[q] = dw * 2.0; p->WW[q] = ww;
	}
}

/* ---------------------------------------------- L-BFGS-B on the GPU */

static int fit_profiles_gpu(struct sxs_profile **profiles, const int *sel, int n, struct sxs_opt_params *params,
                            int rescale)
{
	int rc = sxs_ensure_init();
	if (rc) return rc;
	int Q = profiles[sel[0]]->qnum;
	cudaStream_t s = sxs_default_stream();
	double *h_c = malloc(sizeof(double) * (size_t)n * 6 * Q), *h_o = malloc(sizeof(double) * 4 * n);
	if (!h_c || !h_o) {
		free(h_c); free(h_o);
		return sxs_fail(-5, "out of host memory");
	}
	for (int k = 0; k < n; k++) {
		struct sxs_profile *p = profiles[sel[k]];
		double *dst = h_c + (size_t)k * 6 * Q;
		double sc = 1.0;
		if (rescale) {
			sc = p->VV[0] + p->DD[0] + p->WW[0] + p->VW[0] - p->VD[0] - p->DW[0];
			sc = params->peak / sc;
		}
		const double *src[6] = {p->VV, p->VD, p->VW, p->DD, p->DW, p->WW};
		for (int c = 0; c < 6; c++)
			for (int i = 0; i < Q; i++) dst[c * Q + i] = rescale ? src[c][i] * sc : src[c][i];
	}
	double *d_c = NULL, *d_t = NULL, *d_q = NULL, *d_a = NULL, *d_o = NULL;
	int *d_it = NULL;
	cudaError_t e = cudaMalloc((void **)&d_c, sizeof(double) * (size_t)n * 6 * Q);
	if (!e) e = cudaMalloc((void **)&d_t, sizeof(double) * (size_t)n * 6 * Q);
	if (!e) e = cudaMalloc((void **)&d_q, sizeof(double) * Q);
	if (!e) e = cudaMalloc((void **)&d_a, sizeof(double) * 6 * Q);
	if (!e) e = cudaMalloc((void **)&d_o, sizeof(double) * 4 * n);
	if (!e) e = cudaMalloc((void **)&d_it, sizeof(int) * n);
	if (!e) e = cudaMemcpyAsync(d_c, h_c, sizeof(double) * (size_t)n * 6 * Q, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_q, profiles[sel[0]]->qvals, sizeof(double) * Q, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_a, params->a, sizeof(double) * 6 * Q, cudaMemcpyHostToDevice, s);
	if (!e) {
		e = (cudaError_t)sxs_fit_lbfgsb_launch(d_c, 0, d_t, n, Q, d_q, d_a, params->mult, params->peak, 0, d_o, d_o + n,
		                                       d_o + 2 * n, d_o + 3 * n, d_it, s);
		sxs_count_launches(2);
	}
	if (!e) e = cudaMemcpyAsync(h_o, d_o, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaStreamSynchronize(s);
	cudaFree(d_c); cudaFree(d_t); cudaFree(d_q); cudaFree(d_a); cudaFree(d_o); cudaFree(d_it);
	if (!e) {
		for (int k = 0; k < n; k++) {
			struct sxs_profile *p = profiles[sel[k]];
			double *src = h_c + (size_t)k * 6 * Q;
			double *dst[6] = {p->VV, p->VD, p->VW, p->DD, p->DW, p->WW};
			for (int c = 0; c < 6; c++) memcpy(dst[c], src + c * Q, sizeof(double) * Q);
			p->score = h_o[k];
			p->c1 = h_o[n + k];
			p->c2 = h_o[2 * n + k];
			p->scale = h_o[3 * n + k];
			sxs_compile_intensity(p, params->rm, p->c1, p->c2);
		}
	}
	free(h_c); free(h_o);
	if (e) return sxs_cuda_fail(e, "L-BFGS-B fit");
	return 0;
}

/* src/min_saxs.c:153-194: peak rescale then L-BFGS-B for every masked
 * profile; the fits run as one GPU batch. */
void sxs_fit_params(struct sxs_profile **profiles, struct sxs_opt_params *params, int *mask, int n)
{
	NEED(profiles);
	NEED(params);
	NEED(mask);
	int *sel = XCALLOC(n > 0 ? n : 1, sizeof(int));
	int k = 0;
	for (int i = 0; i < n; i++) if (mask[i] == 1) sel[k++] = i;
	if (k > 0 && fit_profiles_gpu(profiles, sel, k, params, 1)) DIE(sxsg_last_error());
	free(sel);
}

/* src/min_saxs.c:196-259 */
void sxs_lbfgs_fitting(struct sxs_profile *profile, struct sxs_opt_params *params)
{
	NEED(profile);
	NEED(params);
	int sel = 0;
	if (fit_profiles_gpu(&profile, &sel, 1, params, 0)) DIE(sxsg_last_error());
}

/* src/min_saxs.c:507-511 */
void sxs_spf2fitted_profile(struct sxs_profile *p, struct sxs_spf_full *s, struct sxs_opt_params *params)
{
	sxs_spf2cross_terms(p, s);
	sxs_lbfgs_fitting(p, params);
}

/* ===================================================== grids, indices */

/* q grid by cumulative addition (src/saxs_utils.c:50-63). */
double *sxs_mkarray(double begin, double end, int qnum)
{
	if (begin > end || begin < 0 || end < 0) {
		fprintf(stderr, "WRONG Q VALUES WHEN CREATING ARRAY");
		exit(EXIT_FAILURE);
	}
	double step = (end - begin) / (qnum - 1);
	double *q = XCALLOC(qnum, sizeof(double));
	q[0] = begin;
	for (int i = 1; i < qnum; i++) q[i] = q[i - 1] + step;
	return q;
}

/* z-y-z active rotation (src/saxs_utils.c:65-79). */
void sxs_fill_active_rotation_matrix(struct mol_matrix3 *rm, double alpha, double beta, double gamma)
{
	rm->m11 = cos(gamma) * cos(beta) * cos(alpha) - sin(gamma) * sin(alpha);
	rm->m21 = cos(gamma) * cos(beta) * sin(alpha) + sin(gamma) * cos(alpha);
	rm->m31 = -cos(gamma) * sin(beta);
	rm->m12 = -sin(gamma) * cos(beta) * cos(alpha) - cos(gamma) * sin(alpha);
	rm->m22 = -sin(gamma) * cos(beta) * sin(alpha) + cos(gamma) * cos(alpha);
	rm->m32 = sin(gamma) * sin(beta);
	rm->m13 = sin(beta) * cos(alpha);
	rm->m23 = sin(beta) * sin(alpha);
	rm->m33 = cos(beta);
}

/* c = a b (src/saxs_utils.c:81-94). */
void sxs_mult_rot_mats(struct mol_matrix3 *c, struct mol_matrix3 *a, struct mol_matrix3 *b)
{
	struct mol_matrix3 r;
	r.m11 = a->m11 * b->m11 + a->m12 * b->m21 + a->m13 * b->m31;
	r.m12 = a->m11 * b->m12 + a->m12 * b->m22 + a->m13 * b->m32;
	r.m13 = a->m11 * b->m13 + a->m12 * b->m23 + a->m13 * b->m33;
	r.m21 = a->m21 * b->m11 + a->m22 * b->m21 + a->m23 * b->m31;
	r.m22 = a->m21 * b->m12 + a->m22 * b->m22 + a->m23 * b->m32;
	r.m23 = a->m21 * b->m13 + a->m22 * b->m23 + a->m23 * b->m33;
	r.m31 = a->m31 * b->m11 + a->m32 * b->m21 + a->m33 * b->m31;
	r.m32 = a->m31 * b->m12 + a->m32 * b->m22 + a->m33 * b->m32;
	r.m33 = a->m31 * b->m13 + a->m32 * b->m23 + a->m33 * b->m33;
	*c = r;
}

/* src/index.c:3-29 */
size_t sxs_assemble_index(struct sxs_index *id, int nbeta, int L)
{
	int fft = 2 * L + 1;
	return ((((id->z * nbeta + id->b1) * nbeta + id->b2) * fft + id->a2) * fft + id->g1) * fft + id->g2;
}

void sxs_disassemble_index(struct sxs_index *id, size_t index, int nbeta, int L)
{
	size_t fft = 2 * L + 1;
	id->g2 = (int)(index % fft); index /= fft;
	id->g1 = (int)(index % fft); index /= fft;
	id->a2 = (int)(index % fft); index /= fft;
	id->b2 = (int)(index % nbeta); index /= nbeta;
	id->b1 = (int)(index % nbeta);
	id->z = (int)(index / nbeta);
}

static double clamp1(double a) { return a < -1.0 ? -1.0 : (a > 1.0 ? 1.0 : a); }

/* Ligand pose (translation tv of its centre, rotation rm) to
 * (z, beta_rec, gamma_rec, alpha_lig, beta_lig, gamma_lig)
 * (src/index.c:31-75). */
void sxs_ft2euler(struct sxs_euler *eu, struct mol_vector3 *tv, struct mol_matrix3 *rm, struct mol_vector3 *ref)
{
	double vx = tv->X + ref->X, vy = tv->Y + ref->Y, vz = tv->Z + ref->Z;
	double z = round(sqrt(vx * vx + vy * vy + vz * vz));
	double b1 = acos(clamp1(vz / z));
	double g1 = acos(clamp1(-vx / (z * sin(b1))));
	if (vy / (z * sin(b1)) < 0.0) g1 = 2 * SXS_PI - g1;
	struct mol_matrix3 rec, lig;
	sxs_fill_active_rotation_matrix(&rec, 0.0, b1, g1);
	sxs_mult_rot_mats(&lig, &rec, rm);
	double b2 = acos(clamp1(lig.m33));
	double a2 = acos(clamp1(lig.m13 / sin(b2)));
	if (lig.m23 / sin(b2) < 0.0) a2 = 2 * SXS_PI - a2;
	double g2 = acos(clamp1(-lig.m31 / sin(b2)));
	if (lig.m32 / sin(b2) < 0.0) g2 = 2 * SXS_PI - g2;
	eu->z = z; eu->b1 = b1; eu->g1 = g1; eu->a2 = a2; eu->b2 = b2; eu->g2 = g2;
}

/* correlate's grid index of one Euler line (tools/correlate.c:222-240):
 * alpha_lig and gamma_lig are flipped to 2 pi - angle, every angle is
 * rounded to its grid step, with no wrap-around. */
int64_t sxsg_assemble_index_ex(const double *eu, int z_idx, int L, int flags)
{
	int nb = L + 1, N = 2 * L + 1;
	double a2 = 2 * SXS_PI - eu[3];
	double g2 = 2 * SXS_PI - eu[5];
	double bs = SXS_PI / L, as = 2.0 * SXS_PI / (2 * L + 1);
	int da = (int)round(a2 / as), dg1 = (int)round(eu[2] / as), dg2 = (int)round(g2 / as);
	if (flags & SXSG_WRAP_ANGLES) {
		da = ((da % N) + N) % N;
		dg1 = ((dg1 % N) + N) % N;
		dg2 = ((dg2 % N) + N) % N;
	}
	int64_t id = (int64_t)z_idx * nb;
	id = (id + (int)round(eu[1] / bs)) * nb;
	id = (id + (int)round(eu[4] / bs)) * N;
	id = (id + da) * N;
	id = (id + dg1) * N;
	id = id + dg2;
	return id;
}

int64_t sxsg_assemble_index(const double *eu, int z_idx, int L) { return sxsg_assemble_index_ex(eu, z_idx, L, 0); }

double sxs_sbessel(int order, double x) { return sxs_sbessel_host(order, x); }

/* ====================================================== form factors */

/* Zero-angle form factors of the reference's 43 form-factor types, by the
 * index of its enum saxs_ff_type (src/form_factor_table.h:27-37; values
 * src/form_factor_table.c:8-49): zero_ff, vacuum_ff and excluded-volume
 * ("dummy") factor, with the name that the mapping file uses for the type
 * (src/form_factor_table.c:76-107; NULL for types no mapping line can
 * select). */
static const struct { const char *name; double zero, vacuum, dummy; } k_ff[SXS_FF_NTYPES] = {
	{"H", -0.720147, 0.999953, 1.7201},     {"HE", -0.720228, 0.999872, 1.7201},
	{NULL, 1.591, 2.99, 1.399},             {NULL, 2.591, 3.99, 1.399},
	{NULL, 3.591, 4.99, 1.399},             {"C", 0.50824, 5.9992, 5.49096},
	{"N", 6.16294, 6.9946, 0.83166},        {"O", 4.94998, 7.9994, 3.04942},
	{NULL, 7.591, 8.99, 1.399},             {"NE", 6.993, 9.999, 3.006},
	{"SOD+", 7.9864, 10.9924, 3.006},       {"MG2+", 8.9805, 11.9865, 3.006},
	{NULL, 9.984, 12.99, 3.006},            {NULL, 10.984, 13.99, 3.006},
	{"P", 13.0855, 14.9993, 1.91382},       {"S", 9.36656, 15.9998, 6.63324},
	{NULL, 13.984, 16.99, 3.006},           {NULL, 16.591, 17.99, 1.399},
	{"K", 15.984, 18.99, 3.006},            {"CAL2+", 14.9965, 18.0025, 3.006},
	{NULL, 20.984, 23.99, 3.006},           {NULL, 21.984, 24.99, 3.006},
	{"FE2+", 20.9946, 24.0006, 3.006},      {NULL, 23.984, 26.99, 3.006},
	{NULL, 24.984, 27.99, 3.006},           {NULL, 25.984, 28.99, 3.006},
	{"ZN2+", 24.9936, 27.9996, 3.006},      {"SE", 30.9825, 33.99, 3.006},
	{NULL, 31.984, 34.99, 3.006},           {NULL, 49.16, 52.99, 3.83},
	{NULL, 70.35676, 76.99, 6.63324},       {NULL, 71.35676, 77.99, 6.63324},
	{"AU", 72.324, 78.9572, 6.63324},       {NULL, 73.35676, 79.99, 6.63324},
	{"CH", -0.211907, 6.99915, 7.21106},    {"CH2", -0.932054, 7.99911, 8.93116},
	{"CH3", -1.6522, 8.99906, 10.6513},     {"NH", 5.44279, 7.99455, 2.55176},
	{"NH2", 4.72265, 8.99451, 4.27186},     {"NH3", 4.0025, 9.99446, 5.99196},
	{"OH", 4.22983, 8.99935, 4.76952},      {NULL, 3.50968, 9.9993, 6.48962},
	{"SH", 8.64641, 16.9998, 8.35334},
};
/* the hydration-shell weight: zero_ff of OH2 (src/pdb2spf.c:41-43) */
#define SXS_FF_OH2 41

double sxsg_ff_water(void) { return k_ff[SXS_FF_OH2].zero; }

/* type index of a mapping file's type name, SXSG_FF_UNKNOWN for other names
 * (string_to_ff_type compares the name as written: case-sensitive) */
static int ff_type_index(const char *name)
{
	for (int i = 0; i < SXS_FF_NTYPES; i++)
		if (k_ff[i].name && !strcmp(name, k_ff[i].name)) return i;
	return SXSG_FF_UNKNOWN;
}

int sxsg_ff_constants(int type, double *zero_ff, double *vacuum_ff, double *dummy_ff)
{
	if (type < 0 || type >= SXS_FF_NTYPES) return sxs_fail(-2, "sxsg_ff_constants: type %d out of range", type);
	if (zero_ff) *zero_ff = k_ff[type].zero;
	if (vacuum_ff) *vacuum_ff = k_ff[type].vacuum;
	if (dummy_ff) *dummy_ff = k_ff[type].dummy;
	return 0;
}

const char *sxsg_ff_name(int type)
{
	return type >= 0 && type < SXS_FF_NTYPES ? k_ff[type].name : NULL;
}

int sxsg_ff_type(const char *name, double *vac, double *dum)
{
	if (!name) return -1;
	int t = ff_type_index(name);
	if (t == SXSG_FF_UNKNOWN) return -1;
	if (vac) *vac = k_ff[t].vacuum;
	if (dum) *dum = k_ff[t].dummy;
	return 0;
}

/* ------------------------------------------- (residue, atom) -> type map
 * Open-addressing hash of the mapping file's lines; a later line for the
 * same key replaces an earlier one (kh_put then kh_value). */
typedef struct { char res[8], atom[8]; int type; int used; } ff_slot;
struct sxsg_ff_map {
	ff_slot *slot;
	size_t cap, count;
};

static uint64_t ff_hash(const char *res, const char *atom)
{
	uint64_t h = 1469598103934665603ull;
	for (const char *c = res; *c; c++) h = (h ^ (unsigned char)*c) * 1099511628211ull;
	h = (h ^ 0xff) * 1099511628211ull;
	for (const char *c = atom; *c; c++) h = (h ^ (unsigned char)*c) * 1099511628211ull;
	return h;
}

static ff_slot *ff_find(const sxsg_ff_map *m, const char *res, const char *atom)
{
	size_t i = ff_hash(res, atom) & (m->cap - 1);
	while (m->slot[i].used) {
		if (!strcmp(m->slot[i].res, res) && !strcmp(m->slot[i].atom, atom)) return &m->slot[i];
		i = (i + 1) & (m->cap - 1);
	}
	return &m->slot[i];
}

static int ff_put(sxsg_ff_map *m, const char *res, const char *atom, int type)
{
	if (2 * (m->count + 1) > m->cap) {
		size_t oc = m->cap;
		ff_slot *old = m->slot;
		m->cap = oc ? 2 * oc : 256;
		m->slot = calloc(m->cap, sizeof(ff_slot));
		if (!m->slot) return -1;
		for (size_t i = 0; i < oc; i++)
			if (old[i].used) *ff_find(m, old[i].res, old[i].atom) = old[i];
		free(old);
	}
	ff_slot *sl = ff_find(m, res, atom);
	if (!sl->used) {
		sl->used = 1;
		strcpy(sl->res, res);
		strcpy(sl->atom, atom);
		m->count++;
	}
	sl->type = type;
	return 0;
}

sxsg_ff_map *sxsg_ff_map_load(const char *path)
{
	if (!path) {
		sxs_fail(-2, "sxsg_ff_map_load: no path");
		return NULL;
	}
	FILE *f = fopen(path, "r");
	if (!f) {
		sxs_fail(-2, "Could not open file %s", path);
		return NULL;
	}
	sxsg_ff_map *m = calloc(1, sizeof(*m));
	char line[1024];
	int bad = !m;
	/* default_ff_table's loop (src/form_factor_table.c:164-183): skip '#'
	 * and blank lines, read "residue atom type" tokens of at most 7, 7 and
	 * 15 characters into buffers kept across lines (a line with fewer
	 * tokens keeps the previous line's remaining fields, as there) */
	char r[8] = {0}, a[8] = {0}, t[16] = {0};
	while (!bad && fgets(line, sizeof(line), f)) {
		int blank = 1;
		for (char *c = line; *c; c++)
			if (!isspace((unsigned char)*c)) {
				blank = 0;
				break;
			}
		if (line[0] == '#' || blank) continue;
		if (sscanf(line, "%7s %7s %15s", r, a, t) < 1) continue;
		bad = ff_put(m, r, a, ff_type_index(t)) != 0;
	}
	fclose(f);
	if (bad) {
		sxsg_ff_map_free(m);
		sxs_fail(-5, "sxsg_ff_map_load: out of host memory");
		return NULL;
	}
	return m;
}

void sxsg_ff_map_free(sxsg_ff_map *m)
{
	if (!m) return;
	free(m->slot);
	free(m);
}

/* get_ff's key (src/form_factor_table.c:98-121): skip leading blanks, copy
 * up to the next blank, at most 7 characters */
static void trim_token(const char *src, char *dst)
{
	int n = 0;
	while (*src == ' ') src++;
	while (*src && *src != ' ' && n < 7) dst[n++] = *src++;
	dst[n] = 0;
}

int sxsg_ff_map_type(const sxsg_ff_map *m, const char *res, const char *atom)
{
	if (!m || !res || !atom) return -1;
	char r[8], a[8];
	trim_token(res, r);
	trim_token(atom, a);
	if (!m->cap) return -1;
	const ff_slot *sl = ff_find(m, r, a);
	return sl->used ? sl->type : -1;
}

int sxsg_ff_lookup(const char *path, const char *res8, const char *atom8, int n, double *vac, double *dum)
{
	if (!path || n < 0 || (n > 0 && (!res8 || !atom8 || !vac || !dum))) return sxs_fail(-2, "sxsg_ff_lookup: bad arguments");
	sxsg_ff_map *m = sxsg_ff_map_load(path);
	if (!m) return -2;
	int missing = 0;
	for (int i = 0; i < n; i++) {
		char rs[9], as[9];
		memcpy(rs, res8 + 8 * i, 8); rs[8] = 0;
		memcpy(as, atom8 + 8 * i, 8); as[8] = 0;
		int type = sxsg_ff_map_type(m, rs, as);
		if (type < 0 || type >= SXS_FF_NTYPES) {
			vac[i] = dum[i] = NAN;
			missing++;
		} else {
			vac[i] = k_ff[type].vacuum;
			dum[i] = k_ff[type].dummy;
		}
	}
	sxsg_ff_map_free(m);
	return missing;
}

/* =================================================== drop-in scoring */

/* src/fftsaxs.c:608-986.  Same inputs, same outputs: per listed pose the
 * L-BFGS-B chi, c1, c2 of the peak-rescaled cross terms.  skip = 1 uses the
 * twiddles of the reference's simple_ft branch, skip = 0 those of its FFTW
 * branch.  Invalid input ends the process like the reference's ERROR_MSG. */
void sxs_compute_saxs_scores(double *scores, double *c1, double *c2, int *index_list, int nout,
                             struct sxs_spf_full *A, struct sxs_spf_full *B, struct sxs_opt_params *params,
                             double *qvals, int qnum, double *zvals, int znum, int L, int skip)
{
	NEED(A); NEED(B); NEED(params); NEED(qvals); NEED(zvals);
	if (nout <= 0) return;
	NEED(scores); NEED(c1); NEED(c2); NEED(index_list);
	if (A->L != L || B->L != L || A->qnum != qnum || B->qnum != qnum) DIE("expansions do not match L / qnum");
	size_t spf_n = (size_t)3 * qnum * (L + 1) * (L + 1) * 2;
	double *fa = XCALLOC(spf_n, sizeof(double)), *fb = XCALLOC(spf_n, sizeof(double));
	sxsg_spf_to_flat(A, fa);
	sxsg_spf_to_flat(B, fb);
	int64_t *idx = XCALLOC(nout > 0 ? nout : 1, sizeof(int64_t));
	for (int i = 0; i < nout; i++) idx[i] = index_list[i];
	sxsg_plan *p = NULL;
	int rc = sxsg_plan_create(&p, fa, fb, qvals, qnum, zvals, znum, L, params->a, params->mult, params->peak, NULL, 0,
	                          NULL, 0, SXSG_FP64);
	if (!rc) rc = sxsg_plan_set_poses(p, idx, nout, skip);
	if (!rc) rc = sxsg_plan_run(p, SXSG_FIT_LBFGSB);
	if (!rc) rc = sxsg_plan_results(p, scores, c1, c2, NULL, NULL, NULL);
	sxsg_plan_destroy(p);
	free(fa); free(fb); free(idx);
	if (rc) DIE(sxsg_last_error());
}

int64_t sxsg_poses_to_indices(const double *rot, const double *tr, int64_t n, const double *ref, const double *zvals,
                              int znum, int L, int64_t *index, uint8_t *keep)
{
	return sxsg_poses_to_indices_ex(rot, tr, n, ref, zvals, znum, L, index, keep, 0);
}

/* one pose the host way: ft2euler, the "% .3f" round trip, z slot, index;
 * returns 1 if kept */
static int ingest_one(const double *rot9, const double *tr3, const double *ref, const double *zvals, int znum, int L,
                      int flags, int64_t *index)
{
	char buf[64];
	struct mol_vector3 t = {tr3[0], tr3[1], tr3[2]}, r = {ref[0], ref[1], ref[2]};
	const double *m = rot9;
	struct mol_matrix3 mm = {m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]};
	struct sxs_euler e;
	sxs_ft2euler(&e, &t, &mm, &r);
	double v[6] = {e.z, e.b1, e.g1, e.a2, e.b2, e.g2};
	for (int k = 0; k < 6; k++) {
		snprintf(buf, sizeof(buf), "% .3f", v[k]);
		v[k] = strtod(buf, NULL);
	}
	int zi = -1;
	for (int j = 0; j < znum; j++)
		if (zvals[j] > v[0] - 0.001 && zvals[j] < v[0] + 0.001) {
			zi = j;
			break;
		}
	if (zi < 0) {
		*index = -1;
		return 0;
	}
	*index = sxsg_assemble_index_ex(v, zi, L, flags);
	return 1;
}

int64_t sxsg_poses_to_indices_ex(const double *rot, const double *tr, int64_t n, const double *ref,
                                 const double *zvals, int znum, int L, int64_t *index, uint8_t *keep, int flags)
{
	if (n < 0 || (n > 0 && (!rot || !tr || !ref || !zvals || !index || !keep)) || L < 1)
		return sxs_fail(-2, "sxsg_poses_to_indices: bad arguments");
	int64_t kept = 0;
	for (int64_t i = 0; i < n; i++) {
		keep[i] = (uint8_t)ingest_one(rot + 9 * i, tr + 3 * i, ref, zvals, znum, L, flags, index + i);
		kept += keep[i];
	}
	return kept;
}

/* Device batches of at most this many poses (about 120 MB of device memory) */
#define SXS_INGEST_BATCH ((int64_t)1 << 20)

int64_t sxsg_poses_to_indices_gpu(const double *rot, const double *tr, int64_t n, const double *ref,
                                  const double *zvals, int znum, int L, int64_t *index, uint8_t *keep, int flags,
                                  int64_t *host_poses)
{
	if (n < 0 || (n > 0 && (!rot || !tr || !ref || !zvals || !index || !keep)) || L < 1 || znum < 0)
		return sxs_fail(-2, "sxsg_poses_to_indices_gpu: bad arguments");
	if (host_poses) *host_poses = 0;
	if (n == 0) return 0;
	int rc = sxs_ensure_init();
	if (rc) return rc;
	cudaStream_t s = sxs_default_stream();
	int64_t nb = n < SXS_INGEST_BATCH ? n : SXS_INGEST_BATCH;
	double *d_rot = NULL, *d_tr = NULL, *d_z = NULL;
	long long *d_idx = NULL, *d_fl = NULL;
	unsigned char *d_keep = NULL;
	unsigned int *d_nf = NULL;
	long long *h_fl = malloc(sizeof(long long) * (size_t)nb);
	cudaError_t e = h_fl ? cudaSuccess : cudaErrorMemoryAllocation;
	if (!e) e = cudaMallocAsync((void **)&d_rot, sizeof(double) * 9 * nb, s);
	if (!e) e = cudaMallocAsync((void **)&d_tr, sizeof(double) * 3 * nb, s);
	if (!e) e = cudaMallocAsync((void **)&d_z, sizeof(double) * (znum > 0 ? znum : 1), s);
	if (!e) e = cudaMallocAsync((void **)&d_idx, sizeof(long long) * nb, s);
	if (!e) e = cudaMallocAsync((void **)&d_fl, sizeof(long long) * nb, s);
	if (!e) e = cudaMallocAsync((void **)&d_keep, nb, s);
	if (!e) e = cudaMallocAsync((void **)&d_nf, sizeof(unsigned int), s);
	if (!e && znum > 0) e = cudaMemcpyAsync(d_z, zvals, sizeof(double) * znum, cudaMemcpyHostToDevice, s);
	int64_t kept = 0, nhost = 0;
	for (int64_t b0 = 0; !e && b0 < n; b0 += nb) {
		int64_t m = n - b0 < nb ? n - b0 : nb;
		unsigned int nf = 0;
		e = cudaMemcpyAsync(d_rot, rot + 9 * b0, sizeof(double) * 9 * m, cudaMemcpyHostToDevice, s);
		if (!e) e = cudaMemcpyAsync(d_tr, tr + 3 * b0, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, s);
		if (!e) e = cudaMemsetAsync(d_nf, 0, sizeof(unsigned int), s);
		if (!e) {
			e = (cudaError_t)sxsk_pose_ingest(d_rot, d_tr, (long)m, ref, d_z, znum, L, (flags & SXSG_WRAP_ANGLES) != 0,
			                                  d_idx, d_keep, d_nf, d_fl, s);
			sxs_count_launches(1);
		}
		if (!e) e = cudaMemcpyAsync(index + b0, d_idx, sizeof(int64_t) * m, cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaMemcpyAsync(keep + b0, d_keep, m, cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaMemcpyAsync(&nf, d_nf, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaStreamSynchronize(s);
		if (!e && nf > 0) e = cudaMemcpy(h_fl, d_fl, sizeof(long long) * nf, cudaMemcpyDeviceToHost);
		if (e) break;
		/* flagged poses: the host path decides (see kernels_ingest.cu) */
		for (unsigned int k = 0; k < nf; k++) {
			int64_t i = b0 + h_fl[k];
			keep[i] = (uint8_t)ingest_one(rot + 9 * i, tr + 3 * i, ref, zvals, znum, L, flags, index + i);
		}
		nhost += nf;
		for (int64_t i = b0; i < b0 + m; i++) kept += keep[i];
	}
	cudaFreeAsync(d_rot, s); cudaFreeAsync(d_tr, s); cudaFreeAsync(d_z, s); cudaFreeAsync(d_idx, s);
	cudaFreeAsync(d_fl, s); cudaFreeAsync(d_keep, s); cudaFreeAsync(d_nf, s);
	free(h_fl);
	if (e) return sxs_cuda_fail(e, "sxsg_poses_to_indices_gpu");
	if (host_poses) *host_poses = nhost;
	return kept;
}

int sxsg_profile_from_flat(const double *spf, int L, int qnum, double rm, const double *q, double c1, double c2,
                           double *in, double *err)
{
	if (!spf || L < 0 || qnum <= 0 || !q || !in || !err) return sxs_fail(-2, "sxsg_profile_from_flat: bad arguments");
	struct sxs_spf_full *s = sxs_spf_full_create(L, qnum);
	sxsg_spf_from_flat(s, spf);
	s->rm = rm;
	struct sxs_profile *p = sxs_profile_create((double *)q, qnum, 0);
	sxs_profile_from_spf(p, s, c1, c2);
	memcpy(in, p->in, sizeof(double) * qnum);
	memcpy(err, p->err, sizeof(double) * qnum);
	sxs_profile_free(p);
	sxs_spf_full_free(s);
	return 0;
}
