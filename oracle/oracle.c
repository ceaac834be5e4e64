/*
 * CPU oracle for the libfmftsaxs FFT-correlation scoring path.
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker, never the product.
 *
 * Build: oracle/bind.py, build_oracle() (gcc -std=c11 -O2 -ffp-contract=off).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "shim/quad.h"

static inline int lm_idx(int l, int m) { return l * (l + 1) + m; }
static inline int d_idx(int L, int l, int m, int m1) { return (2 * L + 1) * ((2 * L + 1) * l + (L + m)) + (L + m1); }
static inline int iabs(int a) { return a < 0 ? -a : a; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* ------------------------------------------------------------------------
 * Spherical Bessel j_l(x) by the reference's truncated power series
 * (src/sfbessel.c:21-60): term_0 = 1/(2l+1)!!, term_k = term_{k-1} *
 * (-x^2) / (2k (2k+2l+1)), stop once |term/sum| <= 1e-5, times x^l.
 * j_0(0) = 1, j_l(0) = 0.
 * ---------------------------------------------------------------------- */
static double odd_factorial(int n)
{
	double r = 1.0;
	for (int i = 1; i <= n; i += 2) r *= (double)i;
	return r;
}

double orc_sbessel(int l, double x)
{
	if (x > 0.0) {
		double tl1 = 2.0 * (double)l + 1.0;
		double term = 1.0 / odd_factorial((int)tl1);
		double sum = term;
		for (int k = 1; fabs(term / sum) > 0.00001; k++) {
			double ratio = ((-1.0) * x * x) / ((2.0 * (double)k) * (2.0 * (double)k + tl1));
			term = term * ratio;
			sum = sum + term;
		}
		return sum * pow(x, l);
	}
	return l == 0 ? 1.0 : 0.0;
}

/* q grid by cumulative addition (src/saxs_utils.c:50-63). */
void orc_mkarray(double begin, double end, int n, double *out)
{
	double step = (end - begin) / (n - 1);
	out[0] = begin;
	for (int i = 1; i < n; i++) out[i] = out[i - 1] + step;
}

/* ------------------------------------------------------------------------
 * Wigner small-d d^l_{m m1}(beta) for l <= L (src/borrowed.c:243-313):
 * closed forms for l <= 1, the Kostelec-Rockmore eq. 26 edge products for
 * |m| = l or |m1| = l, and the eq. 28 three-term recurrence in l inside.
 * Written in the reference's store order so overlapping edge cells end with
 * the same value.
 * ---------------------------------------------------------------------- */
void orc_wigner_d(int L, double beta, double *d)
{
	size_t n = (size_t)(L + 1) * (2 * L + 1) * (2 * L + 1);
	memset(d, 0, n * sizeof(double));
	d[d_idx(L, 0, 0, 0)] = 1.0;
	if (L >= 1) {
		double c = cos(beta), s = sin(beta), r2 = sqrt(2.0);
		d[d_idx(L, 1, -1, -1)] = 1.0 * (1.0 + c) / 2.0;
		d[d_idx(L, 1, -1, 0)] = 1.0 * s / r2;
		d[d_idx(L, 1, -1, 1)] = 1.0 * (1.0 - c) / 2.0;
		d[d_idx(L, 1, 0, -1)] = -1.0 * s / r2;
		d[d_idx(L, 1, 0, 0)] = 1.0 * c;
		d[d_idx(L, 1, 0, 1)] = 1.0 * s / r2;
		d[d_idx(L, 1, 1, -1)] = 1.0 * (1.0 - c) / 2.0;
		d[d_idx(L, 1, 1, 0)] = -1.0 * s / r2;
		d[d_idx(L, 1, 1, 1)] = 1.0 * (1.0 + c) / 2.0;
	}
	for (int l = 2; l <= L; l++) {
		for (int m = -l; m <= l; m++) {
			double e1 = 1.0, e2 = 1.0, e3 = 1.0, e4 = 1.0;
			for (int k = 1; k <= 2 * l; k++) {
				double den = ((k <= l + m) ? (double)k : 1.0) * ((k <= l - m) ? (double)k : 1.0);
				double f = sqrt(k / den);
				double ch = cos(beta / 2.0), sh = sin(beta / 2.0);
				e1 *= f * ((k <= l + m) ? ch : 1.0) * ((k <= l - m) ? -sh : 1.0);
				e2 *= f * ((k <= l - m) ? ch : 1.0) * ((k <= l + m) ? sh : 1.0);
				e3 *= f * ((k <= l + m) ? ch : 1.0) * ((k <= l - m) ? sh : 1.0);
				e4 *= f * ((k <= l - m) ? ch : 1.0) * ((k <= l + m) ? -sh : 1.0);
			}
			d[d_idx(L, l, l, m)] = e1;
			d[d_idx(L, l, -l, m)] = e2;
			d[d_idx(L, l, m, l)] = e3;
			d[d_idx(L, l, m, -l)] = e4;
			for (int m1 = -l; m1 <= l; m1++) {
				if (!(m1 > -l && m1 < l && m > -l && m < l)) continue;
				int j = l - 1;
				double v = 1.0;
				v *= (j + 1) * (2.0 * j + 1) / sqrt((double)(((j + 1) * (j + 1) - m * m) * ((j + 1) * (j + 1) - m1 * m1)));
				v *= (cos(beta) - (double)(m * m1) / (double)(j * (j + 1))) * d[d_idx(L, j, m, m1)];
				double w = -1.0;
				w *= sqrt((double)((j * j - m * m) * (j * j - m1 * m1)));
				w *= (double)(j + 1.0) * d[d_idx(L, j - 1, m, m1)] / (double)j;
				w /= sqrt(((j + 1.0) * (j + 1.0) - (double)(m * m)) * ((j + 1.0) * (j + 1.0) - (double)(m1 * m1)));
				v += w;
				d[d_idx(L, l, m, m1)] = v;
			}
		}
	}
}

/* ------------------------------------------------------------------------
 * Wigner 3j by the Racah sum (src/borrowed.c:73-222), carried in binary128
 * in the reference's product order, rounded to double towards zero (the
 * rounding of GMP's mpf_get_d).
 * ---------------------------------------------------------------------- */
static sxs_quad *quad_factorials(int n)
{
	sxs_quad *f = malloc(sizeof(sxs_quad) * (n + 1));
	f[0] = 1;
	for (int i = 1; i <= n; i++) f[i] = f[i - 1] * (sxs_quad)i;
	return f;
}

static double w3j_q(int j1, int j2, int j3, int m1, int m2, int m3, const sxs_quad *f)
{
	int t1 = j2 - m1 - j3, t2 = j1 + m2 - j3, t3 = j1 + j2 - j3, t4 = j1 - m1, t5 = j2 + m2;
	int tmin = imax(0, imax(t1, t2)), tmax = imin(t3, imin(t4, t5));
	sxs_quad acc = 0;
	for (int t = tmin; t <= tmax; t++) {
		sxs_quad one = (t % 2 == 0) ? 1 : -1;
		sxs_quad b = f[t4 - t] * f[t5 - t];
		b = f[t3 - t] * b;
		b = f[t - t2] * b;
		b = f[t - t1] * b;
		b = f[t] * b;
		b = one / b;
		acc = acc + b;
	}
	sxs_quad one = ((j1 - j2 - m3) % 2 == 0) ? 1 : -1;
	sxs_quad b = f[j3 + m3] * f[j3 - m3];
	b = f[j2 - m2] * b;
	b = f[j2 + m2] * b;
	b = f[j1 - m1] * b;
	b = f[j1 + m1] * b;
	b = b / f[j1 + j2 + j3 + 1];
	b = f[-j1 + j2 + j3] * b;
	b = f[j1 - j2 + j3] * b;
	b = f[j1 + j2 - j3] * b;
	b = sxs_quad_sqrt(b);
	b = one * b;
	acc = acc * b;
	return sxs_quad_to_double_trunc(acc);
}

double orc_w3j(int j1, int j2, int j3, int m1, int m2, int m3)
{
	sxs_quad *f = quad_factorials(j1 + j2 + j3 + 1);
	double v = w3j_q(j1, j2, j3, m1, m2, m3, f);
	free(f);
	return v;
}

/* d_lm(l1,p) = (2p+1) sqrt((2l+1)(2l1+1)) 3j(l p l1;0 0 0) 3j(l p l1;-m 0 m)
 * (src/fftsaxs.c:138-174). */
void orc_dsymb(int L, double *ds)
{
	size_t n = (size_t)(L + 1) * (L + 1) * (L + 1) * (2 * L + 1);
	memset(ds, 0, n * sizeof(double));
	sxs_quad *f = quad_factorials(4 * L + 1);
	for (int l = 0; l <= L; l++) {
		double k1 = 2 * l + 1;
		for (int l1 = 0; l1 <= L; l1++) {
			double k2 = sqrt((2 * l1 + 1) * k1);
			for (int p = iabs(l - l1); p <= l + l1; p++) {
				double k3 = (2 * p + 1) * k2 * w3j_q(l, p, l1, 0, 0, 0, f);
				for (int m = -imin(l, l1); m <= imin(l, l1); m++) {
					double k4 = w3j_q(l, p, l1, -m, 0, m, f);
					ds[((size_t)lm_idx(l, m) * (L + 1) + l1) * (2 * L + 1) + p] = k3 * k4;
				}
			}
		}
	}
	free(f);
}

/* j_p(q z) for p in [0, 2L] (src/fftsaxs.c:110-121). */
void orc_besselj_n(double z, const double *q, int qnum, int L, double *bes)
{
	for (int iq = 0; iq < qnum; iq++)
		for (int p = 0; p < 2 * L + 1; p++)
			bes[iq * (2 * L + 1) + p] = orc_sbessel(p, z * q[iq]);
}

/* T^{|m|}_{l l1}(qz) = sum_p (-1)^m i^p j_p(qz) d_lm(l1,p), stored [q][|m|][l][l1]
 * and symmetric in (l, l1) (src/fftsaxs.c:182-243). */
void orc_t_matrix(int L, int qnum, const double *bes, const double *ds, double *tre, double *tim)
{
	static const double ipr[4] = {1.0, 0.0, -1.0, 0.0};
	static const double ipi[4] = {0.0, 1.0, 0.0, -1.0};
	int K = L + 1, N = 2 * L + 1;
	for (int iq = 0; iq < qnum; iq++) {
		for (int m = 0; m <= L; m++) {
			double sgn = (m % 2 == 0) ? 1.0 : -1.0;
			for (int l = m; l <= L; l++) {
				for (int l1 = l; l1 <= L; l1++) {
					double re = 0.0, im = 0.0;
					const double *dp = ds + ((size_t)lm_idx(l, m) * K + l1) * N;
					for (int p = iabs(l - l1); p <= l + l1; p++) {
						double v = sgn * dp[p] * bes[iq * N + p];
						re += ipr[p % 4] * v;
						im += ipi[p % 4] * v;
					}
					size_t a = (((size_t)iq * K + m) * K + l) * K + l1;
					size_t b = (((size_t)iq * K + m) * K + l1) * K + l;
					tre[a] = re; tim[a] = im;
					tre[b] = re; tim[b] = im;
				}
			}
		}
	}
}

double orc_average_radius(const double *vdw, int n)
{
	double s = 0.0;
	for (int i = 0; i < n; i++) s += vdw[i];
	return s / n;
}

/* ------------------------------------------------------------------------
 * A_lm expansion (src/pdb2spf.c:9-22, 24-152; Y norm and Legendre recurrence
 * src/borrowed.c:19-65 with N = L+1):
 *   A^{V,D,W}_lm(q) = 4 pi i^l sum_atoms f j_l(q r) norm_lm P_l^|m|(cos th) e^{-i m phi}
 * with f = vacuum_ff, dummy_ff, or h2o_ff * sasa (sasa == NULL gives W = 0).
 * ---------------------------------------------------------------------- */
static inline int LMi(int N, int l, int m) { return N * (m + N - 1) + l; }

static void y_norm(int N, double *Y)
{
	for (int l = 0; l < N; l++) {
		double fact = 1.;
		double tmp0 = (2 * l + 1.) / (4. * ORC_PI);
		for (int m = 0; m <= l; m++) {
			if (m > 0) fact *= (l - m + 1) * (l + m);
			double tmp = sqrt(tmp0 / fact);
			double sgn = (m % 2 == 0) ? 1 : -1;
			Y[LMi(N, l, m)] = tmp;
			Y[LMi(N, l, -m)] = sgn * tmp;
		}
	}
}

static void legendre(int N, double x, double *P)
{
	double y = sqrt(1. - x * x);
	P[LMi(N, 0, 0)] = 1;
	if (N == 1) return;
	P[LMi(N, 1, 0)] = x;
	for (int l = 2; l < N; l++)
		P[LMi(N, l, 0)] = (2. * l - 1.) / l * x * P[LMi(N, l - 1, 0)] - (l - 1.) / l * P[LMi(N, l - 2, 0)];
	for (int m = 1; m < N - 1; m++) {
		P[LMi(N, m, m)] = -1. * (2. * m - 1.) * y * P[LMi(N, m - 1, m - 1)];
		P[LMi(N, m + 1, m)] = (2. * m + 1.) * x * P[LMi(N, m, m)];
		for (int l = m + 2; l < N; l++)
			P[LMi(N, l, m)] = (2. * l - 1.) / (l - m) * x * P[LMi(N, l - 1, m)] - (l + m - 1.) / (l - m) * P[LMi(N, l - 2, m)];
	}
	P[LMi(N, N - 1, N - 1)] = -1. * (2. * (N - 1.) - 1.) * y * P[LMi(N, N - 2, N - 2)];
}

void orc_expand(const double *xyz, const double *vac_ff, const double *dum_ff, const double *sasa,
                double h2o_ff, int natoms, const double *q, int qnum, int L, double *spf)
{
	int N = L + 1, K2 = (L + 1) * (L + 1);
	size_t chs = (size_t)qnum * K2 * 2;
	memset(spf, 0, 3 * chs * sizeof(double));
	double *Y = calloc(N * (2 * N - 1), sizeof(double));
	double *P = calloc(N * (2 * N - 1), sizeof(double));
	double *hre = calloc(K2, sizeof(double)), *him = calloc(K2, sizeof(double));
	y_norm(N, Y);
	for (int a = 0; a < natoms; a++) {
		double x = xyz[3 * a], y = xyz[3 * a + 1], z = xyz[3 * a + 2];
		double r = sqrt(x * x + y * y + z * z);
		double th = acos(z / r);
		double ph = (y > 0.0) ? acos(x / sqrt(x * x + y * y)) : -acos(x / sqrt(x * x + y * y)) + 2.0 * ORC_PI;
		memset(P, 0, N * (2 * N - 1) * sizeof(double));
		legendre(N, cos(th), P);
		double w = sasa ? h2o_ff * sasa[a] : 0.0;
		for (int l = 0; l <= L; l++)
			for (int m = -l; m <= l; m++) {
				double h = Y[LMi(N, l, m)] * P[LMi(N, l, iabs(m))];
				hre[lm_idx(l, m)] = h * cos(ph * m);
				him[lm_idx(l, m)] = h * sin(-ph * m);
			}
		for (int iq = 0; iq < qnum; iq++) {
			double *V = spf + (size_t)iq * K2 * 2;
			double *D = V + chs, *W = V + 2 * chs;
			for (int l = 0; l <= L; l++) {
				double b = orc_sbessel(l, q[iq] * r);
				for (int m = -l; m <= l; m++) {
					int i = lm_idx(l, m);
					double vr = b * hre[i], vi = b * him[i];
					V[2 * i] += vac_ff[a] * vr; V[2 * i + 1] += vac_ff[a] * vi;
					D[2 * i] += dum_ff[a] * vr; D[2 * i + 1] += dum_ff[a] * vi;
					W[2 * i] += w * vr;         W[2 * i + 1] += w * vi;
				}
			}
		}
	}
	double fp = 4.0 * ORC_PI;
	double cre[4] = {fp, 0.0, -fp, 0.0}, cim[4] = {0.0, fp, 0.0, -fp};
	for (int ch = 0; ch < 3; ch++)
		for (int iq = 0; iq < qnum; iq++) {
			double *A = spf + ch * chs + (size_t)iq * K2 * 2;
			for (int l = 0; l <= L; l++)
				for (int m = -l; m <= l; m++) {
					int i = lm_idx(l, m);
					double re = A[2 * i], im = A[2 * i + 1];
					A[2 * i] = cre[l % 4] * re - cim[l % 4] * im;
					A[2 * i + 1] = cre[l % 4] * im + cim[l % 4] * re;
				}
		}
	free(Y); free(P); free(hre); free(him);
}

/* ------------------------------------------------------------------------
 * Fit helpers (src/min_saxs.c).
 * ---------------------------------------------------------------------- */
/* scoring_helper + sxs_opt_params_init (min_saxs.c:116-124, 353-389).  The
 * reference does not bound j (it reads past the last experimental point);
 * this restatement stops at ne. */
void orc_opt_params(const double *eq, const double *ei, const double *ee, int ne,
                    const double *q, int qnum, double rm, double *a, double *mult, double *peak)
{
	memset(a, 0, sizeof(double) * 6 * qnum);
	int j = 0;
	for (int i = 0; i < qnum; i++) {
		double lo = i > 0 ? q[i - 1] : q[0], hi = q[i];
		while (j < ne && eq[j] >= lo && eq[j] <= hi) {
			double e2 = ee[j] * ee[j];
			a[i * 6 + 0] += ei[j] * ei[j] / e2;
			a[i * 6 + 1] += ei[j] / e2;
			a[i * 6 + 2] += eq[j] * ei[j] / e2;
			a[i * 6 + 3] += 1.0 / e2;
			a[i * 6 + 4] += eq[j] / e2;
			a[i * 6 + 5] += eq[j] * eq[j] / e2;
			j++;
		}
	}
	double norm = (double)j;
	for (int i = 0; i < 6 * qnum; i++) a[i] /= norm;
	*mult = pow(4.0 * ORC_PI / 3.0, 1.5) * rm * rm / (16.0 * ORC_PI);
	*peak = ei[0];
}

#define XVV(c, i) (c)[(i)]
static inline double model_in(const double *c, int qnum, int i, double G, double c2)
{
	return c[i] - G * c[qnum + i] + c2 * c[2 * qnum + i] + G * G * c[3 * qnum + i] - G * c2 * c[4 * qnum + i] + c2 * c2 * c[5 * qnum + i];
}

/* sxs_best_scale (min_saxs.c:261-319). */
double orc_best_scale(const double *cr, const double *q, int qnum, const double *a, double mult, double c1, double c2)
{
	double corr = -mult * (c1 * c1 - 1.0);
	double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
	double in_prev = model_in(cr, qnum, 0, G, c2);
	double c1c = c1 * c1 * c1;
	double q_prev = -1.0, up = 0.0, down = 0.0;
	for (int i = 0; i < qnum; i++) {
		double qc = q[i];
		G = c1c * exp(corr * qc * qc);
		double in = model_in(cr, qnum, i, G, c2);
		double tan = (in - in_prev) / (qc - q_prev);
		double buf = in - tan * qc;
		up += buf * a[i * 6 + 1] + tan * a[i * 6 + 2];
		down += buf * buf * a[i * 6 + 3] + 2.0 * tan * buf * a[i * 6 + 4] + tan * tan * a[i * 6 + 5];
		in_prev = in;
		q_prev = qc;
	}
	return up / down;
}

/* point_score (min_saxs.c:391-448): chi^2 at (c1, c2) with the best scale. */
double orc_point_score(const double *cr, const double *q, int qnum, const double *a, double mult, double c1, double c2)
{
	double corr = -mult * (c1 * c1 - 1.0);
	double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
	double in_prev = model_in(cr, qnum, 0, G, c2);
	double k = orc_best_scale(cr, q, qnum, a, mult, c1, c2);
	double c1c = c1 * c1 * c1;
	double q_prev = -1.0, score = 0.0;
	for (int i = 0; i < qnum; i++) {
		double qc = q[i];
		G = c1c * exp(corr * qc * qc);
		double in = model_in(cr, qnum, i, G, c2);
		double tan = (in - in_prev) / (qc - q_prev);
		double buf = in - tan * qc;
		score += a[i * 6] + k * (-2.0 * buf * a[i * 6 + 1] - 2.0 * tan * a[i * 6 + 2]
		                         + k * (buf * buf * a[i * 6 + 3] + 2.0 * buf * tan * a[i * 6 + 4] + tan * tan * a[i * 6 + 5]));
		in_prev = in;
		q_prev = qc;
	}
	return score;
}

/* Peak rescale applied before every fit (min_saxs.c:170-188). */
void orc_rescale(double *c, int qnum, double peak)
{
	double s = c[0] + c[3 * qnum] + c[5 * qnum] + c[2 * qnum] - c[qnum] - c[4 * qnum];
	s = peak / s;
	for (int i = 0; i < qnum; i++) {
		c[i] *= s;             /* VV */
		c[3 * qnum + i] *= s;  /* DD */
		c[5 * qnum + i] *= s;  /* WW */
		c[2 * qnum + i] *= s;  /* VW */
		c[qnum + i] *= s;      /* VD */
		c[4 * qnum + i] *= s;  /* DW */
	}
}

/* sxs_compile_intensity (min_saxs.c:321-350). */
void orc_compile_intensity(const double *cr, const double *q, int qnum, double rm, double rerr,
                           double c1, double c2, double *in, double *err)
{
	double mult = pow(4.0 * ORC_PI / 3.0, 3.0 / 2.0) * rm * rm / (16.0 * ORC_PI);
	double corr = -mult * (c1 * c1 - 1.0);
	for (int i = 0; i < qnum; i++) {
		double G = c1 * c1 * c1 * exp(corr * q[i] * q[i]);
		in[i] = model_in(cr, qnum, i, G, c2);
		err[i] = rerr * in[i];
	}
}

/* sxs_profile_from_spf (profile.c:186-233), including its use of q[0] in G
 * for every q. */
void orc_profile_from_spf(const double *spf, int L, int qnum, double rm, const double *q,
                          double c1, double c2, double *in, double *err)
{
	int K2 = (L + 1) * (L + 1);
	size_t chs = (size_t)qnum * K2 * 2;
	double mult = pow(4.0 * ORC_PI / 3.0, 3.0 / 2.0) * rm * rm / (16.0 * ORC_PI);
	double corr = -mult * (c1 * c1 - 1.0);
	for (int iq = 0; iq < qnum; iq++) {
		const double *V = spf + (size_t)iq * K2 * 2, *D = V + chs, *W = V + 2 * chs;
		double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
		double s = 0.0;
		for (int i = 0; i < K2; i++) {
			double ar = V[2 * i] - G * D[2 * i] + c2 * W[2 * i];
			double ai = V[2 * i + 1] - G * D[2 * i + 1] + c2 * W[2 * i + 1];
			s += ar * ar + ai * ai;
		}
		in[iq] = s;
		err[iq] = s * 0.05;
	}
}

/* sxs_spf2cross_terms (min_saxs.c:450-505). */
void orc_spf2cross_terms(const double *spf, int L, int qnum, double *c)
{
	int K2 = (L + 1) * (L + 1);
	size_t chs = (size_t)qnum * K2 * 2;
	for (int iq = 0; iq < qnum; iq++) {
		const double *V = spf + (size_t)iq * K2 * 2, *D = V + chs, *W = V + 2 * chs;
		double vv = 0, vd = 0, vw = 0, dd = 0, dw = 0, ww = 0;
		for (int i = 0; i < K2; i++) {
			vv += V[2 * i] * V[2 * i] + V[2 * i + 1] * V[2 * i + 1];
			dd += D[2 * i] * D[2 * i] + D[2 * i + 1] * D[2 * i + 1];
			ww += W[2 * i] * W[2 * i] + W[2 * i + 1] * W[2 * i + 1];
			vd += V[2 * i] * D[2 * i] + V[2 * i + 1] * D[2 * i + 1];
			vw += V[2 * i] * W[2 * i] + V[2 * i + 1] * W[2 * i + 1];
			dw += D[2 * i] * W[2 * i] + D[2 * i + 1] * W[2 * i + 1];
		}
		c[iq] = vv; c[qnum + iq] = vd * 2.0; c[2 * qnum + iq] = vw * 2.0;
		c[3 * qnum + iq] = dd; c[4 * qnum + iq] = dw * 2.0; c[5 * qnum + iq] = ww;
	}
}

/* ------------------------------------------------------------------------
 * Pose conversion: sxs_ft2euler (index.c:31-75, rotation helpers
 * saxs_utils.c:65-94) and correlate's grid-index assembly
 * (tools/correlate.c:202-240).
 * ---------------------------------------------------------------------- */
static double clamp1(double a) { return a < -1.0 ? -1.0 : (a > 1.0 ? 1.0 : a); }

void orc_ft2euler(const double *tv, const double *m, const double *ref, double *eu)
{
	double vx = tv[0] + ref[0], vy = tv[1] + ref[1], vz = tv[2] + ref[2];
	double z = round(sqrt(vx * vx + vy * vy + vz * vz));
	double b1 = acos(clamp1(vz / z));
	double g1 = acos(clamp1(-vx / (z * sin(b1))));
	if (vy / (z * sin(b1)) < 0.0) g1 = 2 * ORC_PI - g1;
	double a = 0.0, b = b1, g = g1;
	double r[9];
	r[0] = cos(g) * cos(b) * cos(a) - sin(g) * sin(a);
	r[3] = cos(g) * cos(b) * sin(a) + sin(g) * cos(a);
	r[6] = -cos(g) * sin(b);
	r[1] = -sin(g) * cos(b) * cos(a) - cos(g) * sin(a);
	r[4] = -sin(g) * cos(b) * sin(a) + cos(g) * cos(a);
	r[7] = sin(g) * sin(b);
	r[2] = sin(b) * cos(a);
	r[5] = sin(b) * sin(a);
	r[8] = cos(b);
	double c[9];
	for (int i = 0; i < 3; i++)
		for (int j = 0; j < 3; j++)
			c[3 * i + j] = r[3 * i] * m[j] + r[3 * i + 1] * m[3 + j] + r[3 * i + 2] * m[6 + j];
	double b2 = acos(clamp1(c[8]));
	double a2 = acos(clamp1(c[2] / sin(b2)));
	if (c[5] / sin(b2) < 0.0) a2 = 2 * ORC_PI - a2;
	double g2 = acos(clamp1(-c[6] / sin(b2)));
	if (c[7] / sin(b2) < 0.0) g2 = 2 * ORC_PI - g2;
	eu[0] = z; eu[1] = b1; eu[2] = g1; eu[3] = a2; eu[4] = b2; eu[5] = g2;
}

int orc_assemble_index(const double *eu, int z_idx, int L)
{
	int nb = L + 1, N = 2 * L + 1;
	double a2 = 2 * ORC_PI - eu[3];
	double g2 = 2 * ORC_PI - eu[5];
	double bs = ORC_PI / L, as = 2.0 * ORC_PI / (2 * L + 1);
	int id = z_idx * nb;
	id = (id + (int)round(eu[1] / bs)) * nb;
	id = (id + (int)round(eu[4] / bs)) * N;
	id = (id + (int)round(a2 / as)) * N;
	id = (id + (int)round(eu[2] / as)) * N;
	id = id + (int)round(g2 / as);
	return id;
}

/* ------------------------------------------------------------------------
 * The scoring path (src/fftsaxs.c:608-986), evaluated the reference's way:
 * per touched z the translation matrix, per touched (z, beta2) the ligand
 * sums (compute_sum1, 251-333), per touched (z, beta1, beta2) the 6-channel
 * sums over l (compute_sum2, 416-524) for every (m, m1, m2), then the angular
 * DFT at each listed cell.  Triples with < 30 listed poses use simple_ft
 * (529-606): one twiddle table built from the truncated pi, indexed by the
 * wrapped total phase.  Triples with >= 30 poses (and every triple when
 * skip = 0) use the FFTW branch (899-900): an exact DFT, evaluated here at the
 * listed cells with full-precision twiddles.  Cross terms are
 * fill_const + 2 Re F (52-108).  Outputs per listed pose: raw and
 * peak-rescaled cross terms [6][qnum] and the chi^2 grid [n1][n2].
 * ---------------------------------------------------------------------- */
static void const_int(const double *A, const double *B, int ca, int cb, int qnum, int K2, double *out)
{
	size_t chs = (size_t)qnum * K2 * 2;
	for (int iq = 0; iq < qnum; iq++) {
		const double *a1 = A + ca * chs + (size_t)iq * K2 * 2, *a2 = A + cb * chs + (size_t)iq * K2 * 2;
		const double *b1 = B + ca * chs + (size_t)iq * K2 * 2, *b2 = B + cb * chs + (size_t)iq * K2 * 2;
		double s = 0.0;
		for (int i = 0; i < K2; i++) {
			s += a1[2 * i] * a2[2 * i] + a1[2 * i + 1] * a2[2 * i + 1];
			s += b1[2 * i] * b2[2 * i] + b1[2 * i + 1] * b2[2 * i + 1];
		}
		out[iq] = s;
	}
}

/* S^{ch}[q][m+L][m2+L][l] re/im for one beta2 (compute_sum1). */
static void sum1(const double *B, int ch, int qnum, int L, const double *tre, const double *tim,
                 const double *d, double *sre, double *sim)
{
	int K = L + 1, N = 2 * L + 1, K2 = K * K;
	size_t chs = (size_t)qnum * K2 * 2;
	for (int iq = 0; iq < qnum; iq++) {
		const double *Bq = B + ch * chs + (size_t)iq * K2 * 2;
		const double *tr = tre + (size_t)iq * K * K * K, *ti = tim + (size_t)iq * K * K * K;
		for (int m = -L; m <= L; m++)
			for (int m2 = -L; m2 <= L; m2++) {
				size_t so = (((size_t)iq * N + m + L) * N + m2 + L) * K;
				for (int l = iabs(m); l <= L; l++) {
					double vr = 0.0, vi = 0.0;
					size_t to = ((size_t)iabs(m) * K + l) * K;
					for (int l1 = imax(iabs(m2), iabs(m)); l1 <= L; l1++) {
						double dv = d[d_idx(L, l1, m, m2)];
						double br = Bq[2 * lm_idx(l1, m2)], bi = Bq[2 * lm_idx(l1, m2) + 1];
						vr += dv * (br * tr[to + l1] - bi * ti[to + l1]);
						vi -= dv * (br * ti[to + l1] + bi * tr[to + l1]);
					}
					sre[so + l] = vr;
					sim[so + l] = vi;
				}
			}
	}
}

static inline int wrapm(int m, int N) { return m < 0 ? N + m : m; }

/* 6-channel X[c][m'][m1'][m2'] for one q (compute_sum2). */
static void sum2(const double *A, int iq, int qnum, int L, const double *d,
                 double *const S[6], double *X)
{
	int K = L + 1, N = 2 * L + 1, K2 = K * K;
	size_t chs = (size_t)qnum * K2 * 2, N3 = (size_t)N * N * N;
	const double *Vq = A + (size_t)iq * K2 * 2, *Dq = Vq + chs, *Wq = Vq + 2 * chs;
	const double *svr = S[0], *svi = S[1], *sdr = S[2], *sdi = S[3], *swr = S[4], *swi = S[5];
	for (int m = -L; m <= L; m++)
		for (int m1 = -L; m1 <= L; m1++)
			for (int m2 = -L; m2 <= L; m2++) {
				size_t so = (((size_t)iq * N + m + L) * N + m2 + L) * K;
				double vr[6] = {0}, vi[6] = {0};
				for (int l = imax(iabs(m1), iabs(m)); l <= L; l++) {
					double dv = d[d_idx(L, l, m, m1)];
					int ai = lm_idx(l, m1);
					double Vr = Vq[2 * ai], Vi = Vq[2 * ai + 1], Dr = Dq[2 * ai], Di = Dq[2 * ai + 1];
					double Wr = Wq[2 * ai], Wi = Wq[2 * ai + 1];
					size_t s = so + l;
					vr[0] += dv * (Vr * svr[s] - Vi * svi[s]);
					vi[0] += dv * (Vr * svi[s] + Vi * svr[s]);
					vr[1] += dv * (Vr * sdr[s] + Dr * svr[s] - Vi * sdi[s] - Di * svi[s]);
					vi[1] += dv * (Vr * sdi[s] + Dr * svi[s] + Vi * sdr[s] + Di * svr[s]);
					vr[2] += dv * (Vr * swr[s] + Wr * svr[s] - Vi * swi[s] - Wi * svi[s]);
					vi[2] += dv * (Vr * swi[s] + Wr * svi[s] + Vi * swr[s] + Wi * svr[s]);
					vr[3] += dv * (Dr * sdr[s] - Di * sdi[s]);
					vi[3] += dv * (Dr * sdi[s] + Di * sdr[s]);
					vr[4] += dv * (Dr * swr[s] + Wr * sdr[s] - Di * swi[s] - Wi * sdi[s]);
					vi[4] += dv * (Dr * swi[s] + Wr * sdi[s] + Di * swr[s] + Wi * sdr[s]);
					vr[5] += dv * (Wr * swr[s] - Wi * swi[s]);
					vi[5] += dv * (Wr * swi[s] + Wi * swr[s]);
				}
				size_t cell = ((size_t)wrapm(m, N) * N + wrapm(m1, N)) * N + wrapm(m2, N);
				for (int c = 0; c < 6; c++) {
					X[(c * N3 + cell) * 2] = vr[c];
					X[(c * N3 + cell) * 2 + 1] = vi[c];
				}
			}
}

/* Real part of the angular DFT at one cell with the given twiddle table
 * (simple_ft's loop order, src/fftsaxs.c:555-601). */
static void dft_cell(const double *X, int N, int a2, int g1, int g2, const double *er, const double *ei, double out[6])
{
	size_t N3 = (size_t)N * N * N;
	double v[6] = {0};
	int e = 0;
	size_t k = 0;
	for (int m = 0; m < N; m++) {
		for (int m1 = 0; m1 < N; m1++) {
			for (int m2 = 0; m2 < N; m2++) {
				double r = er[e % N], i = ei[e % N];
				for (int c = 0; c < 6; c++)
					v[c] += r * X[(c * N3 + k) * 2] - i * X[(c * N3 + k) * 2 + 1];
				e += g2;
				k++;
			}
			e += g1;
		}
		e += a2;
	}
	for (int c = 0; c < 6; c++) out[c] = v[c];
}

int orc_score(const double *A, const double *B, const double *q, int qnum, const double *z, int znum,
              int L, const int *index, int nout, int skip, double peak,
              const double *a, double mult, const double *c1g, int n1, const double *c2g, int n2,
              double *cross_raw, double *cross_scaled, double *grid, int *branch)
{
	int K = L + 1, N = 2 * L + 1, nb = L + 1, K2 = K * K;
	size_t N3 = (size_t)N * N * N;
	int ntrip = znum * nb * nb;
	int *pz = malloc(sizeof(int) * (nout + 1)), *pt = malloc(sizeof(int) * (nout + 1));
	int *pa = malloc(sizeof(int) * (nout + 1)), *pg1 = malloc(sizeof(int) * (nout + 1)), *pg2 = malloc(sizeof(int) * (nout + 1));
	int *cnt = calloc(ntrip, sizeof(int));
	for (int i = 0; i < nout; i++) {
		if (index[i] < 0) goto bad;
		long v = index[i];
		pg2[i] = v % N; v /= N;
		pg1[i] = v % N; v /= N;
		pa[i] = v % N; v /= N;
		int b2 = v % nb; v /= nb;
		int b1 = v % nb; v /= nb;
		if (v >= znum) goto bad;
		pz[i] = (int)v;
		pt[i] = ((int)v * nb + b1) * nb + b2;
		cnt[pt[i]]++;
	}

	/* the 3j table depends on L only; keep the last one (the reference
	 * rebuilds it per call, a fixed setup cost outside the per-pose work) */
	static double *ds_cache = NULL;
	static int ds_L = -1;
	if (ds_L != L) {
		free(ds_cache);
		ds_cache = malloc(sizeof(double) * K2 * K * N);
		orc_dsymb(L, ds_cache);
		ds_L = L;
	}
	const double *ds = ds_cache;
	size_t dsz = (size_t)K * N * N;
	double *dt = malloc(sizeof(double) * dsz * nb);
	double step = (ORC_PI - 0.0) / (nb - 1);
	for (int i = 0; i < nb; i++) orc_wigner_d(L, 0.0 + i * step, dt + i * dsz);

	double *cst = malloc(sizeof(double) * 6 * qnum);
	static const int pa_[6] = {0, 0, 0, 1, 1, 2}, pb_[6] = {0, 1, 2, 1, 2, 2};
	static const double mul[6] = {1.0, 2.0, 2.0, 1.0, 2.0, 1.0};
	for (int c = 0; c < 6; c++) const_int(A, B, pa_[c], pb_[c], qnum, K2, cst + c * qnum);

	double *tr_ = malloc(sizeof(double) * N), *ti_ = malloc(sizeof(double) * N);
	double *te_ = malloc(sizeof(double) * N), *tf_ = malloc(sizeof(double) * N);
	double st = 2 * ORC_PI / N, sx = 2 * 3.14159265358979323846 / N;
	for (int i = 0; i < N; i++) {
		tr_[i] = cos(i * st); ti_[i] = -sin(i * st);
		te_[i] = cos(i * sx); tf_[i] = -sin(i * sx);
	}

	double *bes = malloc(sizeof(double) * qnum * N);
	size_t tsz = (size_t)qnum * K * K * K;
	double *tre = calloc(tsz, sizeof(double)), *tim = calloc(tsz, sizeof(double));
	size_t ssz = (size_t)qnum * N * N * K;
	double *S = calloc(ssz * 6 * nb, sizeof(double));
	char *have = calloc(nb, 1);
	double *X = malloc(sizeof(double) * 6 * N3 * 2);

	for (int zi = 0; zi < znum; zi++) {
		int any = 0;
		for (int t = zi * nb * nb; t < (zi + 1) * nb * nb; t++) any |= cnt[t] > 0;
		if (!any) continue;
		orc_besselj_n(z[zi], q, qnum, L, bes);
		orc_t_matrix(L, qnum, bes, ds, tre, tim);
		memset(have, 0, nb);
		for (int b1 = 0; b1 < nb; b1++)
			for (int b2 = 0; b2 < nb; b2++) {
				int t = (zi * nb + b1) * nb + b2;
				if (cnt[t] == 0) continue;
				double *Sb = S + (size_t)b2 * 6 * ssz;
				if (!have[b2]) {
					for (int ch = 0; ch < 3; ch++)
						sum1(B, ch, qnum, L, tre, tim, dt + b2 * dsz, Sb + (2 * ch) * ssz, Sb + (2 * ch + 1) * ssz);
					have[b2] = 1;
				}
				double *Sp[6];
				for (int i = 0; i < 6; i++) Sp[i] = Sb + i * ssz;
				int fftw = (skip != 1) || cnt[t] >= 30;
				const double *er = fftw ? te_ : tr_, *ei = fftw ? tf_ : ti_;
				for (int iq = 0; iq < qnum; iq++) {
					sum2(A, iq, qnum, L, dt + b1 * dsz, Sp, X);
					for (int i = 0; i < nout; i++) {
						if (pt[i] != t) continue;
						double f[6];
						dft_cell(X, N, pa[i], pg1[i], pg2[i], er, ei, f);
						for (int c = 0; c < 6; c++) {
							double v = cst[c * qnum + iq] * mul[c];
							v += 2.0 * f[c];
							cross_raw[((size_t)i * 6 + c) * qnum + iq] = v;
						}
					}
				}
			}
	}
	for (int i = 0; i < nout; i++) {
		if (branch) branch[i] = (skip != 1) || cnt[pt[i]] >= 30;
		double *cs = cross_scaled + (size_t)i * 6 * qnum;
		memcpy(cs, cross_raw + (size_t)i * 6 * qnum, sizeof(double) * 6 * qnum);
		orc_rescale(cs, qnum, peak);
		if (grid)
			for (int x = 0; x < n1; x++)
				for (int y = 0; y < n2; y++)
					grid[((size_t)i * n1 + x) * n2 + y] = orc_point_score(cs, q, qnum, a, mult, c1g[x], c2g[y]);
	}
	free(dt); free(cst); free(tr_); free(ti_); free(te_); free(tf_);
	free(bes); free(tre); free(tim); free(S); free(have); free(X);
	free(pz); free(pt); free(pa); free(pg1); free(pg2); free(cnt);
	return 0;
bad:
	free(pz); free(pt); free(pa); free(pg1); free(pg2); free(cnt);
	return -1;
}
