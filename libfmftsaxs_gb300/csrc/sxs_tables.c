/*
 * Host-side constant tables of the scoring path, computed once per L and
 * kept for the process: Wigner small-d matrices on the beta grid, the
 * translation coefficients d_lm(l1,p) (3j products), the Y_lm norms and the
 * twiddle tables.  These follow the reference's arithmetic step by step
 * (same formulas, same order, one rounding per operation: built with
 * -std=c11 -ffp-contract=off), so the device sees the reference's values.
 */
#define _XOPEN_SOURCE 700
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "sxs_internal.h"

/* ---------------------------------------------------------- binary128
 * x86-64 gcc names IEEE binary128 __float128; on aarch64 it is long double.
 * Both round + - * / correctly, so the tables are identical on both hosts. */
#if defined(__x86_64__) || defined(__i386__)
typedef __float128 quad_t_;
#elif defined(__aarch64__)
typedef long double quad_t_;
#else
#error "no binary128 type known for this host"
#endif

/* Newton refinement of the double estimate.  The 3j prefactors pass the
 * double range from L = 32 on (64!^6 ~ 1e530), so a is first brought into
 * it by an even power of two and the root scaled back by the half power:
 * both exact, and the steps commute with them, so values inside the double
 * range are unchanged. */
static quad_t_ quad_sqrt(quad_t_ a)
{
	if (a <= 0) return 0;
	quad_t_ s = 1;
	while (a > (quad_t_)0x1p1000) {
		a *= (quad_t_)0x1p-1000;
		s *= (quad_t_)0x1p500;
	}
	while (a < (quad_t_)0x1p-1000) {
		a *= (quad_t_)0x1p1000;
		s *= (quad_t_)0x1p-500;
	}
	quad_t_ y = (quad_t_)sqrt((double)a);
	y = (y + a / y) * (quad_t_)0.5;
	y = (y + a / y) * (quad_t_)0.5;
	return y * s;
}

/* towards zero, the rounding of GMP's mpf_get_d used by the reference */
static double quad_to_double_trunc(quad_t_ a)
{
	double d = (double)a;
	if (a > 0 && (quad_t_)d > a) d = nextafter(d, 0.0);
	if (a < 0 && (quad_t_)d < a) d = nextafter(d, 0.0);
	return d;
}

/* ------------------------------------------------- spherical Bessel j_l
 * src/sfbessel.c:21-60: power series from 1/(2l+1)!!, term ratio
 * -x^2 / (2k (2k+2l+1)), stop at |term/sum| <= 1e-5, times x^l. */
double sxs_sbessel_host(int l, double x)
{
	if (x > 0.0) {
		double tl1 = 2.0 * (double)l + 1.0;
		double df = 1.0;
		for (int i = 1; i <= (int)tl1; i += 2) df *= (double)i;
		double term = 1.0 / df;
		double sum = term;
		for (int k = 1; fabs(term / sum) > 0.00001 && k < 100000; k++) {
			double ratio = ((-1.0) * x * x) / ((2.0 * (double)k) * (2.0 * (double)k + tl1));
			term = term * ratio;
			sum = sum + term;
		}
		return sum * pow(x, l);
	}
	return l == 0 ? 1.0 : 0.0;
}

/* ------------------------------------------------------ Wigner small-d
 * src/borrowed.c:243-313 (Kostelec & Rockmore eqs. 26 and 28), layout
 * [l][m+L][m1+L], written in the reference's store order. */
void sxs_wigner_d_host(int L, double beta, double *d)
{
	int N = 2 * L + 1;
#define DI(l, m, m1) (((size_t)(l) * N + (size_t)((m) + L)) * N + (size_t)((m1) + L))
	memset(d, 0, sizeof(double) * (size_t)(L + 1) * N * N);
	d[DI(0, 0, 0)] = 1.0;
	if (L >= 1) {
		double c = cos(beta), s = sin(beta), r2 = sqrt(2.0);
		d[DI(1, -1, -1)] = 1.0 * (1.0 + c) / 2.0;
		d[DI(1, -1, 0)] = 1.0 * s / r2;
		d[DI(1, -1, 1)] = 1.0 * (1.0 - c) / 2.0;
		d[DI(1, 0, -1)] = -1.0 * s / r2;
		d[DI(1, 0, 0)] = 1.0 * c;
		d[DI(1, 0, 1)] = 1.0 * s / r2;
		d[DI(1, 1, -1)] = 1.0 * (1.0 - c) / 2.0;
		d[DI(1, 1, 0)] = -1.0 * s / r2;
		d[DI(1, 1, 1)] = 1.0 * (1.0 + c) / 2.0;
	}
	double ch = cos(beta / 2.0), sh = sin(beta / 2.0), cb = cos(beta);
	for (int l = 2; l <= L; l++) {
		for (int m = -l; m <= l; m++) {
			double e1 = 1.0, e2 = 1.0, e3 = 1.0, e4 = 1.0;
			for (int k = 1; k <= 2 * l; k++) {
				double den = ((k <= l + m) ? (double)k : 1.0) * ((k <= l - m) ? (double)k : 1.0);
				double f = sqrt(k / den);
				e1 *= f * ((k <= l + m) ? ch : 1.0) * ((k <= l - m) ? -sh : 1.0);
				e2 *= f * ((k <= l - m) ? ch : 1.0) * ((k <= l + m) ? sh : 1.0);
				e3 *= f * ((k <= l + m) ? ch : 1.0) * ((k <= l - m) ? sh : 1.0);
				e4 *= f * ((k <= l - m) ? ch : 1.0) * ((k <= l + m) ? -sh : 1.0);
			}
			d[DI(l, l, m)] = e1;
			d[DI(l, -l, m)] = e2;
			d[DI(l, m, l)] = e3;
			d[DI(l, m, -l)] = e4;
			if (m == -l || m == l) continue;
			int j = l - 1;
			for (int m1 = -l + 1; m1 <= l - 1; m1++) {
				double v = 1.0;
				v *= (j + 1) * (2.0 * j + 1) / sqrt((double)(((j + 1) * (j + 1) - m * m) * ((j + 1) * (j + 1) - m1 * m1)));
				v *= (cb - (double)(m * m1) / (double)(j * (j + 1))) * d[DI(j, m, m1)];
				double w = -1.0;
				w *= sqrt((double)((j * j - m * m) * (j * j - m1 * m1)));
				w *= (double)(j + 1.0) * d[DI(j - 1, m, m1)] / (double)j;
				w /= sqrt(((j + 1.0) * (j + 1.0) - (double)(m * m)) * ((j + 1.0) * (j + 1.0) - (double)(m1 * m1)));
				v += w;
				d[DI(l, m, m1)] = v;
			}
		}
	}
#undef DI
}

/* Y_lm norms sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!), (-1)^m for -m
 * (src/borrowed.c:19-38); layout [l][m+L]. */
void sxs_ynorm_host(int L, double *y)
{
	int N = 2 * L + 1;
	memset(y, 0, sizeof(double) * (size_t)(L + 1) * N);
	for (int l = 0; l <= L; l++) {
		double fact = 1.;
		double tmp0 = (2 * l + 1.) / (4. * SXS_PI);
		for (int m = 0; m <= l; m++) {
			if (m > 0) fact *= (l - m + 1) * (l + m);
			double tmp = sqrt(tmp0 / fact);
			double sgn = (m % 2 == 0) ? 1 : -1;
			y[l * N + (m + L)] = tmp;
			y[l * N + (-m + L)] = sgn * tmp;
		}
	}
}

/* twiddles cos(i s), -sin(i s), s = 2 pi / N with the reference's pi
 * (simple_ft, src/fftsaxs.c:536-548) or the full-precision pi (FFTW). */
void sxs_twiddles_host(int N, int exact, double *tw)
{
	double step = 2 * (exact ? SXS_PI_FULL : SXS_PI) / N;
	for (int i = 0; i < N; i++) {
		tw[2 * i] = cos(i * step);
		tw[2 * i + 1] = -sin(i * step);
	}
}

/* -------------------------------------------------------------- 3j
 * Racah sum in binary128 in the reference's product order
 * (src/borrowed.c:73-222), rounded towards zero like mpf_get_d. */
static double w3j(int j1, int j2, int j3, int m1, int m2, int m3, const quad_t_ *f)
{
	int t1 = j2 - m1 - j3, t2 = j1 + m2 - j3, t3 = j1 + j2 - j3, t4 = j1 - m1, t5 = j2 + m2;
	int tmin = t1 > t2 ? t1 : t2;
	if (tmin < 0) tmin = 0;
	int tmax = t3 < t4 ? t3 : t4;
	if (t5 < tmax) tmax = t5;
	quad_t_ acc = 0;
	for (int t = tmin; t <= tmax; t++) {
		quad_t_ one = (t % 2 == 0) ? 1 : -1;
		quad_t_ b = f[t4 - t] * f[t5 - t];
		b = f[t3 - t] * b;
		b = f[t - t2] * b;
		b = f[t - t1] * b;
		b = f[t] * b;
		b = one / b;
		acc = acc + b;
	}
	quad_t_ one = ((j1 - j2 - m3) % 2 == 0) ? 1 : -1;
	quad_t_ b = f[j3 + m3] * f[j3 - m3];
	b = f[j2 - m2] * b;
	b = f[j2 + m2] * b;
	b = f[j1 - m1] * b;
	b = f[j1 + m1] * b;
	b = b / f[j1 + j2 + j3 + 1];
	b = f[-j1 + j2 + j3] * b;
	b = f[j1 - j2 + j3] * b;
	b = f[j1 + j2 - j3] * b;
	b = quad_sqrt(b);
	b = one * b;
	acc = acc * b;
	return quad_to_double_trunc(acc);
}

typedef struct {
	int L, l_begin, l_step;
	const quad_t_ *f;
	double *ds;
} dsymb_job;

static void *dsymb_worker(void *arg)
{
	dsymb_job *j = (dsymb_job *)arg;
	int L = j->L, K = L + 1, N = 2 * L + 1;
	for (int l = j->l_begin; l <= L; l += j->l_step) {
		double k1 = 2 * l + 1;
		for (int l1 = 0; l1 <= L; l1++) {
			double k2 = sqrt((2 * l1 + 1) * k1);
			int lo = l > l1 ? l - l1 : l1 - l;
			int mm = l < l1 ? l : l1;
			for (int p = lo; p <= l + l1; p++) {
				double k3 = (2 * p + 1) * k2 * w3j(l, p, l1, 0, 0, 0, j->f);
				for (int m = -mm; m <= mm; m++) {
					double k4 = w3j(l, p, l1, -m, 0, m, j->f);
					j->ds[((size_t)(l * (l + 1) + m) * K + l1) * N + p] = k3 * k4;
				}
			}
		}
	}
	return NULL;
}

/* d_lm(l1,p) = (2p+1) sqrt((2l+1)(2l1+1)) 3j(l p l1;000) 3j(l p l1;-m 0 m)
 * (src/fftsaxs.c:138-174), layout [lm][l1][p]. */
static double *dsymb_build(int L)
{
	int K = L + 1, N = 2 * L + 1;
	size_t n = (size_t)K * K * K * N;
	double *ds = calloc(n, sizeof(double));
	quad_t_ *f = malloc(sizeof(quad_t_) * (4 * L + 2));
	if (!ds || !f) {
		free(ds); free(f);
		return NULL;
	}
	f[0] = 1;
	for (int i = 1; i <= 4 * L + 1; i++) f[i] = f[i - 1] * (quad_t_)i;
	enum { NT = 8 };
	pthread_t th[NT];
	dsymb_job jobs[NT];
	int nt = K < NT ? K : NT;
	int started[NT] = {0};
	for (int t = 0; t < nt; t++) {
		jobs[t] = (dsymb_job){L, t, nt, f, ds};
		started[t] = pthread_create(&th[t], NULL, dsymb_worker, &jobs[t]) == 0;
		if (!started[t]) dsymb_worker(&jobs[t]);   /* no thread: this share on the caller's */
	}
	for (int t = 0; t < nt; t++) if (started[t]) pthread_join(th[t], NULL);
	free(f);
	return ds;
}

static pthread_mutex_t g_ds_lock = PTHREAD_MUTEX_INITIALIZER;
static double *g_ds[SXS_LMAX + 1];

const double *sxs_dsymb_cached(int L)
{
	if (L < 1 || L > SXS_LMAX) return NULL;
	pthread_mutex_lock(&g_ds_lock);
	if (!g_ds[L]) g_ds[L] = dsymb_build(L);
	const double *r = g_ds[L];
	pthread_mutex_unlock(&g_ds_lock);
	return r;
}

/* ------------------------------------------------- device copies per L */
static pthread_mutex_t g_lt_lock = PTHREAD_MUTEX_INITIALIZER;
static sxs_ltables *g_lt[SXS_LMAX + 1];

int sxs_ltables_get(int L, const sxs_ltables **out)
{
	if (L < 1 || L > SXS_LMAX) return sxs_fail(-2, "L=%d outside [1, %d]", L, SXS_LMAX);
	int rc = sxs_ensure_init();
	if (rc) return rc;
	pthread_mutex_lock(&g_lt_lock);
	if (g_lt[L]) {
		*out = g_lt[L];
		pthread_mutex_unlock(&g_lt_lock);
		return 0;
	}
	int K = L + 1, N = 2 * L + 1;
	sxs_ltables *t = calloc(1, sizeof(*t));
	size_t dsz = (size_t)K * N * N;
	double *h_dt = malloc(sizeof(double) * dsz * K);
	const double *h_ds = sxs_dsymb_cached(L);
	double *h_yn = malloc(sizeof(double) * K * N);
	int nll = K * (K + 1) / 2;
	int2 *h_ll = malloc(sizeof(int2) * nll);
	float *h_df = malloc(sizeof(float) * dsz * K);
	if (!t || !h_dt || !h_ds || !h_yn || !h_ll || !h_df) {
		free(t); free(h_dt); free(h_yn); free(h_ll); free(h_df);
		pthread_mutex_unlock(&g_lt_lock);
		return sxs_fail(-5, "out of host memory (per-L tables, L=%d)", L);
	}
	t->L = L;
	double step = (SXS_PI - 0.0) / (K - 1);
	for (int b = 0; b < K; b++) sxs_wigner_d_host(L, 0.0 + b * step, h_dt + b * dsz);
	sxs_ynorm_host(L, h_yn);
	int k = 0;
	for (int l = 0; l <= L; l++)
		for (int l1 = l; l1 <= L; l1++) { h_ll[k].x = l; h_ll[k].y = l1; k++; }
	t->nll1 = nll;
	cudaError_t e = cudaSuccess;
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->d_dtab, sizeof(double) * dsz * K);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->d_dtabf, sizeof(float) * dsz * K);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->d_dsymb, sizeof(double) * (size_t)K * K * K * N);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->d_ynorm, sizeof(double) * K * N);
	if (e == cudaSuccess) e = cudaMalloc((void **)&t->d_ll1, sizeof(int2) * nll);
	if (e == cudaSuccess) e = cudaMemcpy(t->d_dtab, h_dt, sizeof(double) * dsz * K, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) {
		for (size_t i = 0; i < dsz * K; i++) h_df[i] = (float)h_dt[i];
		e = cudaMemcpy(t->d_dtabf, h_df, sizeof(float) * dsz * K, cudaMemcpyHostToDevice);
	}
	if (e == cudaSuccess) e = cudaMemcpy(t->d_dsymb, h_ds, sizeof(double) * (size_t)K * K * K * N, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(t->d_ynorm, h_yn, sizeof(double) * K * N, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(t->d_ll1, h_ll, sizeof(int2) * nll, cudaMemcpyHostToDevice);
	free(h_dt); free(h_yn); free(h_ll); free(h_df);
	if (e != cudaSuccess) {
		cudaFree(t->d_dtab); cudaFree(t->d_dtabf); cudaFree(t->d_dsymb); cudaFree(t->d_ynorm); cudaFree(t->d_ll1);
		free(t);
		pthread_mutex_unlock(&g_lt_lock);
		return sxs_cuda_fail(e, "per-L table upload");
	}
	g_lt[L] = t;
	*out = t;
	pthread_mutex_unlock(&g_lt_lock);
	return 0;
}
