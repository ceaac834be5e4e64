/*
 * Double-float arithmetic and the per-(pose, c1) work of the mixed path's
 * grid fit.  Shared by the device kernel (kernels_fitdf.cu) and host tests;
 * both compile it without multiply-add contraction (nvcc -fmad=false, gcc
 * -ffp-contract=off), so the host reproduces the device bit for bit.
 *
 * A double-float is the unevaluated sum hi + lo of two floats with
 * |lo| <= ulp(hi)/2 (Dekker's two-product via fmaf, Knuth's two-sum); each
 * operation below is accurate to about 2^-48 relative.
 *
 * The fit follows point_score and best_scale of the reference
 * (src/min_saxs.c:261-320, 391-448): for one c1 the model at q_i is
 * in_i = al_i + c2 be_i + c2^2 ga_i, and with D_i = in_i - in_{i-1} and the
 * per-q constants fc = {a3, e, f, a1, u} (folded on the host from the binned
 * experiment and the q spacing)
 *   up   = sum_i a1 in_i + u D_i               (quadratic in c2)
 *   down = sum_i a3 in_i^2 + 2 e in_i D_i + f D_i^2   (quartic in c2)
 * and the score at the best scale k = up/down is sum a0 - up^2/down.
 */
#ifndef SXS_FITDF_CORE_H
#define SXS_FITDF_CORE_H

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#define DF_HD static inline
#endif

typedef struct {
	float hi, lo;
} dfl;

DF_HD dfl df_mk(float h, float l)
{
	dfl r;
	r.hi = h;
	r.lo = l;
	return r;
}
DF_HD dfl df_from(double x)
{
	float h = (float)x;
	return df_mk(h, (float)(x - (double)h));
}
DF_HD double df_to(dfl a) { return (double)a.hi + (double)a.lo; }
/* |a| >= |b| */
DF_HD dfl df_fast_two_sum(float a, float b)
{
	float s = a + b;
	return df_mk(s, b - (s - a));
}
DF_HD dfl df_two_sum(float a, float b)
{
	float s = a + b;
	float bb = s - a;
	return df_mk(s, (a - (s - bb)) + (b - bb));
}
DF_HD dfl df_add(dfl a, dfl b)
{
	dfl s = df_two_sum(a.hi, b.hi);
	float e = s.lo + (a.lo + b.lo);
	return df_fast_two_sum(s.hi, e);
}
DF_HD dfl df_neg(dfl a) { return df_mk(-a.hi, -a.lo); }
DF_HD dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
DF_HD dfl df_mul(dfl a, dfl b)
{
	float p = a.hi * b.hi;
	float e = fmaf(a.hi, b.hi, -p);
	e = fmaf(a.hi, b.lo, e);
	e = fmaf(a.lo, b.hi, e);
	return df_fast_two_sum(p, e);
}
DF_HD dfl df_fma(dfl a, dfl b, dfl c) { return df_add(df_mul(a, b), c); }
DF_HD dfl df_twice(dfl a) { return df_mk(2.0f * a.hi, 2.0f * a.lo); }
DF_HD int df_gt(dfl a, dfl b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
DF_HD int df_pos(dfl a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo > 0.0f); }

/* compensated float sum: s + c tracks the exact sum of the added floats */
typedef struct {
	float s, c;
} fsum;
DF_HD void fs_add(fsum *a, float x)
{
	dfl t = df_two_sum(a->s, x);
	a->s = t.hi;
	a->c += t.lo;
}
DF_HD dfl fs_df(fsum a) { return df_fast_two_sum(a.s, a.c); }

/* One pose's channel rows c[8][Q] = VV VD VW DD DW WW F3G P4 (model
 * normalised), constants fs[5][Q] = a3 e f a1 u.  For q = i0, i0+step, ...:
 * F3G = a3 ga (double-float), P4 = {e ga + f D_ga, e D_ga} (two floats,
 * D_ga = ga_i - ga_{i-1}), and the partial sums of the c2^2 coefficients. */
DF_HD void df_pose_prep(dfl *c, const dfl *fs, int Q, int i0, int step, dfl *u2, dfl *d4)
{
	const dfl *WW = c + 5 * Q, *F3 = fs, *FE = fs + Q, *FF = fs + 2 * Q, *F1 = fs + 3 * Q, *FU = fs + 4 * Q;
	dfl *F3G = c + 6 * Q, *P4 = c + 7 * Q;
	dfl su = df_mk(0, 0), sd = df_mk(0, 0);
	for (int i = i0; i < Q; i += step) {
		dfl ga = WW[i], dg = i > 0 ? df_sub(ga, WW[i - 1]) : df_mk(0, 0);
		dfl p3 = df_fma(F3[i], ga, df_mul(FE[i], dg));
		dfl p4 = df_fma(FE[i], ga, df_mul(FF[i], dg));
		F3G[i] = df_mul(F3[i], ga);
		P4[i] = df_mk(p4.hi, (FE[i].hi * dg.hi));
		su = df_fma(F1[i], ga, df_fma(FU[i], dg, su));
		sd = df_fma(ga, p3, df_fma(dg, p4, sd));
	}
	*u2 = su;
	*d4 = sd;
}

/* Coefficients for one c1 (G[i] = c1^3 exp(-mult (c1^2-1) q_i^2)):
 * up = u[0] + c2 u[1] + c2^2 U2, down = d[0] + c2 d[1] + ... + c2^4 D4.
 * The model in_i (al + c2 be + c2^2 ga) and the terms that carry the
 * cancellation of the score, a3 in^2 and a1 in, are double-float; the terms
 * with a difference D_i = in_i - in_{i-1} or a bin offset (e, f, u) are at
 * most a few percent of those and are summed as compensated floats. */
DF_HD void df_row(const dfl *c, const dfl *fs, const dfl *G, int Q, dfl *u, dfl *d)
{
	const dfl *VV = c, *VD = c + Q, *VW = c + 2 * Q, *DD = c + 3 * Q, *DW = c + 4 * Q, *WW = c + 5 * Q;
	const dfl *F3G = c + 6 * Q, *P4 = c + 7 * Q;
	const dfl *F3 = fs, *FE = fs + Q, *FF = fs + 2 * Q, *F1 = fs + 3 * Q, *FU = fs + 4 * Q;
	dfl z = df_mk(0, 0);
	dfl U0 = z, U1 = z, D0 = z, D1 = z, D2a = z, D2b = z, D3 = z;
	fsum e0 = {0, 0}, e1 = {0, 0}, e2 = {0, 0}, e3 = {0, 0}, e4 = {0, 0}, eu0 = {0, 0}, eu1 = {0, 0};
	dfl g = G[0];
	dfl alp = df_fma(g, df_fma(g, DD[0], df_neg(VD[0])), VV[0]);
	dfl bep = df_fma(df_neg(g), DW[0], VW[0]);
	for (int i = 0; i < Q; i++) {
		g = G[i];
		dfl al = df_fma(g, df_fma(g, DD[i], df_neg(VD[i])), VV[i]);
		dfl be = df_fma(df_neg(g), DW[i], VW[i]);
		float d0 = (al.hi - alp.hi) + (al.lo - alp.lo);
		float d1 = (be.hi - bep.hi) + (be.lo - bep.lo);
		float a = al.hi, b = be.hi;
		float fe = FE[i].hi, ff = FF[i].hi;
		dfl t = df_mul(F3[i], al), v = df_mul(F3[i], be);
		D0 = df_fma(t, al, D0);                 /* a3 al^2 */
		D1 = df_fma(t, be, D1);                 /* a3 al be */
		D2a = df_fma(v, be, D2a);               /* a3 be^2 */
		D2b = df_fma(al, F3G[i], D2b);          /* a3 al ga */
		D3 = df_fma(be, F3G[i], D3);            /* a3 be ga */
		U0 = df_fma(F1[i], al, U0);
		U1 = df_fma(F1[i], be, U1);
		float p4 = P4[i].hi, edg = P4[i].lo;    /* e ga + f D_ga, e D_ga */
		fs_add(&e0, a * (2.0f * fe * d0) + ff * d0 * d0);
		fs_add(&e1, fe * (a * d1 + b * d0) + ff * d0 * d1);
		fs_add(&e2, b * (2.0f * fe * d1) + ff * d1 * d1);
		fs_add(&e3, a * edg + d0 * p4);
		fs_add(&e4, b * edg + d1 * p4);
		fs_add(&eu0, FU[i].hi * d0);
		fs_add(&eu1, FU[i].hi * d1);
		alp = al;
		bep = be;
	}
	u[0] = df_add(U0, fs_df(eu0));
	u[1] = df_add(U1, fs_df(eu1));
	d[0] = df_add(D0, fs_df(e0));
	d[1] = df_twice(df_add(D1, fs_df(e1)));
	d[2] = df_add(df_add(D2a, fs_df(e2)), df_twice(df_add(D2b, fs_df(e3))));
	d[3] = df_twice(df_add(D3, fs_df(e4)));
}

DF_HD dfl df_up(const dfl *u, dfl U2, dfl c2) { return df_fma(c2, df_fma(c2, U2, u[1]), u[0]); }
DF_HD dfl df_down(const dfl *d, dfl D4, dfl c2)
{
	return df_fma(c2, df_fma(c2, df_fma(c2, df_fma(c2, D4, d[3]), d[2]), d[1]), d[0]);
}

/* Best c2 cell of one c1 row: the largest up^2/down over cells with
 * down > 0 (lowest index on ties); returns its index or -1. */
DF_HD int df_best_c2(const dfl *u, dfl U2, const dfl *d, dfl D4, const dfl *c2s, int n2, dfl *bu, dfl *bd)
{
	int bi = -1;
	dfl xu = df_mk(0, 0), xd = df_mk(0, 0);
	for (int i2 = 0; i2 < n2; i2++) {
		dfl up = df_up(u, U2, c2s[i2]);
		dfl down = df_down(d, D4, c2s[i2]);
		if (df_pos(down) && (bi < 0 || df_gt(df_mul(df_mul(up, up), xd), df_mul(df_mul(xu, xu), down)))) {
			xu = up;
			xd = down;
			bi = i2;
		}
	}
	*bu = xu;
	*bd = xd;
	return bi;
}

#endif
