/*
 * Double-float arithmetic and the per-(pose, c1) work of the mixed path's
 * grid fit.  Shared by the device kernel (kernels_fitdf.cu) and host tests;
 * both compile it without multiply-add contraction (nvcc -fmad=false, gcc
 * -ffp-contract=off), so the host reproduces the device bit for bit.
 *
 * A double-float is the unevaluated sum hi + lo of two floats with
 * |lo| <= ulp(hi)/2 (Dekker's two-product via fmaf, Knuth's two-sum); each
 * operation below is accurate to about 2^-48 relative (the lazy forms to a
 * few units of 2^-48).
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

/* Lazy forms: results are unevaluated sums hi + lo that are not
 * renormalised (|lo| stays a few ulp of hi unless the operands cancel), so
 * each saves the final fast-two-sum of df_mul / df_add.  Products drop
 * only lo*lo; sums keep the two-sum error and add the tails in float. */
DF_HD dfl lz_mul(dfl a, dfl b)
{
	float p = a.hi * b.hi;
	float e = fmaf(a.hi, b.hi, -p);
	e = fmaf(a.hi, b.lo, e);
	e = fmaf(a.lo, b.hi, e);
	return df_mk(p, e);
}
DF_HD dfl lz_add(dfl a, dfl b)
{
	dfl s = df_two_sum(a.hi, b.hi);
	return df_mk(s.hi, s.lo + (a.lo + b.lo));
}
DF_HD dfl lz_norm(dfl a) { return df_fast_two_sum(a.hi, a.lo); }
/* y*x + c, unnormalised */
DF_HD dfl lz_fma(dfl y, dfl x, dfl c) { return lz_add(lz_mul(y, x), c); }

/* Kahan-compensated float sum: s - c is the sum of the added floats to
 * within 2u sum |x| (u = 2^-24), c holding the part lost from s */
typedef struct {
	float s, c;
} fsum;
DF_HD void fs_add(fsum *a, float x)
{
	float y = x - a->c;
	float t = a->s + y;
	a->c = (t - a->s) - y;
	a->s = t;
}
DF_HD dfl fs_df(fsum a) { return df_two_sum(a.s, -a.c); }

/* Per-pose work of one run of n consecutive q.  Channel rows start at c
 * with row stride ld: VV VD VW DD DW WW F3G P4 (model normalised); c[-1] of
 * each row is the previous q unless `first` (the run starts at q = 0).
 * Constants fs[5][ldf] = a3 e f a1 u start at the same q.  For local
 * k = k0, k0+step, ...: F3G = a3 ga (double-float), P4 = {e ga + f D_ga,
 * e D_ga} (two floats, D_ga = ga_q - ga_{q-1}), and the partial sums of the
 * c2^2 coefficients are added to u2, d4. */
DF_HD void df_pose_prep_run(dfl *c, int ld, const dfl *fs, int ldf, int k0, int n, int step, int first, dfl *u2,
                            dfl *d4)
{
	const dfl *WW = c + 5 * ld, *F3 = fs, *FE = fs + ldf, *FF = fs + 2 * ldf, *F1 = fs + 3 * ldf, *FU = fs + 4 * ldf;
	dfl *F3G = c + 6 * ld, *P4 = c + 7 * ld;
	dfl su = *u2, sd = *d4;
	for (int i = k0; i < n; i += step) {
		dfl ga = WW[i], dg = (i > 0 || !first) ? df_sub(ga, WW[i - 1]) : df_mk(0, 0);
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

/* All Q at once: rows c[8][Q], constants fs[5][Q], q = i0, i0+step, ... */
DF_HD void df_pose_prep(dfl *c, const dfl *fs, int Q, int i0, int step, dfl *u2, dfl *d4)
{
	*u2 = df_mk(0, 0);
	*d4 = df_mk(0, 0);
	df_pose_prep_run(c, Q, fs, Q, i0, Q, step, 1, u2, d4);
}

/* Running sums of one (pose, c1) over q (df_row below). */
typedef struct {
	dfl U0, U1, D0, D1, D2a, D2b, D3, alp, bep;
	fsum e0, e1, e2, e3, e4, eu0, eu1;
} df_rowst;

/* model terms at one q: al = VV + g (g DD - VD), be = VW - g DW */
DF_HD void df_model(const dfl *c, int ld, dfl g, dfl *al, dfl *be)
{
	*al = lz_norm(lz_add(c[0], lz_mul(g, lz_add(lz_mul(g, c[3 * ld]), df_neg(c[ld])))));
	*be = lz_norm(lz_add(c[2 * ld], df_neg(lz_mul(g, c[4 * ld]))));
}

/* start at q = 0 (c, g: the rows and G there) */
DF_HD void df_row_init(df_rowst *r, const dfl *c, int ld, dfl g)
{
	dfl z = df_mk(0, 0);
	fsum f = {0, 0};
	r->U0 = r->U1 = r->D0 = r->D1 = r->D2a = r->D2b = r->D3 = z;
	r->e0 = r->e1 = r->e2 = r->e3 = r->e4 = r->eu0 = r->eu1 = f;
	df_model(c, ld, g, &r->alp, &r->bep);
}

/* n consecutive q: rows from c (stride ld, F3G and P4 filled), constants
 * fs (stride ldf) and G from the first of them.
 * The model in_q (al + c2 be + c2^2 ga) and the terms that carry the
 * cancellation of the score, a3 in^2 and a1 in, are double-float (lazy
 * products and sums, renormalised once per q for al and be); the terms with
 * a difference D_q = in_q - in_{q-1} or a bin offset (e, f, u) are at most a
 * few percent of those and are summed as compensated floats. */
DF_HD void df_row_run(df_rowst *r, const dfl *c, int ld, const dfl *fs, int ldf, const dfl *G, int n)
{
	const dfl *F3G = c + 6 * ld, *P4 = c + 7 * ld;
	const dfl *F3 = fs, *FE = fs + ldf, *FF = fs + 2 * ldf, *F1 = fs + 3 * ldf, *FU = fs + 4 * ldf;
	dfl U0 = r->U0, U1 = r->U1, D0 = r->D0, D1 = r->D1, D2a = r->D2a, D2b = r->D2b, D3 = r->D3;
	dfl alp = r->alp, bep = r->bep;
	fsum e0 = r->e0, e1 = r->e1, e2 = r->e2, e3 = r->e3, e4 = r->e4, eu0 = r->eu0, eu1 = r->eu1;
#ifdef __CUDACC__
#pragma unroll 2
#endif
	for (int i = 0; i < n; i++) {
		dfl al, be;
		df_model(c + i, ld, G[i], &al, &be);
		float d0 = (al.hi - alp.hi) + (al.lo - alp.lo);
		float d1 = (be.hi - bep.hi) + (be.lo - bep.lo);
		float a = al.hi, b = be.hi;
		float fe = FE[i].hi, ff = FF[i].hi;
		dfl t = lz_mul(F3[i], al), v = lz_mul(F3[i], be), f3g = F3G[i], f1 = F1[i];
		D0 = lz_fma(t, al, D0);                 /* a3 al^2 */
		D1 = lz_fma(t, be, D1);                 /* a3 al be */
		D2a = lz_fma(v, be, D2a);               /* a3 be^2 */
		D2b = lz_fma(al, f3g, D2b);             /* a3 al ga */
		D3 = lz_fma(be, f3g, D3);               /* a3 be ga */
		U0 = lz_fma(f1, al, U0);
		U1 = lz_fma(f1, be, U1);
		float p4 = P4[i].hi, edg = P4[i].lo;    /* e ga + f D_ga, e D_ga */
		float fa = fe * a, fb = fe * b, fd0 = ff * d0;
		fs_add(&e0, d0 * fmaf(ff, d0, fa + fa));              /* 2 e al D_al + f D_al^2 */
		fs_add(&e1, fmaf(fa, d1, fmaf(fb, d0, fd0 * d1)));  /* e (al D_be + be D_al) + f D_al D_be */
		fs_add(&e2, d1 * fmaf(ff, d1, fb + fb));              /* 2 e be D_be + f D_be^2 */
		fs_add(&e3, fmaf(a, edg, d0 * p4));
		fs_add(&e4, fmaf(b, edg, d1 * p4));
		fs_add(&eu0, FU[i].hi * d0);
		fs_add(&eu1, FU[i].hi * d1);
		alp = al;
		bep = be;
	}
	r->U0 = U0; r->U1 = U1; r->D0 = D0; r->D1 = D1; r->D2a = D2a; r->D2b = D2b; r->D3 = D3;
	r->alp = alp; r->bep = bep;
	r->e0 = e0; r->e1 = e1; r->e2 = e2; r->e3 = e3; r->e4 = e4; r->eu0 = eu0; r->eu1 = eu1;
}

/* up = u[0] + c2 u[1] + c2^2 U2, down = d[0] + c2 d[1] + ... + c2^4 D4 */
DF_HD void df_row_finish(const df_rowst *r, dfl *u, dfl *d)
{
	u[0] = df_add(lz_norm(r->U0), fs_df(r->eu0));
	u[1] = df_add(lz_norm(r->U1), fs_df(r->eu1));
	d[0] = df_add(lz_norm(r->D0), fs_df(r->e0));
	d[1] = df_twice(df_add(lz_norm(r->D1), fs_df(r->e1)));
	d[2] = df_add(df_add(lz_norm(r->D2a), fs_df(r->e2)), df_twice(df_add(lz_norm(r->D2b), fs_df(r->e3))));
	d[3] = df_twice(df_add(lz_norm(r->D3), fs_df(r->e4)));
}

/* Coefficients for one c1 (G[q] = c1^3 exp(-mult (c1^2-1) q^2)) over all
 * Q: rows c[8][Q] after df_pose_prep, constants fs[5][Q]. */
DF_HD void df_row(const dfl *c, const dfl *fs, const dfl *G, int Q, dfl *u, dfl *d)
{
	df_rowst r;
	df_row_init(&r, c, Q, G[0]);
	df_row_run(&r, c, Q, fs, Q, G, Q);
	df_row_finish(&r, u, d);
}

DF_HD dfl df_up(const dfl *u, dfl U2, dfl c2) { return lz_norm(lz_fma(c2, lz_fma(c2, U2, u[1]), u[0])); }
DF_HD dfl df_down(const dfl *d, dfl D4, dfl c2)
{
	return lz_norm(lz_fma(c2, lz_fma(c2, lz_fma(c2, lz_fma(c2, D4, d[3]), d[2]), d[1]), d[0]));
}

/* Best c2 cell of one c1 row: the largest up^2/down over cells with
 * down > 0 (lowest index on ties); returns its index or -1.  The test
 * up^2 xd > xu^2 down is the sign of their lazy difference. */
DF_HD int df_best_c2(const dfl *u, dfl U2, const dfl *d, dfl D4, const dfl *c2s, int n2, dfl *bu, dfl *bd)
{
	int bi = -1;
	dfl xu = df_mk(0, 0), xd = df_mk(0, 0), xuu = df_mk(0, 0);
	for (int i2 = 0; i2 < n2; i2++) {
		dfl up = df_up(u, U2, c2s[i2]);
		dfl down = df_down(d, D4, c2s[i2]);
		if (!df_pos(down)) continue;
		dfl uu = lz_mul(up, up);
		if (bi >= 0) {
			dfl diff = lz_add(lz_mul(uu, xd), df_neg(lz_mul(xuu, down)));
			if (!(diff.hi + diff.lo > 0.0f)) continue;
		}
		xu = up;
		xd = down;
		xuu = uu;
		bi = i2;
	}
	*bu = xu;
	*bd = xd;
	return bi;
}

#endif
