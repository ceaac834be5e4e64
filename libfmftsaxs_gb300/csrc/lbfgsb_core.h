/*
 * This file restates, for two variables, the C translation of L-BFGS-B v3.0
 * that the reference project vendors in lbfgsb/ (its subalgorithms.c,
 * linesearch.c and linpack.c); that code is distributed under the licence
 * below, whose notice is retained here as it requires.
 *
 * BSD 3-clause license
 * Copyright (c) 2015, Stephen Becker
 * All rights reserved.
 *
 * Redistribution and use in source and binary forms, with or without
 * modification, are permitted provided that the following conditions are met:
 *
 * * Redistributions of source code must retain the above copyright notice, this
 *   list of conditions and the following disclaimer.
 *
 * * Redistributions in binary form must reproduce the above copyright notice,
 *   this list of conditions and the following disclaimer in the documentation
 *   and/or other materials provided with the distribution.
 *
 * * Neither the name of the copyright holder nor the names of its
 *   contributors may be used to endorse or promote products derived from
 *   this software without specific prior written permission.
 *
 * THIS SOFTWARE IS PROVIDED BY THE COPYRIGHT HOLDERS AND CONTRIBUTORS "AS IS"
 * AND ANY EXPRESS OR IMPLIED WARRANTIES, INCLUDING, BUT NOT LIMITED TO, THE
 * IMPLIED WARRANTIES OF MERCHANTABILITY AND FITNESS FOR A PARTICULAR PURPOSE ARE
 * DISCLAIMED. IN NO EVENT SHALL THE COPYRIGHT HOLDER OR CONTRIBUTORS BE LIABLE
 * FOR ANY DIRECT, INDIRECT, INCIDENTAL, SPECIAL, EXEMPLARY, OR CONSEQUENTIAL
 * DAMAGES (INCLUDING, BUT NOT LIMITED TO, PROCUREMENT OF SUBSTITUTE GOODS OR
 * SERVICES; LOSS OF USE, DATA, OR PROFITS; OR BUSINESS INTERRUPTION) HOWEVER
 * CAUSED AND ON ANY THEORY OF LIABILITY, WHETHER IN CONTRACT, STRICT LIABILITY,
 * OR TORT (INCLUDING NEGLIGENCE OR OTHERWISE) ARISING IN ANY WAY OUT OF THE USE
 * OF THIS SOFTWARE, EVEN IF ADVISED OF THE POSSIBILITY OF SUCH DAMAGE.
 */
/*
 * Bound-constrained L-BFGS-B (Byrd, Lu, Nocedal & Zhu 1995; version 3.0 of
 * Zhu, Byrd, Lu, Nocedal and Morales 2011, with the Moré-Thuente line search
 * of MINPACK-2) for the two-parameter (c1, c2) SAXS fit, one solver per
 * thread.  The reference drives the vendored C translation of that code
 * through setulb's reverse communication (src/min_saxs.c:196-259, lbfgsb/src);
 * this is a direct-loop restatement for n = 2 variables with m = 3
 * corrections and both variables boxed, keeping the published algorithm's
 * order of operations (generalized Cauchy point with breakpoint heap,
 * subspace minimization with the projected-step fix, line search with
 * stpmax from the box, compact L-BFGS update with the Cholesky factor of
 * theta S'S + L D^-1 L'), so that the iterates follow the reference's.
 *
 * Objective (src/min_saxs.c:3-105, 261-319): f(c1, c2) = chi^2 of the
 * piecewise-linear model against the binned experiment at the best scale
 * k(c1, c2), gradient at fixed k.
 *
 * Compiled as device code (nvcc, -fmad=false) and as host C for tests.
 */
#ifndef SXS_LBFGSB_CORE_H
#define SXS_LBFGSB_CORE_H

#include <math.h>
#include <float.h>

#ifdef __CUDACC__
#define LB_HD __host__ __device__ __forceinline__
#else
#define LB_HD static inline
#endif

#define LB_N 2
#define LB_M 3
#define LB_M2 (2 * LB_M)

/* 1-based access to column-major arrays, as in the published code */
#define V1(a, i) (a)[(i) - 1]
#define M1(a, ld, i, j) (a)[((j) - 1) * (ld) + (i) - 1]

LB_HD double lb_max(double a, double b) { return a >= b ? a : b; }
LB_HD double lb_min(double a, double b) { return a <= b ? a : b; }
LB_HD double lb_abs(double a) { return a >= 0 ? a : -a; }

LB_HD double lb_dot(int n, const double *x, const double *y)
{
	double s = 0.0;
	for (int i = 0; i < n; i++) s = s + x[i] * y[i];
	return s;
}

/* y += a x; a == 0 leaves y untouched */
LB_HD void lb_axpy(int n, double a, const double *x, double *y)
{
	if (n <= 0 || a == 0.0) return;
	for (int i = 0; i < n; i++) y[i] += a * x[i];
}

/* Cholesky factor R'R of the leading n x n block of a (column-major, leading
 * dimension lda), R in the upper triangle; info = j if the j-th pivot is not
 * positive. */
LB_HD void lb_pofa(double *a, int lda, int n, int *info)
{
	for (int j = 1; j <= n; j++) {
		*info = j;
		double s = 0.0;
		for (int k = 1; k <= j - 1; k++) {
			double t = M1(a, lda, k, j) - lb_dot(k - 1, &M1(a, lda, 1, k), &M1(a, lda, 1, j));
			t /= M1(a, lda, k, k);
			M1(a, lda, k, j) = t;
			s += t * t;
		}
		s = M1(a, lda, j, j) - s;
		if (s <= 0.0) return;
		M1(a, lda, j, j) = sqrt(s);
	}
	*info = 0;
}

/* Triangular solves with the upper triangle T of t: job 1 solves T x = b,
 * job 11 solves T' x = b (the two cases the algorithm uses). */
LB_HD void lb_trsl(const double *t, int ldt, int n, double *b, int job, int *info)
{
	for (*info = 1; *info <= n; ++(*info))
		if (M1(t, ldt, *info, *info) == 0.0) return;
	*info = 0;
	if (job == 1) {
		V1(b, n) /= M1(t, ldt, n, n);
		for (int jj = 2; jj <= n; jj++) {
			int j = n - jj + 1;
			double temp = -V1(b, j + 1);
			lb_axpy(j, temp, &M1(t, ldt, 1, j + 1), &V1(b, 1));
			V1(b, j) /= M1(t, ldt, j, j);
		}
	} else {
		V1(b, 1) /= M1(t, ldt, 1, 1);
		for (int j = 2; j <= n; j++) {
			V1(b, j) -= lb_dot(j - 1, &M1(t, ldt, 1, j), &V1(b, 1));
			V1(b, j) /= M1(t, ldt, j, j);
		}
	}
}

typedef struct {
	double x[LB_N], l[LB_N], u[LB_N];
	int nbd[LB_N];
	double f, g[LB_N];
	double ws[LB_N * LB_M], wy[LB_N * LB_M];
	double sy[LB_M * LB_M], ss[LB_M * LB_M], wt[LB_M * LB_M];
	double wn[LB_M2 * LB_M2], snd[LB_M2 * LB_M2];
	double z[LB_N], r[LB_N], d[LB_N], t[LB_N], xp[LB_N];
	double wa[8 * LB_M];
	int index[LB_N], iwhere[LB_N], indx2[LB_N];
	/* iteration state */
	int col, head, itail, iupdat, updatd, iback, iword, nfree, nenter, ileave, iter, nfgv, ifun;
	int cnstnd, boxed, prjctd, info, nseg;
	double theta, fold, dnorm, dtd, gd, gdold, stp, stpmx, sbgnrm, xstep, epsmch, tol;
	/* line-search state */
	int ls_task, ls_brackt, ls_stage;
	double ls_ginit, ls_gtest, ls_gx, ls_gy, ls_finit, ls_fx, ls_fy, ls_stx, ls_sty, ls_stmin, ls_stmax, ls_width,
	    ls_width1;
} lb_state;

/* M^-1 v for the middle matrix of the compact L-BFGS form */
LB_HD void lb_bmv(const double *sy, const double *wt, int col, const double *v, double *p, int *info)
{
	const int m = LB_M;
	if (col == 0) return;
	V1(p, col + 1) = V1(v, col + 1);
	for (int i = 2; i <= col; i++) {
		int i2 = col + i;
		double sum = 0.0;
		for (int k = 1; k <= i - 1; k++) sum += M1(sy, m, i, k) * V1(v, k) / M1(sy, m, k, k);
		V1(p, i2) = V1(v, i2) + sum;
	}
	lb_trsl(wt, m, col, &V1(p, col + 1), 11, info);
	if (*info != 0) return;
	for (int i = 1; i <= col; i++) V1(p, i) = V1(v, i) / sqrt(M1(sy, m, i, i));
	lb_trsl(wt, m, col, &V1(p, col + 1), 1, info);
	if (*info != 0) return;
	for (int i = 1; i <= col; i++) V1(p, i) = -V1(p, i) / sqrt(M1(sy, m, i, i));
	for (int i = 1; i <= col; i++) {
		double sum = 0.0;
		for (int k = i + 1; k <= col; k++) sum += M1(sy, m, k, i) * V1(p, col + k) / M1(sy, m, i, i);
		V1(p, i) += sum;
	}
}

LB_HD void lb_projgr(const lb_state *s, double *sbgnrm)
{
	*sbgnrm = 0.0;
	for (int i = 1; i <= LB_N; i++) {
		double gi = V1(s->g, i);
		if (V1(s->nbd, i) != 0) {
			if (gi < 0.0) {
				if (V1(s->nbd, i) >= 2) gi = lb_max(V1(s->x, i) - V1(s->u, i), gi);
			} else {
				if (V1(s->nbd, i) <= 2) gi = lb_min(V1(s->x, i) - V1(s->l, i), gi);
			}
		}
		*sbgnrm = lb_max(*sbgnrm, lb_abs(gi));
	}
}

/* heap of breakpoints: iheap == 0 builds it first; pops the least into t[n] */
LB_HD void lb_hpsolb(int n, double *t, int *iorder, int iheap)
{
	if (iheap == 0) {
		for (int k = 2; k <= n; k++) {
			double ddum = V1(t, k);
			int indxin = V1(iorder, k);
			int i = k;
			while (i > 1) {
				int j = i / 2;
				if (ddum < V1(t, j)) {
					V1(t, i) = V1(t, j);
					V1(iorder, i) = V1(iorder, j);
					i = j;
				} else {
					break;
				}
			}
			V1(t, i) = ddum;
			V1(iorder, i) = indxin;
		}
	}
	if (n > 1) {
		int i = 1;
		double out = V1(t, 1);
		int indxou = V1(iorder, 1);
		double ddum = V1(t, n);
		int indxin = V1(iorder, n);
		for (;;) {
			int j = i + i;
			if (j <= n - 1) {
				if (V1(t, j + 1) < V1(t, j)) ++j;
				if (V1(t, j) < ddum) {
					V1(t, i) = V1(t, j);
					V1(iorder, i) = V1(iorder, j);
					i = j;
					continue;
				}
			}
			break;
		}
		V1(t, i) = ddum;
		V1(iorder, i) = indxin;
		V1(t, n) = out;
		V1(iorder, n) = indxou;
	}
}

/* Generalized Cauchy point along the projected steepest-descent path. */
LB_HD void lb_cauchy(lb_state *s, int *info)
{
	const int n = LB_N, m = LB_M;
	double *x = s->x, *l = s->l, *u = s->u, *g = s->g, *xcp = s->z, *d = s->d;
	int *nbd = s->nbd, *iwhere = s->iwhere, *iorder = s->indx2;
	double tb[LB_N];
	double *t = tb; /* breakpoints */
	double *p = s->wa, *c = s->wa + 2 * m, *wbp = s->wa + 4 * m, *v = s->wa + 6 * m;
	int col = s->col;
	double theta = s->theta;
	if (s->sbgnrm <= 0.0) {
		for (int i = 0; i < n; i++) xcp[i] = x[i];
		return;
	}
	int bnded = 1, nfree = n + 1, nbreak = 0, ibkmin = 0, col2 = col * 2;
	double bkmin = 0.0, f1 = 0.0, tl = 0.0, tu = 0.0;
	for (int i = 1; i <= col2; i++) V1(p, i) = 0.0;
	for (int i = 1; i <= n; i++) {
		double neggi = -V1(g, i);
		if (V1(iwhere, i) != 3 && V1(iwhere, i) != -1) {
			if (V1(nbd, i) <= 2) tl = V1(x, i) - V1(l, i);
			if (V1(nbd, i) >= 2) tu = V1(u, i) - V1(x, i);
			int xlower = V1(nbd, i) <= 2 && tl <= 0.0;
			int xupper = V1(nbd, i) >= 2 && tu <= 0.0;
			V1(iwhere, i) = 0;
			if (xlower) {
				if (neggi <= 0.0) V1(iwhere, i) = 1;
			} else if (xupper) {
				if (neggi >= 0.0) V1(iwhere, i) = 2;
			} else {
				if (lb_abs(neggi) <= 0.0) V1(iwhere, i) = -3;
			}
		}
		int pointr = s->head;
		if (V1(iwhere, i) != 0 && V1(iwhere, i) != -1) {
			V1(d, i) = 0.0;
		} else {
			V1(d, i) = neggi;
			f1 -= neggi * neggi;
			for (int j = 1; j <= col; j++) {
				V1(p, j) += M1(s->wy, n, i, pointr) * neggi;
				V1(p, col + j) += M1(s->ws, n, i, pointr) * neggi;
				pointr = pointr % m + 1;
			}
			if (V1(nbd, i) <= 2 && V1(nbd, i) != 0 && neggi < 0.0) {
				++nbreak;
				V1(iorder, nbreak) = i;
				V1(t, nbreak) = tl / (-neggi);
				if (nbreak == 1 || V1(t, nbreak) < bkmin) {
					bkmin = V1(t, nbreak);
					ibkmin = nbreak;
				}
			} else if (V1(nbd, i) >= 2 && neggi > 0.0) {
				++nbreak;
				V1(iorder, nbreak) = i;
				V1(t, nbreak) = tu / neggi;
				if (nbreak == 1 || V1(t, nbreak) < bkmin) {
					bkmin = V1(t, nbreak);
					ibkmin = nbreak;
				}
			} else {
				--nfree;
				V1(iorder, nfree) = i;
				if (lb_abs(neggi) > 0.0) bnded = 0;
			}
		}
	}
	if (theta != 1.0)
		for (int j = 1; j <= col; j++) V1(p, col + j) = theta * V1(p, col + j);
	for (int i = 0; i < n; i++) xcp[i] = x[i];
	if (nbreak == 0 && nfree == n + 1) return;
	for (int j = 1; j <= col2; j++) V1(c, j) = 0.0;
	double f2 = -theta * f1;
	double f2_org = f2;
	if (col > 0) {
		lb_bmv(s->sy, s->wt, col, p, v, info);
		if (*info != 0) return;
		f2 -= lb_dot(col2, v, p);
	}
	double dtm = -f1 / f2;
	double tsum = 0.0;
	s->nseg = 1;
	if (nbreak != 0) {
		int nleft = nbreak, iter = 1, ibp = 0;
		double tj = 0.0;
		for (;;) {
			double tj0 = tj;
			if (iter == 1) {
				tj = bkmin;
				ibp = V1(iorder, ibkmin);
			} else {
				if (iter == 2 && ibkmin != nbreak) {
					V1(t, ibkmin) = V1(t, nbreak);
					V1(iorder, ibkmin) = V1(iorder, nbreak);
				}
				lb_hpsolb(nleft, t, iorder, iter - 2);
				tj = V1(t, nleft);
				ibp = V1(iorder, nleft);
			}
			double dt = tj - tj0;
			if (dtm < dt) break;
			tsum += dt;
			--nleft;
			++iter;
			double dibp = V1(d, ibp), zibp;
			V1(d, ibp) = 0.0;
			if (dibp > 0.0) {
				zibp = V1(u, ibp) - V1(x, ibp);
				V1(xcp, ibp) = V1(u, ibp);
				V1(iwhere, ibp) = 2;
			} else {
				zibp = V1(l, ibp) - V1(x, ibp);
				V1(xcp, ibp) = V1(l, ibp);
				V1(iwhere, ibp) = 1;
			}
			if (nleft == 0 && nbreak == n) {
				dtm = dt;
				if (col > 0) lb_axpy(col2, dtm, p, c);
				return;
			}
			++s->nseg;
			double dibp2 = dibp * dibp;
			f1 = f1 + dt * f2 + dibp2 - theta * dibp * zibp;
			f2 -= theta * dibp2;
			if (col > 0) {
				lb_axpy(col2, dt, p, c);
				int pointr = s->head;
				for (int j = 1; j <= col; j++) {
					V1(wbp, j) = M1(s->wy, n, ibp, pointr);
					V1(wbp, col + j) = theta * M1(s->ws, n, ibp, pointr);
					pointr = pointr % m + 1;
				}
				lb_bmv(s->sy, s->wt, col, wbp, v, info);
				if (*info != 0) return;
				double wmc = lb_dot(col2, c, v), wmp = lb_dot(col2, p, v), wmw = lb_dot(col2, wbp, v);
				lb_axpy(col2, -dibp, wbp, p);
				f1 += dibp * wmc;
				f2 = f2 + dibp * 2. * wmp - dibp2 * wmw;
			}
			f2 = lb_max(s->epsmch * f2_org, f2);
			if (nleft > 0) {
				dtm = -f1 / f2;
				continue;
			} else if (bnded) {
				f1 = 0.0;
				f2 = 0.0;
				dtm = 0.0;
			} else {
				dtm = -f1 / f2;
			}
			break;
		}
	}
	if (dtm <= 0.0) dtm = 0.0;
	tsum += dtm;
	lb_axpy(n, tsum, d, xcp);
	if (col > 0) lb_axpy(col2, dtm, p, c);
}

LB_HD void lb_freev(lb_state *s, int *wrk)
{
	const int n = LB_N;
	s->nenter = 0;
	s->ileave = n + 1;
	if (s->iter > 0 && s->cnstnd) {
		for (int i = 1; i <= s->nfree; i++) {
			int k = V1(s->index, i);
			if (V1(s->iwhere, k) > 0) {
				--s->ileave;
				V1(s->indx2, s->ileave) = k;
			}
		}
		for (int i = s->nfree + 1; i <= n; i++) {
			int k = V1(s->index, i);
			if (V1(s->iwhere, k) <= 0) {
				++s->nenter;
				V1(s->indx2, s->nenter) = k;
			}
		}
	}
	*wrk = s->ileave < n + 1 || s->nenter > 0 || s->updatd;
	s->nfree = 0;
	int iact = n + 1;
	for (int i = 1; i <= n; i++) {
		if (V1(s->iwhere, i) <= 0) {
			++s->nfree;
			V1(s->index, s->nfree) = i;
		} else {
			--iact;
			V1(s->index, iact) = i;
		}
	}
}

/* LEL' factorization of the indefinite subspace matrix K (wn), updating
 * the N matrix (snd) incrementally as the published formk does. */
LB_HD void lb_formk(lb_state *s, int *info)
{
	const int n = LB_N, m = LB_M, ld = LB_M2;
	double *wn = s->wn, *wn1 = s->snd;
	const double *ws = s->ws, *wy = s->wy, *sy = s->sy;
	const int *ind = s->index, *indx2 = s->indx2;
	int col = s->col, head = s->head, nsub = s->nfree, upcl;
	double theta = s->theta;
	if (s->updatd) {
		if (s->iupdat > m) {
			for (int jy = 1; jy <= m - 1; jy++) {
				int js = m + jy;
				for (int k = 0; k < m - jy; k++) M1(wn1, ld, jy + k, jy) = M1(wn1, ld, jy + 1 + k, jy + 1);
				for (int k = 0; k < m - jy; k++) M1(wn1, ld, js + k, js) = M1(wn1, ld, js + 1 + k, js + 1);
				for (int k = 0; k < m - 1; k++) M1(wn1, ld, m + 1 + k, jy) = M1(wn1, ld, m + 2 + k, jy + 1);
			}
		}
		int pbegin = 1, pend = nsub, dbegin = nsub + 1, dend = n;
		int iy = col, is = m + col;
		int ipntr = head + col - 1;
		if (ipntr > m) ipntr -= m;
		int jpntr = head;
		for (int jy = 1; jy <= col; jy++) {
			int js = m + jy;
			double temp1 = 0.0, temp2 = 0.0, temp3 = 0.0;
			for (int k = pbegin; k <= pend; k++) {
				int k1 = V1(ind, k);
				temp1 += M1(wy, n, k1, ipntr) * M1(wy, n, k1, jpntr);
			}
			for (int k = dbegin; k <= dend; k++) {
				int k1 = V1(ind, k);
				temp2 += M1(ws, n, k1, ipntr) * M1(ws, n, k1, jpntr);
				temp3 += M1(ws, n, k1, ipntr) * M1(wy, n, k1, jpntr);
			}
			M1(wn1, ld, iy, jy) = temp1;
			M1(wn1, ld, is, js) = temp2;
			M1(wn1, ld, is, jy) = temp3;
			jpntr = jpntr % m + 1;
		}
		int jy = col;
		jpntr = head + col - 1;
		if (jpntr > m) jpntr -= m;
		ipntr = head;
		for (int i = 1; i <= col; i++) {
			is = m + i;
			double temp3 = 0.0;
			for (int k = pbegin; k <= pend; k++) {
				int k1 = V1(ind, k);
				temp3 += M1(ws, n, k1, ipntr) * M1(wy, n, k1, jpntr);
			}
			ipntr = ipntr % m + 1;
			M1(wn1, ld, is, jy) = temp3;
		}
		upcl = col - 1;
	} else {
		upcl = col;
	}
	int ipntr = head;
	for (int iy = 1; iy <= upcl; iy++) {
		int is = m + iy, jpntr = head;
		for (int jy = 1; jy <= iy; jy++) {
			int js = m + jy;
			double temp1 = 0.0, temp2 = 0.0, temp3 = 0.0, temp4 = 0.0;
			for (int k = 1; k <= s->nenter; k++) {
				int k1 = V1(indx2, k);
				temp1 += M1(wy, n, k1, ipntr) * M1(wy, n, k1, jpntr);
				temp2 += M1(ws, n, k1, ipntr) * M1(ws, n, k1, jpntr);
			}
			for (int k = s->ileave; k <= n; k++) {
				int k1 = V1(indx2, k);
				temp3 += M1(wy, n, k1, ipntr) * M1(wy, n, k1, jpntr);
				temp4 += M1(ws, n, k1, ipntr) * M1(ws, n, k1, jpntr);
			}
			M1(wn1, ld, iy, jy) = M1(wn1, ld, iy, jy) + temp1 - temp3;
			M1(wn1, ld, is, js) = M1(wn1, ld, is, js) - temp2 + temp4;
			jpntr = jpntr % m + 1;
		}
		ipntr = ipntr % m + 1;
	}
	ipntr = head;
	for (int is = m + 1; is <= m + upcl; is++) {
		int jpntr = head;
		for (int jy = 1; jy <= upcl; jy++) {
			double temp1 = 0.0, temp3 = 0.0;
			for (int k = 1; k <= s->nenter; k++) {
				int k1 = V1(indx2, k);
				temp1 += M1(ws, n, k1, ipntr) * M1(wy, n, k1, jpntr);
			}
			for (int k = s->ileave; k <= n; k++) {
				int k1 = V1(indx2, k);
				temp3 += M1(ws, n, k1, ipntr) * M1(wy, n, k1, jpntr);
			}
			if (is <= jy + m)
				M1(wn1, ld, is, jy) = M1(wn1, ld, is, jy) + temp1 - temp3;
			else
				M1(wn1, ld, is, jy) = M1(wn1, ld, is, jy) - temp1 + temp3;
			jpntr = jpntr % m + 1;
		}
		ipntr = ipntr % m + 1;
	}
	for (int iy = 1; iy <= col; iy++) {
		int is = col + iy, is1 = m + iy;
		for (int jy = 1; jy <= iy; jy++) {
			int js = col + jy, js1 = m + jy;
			M1(wn, ld, jy, iy) = M1(wn1, ld, iy, jy) / theta;
			M1(wn, ld, js, is) = M1(wn1, ld, is1, js1) * theta;
		}
		for (int jy = 1; jy <= iy - 1; jy++) M1(wn, ld, jy, is) = -M1(wn1, ld, is1, jy);
		for (int jy = iy; jy <= col; jy++) M1(wn, ld, jy, is) = M1(wn1, ld, is1, jy);
		M1(wn, ld, iy, iy) += M1(sy, m, iy, iy);
	}
	lb_pofa(wn, ld, col, info);
	if (*info != 0) {
		*info = -1;
		return;
	}
	int col2 = 2 * col;
	for (int js = col + 1; js <= col2; js++) lb_trsl(wn, ld, col, &M1(wn, ld, 1, js), 11, info);
	for (int is = col + 1; is <= col2; is++)
		for (int js = is; js <= col2; js++)
			M1(wn, ld, is, js) += lb_dot(col, &M1(wn, ld, 1, is), &M1(wn, ld, 1, js));
	lb_pofa(&M1(wn, ld, col + 1, col + 1), ld, col, info);
	if (*info != 0) *info = -2;
}

/* reduced gradient r = -Z'(B(xcp - x) + g) */
LB_HD void lb_cmprlb(lb_state *s, int *info)
{
	const int n = LB_N, m = LB_M;
	int col = s->col;
	if (!s->cnstnd && col > 0) {
		for (int i = 1; i <= n; i++) V1(s->r, i) = -V1(s->g, i);
		return;
	}
	for (int i = 1; i <= s->nfree; i++) {
		int k = V1(s->index, i);
		V1(s->r, i) = -s->theta * (V1(s->z, k) - V1(s->x, k)) - V1(s->g, k);
	}
	lb_bmv(s->sy, s->wt, col, s->wa + 2 * m, s->wa, info);
	if (*info != 0) {
		*info = -8;
		return;
	}
	int pointr = s->head;
	for (int j = 1; j <= col; j++) {
		double a1 = V1(s->wa, j), a2 = s->theta * V1(s->wa, col + j);
		for (int i = 1; i <= s->nfree; i++) {
			int k = V1(s->index, i);
			V1(s->r, i) = V1(s->r, i) + M1(s->wy, n, k, pointr) * a1 + M1(s->ws, n, k, pointr) * a2;
		}
		pointr = pointr % m + 1;
	}
}

/* subspace minimization with the projected Newton step (version 3.0) */
LB_HD void lb_subsm(lb_state *s, int *info)
{
	const int n = LB_N, m = LB_M, ld = LB_M2;
	int nsub = s->nfree, col = s->col;
	double *d = s->r, *x = s->z, *xp = s->xp, *wv = s->wa;
	const double *xx = s->x, *gg = s->g;
	const int *ind = s->index;
	if (nsub <= 0) return;
	int pointr = s->head;
	for (int i = 1; i <= col; i++) {
		double temp1 = 0.0, temp2 = 0.0;
		for (int j = 1; j <= nsub; j++) {
			int k = V1(ind, j);
			temp1 += M1(s->wy, n, k, pointr) * V1(d, j);
			temp2 += M1(s->ws, n, k, pointr) * V1(d, j);
		}
		V1(wv, i) = temp1;
		V1(wv, col + i) = s->theta * temp2;
		pointr = pointr % m + 1;
	}
	int col2 = 2 * col;
	lb_trsl(s->wn, ld, col2, wv, 11, info);
	if (*info != 0) return;
	for (int i = 1; i <= col; i++) V1(wv, i) = -V1(wv, i);
	lb_trsl(s->wn, ld, col2, wv, 1, info);
	if (*info != 0) return;
	pointr = s->head;
	for (int jy = 1; jy <= col; jy++) {
		int js = col + jy;
		for (int i = 1; i <= nsub; i++) {
			int k = V1(ind, i);
			V1(d, i) = V1(d, i) + M1(s->wy, n, k, pointr) * V1(wv, jy) / s->theta + M1(s->ws, n, k, pointr) * V1(wv, js);
		}
		pointr = pointr % m + 1;
	}
	{
		double sc = 1. / s->theta;
		for (int i = 1; i <= nsub; i++) V1(d, i) = sc * V1(d, i);
	}
	s->iword = 0;
	for (int i = 0; i < n; i++) xp[i] = x[i];
	for (int i = 1; i <= nsub; i++) {
		int k = V1(ind, i);
		double dk = V1(d, i), xk = V1(x, k);
		if (V1(s->nbd, k) != 0) {
			if (V1(s->nbd, k) == 1) {
				V1(x, k) = lb_max(V1(s->l, k), xk + dk);
				if (V1(x, k) == V1(s->l, k)) s->iword = 1;
			} else if (V1(s->nbd, k) == 2) {
				xk = lb_max(V1(s->l, k), xk + dk);
				V1(x, k) = lb_min(V1(s->u, k), xk);
				if (V1(x, k) == V1(s->l, k) || V1(x, k) == V1(s->u, k)) s->iword = 1;
			} else if (V1(s->nbd, k) == 3) {
				V1(x, k) = lb_min(V1(s->u, k), xk + dk);
				if (V1(x, k) == V1(s->u, k)) s->iword = 1;
			}
		} else {
			V1(x, k) = xk + dk;
		}
	}
	if (s->iword == 0) return;
	double dd_p = 0.0;
	for (int i = 1; i <= n; i++) dd_p += (V1(x, i) - V1(xx, i)) * V1(gg, i);
	if (dd_p > 0.0) {
		for (int i = 0; i < n; i++) x[i] = xp[i];
	} else {
		return;
	}
	double alpha = 1.0, temp1 = alpha;
	int ibd = 0;
	for (int i = 1; i <= nsub; i++) {
		int k = V1(ind, i);
		double dk = V1(d, i);
		if (V1(s->nbd, k) != 0) {
			if (dk < 0.0 && V1(s->nbd, k) <= 2) {
				double temp2 = V1(s->l, k) - V1(x, k);
				if (temp2 >= 0.0) temp1 = 0.0;
				else if (dk * alpha < temp2) temp1 = temp2 / dk;
			} else if (dk > 0.0 && V1(s->nbd, k) >= 2) {
				double temp2 = V1(s->u, k) - V1(x, k);
				if (temp2 <= 0.0) temp1 = 0.0;
				else if (dk * alpha > temp2) temp1 = temp2 / dk;
			}
			if (temp1 < alpha) {
				alpha = temp1;
				ibd = i;
			}
		}
	}
	if (alpha < 1.0) {
		double dk = V1(d, ibd);
		int k = V1(ind, ibd);
		if (dk > 0.0) {
			V1(x, k) = V1(s->u, k);
			V1(d, ibd) = 0.0;
		} else if (dk < 0.0) {
			V1(x, k) = V1(s->l, k);
			V1(d, ibd) = 0.0;
		}
	}
	for (int i = 1; i <= nsub; i++) {
		int k = V1(ind, i);
		V1(x, k) += alpha * V1(d, i);
	}
}

LB_HD void lb_matupd(lb_state *s, double rr, double dr)
{
	const int n = LB_N, m = LB_M;
	if (s->iupdat <= m) {
		s->col = s->iupdat;
		s->itail = (s->head + s->iupdat - 2) % m + 1;
	} else {
		s->itail = s->itail % m + 1;
		s->head = s->head % m + 1;
	}
	for (int i = 1; i <= n; i++) {
		M1(s->ws, n, i, s->itail) = V1(s->d, i);
		M1(s->wy, n, i, s->itail) = V1(s->r, i);
	}
	s->theta = rr / dr;
	int col = s->col;
	if (s->iupdat > m) {
		for (int j = 1; j <= col - 1; j++) {
			for (int k = 0; k < j; k++) M1(s->ss, m, 1 + k, j) = M1(s->ss, m, 2 + k, j + 1);
			for (int k = 0; k < col - j; k++) M1(s->sy, m, j + k, j) = M1(s->sy, m, j + 1 + k, j + 1);
		}
	}
	int pointr = s->head;
	for (int j = 1; j <= col - 1; j++) {
		M1(s->sy, m, col, j) = lb_dot(n, s->d, &M1(s->wy, n, 1, pointr));
		M1(s->ss, m, j, col) = lb_dot(n, &M1(s->ws, n, 1, pointr), s->d);
		pointr = pointr % m + 1;
	}
	if (s->stp == 1.0) M1(s->ss, m, col, col) = s->dtd;
	else M1(s->ss, m, col, col) = s->stp * s->stp * s->dtd;
	M1(s->sy, m, col, col) = dr;
}

LB_HD void lb_formt(lb_state *s, int *info)
{
	const int m = LB_M;
	int col = s->col;
	for (int j = 1; j <= col; j++) M1(s->wt, m, 1, j) = s->theta * M1(s->ss, m, 1, j);
	for (int i = 2; i <= col; i++)
		for (int j = i; j <= col; j++) {
			int k1 = (i < j ? i : j) - 1;
			double ddum = 0.0;
			for (int k = 1; k <= k1; k++) ddum += M1(s->sy, m, i, k) * M1(s->sy, m, j, k) / M1(s->sy, m, k, k);
			M1(s->wt, m, i, j) = ddum + s->theta * M1(s->ss, m, i, j);
		}
	lb_pofa(s->wt, m, col, info);
	if (*info != 0) *info = -3;
}

/* ----------------------------------------------- Moré-Thuente line search */
enum { LS_START = 1, LS_FG = 10, LS_CONV = 20, LS_WARN = 100, LS_ERROR = 200 };

LB_HD void lb_dcstep(double *stx, double *fx, double *dx, double *sty, double *fy, double *dy, double *stp,
                     double fp, double dp, int *brackt, double stpmin, double stpmax)
{
	double sgnd = dp * (*dx / lb_abs(*dx));
	double stpf, stpc, stpq, theta, s, gamma, p, q, r;
	if (fp > *fx) {
		theta = (*fx - fp) * 3. / (*stp - *stx) + *dx + dp;
		s = lb_max(lb_max(lb_abs(theta), lb_abs(*dx)), lb_abs(dp));
		double t1 = theta / s;
		gamma = s * sqrt(t1 * t1 - *dx / s * (dp / s));
		if (*stp < *stx) gamma = -gamma;
		p = gamma - *dx + theta;
		q = gamma - *dx + gamma + dp;
		r = p / q;
		stpc = *stx + r * (*stp - *stx);
		stpq = *stx + *dx / ((*fx - fp) / (*stp - *stx) + *dx) / 2. * (*stp - *stx);
		if (lb_abs(stpc - *stx) < lb_abs(stpq - *stx)) stpf = stpc;
		else stpf = stpc + (stpq - stpc) / 2.;
		*brackt = 1;
	} else if (sgnd < 0.0) {
		theta = (*fx - fp) * 3. / (*stp - *stx) + *dx + dp;
		s = lb_max(lb_max(lb_abs(theta), lb_abs(*dx)), lb_abs(dp));
		double t1 = theta / s;
		gamma = s * sqrt(t1 * t1 - *dx / s * (dp / s));
		if (*stp > *stx) gamma = -gamma;
		p = gamma - dp + theta;
		q = gamma - dp + gamma + *dx;
		r = p / q;
		stpc = *stp + r * (*stx - *stp);
		stpq = *stp + dp / (dp - *dx) * (*stx - *stp);
		if (lb_abs(stpc - *stp) > lb_abs(stpq - *stp)) stpf = stpc;
		else stpf = stpq;
		*brackt = 1;
	} else if (lb_abs(dp) < lb_abs(*dx)) {
		theta = (*fx - fp) * 3. / (*stp - *stx) + *dx + dp;
		s = lb_max(lb_max(lb_abs(theta), lb_abs(*dx)), lb_abs(dp));
		double t3 = theta / s;
		gamma = s * sqrt(lb_max(0., t3 * t3 - *dx / s * (dp / s)));
		if (*stp > *stx) gamma = -gamma;
		p = gamma - dp + theta;
		q = gamma + (*dx - dp) + gamma;
		r = p / q;
		if (r < 0.0 && gamma != 0.0) stpc = *stp + r * (*stx - *stp);
		else if (*stp > *stx) stpc = stpmax;
		else stpc = stpmin;
		stpq = *stp + dp / (dp - *dx) * (*stx - *stp);
		if (*brackt) {
			if (lb_abs(stpc - *stp) < lb_abs(stpq - *stp)) stpf = stpc;
			else stpf = stpq;
			if (*stp > *stx) stpf = lb_min(*stp + (*sty - *stp) * .66, stpf);
			else stpf = lb_max(*stp + (*sty - *stp) * .66, stpf);
		} else {
			if (lb_abs(stpc - *stp) > lb_abs(stpq - *stp)) stpf = stpc;
			else stpf = stpq;
			stpf = lb_min(stpmax, stpf);
			stpf = lb_max(stpmin, stpf);
		}
	} else {
		if (*brackt) {
			theta = (fp - *fy) * 3. / (*sty - *stp) + *dy + dp;
			s = lb_max(lb_max(lb_abs(theta), lb_abs(*dy)), lb_abs(dp));
			double t1 = theta / s;
			gamma = s * sqrt(t1 * t1 - *dy / s * (dp / s));
			if (*stp > *sty) gamma = -gamma;
			p = gamma - dp + theta;
			q = gamma - dp + gamma + *dy;
			r = p / q;
			stpc = *stp + r * (*sty - *stp);
			stpf = stpc;
		} else if (*stp > *stx) {
			stpf = stpmax;
		} else {
			stpf = stpmin;
		}
	}
	if (fp > *fx) {
		*sty = *stp;
		*fy = fp;
		*dy = dp;
	} else {
		if (sgnd < 0.0) {
			*sty = *stx;
			*fy = *fx;
			*dy = *dx;
		}
		*stx = *stp;
		*fx = fp;
		*dx = dp;
	}
	*stp = stpf;
}

/* one call of the line-search state machine; task in/out */
LB_HD void lb_dcsrch(lb_state *s, double f, double g, double *stp, double stpmax, int *task)
{
	const double ftol = .001, gtol = .9, xtol = .1, stpmin = 0.;
	if (*task == LS_START) {
		if (*stp < stpmin || *stp > stpmax || g >= 0.0 || stpmax < stpmin) {
			*task = LS_ERROR;
			return;
		}
		s->ls_brackt = 0;
		s->ls_stage = 1;
		s->ls_finit = f;
		s->ls_ginit = g;
		s->ls_gtest = ftol * s->ls_ginit;
		s->ls_width = stpmax - stpmin;
		s->ls_width1 = s->ls_width / .5;
		s->ls_stx = 0.0;
		s->ls_fx = s->ls_finit;
		s->ls_gx = s->ls_ginit;
		s->ls_sty = 0.0;
		s->ls_fy = s->ls_finit;
		s->ls_gy = s->ls_ginit;
		s->ls_stmin = 0.0;
		s->ls_stmax = *stp + *stp * 4.;
		*task = LS_FG;
		return;
	}
	double ftest = s->ls_finit + *stp * s->ls_gtest;
	if (s->ls_stage == 1 && f <= ftest && g >= 0.0) s->ls_stage = 2;
	if (s->ls_brackt && (*stp <= s->ls_stmin || *stp >= s->ls_stmax)) *task = LS_WARN;
	if (s->ls_brackt && s->ls_stmax - s->ls_stmin <= xtol * s->ls_stmax) *task = LS_WARN;
	if (*stp == stpmax && f <= ftest && g <= s->ls_gtest) *task = LS_WARN;
	if (*stp == stpmin && (f > ftest || g >= s->ls_gtest)) *task = LS_WARN;
	if (f <= ftest && lb_abs(g) <= gtol * (-s->ls_ginit)) *task = LS_CONV;
	if (*task == LS_WARN || *task == LS_CONV) return;
	if (s->ls_stage == 1 && f <= s->ls_fx && f > ftest) {
		double fm = f - *stp * s->ls_gtest;
		double fxm = s->ls_fx - s->ls_stx * s->ls_gtest;
		double fym = s->ls_fy - s->ls_sty * s->ls_gtest;
		double gm = g - s->ls_gtest;
		double gxm = s->ls_gx - s->ls_gtest;
		double gym = s->ls_gy - s->ls_gtest;
		lb_dcstep(&s->ls_stx, &fxm, &gxm, &s->ls_sty, &fym, &gym, stp, fm, gm, &s->ls_brackt, s->ls_stmin,
		          s->ls_stmax);
		s->ls_fx = fxm + s->ls_stx * s->ls_gtest;
		s->ls_fy = fym + s->ls_sty * s->ls_gtest;
		s->ls_gx = gxm + s->ls_gtest;
		s->ls_gy = gym + s->ls_gtest;
	} else {
		lb_dcstep(&s->ls_stx, &s->ls_fx, &s->ls_gx, &s->ls_sty, &s->ls_fy, &s->ls_gy, stp, f, g, &s->ls_brackt,
		          s->ls_stmin, s->ls_stmax);
	}
	if (s->ls_brackt) {
		if (lb_abs(s->ls_sty - s->ls_stx) >= s->ls_width1 * .66) *stp = s->ls_stx + (s->ls_sty - s->ls_stx) * .5;
		s->ls_width1 = s->ls_width;
		s->ls_width = lb_abs(s->ls_sty - s->ls_stx);
	}
	if (s->ls_brackt) {
		s->ls_stmin = lb_min(s->ls_stx, s->ls_sty);
		s->ls_stmax = lb_max(s->ls_stx, s->ls_sty);
	} else {
		s->ls_stmin = *stp + (*stp - s->ls_stx) * 1.1;
		s->ls_stmax = *stp + (*stp - s->ls_stx) * 4.;
	}
	*stp = lb_max(*stp, stpmin);
	*stp = lb_min(*stp, stpmax);
	if ((s->ls_brackt && (*stp <= s->ls_stmin || *stp >= s->ls_stmax)) ||
	    (s->ls_brackt && s->ls_stmax - s->ls_stmin <= xtol * s->ls_stmax))
		*stp = s->ls_stx;
	*task = LS_FG;
}

/* ------------------------------------------------ the SAXS objective */

typedef struct {
	const double *cr; /* cross terms VV,VD,VW,DD,DW,WW at cr[(c*Q + i) * stride] */
	long stride;
	const double *q, *a;
	double mult;
	int Q;
} lb_saxs;

#define LB_X(o, c, i) ((o)->cr[((long)(c) * (o)->Q + (i)) * (o)->stride])

LB_HD double lb_in(const lb_saxs *o, int i, double G, double c2)
{
	return LB_X(o, 0, i) - G * LB_X(o, 1, i) + c2 * LB_X(o, 2, i) + G * G * LB_X(o, 3, i) - G * c2 * LB_X(o, 4, i) +
	       c2 * c2 * LB_X(o, 5, i);
}

/* sxs_best_scale (src/min_saxs.c:261-319) */
LB_HD double lb_best_scale(const lb_saxs *o, double c1, double c2)
{
	const double *q = o->q, *a = o->a;
	double corr = -o->mult * (c1 * c1 - 1.0);
	double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
	double in_prev = lb_in(o, 0, G, c2);
	double c1c = c1 * c1 * c1, q_prev = -1.0, up = 0.0, down = 0.0;
	for (int i = 0; i < o->Q; i++) {
		double qc = q[i];
		G = c1c * exp(corr * qc * qc);
		double in = lb_in(o, i, G, c2);
		double tan = (in - in_prev) / (qc - q_prev);
		double buf = in - tan * qc;
		up += buf * a[i * 6 + 1] + tan * a[i * 6 + 2];
		down += buf * buf * a[i * 6 + 3] + 2.0 * tan * buf * a[i * 6 + 4] + tan * tan * a[i * 6 + 5];
		in_prev = in;
		q_prev = qc;
	}
	return up / down;
}

/* gradient and chi^2 at fixed scale k (src/min_saxs.c:3-105) */
LB_HD void lb_gradient(const lb_saxs *o, const double *x, double k, double *grad, double *score_val)
{
	const double *q = o->q, *a = o->a;
	double c1 = x[0], c2 = x[1], mult = o->mult;
	double g0 = 0.0, g1 = 0.0;
	double corr = -mult * (c1 * c1 - 1.0);
	double G = c1 * c1 * c1 * exp(corr * q[0] * q[0]);
	double G_der = G * (3.0 / c1 - 2.0 * c1 * mult * q[0] * q[0]);
	double in_prev = lb_in(o, 0, G, c2);
	double idc1_prev = -G_der * LB_X(o, 1, 0) + 2.0 * G * G_der * LB_X(o, 3, 0) - G_der * c2 * LB_X(o, 4, 0);
	double idc2_prev = LB_X(o, 2, 0) - G * LB_X(o, 4, 0) + 2.0 * c2 * LB_X(o, 5, 0);
	double q_prev = -1.0, score = 0.0, c1c = c1 * c1 * c1;
	for (int i = 0; i < o->Q; i++) {
		double qc = q[i];
		G = c1c * exp(corr * qc * qc);
		G_der = G * (3.0 / c1 - 2.0 * c1 * mult * qc * qc);
		double in = lb_in(o, i, G, c2);
		double idc1 = G_der * (-LB_X(o, 1, i) + 2.0 * G * LB_X(o, 3, i) - c2 * LB_X(o, 4, i));
		double idc2 = LB_X(o, 2, i) - G * LB_X(o, 4, i) + 2.0 * c2 * LB_X(o, 5, i);
		double buf = 1.0 / (qc - q_prev);
		double tan = (in - in_prev) * buf;
		double t1 = (idc1 - idc1_prev) * buf;
		double t2 = (idc2 - idc2_prev) * buf;
		const double *ai = a + i * 6;
		g0 += 2.0 * k * (-(idc1 - t1 * qc) * ai[1] - t1 * ai[2] +
		                 k * ((in - tan * qc) * (idc1 - t1 * qc) * ai[3] +
		                      (in * t1 + idc1 * tan - 2.0 * tan * t1 * qc) * ai[4] + tan * t1 * ai[5]));
		g1 += 2.0 * k * (-(idc2 - t2 * qc) * ai[1] - t2 * ai[2] +
		                 k * ((in - tan * qc) * (idc2 - t2 * qc) * ai[3] +
		                      (in * t2 + idc2 * tan - 2.0 * tan * t2 * qc) * ai[4] + tan * t2 * ai[5]));
		buf = in - tan * qc;
		score += ai[0] + k * (-2.0 * buf * ai[1] - 2.0 * tan * ai[2] +
		                      k * (buf * buf * ai[3] + 2.0 * buf * tan * ai[4] + tan * tan * ai[5]));
		in_prev = in;
		idc1_prev = idc1;
		idc2_prev = idc2;
		q_prev = qc;
	}
	grad[0] = g0;
	grad[1] = g1;
	*score_val = score;
}

/* f, g at s->x as the reference's fitting loop computes them: best scale
 * first, then gradient and chi^2 at that scale. */
LB_HD void lb_eval(lb_state *s, const lb_saxs *o, double *scale)
{
	*scale = lb_best_scale(o, s->x[0], s->x[1]);
	lb_gradient(o, s->x, *scale, s->g, &s->f);
}

LB_HD void lb_reset_memory(lb_state *s)
{
	s->info = 0;
	s->col = 0;
	s->head = 1;
	s->theta = 1.0;
	s->iupdat = 0;
	s->updatd = 0;
}

/* The fit of src/min_saxs.c:196-259: x0 = (1, 0), bounds [0.96, 1.04] x
 * [-2, 4], m = 3, factr = 1e7, pgtol = 1e-5.  Returns the number of
 * objective evaluations; chi = sqrt(f), scale = best scale at the result.
 * max_eval bounds the work per pose (the reference has no bound; the
 * algorithm stops long before it in practice). */
LB_HD int lb_saxs_fit(const lb_saxs *o, double *chi, double *c1, double *c2, double *scale, int max_eval)
{
	lb_state st;
	lb_state *s = &st;
	const int n = LB_N;
	s->x[0] = 1.0; s->x[1] = 0.0;
	s->l[0] = 0.96; s->l[1] = -2.00;
	s->u[0] = 1.04; s->u[1] = 4.00;
	s->nbd[0] = 2; s->nbd[1] = 2;
	for (int i = 0; i < LB_M2 * LB_M2; i++) { s->wn[i] = 0.0; s->snd[i] = 0.0; }
	for (int i = 0; i < LB_M * LB_M; i++) { s->sy[i] = 0.0; s->ss[i] = 0.0; s->wt[i] = 0.0; }
	for (int i = 0; i < LB_N * LB_M; i++) { s->ws[i] = 0.0; s->wy[i] = 0.0; }
	for (int i = 0; i < 8 * LB_M; i++) s->wa[i] = 0.0;
	for (int i = 0; i < n; i++) {
		s->z[i] = s->r[i] = s->d[i] = s->t[i] = s->xp[i] = 0.0;
		s->index[i] = s->iwhere[i] = s->indx2[i] = 0;
	}
	s->epsmch = DBL_EPSILON;
	s->col = 0; s->head = 1; s->theta = 1.0; s->iupdat = 0; s->updatd = 0;
	s->iback = 0; s->itail = 0; s->iword = 0; s->nenter = 0; s->ileave = 0;
	s->fold = 0.0; s->dnorm = 0.0; s->gd = 0.0; s->stpmx = 0.0; s->sbgnrm = 0.0; s->stp = 0.0;
	s->gdold = 0.0; s->dtd = 0.0; s->iter = 0; s->nfgv = 0; s->nseg = 0; s->nfree = n; s->ifun = 0;
	s->tol = 1e+7 * s->epsmch;
	s->info = 0;
	s->ls_task = 0;
	/* active: project x0, classify variables */
	s->prjctd = 0; s->cnstnd = 0; s->boxed = 1;
	for (int i = 1; i <= n; i++) {
		if (V1(s->nbd, i) > 0) {
			if (V1(s->nbd, i) <= 2 && V1(s->x, i) <= V1(s->l, i)) {
				if (V1(s->x, i) < V1(s->l, i)) { s->prjctd = 1; V1(s->x, i) = V1(s->l, i); }
			} else if (V1(s->nbd, i) >= 2 && V1(s->x, i) >= V1(s->u, i)) {
				if (V1(s->x, i) > V1(s->u, i)) { s->prjctd = 1; V1(s->x, i) = V1(s->u, i); }
			}
		}
	}
	for (int i = 1; i <= n; i++) {
		if (V1(s->nbd, i) != 2) s->boxed = 0;
		if (V1(s->nbd, i) == 0) {
			V1(s->iwhere, i) = -1;
		} else {
			s->cnstnd = 1;
			V1(s->iwhere, i) = (V1(s->nbd, i) == 2 && V1(s->u, i) - V1(s->l, i) <= 0.0) ? 3 : 0;
		}
	}
	int nevals = 0;
	double sc = 1.0;
	lb_eval(s, o, &sc);
	nevals++;
	s->nfgv = 1;
	lb_projgr(s, &s->sbgnrm);
	const double pgtol = 1e-5;
	if (s->sbgnrm <= pgtol) goto done;
	for (;;) {
		/* L222 */
		s->iword = -1;
		int wrk = 0, info = 0;
		if (!s->cnstnd && s->col > 0) {
			for (int i = 0; i < n; i++) s->z[i] = s->x[i];
			wrk = s->updatd;
			s->nseg = 0;
		} else {
			lb_cauchy(s, &info);
			if (info != 0) {
				lb_reset_memory(s);
				continue;
			}
			lb_freev(s, &wrk);
		}
		/* L333 */
		if (s->nfree != 0 && s->col != 0) {
			if (wrk) lb_formk(s, &info);
			if (info != 0) {
				lb_reset_memory(s);
				continue;
			}
			lb_cmprlb(s, &info);
			if (info == 0) lb_subsm(s, &info);
			if (info != 0) {
				lb_reset_memory(s);
				continue;
			}
		}
		/* L555: line search along d = z - x */
		for (int i = 0; i < n; i++) s->d[i] = s->z[i] - s->x[i];
		s->dtd = lb_dot(n, s->d, s->d);
		s->dnorm = sqrt(s->dtd);
		s->stpmx = 1e10;
		if (s->cnstnd) {
			if (s->iter == 0) {
				s->stpmx = 1.0;
			} else {
				for (int i = 1; i <= n; i++) {
					double a1 = V1(s->d, i);
					if (V1(s->nbd, i) != 0) {
						if (a1 < 0.0 && V1(s->nbd, i) <= 2) {
							double a2 = V1(s->l, i) - V1(s->x, i);
							if (a2 >= 0.0) s->stpmx = 0.0;
							else if (a1 * s->stpmx < a2) s->stpmx = a2 / a1;
						} else if (a1 > 0.0 && V1(s->nbd, i) >= 2) {
							double a2 = V1(s->u, i) - V1(s->x, i);
							if (a2 <= 0.0) s->stpmx = 0.0;
							else if (a1 * s->stpmx > a2) s->stpmx = a2 / a1;
						}
					}
				}
			}
		}
		if (s->iter == 0 && !s->boxed) s->stp = lb_min(1.0 / s->dnorm, s->stpmx);
		else s->stp = 1.0;
		for (int i = 0; i < n; i++) { s->t[i] = s->x[i]; s->r[i] = s->g[i]; }
		s->fold = s->f;
		s->ifun = 0;
		s->iback = 0;
		int task = LS_START;
		int new_x = 0;
		for (;;) {
			s->gd = lb_dot(n, s->g, s->d);
			if (s->ifun == 0) {
				s->gdold = s->gd;
				if (s->gd >= 0.0) {
					s->info = -4;
					break;
				}
			}
			lb_dcsrch(s, s->f, s->gd, &s->stp, s->stpmx, &task);
			s->xstep = s->stp * s->dnorm;
			if (task != LS_WARN && task != LS_CONV) {
				++s->ifun;
				++s->nfgv;
				s->iback = s->ifun - 1;
				if (s->stp == 1.0) {
					for (int i = 0; i < n; i++) s->x[i] = s->z[i];
				} else {
					for (int i = 0; i < n; i++) s->x[i] = s->stp * s->d[i] + s->t[i];
				}
				if (s->iback >= 20) break; /* checked before the evaluation */
				if (nevals >= max_eval) goto done;
				lb_eval(s, o, &sc);
				nevals++;
			} else {
				new_x = 1;
				break;
			}
		}
		if (!new_x || s->info != 0) {
			/* restore the previous iterate */
			for (int i = 0; i < n; i++) { s->x[i] = s->t[i]; s->g[i] = s->r[i]; }
			s->f = s->fold;
			if (s->col == 0) {
				goto done; /* abnormal termination */
			}
			lb_reset_memory(s);
			continue;
		}
		++s->iter;
		lb_projgr(s, &s->sbgnrm);
		/* L777: termination tests */
		if (s->sbgnrm <= pgtol) goto done;
		{
			double ddum = lb_max(lb_max(lb_abs(s->fold), lb_abs(s->f)), 1.0);
			if (s->fold - s->f <= s->tol * ddum) goto done;
		}
		for (int i = 0; i < n; i++) s->r[i] = s->g[i] - s->r[i];
		double rr = lb_dot(n, s->r, s->r), dr, ddum;
		if (s->stp == 1.0) {
			dr = s->gd - s->gdold;
			ddum = -s->gdold;
		} else {
			dr = (s->gd - s->gdold) * s->stp;
			for (int i = 0; i < n; i++) s->d[i] = s->stp * s->d[i];
			ddum = -s->gdold * s->stp;
		}
		if (dr <= s->epsmch * ddum) {
			s->updatd = 0;
			continue;
		}
		s->updatd = 1;
		++s->iupdat;
		lb_matupd(s, rr, dr);
		int finfo = 0;
		lb_formt(s, &finfo);
		if (finfo != 0) lb_reset_memory(s);
	}
done:
	*chi = sqrt(s->f);
	*c1 = s->x[0];
	*c2 = s->x[1];
	*scale = lb_best_scale(o, s->x[0], s->x[1]);
	return nevals;
}

#endif
