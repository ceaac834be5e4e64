/*
 * FP64 kernels whose rounding must follow the reference operation by
 * operation: the spherical-Bessel power series (its cancellation at large
 * q*r amplifies any reordering), the associated-Legendre recurrence, the
 * translation-matrix p-sum, the A_lm accumulation and the self terms.
 *
 * This translation unit is compiled with -fmad=false so that no multiply-add
 * is contracted: every expression below is evaluated in the reference's
 * order with one rounding per operation, as gcc -std=c11 does on the host.
 */
#include "kernels.h"

#include <math.h>

#define SXS_PI 3.14159265358 /* the reference's pi (src/define.h:14-16 under -std=c11) */

namespace {

__device__ __forceinline__ int lm_index(int l, int m) { return l * (l + 1) + m; }

/* (2l+1)!! as the reference's doublefact (src/sfbessel.c:21-37). */
__device__ double odd_factorial(int n)
{
	double r = 1.0;
	for (int i = 1; i <= n; i += 2) r *= (double)i;
	return r;
}

/* j_l(x) by the reference's truncated power series (src/sfbessel.c:40-60). */
__device__ double sbessel(int l, double x)
{
	if (x > 0.0) {
		double tl1 = 2.0 * (double)l + 1.0;
		double term = 1.0 / odd_factorial((int)tl1);
		double sum = term;
		/* the reference has no iteration bound; terms decay factorially, so
		 * the cap (far above any count the series reaches) only guards
		 * against non-finite input */
		for (int k = 1; fabs(term / sum) > 0.00001 && k < 100000; k++) {
			double ratio = ((-1.0) * x * x) / ((2.0 * (double)k) * (2.0 * (double)k + tl1));
			term = term * ratio;
			sum = sum + term;
		}
		return sum * pow(x, (double)l);
	}
	return l == 0 ? 1.0 : 0.0;
}

/* Per atom and m >= 0: P_l^m(cos theta) by the recurrence of
 * src/borrowed.c:40-65 (N = L+1), times the Y norm, times e^{-i m phi}
 * (src/pdb2spf.c:76-84), written for +m and -m. */
__global__ void k_ylm(const double *__restrict__ xyz, int natoms, int L, const double *__restrict__ ynorm,
                      double2 *__restrict__ ylm, double *__restrict__ rad)
{
	int K = L + 1, K2 = K * K;
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)natoms * K) return;
	int a = (int)(t / K), m = (int)(t % K);
	double x = xyz[3 * a], y = xyz[3 * a + 1], z = xyz[3 * a + 2];
	double r = sqrt(x * x + y * y + z * z);
	if (m == 0 && rad) rad[a] = r;
	double th = acos(z / r);
	double ph;
	if (y > 0.0) ph = acos(x / sqrt(x * x + y * y));
	else ph = -acos(x / sqrt(x * x + y * y)) + 2.0 * SXS_PI;
	double c = cos(th);
	double s = sqrt(1. - c * c);
	int N = K;
	/* P_m^m: the reference's diagonal chain (lines 54 and 63 agree on the
	 * formula), then P_{m+1}^m and the upward recurrence in l. */
	double pmm = 1;
	for (int j = 1; j <= m; j++) pmm = -1. * (2. * j - 1.) * s * pmm;
	double p_lm2 = 0.0, p_lm1 = pmm;
	double2 *out = ylm + (size_t)a * K2;
	for (int l = m; l < N; l++) {
		double p;
		if (l == m) {
			p = pmm;
		} else if (l == m + 1) {
			if (m == 0) p = c;                          /* P_1^0 = x */
			else p = (2. * m + 1.) * c * pmm;           /* P_{m+1}^m */
		} else {
			if (m == 0) p = (2. * l - 1.) / l * c * p_lm1 - (l - 1.) / l * p_lm2;
			else p = (2. * l - 1.) / (l - m) * c * p_lm1 - (l + m - 1.) / (l - m) * p_lm2;
		}
		p_lm2 = p_lm1;
		p_lm1 = p;
		if (l == m) { p_lm2 = 0.0; p_lm1 = p; }
		double hp = ynorm[l * (2 * L + 1) + (m + L)] * p;
		out[lm_index(l, m)] = make_double2(hp * cos(ph * m), hp * sin(-ph * m));
		if (m > 0) {
			double hn = ynorm[l * (2 * L + 1) + (-m + L)] * p;
			out[lm_index(l, -m)] = make_double2(hn * cos(ph * (-m)), hn * sin(-ph * (-m)));
		}
	}
}

/* series terms whose divisor (2k)(2k + 2l + 1) and its reciprocal a block
 * of k_expand_ql stages for its l */
#define EXP_KTAB 128

/* num / den, correctly rounded, for an integer den > 0 with y = 1/den
 * rounded to nearest and |num| a normal number: q0 = num y, the remainder
 * num - den q0 exactly by an FMA, and one correction q0 + r y (Markstein's
 * final division step, P. Markstein, "Computation of elementary functions
 * on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34 (1990)): three
 * FP64 operations instead of a full division.  Checked against IEEE
 * division on 3.1e8 (num, den) pairs of this series' range with no
 * difference. */
__device__ __forceinline__ double div_by_int(double num, double den, double y)
{
	double q0 = num * y;
	double r = fma(-q0, den, num);
	return fma(r, y, q0);
}

/* j_l(x) with the series of sbessel and the same value: the same terms in
 * the same order, with three changes that leave the rounded series alone.
 * The stop test fabs(term / sum) > 1e-5 is decided by comparing |term|
 * with |sum| 1e-5 (1 +- 1e-10), whose rounding errors are far below that
 * margin; only a quotient within the margin is divided out.  The ratio of
 * consecutive terms, -x^2 / ((2k)(2k + 2l + 1)), is divided as above with
 * the block's table dk[k] = {(2k)(2k + 2l + 1), its reciprocal} for k <
 * EXP_KTAB.  x^l is a chain of products instead of pow (a few ulps,
 * outside the cancelling sum).  term0 = 1 / (2l+1)!! is the block's. */
__device__ __forceinline__ double sbessel_fast(int l, double x, double term0, const double2 *dk)
{
	if (x > 0.0) {
		double tl1 = 2.0 * (double)l + 1.0;
		double num = (-1.0) * x * x;
		double term = term0, sum = term0;
		const double c = 0.00001, hi = c * (1.0 + 1e-10), lo = c * (1.0 - 1e-10);
		bool tiny = fabs(num) < 0x1p-900;   /* keep the division where num is near the subnormals */
		for (int k = 1; k < 100000; k++) {
			double at = fabs(term), as = fabs(sum);
			bool go;
			if (at > as * hi) go = true;
			else if (at < as * lo) go = false;
			else go = fabs(term / sum) > c;
			if (!go) break;
			double ratio;
			if (k < EXP_KTAB && !tiny) {
				double2 d = dk[k];
				ratio = div_by_int(num, d.x, d.y);
			} else {
				ratio = num / ((2.0 * (double)k) * (2.0 * (double)k + tl1));
			}
			term = term * ratio;
			sum = sum + term;
		}
		double xl = 1.0;
		for (int i = 0; i < l; i++) xl = xl * x;
		return sum * xl;
	}
	return l == 0 ? 1.0 : 0.0;
}

#define EXP_THREADS 128

/* A[ch][q][l m] for one (q, l) per block: atoms in tiles of EXP_THREADS,
 * staged through shared memory as w_ch = f_ch(a) j_l(q r_a) (one series
 * per thread), then accumulated against Y*_lm(a) by (m, slice) threads,
 * each slice a fixed residue class of the tile's atoms; the slices are
 * summed in order and the 4 pi i^l phase applied (src/pdb2spf.c:104-147).
 * Deterministic: the same partition and order on every run. */
__global__ void __launch_bounds__(EXP_THREADS) k_expand_ql(const double2 *__restrict__ ylm,
                                                            const double *__restrict__ rad,
                                                            const double *__restrict__ vac,
                                                            const double *__restrict__ dum,
                                                            const double *__restrict__ wfac, int natoms,
                                                            const double *__restrict__ q, int Q, int L,
                                                            double *__restrict__ spf)
{
	__shared__ double w[3][EXP_THREADS];
	__shared__ double red[EXP_THREADS][6];
	int K = L + 1, K2 = K * K;
	int iq = blockIdx.x / K, l = blockIdx.x % K;
	int nm = 2 * l + 1, nslice = EXP_THREADS / nm;
	int t = threadIdx.x;
	int mi = t % nm, sl = t / nm;
	bool acc_thread = sl < nslice;
	double qv = q[iq];
	double term0 = 1.0 / odd_factorial(2 * l + 1);
	__shared__ double2 dk[EXP_KTAB];
	for (int k = t; k < EXP_KTAB; k += blockDim.x) {
		double den = (2.0 * (double)k) * (2.0 * (double)k + (2.0 * (double)l + 1.0));
		dk[k] = make_double2(den, k > 0 ? 1.0 / den : 0.0);
	}
	__syncthreads();
	double a6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
	const double2 *yl = ylm + l * l;   /* this l's first (l, m) of every atom row */
	for (int a0 = 0; a0 < natoms; a0 += EXP_THREADS) {
		int a = a0 + t;
		if (a < natoms) {
			double j = sbessel_fast(l, qv * rad[a], term0, dk);
			w[0][t] = vac[a] * j;
			w[1][t] = dum[a] * j;
			w[2][t] = wfac[a] * j;
		}
		__syncthreads();
		if (acc_thread) {
			int na = min(EXP_THREADS, natoms - a0);
			for (int k = sl; k < na; k += nslice) {
				double2 y = yl[(size_t)(a0 + k) * K2 + mi];
				double wv = w[0][k], wd = w[1][k], ww = w[2][k];
				a6[0] = fma(wv, y.x, a6[0]); a6[1] = fma(wv, y.y, a6[1]);
				a6[2] = fma(wd, y.x, a6[2]); a6[3] = fma(wd, y.y, a6[3]);
				a6[4] = fma(ww, y.x, a6[4]); a6[5] = fma(ww, y.y, a6[5]);
			}
		}
		__syncthreads();
	}
	if (acc_thread)
		for (int c = 0; c < 6; c++) red[t][c] = a6[c];
	__syncthreads();
	if (t < nm) {
		double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
		for (int sidx = 0; sidx < nslice; sidx++)
			for (int c = 0; c < 6; c++) v[c] = v[c] + red[sidx * nm + t][c];
		const double fp = 4.0 * SXS_PI;
		double cre[4] = {fp, 0.0, -fp, 0.0}, cim[4] = {0.0, fp, 0.0, -fp};
		double c_r = cre[l % 4], c_i = cim[l % 4];
		size_t chs = (size_t)Q * K2 * 2;
		double *o = spf + ((size_t)iq * K2 + l * l + t) * 2;
		o[0] = c_r * v[0] - c_i * v[1];           o[1] = c_r * v[1] + c_i * v[0];
		o[chs] = c_r * v[2] - c_i * v[3];         o[chs + 1] = c_r * v[3] + c_i * v[2];
		o[2 * chs] = c_r * v[4] - c_i * v[5];     o[2 * chs + 1] = c_r * v[5] + c_i * v[4];
	}
}

/* bes[iz][p][q] = j_p(z q) (src/fftsaxs.c:110-121), q fastest. */
__global__ void k_bessel_z(const double *__restrict__ z, int nz, const double *__restrict__ q, int Q, int L,
                           double *__restrict__ bes)
{
	int N = 2 * L + 1;
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)nz * Q * N) return;
	int iq = (int)(t % Q);
	long r2 = t / Q;
	int p = (int)(r2 % N), iz = (int)(r2 / N);
	bes[t] = sbessel(p, z[iz] * q[iq]);
}
/* T^{|m|}_{l l1}(q z) = sum_p (-1)^m i^p j_p d_lm(l1,p) for l <= l1, mirrored
 * (src/fftsaxs.c:182-243).  Thread = (iz, m, l, l1 >= l, q), q fastest.
 * Output in the q-tiled layout of the contraction tables (tiles of SXS_QT q).
 * The 3j factor 3j(l p l1; 0 0 0) vanishes unless l + p + l1 is even, so T
 * is real for even l + l1 and imaginary for odd l + l1 (the other part is
 * the sum of exact zeros and binary128 round-off below 1e-30 relative); the
 * table keeps that one real number, tau = Re T (even) or Im T (odd). */
__global__ void k_tmatrix(const double *__restrict__ bes, const double *__restrict__ ds, int nz, int Q, int L,
                          const int2 *__restrict__ ll1, int nll1, double *__restrict__ tau)
{
	int K = L + 1, N = 2 * L + 1;
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)nz * (K) * nll1 * Q) return;
	int iq = (int)(t % Q);
	long r2 = t / Q;
	int j = (int)(r2 % nll1);
	r2 /= nll1;
	int m = (int)(r2 % K), iz = (int)(r2 / K);
	int l = ll1[j].x, l1 = ll1[j].y;
	if (l < m) return;
	double sgn = (m % 2 == 0) ? 1.0 : -1.0;
	const double *dp = ds + ((size_t)lm_index(l, m) * K + l1) * N;
	const double *bp = bes + (size_t)iz * N * Q + iq;
	/* the reference sums Re and Im with i^p in {1, i, -1, -i}; for the
	 * component kept here (Re for even l + l1, Im for odd) the terms with p
	 * of the other parity add +-0, so summing only p = l + l1 (mod 2), in
	 * the same order, gives the same value bit for bit */
	double v = 0.0;
	int p0 = l1 - l;  /* |l - l1| with l <= l1, same parity as l + l1 */
	int odd = (l + l1) & 1;
	for (int p = p0; p <= l + l1; p += 2) {
		double w = sgn * dp[p] * bp[(size_t)p * Q];
		/* i^p for even p: +1 (p % 4 == 0), -1 (p % 4 == 2); the imaginary unit
		 * of i^p for odd p: +1 (p % 4 == 1), -1 (p % 4 == 3) */
		int neg = odd ? ((p & 3) == 3) : ((p & 3) == 2);
		v += (neg ? -1.0 : 1.0) * w;
	}
	/* q-tiled: [tile][iz][m][l][l1][SXS_QT], tile = q / SXS_QT */
	size_t base = (((size_t)(iq / SXS_QT) * nz + iz) * K + m) * K;
	tau[((base + l) * K + l1) * SXS_QT + iq % SXS_QT] = v;
	tau[((base + l1) * K + l) * SXS_QT + iq % SXS_QT] = v;
}
/* Cross terms of single molecules (src/min_saxs.c:450-494): for each
 * molecule and q, sum over lm of |V|^2, |D|^2, |W|^2, Re(V conj D),
 * Re(V conj W), Re(D conj W) in the reference's order, the three mixed sums
 * doubled; spf in the host flat layout [mol][3][Q][K2][2], cross
 * [mol][6][Q] (VV VD VW DD DW WW).  Thread = (molecule, q). */
__global__ void k_self_cross(const double *__restrict__ spf, int nmol, int Q, int K2, double *__restrict__ cross)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)nmol * Q) return;
	int iq = (int)(t % Q);
	long mol = t / Q;
	const double *V = spf + (((size_t)mol * 3 + 0) * Q + iq) * K2 * 2;
	const double *D = spf + (((size_t)mol * 3 + 1) * Q + iq) * K2 * 2;
	const double *W = spf + (((size_t)mol * 3 + 2) * Q + iq) * K2 * 2;
	double vv = 0.0, vd = 0.0, vw = 0.0, dd = 0.0, dw = 0.0, ww = 0.0;
	for (int id = 0; id < K2; id++) {
		double vr = V[2 * id], vi = V[2 * id + 1], dr = D[2 * id], di = D[2 * id + 1];
		double wr = W[2 * id], wi = W[2 * id + 1];
		vv += vr * vr + vi * vi;
		dd += dr * dr + di * di;
		ww += wr * wr + wi * wi;
		vd += vr * dr + vi * di;
		vw += vr * wr + vi * wi;
		dw += dr * wr + di * wi;
	}
	double *o = cross + (size_t)mol * 6 * Q + iq;
	o[0] = vv;
	o[Q] = vd * 2.0;
	o[2 * Q] = vw * 2.0;
	o[3 * Q] = dd;
	o[4 * Q] = dw * 2.0;
	o[5 * Q] = ww;
}

/* Shrake-Rupley accessible fraction (the restatement the workloads use;
 * the reference takes it from libmol2's accs): block = one atom i; the
 * block scans the atoms SASA_CAP at a time for neighbours j != i with
 * |x_i - x_j| < rr_i + rr_j (rr = radius + probe), keeps them in shared
 * memory, and each thread tests its sphere points p = x_i + rr_i s_k
 * against them (buried when |p - x_j|^2 < rr_j^2).  fraction = free points
 * / npts; 0 for a zero radius.  Compiled without contraction: the same
 * arithmetic as the host restatement, point for point. */
#define SASA_CAP 512
#define SASA_PPT 8
__global__ void __launch_bounds__(128) k_sasa(const double *__restrict__ xyz, const double *__restrict__ rad, int n,
                                              double probe, const double *__restrict__ sph, int npts,
                                              double *__restrict__ frac)
{
	__shared__ double nb[SASA_CAP][4];
	__shared__ int cnt;
	__shared__ int nfree[128];
	int i = blockIdx.x;
	double ri = rad[i];
	if (ri <= 0.0) {
		if (threadIdx.x == 0) frac[i] = 0.0;
		return;
	}
	double xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2];
	double rri = ri + probe;
	/* points of this thread: k = threadIdx.x + j blockDim.x, j < SASA_PPT */
	unsigned freebits = 0;
	for (int j = 0; j < SASA_PPT; j++)
		if (threadIdx.x + j * (int)blockDim.x < npts) freebits |= 1u << j;
	for (int j0 = 0; j0 < n; j0 += SASA_CAP) {
		__syncthreads();
		if (threadIdx.x == 0) cnt = 0;
		__syncthreads();
		int j1 = min(n, j0 + SASA_CAP);
		for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
			if (j == i) continue;
			double rrj = rad[j] + probe;
			double dx = xyz[3 * j] - xi, dy = xyz[3 * j + 1] - yi, dz = xyz[3 * j + 2] - zi;
			double d = sqrt(dx * dx + dy * dy + dz * dz);
			if (d < rri + rrj) {
				int slot = atomicAdd(&cnt, 1);   /* < SASA_CAP: at most SASA_CAP candidates per pass */
				nb[slot][0] = xyz[3 * j];
				nb[slot][1] = xyz[3 * j + 1];
				nb[slot][2] = xyz[3 * j + 2];
				nb[slot][3] = rrj * rrj;
			}
		}
		__syncthreads();
		int m = cnt;
		for (int pj = 0; pj < SASA_PPT; pj++) {
			if (!(freebits >> pj & 1u)) continue;
			int k = threadIdx.x + pj * blockDim.x;
			double px = xi + rri * sph[3 * k], py = yi + rri * sph[3 * k + 1], pz = zi + rri * sph[3 * k + 2];
			for (int t = 0; t < m; t++) {
				double ex = px - nb[t][0], ey = py - nb[t][1], ez = pz - nb[t][2];
				if (!(ex * ex + ey * ey + ez * ez >= nb[t][3])) {
					freebits &= ~(1u << pj);
					break;
				}
			}
		}
	}
	nfree[threadIdx.x] = __popc(freebits);
	__syncthreads();
	if (threadIdx.x == 0) {
		int c = 0;
		for (int t = 0; t < (int)blockDim.x; t++) c += nfree[t];
		frac[i] = (double)c / (double)npts;
	}
}

/* Self terms of fill_const (src/fftsaxs.c:27-50, 52-85): per channel pair
 * and q, sum over lm of Re(A1 conj A2) then Re(B1 conj B2), interleaved as in
 * comp_const_int, times {1,2,2,1,2,1}.  spf in the host flat layout. */
__global__ void k_const_int(const double *__restrict__ A, const double *__restrict__ B, int Q, int L,
                            double *__restrict__ cst)
{
	int K2 = (L + 1) * (L + 1);
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= 6 * Q) return;
	int c = t / Q, iq = t % Q;
	const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
	const double mul[6] = {1.0, 2.0, 2.0, 1.0, 2.0, 1.0};
	size_t chs = (size_t)Q * K2 * 2;
	const double *a1 = A + pa[c] * chs + (size_t)iq * K2 * 2, *a2 = A + pb[c] * chs + (size_t)iq * K2 * 2;
	const double *b1 = B + pa[c] * chs + (size_t)iq * K2 * 2, *b2 = B + pb[c] * chs + (size_t)iq * K2 * 2;
	double s = 0.0;
	for (int i = 0; i < K2; i++) {
		s += a1[2 * i] * a2[2 * i] + a1[2 * i + 1] * a2[2 * i + 1];
		s += b1[2 * i] * b2[2 * i] + b1[2 * i + 1] * b2[2 * i + 1];
	}
	cst[t] = s * mul[c];
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

} // namespace

extern "C" {

size_t sxsk_expand_ws_ylm(int natoms, int L) { return (size_t)natoms * (L + 1) * (L + 1) * sizeof(double2); }
size_t sxsk_expand_ws_rad(int natoms) { return (size_t)natoms * sizeof(double); }

int sxsk_expand(const double *xyz, const double *vac, const double *dum, const double *wfac, int natoms,
                 const double *q, int Q, int L, const double *ynorm, double2 *ylm_ws, double *rad_ws,
                 double *spf_out, cudaStream_t s)
{
	int K = L + 1;
	if (natoms <= 0) {
		cudaMemsetAsync(spf_out, 0, (size_t)3 * Q * K * K * 2 * sizeof(double), s);
		return cudaGetLastError();
	}
	if ((long)Q * K > 0x7fffffffL) return cudaErrorInvalidValue;
	k_ylm<<<nblk((long)natoms * K, 128), 128, 0, s>>>(xyz, natoms, L, ynorm, ylm_ws, rad_ws);
	k_expand_ql<<<Q * K, EXP_THREADS, 0, s>>>(ylm_ws, rad_ws, vac, dum, wfac, natoms, q, Q, L, spf_out);
	return cudaGetLastError();
}

/* kernel launches of one sxsk_expand call with atoms */
int sxsk_expand_launches(void) { return 2; }

int sxsk_bessel_z(const double *z, int nz, const double *q, int Q, int L, double *bes, cudaStream_t s)
{
	long n = (long)nz * Q * (2 * L + 1);
	if (n == 0) return 0;
	k_bessel_z<<<nblk(n, 128), 128, 0, s>>>(z, nz, q, Q, L, bes);
	return cudaGetLastError();
}

int sxsk_self_cross(const double *spf, int nmol, int Q, int L, double *cross, cudaStream_t s)
{
	long n = (long)nmol * Q;
	if (n <= 0) return 0;
	k_self_cross<<<nblk(n, 128), 128, 0, s>>>(spf, nmol, Q, (L + 1) * (L + 1), cross);
	return cudaGetLastError();
}

int sxsk_sasa(const double *xyz, const double *rad, int n, double probe, const double *sph, int npts, double *frac,
              cudaStream_t s)
{
	if (n <= 0) return 0;
	if (npts <= 0 || npts > 128 * SASA_PPT) return cudaErrorInvalidValue;
	k_sasa<<<n, 128, 0, s>>>(xyz, rad, n, probe, sph, npts, frac);
	return cudaGetLastError();
}

int sxsk_tmatrix(const double *bes, const double *dsymb, int nz, int Q, int L, const int2 *ll1, int nll1,
                 double *tau, cudaStream_t s)
{
	int K = L + 1;
	long n = (long)nz * K * nll1 * Q;
	if (n == 0) return 0;
	size_t nt = (size_t)(Q + SXS_QT - 1) / SXS_QT;
	cudaMemsetAsync(tau, 0, nt * nz * K * K * K * SXS_QT * sizeof(double), s);
	k_tmatrix<<<nblk(n, 128), 128, 0, s>>>(bes, dsymb, nz, Q, L, ll1, nll1, tau);
	return cudaGetLastError();
}

int sxsk_const_int(const double *A, const double *B, int Q, int L, double *cst, cudaStream_t s)
{
	k_const_int<<<nblk(6 * Q, 64), 64, 0, s>>>(A, B, Q, L, cst);
	return cudaGetLastError();
}

} // extern "C"

/* ------------------------------------------------------------------------
 * Expansion with no allocation (sxsg_expand_noalloc).
 *
 * For callers that must not allocate device memory themselves or through
 * this library: code that receives all device memory from a host
 * application's own pool, or runs where a (synchronising) cudaMalloc is not
 * allowed.  The work buffers of the expansion (Y_lm norms, Y_lm per atom,
 * j_l(q r) per atom) live in one file-scope device array of fixed size that
 * every GPU which loads this library keeps until the process exits.
 * ---------------------------------------------------------------------- */
#include <mutex>

#define SXS_NOALLOC_DOUBLES (8u * 1024u * 1024u) /* 64 MiB of doubles */
#define SXS_NOALLOC_LMAX 40

static __device__ __align__(256) double g_noalloc_scratch[SXS_NOALLOC_DOUBLES];

extern "C" void sxs_count_launches(int n);

/* The Y_lm normalisation table y[l][m + L] = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!),
 * times (-1)^m for -m, zero for |m| > l: the arithmetic of sxs_ynorm_host
 * (src/borrowed.c:19-38) in the same order with IEEE division and square
 * root, so both give the same bits.  One thread per l. */
__global__ void k_ynorm(int L, double *__restrict__ y)
{
	int l = blockIdx.x * blockDim.x + threadIdx.x;
	if (l > L) return;
	int N = 2 * L + 1;
	double *row = y + (size_t)l * N;
	for (int m = l + 1; m <= L; m++) {
		row[m + L] = 0.0;
		row[-m + L] = 0.0;
	}
	double fact = 1.;
	double tmp0 = __ddiv_rn(2 * l + 1., 4. * SXS_PI);
	for (int m = 0; m <= l; m++) {
		if (m > 0) fact = __dmul_rn(fact, (double)((l - m + 1) * (l + m)));
		double tmp = __dsqrt_rn(__ddiv_rn(tmp0, fact));
		double sgn = (m % 2 == 0) ? 1 : -1;
		row[m + L] = tmp;
		row[-m + L] = __dmul_rn(sgn, tmp);
	}
}

namespace {
std::mutex g_noalloc_lock;
double *g_noalloc_ptr[64]; /* device address of the scratch array, per device */
} // namespace

extern "C" int sxsg_expand_noalloc(const double *xyz, const double *vac, const double *dum, const double *water_w,
                                   int natoms, const double *q, int Q, int L, double *spf_out, void *stream)
{
	if (natoms < 0 || Q < 1 || Q > 4096 || L < 1 || L > SXS_NOALLOC_LMAX || !q || !spf_out ||
	    (natoms > 0 && (!xyz || !vac || !dum)))
		return -2;
	int K = L + 1, N = 2 * L + 1, K2 = K * K;
	/* layout in doubles: ynorm | Y_lm (complex) | radii | zero water weights */
	size_t off_y = ((size_t)K * N + 31) / 32 * 32;
	size_t off_r = off_y + ((size_t)natoms * K2 * 2 + 31) / 32 * 32;
	size_t off_w = off_r + ((size_t)natoms + 31) / 32 * 32;
	size_t need = off_w + (water_w ? 0 : (size_t)natoms);
	if (need > SXS_NOALLOC_DOUBLES) return -3;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -4;
	double *base;
	{
		std::lock_guard<std::mutex> lk(g_noalloc_lock);
		if (!g_noalloc_ptr[dev]) {
			void *p = NULL;
			cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
			if (e != cudaSuccess || !p) return (int)(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
			g_noalloc_ptr[dev] = (double *)p;
		}
		base = g_noalloc_ptr[dev];
	}
	cudaStream_t s = (cudaStream_t)stream;
	/* every call rewrites the norm table: a call with another L may have
	 * left other values there */
	k_ynorm<<<1, 64, 0, s>>>(L, base);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return (int)e;
	sxs_count_launches(1);
	const double *w = water_w;
	if (!w && natoms > 0) {
		/* no hydration shell: the weights must start at zero on every call */
		e = cudaMemsetAsync(base + off_w, 0, sizeof(double) * natoms, s);
		if (e != cudaSuccess) return (int)e;
		w = base + off_w;
	}
	int rc = sxsk_expand(xyz, vac, dum, w, natoms, q, Q, L, base, (double2 *)(base + off_y), base + off_r, spf_out, s);
	sxs_count_launches(natoms > 0 ? sxsk_expand_launches() : 0);
	return rc;
}
