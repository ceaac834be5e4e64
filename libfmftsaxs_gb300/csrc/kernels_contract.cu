/*
 * Contraction kernels of the factorized correlation, in FP64 (plain path)
 * or FP32 (mixed path); multiply-add fusion allowed.
 *
 * The reference evaluates, per touched (z, beta1, beta2) triple, the 6-channel
 * sums X[m,m1,m2] (src/fftsaxs.c:416-524) and then an angular DFT at each
 * listed cell (529-606 or FFTW).  Writing the DFT phase as a product of the
 * per-angle phases and moving each sum next to the angle it depends on gives,
 * for one listed pose (z, b1, b2, a2, g1, g2) and one q,
 *
 *   P^a[m,l](b1,g1) = sum_{m1} w^{m1' g1} d^l_{m m1}(beta_b1) A^a_{l m1}
 *   U^b[m,l1](b2,g2)= sum_{m2} w^{m2' g2} d^l1_{m m2}(beta_b2) conj(B^b_{l1 m2})
 *   R^b[m,l]        = sum_{l1>=|m|} conj(T^{|m|}_{l l1}(q z)) U^b[m,l1]
 *   F^{ab}          = sum_m w^{m' a2} sum_{l>=|m|} P^a[m,l] R^b[m,l]
 *
 * (w = the twiddle table, x' = x mod N), the reference's F with the same terms
 * regrouped.  A and B expand real densities, so A_{l,-m} = (-1)^{l+m}
 * conj(A_{lm}); with d^l_{-m,-m1} = (-1)^{m-m1} d^l_{m m1} and T real or
 * imaginary by the parity of l + l1 this gives P[-m,l] = (-1)^{l+m} conj(P[m,l])
 * and the same for U and R, so the m-sum is Re F = Re(w_0 G_0) +
 * 2 sum_{m>0} Re(w_m G_m) with G_m = sum_l P[m,l] R[m,l].  Only m >= 0 is
 * tabulated: pairs (m, l), m = 0..L, l = m..L, (L+1)(L+2)/2 of them.
 */
#include "kernels.h"

namespace {

template <typename S> struct Cx;
template <> struct Cx<double> { typedef double2 T; };
template <> struct Cx<float> { typedef float2 T; };

__device__ __forceinline__ int lm_index(int l, int m) { return l * (l + 1) + m; }

/* first pair of row m >= 0 */
__device__ __forceinline__ int psym(int m, int K) { return m * K - m * (m - 1) / 2; }

__device__ __forceinline__ void cfma(double2 &acc, double2 a, double2 b)
{
	acc.x = fma(a.x, b.x, acc.x);
	acc.x = fma(-a.y, b.y, acc.x);
	acc.y = fma(a.x, b.y, acc.y);
	acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfma(float2 &acc, float2 a, float2 b)
{
	acc.x = fmaf(a.x, b.x, acc.x);
	acc.x = fmaf(-a.y, b.y, acc.x);
	acc.y = fmaf(a.x, b.y, acc.y);
	acc.y = fmaf(a.y, b.x, acc.y);
}
template <typename V> __device__ __forceinline__ V zero2() { V v; v.x = 0; v.y = 0; return v; }
template <typename V> __device__ __forceinline__ V from2(double2 a) { V v; v.x = a.x; v.y = a.y; return v; }

/* [3][Q][K2][2] -> [3][K2][Q] complex */
template <typename S>
__global__ void k_spf_transpose(const double *__restrict__ flat, typename Cx<S>::T *__restrict__ t, int Q, int K2)
{
	typedef typename Cx<S>::T V;
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= 3L * Q * K2) return;
	int iq = (int)(i % Q);
	long r = i / Q;
	int lm = (int)(r % K2), ch = (int)(r / K2);
	const double *s = flat + (((size_t)ch * Q + iq) * K2 + lm) * 2;
	V v;
	v.x = (S)s[0];
	v.y = (S)s[1];
	t[i] = v;
}

/* block = (b*N+g, m >= 0); threads over q */
template <typename S>
__global__ void k_rotate(const typename Cx<S>::T *__restrict__ spf_t, const double *__restrict__ dtab,
                         const double2 *__restrict__ tw, int Q, int L, int conj, typename Cx<S>::T *__restrict__ out)
{
	typedef typename Cx<S>::T V;
	int K = L + 1, N = 2 * L + 1, K2 = K * K, NP = K * (K + 1) / 2;
	int bg = blockIdx.x, m = blockIdx.y;
	int b = bg / N, g = bg % N;
	int iq = threadIdx.x;
	if (iq >= Q) return;
	const double *db = dtab + (size_t)b * K * N * N;
	S sg = conj ? (S)-1 : (S)1;
	int po = psym(m, K);
	for (int l = m; l <= L; l++) {
		V acc0 = zero2<V>(), acc1 = acc0, acc2 = acc0;
		const double *drow = db + ((size_t)l * N + m + L) * N;
		for (int m1 = -l; m1 <= l; m1++) {
			int e = ((m1 < 0 ? m1 + N : m1) * g) % N;
			S dv = (S)drow[m1 + L];
			V f;
			f.x = (S)tw[e].x * dv;
			f.y = (S)tw[e].y * dv;
			int lm = lm_index(l, m1);
			V c0 = spf_t[((size_t)0 * K2 + lm) * Q + iq];
			V c1 = spf_t[((size_t)1 * K2 + lm) * Q + iq];
			V c2 = spf_t[((size_t)2 * K2 + lm) * Q + iq];
			c0.y *= sg; c1.y *= sg; c2.y *= sg;
			cfma(acc0, f, c0);
			cfma(acc1, f, c1);
			cfma(acc2, f, c2);
		}
		V *o = out + (((size_t)bg * NP + po + (l - m)) * 3) * Q + iq;
		o[0] = acc0;
		o[Q] = acc1;
		o[2 * Q] = acc2;
	}
}

/* block = (combo, m >= 0); threads over q; l blocked by LB for register
 * reuse of U.  conj(T) U = tau U for even l + l1, tau (-i U) for odd. */
template <typename S, int LB>
__global__ void k_translate(const typename Cx<S>::T *__restrict__ U, const S *__restrict__ tau,
                            const int32_t *__restrict__ combo_zbg, int Q, int L, typename Cx<S>::T *__restrict__ out)
{
	typedef typename Cx<S>::T V;
	int K = L + 1, N = 2 * L + 1, NP = K * (K + 1) / 2;
	int c = blockIdx.x, m = blockIdx.y;
	int iq = threadIdx.x;
	if (iq >= Q) return;
	int zi = combo_zbg[3 * c], b2 = combo_zbg[3 * c + 1], g2 = combo_zbg[3 * c + 2];
	const V *Ub = U + (size_t)(b2 * N + g2) * NP * 3 * Q;
	const S *Tm = tau + ((size_t)zi * K + m) * K * K * Q;
	int po = psym(m, K);
	V *Ob = out + (size_t)c * NP * 3 * Q;
	for (int l0 = m; l0 <= L; l0 += LB) {
		V acc[LB][3];
#pragma unroll
		for (int j = 0; j < LB; j++) acc[j][0] = acc[j][1] = acc[j][2] = zero2<V>();
		for (int l1 = m; l1 <= L; l1++) {
			const V *u = Ub + ((size_t)(po + l1 - m) * 3) * Q + iq;
			V u0 = u[0], u1 = u[Q], u2 = u[2 * Q];
#pragma unroll
			for (int j = 0; j < LB; j++) {
				int l = l0 + j;
				if (l > L) break;
				S t = Tm[((size_t)l * K + l1) * Q + iq];
				if (((l + l1) & 1) == 0) {
					acc[j][0].x += t * u0.x; acc[j][0].y += t * u0.y;
					acc[j][1].x += t * u1.x; acc[j][1].y += t * u1.y;
					acc[j][2].x += t * u2.x; acc[j][2].y += t * u2.y;
				} else {
					acc[j][0].x += t * u0.y; acc[j][0].y -= t * u0.x;
					acc[j][1].x += t * u1.y; acc[j][1].y -= t * u1.x;
					acc[j][2].x += t * u2.y; acc[j][2].y -= t * u2.x;
				}
			}
		}
#pragma unroll
		for (int j = 0; j < LB; j++) {
			int l = l0 + j;
			if (l > L) break;
			V *o = Ob + ((size_t)(po + l - m) * 3) * Q + iq;
			o[0] = acc[j][0];
			o[Q] = acc[j][1];
			o[2 * Q] = acc[j][2];
		}
	}
}

/* block = one pose; threads over q.  Writes cross[src][c][q] (FP64). */
template <typename S>
__global__ void k_pose_cross(const sxsk_pose *__restrict__ poses, int combo_base, const typename Cx<S>::T *__restrict__ P,
                             const typename Cx<S>::T *__restrict__ R, const double2 *__restrict__ tw,
                             const double *__restrict__ cst, int Q, int L, double *__restrict__ cross)
{
	typedef typename Cx<S>::T V;
	int K = L + 1, N = 2 * L + 1, NP = K * (K + 1) / 2;
	sxsk_pose ps = poses[blockIdx.x];
	int iq = threadIdx.x;
	if (iq >= Q) return;
	const V *Pb = P + (size_t)(ps.b1 * N + ps.g1) * NP * 3 * Q + iq;
	const V *Rb = R + (size_t)(ps.combo - combo_base) * NP * 3 * Q + iq;
	S f[6] = {0, 0, 0, 0, 0, 0};
	int p = 0;
	for (int m = 0; m <= L; m++) {
		V g[6];
#pragma unroll
		for (int c = 0; c < 6; c++) g[c] = zero2<V>();
		for (int l = m; l <= L; l++, p++) {
			const V *pp = Pb + (size_t)p * 3 * Q;
			const V *rr = Rb + (size_t)p * 3 * Q;
			V pv = pp[0], pd = pp[Q], pw = pp[2 * Q];
			V rv = rr[0], rd = rr[Q], rw = rr[2 * Q];
			cfma(g[0], pv, rv);
			cfma(g[1], pv, rd); cfma(g[1], pd, rv);
			cfma(g[2], pv, rw); cfma(g[2], pw, rv);
			cfma(g[3], pd, rd);
			cfma(g[4], pd, rw); cfma(g[4], pw, rd);
			cfma(g[5], pw, rw);
		}
		V w = from2<V>(tw[(m * ps.a2) % N]);
		S wt = m == 0 ? (S)1 : (S)2;
#pragma unroll
		for (int c = 0; c < 6; c++) f[c] += wt * (w.x * g[c].x - w.y * g[c].y);
	}
	double *o = cross + (size_t)ps.src * 6 * Q + iq;
#pragma unroll
	for (int c = 0; c < 6; c++) {
		double v = cst[c * Q + iq];
		v += 2.0 * (double)f[c];
		o[c * Q] = v;
	}
}

__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, long n)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) b[i] = (float)a[i];
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

/* Grid fit (src/min_saxs.c:170-188 peak rescale, 261-320 best scale,
 * 391-448 point_score).  For one pose and one (c1, c2) cell the model at q_i
 * is in_i = al_i + c2 be_i + c2^2 ga_i with G_i = c1^3 exp(-mult (c1^2-1) q_i^2),
 * al = VV - G VD + G^2 DD, be = VW - G DW, ga = WW; point_score's piecewise
 * line is tan_i = (in_i - in_{i-1}) h_i (tan_0 = 0), buf_i = in_i - tan_i q_i,
 * and with the best scale k = up/down the score is sum a0 + k(-2 up + k down),
 *   up   = sum_i a1 buf + a2 tan = sum_i a1 in + u_i D_i
 *   down = sum_i a3 buf^2 + 2 a4 buf tan + a5 tan^2
 *        = sum_i a3 in^2 + 2 e_i in D_i + f_i D_i^2
 * where D_i = in_i - in_{i-1} and the per-q constants are folded on the host:
 *   fc[i] = {a3, e = (a4 - q a3) h, f = (a5 - 2 q a4 + q^2 a3) h^2, a1,
 *            u = (a2 - q a1) h}.
 * up is quadratic and down quartic in c2, so per (pose, c1) one pass over q
 * yields their coefficients and every c2 cell costs a few multiply-adds.
 * One thread per (pose, c1): no reductions and no repeated q work.  Within
 * a thread cells are ranked by up^2/down (score = sum a0 - up^2/down); the
 * threads of a pose then compare their best scores, ties going to the lower
 * cell index as in a c1-major scan. */
#define FIT_THREADS 128
#define FIT_NFC 5
/* Persistent: block b handles pose groups b, b + gridDim.x, ...; a group is
 * ppb consecutive slots of the pose order (order[slot].src is the pose's
 * position in cross and in the outputs; slot itself when order is NULL). */
__global__ void __launch_bounds__(FIT_THREADS)
k_fit_grid(const double *__restrict__ cross, const sxsk_pose *__restrict__ order, int slot0, int nslot, int Q,
           const double *__restrict__ fc, double a0sum, double peak, const double *__restrict__ gtab,
           const double *__restrict__ c1g, int n1, const double *__restrict__ c2g, int n2, int tp, int ppb,
           double *__restrict__ chi, double *__restrict__ c1o, double *__restrict__ c2o, int32_t *__restrict__ cello,
           double *__restrict__ grid, double *__restrict__ scaled)
{
	extern __shared__ double sm[];
	double *cs = sm;                                   /* [ppb][8][Q]: VV VD VW DD DW WW P3 P4 */
	double *fs = cs + (size_t)ppb * 8 * Q;             /* [FIT_NFC][Q] */
	double *c2s = fs + (size_t)FIT_NFC * Q;            /* [n2] */
	double *red = c2s + n2;                            /* [ppb*tp][2] partials / best score */
	int *redc = (int *)(red + 2 * ppb * tp);           /* [ppb*tp] best cell */
	double *sf = (double *)(redc + ((ppb * tp + 1) & ~1)); /* [ppb][3]: scale, U2, D4 */
	int *srcs = (int *)(sf + 3 * ppb);                 /* [ppb] pose index of each slot */
	int tid = threadIdx.x;
	int nthr = ppb * tp;
	int lp = tid / tp, lt = tid % tp;
	const double *F3 = fs, *FE = fs + Q, *FF = fs + 2 * Q, *F1 = fs + 3 * Q, *FU = fs + 4 * Q;

	for (int k = tid; k < FIT_NFC * Q; k += blockDim.x) fs[k] = fc[(k % Q) * FIT_NFC + k / Q];
	for (int k = tid; k < n2; k += blockDim.x) c2s[k] = c2g[k];
	int ngroup = (nslot + ppb - 1) / ppb;
	for (int grp = blockIdx.x; grp < ngroup; grp += gridDim.x) {
		int s0 = grp * ppb;
		int nhere = min(ppb, nslot - s0);
		bool live = tid < nthr && lp < nhere;
		__syncthreads();   /* previous group done with the shared arrays */
		if (tid < nhere) srcs[tid] = order ? order[slot0 + s0 + tid].src : slot0 + s0 + tid;
		__syncthreads();
		for (int k = tid; k < nhere * 6 * Q; k += blockDim.x) {
			int p = k / (6 * Q), r = k % (6 * Q);
			cs[(size_t)p * 8 * Q + r] = cross[(size_t)srcs[p] * 6 * Q + r];
		}
		__syncthreads();
		if (live && lt == 0) {
			const double *c = cs + (size_t)lp * 8 * Q;
			double sc = c[0] + c[3 * Q] + c[5 * Q] + c[2 * Q] - c[Q] - c[4 * Q];
			sf[3 * lp] = peak / sc;
		}
		__syncthreads();
		for (int k = tid; k < nhere * 6 * Q; k += blockDim.x) {
			int p = k / (6 * Q), r = k % (6 * Q);
			double v = cs[(size_t)p * 8 * Q + r] * sf[3 * p];
			cs[(size_t)p * 8 * Q + r] = v;
			if (scaled) scaled[(size_t)srcs[p] * 6 * Q + r] = v;
		}
		__syncthreads();
		double *c = cs + (size_t)lp * 8 * Q;
		const double *VV = c, *VD = c + Q, *VW = c + 2 * Q, *DD = c + 3 * Q, *DW = c + 4 * Q, *WW = c + 5 * Q;
		double *P3 = c + 6 * Q, *P4 = c + 7 * Q;
		/* c1-independent part: M (ga, D_ga) per q, and the c2^2 coefficients */
		if (live) {
			double u2 = 0, d4 = 0;
			for (int i = lt; i < Q; i += tp) {
				double ga = WW[i], dg = i > 0 ? ga - WW[i - 1] : 0.0;
				double p3 = fma(F3[i], ga, FE[i] * dg);
				double p4 = fma(FE[i], ga, FF[i] * dg);
				P3[i] = p3;
				P4[i] = p4;
				u2 = fma(F1[i], ga, fma(FU[i], dg, u2));
				d4 = fma(ga, p3, fma(dg, p4, d4));
			}
			red[2 * tid] = u2;
			red[2 * tid + 1] = d4;
		}
		__syncthreads();
		if (live && lt == 0) {
			double u2 = 0, d4 = 0;
			for (int t = 0; t < tp; t++) {
				u2 += red[2 * (tid + t)];
				d4 += red[2 * (tid + t) + 1];
			}
			sf[3 * lp + 1] = u2;
			sf[3 * lp + 2] = d4;
		}
		__syncthreads();
		double bscore = __longlong_as_double(0x7ff0000000000000LL);
		int bcell = -1;
		int pid = live ? srcs[lp] : 0;
		if (live) {
			double U2 = sf[3 * lp + 1], D4 = sf[3 * lp + 2];
			for (int j = lt; j < n1; j += tp) {
				const double *G = gtab + (size_t)j * Q;
				double U0 = 0, U1 = 0, D0 = 0, D1 = 0, D2a = 0, D2b = 0, D3 = 0;
				double g = __ldg(G);
				double alp = fma(g, fma(g, DD[0], -VD[0]), VV[0]);
				double bep = fma(-g, DW[0], VW[0]);
				for (int i = 0; i < Q; i++) {
					g = __ldg(G + i);
					double al = fma(g, fma(g, DD[i], -VD[i]), VV[i]);
					double be = fma(-g, DW[i], VW[i]);
					double d0 = al - alp, d1 = be - bep;
					double f3 = F3[i], fe = FE[i], ff = FF[i];
					double m0a = fma(f3, al, fe * d0), m0b = fma(fe, al, ff * d0);
					double m1a = fma(f3, be, fe * d1), m1b = fma(fe, be, ff * d1);
					double p3 = P3[i], p4 = P4[i];
					D0 = fma(al, m0a, fma(d0, m0b, D0));
					D1 = fma(be, m0a, fma(d1, m0b, D1));
					D2a = fma(be, m1a, fma(d1, m1b, D2a));
					D2b = fma(al, p3, fma(d0, p4, D2b));
					D3 = fma(be, p3, fma(d1, p4, D3));
					double f1 = F1[i], fu = FU[i];
					U0 = fma(f1, al, fma(fu, d0, U0));
					U1 = fma(f1, be, fma(fu, d1, U1));
					alp = al;
					bep = be;
				}
				D1 *= 2.0;
				double D2 = fma(2.0, D2b, D2a);
				D3 *= 2.0;
				/* best c2 of this c1 by up^2/down, then its score */
				double bu = 0, bd = 0;
				int bi = -1;
				for (int i2 = 0; i2 < n2; i2++) {
					double c2 = c2s[i2];
					double up = fma(c2, fma(c2, U2, U1), U0);
					double down = fma(c2, fma(c2, fma(c2, fma(c2, D4, D3), D2), D1), D0);
					if (grid) {
						double k = up / down;
						grid[((size_t)pid * n1 + j) * n2 + i2] = a0sum + k * (-2.0 * up + k * down);
					}
					if (down > 0.0) {
						double num = up * up;
						if (bi < 0 || num * bd > bu * bu * down) { bu = up; bd = down; bi = i2; }
					}
				}
				if (bi >= 0) {
					double k = bu / bd;
					double score = a0sum + k * (-2.0 * bu + k * bd);
					int cell = j * n2 + bi;
					if (score < bscore || (score == bscore && cell < bcell)) { bscore = score; bcell = cell; }
				}
			}
			red[2 * tid] = bscore;
			redc[tid] = bcell;
		}
		__syncthreads();
		if (live && lt == 0) {
			for (int t = 1; t < tp; t++) {
				double os = red[2 * (tid + t)];
				int oc = redc[tid + t];
				if (oc >= 0 && (bcell < 0 || os < bscore || (os == bscore && oc < bcell))) { bscore = os; bcell = oc; }
			}
			if (bcell >= 0) {
				chi[pid] = sqrt(bscore);
				c1o[pid] = c1g[bcell / n2];
				c2o[pid] = c2g[bcell % n2];
			} else {
				chi[pid] = __longlong_as_double(0x7ff8000000000000LL);
				c1o[pid] = __longlong_as_double(0x7ff8000000000000LL);
				c2o[pid] = __longlong_as_double(0x7ff8000000000000LL);
			}
			if (cello) cello[pid] = bcell;
		}
	}
}

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }
inline int qthreads(int Q) { return ((Q + 31) / 32) * 32; }

} // namespace

extern "C" {

int sxsk_spf_transpose(const double *flat, void *spf_t, int Q, int L, int fp32, cudaStream_t s)
{
	int K2 = (L + 1) * (L + 1);
	if (fp32) k_spf_transpose<float><<<nblk(3L * Q * K2, 256), 256, 0, s>>>(flat, (float2 *)spf_t, Q, K2);
	else k_spf_transpose<double><<<nblk(3L * Q * K2, 256), 256, 0, s>>>(flat, (double2 *)spf_t, Q, K2);
	return cudaGetLastError();
}

int sxsk_rotate(const void *spf_t, const double *dtab, const double2 *tw, int Q, int L, int conj, void *out, int fp32,
                cudaStream_t s)
{
	int K = L + 1, N = 2 * L + 1;
	dim3 grid(K * N, K);
	if (fp32) k_rotate<float><<<grid, qthreads(Q), 0, s>>>((const float2 *)spf_t, dtab, tw, Q, L, conj, (float2 *)out);
	else k_rotate<double><<<grid, qthreads(Q), 0, s>>>((const double2 *)spf_t, dtab, tw, Q, L, conj, (double2 *)out);
	return cudaGetLastError();
}

int sxsk_to_float(const double *a, float *b, long n, cudaStream_t s)
{
	if (n <= 0) return 0;
	k_to_float<<<nblk(n, 256), 256, 0, s>>>(a, b, n);
	return cudaGetLastError();
}

int sxsk_translate(const void *U, const void *tau, const int32_t *combo_zbg, int ncombo, int Q, int L, void *out,
                   int fp32, cudaStream_t s)
{
	if (ncombo <= 0) return 0;
	dim3 grid(ncombo, L + 1);
	if (fp32)
		k_translate<float, 4><<<grid, qthreads(Q), 0, s>>>((const float2 *)U, (const float *)tau, combo_zbg, Q, L,
		                                                    (float2 *)out);
	else
		k_translate<double, 4><<<grid, qthreads(Q), 0, s>>>((const double2 *)U, (const double *)tau, combo_zbg, Q, L,
		                                                     (double2 *)out);
	return cudaGetLastError();
}

int sxsk_pose_cross(const sxsk_pose *poses, int npose, int combo_base, const void *P, const void *R,
                    const double2 *tw, const double *cst, int Q, int L, double *cross, int fp32, cudaStream_t s)
{
	if (npose <= 0) return 0;
	if (fp32)
		k_pose_cross<float><<<npose, qthreads(Q), 0, s>>>(poses, combo_base, (const float2 *)P, (const float2 *)R, tw,
		                                                   cst, Q, L, cross);
	else
		k_pose_cross<double><<<npose, qthreads(Q), 0, s>>>(poses, combo_base, (const double2 *)P, (const double2 *)R,
		                                                    tw, cst, Q, L, cross);
	return cudaGetLastError();
}

int sxsk_fit_grid(const double *cross, const sxsk_pose *order, int slot0, int nslot, int Q, const double *fc,
                  double a0sum, double peak, const double *gtab, const double *c1g, int n1, const double *c2g, int n2,
                  int max_blocks, double *chi, double *c1, double *c2, int32_t *cell, double *grid, double *scaled,
                  cudaStream_t s)
{
	if (nslot <= 0) return 0;
	if (n1 <= 0 || n2 <= 0) return cudaErrorInvalidValue;
	int tp = n1 < FIT_THREADS ? n1 : FIT_THREADS;
	int ppb = FIT_THREADS / tp;
	size_t smem;
	for (;;) {
		size_t nthr = (size_t)ppb * tp;
		smem = sizeof(double) * ((size_t)ppb * 8 * Q + (size_t)FIT_NFC * Q + n2 + 2 * nthr + 3 * ppb) +
		       sizeof(int) * (((nthr + 1) & ~(size_t)1) + ppb);
		if (smem <= 227 * 1024 || ppb == 1) break;
		ppb = (ppb + 1) / 2;
	}
	if (smem > 227 * 1024) return cudaErrorInvalidValue;
	if (smem > 48 * 1024) {
		cudaError_t e = cudaFuncSetAttribute(k_fit_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
	}
	long ngroup = (nslot + ppb - 1) / ppb;
	int grid_n = (int)(ngroup < (long)max_blocks || max_blocks <= 0 ? ngroup : max_blocks);
	k_fit_grid<<<grid_n, FIT_THREADS, smem, s>>>(cross, order, slot0, nslot, Q, fc, a0sum, peak, gtab, c1g, n1, c2g,
	                                              n2, tp, ppb, chi, c1, c2, cell, grid, scaled);
	return cudaGetLastError();
}

} // extern "C"

namespace {
/* independent FMA chains per thread, register resident */
__global__ void k_fp64_probe(double *out, int iters)
{
	double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
	double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
	const double b = 0.999999999, c = 1e-12;
	for (int i = 0; i < iters; i++) {
		a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
		a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
	}
	double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
	if (s == 12345.678) out[threadIdx.x] = s; /* keeps the chains live */
}
} // namespace

extern "C" double sxsk_fp64_probe(cudaStream_t s)
{
	int dev = 0, nsm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	double *out = NULL;
	if (cudaMalloc((void **)&out, 1024 * sizeof(double)) != cudaSuccess) return -1.0;
	int blocks = nsm * 8, threads = 256, iters = 4096;
	k_fp64_probe<<<blocks, threads, 0, s>>>(out, 64);
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	cudaEventRecord(e0, s);
	k_fp64_probe<<<blocks, threads, 0, s>>>(out, iters);
	cudaEventRecord(e1, s);
	cudaEventSynchronize(e1);
	float ms = 0;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
	return ms > 0 ? flops / (ms * 1e-3) / 1e12 : -1.0;
}
