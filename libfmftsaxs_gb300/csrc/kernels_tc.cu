/*
 * Rotation tables of the mixed path on the tcgen05 tensor cores.
 *
 * For a fixed beta_b the rotation of one molecule's coefficients is a
 * complex matrix product over m1:
 *   P[g][c] = sum_{m1} W[g][m1] X[m1][c],   W[g][m1] = tw[(m1' g) mod N],
 *   X[m1][c] = d^l_{m m1}(beta_b) C[ch][l, m1][q]   (0 for |m1| > l)
 * with one column c per (pair (m, l), channel, q) in the q-tiled order of the
 * output table.  Written over the reals, [Re P; Im P] = [[Wr, -Wi], [Wi, Wr]]
 * [Re X; Im X]: an M = 2N (padded to 128) by K = 2N (padded to a multiple of
 * 8) matrix times K x NTILE columns per block.  Each block builds both
 * operands in shared memory (canonical K-major layout without swizzle: 8-row
 * x 16-byte core matrices, consecutive along K, K/4 of them per 8-row
 * group), one thread issues the MMAs (kind::tf32, 128 x NTILE x 8 each,
 * FP32 accumulator in tensor memory), the block waits on an mbarrier that
 * the MMA commit arrives on, reads the accumulator back with tcgen05.ld and
 * writes the complex rows.  Accuracy: each operand is split into a TF32
 * high part and the FP32 remainder (a = a_hi + a_lo), and the products
 * a_hi b_hi + a_hi b_lo + a_lo b_hi are accumulated (three MMAs per K step),
 * which keeps the result at FP32 level.
 *
 * The mbarrier wait is bounded.  A block that gives up records it in the
 * caller's status word and waits (bounded again) for the MMAs it issued:
 * status 1 means they then finished and the block freed its tensor memory
 * as usual; status 2 means the second wait gave up too, and the block
 * returns without freeing tensor memory that an MMA may still be writing.
 * The tables of a launch with a nonzero status are not valid; after
 * status 2 the CUDA context itself must be considered unusable.
 */
#include "kernels.h"

#include <stdint.h>

namespace {

#define TC_THREADS 128
#define TC_M 128
#define TC_WAIT_LIMIT (1 << 20)

__device__ __forceinline__ int psym_tc(int m, int K) { return m * K - m * (m - 1) / 2; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* shared memory matrix descriptor: start address, leading-dimension (K)
 * byte offset between core matrices, stride (M/N) byte offset between 8-row
 * groups, descriptor version 1, no swizzle */
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
	return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
	       ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* instruction descriptor, kind::tf32: D F32, A and B TF32, both K-major */
__host__ __device__ __forceinline__ uint32_t idesc_tf32(int M, int N)
{
	return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* byte offset of element (row, k) in the canonical K-major layout, KP columns */
__device__ __forceinline__ uint32_t koff(int row, int k, int KP)
{
	return (uint32_t)((row >> 3) * (KP >> 2) * 128 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo)
{
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	hi = __uint_as_float(r);
	lo = x - hi;
}

__device__ __forceinline__ void mbar_init(uint64_t *m, unsigned cnt)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(cnt) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *m, unsigned phase)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	             "selp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok)
	             : "r"(smem_u32(m)), "r"(phase)
	             : "memory");
	return ok != 0;
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
	             "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t *r)
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	             : "r"(taddr));
}

/* The real form of the twiddle matrix, hi and lo TF32 parts, in the
 * canonical K-major layout (128 rows x KP): rows r < N -> Re P[g = r],
 * r in [N, 2N) -> Im P[g = r - N]; columns k < N -> Re X[m1 = k - L],
 * k in [N, 2N) -> Im X[m1 = k - N - L]; padding zero. */
__global__ void k_tc_amat(const double2 *__restrict__ tw, int L, int KP, float *__restrict__ ahi,
                          float *__restrict__ alo)
{
	int N = 2 * L + 1;
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= TC_M * KP) return;
	int r = e / KP, k = e % KP;
	float v = 0.0f;
	if (r < 2 * N && k < 2 * N) {
		int g = r < N ? r : r - N;
		int m1 = (k < N ? k : k - N) - L;
		int ep = ((m1 < 0 ? m1 + N : m1) * g) % N;
		double2 wd = tw[ep];
		float wx = (float)wd.x, wy = (float)wd.y;
		bool rre = r < N, kre = k < N;
		v = rre ? (kre ? wx : -wy) : (kre ? wy : wx);
	}
	float hi, lo;
	split_tf32(v, hi, lo);
	uint32_t o = koff(r, k, KP) >> 2;
	ahi[o] = hi;
	alo[o] = lo;
}

#define TC_BLOCK 512

/* Persistent: block loops over items (beta_b, q tile t, chunk j of NTILE
 * columns); columns of tile t are c = (pair 3 + ch) 8 + qq.  The twiddle
 * operand is loaded once per block. */
__global__ void __launch_bounds__(TC_BLOCK) k_rotate_tc(const float2 *__restrict__ spf_t,
                                                        const float *__restrict__ dtab,
                                                        const float *__restrict__ ahi_g,
                                                        const float *__restrict__ alo_g, int Q, int L, int conj,
                                                        int KP, int NTILE, float2 *__restrict__ out,
                                                        int *__restrict__ status)
{
	extern __shared__ __align__(1024) unsigned char tsm[];
	int K = L + 1, N = 2 * L + 1, K2 = K * K, NP = K * (K + 1) / 2, nrow = K * N;
	int NT = (Q + SXS_QT - 1) / SXS_QT;
	int NCT = NP * 3 * SXS_QT;
	int nchunk = (NCT + NTILE - 1) / NTILE;
	int nitem = K * NT * nchunk;
	/* B area: both B halves, later the [NTILE][128] accumulator copy */
	int barea = max(2 * NTILE * KP * 4, NTILE * TC_M * 4);
	unsigned char *Ahi = tsm, *Alo = tsm + TC_M * KP * 4;
	unsigned char *Bhi = Alo + TC_M * KP * 4, *Blo = Bhi + NTILE * KP * 4;
	uint64_t *mbar = reinterpret_cast<uint64_t *>(Bhi + barea);
	uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
	int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

	if (tid == 0) {
		mbar_init(mbar, 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
		             "r"(NTILE)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	{
		const uint4 *sh = reinterpret_cast<const uint4 *>(ahi_g), *sl = reinterpret_cast<const uint4 *>(alo_g);
		uint4 *dh = reinterpret_cast<uint4 *>(Ahi), *dl = reinterpret_cast<uint4 *>(Alo);
		for (int k = tid; k < TC_M * KP / 4; k += TC_BLOCK) {
			dh[k] = sh[k];
			dl[k] = sl[k];
		}
	}
	__syncthreads();
	uint32_t taddr = *tslot;
	uint32_t idesc = idesc_tf32(TC_M, NTILE);
	uint32_t sbo = (uint32_t)(KP >> 2) * 128;
	float sg = conj ? -1.0f : 1.0f;
	float *Out = reinterpret_cast<float *>(Bhi);
	int mma_live = 0;   /* both bounded waits gave up: an MMA may still run */
	unsigned phase = 0;
	for (int item = blockIdx.x; item < nitem; item += gridDim.x) {
		int j = item % nchunk, bt = item / nchunk;
		int t = bt % NT, b = bt / NT;
		int c0 = j * NTILE;
		const float *db = dtab + (size_t)b * K * N * N;
		/* B: TC_BLOCK / NTILE threads per column, each decoding its column
		 * once and filling every (TC_BLOCK / NTILE)-th k; Re X then Im X
		 * over m1 */
		{
			int tpc = TC_BLOCK / NTILE;
			int cl = tid / tpc, k0 = tid % tpc;
			int c = c0 + cl;
			int qq = c % SXS_QT, pc = c / SXS_QT;
			int ch = pc % 3, pr = pc / 3;
			int q = t * SXS_QT + qq;
			bool col_ok = c < NCT && q < Q;
			int m = 0;
			if (col_ok)
				while (pr >= psym_tc(m + 1, K)) m++;
			int l = m + pr - psym_tc(m, K);
			const float *drow = db + ((size_t)l * N + m + L) * N;
			const float2 *crow = spf_t + ((size_t)ch * K2 + l * (l + 1)) * Q + q;
			for (int k = k0; k < KP; k += tpc) {
				float v = 0.0f;
				if (col_ok && k < 2 * N) {
					int mi = k < N ? k : k - N;
					int m1 = mi - L;
					if (m1 >= -l && m1 <= l) {
						float dv = drow[mi];
						float2 cv = crow[(ptrdiff_t)m1 * Q];
						v = k < N ? dv * cv.x : dv * (sg * cv.y);
					}
				}
				float hi, lo;
				split_tf32(v, hi, lo);
				*reinterpret_cast<float *>(Bhi + koff(cl, k, KP)) = hi;
				*reinterpret_cast<float *>(Blo + koff(cl, k, KP)) = lo;
			}
		}
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		__syncthreads();
		if (tid == 0) {
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			uint32_t aH = smem_u32(Ahi), aL = smem_u32(Alo), bH = smem_u32(Bhi), bL = smem_u32(Blo);
			for (int s = 0; s < KP / 8; s++) {
				uint32_t off = (uint32_t)s * 256;   /* two core matrices along K per step */
				tc_mma(taddr, sdesc(aH + off, 128, sbo), sdesc(bH + off, 128, sbo), idesc, s > 0);
				tc_mma(taddr, sdesc(aH + off, 128, sbo), sdesc(bL + off, 128, sbo), idesc, 1);
				tc_mma(taddr, sdesc(aL + off, 128, sbo), sdesc(bH + off, 128, sbo), idesc, 1);
			}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
			                 smem_u32(mbar))
			             : "memory");
		}
		bool done = false;
		for (int it = 0; it < TC_WAIT_LIMIT; it++)
			if (mbar_try_wait(mbar, phase)) {
				done = true;
				break;
			}
		phase ^= 1u;
		done = __syncthreads_and(done);
		if (!done) {
			/* a second bounded wait for the MMAs in flight before the
			 * accumulator's TMEM is freed below */
			bool drained = false;
			for (int it = 0; it < TC_WAIT_LIMIT; it++)
				if (mbar_try_wait(mbar, phase ^ 1u)) {
					drained = true;
					break;
				}
			drained = __syncthreads_and(drained);
			if (tid == 0) atomicMax(status, drained ? 1 : 2);
			mma_live = !drained;
			break;
		}
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		/* accumulator -> shared [NTILE][128]: warp w reads lane quadrant w % 4,
		 * column groups w / 4, w / 4 + 4, ... */
		for (int cc = warp >> 2; cc < NTILE / 32; cc += TC_BLOCK / 128) {
			uint32_t r[32];
			tc_ld32(taddr + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * cc), r);
			asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
			for (int i = 0; i < 32; i++)
				Out[(32 * cc + i) * TC_M + 32 * (warp & 3) + lane] = __uint_as_float(r[i]);
		}
		asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
		__syncthreads();
		/* complex rows: out[t][b N + g][c] = (Out[c][g], Out[c][N + g]) */
		int ncl = min(NTILE, NCT - c0);
		for (int e = tid; e < N * ncl; e += TC_BLOCK) {
			int g = e / ncl, cl = e % ncl;
			float2 v = make_float2(Out[cl * TC_M + g], Out[cl * TC_M + N + g]);
			out[((size_t)t * nrow + b * N + g) * NCT + c0 + cl] = v;
		}
		__syncthreads();   /* Out is the next item's B */
	}
	if (mma_live) return;   /* never free TMEM under a live MMA (status 2) */
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(NTILE) : "memory");
}

} // namespace

extern "C" int sxsk_rotate_tc(const void *spf_t, const float *dtabf, const double2 *tw, int Q, int L, int conj,
                              void *out, float *amat, int *status, cudaStream_t s)
{
	int K = L + 1, N = 2 * L + 1;
	if (2 * N > TC_M) return cudaErrorInvalidValue;
	int KP = ((2 * N + 7) / 8) * 8;
	int NT = (Q + SXS_QT - 1) / SXS_QT;
	int NP = K * (K + 1) / 2, NCT = NP * 3 * SXS_QT;
	int NTILE = 128;
	size_t smem = 0;
	for (;;) {
		size_t barea = (size_t)2 * NTILE * KP * 4;
		if (barea < (size_t)NTILE * TC_M * 4) barea = (size_t)NTILE * TC_M * 4;
		smem = (size_t)2 * TC_M * KP * 4 + barea + 16;
		if (smem <= 200 * 1024 || NTILE == 32) break;
		NTILE /= 2;
	}
	if (smem > 227 * 1024) return cudaErrorInvalidValue;
	int ae = TC_M * KP;
	k_tc_amat<<<(ae + 255) / 256, 256, 0, s>>>(tw, L, KP, amat, amat + ae);
	cudaError_t e = cudaFuncSetAttribute(k_rotate_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	int dev = 0, nsm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	int nchunk = (NCT + NTILE - 1) / NTILE;
	long nitem = (long)K * NT * nchunk;
	int grid = (int)(nitem < nsm ? nitem : nsm);
	k_rotate_tc<<<grid, TC_BLOCK, smem, s>>>((const float2 *)spf_t, dtabf, amat, amat + ae, Q, L, conj, KP, NTILE,
	                                         (float2 *)out, status);
	return cudaGetLastError();
}

/* floats of the scratch sxsk_rotate_tc needs for the twiddle operand */
extern "C" size_t sxsk_rotate_tc_scratch(int L)
{
	int N = 2 * L + 1, KP = ((2 * N + 7) / 8) * 8;
	return (size_t)2 * TC_M * KP;
}
