/*
 * Device top-k of per-pose scores: the k smallest chi of a pose list in
 * ascending order, ties in list order, NaN after every number (the order of
 * a stable argsort), without copying the scores to the host.  The reference
 * writes every pose's score instead (tools/correlate.c:362-375).
 *
 *  1. keys: chi as an order-preserving unsigned 64-bit key (NaN -> all ones);
 *  2. radix select of the key of rank k-1: eight passes over the keys, one
 *     8-bit digit each, from the top; a pass histograms the digit of the
 *     keys that match the digits found so far (per-block shared-memory
 *     histograms merged with atomics) and one block picks the digit whose
 *     bin holds the rank;
 *  3. stable compaction: every key below the threshold key, then the first
 *     (in list order) of the keys equal to it, as many as the rank needs;
 *     the equal keys are counted per block of a contiguous segment, the
 *     counts scanned, and each warp places its keys by ballot prefix;
 *  4. one block sorts the k (key, position) pairs in shared memory (bitonic)
 *     and writes positions and scores.
 * The state (digits found, rank left) stays on the device, so a call queues
 * its launches without a host round trip.
 */
#include "kernels.h"

#include <stdint.h>

namespace {

#define TK_THREADS 256
#define TK_BINS 256
#define TK_SEG 4096   /* keys per block in the counting and selection passes */

struct TopkState {
	unsigned long long prefix;   /* digits found so far */
	unsigned long long mask;     /* bits they cover */
	unsigned long long rank;     /* rank of the target among keys matching prefix */
	unsigned long long nless;    /* keys below the threshold (after the last pass) */
	unsigned long long take_eq;  /* keys equal to the threshold to take */
	unsigned long long placed;   /* compaction cursor for keys below */
};

__device__ __forceinline__ unsigned long long chi_key(double x)
{
	if (isnan(x)) return ~0ull;
	unsigned long long u = (unsigned long long)__double_as_longlong(x);
	return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__global__ void k_topk_init(TopkState *__restrict__ st, int k, unsigned int *__restrict__ hist)
{
	if (threadIdx.x == 0) {
		st->prefix = 0ull;
		st->mask = 0ull;
		st->rank = (unsigned long long)(k - 1);
		st->nless = 0ull;
		st->take_eq = 0ull;
		st->placed = 0ull;
	}
	for (int i = threadIdx.x; i < TK_BINS; i += blockDim.x) hist[i] = 0;
}

__global__ void k_topk_hist(const double *__restrict__ chi, long n, int shift, const TopkState *__restrict__ st,
                            unsigned int *__restrict__ hist)
{
	__shared__ unsigned int h[TK_BINS];
	for (int i = threadIdx.x; i < TK_BINS; i += blockDim.x) h[i] = 0;
	__syncthreads();
	unsigned long long prefix = st->prefix, mask = st->mask;
	for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
		unsigned long long key = chi_key(chi[i]);
		if ((key & mask) == prefix) atomicAdd(&h[(key >> shift) & (TK_BINS - 1)], 1u);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < TK_BINS; i += blockDim.x)
		if (h[i]) atomicAdd(&hist[i], h[i]);
}

/* one block of TK_BINS threads: the digit whose bin holds the rank */
__global__ void k_topk_pick(int shift, TopkState *__restrict__ st, unsigned int *__restrict__ hist, int last)
{
	__shared__ unsigned long long cum[TK_BINS];
	int t = threadIdx.x;
	cum[t] = hist[t];
	__syncthreads();
	for (int off = 1; off < TK_BINS; off <<= 1) {   /* inclusive scan */
		unsigned long long v = t >= off ? cum[t - off] : 0;
		__syncthreads();
		cum[t] += v;
		__syncthreads();
	}
	unsigned long long rank = st->rank;
	unsigned long long below = t ? cum[t - 1] : 0;
	__syncthreads();
	if (below <= rank && rank < cum[t]) {
		st->prefix |= (unsigned long long)t << shift;
		st->mask |= (unsigned long long)(TK_BINS - 1) << shift;
		st->rank = rank - below;
		st->nless += below;
		if (last) st->take_eq = rank - below + 1;
	}
	hist[t] = 0;
}

/* keys equal to the threshold, per block of a contiguous segment */
__global__ void k_topk_count_eq(const double *__restrict__ chi, long n, const TopkState *__restrict__ st,
                                unsigned int *__restrict__ cnt)
{
	__shared__ unsigned int c;
	if (threadIdx.x == 0) c = 0;
	__syncthreads();
	unsigned long long thr = st->prefix;
	long b0 = blockIdx.x * (long)TK_SEG, b1 = min(n, b0 + TK_SEG);
	unsigned int mine = 0;
	for (long i = b0 + threadIdx.x; i < b1; i += blockDim.x) mine += chi_key(chi[i]) == thr;
	atomicAdd(&c, mine);
	__syncthreads();
	if (threadIdx.x == 0) cnt[blockIdx.x] = c;
}

/* exclusive scan of the per-block equal counts (one thread) */
__global__ void k_topk_scan(unsigned int *__restrict__ cnt, int nb)
{
	if (threadIdx.x == 0) {
		unsigned int run = 0;
		for (int b = 0; b < nb; b++) {
			unsigned int v = cnt[b];
			cnt[b] = run;
			run += v;
		}
	}
}

/* keys below the threshold anywhere in out[0, nless); equal keys of list
 * rank r < take_eq at out[nless + r]; segments as in k_topk_count_eq.  Every
 * write is checked against k (the counts make them fit). */
__global__ void k_topk_select(const double *__restrict__ chi, long n, int k, TopkState *__restrict__ st,
                              const unsigned int *__restrict__ eq_base, unsigned long long *__restrict__ okey,
                              unsigned int *__restrict__ opos)
{
	__shared__ unsigned int warp_eq[TK_THREADS / 32];
	__shared__ unsigned int run;
	unsigned long long thr = st->prefix, nless = st->nless, take = st->take_eq;
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	long b0 = blockIdx.x * (long)TK_SEG, b1 = min(n, b0 + TK_SEG);
	if (threadIdx.x == 0) run = eq_base[blockIdx.x];
	__syncthreads();
	for (long base = b0; base < b1; base += blockDim.x) {
		long i = base + threadIdx.x;
		unsigned long long key = i < b1 ? chi_key(chi[i]) : ~0ull;
		bool less = i < b1 && key < thr, eq = i < b1 && key == thr;
		if (less) {
			unsigned long long at = atomicAdd(&st->placed, 1ull);
			if (at < (unsigned long long)k) {
				okey[at] = key;
				opos[at] = (unsigned int)i;
			}
		}
		/* equal keys: list rank = block base + warps before + lanes before */
		unsigned int bal = __ballot_sync(0xffffffffu, eq);
		if (lane == 0) warp_eq[warp] = __popc(bal);
		__syncthreads();
		unsigned int before = run;
		for (int w = 0; w < warp; w++) before += warp_eq[w];
		before += __popc(bal & ((1u << lane) - 1u));
		if (eq && before < take && nless + before < (unsigned long long)k) {
			okey[nless + before] = key;
			opos[nless + before] = (unsigned int)i;
		}
		__syncthreads();
		if (threadIdx.x == 0)
			for (int w = 0; w < TK_THREADS / 32; w++) run += warp_eq[w];
		__syncthreads();
	}
}

/* bitonic sort of k (key, position) pairs by key then position, padded to
 * kp (a power of two) with the largest key; writes positions and scores */
__global__ void k_topk_sort(const unsigned long long *__restrict__ key, const unsigned int *__restrict__ pos, int k,
                            int kp, const double *__restrict__ chi, const double *__restrict__ c1,
                            const double *__restrict__ c2, int64_t *__restrict__ out_pos, double *__restrict__ out_chi,
                            double *__restrict__ out_c1, double *__restrict__ out_c2)
{
	extern __shared__ unsigned long long sk[];
	unsigned int *sp = reinterpret_cast<unsigned int *>(sk + kp);
	for (int i = threadIdx.x; i < kp; i += blockDim.x) {
		sk[i] = i < k ? key[i] : ~0ull;
		sp[i] = i < k ? pos[i] : 0xffffffffu;
	}
	__syncthreads();
	for (int size = 2; size <= kp; size <<= 1)
		for (int stride = size >> 1; stride > 0; stride >>= 1) {
			for (int i = threadIdx.x; i < kp; i += blockDim.x) {
				int j = i ^ stride;
				if (j > i) {
					bool up = (i & size) == 0;
					unsigned long long a = sk[i], b = sk[j];
					unsigned int pa = sp[i], pb = sp[j];
					bool gt = a > b || (a == b && pa > pb);
					if (gt == up) {
						sk[i] = b;
						sk[j] = a;
						sp[i] = pb;
						sp[j] = pa;
					}
				}
			}
			__syncthreads();
		}
	for (int i = threadIdx.x; i < k; i += blockDim.x) {
		unsigned int p = sp[i];
		if (out_pos) out_pos[i] = p;
		if (out_chi) out_chi[i] = chi[p];
		if (out_c1) out_c1[i] = c1[p];
		if (out_c2) out_c2[i] = c2[p];
	}
}

} // namespace

extern "C" {

size_t sxsk_topk_scratch(long n, int k)
{
	long nb = (n + TK_SEG - 1) / TK_SEG;
	return 256 + sizeof(unsigned int) * (TK_BINS + (size_t)nb) + 16 +
	       (sizeof(unsigned long long) + sizeof(unsigned int)) * (size_t)k;
}

int sxsk_topk_launches(void) { return 1 + 2 * 8 + 4; }

int sxsk_topk(const double *chi, const double *c1, const double *c2, long n, int k, void *scratch, int64_t *out_pos,
              double *out_chi, double *out_c1, double *out_c2, cudaStream_t s)
{
	if (n <= 0 || k <= 0 || k > n || k > SXSK_TOPK_MAX || n > 0xffffffffL || !scratch) return cudaErrorInvalidValue;
	unsigned char *w = (unsigned char *)scratch;
	TopkState *st = (TopkState *)w;                       /* 48 bytes in the first 256 */
	unsigned int *hist = (unsigned int *)(w + 256);
	long nb = (n + TK_SEG - 1) / TK_SEG;
	unsigned int *eq = hist + TK_BINS;
	size_t koff = 256 + sizeof(unsigned int) * (TK_BINS + (size_t)nb);
	koff = (koff + 15) / 16 * 16;
	unsigned long long *okey = (unsigned long long *)(w + koff);
	unsigned int *opos = (unsigned int *)(okey + k);
	k_topk_init<<<1, TK_BINS, 0, s>>>(st, k, hist);
	int dev = 0, nsm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	long hb = (n + TK_THREADS - 1) / TK_THREADS;
	int grid = (int)(hb < 4L * nsm ? hb : 4L * nsm);
	for (int pass = 0; pass < 8; pass++) {
		int shift = 56 - 8 * pass;
		k_topk_hist<<<grid, TK_THREADS, 0, s>>>(chi, n, shift, st, hist);
		k_topk_pick<<<1, TK_BINS, 0, s>>>(shift, st, hist, pass == 7);
	}
	k_topk_count_eq<<<(unsigned)nb, TK_THREADS, 0, s>>>(chi, n, st, eq);
	k_topk_scan<<<1, 32, 0, s>>>(eq, (int)nb);
	k_topk_select<<<(unsigned)nb, TK_THREADS, 0, s>>>(chi, n, k, st, eq, okey, opos);
	int kp = 1;
	while (kp < k) kp <<= 1;
	size_t smem = (size_t)kp * (sizeof(unsigned long long) + sizeof(unsigned int));
	if (smem > 48 * 1024) {
		cudaError_t e = cudaFuncSetAttribute(k_topk_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e) return e;
	}
	k_topk_sort<<<1, 1024, smem, s>>>(okey, opos, k, kp, chi, c1, c2, out_pos, out_chi, out_c1, out_c2);
	return cudaGetLastError();
}

} // extern "C"
