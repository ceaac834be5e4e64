/*
 * Grid fit of the mixed-precision path in double-float arithmetic: every
 * quantity is an unevaluated sum hi + lo of two floats (about 48 significant
 * bits), so the fit runs on the FP32 pipe, 64 times wider than the FP64 pipe
 * on this GPU.  The score sum a0 - up^2/down cancels by A0/chi^2 (10^3 to
 * 10^4 on SAXS data), which rules out plain FP32; 48 bits leave it far
 * inside the mixed path's |dchi| <= 1e-4 chi.
 *
 * Same algorithm and thread layout as k_fit_grid in kernels_contract.cu
 * (point_score of src/min_saxs.c:391-448 with the per-q constants folded on
 * the host); the model is normalised to 1 at q_0 instead of to the peak, and
 * the constants are scaled by peak (a1, u) and peak^2 (a3, e, f), which
 * leaves up and down unchanged and keeps every intermediate near 1.  The
 * cross terms arrive as double-float pairs (the FP32 per-pose kernel), so the
 * FP64 pipe sees one division per pose.
 *
 * Compiled with -fmad=false: the error-free transformations of
 * fitdf_core.h must not be contracted.
 */
#include "kernels.h"
#include "fitdf_core.h"

#include <string.h>

namespace {

#define FITD_THREADS 128
#define FITD_NFC 5
/* q per staged chunk at most: the pose rows of a block take
 * ppb * 8 * (qc + 1) double-floats of shared memory instead of ppb * 8 * Q */
#define FITD_QC 32
/* G(c1, q) is staged in shared memory up to this size, else read from global */
#define FITD_GSMEM (64 * 1024)

/* shared-memory carve-up of a fit block (sizes from the job's shape) */
struct FitSm {
	dfl *cs;      /* [ppb][8][qc + 1]: VV VD VW DD DW WW F3G P4 */
	dfl *fs;      /* [FITD_NFC][Q] */
	dfl *c2s;     /* [n2] */
	dfl *gs;      /* [n1][Q] G(c1, q) when gsm */
	double *red;  /* [ppb*tp][2] */
	int *redc;    /* [ppb*tp] */
	dfl *sf;      /* [ppb]: 1/norm */
	dfl *sfd;     /* [ppb][2]: U2, D4 */
	int *srcs;    /* [ppb] */
};

__device__ __forceinline__ FitSm fit_sm(const sxsk_fit_job &J, double *sm)
{
	FitSm r;
	int ld = J.qc + 1, nthr = J.ppb * J.tp;
	r.cs = reinterpret_cast<dfl *>(sm);
	r.fs = r.cs + (size_t)J.ppb * 8 * ld;
	r.c2s = r.fs + (size_t)FITD_NFC * J.Q;
	r.gs = r.c2s + J.n2;
	r.red = reinterpret_cast<double *>(r.gs + (J.gsm ? (size_t)J.n1 * J.Q : 0));
	r.redc = (int *)(r.red + 2 * nthr);
	r.sf = reinterpret_cast<dfl *>(r.redc + ((nthr + 1) & ~1));
	r.sfd = r.sf + J.ppb;
	r.srcs = (int *)(r.sfd + 2 * J.ppb);
	return r;
}

/* per-job constants of a fit block: the scaled fit constants, the c2 grid
 * and (gsm) G(c1, q) */
__device__ __forceinline__ void fit_stage(const sxsk_fit_job &J, const FitSm &m)
{
	int tid = threadIdx.x, Q = J.Q;
	double pk2 = J.peak * J.peak;
	for (int k = tid; k < FITD_NFC * Q; k += blockDim.x) {
		int c = k / Q, i = k % Q;
		m.fs[k] = df_from(J.fc[i * FITD_NFC + c] * (c < 3 ? pk2 : J.peak));
	}
	for (int k = tid; k < J.n2; k += blockDim.x) m.c2s[k] = df_from(J.c2g[k]);
	if (J.gsm)
		for (int k = tid; k < J.n1 * Q; k += blockDim.x) {
			float2 v = J.gdf[k];
			m.gs[k] = df_mk(v.x, v.y);
		}
}

/* Block = ppb poses x tp threads; thread (pose, c1 row lt, lt + tp, ...).
 * Per group of poses the q range runs in chunks of qc: the block stages the
 * chunk's normalised channel rows (plus the q before it), fills F3G and P4,
 * and every thread advances the running sums of its (pose, c1) over the
 * chunk.  After the last chunk a thread has the polynomial coefficients of
 * its row and scans the c2 cells.  One call = one group grp (block-wide,
 * after fit_stage). */
__device__ __forceinline__ void fit_group(const sxsk_fit_job &J, const FitSm &m, int grp)
{
	const float2 *__restrict__ cross = J.cross;
	int Q = J.Q, n1 = J.n1, n2 = J.n2, tp = J.tp, ppb = J.ppb, qc = J.qc;
	double a0sum = J.a0sum;
	int ld = qc + 1;                                   /* staged q per row: the previous q + the chunk */
	dfl *cs = m.cs, *fs = m.fs, *c2s = m.c2s, *sf = m.sf, *sfd = m.sfd;
	double *red = m.red;
	int *redc = m.redc, *srcs = m.srcs;
	int tid = threadIdx.x;
	int nthr = ppb * tp;
	int lp = tid / tp, lt = tid % tp;
	const dfl *gtab = J.gsm ? m.gs : reinterpret_cast<const dfl *>(J.gdf);
	int nround = (n1 + tp - 1) / tp;
	{
		int s0 = grp * ppb;
		int nhere = min(ppb, J.nslot - s0);
		bool live = tid < nthr && lp < nhere;
		__syncthreads();
		if (tid < nhere) srcs[tid] = J.order ? J.order[J.slot0 + s0 + tid].src : J.slot0 + s0 + tid;
		__syncthreads();
		if (tid < nhere) {
			/* norm = VV + DD + WW + VW - VD - DW at q_0 (the model at q_0 with
			 * c1 = 1, c2 = 1), in double-float; its inverse once in double */
			const dfl *c = reinterpret_cast<const dfl *>(cross) + (size_t)srcs[tid] * 6 * Q;
			dfl sc = df_add(df_add(df_add(c[0], c[3 * Q]), df_add(c[5 * Q], c[2 * Q])), df_neg(df_add(c[Q], c[4 * Q])));
			sf[tid] = df_from(1.0 / df_to(sc));
		}
		double bscore = __longlong_as_double(0x7ff0000000000000LL);
		int bcell = -1;
		int pid = live ? srcs[lp] : 0;
		dfl *c = cs + (size_t)lp * 8 * ld;
		for (int round = 0; round < nround; round++) {
			int j = lt + round * tp;
			bool row = live && j < n1;
			const dfl *G = gtab + (size_t)(row ? j : 0) * Q;
			df_rowst st;
			dfl u2 = df_mk(0, 0), d4 = df_mk(0, 0);
			for (int q0 = 0; q0 < Q; q0 += qc) {
				int n = min(qc, Q - q0);
				__syncthreads();   /* previous chunk done (and sf written) */
				int w = n + 1;
				for (int k = tid; k < nhere * 6 * w; k += blockDim.x) {
					int p = k / (6 * w), r = k % (6 * w);
					int ch = r / w, kk = r % w;
					int q = q0 - 1 + kk;
					dfl v = df_mk(0, 0);
					if (q >= 0) {
						float2 x = cross[(size_t)srcs[p] * 6 * Q + ch * Q + q];
						v = df_mul(df_mk(x.x, x.y), sf[p]);
					}
					cs[(size_t)p * 8 * ld + ch * ld + kk] = v;
				}
				__syncthreads();
				if (live) df_pose_prep_run(c + 1, ld, fs + q0, Q, lt, n, tp, q0 == 0, &u2, &d4);
				__syncthreads();
				if (row) {
					if (q0 == 0) df_row_init(&st, c + 1, ld, G[0]);
					df_row_run(&st, c + 1, ld, fs + q0, Q, G + q0, n);
				}
			}
			if (live) {
				red[2 * tid] = df_to(u2);
				red[2 * tid + 1] = df_to(d4);
			}
			__syncthreads();
			if (live && lt == 0) {
				/* partial sums added in double: exact enough and order-fixed */
				double a = 0, b = 0;
				for (int t = 0; t < tp; t++) {
					a += red[2 * (tid + t)];
					b += red[2 * (tid + t) + 1];
				}
				sfd[2 * lp] = df_from(a);
				sfd[2 * lp + 1] = df_from(b);
			}
			__syncthreads();
			if (row) {
				dfl U2 = sfd[2 * lp], D4 = sfd[2 * lp + 1];
				dfl u[2], d[4];
				df_row_finish(&st, u, d);
				if (J.grid) {
					for (int i2 = 0; i2 < n2; i2++) {
						double uu = df_to(df_up(u, U2, c2s[i2])), dd = df_to(df_down(d, D4, c2s[i2]));
						double k = uu / dd;
						J.grid[((size_t)pid * n1 + j) * n2 + i2] = a0sum + k * (-2.0 * uu + k * dd);
					}
				}
				dfl bu, bd;
				int bi = df_best_c2(u, U2, d, D4, c2s, n2, &bu, &bd);
				if (bi >= 0) {
					double uu = df_to(bu), dd = df_to(bd);
					double k = uu / dd;
					double score = a0sum + k * (-2.0 * uu + k * dd);
					int cell = j * n2 + bi;
					if (score < bscore || (score == bscore && cell < bcell)) {
						bscore = score;
						bcell = cell;
					}
				}
			}
		}
		if (live) {
			red[2 * tid] = bscore;
			redc[tid] = bcell;
		}
		__syncthreads();
		if (live && lt == 0) {
			for (int t = 1; t < tp; t++) {
				double os = red[2 * (tid + t)];
				int oc = redc[tid + t];
				if (oc >= 0 && (bcell < 0 || os < bscore || (os == bscore && oc < bcell))) {
					bscore = os;
					bcell = oc;
				}
			}
			if (bcell >= 0) {
				J.chi[pid] = sqrt(bscore);
				J.c1[pid] = J.c1g[bcell / n2];
				J.c2[pid] = J.c2g[bcell % n2];
			} else {
				J.chi[pid] = __longlong_as_double(0x7ff8000000000000LL);
				J.c1[pid] = __longlong_as_double(0x7ff8000000000000LL);
				J.c2[pid] = __longlong_as_double(0x7ff8000000000000LL);
			}
			if (J.cell) J.cell[pid] = bcell;
		}
	}
}

__global__ void __launch_bounds__(FITD_THREADS, 6) k_fit_grid_df(sxsk_fit_job J)   /* 6 blocks: measured faster than 5, 7, 8 */
{
	extern __shared__ double sm[];
	FitSm m = fit_sm(J, sm);
	fit_stage(J, m);
	int ngroup = (J.nslot + J.ppb - 1) / J.ppb;
	for (int grp = blockIdx.x; grp < ngroup; grp += gridDim.x) fit_group(J, m, grp);
}

/* fit groups of many dimers: items {job, group}; a block restages the
 * per-job constants when an item's job differs from the previous item's */
__global__ void __launch_bounds__(FITD_THREADS, 5)
k_fit_grid_df_batch(const sxsk_fit_job *__restrict__ jobs, const int2 *__restrict__ items, int nitems, int *ctr)
{
	extern __shared__ double sm[];
	__shared__ int s_it;
	int cur = -1;
	/* items as in the batched contraction kernels: persistent (ctr), the
	 * next item claimed while the block works on the current one, or one
	 * block per item */
	int it = (int)blockIdx.x;
	if (ctr) {
		if (threadIdx.x == 0) s_it = atomicAdd(ctr, 1);
		__syncthreads();
		it = s_it;
	}
	for (; it < nitems;) {
		int nxt = ctr && threadIdx.x == 0 ? atomicAdd(ctr, 1) : 0;
		int2 w = items[it];
		sxsk_fit_job J = jobs[w.x];
		FitSm m = fit_sm(J, sm);
		if (w.x != cur) {
			fit_stage(J, m);
			cur = w.x;
		}
		fit_group(J, m, w.y);   /* starts with a barrier: the staged constants are visible */
		if (!ctr) break;
		__syncthreads();
		if (threadIdx.x == 0) s_it = nxt;
		__syncthreads();
		it = s_it;
	}
}

} // namespace

extern "C" int sxsk_fit_df_shape(int Q, int n1, int n2, int *tp_out, int *ppb_out, int *qc_out, int *gsm_out,
                                 size_t *smem_out)
{
	if (n1 <= 0 || n2 <= 0 || Q <= 0) return cudaErrorInvalidValue;
	int tp = n1 < FITD_THREADS ? n1 : FITD_THREADS;
	int ppb = FITD_THREADS / tp;
	int nchunk = (Q + FITD_QC - 1) / FITD_QC;
	int qc = (Q + nchunk - 1) / nchunk;
	int gsm = sizeof(dfl) * (size_t)n1 * Q <= FITD_GSMEM;
	size_t smem;
	for (;;) {
		size_t nthr = (size_t)ppb * tp;
		smem = sizeof(dfl) * ((size_t)ppb * 8 * (qc + 1) + (size_t)FITD_NFC * Q + n2 + (gsm ? (size_t)n1 * Q : 0)) +
		       sizeof(double) * 2 * nthr + sizeof(int) * ((nthr + 1) & ~(size_t)1) + sizeof(dfl) * 3 * ppb +
		       sizeof(int) * ppb;
		if (smem <= 227 * 1024 || ppb == 1) break;
		ppb = (ppb + 1) / 2;
	}
	if (smem > 227 * 1024) return cudaErrorInvalidValue;
	*tp_out = tp;
	*ppb_out = ppb;
	*qc_out = qc;
	*gsm_out = gsm;
	*smem_out = smem;
	return 0;
}

extern "C" int sxsk_fit_grid_df(const float2 *cross, const sxsk_pose *order, int slot0, int nslot, int Q,
                                const double *fc, double a0sum, double peak, const float2 *gdf, const double *c1g,
                                int n1, const double *c2g, int n2, int max_blocks, double *chi, double *c1,
                                double *c2, int32_t *cell, double *grid, cudaStream_t s)
{
	if (nslot <= 0) return 0;
	sxsk_fit_job J;
	memset(&J, 0, sizeof(J));
	size_t smem = 0;
	int rc = sxsk_fit_df_shape(Q, n1, n2, &J.tp, &J.ppb, &J.qc, &J.gsm, &smem);
	if (rc) return rc;
	J.cross = cross; J.order = order; J.fc = fc; J.gdf = gdf; J.c1g = c1g; J.c2g = c2g;
	J.chi = chi; J.c1 = c1; J.c2 = c2; J.cell = cell; J.grid = grid;
	J.a0sum = a0sum; J.peak = peak; J.slot0 = slot0; J.nslot = nslot; J.Q = Q; J.n1 = n1; J.n2 = n2;
	if (smem > 48 * 1024) {
		cudaError_t e = cudaFuncSetAttribute(k_fit_grid_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
	}
	long ngroup = (nslot + J.ppb - 1) / J.ppb;
	int grid_n = (int)(ngroup < (long)max_blocks || max_blocks <= 0 ? ngroup : max_blocks);
	k_fit_grid_df<<<grid_n, FITD_THREADS, smem, s>>>(J);
	return cudaGetLastError();
}

extern "C" int sxsk_fit_grid_df_batch(const sxsk_fit_job *jobs, const int2 *items, int nitems, size_t smem, int *ctr,
                                      cudaStream_t s)
{
	if (nitems <= 0) return 0;
	cudaError_t e = cudaSuccess;
	if (smem > 48 * 1024)
		e = cudaFuncSetAttribute(k_fit_grid_df_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	int dev = 0, nsm = 0, per = 1;
	if (!e) e = cudaGetDevice(&dev);
	if (!e) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	if (!e && ctr) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fit_grid_df_batch, FITD_THREADS, smem);
	if (e) return e;
	if (per < 1) return cudaErrorInvalidConfiguration;
	long g = (long)nsm * per;
	int grid = ctr ? (int)(g < nitems ? g : nitems) : nitems;   /* persistent, or one block per item */
	k_fit_grid_df_batch<<<grid, FITD_THREADS, smem, s>>>(jobs, items, nitems, ctr);
	return cudaGetLastError();
}

namespace {
__global__ void k_to_df(const double *__restrict__ a, float2 *__restrict__ b, long n)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		dfl v = df_from(a[i]);
		b[i] = make_float2(v.hi, v.lo);
	}
}
__global__ void k_df_to_double(const float2 *a, double *b, long n)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		float2 v = a[i];             /* read before the write: a and b may alias */
		b[i] = (double)v.x + (double)v.y;
	}
}
} // namespace

extern "C" int sxsk_to_df(const double *a, float2 *b, long n, cudaStream_t s)
{
	if (n <= 0) return 0;
	if ((n + 255) / 256 > 0x7fffffffL) return cudaErrorInvalidValue;
	k_to_df<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n);
	return cudaGetLastError();
}

extern "C" int sxsk_df_to_double(const float2 *a, double *b, long n, cudaStream_t s)
{
	if (n <= 0) return 0;
	if ((n + 255) / 256 > 0x7fffffffL) return cudaErrorInvalidValue;
	k_df_to_double<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n);
	return cudaGetLastError();
}
