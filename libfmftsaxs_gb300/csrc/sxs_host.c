/*
 * Host orchestration of the GPU scoring path: device context, reusable
 * plans, the expansion entry point and the drop-in sxs_compute_saxs_scores
 * (src/fftsaxs.c:608-986 of the reference).
 *
 * The device computes, per call:
 *   tables   twiddles; self terms (fill_const); receptor rotation table
 *            P(b1,g1) and ligand rotation table U(b2,g2); j_p(qz) and the
 *            translation matrices T for every touched z
 *   per chunk of touched (z, b2, g2) combos: the translated ligand table R,
 *            then the per-pose cross terms of every pose in those combos
 *   fit      grid chi^2 over (c1, c2) or L-BFGS-B, per pose
 * Poses are grouped by (z, b2, g2) with a counting sort on the host.
 */
#define _XOPEN_SOURCE 700
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "sxs_internal.h"

/* ------------------------------------------------------------- errors */
static _Thread_local char g_err[512];

const char *sxsg_last_error(void) { return g_err; }

int sxs_fail(int code, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
	return code;
}

int sxs_cuda_fail(cudaError_t e, const char *what)
{
	return sxs_fail(-100 - (int)e, "%s: %s", what, cudaGetErrorString(e));
}

void sxs_die(const char *func, const char *msg)
{
	fprintf(stderr, "[Error] fmftsaxs-gb300, function %s: %s\n", func, msg);
	exit(EXIT_FAILURE);
}

/* ------------------------------------------------------------ context */
static pthread_mutex_t g_init_lock = PTHREAD_MUTEX_INITIALIZER;
static int g_inited = 0;
static int g_device = 0;
static cudaStream_t g_stream;
static long long g_launches = 0;

void sxs_count_launches(int n) { __atomic_add_fetch(&g_launches, n, __ATOMIC_RELAXED); }
long long sxsg_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

int sxsg_device_memory(size_t *free_bytes, size_t *total_bytes)
{
	int rc = sxs_ensure_init();
	if (rc) return rc;
	size_t f = 0, t = 0;
	SXS_CU(cudaMemGetInfo(&f, &t));
	if (free_bytes) *free_bytes = f;
	if (total_bytes) *total_bytes = t;
	return 0;
}

int sxsg_init(int device)
{
	pthread_mutex_lock(&g_init_lock);
	if (g_inited) {
		pthread_mutex_unlock(&g_init_lock);
		return 0;
	}
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if (e != cudaSuccess || n == 0) {
		pthread_mutex_unlock(&g_init_lock);
		return sxs_fail(-1, "no CUDA device available (%s)", cudaGetErrorString(e));
	}
	if (device < 0 || device >= n) {
		pthread_mutex_unlock(&g_init_lock);
		return sxs_fail(-1, "device %d out of range (%d devices)", device, n);
	}
	e = cudaSetDevice(device);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) {
		/* keep freed plan memory in this process's stream-ordered pool for
		 * the next plan instead of unmapping it at every synchronisation */
		cudaMemPool_t pool;
		if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
			uint64_t thr = UINT64_MAX;
			cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
		}
	}
	if (e != cudaSuccess) {
		pthread_mutex_unlock(&g_init_lock);
		return sxs_cuda_fail(e, "device init");
	}
	g_device = device;
	g_inited = 1;
	pthread_mutex_unlock(&g_init_lock);
	return 0;
}

int sxs_ensure_init(void)
{
	if (g_inited) {
		cudaSetDevice(g_device);
		return 0;
	}
	return sxsg_init(0);
}

cudaStream_t sxs_default_stream(void) { return g_stream; }

/* --------------------------------------------------------- expansion */
int sxsg_expand(const double *xyz, const double *vac, const double *dum, const double *sasa, double water_ff,
                int natoms, const double *q, int Q, int L, double *spf_out)
{
	if (natoms < 0 || Q <= 0 || !q || !spf_out || (natoms > 0 && (!xyz || !vac || !dum)))
		return sxs_fail(-2, "sxsg_expand: bad arguments");
	const sxs_ltables *lt;
	int rc = sxs_ltables_get(L, &lt);
	if (rc) return rc;
	cudaStream_t s = g_stream;
	int K = L + 1;
	size_t spf_n = (size_t)3 * Q * K * K * 2;
	double *wf = malloc(sizeof(double) * (natoms > 0 ? natoms : 1));
	if (!wf) return sxs_fail(-5, "out of host memory");
	for (int i = 0; i < natoms; i++) wf[i] = sasa ? water_ff * sasa[i] : 0.0;
	double *d_xyz = NULL, *d_vac = NULL, *d_dum = NULL, *d_wf = NULL, *d_q = NULL, *d_rad = NULL, *d_out = NULL;
	double2 *d_ylm = NULL;
	int na = natoms > 0 ? natoms : 1;
	cudaError_t e = cudaSuccess;
	if (!e) e = cudaMalloc((void **)&d_xyz, sizeof(double) * 3 * na);
	if (!e) e = cudaMalloc((void **)&d_vac, sizeof(double) * na);
	if (!e) e = cudaMalloc((void **)&d_dum, sizeof(double) * na);
	if (!e) e = cudaMalloc((void **)&d_wf, sizeof(double) * na);
	if (!e) e = cudaMalloc((void **)&d_q, sizeof(double) * Q);
	if (!e) e = cudaMalloc((void **)&d_rad, sxsk_expand_ws_rad(na));
	if (!e) e = cudaMalloc((void **)&d_ylm, sxsk_expand_ws_ylm(na, L));
	if (!e) e = cudaMalloc((void **)&d_out, sizeof(double) * spf_n);
	if (!e && natoms > 0) {
		e = cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, s);
		if (!e) e = cudaMemcpyAsync(d_vac, vac, sizeof(double) * natoms, cudaMemcpyHostToDevice, s);
		if (!e) e = cudaMemcpyAsync(d_dum, dum, sizeof(double) * natoms, cudaMemcpyHostToDevice, s);
		if (!e) e = cudaMemcpyAsync(d_wf, wf, sizeof(double) * natoms, cudaMemcpyHostToDevice, s);
	}
	if (!e) e = cudaMemcpyAsync(d_q, q, sizeof(double) * Q, cudaMemcpyHostToDevice, s);
	if (!e) {
		e = (cudaError_t)sxsk_expand(d_xyz, d_vac, d_dum, d_wf, natoms, d_q, Q, L, lt->d_ynorm, d_ylm, d_rad, d_out, s);
		sxs_count_launches(natoms > 0 ? sxsk_expand_launches() : 0);
	}
	if (!e) e = cudaMemcpyAsync(spf_out, d_out, sizeof(double) * spf_n, cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaStreamSynchronize(s);
	cudaFree(d_xyz); cudaFree(d_vac); cudaFree(d_dum); cudaFree(d_wf); cudaFree(d_q);
	cudaFree(d_rad); cudaFree(d_ylm); cudaFree(d_out);
	free(wf);
	if (e) return sxs_cuda_fail(e, "sxsg_expand");
	return 0;
}

/* Per-q constants of the grid fit, fc[i][5] = {a3, (a4 - q a3) h,
 * (a5 - 2 q a4 + q^2 a3) h^2, a1, (a2 - q a1) h} with h = 1 / (q_i - q_{i-1})
 * and q_{-1} = -1: point_score's buf = in - tan q and tan = D h
 * (src/min_saxs.c:391-448) substituted into its sums so that the device
 * works with in and D = in_i - in_{i-1} directly. */
void sxs_fit_constants(const double *q, const double *a, int Q, double *fc)
{
	for (int i = 0; i < Q; i++) {
		double qi = q[i], h = 1.0 / (qi - (i > 0 ? q[i - 1] : -1.0));
		const double *ai = a + 6 * i;
		fc[5 * i] = ai[3];
		fc[5 * i + 1] = (ai[4] - qi * ai[3]) * h;
		fc[5 * i + 2] = ((ai[5] - 2.0 * qi * ai[4]) + qi * qi * ai[3]) * (h * h);
		fc[5 * i + 3] = ai[1];
		fc[5 * i + 4] = (ai[2] - qi * ai[1]) * h;
	}
}

/* --------------------------------------------------------------- plan */

struct sxsg_plan {
	int L, K, N, K2, Q, nz, n1, n2, precision;
	const sxs_ltables *lt;
	cudaStream_t s;
	cudaStream_t s2;            /* per-z tables beside the rotations (ev[2], ev[3]) */
	int nsm;
	cudaEvent_t *cev;           /* per-chunk events, 3 per chunk */
	int ncev;
	double mult, peak, a0sum;
	/* resident inputs */
	double *d_A, *d_B, *d_q, *d_fc, *d_a, *d_gtab, *d_c1g, *d_c2g, *d_cst;
	float2 *d_cstf;             /* cst as double-float pairs (mixed path) */
	float2 *d_gdf;              /* gtab as {hi, lo} floats (mixed path fit) */
	double2 *d_tw;
	void *d_At, *d_Bt;          /* transposed coefficients, table precision */
	double *h_z;
	int fp32;                   /* tables in float (mixed path) */
	size_t celem;               /* bytes of one complex table entry */
	int NP;                     /* (m >= 0, l >= m) pairs */
	int NT;                     /* q tiles of 8 */
	/* rotation tables (depend on the twiddle variant) */
	void *d_P, *d_U;
	int ext_tables;             /* P and U belong to the caller (serving cache) */
	int rot_engine;             /* SXSG_ROT_*: rotation on CUDA cores or tensor cores */
	int tr_slices, rot_gamma;   /* tile choices (sxsg_plan_set_tiles; 0 = the tuned table's) */
	int tc_used;                /* the last run rotated on the tensor cores */
	float *d_amat;              /* twiddle operand of the tensor-core rotation */
	int *d_tcstat;              /* its status word (kernels.h, sxsk_rotate_tc) */
	int P_valid, U_valid;       /* caller tables already hold this run's rows */
	int tw_variant; /* -1 none, 0 simple_ft, 1 exact */
	double *h_tw;               /* host copy of the twiddles (lives with the plan) */
	int64_t run_nch;            /* chunks of the prepared run */
	int64_t *h_chunk;           /* [run_nch + 1] first slice of each chunk */
	int fuse_mode;              /* SXSG_FUSE_*: translation fused with the per-pose contraction */
	int run_fused;              /* the prepared run uses the fused path */
	int32_t *d_cstart;          /* [ncombo + 1] first sorted pose of each combo (fused path) */
	float *d_part;              /* per-pose, per-m sums of the fused path */
	size_t part_cap;            /* floats in d_part */
	/* poses */
	int64_t npose;
	int skip;
	sxsk_pose *d_poses;         /* sorted by combo */
	int ncombo;
	int32_t *h_combo, *d_combo; /* [ncombo][3]: tslot, b2, g2 */
	int64_t *h_cstart;          /* [ncombo+1] first sorted pose of each combo */
	int nslice;                 /* runs of <= SXS_SLICE combos sharing z (kernels.h) */
	int32_t *h_slices, *d_slices; /* [nslice][2]: first combo, count */
	int nzt;                    /* touched z count */
	double *h_zt, *d_zt;        /* touched z values */
	double *d_bes;
	double *d_tau;              /* [nzt][K][K][K][Q] */
	float *d_tauf;              /* float copy (mixed path) */
	/* per-chunk translated table */
	void *d_R;
	int64_t R_combos;
	size_t r_budget;
	/* outputs */
	/* cross terms [npose][6][Q]: double on the FP64 path, double-float
	 * pairs {hi, lo} (same size) on the mixed path; d_scaled is the
	 * L-BFGS-B fit's rescaled, transposed copy, allocated on its first use */
	double *d_cross, *d_chi, *d_c1, *d_c2, *d_grid, *d_scaled, *d_scale;
	int32_t *d_cell;
	int *d_iters;
	size_t out_cap;
	int last_fit;
	int last_chunks;
	int grid_valid;
	cudaEvent_t ev[6];
	double ms[5];
};

/* stream-ordered allocation on the plan's stream: plans on different
 * streams (the serving loop) never synchronise the device through the
 * allocator */
static void pfree(const sxsg_plan *p, void *x)
{
	if (x) cudaFreeAsync(x, p->s);
}

static void plan_free_poses(sxsg_plan *p)
{
	/* the side stream's last per-z tables are done before their buffers
	 * return to the pool (an unrecorded event is complete) */
	if (p->s2) cudaStreamWaitEvent(p->s, p->ev[3], 0);
	free(p->h_combo); free(p->h_cstart); free(p->h_zt); free(p->h_slices);
	pfree(p, p->d_slices);
	p->h_slices = NULL; p->d_slices = NULL; p->nslice = 0;
	pfree(p, p->d_poses); pfree(p, p->d_combo); pfree(p, p->d_zt); pfree(p, p->d_bes); pfree(p, p->d_tau);
	pfree(p, p->d_tauf); pfree(p, p->d_cstart);
	p->d_cstart = NULL;
	p->h_combo = NULL; p->h_cstart = NULL; p->h_zt = NULL;
	p->d_poses = NULL; p->d_combo = NULL; p->d_zt = NULL; p->d_bes = NULL; p->d_tau = NULL; p->d_tauf = NULL;
}

void sxsg_plan_destroy(sxsg_plan *p)
{
	if (!p) return;
	if (p->s2) cudaStreamSynchronize(p->s2);
	cudaStreamSynchronize(p->s);
	plan_free_poses(p);
	pfree(p, p->d_A); pfree(p, p->d_B); pfree(p, p->d_q); pfree(p, p->d_fc); pfree(p, p->d_a); pfree(p, p->d_gtab); pfree(p, p->d_gdf);
	pfree(p, p->d_c1g); pfree(p, p->d_c2g); pfree(p, p->d_cst); pfree(p, p->d_cstf); pfree(p, p->d_At); pfree(p, p->d_Bt);
	pfree(p, p->d_tw); pfree(p, p->d_R); pfree(p, p->d_amat); pfree(p, p->d_tcstat); pfree(p, p->d_part);
	if (!p->ext_tables) {
		pfree(p, p->d_P);
		pfree(p, p->d_U);
	}
	pfree(p, p->d_cross); pfree(p, p->d_chi); pfree(p, p->d_c1); pfree(p, p->d_c2); pfree(p, p->d_grid);
	pfree(p, p->d_scaled); pfree(p, p->d_scale); pfree(p, p->d_cell); pfree(p, p->d_iters);
	for (int i = 0; i < 6; i++) if (p->ev[i]) cudaEventDestroy(p->ev[i]);
	if (p->s2) cudaStreamDestroy(p->s2);
	for (int i = 0; i < p->ncev; i++) cudaEventDestroy(p->cev[i]);
	free(p->cev);
	free(p->h_z);
	free(p->h_tw);
	free(p->h_chunk);
	free(p);
}

int sxsg_plan_create(sxsg_plan **out, const double *A, const double *B, const double *q, int Q, const double *z,
                     int nz, int L, const double *a, double mult, double peak, const double *c1g, int n1,
                     const double *c2g, int n2, int precision)
{
	return sxs_plan_create_on(out, A, B, q, Q, z, nz, L, a, mult, peak, c1g, n1, c2g, n2, precision, NULL, 0);
}

int sxs_plan_create_on(sxsg_plan **out, const double *A, const double *B, const double *q, int Q, const double *z,
                       int nz, int L, const double *a, double mult, double peak, const double *c1g, int n1,
                       const double *c2g, int n2, int precision, cudaStream_t stream, int ext_tables)
{
	if (!out || !A || !B || !q || Q <= 0 || Q > 1024 || !z || nz <= 0 || !a)
		return sxs_fail(-2, "sxsg_plan_create: bad arguments (Q must be in [1, 1024])");
	if ((n1 > 0 && !c1g) || (n2 > 0 && !c2g) || n1 < 0 || n2 < 0)
		return sxs_fail(-2, "sxsg_plan_create: bad fit grid");
	if (precision != SXSG_FP64 && precision != SXSG_MIXED)
		return sxs_fail(-2, "sxsg_plan_create: unknown precision %d", precision);
	const sxs_ltables *lt;
	int rc = sxs_ltables_get(L, &lt);
	if (rc) return rc;
	sxsg_plan *p = calloc(1, sizeof(*p));
	if (!p) return sxs_fail(-5, "out of host memory");
	p->L = L; p->K = L + 1; p->N = 2 * L + 1; p->K2 = p->K * p->K; p->Q = Q; p->nz = nz;
	p->n1 = n1; p->n2 = n2; p->precision = precision; p->lt = lt; p->s = stream ? stream : g_stream;
	p->ext_tables = ext_tables;
	p->mult = mult; p->peak = peak; p->tw_variant = -1;
	p->fp32 = precision == SXSG_MIXED;
	p->celem = p->fp32 ? 2 * sizeof(float) : 2 * sizeof(double);
	p->NP = p->K * (p->K + 1) / 2;
	p->NT = (Q + SXS_QT - 1) / SXS_QT;
	double s0 = 0.0;
	for (int i = 0; i < Q; i++) s0 += a[6 * i];
	p->a0sum = s0;
	p->h_z = malloc(sizeof(double) * nz);
	if (!p->h_z) {
		free(p);
		return sxs_fail(-5, "out of host memory");
	}
	memcpy(p->h_z, z, sizeof(double) * nz);
	size_t spf_n = (size_t)3 * Q * p->K2 * 2;
	cudaError_t e = cudaSuccess;
	for (int i = 0; i < 6 && !e; i++) e = cudaEventCreate(&p->ev[i]);
	if (!e) e = cudaStreamCreateWithFlags(&p->s2, cudaStreamNonBlocking);
	if (!e) {
		int dev = 0;
		e = cudaGetDevice(&dev);
		if (!e) e = cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev);
	}
	if (!e) e = cudaMallocAsync((void **)&p->d_A, sizeof(double) * spf_n, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_B, sizeof(double) * spf_n, p->s);
	if (!e) e = cudaMallocAsync(&p->d_At, p->celem * spf_n / 2, p->s);
	if (!e) e = cudaMallocAsync(&p->d_Bt, p->celem * spf_n / 2, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_q, sizeof(double) * Q, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_fc, sizeof(double) * 5 * Q, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_a, sizeof(double) * 6 * Q, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_cst, sizeof(double) * 6 * Q, p->s);
	if (!e && p->fp32) e = cudaMallocAsync((void **)&p->d_cstf, sizeof(float2) * 6 * Q, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_tw, sizeof(double2) * p->N, p->s);
	if (!e && n1 > 0) e = cudaMallocAsync((void **)&p->d_gtab, sizeof(double) * n1 * Q, p->s);
	if (!e && n1 > 0) e = cudaMallocAsync((void **)&p->d_c1g, sizeof(double) * n1, p->s);
	if (!e && n2 > 0) e = cudaMallocAsync((void **)&p->d_c2g, sizeof(double) * n2, p->s);
	size_t rot_n = (size_t)p->NT * p->K * p->N * p->NP * 3 * SXS_QT;
	if (!ext_tables) {
		if (!e) e = cudaMallocAsync(&p->d_P, p->celem * rot_n, p->s);
		if (!e) e = cudaMallocAsync(&p->d_U, p->celem * rot_n, p->s);
		/* q-tile padding stays zero */
		if (!e) e = cudaMemsetAsync(p->d_P, 0, p->celem * rot_n, p->s);
		if (!e) e = cudaMemsetAsync(p->d_U, 0, p->celem * rot_n, p->s);
	}
	if (e) {
		sxsg_plan_destroy(p);
		return sxs_cuda_fail(e, "sxsg_plan_create allocation");
	}
	cudaStream_t s = p->s;
	e = cudaMemcpyAsync(p->d_A, A, sizeof(double) * spf_n, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(p->d_B, B, sizeof(double) * spf_n, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(p->d_q, q, sizeof(double) * Q, cudaMemcpyHostToDevice, s);
	if (!e) {
		double *fc = malloc(sizeof(double) * 5 * Q);
		if (!fc) {
			e = cudaErrorMemoryAllocation;
		} else {
			sxs_fit_constants(q, a, Q, fc);
			e = cudaMemcpyAsync(p->d_fc, fc, sizeof(double) * 5 * Q, cudaMemcpyHostToDevice, p->s);
			/* pageable source: the copy has taken it when the call returns */
			free(fc);
		}
	}
	if (!e) e = cudaMemcpyAsync(p->d_a, a, sizeof(double) * 6 * Q, cudaMemcpyHostToDevice, s);
	if (!e && n1 > 0) {
		/* G(c1, q) = c1^3 exp(-mult (c1^2 - 1) q^2) exactly as point_score
		 * evaluates it (src/min_saxs.c:404-423) */
		double *g = malloc(sizeof(double) * n1 * Q);
		if (!g) {
			sxsg_plan_destroy(p);
			return sxs_fail(-5, "out of host memory");
		}
		for (int i = 0; i < n1; i++) {
			double c1 = c1g[i];
			double corr = -mult * (c1 * c1 - 1.0);
			double c1c = c1 * c1 * c1;
			for (int k = 0; k < Q; k++) g[(size_t)i * Q + k] = c1c * exp(corr * q[k] * q[k]);
		}
		e = cudaMemcpyAsync(p->d_gtab, g, sizeof(double) * n1 * Q, cudaMemcpyHostToDevice, p->s);
		if (!e && p->fp32) {
			float *gd = malloc(sizeof(float) * 2 * n1 * Q);
			if (!gd) {
				free(g);
				sxsg_plan_destroy(p);
				return sxs_fail(-5, "out of host memory");
			}
			for (size_t k = 0; k < (size_t)n1 * Q; k++) {
				float h = (float)g[k];
				gd[2 * k] = h;
				gd[2 * k + 1] = (float)(g[k] - (double)h);
			}
			e = cudaMallocAsync((void **)&p->d_gdf, sizeof(float2) * n1 * Q, p->s);
			if (!e) e = cudaMemcpyAsync(p->d_gdf, gd, sizeof(float2) * n1 * Q, cudaMemcpyHostToDevice, p->s);
			free(gd);
		}
		free(g);
		if (!e) e = cudaMemcpyAsync(p->d_c1g, c1g, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
	}
	if (!e && n2 > 0) e = cudaMemcpyAsync(p->d_c2g, c2g, sizeof(double) * n2, cudaMemcpyHostToDevice, s);
	if (!e) {
		e = (cudaError_t)sxsk_spf_transpose(p->d_A, p->d_At, Q, L, p->fp32, s);
		if (!e) e = (cudaError_t)sxsk_spf_transpose(p->d_B, p->d_Bt, Q, L, p->fp32, s);
		if (!e) e = (cudaError_t)sxsk_const_int(p->d_A, p->d_B, Q, L, p->d_cst, s);
		sxs_count_launches(3);
		if (!e && p->fp32) {
			e = (cudaError_t)sxsk_to_df(p->d_cst, p->d_cstf, 6L * Q, s);
			sxs_count_launches(1);
		}
	}
	if (!e) e = cudaStreamSynchronize(s);
	if (e) {
		sxsg_plan_destroy(p);
		return sxs_cuda_fail(e, "sxsg_plan_create upload");
	}
	size_t fr = 0, tot = 0;
	cudaMemGetInfo(&fr, &tot);
	p->r_budget = fr / 2;
	sxsg_tiles_default(L, Q, &p->tr_slices, &p->rot_gamma);
	*out = p;
	return 0;
}

#include "tiles_table.h"

int sxsg_tiles_default(int L, int Q, int *tr_slices, int *rot_gamma)
{
	int best = 0;
	long bd = -1;
	for (int i = 0; i < (int)(sizeof(sxs_tiles_table) / sizeof(sxs_tiles_table[0])); i++) {
		long d = 100000L * labs((long)sxs_tiles_table[i].L - L) + labs((long)sxs_tiles_table[i].Q - Q);
		if (bd < 0 || d < bd) {
			bd = d;
			best = i;
		}
	}
	if (tr_slices) *tr_slices = sxs_tiles_table[best].tr_slices;
	if (rot_gamma) *rot_gamma = sxs_tiles_table[best].rot_gamma;
	return 0;
}

int sxsg_plan_set_tiles(sxsg_plan *p, int tr_slices, int rot_gamma)
{
	if (!p || tr_slices < 0 || tr_slices > 64 || (rot_gamma != 0 && rot_gamma != 2 && rot_gamma != 4 &&
	                                              rot_gamma != 6 && rot_gamma != 8 && rot_gamma != 12 &&
	                                              rot_gamma != 16))
		return sxs_fail(-2, "sxsg_plan_set_tiles: bad tile choice");
	int dsb = 0, dg = 0;
	sxsg_tiles_default(p->L, p->Q, &dsb, &dg);
	p->tr_slices = tr_slices ? tr_slices : dsb;
	p->rot_gamma = rot_gamma ? rot_gamma : dg;
	return 0;
}

int sxsg_plan_set_rotation(sxsg_plan *p, int engine)
{
	if (!p || (engine != SXSG_ROT_CUDA && engine != SXSG_ROT_TC))
		return sxs_fail(-2, "sxsg_plan_set_rotation: bad arguments");
	p->rot_engine = engine;
	return 0;
}

int sxsg_plan_set_budget(sxsg_plan *p, size_t bytes)
{
	if (!p) return sxs_fail(-2, "sxsg_plan_set_budget: null plan");
	p->r_budget = bytes;
	size_t per_combo = (size_t)p->NP * 3 * SXS_QT * p->NT * p->celem;
	if (p->d_R && (size_t)p->R_combos * per_combo > bytes) {
		/* stream-ordered: runs already queued keep their buffer */
		pfree(p, p->d_R);
		p->d_R = NULL;
		p->R_combos = 0;
	}
	return 0;
}

static int grow(sxsg_plan *p, void **ptr, size_t *cap, size_t need, size_t elem)
{
	if (*cap >= need && *ptr) return 0;
	pfree(p, *ptr);
	*ptr = NULL;
	size_t n = need > 0 ? need : 1;
	cudaError_t e = cudaMallocAsync(ptr, n * elem, p->s);
	if (e) {
		*cap = 0;
		return sxs_cuda_fail(e, "device allocation");
	}
	*cap = n;
	return 0;
}

int sxsg_plan_set_poses(sxsg_plan *p, const int64_t *index, int64_t n, int skip)
{
	if (!p || n < 0 || (n > 0 && !index)) return sxs_fail(-2, "sxsg_plan_set_poses: bad arguments");
	if (n > INT32_MAX) return sxs_fail(-2, "sxsg_plan_set_poses: at most 2^31-1 poses per plan");
	int L = p->L, N = p->N, nb = p->K, nz = p->nz;
	int64_t nkey = (int64_t)nz * nb * N;
	if (nkey > INT32_MAX) return sxs_fail(-2, "sxsg_plan_set_poses: znum (L+1) (2L+1) must be below 2^31");
	plan_free_poses(p);
	p->npose = n;
	p->skip = skip;
	p->grid_valid = 0;
	cudaStream_t s = p->s;
	size_t nn = (size_t)(n > 0 ? n : 1);
	/* decode and count keys (zi, b2, g2) on the device */
	int64_t *d_idx = NULL;
	sxsk_pose *d_tmp = NULL;
	int32_t *d_key = NULL, *d_cnt = NULL, *d_zu = NULL, *d_cid = NULL;
	unsigned long long *d_err = NULL, h_err[2] = {0, 0};
	int32_t *h_cnt = malloc(sizeof(int32_t) * (size_t)(nkey > 0 ? nkey : 1));
	int32_t *h_zu = malloc(sizeof(int32_t) * (size_t)(nz > 0 ? nz : 1));
	int32_t *h_cid = malloc(sizeof(int32_t) * (size_t)(nkey > 0 ? nkey : 1));
	int *zslot = malloc(sizeof(int) * (size_t)(nz > 0 ? nz : 1));
	int rc = 0;
	cudaError_t e = (h_cnt && h_zu && h_cid && zslot) ? cudaSuccess : cudaErrorMemoryAllocation;
	if (!e) e = cudaMallocAsync((void **)&d_idx, sizeof(int64_t) * nn, s);
	if (!e) e = cudaMallocAsync((void **)&d_tmp, sizeof(sxsk_pose) * nn, s);
	if (!e) e = cudaMallocAsync((void **)&d_key, sizeof(int32_t) * nn, s);
	if (!e) e = cudaMallocAsync((void **)&d_cnt, sizeof(int32_t) * (size_t)(nkey > 0 ? nkey : 1), s);
	if (!e) e = cudaMallocAsync((void **)&d_cid, sizeof(int32_t) * (size_t)(nkey > 0 ? nkey : 1), s);
	if (!e) e = cudaMallocAsync((void **)&d_zu, sizeof(int32_t) * (size_t)(nz > 0 ? nz : 1), s);
	if (!e) e = cudaMallocAsync((void **)&d_err, sizeof(h_err), s);
	if (!e) e = cudaMemsetAsync(d_cnt, 0, sizeof(int32_t) * (size_t)nkey, s);
	if (!e) e = cudaMemsetAsync(d_zu, 0, sizeof(int32_t) * (size_t)nz, s);
	if (!e) e = cudaMemsetAsync(d_err, 0xff, sizeof(h_err), s);
	if (!e && n > 0) e = cudaMemcpyAsync(d_idx, index, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, s);
	if (!e) e = (cudaError_t)sxsk_pose_decode(d_idx, n, N, nb, nz, d_tmp, d_key, d_cnt, d_zu, d_err, s);
	if (!e) e = cudaMemcpyAsync(h_err, d_err, sizeof(h_err), cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaMemcpyAsync(h_cnt, d_cnt, sizeof(int32_t) * (size_t)nkey, cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaMemcpyAsync(h_zu, d_zu, sizeof(int32_t) * (size_t)nz, cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaStreamSynchronize(s);
	if (!e) sxs_count_launches(n > 0 ? 1 : 0);
	if (!e && (h_err[0] != ~0ULL || h_err[1] != ~0ULL)) {
		/* the first bad pose in list order, with the reference's message */
		long long i = (long long)(h_err[0] < h_err[1] ? h_err[0] : h_err[1]);
		if (h_err[0] < h_err[1])
			rc = sxs_fail(-3, "pose %lld: negative grid index %lld", i, (long long)index[i]);
		else
			rc = sxs_fail(-3, "pose %lld: translation slot %lld >= znum %d", i,
			              (long long)(index[i] / ((int64_t)N * N * N * nb * nb)), nz);
	}
	int ncombo = 0, nzt = 0;
	if (!e && !rc) {
		/* touched z -> slot */
		for (int i = 0; i < nz; i++) zslot[i] = h_zu[i] ? nzt++ : -1;
		p->nzt = nzt;
		for (int64_t k = 0; k < nkey; k++) if (h_cnt[k]) ncombo++;
		p->ncombo = ncombo;
		p->h_zt = malloc(sizeof(double) * (nzt > 0 ? nzt : 1));
		p->h_combo = malloc(sizeof(int32_t) * 3 * (ncombo > 0 ? ncombo : 1));
		p->h_cstart = malloc(sizeof(int64_t) * (ncombo + 1));
		p->h_slices = malloc(sizeof(int32_t) * 2 * (ncombo > 0 ? ncombo : 1));
		if (!p->h_zt || !p->h_combo || !p->h_cstart || !p->h_slices) rc = sxs_fail(-5, "out of host memory");
	}
	if (!e && !rc) {
		for (int i = 0; i < nz; i++) if (zslot[i] >= 0) p->h_zt[zslot[i]] = p->h_z[i];
		/* combos in key order; h_cnt becomes the first slot of each key */
		int c = 0;
		int32_t run = 0;
		for (int64_t k = 0; k < nkey; k++) {
			int32_t m = h_cnt[k];
			h_cnt[k] = run;
			if (m) {
				h_cid[k] = c;
				int g2 = (int)(k % N), b2 = (int)((k / N) % nb), zi = (int)(k / N / nb);
				p->h_combo[3 * c] = zslot[zi];
				p->h_combo[3 * c + 1] = b2;
				p->h_combo[3 * c + 2] = g2;
				p->h_cstart[c] = run;
				c++;
			} else {
				h_cid[k] = -1;
			}
			run += m;
		}
		p->h_cstart[ncombo] = n;
		/* slices for the translation kernel */
		p->nslice = 0;
		for (int k = 0; k < ncombo; k++) {
			int ns = p->nslice;
			if (ns > 0 && p->h_slices[2 * ns - 1] < SXS_SLICE && p->h_combo[3 * (k - 1)] == p->h_combo[3 * k]) {
				p->h_slices[2 * ns - 1]++;
			} else {
				p->h_slices[2 * ns] = k;
				p->h_slices[2 * ns + 1] = 1;
				p->nslice++;
			}
		}
		/* sorted by combo on the device (order inside a combo is free: each
		 * pose's result depends only on its own rows) */
		e = cudaMallocAsync((void **)&p->d_poses, sizeof(sxsk_pose) * nn, s);
		if (!e) e = cudaMemcpyAsync(d_cnt, h_cnt, sizeof(int32_t) * (size_t)nkey, cudaMemcpyHostToDevice, s);
		if (!e) e = cudaMemcpyAsync(d_cid, h_cid, sizeof(int32_t) * (size_t)nkey, cudaMemcpyHostToDevice, s);
		if (!e) e = (cudaError_t)sxsk_pose_scatter(d_tmp, d_key, n, d_cnt, d_cid, p->d_poses, s);
		if (!e) sxs_count_launches(n > 0 ? 1 : 0);
		/* the host arrays above are read by the copies: wait before freeing */
		if (!e) e = cudaStreamSynchronize(s);
	}
	pfree(p, d_idx); pfree(p, d_tmp); pfree(p, d_key); pfree(p, d_cnt);
	pfree(p, d_cid); pfree(p, d_zu); pfree(p, d_err);
	free(h_cnt); free(h_zu); free(h_cid); free(zslot);
	if (e || rc) {
		plan_free_poses(p);
		p->npose = 0;
		p->ncombo = p->nzt = 0;
		return e ? sxs_cuda_fail(e, "sxsg_plan_set_poses") : rc;
	}

	/* upload */
	e = cudaSuccess;
	if (!e) e = cudaMallocAsync((void **)&p->d_combo, sizeof(int32_t) * 3 * (ncombo > 0 ? ncombo : 1), p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_zt, sizeof(double) * (nzt > 0 ? nzt : 1), p->s);
	if (!e && nzt > 0) e = cudaMallocAsync((void **)&p->d_bes, sizeof(double) * (size_t)nzt * p->Q * N, p->s);
	size_t tau_n = (size_t)p->NT * nzt * p->K * p->K * p->K * SXS_QT;
	if (!e && nzt > 0) e = cudaMallocAsync((void **)&p->d_tau, sizeof(double) * tau_n, p->s);
	if (!e && nzt > 0 && p->fp32) e = cudaMallocAsync((void **)&p->d_tauf, sizeof(float) * tau_n, p->s);
	if (!e && ncombo > 0) e = cudaMemcpyAsync(p->d_combo, p->h_combo, sizeof(int32_t) * 3 * ncombo, cudaMemcpyHostToDevice, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_slices, sizeof(int32_t) * 2 * (p->nslice > 0 ? p->nslice : 1), p->s);
	if (!e && p->nslice > 0)
		e = cudaMemcpyAsync(p->d_slices, p->h_slices, sizeof(int32_t) * 2 * p->nslice, cudaMemcpyHostToDevice, p->s);
	if (!e && nzt > 0) e = cudaMemcpyAsync(p->d_zt, p->h_zt, sizeof(double) * nzt, cudaMemcpyHostToDevice, p->s);
	if (!e) {
		/* combo starts for the fused path (pose counts fit int32) */
		int32_t *cs = malloc(sizeof(int32_t) * (ncombo + 1));
		if (!cs) return sxs_fail(-5, "out of host memory");
		for (int k = 0; k <= ncombo; k++) cs[k] = (int32_t)p->h_cstart[k];
		e = cudaMallocAsync((void **)&p->d_cstart, sizeof(int32_t) * (ncombo + 1), p->s);
		if (!e) e = cudaMemcpyAsync(p->d_cstart, cs, sizeof(int32_t) * (ncombo + 1), cudaMemcpyHostToDevice, p->s);
		if (!e) e = cudaStreamSynchronize(p->s);
		free(cs);
	}
	if (e) return sxs_cuda_fail(e, "sxsg_plan_set_poses upload");
	size_t need = (size_t)nn;
	if ((rc = grow(p, (void **)&p->d_cross, &p->out_cap, need * 6 * p->Q, sizeof(double)))) return rc;
	/* out_cap tracks d_cross in doubles; the per-pose vectors follow it */
	pfree(p, p->d_chi); pfree(p, p->d_c1); pfree(p, p->d_c2); pfree(p, p->d_cell); pfree(p, p->d_scaled);
	pfree(p, p->d_scale); pfree(p, p->d_iters); pfree(p, p->d_grid);
	p->d_chi = p->d_c1 = p->d_c2 = p->d_scaled = p->d_scale = p->d_grid = NULL;
	p->d_cell = NULL; p->d_iters = NULL;
	e = cudaMallocAsync((void **)&p->d_chi, sizeof(double) * nn, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_c1, sizeof(double) * nn, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_c2, sizeof(double) * nn, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_cell, sizeof(int32_t) * nn, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_scale, sizeof(double) * nn, p->s);
	if (!e) e = cudaMallocAsync((void **)&p->d_iters, sizeof(int) * nn, p->s);
	if (e) return sxs_cuda_fail(e, "sxsg_plan_set_poses outputs");
	(void)L;
	return 0;
}

/* per-z tables: Bessel values and translation matrices (FP64), with their
 * float copy on the mixed path */
static int plan_ztables(sxsg_plan *p, cudaStream_t s)
{
	int L = p->L, Q = p->Q;
	SXS_K(sxsk_bessel_z(p->d_zt, p->nzt, p->d_q, Q, L, p->d_bes, s));
	SXS_K(sxsk_tmatrix(p->d_bes, p->lt->d_dsymb, p->nzt, Q, L, p->lt->d_ll1, p->lt->nll1, p->d_tau, s));
	sxs_count_launches(2);
	if (p->fp32) {
		SXS_K(sxsk_to_float(p->d_tau, p->d_tauf, (long)p->NT * p->nzt * p->K * p->K * p->K * SXS_QT, s));
		sxs_count_launches(1);
	}
	return 0;
}

static int plan_rotations(sxsg_plan *p);

/* The per-z tables (FP64 pipe) run on the side stream beside the
 * rotations (FP32 pipe); the plan stream waits for them before it goes on,
 * also when a rotation launch failed, so no later work of the plan stream
 * overtakes them. */
static int plan_tables(sxsg_plan *p)
{
	cudaStream_t s = p->s;
	int side = p->nzt > 0 && p->s2, rc = 0;
	if (!side) {
		rc = plan_rotations(p);
		if (!rc && p->nzt > 0) rc = plan_ztables(p, s);
		return rc;
	}
	SXS_CU(cudaEventRecord(p->ev[2], s));
	SXS_CU(cudaStreamWaitEvent(p->s2, p->ev[2], 0));
	rc = plan_ztables(p, p->s2);
	cudaError_t e = cudaEventRecord(p->ev[3], p->s2);
	if (!rc && !e) rc = plan_rotations(p);
	if (!e) e = cudaStreamWaitEvent(s, p->ev[3], 0);
	if (e) return sxs_cuda_fail(e, "side stream of the per-z tables");
	return rc;
}

static int plan_rotations(sxsg_plan *p)
{
	int L = p->L, Q = p->Q, N = p->N;
	cudaStream_t s = p->s;
	/* every run rebuilds the rotation tables: a run is the whole per-call
	 * work of the reference's sxs_compute_saxs_scores */
	{
		const void *dtab = p->fp32 ? (const void *)p->lt->d_dtabf : (const void *)p->lt->d_dtab;
		int tc = p->fp32 && p->rot_engine == SXSG_ROT_TC && 2 * N <= 128;
		if (tc) SXS_CU(cudaMemsetAsync(p->d_tcstat, 0, sizeof(int), s));
		if (!p->ext_tables || !p->P_valid) {
			if (tc) SXS_K(sxsk_rotate_tc(p->d_At, p->lt->d_dtabf, p->d_tw, Q, L, 0, p->d_P, p->d_amat, p->d_tcstat, s));
			else SXS_K(sxsk_rotate(p->d_At, dtab, p->d_tw, Q, L, 0, p->d_P, p->fp32, p->rot_gamma, s));
			sxs_count_launches(tc ? 2 : 1);
		}
		if (!p->ext_tables || !p->U_valid) {
			if (tc) SXS_K(sxsk_rotate_tc(p->d_Bt, p->lt->d_dtabf, p->d_tw, Q, L, 1, p->d_U, p->d_amat, p->d_tcstat, s));
			else SXS_K(sxsk_rotate(p->d_Bt, dtab, p->d_tw, Q, L, 1, p->d_U, p->fp32, p->rot_gamma, s));
			sxs_count_launches(tc ? 2 : 1);
		}
		p->tc_used = tc;
		if (p->ext_tables) p->P_valid = p->U_valid = 1;
	}
	return 0;
}

/* grid fit of all n poses (list order) in the plan's precision: FP64 on
 * the plain path, double-float on the FP32 pipe on the mixed path (whose
 * cross terms are double-float pairs); one block per group of poses */
static int plan_fit_grid(sxsg_plan *p, int n, double *chi, double *c1, double *c2, int32_t *cell, double *grid,
                         cudaStream_t st)
{
	if (p->fp32)
		return sxsk_fit_grid_df((const float2 *)p->d_cross, NULL, 0, n, p->Q, p->d_fc, p->a0sum, p->peak, p->d_gdf,
		                        p->d_c1g, p->n1, p->d_c2g, p->n2, 0, chi, c1, c2, cell, grid, st);
	return sxsk_fit_grid(p->d_cross, NULL, 0, n, p->Q, p->d_fc, p->a0sum, p->peak, p->d_gtab, p->d_c1g, p->n1,
	                     p->d_c2g, p->n2, 0, chi, c1, c2, cell, grid, st);
}

static int plan_events(sxsg_plan *p, int need)
{
	if (need <= p->ncev) return 0;
	cudaEvent_t *ev = realloc(p->cev, sizeof(cudaEvent_t) * need);
	if (!ev) return sxs_fail(-5, "out of host memory");
	p->cev = ev;
	while (p->ncev < need) {
		SXS_CU(cudaEventCreate(&p->cev[p->ncev]));
		p->ncev++;
	}
	return 0;
}

/* SXSG_FUSE_AUTO keeps the stored rows: on GB300 the fused form measured
 * slower at every density tried (1.1-12 poses per translated row, L 10-30):
 * its receptor-row gathers run at the translation's occupancy (1-2 blocks of
 * 4 warps per SM), where the per-pose kernel streams them at 6 blocks */
int sxs_plan_uses_fused(const sxsg_plan *p)
{
	return p->fp32 && p->L + 1 <= 32 && p->ncombo > 0 && p->fuse_mode == SXSG_FUSE_ON;
}

int sxsg_plan_set_fused(sxsg_plan *p, int mode)
{
	if (!p) return sxs_fail(-2, "sxsg_plan_set_fused: null plan");
	if (mode < SXSG_FUSE_AUTO || mode > SXSG_FUSE_OFF) return sxs_fail(-2, "sxsg_plan_set_fused: unknown mode %d", mode);
	if (mode == SXSG_FUSE_ON && (!p->fp32 || p->L + 1 > 32))
		return sxs_fail(-2, "sxsg_plan_set_fused: the fused path needs a mixed-precision plan with L <= 31");
	p->fuse_mode = mode;
	return 0;
}

int sxs_plan_batch_view(sxsg_plan *p, sxs_plan_view *v)
{
	int variant = p->skip == 1 ? 0 : 1;
	if (!p->h_tw) {
		p->h_tw = malloc(sizeof(double) * 2 * p->N);
		if (!p->h_tw) return sxs_fail(-5, "out of host memory");
	}
	if (p->tw_variant != variant) {
		sxs_twiddles_host(p->N, variant, p->h_tw);
		SXS_CU(cudaMemcpyAsync(p->d_tw, p->h_tw, sizeof(double2) * p->N, cudaMemcpyHostToDevice, p->s));
		p->tw_variant = variant;
	}
	SXS_CU(cudaStreamSynchronize(p->s));
	memset(v, 0, sizeof(*v));
	v->L = p->L; v->Q = p->Q; v->NT = p->NT; v->NP = p->NP; v->n1 = p->n1; v->n2 = p->n2; v->fp32 = p->fp32;
	v->ext_tables = p->ext_tables; v->nzt = p->nzt; v->ncombo = p->ncombo; v->nslice = p->nslice;
	v->tr_slices = p->tr_slices; v->rot_gamma = p->rot_gamma; v->npose = p->npose;
	v->fused = sxs_plan_uses_fused(p); v->cstart = p->d_cstart;
	v->At = p->d_At; v->Bt = p->d_Bt; v->dtabf = p->lt->d_dtabf; v->tw = p->d_tw; v->P = p->d_P; v->U = p->d_U;
	v->tauf = p->d_tauf; v->combo = p->d_combo; v->slices = p->d_slices; v->h_slices = p->h_slices;
	v->h_cstart = p->h_cstart; v->poses = p->d_poses; v->cst = p->d_cstf; v->cross = p->d_cross;
	v->fc = p->d_fc; v->c1g = p->d_c1g; v->c2g = p->d_c2g; v->gdf = p->d_gdf; v->a0sum = p->a0sum; v->peak = p->peak;
	v->chi = p->d_chi; v->c1 = p->d_c1; v->c2 = p->d_c2; v->cell = p->d_cell;
	return 0;
}

int sxs_plan_ztables_on(sxsg_plan *p, cudaStream_t s)
{
	return p->nzt > 0 ? plan_ztables(p, s) : 0;
}

void sxs_plan_mark_run(sxsg_plan *p, int fit_mode, const float *ms)
{
	p->last_fit = fit_mode;
	p->grid_valid = 0;
	p->tc_used = 0;
	for (int i = 0; i < 5; i++) p->ms[i] = ms ? ms[i] : 0.0;
}

/* Host work before a run's launches: the twiddles (host copy kept with the
 * plan, so the upload needs no wait), the tensor-core scratch, the
 * translated table's chunking, its buffer and the timing events, the
 * L-BFGS-B workspace.  After it, sxs_plan_enqueue issues only stream work
 * that a CUDA graph can capture. */
int sxs_plan_prepare(sxsg_plan *p, int fit_mode)
{
	if (fit_mode == SXSG_FIT_GRID && (p->n1 <= 0 || p->n2 <= 0))
		return sxs_fail(-2, "sxsg_plan_run: grid fit needs a (c1, c2) grid");
	if (fit_mode < 0 || fit_mode > 2) return sxs_fail(-2, "sxsg_plan_run: unknown fit mode %d", fit_mode);
	cudaStream_t s = p->s;
	int N = p->N, rc;
	int variant = p->skip == 1 ? 0 : 1;
	if (!p->h_tw) {
		p->h_tw = malloc(sizeof(double) * 2 * N);
		if (!p->h_tw) return sxs_fail(-5, "out of host memory");
	}
	if (p->tw_variant != variant) {
		sxs_twiddles_host(N, variant, p->h_tw);
		SXS_CU(cudaMemcpyAsync(p->d_tw, p->h_tw, sizeof(double2) * N, cudaMemcpyHostToDevice, s));
		p->tw_variant = variant;
	}
	int tc = p->fp32 && p->rot_engine == SXSG_ROT_TC && 2 * N <= 128;
	if (tc && !p->d_amat)
		SXS_CU(cudaMallocAsync((void **)&p->d_amat, sizeof(float) * sxsk_rotate_tc_scratch(p->L), s));
	if (tc && !p->d_tcstat) SXS_CU(cudaMallocAsync((void **)&p->d_tcstat, sizeof(int), s));
	p->run_fused = sxs_plan_uses_fused(p);
	free(p->h_chunk);
	p->h_chunk = malloc(sizeof(int64_t) * (size_t)(p->nslice + 1));
	if (!p->h_chunk) return sxs_fail(-5, "out of host memory");
	int64_t nch = 0;
	if (p->run_fused) {
		/* chunks of whole slices whose poses' sums fit the budget */
		size_t per_pose = sizeof(float) * sxsk_fused_part_floats(p->L, p->Q);
		int64_t cap = (int64_t)(p->r_budget / per_pose), most = 0;
		int64_t s0 = 0;
		while (s0 < p->nslice) {
			int64_t s1 = s0 + 1;
			int64_t base = p->h_cstart[p->h_slices[2 * s0]];
			while (s1 < p->nslice && p->h_cstart[p->h_slices[2 * s1] + p->h_slices[2 * s1 + 1]] - base <= cap) s1++;
			int64_t np = p->h_cstart[p->h_slices[2 * (s1 - 1)] + p->h_slices[2 * (s1 - 1) + 1]] - base;
			if (np > most) most = np;
			p->h_chunk[nch++] = s0;
			s0 = s1;
		}
		size_t need = (size_t)most * sxsk_fused_part_floats(p->L, p->Q);
		if (need > p->part_cap) {
			pfree(p, p->d_part);
			p->d_part = NULL;
			SXS_CU(cudaMallocAsync((void **)&p->d_part, sizeof(float) * need, s));
			p->part_cap = need;
		}
	} else {
		/* translated table in chunks of whole slices that fit the budget */
		size_t per_combo = (size_t)p->NP * 3 * SXS_QT * p->NT * p->celem;
		int64_t chunk = (int64_t)(p->r_budget / (per_combo * SXS_SLICE));   /* slices per chunk */
		if (chunk < 1) chunk = 1;
		if (chunk > p->nslice) chunk = p->nslice;
		for (int64_t s0 = 0; s0 < p->nslice; s0 += chunk) p->h_chunk[nch++] = s0;
		int64_t rcap = chunk * SXS_SLICE;
		if (rcap > p->ncombo) rcap = p->ncombo;
		if (rcap > 0 && p->R_combos < rcap) {
			pfree(p, p->d_R);
			p->d_R = NULL;
			SXS_CU(cudaMallocAsync(&p->d_R, per_combo * rcap, s));
			p->R_combos = rcap;
		}
	}
	p->h_chunk[nch] = p->nslice;
	if (nch > INT32_MAX / 3) return sxs_fail(-2, "sxsg_plan_run: too many chunks");
	if ((rc = plan_events(p, (int)(3 * nch)))) return rc;
	if (fit_mode == SXSG_FIT_LBFGSB && !p->d_scaled && p->npose > 0)
		SXS_CU(cudaMallocAsync((void **)&p->d_scaled, sizeof(double) * (size_t)p->npose * 6 * p->Q, s));
	p->run_nch = nch;
	p->last_chunks = (int)(nch < INT32_MAX ? nch : INT32_MAX);
	return 0;
}

/* The launches of a prepared run on the plan's stream (its side stream
 * forks from and joins it): tables, the chunks of translation and per-pose
 * contraction, and the fit unless fit_mode is SXSG_FIT_NONE.  timed: record
 * the stage events that sxsg_plan_timings reads. */
int sxs_plan_enqueue(sxsg_plan *p, int fit_mode, int timed)
{
	int rc;
	cudaStream_t s = p->s;
	int Q = p->Q, L = p->L;
	int64_t nch = p->run_nch;
	if (timed) SXS_CU(cudaEventRecord(p->ev[0], s));
	if ((rc = plan_tables(p))) return rc;
	if (timed) SXS_CU(cudaEventRecord(p->ev[1], s));
	const void *tau = p->fp32 ? (const void *)p->d_tauf : (const void *)p->d_tau;
	for (int64_t k = 0; k < nch; k++) {
		int64_t s0 = p->h_chunk[k], s1 = p->h_chunk[k + 1];
		int64_t c0 = p->h_slices[2 * s0], c1 = p->h_slices[2 * (s1 - 1)] + p->h_slices[2 * (s1 - 1) + 1];
		int64_t p0 = p->h_cstart[c0], p1 = p->h_cstart[c1];
		cudaEvent_t *e = p->cev + 3 * k;
		if (timed) SXS_CU(cudaEventRecord(e[0], s));
		if (p->run_fused) {
			/* translation and per-pose sums in one pass, then the sum over m */
			SXS_K(sxsk_translate_fused(p->d_U, tau, p->d_combo + 3 * c0, p->d_slices + 2 * s0, (int)(s1 - s0),
			                           (int)c0, p->nzt, Q, L, p->tr_slices, p->d_poses, p->d_cstart, (int)p0, p->d_P,
			                           p->d_tw, p->d_part, s));
			if (timed) SXS_CU(cudaEventRecord(e[1], s));
			SXS_K(sxsk_fused_reduce(p->d_poses + p0, (int)(p1 - p0), p->d_part, Q, L, p->d_cstf, p->d_cross, s));
		} else {
			SXS_K(sxsk_translate(p->d_U, tau, p->d_combo + 3 * c0, p->d_slices + 2 * s0, (int)(s1 - s0), (int)c0,
			                     (int)(c1 - c0), p->nzt, Q, L, p->d_R, p->fp32, p->tr_slices, s));
			if (timed) SXS_CU(cudaEventRecord(e[1], s));
			SXS_K(sxsk_pose_cross(p->d_poses + p0, (int)(p1 - p0), (int)c0, (int)(c1 - c0), p->d_P, p->d_R, p->d_tw,
			                      p->fp32 ? (const void *)p->d_cstf : (const void *)p->d_cst, Q, L,
			                      p->d_cross, p->fp32, s));
		}
		if (timed) SXS_CU(cudaEventRecord(e[2], s));
		sxs_count_launches(sxsk_translate_launches(L) + 1);
	}
	if (timed) SXS_CU(cudaEventRecord(p->ev[5], s));
	int n = (int)p->npose;
	if (fit_mode == SXSG_FIT_GRID) {
		SXS_K(plan_fit_grid(p, n, p->d_chi, p->d_c1, p->d_c2, p->d_cell, NULL, s));
		sxs_count_launches(n > 0 ? 1 : 0);
	} else if (fit_mode == SXSG_FIT_LBFGSB) {
		SXS_K(sxs_fit_lbfgsb_launch(p->d_cross, p->fp32, p->d_scaled, n, Q, p->d_q, p->d_a, p->mult, p->peak, 1, p->d_chi,
		                            p->d_c1, p->d_c2, p->d_scale, p->d_iters, s));
		sxs_count_launches(n > 0 ? 2 : 0);
		if (n > 0) SXS_CU(cudaMemsetAsync(p->d_cell, 0xff, sizeof(int32_t) * n, s));
	}
	p->last_fit = fit_mode;
	p->grid_valid = 0;
	return 0;
}

int sxsg_plan_run(sxsg_plan *p, int fit_mode)
{
	if (!p) return sxs_fail(-2, "sxsg_plan_run: null plan");
	int rc = sxs_plan_prepare(p, fit_mode);
	if (!rc) rc = sxs_plan_enqueue(p, fit_mode, 1);
	if (rc) return rc;
	cudaStream_t s = p->s;
	int64_t nch = p->run_nch;
	cudaEvent_t end;
	SXS_CU(cudaEventCreate(&end));
	SXS_CU(cudaEventRecord(end, s));
	SXS_CU(cudaEventSynchronize(end));
	float t_tab = 0, t_fit = 0, t_all = 0;
	double t_tr = 0, t_pc = 0;
	cudaEventElapsedTime(&t_tab, p->ev[0], p->ev[1]);
	cudaEventElapsedTime(&t_all, p->ev[0], end);
	for (int64_t k = 0; k < nch; k++) {
		cudaEvent_t *e = p->cev + 3 * k;
		float a = 0, b = 0;
		cudaEventElapsedTime(&a, e[0], e[1]);
		cudaEventElapsedTime(&b, e[1], e[2]);
		t_tr += a;
		t_pc += b;
	}
	cudaEventElapsedTime(&t_fit, p->ev[5], end);
	cudaEventDestroy(end);
	p->ms[0] = t_tab; p->ms[1] = t_tr; p->ms[2] = t_pc; p->ms[3] = t_fit; p->ms[4] = t_all;
	if (p->tc_used) {
		int st = 0;
		SXS_CU(cudaMemcpyAsync(&st, p->d_tcstat, sizeof(int), cudaMemcpyDeviceToHost, s));
		SXS_CU(cudaStreamSynchronize(s));
		if (st == 1)
			return sxs_fail(-6, "sxsg_plan_run: the tensor-core rotation did not complete (MMA wait gave up)");
		if (st)
			return sxs_fail(-7, "sxsg_plan_run: the tensor-core rotation's MMAs did not finish; the CUDA context "
			                    "is unusable");
	}
	return 0;
}

int sxsg_plan_results(sxsg_plan *p, double *chi, double *c1, double *c2, int32_t *cell, double *cross, double *grid)
{
	if (!p) return sxs_fail(-2, "sxsg_plan_results: null plan");
	size_t n = (size_t)p->npose;
	cudaStream_t s = p->s;
	if (n == 0) return 0;
	if (chi) SXS_CU(cudaMemcpyAsync(chi, p->d_chi, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
	if (c1) SXS_CU(cudaMemcpyAsync(c1, p->d_c1, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
	if (c2) SXS_CU(cudaMemcpyAsync(c2, p->d_c2, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
	if (cell) SXS_CU(cudaMemcpyAsync(cell, p->d_cell, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
	if (cross) {
		/* the mixed path keeps double-float pairs: same size, widened here */
		SXS_CU(cudaMemcpyAsync(cross, p->d_cross, sizeof(double) * n * 6 * p->Q, cudaMemcpyDeviceToHost, s));
		if (p->fp32) {
			SXS_CU(cudaStreamSynchronize(s));
			size_t m = n * 6 * (size_t)p->Q;
			for (size_t i = 0; i < m; i++) {
				float v[2];
				memcpy(v, cross + i, sizeof(v));
				cross[i] = (double)v[0] + (double)v[1];
			}
		}
	}
	if (grid) {
		if (p->n1 <= 0 || p->n2 <= 0) return sxs_fail(-2, "no fit grid in this plan");
		size_t gn = n * p->n1 * p->n2;
		double *d_g = NULL;
		SXS_CU(cudaMallocAsync((void **)&d_g, sizeof(double) * gn, p->s));
		double *tc = NULL, *t1 = NULL, *t2 = NULL;
		int32_t *tcell = NULL;
		cudaError_t e = cudaMallocAsync((void **)&tc, sizeof(double) * n, p->s);
		if (!e) e = cudaMallocAsync((void **)&t1, sizeof(double) * n, p->s);
		if (!e) e = cudaMallocAsync((void **)&t2, sizeof(double) * n, p->s);
		if (!e) e = cudaMallocAsync((void **)&tcell, sizeof(int32_t) * n, p->s);
		if (!e) {
			e = (cudaError_t)plan_fit_grid(p, (int)n, tc, t1, t2, tcell, d_g, s);
			sxs_count_launches(1);
		}
		if (!e) e = cudaMemcpyAsync(grid, d_g, sizeof(double) * gn, cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaStreamSynchronize(s);
		pfree(p, d_g); pfree(p, tc); pfree(p, t1); pfree(p, t2); pfree(p, tcell);
		if (e) return sxs_cuda_fail(e, "grid results");
	}
	SXS_CU(cudaStreamSynchronize(s));
	return 0;
}

int sxsg_plan_topk(sxsg_plan *p, int k, int64_t *pose, double *chi, double *c1, double *c2)
{
	if (!p || k < 0) return sxs_fail(-2, "sxsg_plan_topk: bad arguments");
	if (p->last_fit != SXSG_FIT_GRID && p->last_fit != SXSG_FIT_LBFGSB)
		return sxs_fail(-2, "sxsg_plan_topk: no fitted run");
	int64_t n = p->npose;
	if (k > n) k = (int)n;
	if (k == 0) return 0;
	if (k > SXSK_TOPK_MAX) return sxs_fail(-2, "sxsg_plan_topk: k above %d", SXSK_TOPK_MAX);
	cudaStream_t s = p->s;
	void *ws = NULL;
	int64_t *d_pos = NULL;
	double *d_out = NULL;
	cudaError_t e = cudaMallocAsync(&ws, sxsk_topk_scratch((long)n, k), s);
	if (!e) e = cudaMallocAsync((void **)&d_pos, sizeof(int64_t) * k, s);
	if (!e) e = cudaMallocAsync((void **)&d_out, sizeof(double) * 3 * (size_t)k, s);
	if (!e) {
		e = (cudaError_t)sxsk_topk(p->d_chi, p->d_c1, p->d_c2, (long)n, k, ws, d_pos, d_out, c1 ? d_out + k : NULL,
		                           c2 ? d_out + 2 * (size_t)k : NULL, s);
		sxs_count_launches(sxsk_topk_launches());
	}
	if (!e && pose) e = cudaMemcpyAsync(pose, d_pos, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, s);
	if (!e && chi) e = cudaMemcpyAsync(chi, d_out, sizeof(double) * k, cudaMemcpyDeviceToHost, s);
	if (!e && c1) e = cudaMemcpyAsync(c1, d_out + k, sizeof(double) * k, cudaMemcpyDeviceToHost, s);
	if (!e && c2) e = cudaMemcpyAsync(c2, d_out + 2 * (size_t)k, sizeof(double) * k, cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaStreamSynchronize(s);
	pfree(p, ws);
	pfree(p, d_pos);
	pfree(p, d_out);
	if (e) return sxs_cuda_fail(e, "sxsg_plan_topk");
	return k;
}

int sxsg_plan_chunks(const sxsg_plan *p) { return p ? p->last_chunks : 0; }

int sxsg_plan_timings(sxsg_plan *p, double *ms5)
{
	if (!p || !ms5) return sxs_fail(-2, "sxsg_plan_timings: bad arguments");
	for (int i = 0; i < 5; i++) ms5[i] = p->ms[i];
	return 0;
}

int sxsg_score_flat(const double *A, const double *B, const double *q, int Q, const double *z, int nz, int L,
                    const int64_t *index, int64_t n, int skip, const double *a, double mult, double peak, int fit_mode,
                    const double *c1g, int n1, const double *c2g, int n2, double *chi, double *c1, double *c2,
                    double *cross, int precision)
{
	sxsg_plan *p = NULL;
	int rc = sxsg_plan_create(&p, A, B, q, Q, z, nz, L, a, mult, peak, c1g, n1, c2g, n2, precision);
	if (!rc) rc = sxsg_plan_set_poses(p, index, n, skip);
	if (!rc) rc = sxsg_plan_run(p, fit_mode);
	if (!rc) rc = sxsg_plan_results(p, chi, c1, c2, NULL, cross, NULL);
	sxsg_plan_destroy(p);
	return rc;
}

/* Caller-owned rotation tables for a plan created with ext_tables (the
 * serving cache): P and U of sxs_plan_table_bytes each, zero-filled by the
 * owner; *_valid says whether they already hold this plan's rows (same
 * molecule, L, q grid, twiddle variant and precision). */
void sxs_plan_set_tables(sxsg_plan *p, void *P, int P_valid, void *U, int U_valid)
{
	p->d_P = P;
	p->d_U = U;
	p->P_valid = P_valid;
	p->U_valid = U_valid;
}

size_t sxs_plan_table_bytes(int L, int Q, int precision)
{
	size_t K = L + 1, N = 2 * L + 1, NP = K * (K + 1) / 2, NT = (Q + SXS_QT - 1) / SXS_QT;
	return NT * K * N * NP * 3 * SXS_QT * (precision == SXSG_MIXED ? 2 * sizeof(float) : 2 * sizeof(double));
}

/* Device bytes of a plan besides its rotation tables and translated-table
 * chunk: molecules, per-z tables for nzt touched z, pose lists and outputs. */
size_t sxs_plan_base_bytes(int L, int Q, int nzt, int64_t npose, int n1, int precision, int fit_mode)
{
	size_t K = L + 1, N = 2 * L + 1, NT = (Q + SXS_QT - 1) / SXS_QT, K2 = K * K;
	size_t celem = precision == SXSG_MIXED ? 8 : 16;
	size_t spf = (size_t)3 * Q * K2;
	size_t b = spf * (16 * 2 + celem * 2);                       /* A, B, At, Bt */
	b += (size_t)nzt * Q * N * 8;                                /* Bessel */
	b += NT * nzt * K * K * K * SXS_QT * (precision == SXSG_MIXED ? 12 : 8); /* tau */
	b += (size_t)npose * (sizeof(sxsk_pose) + 6 * Q * 8 + 40);   /* poses, cross, outputs */
	if (fit_mode == SXSG_FIT_LBFGSB) b += (size_t)npose * 6 * Q * 8; /* its rescaled copy */
	b += (size_t)n1 * Q * 16 + (size_t)64 * Q + (1 << 20);
	return b;
}

/* bytes of one combo of the translated table */
size_t sxs_plan_combo_bytes(int L, int Q, int precision)
{
	size_t K = L + 1, NP = K * (K + 1) / 2, NT = (Q + SXS_QT - 1) / SXS_QT;
	return NP * 3 * SXS_QT * NT * (precision == SXSG_MIXED ? 8 : 16);
}

/* ------------------------------------------------------------ timing */
static cudaEvent_t g_t0, g_t1;
static int g_tinit = 0;

int sxsg_timer_start(void)
{
	int rc = sxs_ensure_init();
	if (rc) return rc;
	if (!g_tinit) {
		SXS_CU(cudaEventCreate(&g_t0));
		SXS_CU(cudaEventCreate(&g_t1));
		g_tinit = 1;
	}
	SXS_CU(cudaEventRecord(g_t0, g_stream));
	return 0;
}

double sxsg_timer_stop(void)
{
	if (!g_tinit) return -1.0;
	if (cudaEventRecord(g_t1, g_stream) != cudaSuccess) return -1.0;
	if (cudaEventSynchronize(g_t1) != cudaSuccess) return -1.0;
	float ms = 0;
	cudaEventElapsedTime(&ms, g_t0, g_t1);
	return ms;
}

double sxsg_fp32_fma_tflops(void)
{
	if (sxs_ensure_init()) return -1.0;
	extern double sxsk_fp32_probe(cudaStream_t s);
	sxs_count_launches(2);
	return sxsk_fp32_probe(g_stream);
}

double sxsg_l2_read_gbs(void)
{
	if (sxs_ensure_init()) return -1.0;
	extern double sxsk_l2_probe(cudaStream_t s);
	sxs_count_launches(2);
	return sxsk_l2_probe(g_stream);
}

double sxsg_fp64_fma_tflops(void)
{
	if (sxs_ensure_init()) return -1.0;
	extern double sxsk_fp64_probe(cudaStream_t s);
	sxs_count_launches(2);
	return sxsk_fp64_probe(g_stream);
}
