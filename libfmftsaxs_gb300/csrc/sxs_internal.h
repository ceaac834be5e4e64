/*
 * Internal declarations shared by the host C files of fmftsaxs-gb300.
 */
#ifndef SXS_INTERNAL_H
#define SXS_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "fmftsaxs_gb300.h"
#include "kernels.h"

/* The reference is compiled with -std=c11, where <math.h> does not define
 * M_PI, so src/define.h:14-16's fallback value is the pi of every formula on
 * the path; the FFTW branch (exact DFT) uses the full-precision value. */
#define SXS_PI 3.14159265358
#define SXS_PI_FULL 3.14159265358979323846
#define SXS_REL_ERR 0.05   /* src/define.h:21 */
#define SXS_C1_LOWER 0.96  /* src/define.h:28-34 */
#define SXS_C1_UPPER 1.04
#define SXS_C2_LOWER -2.00
#define SXS_C2_UPPER 4.00
#define SXS_C1_DEFAULT 1.0
#define SXS_C2_DEFAULT 0.0
#define SXS_LMAX 60
#define SXS_FF_NTYPES 43   /* HEAVY_ATOM_SIZE, src/form_factor_table.h:35 */

/* error state (thread-local message) */
int sxs_fail(int code, const char *fmt, ...);
int sxs_cuda_fail(cudaError_t e, const char *what);
#define SXS_CU(call)                                                      \
	do {                                                                  \
		cudaError_t e_ = (call);                                          \
		if (e_ != cudaSuccess) return sxs_cuda_fail(e_, #call);           \
	} while (0)
#define SXS_K(call)                                                       \
	do {                                                                  \
		int e_ = (call);                                                  \
		if (e_ != 0) return sxs_cuda_fail((cudaError_t)e_, #call);        \
	} while (0)
/* abort the process like the reference's ERROR_MSG (src/common.h:26-30) */
void sxs_die(const char *func, const char *msg);

int sxs_ensure_init(void);
cudaStream_t sxs_default_stream(void);
void sxs_count_launches(int n);

/* host tables (sxs_tables.c) */
double sxs_sbessel_host(int l, double x);
void sxs_wigner_d_host(int L, double beta, double *d);   /* [K][N][N] */
void sxs_ynorm_host(int L, double *y);                    /* [K][N] (l, m+L) */
void sxs_twiddles_host(int N, int exact, double *tw2);   /* [N][2] */
const double *sxs_dsymb_cached(int L);                    /* [K2][K][N], built once per L */

/* per-L device tables, cached for the process */
typedef struct {
	int L;
	double *d_dtab;   /* [K][K][N][N] */
	float *d_dtabf;   /* the same in float (mixed-path rotation) */
	double *d_dsymb;  /* [K2][K][N] */
	double *d_ynorm;  /* [K][N] */
	int2 *d_ll1;      /* (l, l1 >= l) pairs */
	int nll1;
} sxs_ltables;
int sxs_ltables_get(int L, const sxs_ltables **out);

/* plans for the serving loop: on a caller stream (NULL = the library's),
 * with caller-owned rotation tables when ext_tables != 0 */
int sxs_plan_create_on(sxsg_plan **out, const double *A, const double *B, const double *q, int Q, const double *z,
                       int nz, int L, const double *a, double mult, double peak, const double *c1g, int n1,
                       const double *c2g, int n2, int precision, cudaStream_t stream, int ext_tables);
void sxs_plan_set_tables(sxsg_plan *p, void *P, int P_valid, void *U, int U_valid);
size_t sxs_plan_table_bytes(int L, int Q, int precision);
size_t sxs_plan_base_bytes(int L, int Q, int nzt, int64_t npose, int n1, int precision, int fit_mode);
size_t sxs_plan_combo_bytes(int L, int Q, int precision);

/* What a batch of plans (sxs_batch.c) reads of one plan: its sizes, the
 * device tables its kernels use and its outputs. */
typedef struct {
	int L, Q, NT, NP, n1, n2, fp32, ext_tables, nzt, ncombo, nslice, tr_slices, rot_gamma;
	int fused;                      /* the plan's runs fuse translation and per-pose contraction */
	const int32_t *cstart;          /* device first sorted pose of each combo */
	int64_t npose;
	const void *At, *Bt;            /* transposed coefficients */
	const float *dtabf;             /* float Wigner-d table of L */
	const double2 *tw;              /* twiddles (uploaded) */
	void *P, *U;                    /* rotation tables */
	const float *tauf;              /* float per-z translation tables */
	const int32_t *combo, *slices;  /* device combos [ncombo][3], slices [nslice][2] */
	const int32_t *h_slices;        /* host copy of the slices */
	const int64_t *h_cstart;        /* first sorted pose of each combo [ncombo + 1] */
	const sxsk_pose *poses;         /* sorted by combo */
	const void *cst;                /* double-float self terms */
	void *cross;                    /* double-float cross terms [npose][6][Q] */
	const double *fc, *c1g, *c2g;
	const float2 *gdf;
	double a0sum, peak;
	double *chi, *c1, *c2;
	int32_t *cell;
} sxs_plan_view;
/* the next run of the plan fuses the translation with the per-pose
 * contraction (mode and pose density) */
int sxs_plan_uses_fused(const sxsg_plan *p);
/* fills v after uploading the twiddles of the plan's pose list (waits for
 * the plan's stream) */
int sxs_plan_batch_view(sxsg_plan *p, sxs_plan_view *v);
/* the per-z tables of the plan's touched z on stream s */
int sxs_plan_ztables_on(sxsg_plan *p, cudaStream_t s);
/* a batch filled the plan's outputs with this fit */
void sxs_plan_mark_run(sxsg_plan *p, int fit_mode, const float *ms);

/* first-fit packing of the batch's chunks into arena phases (sxs_batch.c) */
int sxs_pack_first_fit(const size_t *bytes, size_t n, size_t cap, int *phase, size_t *off, size_t *used);

/* per-q constants of the grid fit: fc[Q][5] */
void sxs_fit_constants(const double *q, const double *a, int Q, double *fc);

/* device L-BFGS-B over (c1, c2) for a batch of poses: cross [n][6][Q]
 * (rescaled here by peak when rescale != 0), ct a workspace of n*6*Q
 * doubles; two kernel launches */
/* cross: double, or double-float pairs {hi, lo} when cross_df (the mixed
 * path's per-pose terms) */
int sxs_fit_lbfgsb_launch(const void *cross, int cross_df, double *ct, int npose, int Q, const double *q,
                          const double *a, double mult, double peak, int rescale, double *chi, double *c1, double *c2,
                          double *scale, int *nevals, cudaStream_t s);

#endif
