/*
 * C-ABI launchers for the sm_103a kernels of the FFT-correlation scoring path.
 * Host C (sxs_host.c) calls these; every pointer is a device pointer unless
 * named h_*.  All launches go to the given stream; none synchronises.
 *
 * Device layouts (K = L+1, N = 2L+1, K2 = K*K, NP = K(K+1)/2, NT = ceil(Q/QT)
 * q tiles of QT = SXS_QT; a table of precision S holds complex values as {re, im}
 * pairs of S, S = double on the plain path and float on the mixed path):
 *   spf_t [3 ch][K2 lm][Q]                     lm = l(l+1)+m, q fastest (S)
 *   dtab  [K b][K l][N m+L][N m1+L]            Wigner small-d per beta_b = b*pi/L
 *   dsymb [K2 lm][K l1][N p]
 *   bes   [nz][N p][Q]
 *   tau   [NT][nz][K m][K l][K l1][QT]         T^m_{l l1} = i^{l+l1} tau (real)
 *   rot   [NT][K*N (b,g)][NP pair][3 ch][QT]   pair = (m >= 0, l >= m), m-major (S)
 *   trans [NT][ncombo][NP pair][3 ch][QT]      (S)
 *   cross [npose][6][Q]                        (double)
 * Entries of the q tiles past Q are padding: never written by the kernels
 * that fill a table and never read into a result.
 */
#ifndef SXS_KERNELS_H
#define SXS_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

/* q values per tile of the contraction tables; kernels move 2 adjacent q
 * per thread, SXS_QT / 2 threads per tile row */
#define SXS_QT 8
#define SXS_QP (SXS_QT / 2)
/* combos per translation slice (a run of combos sharing z): one block of
 * the column translation kernel holds SXS_QT q x 3 channels x SXS_SLICE */
#define SXS_SLICE (384 / (3 * SXS_QT))
/* largest L + 1 the plans accept */
#define SXS_LMAX_K 61

#ifdef __cplusplus
extern "C" {
#endif

/* Decoded pose: grid cell of one listed pose. */
typedef struct {
	int32_t zi, b1, b2, a2, g1, g2;
	int32_t combo;   /* index of (zi, b2, g2) in the translated-table list */
	int32_t src;     /* position in the caller's list */
} sxsk_pose;

/* A_lm expansion (FP64, the reference's j_l series and Legendre recurrence):
 * per-atom Y_lm and radius into ylm_ws / rad_ws, then one block per (q, l)
 * with the atoms staged through shared memory (series, accumulation, 4 pi
 * i^l phase).  spf_out uses the host flat layout [3][Q][K2][2]. */
int sxsk_expand(const double *xyz, const double *vac, const double *dum, const double *wfac,
                int natoms, const double *q, int Q, int L, const double *ynorm,
                double2 *ylm_ws, double *rad_ws, double *spf_out, cudaStream_t s);
size_t sxsk_expand_ws_ylm(int natoms, int L);
size_t sxsk_expand_ws_rad(int natoms);
int sxsk_expand_launches(void);

/* host-flat [3][Q][K2][2] -> spf_t [3][K2][Q] complex, in float when fp32 */
int sxsk_spf_transpose(const double *flat, void *spf_t, int Q, int L, int fp32, cudaStream_t s);

/* cross terms of single molecules: spf [nmol][3][Q][K2][2] (host flat
 * layout) -> cross [nmol][6][Q] */
int sxsk_self_cross(const double *spf, int nmol, int Q, int L, double *cross, cudaStream_t s);

/* Shrake-Rupley accessible fraction per atom: sphere points sph[npts][3]
 * (npts <= 1024) */
int sxsk_sasa(const double *xyz, const double *rad, int n, double probe, const double *sph, int npts, double *frac,
              cudaStream_t s);

/* j_p(q z) for p in [0,2L]: bes[nz][N][Q] (faithful series) */
int sxsk_bessel_z(const double *z, int nz, const double *q, int Q, int L, double *bes, cudaStream_t s);

/* translation matrix T^m_{l l1}(q z) = i^{l+l1} tau -> tau; ll1 lists the
 * (l, l1 >= l) pairs */
int sxsk_tmatrix(const double *bes, const double *dsymb, int nz, int Q, int L, const int2 *ll1, int nll1,
                 double *tau, cudaStream_t s);

/* b[i] = (float)a[i] */
int sxsk_to_float(const double *a, float *b, long n, cudaStream_t s);

/* self terms cst[6][Q] (already times {1,2,2,1,2,1}); A, B in the host flat layout */
int sxsk_const_int(const double *A, const double *B, int Q, int L, double *cst, cudaStream_t s);

/* rotation table, m >= 0: out[(b,g)][pair][ch][q] = sum_{m1} tw[(m1' g) mod N] d^l_{m m1}(beta_b) C[ch][l,m1][q]
 * with C = spf_t, conjugated when conj != 0. */
int sxsk_rotate(const void *spf_t, const void *dtab, const double2 *tw, int Q, int L, int conj, void *out,
                int fp32, int gsel, cudaStream_t s);   /* dtab in float when fp32; gsel: gamma pairs per
                                                       * thread (0 = the fewest that cover L + 1) */

/* The mixed path's rotation table on the tcgen05 tensor cores (3xTF32,
 * FP32 accumulation in tensor memory); same output as sxsk_rotate with
 * fp32; 2L + 1 <= 64.  dtabf: the float Wigner-d table. */
int sxsk_rotate_tc(const void *spf_t, const float *dtabf, const double2 *tw, int Q, int L, int conj, void *out,
                   float *amat, int *status, cudaStream_t s);
/* floats of the scratch (amat) that sxsk_rotate_tc needs */
size_t sxsk_rotate_tc_scratch(int L);
/* *status (device int, zeroed by the caller) after sxsk_rotate_tc: the
 * largest of 0 (every block saw its MMAs finish), 1 (a block gave up
 * waiting, its MMAs then finished: output invalid) and 2 (a block's MMAs
 * did not finish in either bounded wait: output invalid, its tensor memory
 * was not freed and the context must be considered unusable). */

/* Pose list on the device (src/index.c:3-29 packing, most significant
 * first: z slot, beta1, beta2, alpha2, gamma1, gamma2).  decode: one thread
 * per pose writes the decoded pose and its combo key (zi nb + b2) N + g2,
 * counts keys and touched z slots, and records in err[0] / err[1] the
 * smallest pose index with a negative index / a z slot >= nz (err preset to
 * all ones).  scatter: places pose i at pos[key]++ with its combo id. */
int sxsk_pose_decode(const int64_t *index, int64_t n, int N, int nb, int nz, sxsk_pose *tmp, int32_t *key,
                     int32_t *cnt, int32_t *zused, unsigned long long *err, cudaStream_t s);
int sxsk_pose_scatter(const sxsk_pose *tmp, const int32_t *key, int64_t n, int32_t *pos, const int32_t *cid,
                      sxsk_pose *out, cudaStream_t s);
/* gamma pairs per thread of the rotation for L and a tile choice gsel
 * (0 = the fewest that cover L + 1): 2, 4, 6, 8, 12 or 16; 0 if none */
int sxsk_rotate_group(int L, int gsel);
/* slices per block of the pipelined FP32 translation when a plan sets none */
#define SXSK_TP_SB 8
/* the launch of sxsk_translate (FP32) for column class NB alone (the m with
 * L + 1 - m in (NB - 4, NB]); nothing when the class has no m for L */
int sxsk_translate_class(const void *U, const void *tau, const int32_t *combo_zbg, const int32_t *slices, int nslice,
                         int cbase, int ncombo, int nzt, int Q, int L, void *R, int sb, int NB, cudaStream_t s);
/* kernel launches one sxsk_translate call makes for this L */
int sxsk_translate_launches(int L);
/* translated ligand table for the combos of a run of slices, m >= 0, all q tiles:
 * R[t][c][pair(m,l)][ch][q] = sum_{l1>=m} conj(T[t][zi][m][l][l1][q]) U[t][(b2,g2)][pair(m,l1)][ch][q].
 * combo_zbg = the combos of the chunk (cbase = the first one's index),
 * slices[nslice][2] = {first combo, count} runs of <= 16 combos sharing z;
 * R holds ncombo combos; tau is float when fp32; nzt = z count of tau */
int sxsk_translate(const void *U, const void *tau, const int32_t *combo_zbg, const int32_t *slices, int nslice,
                   int cbase, int ncombo, int nzt, int Q, int L, void *R, int fp32, int sb, cudaStream_t s);
/* sb: slices per block of the pipelined FP32 kernel (0 = 8) */

/* per-pose raw cross terms: cross[p][c][q] = cst[c][q] + 2 Re sum_m tw(m' a2) sum_l P R,
 * the m < 0 half folded in by symmetry; R holds the ncombo combos from combo_base.
 * FP64 path: cst and cross are double.  FP32 path: cst and cross are
 * double-float pairs {hi, lo} (float2), so that neither this kernel nor the
 * fit that reads the terms touches the FP64 pipe. */
int sxsk_pose_cross(const sxsk_pose *poses, int npose, int combo_base, int ncombo, const void *P, const void *R,
                    const double2 *tw, const void *cst, int Q, int L, void *cross, int fp32, cudaStream_t s);
/* The mixed path's translation fused with the per-pose contraction, for
 * sparse pose lists (few poses per translated row): the translated rows of
 * the chunk's combos are never stored; per pose and m the six channel sums
 * go to part[pose - pose_base][m][6][NT 8] (sxsk_fused_part_floats floats
 * per pose), and sxsk_fused_reduce adds them over m (ascending) into the
 * double-float cross terms.  poses: the plan's sorted poses; cstart[c]: the
 * first sorted pose of global combo c; L + 1 <= 32. */
size_t sxsk_fused_part_floats(int L, int Q);
int sxsk_translate_fused(const void *U, const void *tau, const int32_t *combo_zbg, const int32_t *slices, int nslice,
                         int cbase, int nzt, int Q, int L, int sb, const sxsk_pose *poses, const int32_t *cstart,
                         int pose_base, const void *P, const double2 *tw, float *part, cudaStream_t s);
/* sxsk_translate_fused for column class NB alone */
int sxsk_translate_fused_class(const void *U, const void *tau, const int32_t *combo_zbg, const int32_t *slices,
                               int nslice, int cbase, int nzt, int Q, int L, int sb, const sxsk_pose *poses,
                               const int32_t *cstart, int pose_base, const void *P, const double2 *tw, float *part,
                               int NB, cudaStream_t s);
/* cross of the npose poses from `poses` (their part rows from 0) */
int sxsk_fused_reduce(const sxsk_pose *poses, int npose, const float *part, int Q, int L, const void *cst,
                      void *cross, cudaStream_t s);
/* double -> double-float pairs {hi, lo} */
int sxsk_to_df(const double *a, float2 *b, long n, cudaStream_t s);
/* double-float pairs -> double (hi + lo), in place allowed */
int sxsk_df_to_double(const float2 *a, double *b, long n, cudaStream_t s);

/* grid fit: per pose, peak rescale then chi^2 at every (c1, c2) cell; best cell.
 * Scores the poses at slots [slot0, slot0 + nslot) of order (order[i].src
 * indexes cross and every output; the slot itself when order is NULL).
 * gtab[n1][Q] = c1^3 exp(-mult (c1^2-1) q^2); fc[Q][5] per-q constants of the
 * binned experiment (sxs_fit_constants); a0sum = sum_i a[6i]; at most
 * max_blocks resident blocks (persistent loop; <= 0: one block per group). */
int sxsk_fit_grid(const double *cross, const sxsk_pose *order, int slot0, int nslot, int Q, const double *fc,
                  double a0sum, double peak, const double *gtab, const double *c1g, int n1, const double *c2g, int n2,
                  int max_blocks, double *chi, double *c1, double *c2, int32_t *cell, double *grid, cudaStream_t s);

/* the grid fit of the mixed path in double-float arithmetic (FP32 pipe);
 * same arguments as sxsk_fit_grid, with the cross terms as double-float
 * pairs (sxsk_pose_cross, FP32 path) and gdf[n1][Q] = gtab split into
 * {hi, lo} floats */
int sxsk_fit_grid_df(const float2 *cross, const sxsk_pose *order, int slot0, int nslot, int Q, const double *fc,
                     double a0sum, double peak, const float2 *gdf, const double *c1g, int n1, const double *c2g,
                     int n2, int max_blocks, double *chi, double *c1, double *c2, int32_t *cell, double *grid,
                     cudaStream_t s);

/* device top-k (kernels_topk.cu): the k smallest chi[0, n) in ascending
 * order, ties in list order, NaN last (a stable argsort); 1 <= k <=
 * min(n, SXSK_TOPK_MAX); outputs list positions and the chi, c1, c2 of
 * them (any output may be NULL; c1, c2 are read only for their outputs);
 * scratch: device memory of sxsk_topk_scratch(n, k) bytes */
#define SXSK_TOPK_MAX 16384
size_t sxsk_topk_scratch(long n, int k);
int sxsk_topk_launches(void);
int sxsk_topk(const double *chi, const double *c1, const double *c2, long n, int k, void *scratch, int64_t *out_pos,
              double *out_chi, double *out_c1, double *out_c2, cudaStream_t s);

/* pose ingestion (kernels_ingest.cu): rot[9n] row-major, tr[3n], ref (host
 * pointer, 3 values) -> index[n] (-1 when z is off the grid), keep[n];
 * poses the host must recompute are appended to flagged[] (n slots), their
 * count in *nflag (zeroed by the caller) */
int sxsk_pose_ingest(const double *rot, const double *tr, long n, const double *ref, const double *zvals, int znum,
                     int L, int wrap, long long *index, unsigned char *keep, unsigned int *nflag, long long *flagged,
                     cudaStream_t s);

/* ------------------------------------------------------------------
 * Batched launches of the mixed path (many dimers at once).  With a
 * counter (*ctr, zeroed by the caller) a kernel runs persistently: a grid
 * of (SMs x resident blocks) that take work items from an array in order
 * through the counter (a block takes the next item when it finishes one,
 * so the array is ordered largest first).  With ctr = NULL it runs one
 * block per item, in array order.  An item is one block's work of the
 * single-dimer kernel, on the job its first field names, and runs that
 * kernel's own block code: results equal the single-dimer launches bit
 * for bit.
 */
typedef struct {
	const void *spf_t;      /* transposed coefficients (float) */
	const void *dtab;       /* float Wigner-d table of L */
	const double2 *tw;      /* twiddles [N] */
	void *out;              /* rotation table (float) */
	int Q, L, conj, pad;
} sxsk_rot_job;
/* items {job, q tile, beta b, m}; G = gamma pairs per thread (the
 * single-dimer choice: 2, 4, 6, 8, 12 or 16); every job with N + (G-1) L
 * <= tw_max twiddle pairs */
int sxsk_rotate_batch(const sxsk_rot_job *jobs, const int4 *items, int nitems, int G, int tw_max, int *ctr,
                      cudaStream_t s);

typedef struct {
	const void *U, *tau;              /* ligand rotation table, float tau of the job's z */
	const int32_t *combo_zbg;         /* the chunk's combos (cbase = the first one's index) */
	const int32_t *slices;            /* the chunk's slices */
	void *R;                          /* the chunk's translated table */
	int nslice, cbase, ncombo, L, nzt, sb, Q, pad;
} sxsk_tr_job;
/* items {job, q tile, slice group, m} for the m with L + 1 - m in
 * (NB - 4, NB] (the pipelined FP32 kernel of that NB; L + 1 <= 32) */
int sxsk_translate_batch(const sxsk_tr_job *jobs, const int4 *items, int nitems, int NB, int *ctr, cudaStream_t s);

typedef struct {
	const sxsk_pose *poses;           /* the chunk's poses */
	const void *P, *R;                /* receptor rotation table, the chunk's translated table */
	const double2 *tw;
	const void *cst;                  /* double-float self terms */
	void *cross;                      /* double-float cross terms of the dimer */
	int npose, combo_base, ncombo, Q, L, pad;
} sxsk_pc_job;
/* items {job, q tile, block of 32 poses, 0} */
int sxsk_pose_cross_batch(const sxsk_pc_job *jobs, const int4 *items, int nitems, int *ctr, cudaStream_t s);

typedef struct {
	const void *U, *tau;              /* ligand rotation table, float tau of the job's z */
	const int32_t *combo_zbg;         /* the chunk's combos (cbase = the first one's index) */
	const int32_t *slices;            /* the chunk's slices */
	const sxsk_pose *poses;           /* the plan's sorted poses */
	const int32_t *cstart;            /* first sorted pose of each combo of the plan */
	const void *P;                    /* receptor rotation table */
	const double2 *tw;
	float *part;                      /* the chunk's per-pose sums */
	int nslice, cbase, L, nzt, sb, pose_base, Q, pad;
} sxsk_tf_job;
/* fused translation (sxsk_translate_fused) of many chunks: items {job, q
 * tile, slice group, m} for the m of column class NB */
int sxsk_translate_fused_batch(const sxsk_tf_job *jobs, const int4 *items, int nitems, int NB, int *ctr,
                               cudaStream_t s);

typedef struct {
	const sxsk_pose *poses;           /* the chunk's poses */
	const float *part;                /* their per-pose sums */
	const void *cst;                  /* double-float self terms */
	void *cross;                      /* double-float cross terms of the dimer */
	int npose, Q, L, pad;
} sxsk_fr_job;
/* sxsk_fused_reduce of many chunks: items {job, block of 128 (pose, q), 0, 0} */
int sxsk_fused_reduce_batch(const sxsk_fr_job *jobs, const int4 *items, int nitems, int *ctr, cudaStream_t s);

typedef struct {
	const float2 *cross;
	const sxsk_pose *order;
	const double *fc;
	const float2 *gdf;
	const double *c1g, *c2g;
	double *chi, *c1, *c2;
	int32_t *cell;
	double *grid;
	double a0sum, peak;
	int slot0, nslot, Q, n1, n2, tp, ppb, qc, gsm, pad;
} sxsk_fit_job;
/* the double-float grid fit's block shape for (Q, n1, n2): threads per pose
 * tp, poses per block ppb, q per staged chunk qc, G staged in shared memory
 * gsm, shared bytes; nonzero when no shape fits */
int sxsk_fit_df_shape(int Q, int n1, int n2, int *tp, int *ppb, int *qc, int *gsm, size_t *smem);
/* items {job, group of ppb poses}; smem = the largest shape's bytes */
int sxsk_fit_grid_df_batch(const sxsk_fit_job *jobs, const int2 *items, int nitems, size_t smem, int *ctr,
                           cudaStream_t s);

#ifdef __cplusplus
}
#endif
#endif
