/*
 * fmftsaxs-gb300: GB300 (sm_103a) implementation of libfmftsaxs's
 * FFT-correlation dimer scoring path.
 *
 * Two layers, both plain C ABI (no C++ or torch types):
 *
 *  1. Drop-in: the reference's own functions, names, argument meanings,
 *     struct layouts and error behaviour (print + exit(EXIT_FAILURE)), so a
 *     program written against libfmftsaxs links against this library
 *     instead.  Each declaration cites the reference header line it
 *     replaces (paths relative to the reference project).
 *
 *  2. sxsg_*: status-returning extensions (0 = success, negative = error,
 *     message from sxsg_last_error()) that the reference has no equivalent
 *     for: flat-array inputs, 64-bit pose indices, grid fit over (c1, c2),
 *     cross-term output, reusable device plans.
 *
 * Everything numerical runs on the GPU; the CUDA extension must be present,
 * there is no CPU path for the scoring.
 */
#ifndef FMFTSAXS_GB300_H
#define FMFTSAXS_GB300_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- types */

/* src/pdb2spf.h:30-35: coefficients A_lm for one q, lm = l(l+1)+m. */
struct sxs_spf_sing {
	int L;
	double *re;
	double *im;
};

/* src/pdb2spf.h:41-53: vacuum (V), excluded-volume (D) and hydration (W)
 * coefficients for every q. */
struct sxs_spf_full {
	int L;
	int qnum;
	double rm;
	struct sxs_spf_sing **V;
	struct sxs_spf_sing **D;
	struct sxs_spf_sing **W;
};

/* src/profile.h:23-49 */
struct sxs_profile {
	int qnum;
	double rerr;
	double *in;
	double *err;
	double *qvals;
	double *VV, *VD, *VW, *DD, *DW, *WW;
	double score;
	double scale;
	double c1;
	double c2;
	double b1, g1, a2, b2, g2;
};

/* src/min_saxs.h:32-46 (the L-BFGS-B workspace is kept for layout
 * compatibility; `integer` and `logical` there are `long int`). */
struct sxs_opt_params {
	double rm;
	double mult;
	double peak;
	double *a;
	double wa[43251];
	long iwa[3072];
	double dsave[29];
	long isave[44];
	long lsave[4];
};

/* src/index.h:25-43 */
struct sxs_euler { double z, b1, g1, a2, b2, g2; };
struct sxs_index { int z, b1, g1, a2, b2, g2; };

#ifndef SXS_HAVE_MOL2_TYPES
/* libmol2's 3-vector and 3x3 matrix, as used by src/index.h and
 * src/saxs_utils.h (define SXS_HAVE_MOL2_TYPES when libmol2's headers are
 * already included). */
struct mol_vector3 { double X, Y, Z; };
struct mol_matrix3 { double m11, m12, m13, m21, m22, m23, m31, m32, m33; };
#endif

/* -------------------------------------------------- drop-in: scoring path */

/* src/fftsaxs.h:95-105.  Scores every grid pose in index_list; outputs are
 * caller-allocated, length nout.  Index packing (src/index.c:3-7):
 * ((((z (L+1) + b1)(L+1) + b2)(2L+1) + a2)(2L+1) + g1)(2L+1) + g2.
 * The fit is the reference's L-BFGS-B over (c1, c2), run on the GPU. */
void sxs_compute_saxs_scores(double *scores_list, double *c1_list, double *c2_list,
                             int *index_list, int nout,
                             struct sxs_spf_full *A, struct sxs_spf_full *B,
                             struct sxs_opt_params *params,
                             double *qvals, int qnum, double *zvals, int znum, int L, int skip);

/* ------------------------------------------------ drop-in: containers, I/O */

struct sxs_spf_sing *sxs_spf_sing_create(int L);          /* src/pdb2spf.h:98 */
void sxs_spf_sing_init(struct sxs_spf_sing *s, int L);    /* src/pdb2spf.h:105 */
void sxs_spf_sing_destroy(struct sxs_spf_sing *s);        /* src/pdb2spf.h:111 */
void sxs_spf_sing_free(struct sxs_spf_sing *s);           /* src/pdb2spf.h:117 */
struct sxs_spf_full *sxs_spf_full_create(int L, int qnum);                /* src/pdb2spf.h:125 */
void sxs_spf_full_init(struct sxs_spf_full *s, int L, int qnum);          /* src/pdb2spf.h:133 */
void sxs_spf_full_free(struct sxs_spf_full *s);                           /* src/pdb2spf.h:139 */
void sxs_spf_full_destroy(struct sxs_spf_full *s);                        /* src/pdb2spf.h:145 */
void sxs_spf_full_reset(struct sxs_spf_full *s);                          /* src/pdb2spf.h:151 */
void sxs_spf_full_write(char *path, struct sxs_spf_full *s);              /* src/pdb2spf.h:158 */
struct sxs_spf_full *sxs_spf_full_read(char *path);                       /* src/pdb2spf.h:165 */
struct sxs_spf_full *sxs_spf_full_fread(FILE *f);                         /* src/pdb2spf.h:172 */

struct sxs_profile *sxs_profile_create(double *qvals, int qnum, int cross_terms_flag);        /* src/profile.h:59 */
void sxs_profile_init(struct sxs_profile *p, double *qvals, int qnum, int cross_terms_flag);  /* src/profile.h:69 */
void sxs_profile_alloc_cross_terms(struct sxs_profile *p, int qnum);                         /* src/profile.h:76 */
void sxs_profile_destroy(struct sxs_profile *p);                                             /* src/profile.h:84 */
void sxs_profile_free(struct sxs_profile *p);                                                /* src/profile.h:91 */
void sxs_profile_write(char *path, struct sxs_profile *p);                                   /* src/profile.h:98 */
struct sxs_profile *sxs_profile_read(char *path);                                            /* src/profile.h:104 */
struct sxs_profile *sxs_profile_fread(FILE *f);                                              /* src/profile.h:110 */
void sxs_profile_from_spf(struct sxs_profile *p, struct sxs_spf_full *spf, double c1, double c2); /* src/profile.h:120 */

/* ---------------------------------------------------- drop-in: fitting */

struct sxs_opt_params *sxs_opt_params_create(struct sxs_profile *exp, double *qvals, int qnum, double rm); /* src/min_saxs.h:57 */
void sxs_opt_params_init(struct sxs_opt_params *p, struct sxs_profile *exp, double *qvals, int qnum, double rm); /* :68 */
void sxs_opt_params_destroy(struct sxs_opt_params *p);     /* src/min_saxs.h:75 */
void sxs_opt_params_free(struct sxs_opt_params *p);        /* src/min_saxs.h:81 */
/* src/min_saxs.h:94.  Peak rescale + L-BFGS-B of every masked profile (GPU). */
void sxs_fit_params(struct sxs_profile **profiles, struct sxs_opt_params *params, int *mask, int n);
/* src/min_saxs.h:104.  L-BFGS-B of one profile (GPU). */
void sxs_lbfgs_fitting(struct sxs_profile *profile, struct sxs_opt_params *params);
double *scoring_helper(struct sxs_profile *exp, int qnum, double *qvals);                          /* src/min_saxs.h:114 */
void sxs_compile_intensity(struct sxs_profile *p, double rm, double c1, double c2);                /* src/min_saxs.h:136 */
double sxs_best_scale(struct sxs_profile *p, struct sxs_opt_params *params, double c1, double c2);  /* src/min_saxs.h:148 */
/* src/min_saxs.h:161 declares sxs_point_score; the reference defines it as
 * point_score (src/min_saxs.c:391).  Both names are exported here. */
double sxs_point_score(struct sxs_profile *p, struct sxs_opt_params *params, double c1, double c2);
double point_score(struct sxs_profile *p, struct sxs_opt_params *params, double c1, double c2);
void sxs_spf2cross_terms(struct sxs_profile *p, struct sxs_spf_full *s);                           /* src/min_saxs.h:169 */
void sxs_spf2fitted_profile(struct sxs_profile *p, struct sxs_spf_full *s, struct sxs_opt_params *params); /* :179 */

/* ----------------------------------------------- drop-in: grids, indices */

double *sxs_mkarray(double begin, double end, int qnum);                                        /* src/saxs_utils.h:30 */
void sxs_fill_active_rotation_matrix(struct mol_matrix3 *rm, double alpha, double beta, double gamma); /* :39 */
void sxs_mult_rot_mats(struct mol_matrix3 *c, struct mol_matrix3 *a, struct mol_matrix3 *b);    /* src/saxs_utils.h:44 */
size_t sxs_assemble_index(struct sxs_index *id, int nbeta, int L);                              /* src/index.h:45 */
void sxs_disassemble_index(struct sxs_index *id, size_t index, int nbeta, int L);               /* src/index.h:47 */
void sxs_ft2euler(struct sxs_euler *euler, struct mol_vector3 *tv, struct mol_matrix3 *rm, struct mol_vector3 *ref_lig); /* :59 */
double sxs_sbessel(int order, double x);                                                        /* src/sfbessel.h:19 */

/* ======================================================== extensions */

const char *sxsg_last_error(void);
/* Initialise the library on a CUDA device (called implicitly with device 0). */
int sxsg_init(int device);
/* Number of kernel launches issued by this library since load. */
long long sxsg_launch_count(void);
/* Free and total memory of the library's device (cudaMemGetInfo). */
int sxsg_device_memory(size_t *free_bytes, size_t *total_bytes);

/* Form-factor constants of one type name of the reference's mapping file
 * ("C", "N", "O", "S", "CH2", ...; src/form_factor_table.c:8-49, 76-107):
 * vacuum and excluded-volume zero-angle form factors.  Returns -1 for an
 * unknown name. */
int sxsg_ff_type(const char *name, double *vacuum_ff, double *dummy_ff);
/* zero-angle form factor of water, the hydration-shell weight (s_OH2) */
double sxsg_ff_water(void);
/* Load a (residue, atom) -> type mapping file in the reference's format
 * (prms/pdb_formfactor_mapping_clean.prm) and resolve n atoms (names in
 * 8-byte slots) to (vacuum_ff, dummy_ff).  Returns the number of atoms that
 * had no mapping (their factors are set to NaN), or < 0 on error. */
int sxsg_ff_lookup(const char *mapping_path, const char *res8, const char *atom8, int n,
                   double *vacuum_ff, double *dummy_ff);

/* Zero-angle form factors (zero_ff, vacuum_ff, dummy_ff; any may be NULL)
 * of form-factor type `type`, the index of the reference's enum
 * saxs_ff_type (0 = H ... 41 = s_OH2, 42 = SH; src/form_factor_table.h:27-37,
 * values src/form_factor_table.c:8-49).  Returns 0, or -2 for a type
 * outside [0, 43). */
int sxsg_ff_constants(int type, double *zero_ff, double *vacuum_ff, double *dummy_ff);
/* The mapping-file name of a type ("C", "CH2", "SOD+", ...), NULL for types
 * that no mapping line can select (ff_type_to_string,
 * src/form_factor_table.c:109-136). */
const char *sxsg_ff_name(int type);

/* A (residue, atom) -> form-factor type map read from a mapping file in the
 * reference's format (default_ff_table, src/form_factor_table.c:138-188):
 * '#' and blank lines skipped, "residue atom type" per line, a later line
 * for the same pair replacing an earlier one.  NULL on error
 * (sxsg_last_error). */
typedef struct sxsg_ff_map sxsg_ff_map;
#define SXSG_FF_UNKNOWN 99   /* s_UNK: the line names a type the reference does not know */
sxsg_ff_map *sxsg_ff_map_load(const char *mapping_path);
/* Type of one atom: the names are trimmed as get_ff does (leading blanks
 * skipped, up to the next blank, at most 7 characters); returns the type
 * index, SXSG_FF_UNKNOWN, or -1 when the pair has no mapping line. */
int sxsg_ff_map_type(const sxsg_ff_map *map, const char *residue, const char *atom);
void sxsg_ff_map_free(sxsg_ff_map *map);

/* A_lm(q) of one molecule on the GPU (atom_grp2spf_inplace, src/pdb2spf.c:24-152)
 * from arrays: coordinates xyz[3n] (already centred), per-atom vacuum and
 * excluded-volume form factors, per-atom accessible fraction sasa (NULL:
 * no hydration shell, W = 0), water form factor.  spf_out is the flat
 * layout [3 (V,D,W)][qnum][(L+1)^2][re,im].  rm (mean vdW radius) is not
 * computed here. */
int sxsg_expand(const double *xyz, const double *vacuum_ff, const double *dummy_ff, const double *sasa,
                double water_ff, int natoms, const double *qvals, int qnum, int L, double *spf_out);

/* Binned experiment for the fit from flat arrays: a[6 qnum], mult and peak
 * exactly as sxs_opt_params_create computes them (min_saxs.c:116-124,
 * 353-389; the bin loop stops at the last experimental point). */
int sxsg_bin_experiment(const double *exp_q, const double *exp_i, const double *exp_err, int nexp,
                        const double *qvals, int qnum, double rm, double *a, double *mult, double *peak);

/* sxs_profile_from_spf on a flat expansion (profile.c:186-233): I(q) and
 * err = 0.05 I of a single molecule at (c1, c2). */
int sxsg_profile_from_flat(const double *spf, int L, int qnum, double rm, const double *qvals, double c1, double c2,
                           double *in, double *err);

/* The expansion of sxsg_expand without any device allocation.  It has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory (all their memory comes from a host application's own
 * pool, or they run where a synchronising cudaMalloc is not allowed).
 * Every pointer is a DEVICE pointer the caller owns: xyz[3 natoms],
 * vacuum_ff, dummy_ff, water_w[natoms] (water form factor x accessible
 * fraction per atom; NULL for no hydration shell), qvals[qnum], spf_out in
 * the flat layout [3][qnum][(L+1)^2][2].  Work buffers (the Y_lm norm
 * table, Y_lm and the radius of each atom) live in one static device array
 * of 64 MiB (8 Mi doubles) that every GPU loading this library keeps until
 * exit; a call needs about natoms (2 (L+1)^2 + 2) doubles of it, L <= 40,
 * and a larger request returns -3 without touching the GPU.  Work is queued
 * on `stream` (a cudaStream_t; NULL for the default stream) and the call
 * returns without waiting for it.  The first call on each device looks up
 * the array's device address (cudaGetSymbolAddress), so make that first
 * call before any stream capture; like the library's other per-device
 * state, the address is not looked up again after a cudaDeviceReset.  All
 * calls share the array: calls that overlap on the GPU race with each
 * other.  Returns 0, -2 (bad argument), -3 (too large for the static
 * array), -4 (no current device) or a CUDA error code. */
int sxsg_expand_noalloc(const double *xyz, const double *vacuum_ff, const double *dummy_ff, const double *water_w,
                        int natoms, const double *qvals, int qnum, int L, double *spf_out, void *stream);

/* Flat-array view of an sxs_spf_full ([3][qnum][(L+1)^2][2]). */
int sxsg_spf_to_flat(const struct sxs_spf_full *s, double *flat);
int sxsg_spf_from_flat(struct sxs_spf_full *s, const double *flat);

/* Reusable scoring plan: receptor/ligand coefficients, grids and the
 * experiment stay resident on the device between runs. */
typedef struct sxsg_plan sxsg_plan;

enum { SXSG_FIT_NONE = 0, SXSG_FIT_GRID = 1, SXSG_FIT_LBFGSB = 2 };
/* Precision of the contraction tables.  SXSG_FP64: every stage in FP64,
 * matching the reference to ~1e-10 relative in I(q) and chi.  SXSG_MIXED:
 * the expansion, Bessel, translation-coefficient and fit stages stay FP64;
 * the rotation, translation and per-pose contractions run in FP32 (tables
 * and accumulation) and the cross terms return to FP64 before the self
 * terms are added; chi agrees with the FP64 path to ~1e-6 relative. */
enum { SXSG_FP64 = 0, SXSG_MIXED = 1 };

/* A, B: flat [3][qnum][(L+1)^2][2]; a[6 qnum], mult, peak: the binned
 * experiment of scoring_helper / sxs_opt_params (min_saxs.c:116-124,
 * 353-389); c1grid/c2grid: fit grid (may be NULL with n = 0 when no grid fit
 * is run). */
int sxsg_plan_create(sxsg_plan **plan, const double *A, const double *B, const double *qvals, int qnum,
                     const double *zvals, int znum, int L, const double *a, double mult, double peak,
                     const double *c1grid, int n1, const double *c2grid, int n2, int precision);
/* Pose list (64-bit packed indices as above).  skip = 1 scores the listed
 * poses the way the reference's skip = 1 does (simple_ft twiddles);
 * skip = 0 as its FFTW branch. */
int sxsg_plan_set_poses(sxsg_plan *plan, const int64_t *index, int64_t n, int skip);
/* Upper bound on the device memory of the per-chunk translated table (the
 * default is half the free memory at plan creation); touched (z, b2, g2)
 * combos are processed in chunks that fit.  A bound below the plan's
 * current buffer releases that buffer (after the plan's queued work). */
int sxsg_plan_set_budget(sxsg_plan *plan, size_t bytes);
/* Rotation engine of a mixed-precision plan: SXSG_ROT_CUDA (CUDA cores,
 * the default) or SXSG_ROT_TC (tcgen05 tensor cores, 3xTF32 with FP32
 * accumulation, for 2L + 1 <= 64; larger L stays on CUDA cores).  FP64
 * plans always rotate on CUDA cores.  The tensor-core kernel's waits for its
 * MMAs are bounded: sxsg_plan_run returns -6 when a wait gave up (the run's
 * results are invalid) and -7 when the MMAs did not finish in a second
 * bounded wait either (tensor memory was left allocated: treat the CUDA
 * context as unusable). */
enum { SXSG_ROT_CUDA = 0, SXSG_ROT_TC = 1 };
int sxsg_plan_set_rotation(sxsg_plan *plan, int engine);
/* Tile choices of a mixed-precision plan: slices of combos per block of the
 * pipelined translation (1..64) and gamma pairs per thread of the rotation
 * (2, 4, 6, 8, 12 or 16; values below what L + 1 needs are raised to it);
 * 0 keeps the default, the entry of the library's autotuned table nearest
 * to the plan's (L, Q) (sxsg_tiles_default).  Results do not depend on
 * them. */
int sxsg_plan_set_tiles(sxsg_plan *plan, int tr_slices, int rot_gamma);
int sxsg_tiles_default(int L, int Q, int *tr_slices, int *rot_gamma);
/* Translation fused with the per-pose contraction (mixed precision,
 * L <= 31): the translated rows of a chunk's combos are contracted with
 * their poses' receptor rows as they are formed, never stored; per pose and
 * m the six channel sums are kept and added over m.  It saves the round
 * trip of the translated rows through device memory (2.5 MB per row at
 * L = 30, Q = 201, for ~1-3 poses each in sparse lists) but gathers the
 * receptor rows at the translation's low occupancy, and measured slower on
 * GB300 at every density tried, so SXSG_FUSE_AUTO (default) keeps the
 * stored rows; SXSG_FUSE_ON selects it.  Results differ from the stored-row
 * path only by FP32 rounding (another summation order). */
enum { SXSG_FUSE_AUTO = 0, SXSG_FUSE_ON = 1, SXSG_FUSE_OFF = 2 };
int sxsg_plan_set_fused(sxsg_plan *plan, int mode);
/* Run the GPU work for the current pose list (asynchronous until results). */
int sxsg_plan_run(sxsg_plan *plan, int fit_mode);
/* Copy results to the host.  Any pointer may be NULL.  chi/c1/c2/cell: [n];
 * cross: raw cross terms [n][6][qnum] (VV,VD,VW,DD,DW,WW before the peak
 * rescale); grid: chi^2 [n][n1][n2] (grid fit only). */
int sxsg_plan_results(sxsg_plan *plan, double *chi, double *c1, double *c2, int32_t *cell,
                      double *cross, double *grid);
/* The k best poses of the last fitted run (grid or L-BFGS-B), selected on
 * the device: pose[i] = position in the plan's pose list, with its chi, c1,
 * c2 (any output may be NULL), in ascending chi, ties in list order, NaN
 * last (the order of a stable argsort).  k <= 16384; a k above the number of
 * poses returns every pose.  Returns the number written, or a negative
 * error.  It has no counterpart in the reference, which writes every pose's
 * score (tools/correlate.c:362-375). */
int sxsg_plan_topk(sxsg_plan *plan, int k, int64_t *pose, double *chi, double *c1, double *c2);
/* Stage timings of the last run in ms (CUDA events on the plan stream):
 * [0] tables, [1] translate, [2] per-pose, [3] fit, [4] whole run. */
int sxsg_plan_timings(sxsg_plan *plan, double *ms5);
/* Chunks of the translated table the last run was split into (the pose
 * list is processed one chunk of whole z slices at a time, sized by the
 * plan's budget); 0 before the first run. */
int sxsg_plan_chunks(const sxsg_plan *plan);
void sxsg_plan_destroy(sxsg_plan *plan);

/* ------------------------------------------------------------ batches
 * Many dimers of uneven size (each its own L, q grid, experiment, pose list
 * and fit grid) scored together: a batch captures, once, one CUDA graph
 * over all of them: the per-z tables per dimer; one persistent launch per
 * rotation group size whose blocks take (table, tile, beta, m) work items,
 * largest dimers first; phases, each translating the chunks of several
 * dimers into one shared device arena and then contracting them with their
 * poses (single-dimer launches per chunk, or work-item launches with
 * SXSG_BATCH_ITEMS); one persistent fit launch over (dimer, pose group)
 * items.  Plans: mixed precision, L <= 31, own rotation tables, pose lists
 * set; each plan's results equal a sxsg_plan_run of it bit for bit and are
 * read with sxsg_plan_results / sxsg_plan_topk after sxsg_batch_run.
 * A batch holds the plans' device pointers: changing a plan's poses, tiles
 * or budget, or destroying it, needs a new batch; the batches (and plan
 * runs) of one plan must not run at the same time, as they write its
 * outputs.  After a run each plan's sxsg_plan_timings reports the batch's
 * stages ([0] tables, [1] translation + per-pose, [3] fit, [4] graph). */
typedef struct sxsg_batch sxsg_batch;
typedef struct {
	int plans;          /* dimers */
	int phases;         /* arena fills of the translated tables */
	int launches;       /* kernel launches of one replay */
	int64_t items;      /* work items of all persistent launches */
	int64_t poses;      /* poses scored by one replay */
	size_t arena_bytes; /* translated-table arena */
	double ms[4];       /* last replay: [0] tables, [1] translation + per-pose, [2] fit, [3] whole graph */
} sxsg_batch_stats;
/* Launch forms of a batch (flags):
 *   SXSG_BATCH_PERSISTENT  work-item launches run persistently (SMs x
 *                          resident blocks taking items through an atomic
 *                          counter); without it one block per item, in order
 *   SXSG_BATCH_ITEMS       the translation and per-pose work of a phase as
 *                          work-item launches over all its chunks too;
 *                          without it (faster on GB300) each chunk's
 *                          translation and per-pose work are the single-dimer
 *                          launches, inside the same graph and phases; the
 *                          rotations and the fit are work-item launches in
 *                          every form
 *   SXSG_BATCH_OVERLAP     two arena halves: the translations of phase
 *                          k + 1 run beside the per-pose work of phase k */
enum { SXSG_BATCH_PERSISTENT = 1, SXSG_BATCH_OVERLAP = 2, SXSG_BATCH_ITEMS = 4 };
/* fit_mode: SXSG_FIT_GRID or SXSG_FIT_NONE; arena_bytes: upper bound on
 * the translated-table arena (0 = what the dimers need, at most half the
 * free device memory) */
int sxsg_batch_create(sxsg_plan *const *plans, int nplan, int fit_mode, size_t arena_bytes, int flags,
                      sxsg_batch **batch);
/* one replay of the graph; returns when it has finished */
int sxsg_batch_run(sxsg_batch *batch);
int sxsg_batch_stats_get(const sxsg_batch *batch, sxsg_batch_stats *stats);
void sxsg_batch_destroy(sxsg_batch *batch);

/* ------------------------------------------------------------ serving
 * A persistent pool of workers that keeps the GPU busy with many scoring
 * jobs (the FFT-correlate work of sxs_compute_saxs_scores for one dimer
 * each).  Jobs are admitted in arrival order as device memory frees up under
 * an HBM cap, run concurrently on separate streams, and their results are
 * bitwise those of the same job run alone.  Rotation tables of molecules
 * with a nonzero key are cached on the device across jobs; a table is shared
 * once the job that filled it has finished, and a job whose table is still
 * being filled by another one fills its own copy. */
typedef struct sxsg_server sxsg_server;

typedef struct {
	const double *A, *B;          /* flat expansions [3][qnum][(L+1)^2][2] */
	uint64_t keyA, keyB;          /* nonzero: cache this molecule's rotation table on the
	                               * device (the key is combined with a digest of the
	                               * coefficients, so a reused key never returns another
	                               * molecule's table); 0 = not cached */
	const double *qvals;
	int qnum;
	const double *zvals;
	int znum;
	int L;
	const double *a;              /* binned experiment a[6 qnum], mult, peak */
	double mult, peak;
	const double *c1grid;         /* fit grid (grid fit) */
	int n1;
	const double *c2grid;
	int n2;
	const int64_t *index;         /* packed grid indices of the poses */
	int64_t n;
	int skip;
	int fit_mode;                 /* SXSG_FIT_* */
	int precision;                /* SXSG_FP64 or SXSG_MIXED */
} sxsg_request;

/* hbm_cap: device bytes the server may hold (0 = 90% of the free memory);
 * max_active: jobs on the device at once (workers, 1..64). */
int sxsg_server_create(sxsg_server **server, size_t hbm_cap, int max_active);
/* Queue a job; every input is copied, so the caller may reuse its buffers.
 * Returns the ticket (>= 0) or a negative error. */
int64_t sxsg_server_submit(sxsg_server *server, const sxsg_request *request);
/* 1 when the job is done, 0 while queued or running. */
int sxsg_server_poll(sxsg_server *server, int64_t ticket);
/* Block until the job is done and collect chi, c1, c2 [n] (any may be
 * NULL) and ms3 = {queued, running, submit-to-done} milliseconds.  A ticket
 * is collected once.  Returns the job's status (0 or the error of the run,
 * with its message in sxsg_last_error). */
int sxsg_server_wait(sxsg_server *server, int64_t ticket, double *chi, double *c1, double *c2, double *ms3);
/* out8 = {jobs done, poses done, jobs queued, bytes held by running jobs,
 * bytes of cached tables, cached tables, cache hits, cache misses} */
int sxsg_server_stats(sxsg_server *server, double *out8);
/* Finish every queued job, then release the workers and the cache. */
void sxsg_server_destroy(sxsg_server *server);

/* One-shot scoring from host buffers: plan, poses, run, results, release.
 * chi/c1/c2 may be NULL; cross [n][6][qnum] may be NULL; precision is
 * SXSG_FP64 or SXSG_MIXED. */
int sxsg_score_flat(const double *A, const double *B, const double *qvals, int qnum, const double *zvals, int znum,
                    int L, const int64_t *index, int64_t n, int skip, const double *a, double mult, double peak,
                    int fit_mode, const double *c1grid, int n1, const double *c2grid, int n2,
                    double *chi, double *c1, double *c2, double *cross, int precision);

/* Exact per-pose scoring, the reference's score_ft_naive flow
 * (tools/score_ft_naive.c:156-212), for cross-checking the grid method:
 * for each Euler pose eu[6 i .. 6 i + 5] = (z, beta1, gamma1, alpha2,
 * beta2, gamma2) the receptor (rec_xyz[3 nrec], centred at its centre of
 * extrema) is turned by the active rotation R(0, beta1, gamma1), the ligand
 * (lig_xyz[3 nlig], centred at its centroid) by R(alpha2, beta2, gamma2)
 * and moved by (0, 0, z); the joined complex (receptor first) is centred at
 * its centroid, expanded to A_lm at L on qvals (the kernels of
 * sxsg_expand), reduced to its cross terms (sxs_spf2cross_terms) and fitted
 * by L-BFGS-B without the peak rescale (sxs_spf2fitted_profile).
 * vac, dum, water_w: per atom of the joined order (water_w = water form
 * factor x accessible fraction, NULL for none); a[6 qnum], mult: the binned
 * experiment.  chi, c1, c2 [n] and cross [n][6][qnum] may be NULL. */
int sxsg_score_exact(const double *rec_xyz, int nrec, const double *lig_xyz, int nlig, const double *vac,
                     const double *dum, const double *water_w, const double *euler, int64_t n, const double *qvals,
                     int qnum, int L, const double *a, double mult, double *chi, double *c1, double *c2,
                     double *cross);

/* Accessible fraction per atom on the GPU (Shrake-Rupley: the solvent
 * sphere of radius + probe sampled at sph[npts][3] unit points, a golden
 * spiral of npts points when sph is NULL; fraction of points not inside
 * any neighbour's sphere; 0 for a zero radius).  The reference takes this
 * input from libmol2's accs (sxs_faccs, src/saxs_utils.c:30-48), which is
 * not part of it; this is the restatement the synthetic workloads use.
 * 1 <= npts <= 1024. */
int sxsg_sasa(const double *xyz, const double *radius, int natoms, double probe, const double *sph, int npts,
              double *frac);

/* Pose ingestion helpers (tools/correlate.c:202-240): grid index of one
 * Euler 6-tuple (z, b1, g1, a2, b2, g2 as written by sxs_ft2euler) at
 * translation slot z_idx. */
int64_t sxsg_assemble_index(const double *euler6, int z_idx, int L);

/* Batch pose ingestion, the way correlate builds its index list
 * (index.c:38-75 then tools/correlate.c:172-251): for each pose i the
 * ligand rotation rot[9i..9i+8] (row-major) and translation tr[3i..3i+2]
 * go through sxs_ft2euler (reference ligand offset ref_lig[3]), the Euler
 * values through the "% .3f" text round trip of the Euler file, z is
 * matched to zvals within 1e-3, and the grid index is assembled.  keep[i]
 * is 0 for poses whose z is not in zvals (index[i] = -1).  Returns the
 * number kept. */
int64_t sxsg_poses_to_indices(const double *rot, const double *tr, int64_t n, const double *ref_lig,
                              const double *zvals, int znum, int L, int64_t *index, uint8_t *keep);

/* Options of the _ex forms.  SXSG_WRAP_ANGLES: the alpha/gamma grid digits
 * are taken mod N.  The reference rounds them without wrapping
 * (tools/correlate.c:233-240), so an angle within half a step of 2 pi
 * (alpha2' = 2 pi - alpha2 for alpha2 < pi/N, about 1/N of random poses)
 * gets digit N, which carries into the next digit of the packed index and
 * scores a different cell; the plain forms keep that for bit-exact parity. */
enum { SXSG_WRAP_ANGLES = 1 };
int64_t sxsg_assemble_index_ex(const double *euler6, int z_idx, int L, int flags);
int64_t sxsg_poses_to_indices_ex(const double *rot, const double *tr, int64_t n, const double *ref_lig,
                                 const double *zvals, int znum, int L, int64_t *index, uint8_t *keep, int flags);

/* sxsg_poses_to_indices_ex on the GPU, with the same results: the device
 * converts every pose (a thread each), and the few poses whose result could
 * depend on the last bits of acos, sin or cos (a value within a few ulps of
 * a "% .3f" rounding boundary, or an ill-conditioned angle: acos argument
 * near +-1, sin beta near 0, a tested sign of a near-zero entry) are redone
 * by the host path; *host_poses (may be NULL) gives their number.  Host
 * buffers in and out, processed in device batches of 2^20 poses. */
int64_t sxsg_poses_to_indices_gpu(const double *rot, const double *tr, int64_t n, const double *ref_lig,
                                  const double *zvals, int znum, int L, int64_t *index, uint8_t *keep, int flags,
                                  int64_t *host_poses);

/* Timing on the library's stream: start records an event; stop records a
 * second one, waits for it and returns the elapsed milliseconds. */
int sxsg_timer_start(void);
double sxsg_timer_stop(void);

/* Dense FP64 multiply-add rate of this GPU (TFLOP/s), measured with a
 * register-resident FMA chain on every SM. */
double sxsg_fp64_fma_tflops(void);
/* Dense FP32 multiply-add rate of this GPU (TFLOP/s), measured the same way. */
double sxsg_fp32_fma_tflops(void);
/* L2-to-SM read bandwidth of this GPU (GB/s): 16-byte L2-only loads by every
 * SM over a 32 MiB L2-resident buffer. */
double sxsg_l2_read_gbs(void);

#ifdef __cplusplus
}
#endif
#endif
