/*
 * CPU oracle: a plain-C restatement of libfmftsaxs's FFT-correlation scoring
 * path (the path `correlate` drives through sxs_compute_saxs_scores) and of
 * the per-molecule A_lm expansion that feeds it.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it, and only as the checker.  The product
 * (libfmftsaxs_gb300) never links, loads or calls it.
 *
 * Every routine cites the reference file:line it restates.  Where rounding
 * matters for 1e-10 parity (the spherical-Bessel power series, the Wigner-d
 * recurrence, the 3j table, the twiddle tables) the operation order follows
 * the reference exactly; the build disables multiply-add contraction.
 *
 * pi: the reference is compiled with -std=c11 (CMakeLists.txt:57-58), so
 * <math.h> does not define M_PI and src/define.h:14-16 supplies
 * 3.14159265358.  That truncated value is the pi of every reference formula
 * (beta grid, twiddles, 4*pi factors, Y_lm norms) and the oracle uses it.
 *
 * Flat layouts (all row-major, doubles):
 *   spf   [3 ch: V,D,W][qnum][(L+1)^2 lm][re,im], lm = l(l+1)+m
 *   cross [6: VV,VD,VW,DD,DW,WW][qnum]
 *   dtab  [L+1 l][2L+1 m+L][2L+1 m1+L]   (index_d_array, src/borrowed.h:78-81)
 *   dsymb [(L+1)^2 lm][L+1 l1][2L+1 p]   (d_symb_index, src/fftsaxs.c:3-6)
 */
#ifndef SXS_ORACLE_H
#define SXS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PI 3.14159265358

double orc_sbessel(int l, double x);
void orc_mkarray(double begin, double end, int n, double *out);
void orc_wigner_d(int L, double beta, double *dtab);
double orc_w3j(int j1, int j2, int j3, int m1, int m2, int m3);
void orc_dsymb(int L, double *dsymb);
void orc_besselj_n(double z, const double *q, int qnum, int L, double *bes);
void orc_t_matrix(int L, int qnum, const double *bes, const double *dsymb, double *t_re, double *t_im);
double orc_average_radius(const double *vdw, int n);
void orc_expand(const double *xyz, const double *vac_ff, const double *dum_ff, const double *sasa,
                double h2o_ff, int natoms, const double *q, int qnum, int L, double *spf);
void orc_opt_params(const double *eq, const double *ei, const double *ee, int ne,
                    const double *q, int qnum, double rm, double *a, double *mult, double *peak);
double orc_best_scale(const double *cross, const double *q, int qnum, const double *a, double mult,
                      double c1, double c2);
double orc_point_score(const double *cross, const double *q, int qnum, const double *a, double mult,
                       double c1, double c2);
void orc_rescale(double *cross, int qnum, double peak);
void orc_compile_intensity(const double *cross, const double *q, int qnum, double rm, double rerr,
                           double c1, double c2, double *in, double *err);
void orc_profile_from_spf(const double *spf, int L, int qnum, double rm, const double *q,
                          double c1, double c2, double *in, double *err);
void orc_spf2cross_terms(const double *spf, int L, int qnum, double *cross);
void orc_ft2euler(const double *tv, const double *rm9, const double *ref_lig, double *eu6);
int orc_assemble_index(const double *eu6, int z_idx, int L);
int orc_score(const double *A, const double *B, const double *q, int qnum, const double *z, int znum,
              int L, const int *index, int nout, int skip, double peak,
              const double *a, double mult, const double *c1g, int n1, const double *c2g, int n2,
              double *cross_raw, double *cross_scaled, double *grid, int *branch);

#ifdef __cplusplus
}
#endif
#endif
