/*
 * A libfmftsaxs-style caller of the scoring path, compiled against
 * include/fmftsaxs_gb300.h and linked with libfmftsaxs_gb300.so.
 *
 * It uses only the reference's own API and struct layouts, the way
 * tools/correlate.c does (tools/correlate.c:71-93 builds the SPFs, the
 * experimental profile and the fit parameters; :264-272 scores):
 * sxs_spf_full_create + the V/D/W coefficient arrays, sxs_profile_create +
 * in/err, sxs_opt_params_create, sxs_assemble_index /
 * sxs_disassemble_index, sxs_compute_saxs_scores.  No sxsg_* extension is
 * called.
 *
 * Input (binary, native endianness), written by the test that runs this:
 *   int32  L, qnum, nexp, znum, n, skip
 *   double rmA, rmB, rm
 *   double q[qnum], z[znum], exp_q[nexp], exp_i[nexp], exp_err[nexp]
 *   double A[3][qnum][(L+1)^2][2], B[...]      (V, D, W; re, im)
 *   int32  index[n]
 * Output: one line per pose, "chi c1 c2" with 17 significant digits.
 */
#include "fmftsaxs_gb300.h"

#include <stdlib.h>

static void need(int ok, const char *what)
{
	if (!ok) {
		fprintf(stderr, "dropin_caller: %s\n", what);
		exit(2);
	}
}

static double *read_doubles(FILE *f, size_t n)
{
	double *v = malloc(sizeof(double) * (n ? n : 1));
	need(v != NULL, "out of memory");
	need(fread(v, sizeof(double), n, f) == n, "short read (doubles)");
	return v;
}

static struct sxs_spf_full *read_spf(FILE *f, int L, int qnum, double rm)
{
	int K2 = (L + 1) * (L + 1);
	struct sxs_spf_full *s = sxs_spf_full_create(L, qnum);
	double *flat = read_doubles(f, (size_t)3 * qnum * K2 * 2);
	for (int ch = 0; ch < 3; ch++) {
		struct sxs_spf_sing **c = ch == 0 ? s->V : (ch == 1 ? s->D : s->W);
		for (int q = 0; q < qnum; q++)
			for (int i = 0; i < K2; i++) {
				const double *v = flat + (((size_t)ch * qnum + q) * K2 + i) * 2;
				c[q]->re[i] = v[0];
				c[q]->im[i] = v[1];
			}
	}
	s->rm = rm;
	free(flat);
	return s;
}

int main(int argc, char **argv)
{
	need(argc == 3, "usage: dropin_caller <input.bin> <output.txt>");
	FILE *f = fopen(argv[1], "rb");
	need(f != NULL, "cannot open input");
	int32_t hdr[6];
	need(fread(hdr, sizeof(int32_t), 6, f) == 6, "short read (header)");
	int L = hdr[0], qnum = hdr[1], nexp = hdr[2], znum = hdr[3], n = hdr[4], skip = hdr[5];
	need(L > 0 && qnum > 0 && nexp > 0 && znum > 0 && n >= 0, "bad header");
	double *rms = read_doubles(f, 3);
	double *qvals = read_doubles(f, (size_t)qnum);
	double *zvals = read_doubles(f, (size_t)znum);
	double *eq = read_doubles(f, (size_t)nexp);
	double *ei = read_doubles(f, (size_t)nexp);
	double *ee = read_doubles(f, (size_t)nexp);
	struct sxs_spf_full *A = read_spf(f, L, qnum, rms[0]);
	struct sxs_spf_full *B = read_spf(f, L, qnum, rms[1]);
	int *index = malloc(sizeof(int) * (n ? n : 1));
	need(index != NULL, "out of memory");
	need(fread(index, sizeof(int), (size_t)n, f) == (size_t)n, "short read (index)");
	fclose(f);

	/* the grid-index helpers of src/index.h round-trip every pose index */
	for (int i = 0; i < n; i++) {
		struct sxs_index id;
		sxs_disassemble_index(&id, (size_t)index[i], L + 1, L);
		need(sxs_assemble_index(&id, L + 1, L) == (size_t)index[i], "index helpers do not round-trip");
	}

	struct sxs_profile *exp_profile = sxs_profile_create(eq, nexp, 0);
	for (int i = 0; i < nexp; i++) {
		exp_profile->in[i] = ei[i];
		exp_profile->err[i] = ee[i];
	}
	struct sxs_opt_params *params = sxs_opt_params_create(exp_profile, qvals, qnum, rms[2]);
	sxs_profile_free(exp_profile);

	double *chi = calloc((size_t)(n ? n : 1), sizeof(double));
	double *c1 = calloc((size_t)(n ? n : 1), sizeof(double));
	double *c2 = calloc((size_t)(n ? n : 1), sizeof(double));
	need(chi && c1 && c2, "out of memory");
	sxs_compute_saxs_scores(chi, c1, c2, index, n, A, B, params, qvals, qnum, zvals, znum, L, skip);

	FILE *o = fopen(argv[2], "w");
	need(o != NULL, "cannot open output");
	for (int i = 0; i < n; i++)
		fprintf(o, "%.17g %.17g %.17g\n", chi[i], c1[i], c2[i]);
	fclose(o);

	sxs_opt_params_free(params);
	sxs_spf_full_free(A);
	sxs_spf_full_free(B);
	free(chi); free(c1); free(c2); free(index);
	free(rms); free(qvals); free(zvals); free(eq); free(ei); free(ee);
	return 0;
}
