/*
 * Test-infrastructure shim bodies for the checker build under oracle/_ref/:
 * FFTW3 forward DFT (restated: exact-twiddle separable DFT), the libmol2
 * utilities the reference calls, and an accs() that refuses to run (the
 * checker harness passes accessible fractions straight to
 * atom_grp2spf_inplace, src/pdb2spf.c:24-31).
 */
#include <complex.h>
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "fftw3.h"
#include "mol2/atom_group.h"
#include "mol2/sasa.h"
#include "mol2/lists.h"

/* Full-precision pi: FFTW's twiddles are accurate to the last bit. */
static const double SHIM_PI = 3.14159265358979323846;

struct shim_fftw_plan_s {
	int rank;
	int n[3];
	int howmany;
	fftw_complex *in, *out;
	int idist, odist;
	int sign;
};

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed, int istride, int idist,
                             fftw_complex *out, const int *onembed, int ostride, int odist,
                             int sign, unsigned flags)
{
	(void)flags;
	if (rank < 1 || rank > 3 || inembed || onembed || istride != 1 || ostride != 1) {
		fprintf(stderr, "fftw shim: unsupported plan\n");
		exit(EXIT_FAILURE);
	}
	struct shim_fftw_plan_s *p = calloc(1, sizeof(*p));
	p->rank = rank;
	for (int i = 0; i < 3; i++) p->n[i] = i < rank ? n[i] : 1;
	p->howmany = howmany;
	p->in = in; p->out = out; p->idist = idist; p->odist = odist; p->sign = sign;
	return p;
}

/* One pass of 1-D DFTs along axis `ax` of an n0 x n1 x n2 row-major block. */
static void dft_axis(fftw_complex *data, const int n[3], int ax, int sign, fftw_complex *line, fftw_complex *res)
{
	int len = n[ax];
	int stride = ax == 2 ? 1 : (ax == 1 ? n[2] : n[1] * n[2]);
	int outer = n[0] * n[1] * n[2] / len;
	double *c = malloc(sizeof(double) * len), *s = malloc(sizeof(double) * len);
	for (int k = 0; k < len; k++) {
		double ang = 2.0 * SHIM_PI * (double)k / (double)len;
		c[k] = cos(ang);
		s[k] = sign * sin(ang);
	}
	for (int o = 0; o < outer; o++) {
		/* base offset of line o */
		int base;
		if (ax == 2) base = o * len;
		else if (ax == 1) base = (o / n[2]) * n[1] * n[2] + (o % n[2]);
		else base = o;
		for (int j = 0; j < len; j++) line[j] = data[base + j * stride];
		for (int k = 0; k < len; k++) {
			double re = 0.0, im = 0.0;
			for (int j = 0; j < len; j++) {
				int t = (int)(((long)j * k) % len);
				double xr = creal(line[j]), xi = cimag(line[j]);
				re += xr * c[t] - xi * s[t];
				im += xr * s[t] + xi * c[t];
			}
			res[k] = CMPLX(re, im);
		}
		for (int k = 0; k < len; k++) data[base + k * stride] = res[k];
	}
	free(c); free(s);
}

void fftw_execute(const fftw_plan p)
{
	int total = p->n[0] * p->n[1] * p->n[2];
	int maxn = p->n[0] > p->n[1] ? p->n[0] : p->n[1];
	if (p->n[2] > maxn) maxn = p->n[2];
	fftw_complex *line = malloc(sizeof(fftw_complex) * maxn);
	fftw_complex *res = malloc(sizeof(fftw_complex) * maxn);
	for (int h = 0; h < p->howmany; h++) {
		fftw_complex *dst = p->out + (size_t)h * p->odist;
		const fftw_complex *src = p->in + (size_t)h * p->idist;
		memcpy(dst, src, sizeof(fftw_complex) * total);
		for (int ax = 0; ax < 3; ax++)
			if (p->n[ax] > 1) dft_axis(dst, p->n, ax, p->sign, line, res);
	}
	free(line); free(res);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

bool is_whitespace_line(const char *line)
{
	for (; *line; line++)
		if (!isspace((unsigned char)*line)) return false;
	return true;
}

void free_if_not_null(void *p) { if (p) free(p); }

void accs(double *as, const struct mol_atom_group *ag, double r_solv, short cont_acc)
{
	(void)as; (void)ag; (void)r_solv; (void)cont_acc;
	fprintf(stderr, "accs shim: accessible areas must be supplied by the caller\n");
	exit(EXIT_FAILURE);
}

struct mol_matrix3_list *mol_matrix3_list_from_file(const char *path)
{
	fprintf(stderr, "mol2 shim: rotation list files are not read here (%s)\n", path);
	exit(EXIT_FAILURE);
}
