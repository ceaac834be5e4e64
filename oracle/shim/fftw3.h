/*
 * Test-infrastructure shim: the FFTW3 calls made by the reference
 * (src/fftsaxs.c:675-683, 899-900, 974-976), so that its own sources compile
 * into the checker library under oracle/_ref/.  FFTW3 (linked as `fftw3`,
 * reference CMakeLists.txt:121, no pinned version) is absent here.
 *
 * Published semantics restated: FFTW_FORWARD computes, per transform,
 *   out[k0,k1,k2] = sum_j in[j0,j1,j2] exp(-2 pi i (j0 k0/n0 + j1 k1/n1 + j2 k2/n2)),
 * row-major, `howmany` transforms spaced `idist` / `odist` apart.  The shim
 * evaluates it as three passes of exact-twiddle 1-D DFTs in double.  FFTW's
 * own rounding differs at the 1e-16 level; no reference test pins that branch.
 * <complex.h> is included before this header (src/fftsaxs.h:38-39), so
 * fftw_complex is C99 `double _Complex`, as with real FFTW.
 */
#ifndef SXS_SHIM_FFTW3_H
#define SXS_SHIM_FFTW3_H

#include <complex.h>
#include <stddef.h>

typedef double _Complex fftw_complex;
typedef struct shim_fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_PATIENT (1U << 5)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed, int istride, int idist,
                             fftw_complex *out, const int *onembed, int ostride, int odist,
                             int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#endif
