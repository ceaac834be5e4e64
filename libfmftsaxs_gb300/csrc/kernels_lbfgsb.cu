/*
 * Batched L-BFGS-B fit of (c1, c2) on the device: one thread per pose,
 * the solver of lbfgsb_core.h (the reference's fit, src/min_saxs.c:153-259).
 * Compiled with -fmad=false so that every objective and solver step rounds
 * like the reference's C code.
 */
#include "kernels.h"
#include "lbfgsb_core.h"

namespace {

/* raw [pose][6][Q] -> transposed [6*Q][pose], with the peak rescale of
 * src/min_saxs.c:170-188 when rescale != 0 */
__device__ __forceinline__ double cross_at(const double *c, size_t i) { return c[i]; }
__device__ __forceinline__ double cross_at(const float2 *c, size_t i) { return (double)c[i].x + (double)c[i].y; }

template <typename T>
__global__ void k_rescale_transpose(const T *__restrict__ cross, double *__restrict__ ct, int npose, int Q,
                                    double peak, int rescale)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= (long)npose * 6 * Q) return;
	int p = (int)(i % npose);
	int cq = (int)(i / npose);
	size_t b = (size_t)p * 6 * Q;
	double v = cross_at(cross, b + cq);
	if (rescale) {
		double s = cross_at(cross, b) + cross_at(cross, b + 3 * Q) + cross_at(cross, b + 5 * Q) +
		           cross_at(cross, b + 2 * Q) - cross_at(cross, b + Q) - cross_at(cross, b + 4 * Q);
		s = peak / s;
		v *= s;
	}
	ct[i] = v;
}

__global__ void k_lbfgsb(const double *__restrict__ ct, int npose, int Q, const double *__restrict__ q,
                         const double *__restrict__ a, double mult, int max_eval, double *__restrict__ chi,
                         double *__restrict__ c1, double *__restrict__ c2, double *__restrict__ scale,
                         int *__restrict__ nevals)
{
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= npose) return;
	lb_saxs o;
	o.cr = ct + p;
	o.stride = npose;
	o.q = q;
	o.a = a;
	o.mult = mult;
	o.Q = Q;
	double x, y, z, w;
	int ne = lb_saxs_fit(&o, &x, &y, &z, &w, max_eval);
	chi[p] = x;
	c1[p] = y;
	c2[p] = z;
	if (scale) scale[p] = w;
	if (nevals) nevals[p] = ne;
}

} // namespace

/* cross: [npose][6][Q] (raw when rescale != 0, already rescaled otherwise);
 * ct: workspace of npose*6*Q doubles that receives the transposed terms. */
extern "C" int sxs_fit_lbfgsb_launch(const void *cross, int cross_df, double *ct, int npose, int Q, const double *q,
                                     const double *a, double mult, double peak, int rescale, double *chi, double *c1,
                                     double *c2, double *scale, int *nevals, cudaStream_t s)
{
	if (npose <= 0) return 0;
	long n = (long)npose * 6 * Q;
	if (cross_df)
		k_rescale_transpose<float2><<<(int)((n + 255) / 256), 256, 0, s>>>((const float2 *)cross, ct, npose, Q, peak,
		                                                                 rescale);
	else
		k_rescale_transpose<double><<<(int)((n + 255) / 256), 256, 0, s>>>((const double *)cross, ct, npose, Q, peak,
		                                                                 rescale);
	k_lbfgsb<<<(npose + 63) / 64, 64, 0, s>>>(ct, npose, Q, q, a, mult, 100000, chi, c1, c2, scale, nevals);
	return (int)cudaGetLastError();
}
