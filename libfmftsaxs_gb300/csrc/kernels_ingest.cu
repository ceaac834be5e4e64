/*
 * Pose ingestion on the GPU: a ligand pose given as an FT-style rotation
 * and translation becomes the packed grid index that correlate builds for
 * it (src/index.c:38-75, then tools/correlate.c:202-251): Euler angles by
 * ft2euler, the "% .3f" text round trip of the Euler file, z matched to the
 * translation grid within 1e-3, the angle digits rounded without wrap (or
 * mod N with SXSG_WRAP_ANGLES).
 *
 * Compiled with -fmad=false: every expression is evaluated with one rounding
 * per operation in the host code's order (csrc/sxs_api.c, sxs_ft2euler and
 * sxsg_poses_to_indices_ex).  The device's acos, sin, cos may differ from
 * the host C library's in the last bits; that can change a result only where
 * a value lies within a few ulps of a "% .3f" rounding boundary, or where the
 * formula amplifies such differences (acos near +-1, division by a small
 * sin beta, the sign of a near-zero matrix entry).  Those poses are flagged
 * and recomputed on the host, so every index equals the host path's.
 *
 * The "% .3f" round trip is exact: v * 1000 is split into its rounded value
 * and the exact residual (an FMA), which decide the nearest multiple of
 * 0.001 as printf does (ties to even); reading "n/1000" back is the
 * correctly rounded quotient n / 1000.
 */
#include "kernels.h"

#include <math.h>

#define SXS_PI 3.14159265358 /* the reference's pi (src/define.h:14-16 under -std=c11) */

namespace {

/* margins of the host fallback: acos arguments within ING_EDGE of +-1 on
 * either side (inside, the slope 1/sqrt(1 - x^2) passes 700; just outside,
 * the value is clamped, and both machines must land on the same side),
 * sin beta below ING_SIN, matrix entries whose sign is tested below
 * ING_SIGN, values whose 1000-fold fractional part is within ING_HALF of
 * 1/2.  Arguments further outside [-1, 1] clamp to exactly +-1 on both. */
#define ING_EDGE 1e-6
#define ING_SIN 1e-3
#define ING_SIGN 1e-9
#define ING_HALF 1e-5

__device__ __forceinline__ double clamp1(double a) { return a < -1.0 ? -1.0 : (a > 1.0 ? 1.0 : a); }

__device__ __forceinline__ bool near_one(double x) { return fabs(fabs(x) - 1.0) < ING_EDGE; }

__device__ __forceinline__ bool near_half(double v)
{
	double p = fabs(v) * 1000.0;
	double f = p - floor(p);
	return fabs(f - 0.5) < ING_HALF;
}

/* printf("% .3f", v) read back with strtod */
__device__ double round3(double v)
{
	double a = fabs(v);
	double p = a * 1000.0;
	double err = fma(a, 1000.0, -p);   /* exact: a * 1000 = p + err */
	double n = floor(p);
	double f = p - n;                  /* exact for p < 2^52 */
	bool up;
	if (f > 0.5) up = true;
	else if (f < 0.5) up = false;
	else if (err != 0.0) up = err > 0.0;
	else up = fmod(n, 2.0) != 0.0;     /* a tie: to the even digit */
	if (up) n += 1.0;
	return copysign(n / 1000.0, v);
}

__global__ void k_pose_ingest(const double *__restrict__ rot, const double *__restrict__ tr, long n, double rx,
                              double ry, double rz, const double *__restrict__ zvals, int znum, int L, int wrap,
                              long long *__restrict__ index, unsigned char *__restrict__ keep,
                              unsigned int *__restrict__ nflag, long long *__restrict__ flagged)
{
	long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const double *m = rot + 9 * i;
	double vx = tr[3 * i] + rx, vy = tr[3 * i + 1] + ry, vz = tr[3 * i + 2] + rz;
	double z = round(sqrt(vx * vx + vy * vy + vz * vz));
	bool flag = false;
	double x = vz / z;
	flag |= near_one(x);
	double b1 = acos(clamp1(x));
	double sb1 = sin(b1);
	flag |= sb1 < ING_SIN;
	x = -vx / (z * sb1);
	flag |= near_one(x);
	double g1 = acos(clamp1(x));
	if (vy / (z * sb1) < 0.0) g1 = 2 * SXS_PI - g1;
	/* receptor rotation R(0, b1, g1) (sxs_fill_active_rotation_matrix with
	 * cos 0 = 1, sin 0 = 0), times the ligand rotation */
	double ca = cos(0.0), sa = sin(0.0), cb = cos(b1), sb = sin(b1), cg = cos(g1), sg = sin(g1);
	double a11 = cg * cb * ca - sg * sa, a21 = cg * cb * sa + sg * ca, a31 = -cg * sb;
	double a12 = -sg * cb * ca - cg * sa, a22 = -sg * cb * sa + cg * ca, a32 = sg * sb;
	double a13 = sb * ca, a23 = sb * sa, a33 = cb;
	double l13 = a11 * m[2] + a12 * m[5] + a13 * m[8];
	double l23 = a21 * m[2] + a22 * m[5] + a23 * m[8];
	double l31 = a31 * m[0] + a32 * m[3] + a33 * m[6];
	double l32 = a31 * m[1] + a32 * m[4] + a33 * m[7];
	double l33 = a31 * m[2] + a32 * m[5] + a33 * m[8];
	flag |= near_one(l33);
	double b2 = acos(clamp1(l33));
	double sb2 = sin(b2);
	flag |= sb2 < ING_SIN;
	x = l13 / sb2;
	flag |= near_one(x);
	double a2 = acos(clamp1(x));
	flag |= fabs(l23) < ING_SIGN;
	if (l23 / sb2 < 0.0) a2 = 2 * SXS_PI - a2;
	x = -l31 / sb2;
	flag |= near_one(x);
	double g2 = acos(clamp1(x));
	flag |= fabs(l32) < ING_SIGN;
	if (l32 / sb2 < 0.0) g2 = 2 * SXS_PI - g2;
	double v[6] = {z, b1, g1, a2, b2, g2};
#pragma unroll
	for (int k = 0; k < 6; k++) {
		flag |= k > 0 && near_half(v[k]);
		v[k] = round3(v[k]);
	}
	if (flag) {
		unsigned int at = atomicAdd(nflag, 1u);
		if (at < (unsigned long)n) flagged[at] = i;   /* n slots: never full */
	}
	int zi = -1;
	for (int j = 0; j < znum; j++)
		if (zvals[j] > v[0] - 0.001 && zvals[j] < v[0] + 0.001) {
			zi = j;
			break;
		}
	if (zi < 0) {
		keep[i] = 0;
		index[i] = -1;
		return;
	}
	int nb = L + 1, N = 2 * L + 1;
	double ea2 = 2 * SXS_PI - v[3];
	double eg2 = 2 * SXS_PI - v[5];
	double bs = SXS_PI / L, as = 2.0 * SXS_PI / (2 * L + 1);
	int da = (int)round(ea2 / as), dg1 = (int)round(v[2] / as), dg2 = (int)round(eg2 / as);
	if (wrap) {
		da = ((da % N) + N) % N;
		dg1 = ((dg1 % N) + N) % N;
		dg2 = ((dg2 % N) + N) % N;
	}
	long long id = (long long)zi * nb;
	id = (id + (int)round(v[1] / bs)) * nb;
	id = (id + (int)round(v[4] / bs)) * N;
	id = (id + da) * N;
	id = (id + dg1) * N;
	id = id + dg2;
	keep[i] = 1;
	index[i] = id;
}

} // namespace

extern "C" int sxsk_pose_ingest(const double *rot, const double *tr, long n, const double *ref, const double *zvals,
                                int znum, int L, int wrap, long long *index, unsigned char *keep, unsigned int *nflag,
                                long long *flagged, cudaStream_t s)
{
	if (n <= 0) return 0;
	if (n > 0x7fffffffL * 128L) return cudaErrorInvalidValue;
	k_pose_ingest<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(rot, tr, n, ref[0], ref[1], ref[2], zvals, znum, L, wrap,
	                                                           index, keep, nflag, flagged);
	return cudaGetLastError();
}
