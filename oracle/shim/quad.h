/*
 * IEEE binary128 ("quad") helpers shared by the oracle and the checker shims.
 * x86-64 gcc spells the type __float128; aarch64 gcc makes `long double`
 * binary128.  Both give correctly rounded + - * /, so results agree bit for
 * bit on both hosts.  Square root is a Newton refinement from the double
 * estimate (two steps reach quad precision), which avoids libquadmath.
 */
#ifndef SXS_QUAD_H
#define SXS_QUAD_H

#include <math.h>

#if defined(__x86_64__) || defined(__i386__)
typedef __float128 sxs_quad;
#elif defined(__aarch64__)
typedef long double sxs_quad;
#else
#error "binary128 type not known for this host"
#endif

/* Arguments outside the double range (the 3j prefactors from L = 32 on)
 * are first scaled by an even power of two, exactly, and the root by the
 * half power, so the double estimate stays finite; inside the double range
 * the result is unchanged. */
static inline sxs_quad sxs_quad_sqrt(sxs_quad a)
{
	if (a <= 0) return 0;
	sxs_quad s = 1;
	while (a > (sxs_quad)0x1p1000) {
		a *= (sxs_quad)0x1p-1000;
		s *= (sxs_quad)0x1p500;
	}
	while (a < (sxs_quad)0x1p-1000) {
		a *= (sxs_quad)0x1p1000;
		s *= (sxs_quad)0x1p-500;
	}
	sxs_quad y = (sxs_quad)sqrt((double)a);
	y = (y + a / y) * (sxs_quad)0.5;
	y = (y + a / y) * (sxs_quad)0.5;
	return y * s;
}

/* Round a quad to double towards zero (the rounding GMP's mpf_get_d uses). */
static inline double sxs_quad_to_double_trunc(sxs_quad a)
{
	double d = (double)a;
	if (a > 0 && (sxs_quad)d > a) d = nextafter(d, 0.0);
	if (a < 0 && (sxs_quad)d < a) d = nextafter(d, 0.0);
	return d;
}

#endif
