/*
 * Test-infrastructure shim: the subset of the GMP `mpf_t` interface that the
 * reference calls (src/borrowed.c:73-222, src/fftsaxs.c:145-173), implemented
 * on IEEE binary128 so that the reference's own sources compile into the
 * checker library under oracle/_ref/.  GMP itself (libgmp, no pinned version
 * in the reference's CMakeLists.txt:121) has no development headers here.
 *
 * Published semantics restated:
 *   - mpf arithmetic carries at least the default precision (64 bits; GMP keeps
 *     two or three 64-bit limbs).  binary128 carries 113 bits.
 *   - mpf_get_d truncates towards zero (GMP manual, "Converting Floats").
 * Used only by oracle/_ref; nothing in the product links it.
 */
#ifndef SXS_SHIM_GMP_H
#define SXS_SHIM_GMP_H

#include "quad.h"

typedef struct { sxs_quad v; } shim_mpf_struct;
typedef shim_mpf_struct mpf_t[1];
typedef shim_mpf_struct *mpf_ptr;
typedef const shim_mpf_struct *mpf_srcptr;

static inline void mpf_init(mpf_ptr x) { x->v = 0; }
static inline void mpf_clear(mpf_ptr x) { (void)x; }
static inline void mpf_set_d(mpf_ptr x, double d) { x->v = (sxs_quad)d; }
static inline void mpf_init_set_d(mpf_ptr x, double d) { x->v = (sxs_quad)d; }
static inline void mpf_set(mpf_ptr r, mpf_srcptr a) { r->v = a->v; }
static inline void mpf_mul(mpf_ptr r, mpf_srcptr a, mpf_srcptr b) { r->v = a->v * b->v; }
static inline void mpf_mul_ui(mpf_ptr r, mpf_srcptr a, unsigned long b) { r->v = a->v * (sxs_quad)b; }
static inline void mpf_div(mpf_ptr r, mpf_srcptr a, mpf_srcptr b) { r->v = a->v / b->v; }
static inline void mpf_add(mpf_ptr r, mpf_srcptr a, mpf_srcptr b) { r->v = a->v + b->v; }
static inline void mpf_sqrt(mpf_ptr r, mpf_srcptr a) { r->v = sxs_quad_sqrt(a->v); }
static inline double mpf_get_d(mpf_srcptr a) { return sxs_quad_to_double_trunc(a->v); }

#endif
