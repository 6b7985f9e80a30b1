// Branch-free sin/cos for the phase factors of the precise form.
#pragma once
#include <cuda_runtime.h>

namespace wdm {

// sin(h) and cos(h) for |h| <= pi/2 (the half angle of a phase reduced to
// [-pi, pi]): Taylor series to degree 13 (sin) and 12 (cos) evaluated by
// Horner's rule in FP32.  The truncation error on |h| <= pi/2 is below
// (pi/2)^15/15! < 8.1e-10 for sin and (pi/2)^14/14! < 6.0e-9 for cos, under a
// tenth of the FP32 rounding of the evaluation (about 1 ulp); the degrees
// 15/16 used before gave the same results to within that rounding.  Unlike a
// general sincosf there is no range reduction and no slow path, so it costs
// ~14 FMAs and few registers.
__device__ __forceinline__ void sincos_half(float h, float* s, float* c) {
  const float x2 = h * h;
  float ps = fmaf(x2, 1.6059043836821614599e-10f, -2.5052108385441718775e-8f);  // 1/13!, -1/11!
  ps = fmaf(x2, ps, 2.7557319223985890653e-6f);                                  // 1/9!
  ps = fmaf(x2, ps, -1.9841269841269841270e-4f);                                 // -1/7!
  ps = fmaf(x2, ps, 8.3333333333333333333e-3f);                                  // 1/5!
  ps = fmaf(x2, ps, -1.6666666666666666667e-1f);                                 // -1/3!
  *s = fmaf(h * x2, ps, h);
  float pc = fmaf(x2, 2.0876756987868098979e-9f, -2.7557319223985890653e-7f);    // 1/12!, -1/10!
  pc = fmaf(x2, pc, 2.4801587301587301587e-5f);                                  // 1/8!
  pc = fmaf(x2, pc, -1.3888888888888888889e-3f);                                 // -1/6!
  pc = fmaf(x2, pc, 4.1666666666666666667e-2f);                                  // 1/4!
  pc = fmaf(x2, pc, -0.5f);                                                      // -1/2!
  *c = fmaf(x2, pc, 1.f);
}

// (sin th, cos th) of the plain phase form: one FP32 sincosf, kept out of line.
// Inlined at every point of the unrolled kick and drift loops, its range
// reduction (with the slow path for large arguments) made those kernels about
// twice as large, and the precise form, which shares the kernels, paid for it
// in instruction-cache misses.
static __device__ __noinline__ float2 sincos_plain(float th) {
  float s, c;
  sincosf(th, &s, &c);
  return make_float2(s, c);
}

// exp(-i r) - 1 = (-2 sin^2(r/2), -2 sin(r/2) cos(r/2)) for |r| <= pi, accurate
// relative to |exp(-i r) - 1| (no cancellation for small r).
__device__ __forceinline__ float2 expm1_neg_i(float r) {
  float s, c;
  sincos_half(0.5f * r, &s, &c);
  return make_float2(-2.f * s * s, -2.f * s * c);
}

}  // namespace wdm
