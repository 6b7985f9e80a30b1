// Mixed-radix Stockham line FFTs for sm_103a.
//
// A CTA transforms L lines of length N at once.  Thread (t, l) owns line l
// (l = threadIdx.x % L, the fast lane index) and slot t in [0, T).  Between
// radix stages the line is exchanged through shared memory laid out as
// s[p * LP + l] (point-major, line-minor, LP = L + 1): a half-warp touches 16
// consecutive lines at one point, so every exchange pattern of every stage is
// bank-conflict free, and the same layout takes the coalesced row-major tiles
// of the x axis with a one-word pad.
//
// Stage s of radix R with Ns = product of the earlier radices: butterfly j in
// [0, N/R) reads x[j + k N/R], twiddles input k by W_N^{k (j mod Ns) N/(Ns R)},
// does an R-point DFT and writes y[(j/Ns) Ns R + (j mod Ns) + k Ns].  Thread t
// runs butterflies j = t + T i; every plan has T | N/R for all its radices, so
// a thread always holds E = N/T points in registers, the first stage reads
// points congruent to t (mod T) and the last stage leaves frequencies
// congruent to t (mod T) at the same register slots that a reversed-order
// plan's first stage reads: a forward transform, a pointwise k-space
// multiply and the inverse transform therefore chain in registers.
//
// Twiddles W_N^m are built in FP64 on the host and kept as FP32 (hi, lo)
// pairs, in stage-major tables (see stage_compute).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace wdm {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (forward sign) or +i (inverse sign)
template <bool INV>
__device__ __forceinline__ float2 mul_i(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ----------------------------------------------------------------------------
// small DFTs in registers (forward: exp(-2 pi i nk/R), inverse: exp(+...))
//
// The irrational butterfly constants sqrt(2)/2 and sqrt(3)/2 both round *down*
// in FP32 (2 fl(sqrt2/2)^2 = 1 - 1.4e-8), which would shrink |psi| by a fixed
// fraction at every butterfly and show up as a steady mass drift over
// thousands of steps.  They are applied as a two-term product c_hi x + c_lo x
// (c_lo = c - c_hi), leaving only the unbiased rounding of the result.
// ----------------------------------------------------------------------------
struct Const {
  static constexpr float r_hi = 0.70710678118654752440f;  // sqrt(2)/2
  static constexpr float r_lo = 1.2101617e-08f;           // sqrt(2)/2 - r_hi
  static constexpr float h_hi = 0.86602540378443864676f;  // sqrt(3)/2
  static constexpr float h_lo = 1.5543625e-08f;           // sqrt(3)/2 - h_hi
};
__device__ __forceinline__ float mul_r(float a) { return fmaf(a, Const::r_hi, a * Const::r_lo); }
__device__ __forceinline__ float mul_h(float a) { return fmaf(a, Const::h_hi, a * Const::h_lo); }

template <bool INV>
__device__ __forceinline__ void dft2(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <bool INV>
__device__ __forceinline__ void dft3(float2* v) {
  float2 a = v[0], b = v[1], c = v[2];
  float2 s = cadd(b, c), d = csub(b, c);
  float2 m = make_float2(fmaf(-0.5f, s.x, a.x), fmaf(-0.5f, s.y, a.y));
  float2 r = mul_i<INV>(make_float2(mul_h(d.x), mul_h(d.y)));
  v[0] = cadd(a, s);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2* v) {
  float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  float2 t2 = cadd(v[1], v[3]), t3 = mul_i<INV>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

// x * W8^1 and x * W8^3 (forward W8 = exp(-i pi/4))
template <bool INV>
__device__ __forceinline__ float2 w8_1(float2 a) {
  return INV ? make_float2(mul_r(a.x - a.y), mul_r(a.x + a.y)) : make_float2(mul_r(a.x + a.y), mul_r(a.y - a.x));
}
template <bool INV>
__device__ __forceinline__ float2 w8_3(float2 a) {
  return INV ? make_float2(-mul_r(a.x + a.y), mul_r(a.x - a.y)) : make_float2(mul_r(a.y - a.x), -mul_r(a.x + a.y));
}

template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  dft4<INV>(e);
  dft4<INV>(o);
  o[1] = w8_1<INV>(o[1]);
  o[2] = mul_i<INV>(o[2]);
  o[3] = w8_3<INV>(o[3]);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// 6 = 3 x 2 Cooley-Tukey: A_n2 = DFT3(x[n2], x[2+n2], x[4+n2]), B1 *= W6^k1,
// y[k1 + 3 k2] = A0[k1] + (-1)^k2 B1[k1].
template <bool INV>
__device__ __forceinline__ void dft6(float2* v) {
  float2 a[3] = {v[0], v[2], v[4]};
  float2 b[3] = {v[1], v[3], v[5]};
  dft3<INV>(a);
  dft3<INV>(b);
  // W6^1 = (1/2, -+h), W6^2 = (-1/2, -+h); sg = -1 forward, +1 inverse
  const float sg = INV ? 1.f : -1.f;
  const float2 b1 = b[1], b2 = b[2];
  b[1] = make_float2(fmaf(0.5f, b1.x, -sg * mul_h(b1.y)), fmaf(0.5f, b1.y, sg * mul_h(b1.x)));
  b[2] = make_float2(fmaf(-0.5f, b2.x, -sg * mul_h(b2.y)), fmaf(-0.5f, b2.y, sg * mul_h(b2.x)));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v[k] = cadd(a[k], b[k]);
    v[k + 3] = csub(a[k], b[k]);
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dftR(float2* v) {
  if constexpr (R == 2) dft2<INV>(v);
  else if constexpr (R == 3) dft3<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else if constexpr (R == 6) dft6<INV>(v);
  else if constexpr (R == 8) dft8<INV>(v);
  else static_assert(R == 2, "unsupported radix");
}

// ----------------------------------------------------------------------------
// plans
// ----------------------------------------------------------------------------
template <int... Rs>
struct Radices {};

template <int R0, int... Rs>
struct First { static constexpr int value = R0; };
template <int... Rs>
struct Last;
template <int R0>
struct Last<R0> { static constexpr int value = R0; };
template <int R0, int R1, int... Rs>
struct Last<R0, R1, Rs...> { static constexpr int value = Last<R1, Rs...>::value; };

// Plan<N>: threads per line T and the radix order.  Rev is the same radices in
// reverse order (used for the inverse half of a fused forward/op/inverse pass).
template <int N>
struct Plan;
#define WDM_PLAN(N_, T_, ...)                                              \
  template <>                                                              \
  struct Plan<N_> {                                                        \
    static constexpr int N = N_;                                           \
    static constexpr int T = T_;                                           \
    using Fwd = Radices<__VA_ARGS__>;                                      \
  };
WDM_PLAN(8, 1, 8)
WDM_PLAN(12, 2, 6, 2)
WDM_PLAN(16, 4, 4, 4)
WDM_PLAN(24, 2, 6, 4)
WDM_PLAN(32, 4, 8, 4)
WDM_PLAN(48, 4, 4, 4, 3)
WDM_PLAN(64, 8, 8, 8)
WDM_PLAN(96, 8, 4, 4, 6)
WDM_PLAN(128, 16, 8, 4, 4)
WDM_PLAN(192, 16, 4, 4, 4, 3)
#if defined(WDM_LINE_PLAN_T32)
WDM_PLAN(256, 32, 8, 8, 4)
WDM_PLAN(384, 32, 6, 4, 4, 4)
#else
WDM_PLAN(256, 16, 8, 8, 4)
WDM_PLAN(384, 16, 8, 8, 6)
#endif
WDM_PLAN(512, 32, 8, 8, 8)
#undef WDM_PLAN

template <class Rad>
struct Reverse;
template <>
struct Reverse<Radices<>> { using type = Radices<>; };
template <int R0, int... Rs>
struct Reverse<Radices<R0, Rs...>> {
  template <class A, int X>
  struct Append;
  template <int... As, int X>
  struct Append<Radices<As...>, X> { using type = Radices<As..., X>; };
  using type = typename Append<typename Reverse<Radices<Rs...>>::type, R0>::type;
};

template <class Rad>
struct RadInfo;
template <int... Rs>
struct RadInfo<Radices<Rs...>> {
  static constexpr int first = First<Rs...>::value;
  static constexpr int last = Last<Rs...>::value;
};

// ----------------------------------------------------------------------------
// stages
// ----------------------------------------------------------------------------
// Twiddle W = (x, y) + (z, w): FP32 nearest value plus its FP32 remainder
// from the FP64 value, so the rotation is exact up to the rounding of the
// result.  A plain FP32 table rounds each |W| slightly off 1 in a fixed way
// and the mean of those errors compounds into a mass drift step after step.
//
// The remainder terms are small, below half an ulp of the result, so they
// survive only if they are added inside an FMA whose product is not already
// on the FP32 grid: there the exact sum falls at a random place between grid
// points and the rounding keeps the correction on average.  Both components
// are therefore formed as fma(outer, fma(inner, corrections)) with the inner
// product on the y part of W.  That part must not be exactly +-1/2 (the only
// value between 0 and 1 in magnitude that cos/sin of a rational angle takes
// on the grid): a*(1/2) is exact, the correction would round away and
// |W| would act as its uncompensated FP32 value.  Entries with sin = +-1/2
// (angles of 30 degrees mod 180, present once 3 divides the length) are
// stored as i W instead, flagged in the last bit of the y remainder, and
// rotate the input by -i (forward) or +i (inverse) to match:
// a W = (-i a)(i W), a conj(W) = (i a) conj(i W).
__host__ __device__ inline float4 pack_twiddle(double c, double s) {
  float hx = (float)c, hy = (float)s;
  float lx = (float)(c - (double)hx), ly = (float)(s - (double)hy);
  unsigned flag = 0;
  if (hy == 0.5f || hy == -0.5f) {
    const float tx = hx, tl = lx;
    hx = -hy;
    lx = -ly;
    hy = tx;
    ly = tl;
    flag = 1;
  }
  unsigned bits;
  memcpy(&bits, &ly, sizeof(bits));
  bits = (bits & ~1u) | flag;  // moves the remainder by at most one of its ulps
  memcpy(&ly, &bits, sizeof(bits));
  return make_float4(hx, hy, lx, ly);
}

// ROT: the stage's table can hold flagged entries.  A stage twiddles by
// W_{NS R}^m, and sin = +-1/2 needs an angle of 30 degrees mod 180, so only
// stages with 12 | NS R can; the others skip the flag test.
template <bool ROT>
__device__ __forceinline__ float2 twiddle_mul(float2 a, float4 w, bool inv) {
  const bool rot = ROT && (__float_as_uint(w.w) & 1u) != 0;
  const float ax = rot ? (inv ? -a.y : a.y) : a.x;
  const float ay = rot ? (inv ? a.x : -a.x) : a.y;
  const float wy = inv ? -w.y : w.y, ly = inv ? -w.w : w.w;
  const float cx = fmaf(ax, w.z, -ay * ly);
  const float cy = fmaf(ax, ly, ay * w.z);
  return make_float2(fmaf(ax, w.x, fmaf(-ay, wy, cx)), fmaf(ay, w.x, fmaf(ax, wy, cy)));
}

// Tuning variant (WDM_FFT_TW_PLAIN): the stages multiply by the FP32 nearest
// twiddle alone (a plain complex product), leaving out the remainder terms.
template <bool ROT>
__device__ __forceinline__ float2 stage_twiddle_mul(float2 a, float4 w, bool inv) {
#if defined(WDM_FFT_TW_PLAIN)
  const bool rot = ROT && (__float_as_uint(w.w) & 1u) != 0;
  const float ax = rot ? (inv ? -a.y : a.y) : a.x;
  const float ay = rot ? (inv ? a.x : -a.x) : a.y;
  const float wy = inv ? -w.y : w.y;
  return make_float2(fmaf(ax, w.x, -ay * wy), fmaf(ax, wy, ay * w.x));
#else
  return twiddle_mul<ROT>(a, w, inv);
#endif
}

// Stage twiddles are laid out per stage as [jm][k-1] (jm < NS, 1 <= k < R),
// stage after stage in the plan's radix order: stage s starts at OFF = sum of
// NS (R - 1) over the earlier stages (N - 1 entries in all).  Lanes that run
// consecutive butterflies then read consecutive entries, which keeps the
// per-lane twiddle loads of the warp-per-line passes free of bank conflicts.
template <int N, int T, int R, int NS, bool INV, int OFF>
__device__ __forceinline__ void stage_compute(float2* v, const float4* __restrict__ tw, int t) {
  constexpr int NB = N / (R * T);
  static_assert(NB * R * T == N, "plan: T must divide N/R");
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    if constexpr (NS > 1) {
      const int j = t + T * i;
      const int jm = j % NS;
      const float4* w = tw + OFF + jm * (R - 1);
#pragma unroll
      for (int k = 1; k < R; ++k) v[i * R + k] = stage_twiddle_mul<(NS * R) % 12 == 0>(v[i * R + k], w[k - 1], INV);
    }
    dftR<R, INV>(v + i * R);
  }
}

// stage_compute on two lines at once, sharing each twiddle load.
template <int N, int T, int R, int NS, bool INV, int OFF>
__device__ __forceinline__ void stage_compute2(float2* va, float2* vb, const float4* __restrict__ tw, int t) {
  constexpr int NB = N / (R * T);
  static_assert(NB * R * T == N, "plan: T must divide N/R");
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    if constexpr (NS > 1) {
      const int j = t + T * i;
      const int jm = j % NS;
      const float4* w = tw + OFF + jm * (R - 1);
#pragma unroll
      for (int k = 1; k < R; ++k) {
        const float4 wk = w[k - 1];
        va[i * R + k] = stage_twiddle_mul<(NS * R) % 12 == 0>(va[i * R + k], wk, INV);
        vb[i * R + k] = stage_twiddle_mul<(NS * R) % 12 == 0>(vb[i * R + k], wk, INV);
      }
    }
    dftR<R, INV>(va + i * R);
    dftR<R, INV>(vb + i * R);
  }
}

// Host-side builder of the stage-major twiddle table of a radix order
// (W_N^m in FP64, stored as FP32 hi + lo); writes N - 1 entries.
template <int N, class TW, class F, int... Rs>
inline void fill_stage_twiddles(Radices<Rs...>, TW* out, F make) {
  const int radices[] = {Rs...};
  int ns = 1, off = 0;
  for (int R : radices) {
    for (int jm = 0; jm < ns; ++jm)
      for (int k = 1; k < R; ++k) out[off + jm * (R - 1) + (k - 1)] = make((long long)k * jm * (N / (ns * R)));
    off += ns * (R - 1);
    ns *= R;
  }
}

// Exchange writes/reads.  Line slots l >= LACT are idle (their registers hold
// don't-care values) and touch no shared memory, so a buffer with pitch LP can
// serve LACT < LP lines.
template <int N, int T, int R, int NS, int LP, int LACT = (1 << 30)>
__device__ __forceinline__ void stage_write(float2* s, const float2* v, int t, int l) {
  constexpr int NB = N / (R * T);
  if (l >= LACT) return;
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = t + T * i;
    const int b = (j / NS) * NS * R + (j % NS);
#pragma unroll
    for (int k = 0; k < R; ++k) s[(b + k * NS) * LP + l] = v[i * R + k];
  }
}

template <int N, int T, int R, int LP, int LACT = (1 << 30)>
__device__ __forceinline__ void stage_read(const float2* s, float2* v, int t, int l) {
  constexpr int NB = N / (R * T);
  if (l >= LACT) return;
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = t + T * i;
#pragma unroll
    for (int k = 0; k < R; ++k) v[i * R + k] = s[(j + k * (N / R)) * LP + l];
  }
}

template <int N, int T, int LP, bool INV, int LACT, int NS, int OFF, int R, int... Rest>
__device__ __forceinline__ void run_stages_impl(float2* v, float2* s, const float4* tw, int t, int l) {
  stage_compute<N, T, R, NS, INV, OFF>(v, tw, t);
  if constexpr (sizeof...(Rest) > 0) {
    constexpr int RN = First<Rest...>::value;
    __syncthreads();
    stage_write<N, T, R, NS, LP, LACT>(s, v, t, l);
    __syncthreads();
    stage_read<N, T, RN, LP, LACT>(s, v, t, l);
    run_stages_impl<N, T, LP, INV, LACT, NS * R, OFF + NS * (R - 1), Rest...>(v, s, tw, t, l);
  }
}

// tw: the stage-major table of this radix order
template <int N, int T, int LP, bool INV, int... Rs>
__device__ __forceinline__ void run_stages(Radices<Rs...>, float2* v, float2* s, const float4* tw, int t, int l) {
  run_stages_impl<N, T, LP, INV, (1 << 30), 1, 0, Rs...>(v, s, tw, t, l);
}

// Same with only line slots l < LACT exchanging through s.
template <int N, int T, int LP, bool INV, int LACT, int... Rs>
__device__ __forceinline__ void run_stages_act(Radices<Rs...>, float2* v, float2* s, const float4* tw, int t, int l) {
  run_stages_impl<N, T, LP, INV, LACT, 1, 0, Rs...>(v, s, tw, t, l);
}

// cp.async: 8-byte global -> shared copies that do not pass through registers
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Position along the line of register slot (i, k) before the first stage of
// radix R (the load pattern) or after the last stage of radix R (the store
// pattern): both are t + T i + k N/R.
template <int N, int T, int R>
__device__ __forceinline__ int slot_pos(int t, int i, int k) { return t + T * i + k * (N / R); }

// Load `count` entries of a (hi, lo) twiddle table into shared memory.
__device__ __forceinline__ void load_twiddles(float4* tw_s, const float4* __restrict__ tw_g, int count) {
  for (int i = threadIdx.x; i < count; i += blockDim.x) tw_s[i] = tw_g[i];
}

// Per-axis twiddle tables (N entries each, N - 1 used): the line passes'
// radix order and its reverse, then the x passes' order and its reverse.
enum { TW_LINE_FWD = 0, TW_LINE_REV = 1, TW_X_FWD = 2, TW_X_REV = 3, TW_TABLES = 4 };

}  // namespace wdm
