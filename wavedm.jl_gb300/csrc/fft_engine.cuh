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
// Twiddles come from a per-N table W_N^m (m < N) built in FP64 on the host and
// rounded once to FP32.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

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
// ----------------------------------------------------------------------------
template <bool INV>
__device__ __forceinline__ void dft2(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <bool INV>
__device__ __forceinline__ void dft3(float2* v) {
  const float h = 0.86602540378443864676f;  // sqrt(3)/2
  float2 a = v[0], b = v[1], c = v[2];
  float2 s = cadd(b, c), d = csub(b, c);
  float2 m = make_float2(fmaf(-0.5f, s.x, a.x), fmaf(-0.5f, s.y, a.y));
  float2 r = mul_i<INV>(cscale(d, h));
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

// x * W8^1 (forward W8 = exp(-i pi/4))
template <bool INV>
__device__ __forceinline__ float2 w8_1(float2 a) {
  const float r = 0.70710678118654752440f;
  return INV ? make_float2(r * (a.x - a.y), r * (a.x + a.y)) : make_float2(r * (a.x + a.y), r * (a.y - a.x));
}
template <bool INV>
__device__ __forceinline__ float2 w8_3(float2 a) {
  const float r = 0.70710678118654752440f;
  return INV ? make_float2(-r * (a.x + a.y), r * (a.x - a.y)) : make_float2(r * (a.y - a.x), -r * (a.x + a.y));
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
  const float h = 0.86602540378443864676f;
  // W6^1 = (1/2, -+h), W6^2 = (-1/2, -+h)
  const float sg = INV ? 1.f : -1.f;
  b[1] = cmul(b[1], make_float2(0.5f, sg * h));
  b[2] = cmul(b[2], make_float2(-0.5f, sg * h));
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
WDM_PLAN(256, 16, 8, 8, 4)
WDM_PLAN(384, 16, 8, 8, 6)
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
template <int N, int T, int R, int NS, bool INV>
__device__ __forceinline__ void stage_compute(float2* v, const float2* __restrict__ tw, int t) {
  constexpr int NB = N / (R * T);
  static_assert(NB * R * T == N, "plan: T must divide N/R");
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    if constexpr (NS > 1) {
      const int j = t + T * i;
      const int jm = j % NS;
      constexpr int STEP = N / (NS * R);
#pragma unroll
      for (int k = 1; k < R; ++k) {
        float2 w = tw[k * jm * STEP];
        if (INV) w.y = -w.y;
        v[i * R + k] = cmul(v[i * R + k], w);
      }
    }
    dftR<R, INV>(v + i * R);
  }
}

template <int N, int T, int R, int NS, int LP>
__device__ __forceinline__ void stage_write(float2* s, const float2* v, int t, int l) {
  constexpr int NB = N / (R * T);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = t + T * i;
    const int b = (j / NS) * NS * R + (j % NS);
#pragma unroll
    for (int k = 0; k < R; ++k) s[(b + k * NS) * LP + l] = v[i * R + k];
  }
}

template <int N, int T, int R, int LP>
__device__ __forceinline__ void stage_read(const float2* s, float2* v, int t, int l) {
  constexpr int NB = N / (R * T);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = t + T * i;
#pragma unroll
    for (int k = 0; k < R; ++k) v[i * R + k] = s[(j + k * (N / R)) * LP + l];
  }
}

template <int N, int T, int LP, bool INV, int NS, int R, int... Rest>
__device__ __forceinline__ void run_stages_impl(float2* v, float2* s, const float2* tw, int t, int l) {
  stage_compute<N, T, R, NS, INV>(v, tw, t);
  if constexpr (sizeof...(Rest) > 0) {
    constexpr int RN = First<Rest...>::value;
    __syncthreads();
    stage_write<N, T, R, NS, LP>(s, v, t, l);
    __syncthreads();
    stage_read<N, T, RN, LP>(s, v, t, l);
    run_stages_impl<N, T, LP, INV, NS * R, Rest...>(v, s, tw, t, l);
  }
}

template <int N, int T, int LP, bool INV, int... Rs>
__device__ __forceinline__ void run_stages(Radices<Rs...>, float2* v, float2* s, const float2* tw, int t, int l) {
  run_stages_impl<N, T, LP, INV, 1, Rs...>(v, s, tw, t, l);
}

// Position along the line of register slot (i, k) before the first stage of
// radix R (the load pattern) or after the last stage of radix R (the store
// pattern): both are t + T i + k N/R.
template <int N, int T, int R>
__device__ __forceinline__ int slot_pos(int t, int i, int k) { return t + T * i + k * (N / R); }

// Load the twiddle table of length N into shared memory.
template <int N>
__device__ __forceinline__ void load_twiddles(float2* tw_s, const float2* __restrict__ tw_g) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw_s[i] = tw_g[i];
}

}  // namespace wdm
