// x-axis (contiguous rows) passes, one lane group per row pair.
//
// A lane group is T = Plan<N>::T consecutive lanes of a warp (T divides 32).
// It owns a pair of rows (A, B) = (2p, 2p+1): it transforms row A, then row
// B, each straight from and back to global memory (lane t touches points
// t + T m, so every access is a coalesced run along x), and transforms the
// two real rows of the density / potential together as the complex line
// A + iB.  Exchanges between radix stages go through the group's own shared
// buffer (padded or swizzled per stage boundary, xaddr) with __syncwarp only:
// no CTA-wide barrier after the twiddle table is loaded, so warps run
// independently and hide each other's latency.
#pragma once
#include "passes.cuh"

// resident CTAs per SM the x passes are compiled for (registers per thread
// = 65536 / (128 threads x WDM_X_MINB))
#ifndef WDM_X_MINB
#define WDM_X_MINB 4
#endif
// largest points per lane at which the adjoint kick loads the lam and pre
// rows of its pair ahead into registers (0: never)
#ifndef WDM_ADJ_PF
#define WDM_ADJ_PF 8
#endif

namespace wdm {

// Exchange buffer addressing: point p of a group lives at word base +
// xaddr(p, code), with a map chosen per stage boundary at compile time by
// simulating the shared-memory banks of that boundary's write pattern (the
// Stockham scatter of radix R at stride NS) and the next stage's read pattern
// for the 32 lanes of a warp (8-byte words, 16 lanes per wavefront).  The
// candidates are a padding p + (p >> s) (code s = 2..6; 30: none) and an XOR
// swizzle of W bits at bit B by the W bits at bit A >= B + W,
// p ^ (((p >> A) & (2^W - 1)) << B) (code 100 + 100 (A - B - W) + 10 W + B),
// which permutes p within its aligned block of 2^(B + W) words and so needs
// no room beyond the line.
__host__ __device__ constexpr int xaddr(int p, int code) {
  if (code < 100) return p + (p >> code);
  const int b = code % 10, w = (code / 10) % 10, a = b + w + (code - 100) / 100;
  return p ^ (((p >> a) & ((1 << w) - 1)) << b);
}

// Largest number of distinct words that share a bank pair among 16 lane
// addresses (8-byte words: bank pair = word mod 16).
__host__ __device__ constexpr int xbank_degree16(const int* a) {
  int cnt[16] = {};
  for (int y = 0; y < 16; ++y) {
    bool first = true;
    for (int z = 0; z < y; ++z)
      if (a[z] == a[y]) first = false;
    if (first) ++cnt[a[y] & 15];
  }
  int worst = 1;
  for (int b = 0; b < 16; ++b)
    if (cnt[b] > worst) worst = cnt[b];
  return worst;
}

template <int N, int T, int NP>
struct XPad {
  __host__ __device__ static constexpr int cost(int R, int NS, int RN, int code) {
    int total = 0;
    for (int i = 0; i < N / (R * T); ++i)
      for (int k = 0; k < R; ++k)
        for (int half = 0; half < 2; ++half) {
          int a[16] = {};
          for (int q = 0; q < 16; ++q) {
            const int lane = half * 16 + q, g = lane / T, t = lane % T, j = t + T * i;
            const int p = (j / NS) * NS * R + (j % NS) + k * NS;
            a[q] = g * NP + xaddr(p, code);
          }
          total += xbank_degree16(a);
        }
    for (int i = 0; i < N / (RN * T); ++i)
      for (int k = 0; k < RN; ++k)
        for (int half = 0; half < 2; ++half) {
          int a[16] = {};
          for (int q = 0; q < 16; ++q) {
            const int lane = half * 16 + q, g = lane / T, t = lane % T, j = t + T * i;
            const int p = j + k * (N / RN);
            a[q] = g * NP + xaddr(p, code);
          }
          total += xbank_degree16(a);
        }
    return total;
  }
};

// Candidate maps in order of preference on a tie: no padding, the paddings
// s = 6..2 that fit below NP words, the swizzles (A - B - W = 0..3, then
// W = 2, 3, 1, then B = 0..3).  A candidate that does not apply stands in as
// no padding.
constexpr int XCAND = 1 + 5 + 48;
template <int N, int NP>
__host__ __device__ constexpr int xcand(int i) {
  if (i == 0) return 30;
  if (i <= 5) {
    const int sh = 7 - i;
    return xaddr(N - 1, sh) < NP ? sh : 30;
  }
  const int j = i - 6, gap = j / 12, w = (j / 4) % 3 == 2 ? 1 : 2 + (j / 4) % 3, b = j % 4;
  return N % (1 << (b + w)) == 0 ? 100 + 100 * gap + 10 * w + b : 30;
}

// Each candidate's cost is its own constant evaluation (one search over all of
// them would exceed the compiler's budget for a single evaluation).
template <int N, int T, int NP, int R, int NS, int RN, int CODE>
struct XCost {
  static constexpr int value = XPad<N, T, NP>::cost(R, NS, RN, CODE);
};

template <int N, int T, int NP, int R, int NS, int RN, int I = 0>
struct XBest {
  using Rest = XBest<N, T, NP, R, NS, RN, I + 1>;
  static constexpr int here = xcand<N, NP>(I);
  static constexpr int here_cost = XCost<N, T, NP, R, NS, RN, here>::value;
  static constexpr int code = here_cost <= Rest::cost ? here : Rest::code;
  static constexpr int cost = here_cost <= Rest::cost ? here_cost : Rest::cost;
};
template <int N, int T, int NP, int R, int NS, int RN>
struct XBest<N, T, NP, R, NS, RN, XCAND> {
  static constexpr int code = 30;
  static constexpr int cost = 1 << 30;
};

// The map of one stage boundary (group buffers NP words apart).
template <int N, int T, int NP, int R, int NS, int RN>
struct XMap {
  static constexpr int code = XBest<N, T, NP, R, NS, RN>::code;
};

// Words one group's exchange buffer needs for the maps of the stage
// boundaries from stride NS on (NP0: the row pitch the maps were chosen with).
template <int N, int T, int NP0, int NS, int R, int... Rest>
__host__ __device__ constexpr int xextent_from() {
  if constexpr (sizeof...(Rest) == 0) {
    return N;
  } else {
    constexpr int code = XMap<N, T, NP0, R, NS, First<Rest...>::value>::code;
    constexpr int here = code < 100 ? xaddr(N - 1, code) + 1 : N;
    constexpr int rest = xextent_from<N, T, NP0, NS * R, Rest...>();
    return here > rest ? here : rest;
  }
}
template <int N, int T, int NP0, int... Rs>
__host__ __device__ constexpr int xextent(Radices<Rs...>) {
  return xextent_from<N, T, NP0, 1, Rs...>();
}

template <int N, int T, int R, int NS, int CODE>
__device__ __forceinline__ void wstage_write(float2* b, const float2* v, int t) {
  constexpr int NB = N / (R * T);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = t + T * i;
    const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
    for (int k = 0; k < R; ++k) b[xaddr(base + k * NS, CODE)] = v[i * R + k];
  }
}

template <int N, int T, int R, int CODE>
__device__ __forceinline__ void wstage_read(const float2* b, float2* v, int t) {
  constexpr int NB = N / (R * T);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = t + T * i;
#pragma unroll
    for (int k = 0; k < R; ++k) v[i * R + k] = b[xaddr(j + k * (N / R), CODE)];
  }
}

template <int N, int T, int NP, bool INV, int NS, int OFF, int R, int... Rest>
__device__ __forceinline__ void run_wstages_impl(float2* v, float2* b, const float4* tw, int t) {
  stage_compute<N, T, R, NS, INV, OFF>(v, tw, t);
  if constexpr (sizeof...(Rest) > 0) {
    constexpr int RN = First<Rest...>::value;
    constexpr int CODE = XMap<N, T, NP, R, NS, RN>::code;
    __syncwarp();
    wstage_write<N, T, R, NS, CODE>(b, v, t);
    __syncwarp();
    wstage_read<N, T, RN, CODE>(b, v, t);
    run_wstages_impl<N, T, NP, INV, NS * R, OFF + NS * (R - 1), Rest...>(v, b, tw, t);
  }
}

// tw: the stage-major table of this radix order; b: the group's buffer (NP words)
template <int N, int T, int NP, bool INV, int... Rs>
__device__ __forceinline__ void run_wstages(Radices<Rs...>, float2* v, float2* b, const float4* tw, int t) {
  run_wstages_impl<N, T, NP, INV, 1, 0, Rs...>(v, b, tw, t);
}

// Two rows through the same stages side by side (row A exchanging through ba,
// row B through bb): each twiddle is loaded once for both rows and each stage
// boundary costs one pair of warp barriers, with two independent chains of
// arithmetic in flight.
template <int N, int T, int NP, bool INV, int NS, int OFF, int R, int... Rest>
__device__ __forceinline__ void run_wstages2_impl(float2* va, float2* vb, float2* ba, float2* bb, const float4* tw,
                                                  int t) {
  stage_compute2<N, T, R, NS, INV, OFF>(va, vb, tw, t);
  if constexpr (sizeof...(Rest) > 0) {
    constexpr int RN = First<Rest...>::value;
    constexpr int CODE = XMap<N, T, NP, R, NS, RN>::code;
    __syncwarp();
    wstage_write<N, T, R, NS, CODE>(ba, va, t);
    wstage_write<N, T, R, NS, CODE>(bb, vb, t);
    __syncwarp();
    wstage_read<N, T, RN, CODE>(ba, va, t);
    wstage_read<N, T, RN, CODE>(bb, vb, t);
    run_wstages2_impl<N, T, NP, INV, NS * R, OFF + NS * (R - 1), Rest...>(va, vb, ba, bb, tw, t);
  }
}

template <int N, int T, int NP, bool INV, int... Rs>
__device__ __forceinline__ void run_wstages2(Radices<Rs...>, float2* va, float2* vb, float2* ba, float2* bb,
                                             const float4* tw, int t) {
  run_wstages2_impl<N, T, NP, INV, 1, 0, Rs...>(va, vb, ba, bb, tw, t);
}

// Register slot q = i R + k holds point slot_pos<R>(t, i, k) = t + T (i + k N/(R T)).
// reorder<RA, RB>: registers positioned for radix RA -> positioned for RB
// (the same set of points t + T m, only the slot order differs).
template <int N, int T, int RA, int RB>
__device__ __forceinline__ void reorder(const float2* a, float2* b) {
  constexpr int MA = N / (RA * T), MB = N / (RB * T);
#pragma unroll
  for (int ib = 0; ib < MB; ++ib)
#pragma unroll
    for (int kb = 0; kb < RB; ++kb) {
      const int m = ib + kb * MB;      // point t + T m
      const int ia = m % MA, ka = m / MA;
      b[ib * RB + kb] = a[ia * RA + ka];
    }
}

// Plans of the x passes: lanes per line T (dividing 32) and radix order.  A
// full warp per line where the radices allow it keeps the points per lane
// (and so the registers) low.
template <int N>
struct XPlan : Plan<N> {};
template <>
struct XPlan<256> {
  static constexpr int N = 256, T = 32;
  using Fwd = Radices<8, 8, 4>;
};
// 384 = 4 4 4 6: the strides NS = 1, 4, 16, 64 of the stages are powers of two,
// so each lane's exchange addresses (j / NS, j % NS of j = t + 32 i) cost
// shifts and masks; the order 6 4 4 4 (NS = 1, 6, 24, 96) costs a division by
// a constant per point and exchange, and measured 8% slower in the density pass.
template <>
struct XPlan<384> {
#if defined(WDM_X384_T16)
  // tuning variant: 16 lanes per row, 24 points per lane, two exchanges
  static constexpr int N = 384, T = 16;
  using Fwd = Radices<8, 8, 6>;
#elif defined(WDM_X384_ORDER_6444)
  // the order 6 4 4 4, for comparison
  static constexpr int N = 384, T = 32;
  using Fwd = Radices<6, 4, 4, 4>;
#else
  static constexpr int N = 384, T = 32;
  using Fwd = Radices<4, 4, 4, 6>;
#endif
};

// Group pitch of the exchange buffers where a warp holds several groups: the
// pitch in N .. N + N/4 + 1 with the lowest total bank cost over the plan's
// stage boundaries, each with its best map (a search over those pitches with
// the bank simulation of XPad; every listed plan is conflict-free with it).
// Other sizes take N + N/4 + 1.
template <int N>
struct XPitch {
  static constexpr int value = N + N / 4 + 1;
};
template <> struct XPitch<12> { static constexpr int value = 14; };
template <> struct XPitch<16> { static constexpr int value = 20; };
template <> struct XPitch<24> { static constexpr int value = 26; };
template <> struct XPitch<32> { static constexpr int value = 36; };
template <> struct XPitch<48> { static constexpr int value = 52; };
template <> struct XPitch<64> { static constexpr int value = 72; };
template <> struct XPitch<96> { static constexpr int value = 104; };

template <int N>
struct XCfg {
  static constexpr int T = XPlan<N>::T;
  static_assert(32 % T == 0, "x pass: threads per line must divide the warp");
  static constexpr int GROUPS = 32 / T;                // row pairs per warp
  static constexpr int WARPS = 4;                      // warps per CTA
  static constexpr int NT = 32 * WARPS;
  // exchange buffer per group: with one group per warp only the maps' room
  // (xextent); with several, the pitch XPitch, which the maps are chosen for
  static constexpr int NP0 = N + N / 4 + 1;
  static constexpr int NP = GROUPS == 1 ? xextent<N, T, NP0>(typename XPlan<N>::Fwd{}) : XPitch<N>::value;
#if defined(WDM_XTW_GLOBAL)
  static constexpr size_t TW_BYTES = 0;  // twiddles read from global memory (L1), not staged
#else
  static constexpr size_t TW_BYTES = sizeof(float4) * N;  // the forward-order table (both directions)
#endif
  static constexpr size_t SMEM = TW_BYTES + sizeof(float2) * (size_t)NP * GROUPS * WARPS;
};

// Work distribution: warp-units of GROUPS row pairs, grid-stride over all
// batch items; every lane of a warp runs the same number of iterations.
struct XWork {
  int pairs_per_item;   // nrows / 2
  int batch;
  __device__ __forceinline__ long long units(int groups) const {
    return ((long long)pairs_per_item * batch + groups - 1) / groups;
  }
};

// Packed potential line of rows (A, B) from their half spectra, loaded at the
// register slots of radix R: Z[p] = A[p] + i B[p], Z[N-p] = conj A[p] + i conj B[p].
template <int N, int T, int R>
__device__ __forceinline__ void load_packed_half(float2* v, const float2* __restrict__ ha,
                                                 const float2* __restrict__ hb, bool ok, int t) {
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int p = slot_pos<N, T, R>(t, i, k);
      const int q = p <= N / 2 ? p : N - p;
      float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
      if (ok) {
        a = ha[q];
        b = hb[q];
      }
      v[i * R + k] = p <= N / 2 ? make_float2(a.x - b.y, a.y + b.x) : make_float2(a.x + b.y, b.x - a.y);
    }
}

// Hermitian split of the packed forward transform (registers at radix-R slots)
// into the half spectra of rows A and B (k = 0..N/2), via the group buffer.
template <int N, int T, int R>
__device__ __forceinline__ void store_packed_half(const float2* v, float2* buf, float2* __restrict__ ha,
                                                  float2* __restrict__ hb, bool ok, int t) {
  __syncwarp();
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) buf[slot_pos<N, T, R>(t, i, k)] = v[i * R + k];
  __syncwarp();
  if (!ok) return;
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int p = slot_pos<N, T, R>(t, i, k);
      if (p > N / 2) continue;
      const float2 zk = v[i * R + k];
      const float2 zn = buf[(N - p) % N];
      ha[p] = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
      hb[p] = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
    }
}

// The x twiddle table of the forward radix order (N entries), which every
// x-pass transform uses in both directions: staged in shared memory, or
// (WDM_XTW_GLOBAL, a tuning variant) read through L1 from global memory.
#if defined(WDM_XTW_GLOBAL)
#define WDM_XPASS_TWIDDLES const float4* tw = twg + TW_X_FWD * N;
#else
#define WDM_XPASS_TWIDDLES                                   \
  float4* tw = reinterpret_cast<float4*>(smem);              \
  load_twiddles(tw, twg + TW_X_FWD * N, N);                  \
  __syncthreads();
#endif

#define WDM_XPASS_PROLOGUE                                                          \
  using C = XCfg<N>;                                                                \
  constexpr int T = C::T;                                                           \
  using Rad = typename XPlan<N>::Fwd;                                               \
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;                  \
  (void)R1;                                                                         \
  (void)RS;                                                                         \
  extern __shared__ float2 smem[];                                                  \
  WDM_XPASS_TWIDDLES                                                                \
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;                       \
  const int g = lane / T, t = lane % T;                                             \
  float2* buf = smem + C::TW_BYTES / sizeof(float2) + (size_t)(warp * C::GROUPS + g) * C::NP; \
  const long long nunits = w.units(C::GROUPS);                                      \
  const long long wstride = (long long)gridDim.x * C::WARPS;

// ----------------------------------------------------------------------------
// P1: Phi rows from H (C2R of the packed pair), kick, forward x-FFT (or not)
// ----------------------------------------------------------------------------
// The kick of one row: v holds psi row r at radix-R slots (R: the last radix
// of the x plan, where the potential's C2R leaves it), phi its potential at the
// same slots; v <- v exp(-i dt pot).
template <int N, int R1 = RadInfo<typename XPlan<N>::Fwd>::last>
__device__ __forceinline__ void kick_points(float2* v, float* phi, const float* T6, const KickArgs& a,
                                            const RowGeom& rg, int r, int b, bool ok, int t) {
  using C = XCfg<N>;
  constexpr int T = C::T;
  const float* vrow = a.V ? a.V + b * a.v_bstride + (long long)r * rg.pitch : nullptr;
  const int y = r % rg.ny, z = r / rg.ny;
  // coordinates in the tide's frame (T6[6..8]: cell 0's, T6[9]: constant)
  const float fy = T6[7] + a.dy * y, fz = T6[8] + a.dz * z;
  // 1/2 x^T T x = 1/2 Txx x^2 + Txy x y + Txz x z + (1/2 Tyy y^2 + Tyz y z + 1/2 Tzz z^2) + C
  const float cyz = 0.5f * T6[1] * fy * fy + T6[5] * fy * fz + 0.5f * T6[2] * fz * fz + T6[9];
  const float lin = T6[3] * fy + T6[4] * fz;
  // The potential is completed in phi (which the caller gives up), each
  // optional term tested once for the row's points and added in the same
  // order at every point; the phase form is chosen once as well, so that the
  // loop of the precise form holds no call of the plain form's out-of-line
  // sincos.  Per-point tests had kept the compiler from interleaving the
  // points' arithmetic: this took the kick from 276 M to 244 M warp
  // instructions and from 0.337 to 0.288 ms at 384^3.
  constexpr int NQ = N / T;
  if (a.tidal) {
#pragma unroll
    for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
      for (int k = 0; k < R1; ++k) {
        const float fx = T6[6] + a.dx * slot_pos<N, T, R1>(t, i, k);
        phi[i * R1 + k] += fmaf(fx, fmaf(0.5f * T6[0], fx, lin), cyz);
      }
  }
  if (a.kerr != 0.f) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) phi[q] = fmaf(a.kerr, fmaf(v[q].x, v[q].x, v[q].y * v[q].y), phi[q]);
  }
  if (vrow && ok) {
#pragma unroll
    for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
      for (int k = 0; k < R1; ++k) phi[i * R1 + k] += vrow[slot_pos<N, T, R1>(t, i, k)];
  }
  if (a.precise) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = kick_by_t<true>(v[q], kick_factor_t<true>(phi[q], a));
  } else {
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = kick_by_t<false>(v[q], kick_factor_t<false>(phi[q], a));
  }
}

// Store a row held at radix-R slots (when ok).
template <int N, int R>
__device__ __forceinline__ void store_row(float2* row, const float2* v, bool ok, int t) {
  constexpr int T = XCfg<N>::T;
  if (!ok) return;
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) row[slot_pos<N, T, R>(t, i, k)] = v[i * R + k];
}

// One row of the kick pass: v holds psi row r at radix-RS slots (where the
// potential's C2R leaves phi); kick, then (FWD) the forward x transform, whose
// first stage wants radix-R1 slots (a renaming of the same registers), and
// store to `row` (when ok).
template <int N, bool FWD>
__device__ __forceinline__ void kick_row(float2* v, float* phi, const float* T6, const KickArgs& a,
                                         const RowGeom& rg, int r, int b, bool ok, float2* row, float2* buf,
                                         const float4* tw, int t) {
  using C = XCfg<N>;
  constexpr int T = C::T;
  using Rad = typename XPlan<N>::Fwd;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  kick_points<N, RS>(v, phi, T6, a, rg, r, b, ok, t);
  if constexpr (FWD) {
    float2 w[N / T];
    reorder<N, T, RS, R1>(v, w);
    run_wstages<N, T, C::NP, false>(Rad{}, w, buf, tw, t);
    store_row<N, RS>(row, w, ok, t);
  } else {
    store_row<N, RS>(row, v, ok, t);
  }
}

// Tidal tensor of batch item b in T6[0..5] and the tide's frame in T6[6..9]
// (cell-0 coordinates and a constant; the box centre and 0 without a frame).
template <int N>
__device__ __forceinline__ void kick_tidal(float* T6, const KickArgs& a, const RowGeom&, int b) {
#pragma unroll
  for (int q = 0; q < 6; ++q) T6[q] = a.T6b ? a.T6b[b * 6 + q] : a.T6[q];
  if (a.frame) {
#pragma unroll
    for (int q = 0; q < 4; ++q) T6[6 + q] = a.frame[4 * b + q];
  } else {
    T6[6] = a.x0;
    T6[7] = a.y0;
    T6[8] = a.z0;
    T6[9] = 0.f;
  }
}

// Density maximum and first moments of one row pair, per lane (CentreWords).
struct CentreAcc {
  float best;      // largest rho seen (-1: none)
  unsigned cell;   // its flat cell index in the item
  float s0[2];     // sum of rho of rows A and B
  float si;        // sum of rho i (i the x index) over both rows
  __device__ __forceinline__ void reset() {
    best = -1.f;
    cell = 0xffffffffu;
    s0[0] = s0[1] = si = 0.f;
  }
  __device__ __forceinline__ void add(float d, unsigned c, int i, int half) {
    if (d > best || (d == best && c < cell)) {
      best = d;
      cell = c;
    }
    s0[half] += d;
    si = fmaf(d, (float)i, si);
  }
};

// Per lane group: the pair sums carried in FP64 over the units a group runs,
// written to the item's words when the item changes and at the end.
struct CentreSum {
  double s0, si, sj, sk;
  unsigned long long key;
  int item;
  __device__ __forceinline__ void reset(int b) {
    s0 = si = sj = sk = 0.0;
    key = 0ull;
    item = b;
  }
  __device__ __forceinline__ void flush(unsigned long long* words) const {
    if (item < 0) return;
    unsigned long long* w = words + (long long)CENTRE_WORDS * item;
    atomicMax(w, key);
    atomicAdd(reinterpret_cast<double*>(w + 1), s0);
    atomicAdd(reinterpret_cast<double*>(w + 2), si);
    atomicAdd(reinterpret_cast<double*>(w + 3), sj);
    atomicAdd(reinterpret_cast<double*>(w + 4), sk);
  }
};

// The row pair (ra, ra + 1) of item b is done: reduce its lanes' CentreAcc over
// the lane group (T lanes) and add it to the group's CentreSum (on lane t = 0).
template <int N>
__device__ __forceinline__ void centre_pair_done(const RhoArgs& a, const RowGeom& rg, const CentreAcc& ca,
                                                 CentreSum& cs, int b, int ra, bool ok, int t) {
  constexpr int T = XCfg<N>::T;
  float best = ca.best, s0a = ca.s0[0], s0b = ca.s0[1], si = ca.si;
  unsigned cell = ca.cell;
#pragma unroll
  for (int off = T / 2; off > 0; off >>= 1) {
    const float ob = __shfl_xor_sync(0xffffffffu, best, off, T);
    const unsigned oc = __shfl_xor_sync(0xffffffffu, cell, off, T);
    if (ob > best || (ob == best && oc < cell)) {
      best = ob;
      cell = oc;
    }
    s0a += __shfl_xor_sync(0xffffffffu, s0a, off, T);
    s0b += __shfl_xor_sync(0xffffffffu, s0b, off, T);
    si += __shfl_xor_sync(0xffffffffu, si, off, T);
  }
  if (t != 0 || !ok) return;
  if (cs.item != b) {
    cs.flush(a.centre);
    cs.reset(b);
  }
  const int ja = ra % rg.ny, ka = ra / rg.ny, jb = (ra + 1) % rg.ny, kb = (ra + 1) / rg.ny;
  cs.s0 += (double)s0a + (double)s0b;
  cs.si += (double)si;
  cs.sj += (double)s0a * ja + (double)s0b * jb;
  cs.sk += (double)s0a * ka + (double)s0b * kb;
  if (best >= 0.f) {
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(best) << 32) | (unsigned long long)(0xffffffffu - cell);
    if (key > cs.key) cs.key = key;
  }
}

// The slice of an x pass one warp runs: warp units u0, u0 + ustride, ...,
// with the twiddle tables of the pass (x fwd | x rev) in shared memory at tw
// and this lane group's exchange buffer (XCfg<N>::NP entries) at buf.
struct XSlice {
  long long u0, ustride;
  const float4* tw;
  float2* buf;
};

template <int N, bool FWD>
__device__ __forceinline__ void xw_kick_units(const float2* psi_in, float2* psi, const float2* __restrict__ H,
                                              const RowGeom& rg, long long hpitch, long long hbstride,
                                              const KickArgs& a, const XWork& w, const XSlice& sl) {
  using C = XCfg<N>;
  constexpr int T = C::T;
  using Rad = typename XPlan<N>::Fwd;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  const int lane = threadIdx.x & 31, g = lane / T, t = lane % T;
  const float4* tw = sl.tw;
  float2* buf = sl.buf;
  const long long nunits = w.units(C::GROUPS);
  for (long long u = sl.u0; u < nunits; u += sl.ustride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
    const float2* hrow = H + b * hbstride + ra * hpitch;
    float2 v[N / T];
    load_packed_half<N, T, R1>(v, hrow, hrow + hpitch, ok, t);
    run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);  // ends with radix RS
    float phi[2][N / T];
#pragma unroll
    for (int q = 0; q < N / T; ++q) {
      phi[0][q] = v[q].x;
      phi[1][q] = v[q].y;
    }
    float T6[10];
    kick_tidal<N>(T6, a, rg, b);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int r = ra + half;
      const float2* irow = psi_in + b * rg.bstride + (long long)r * rg.pitch;
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k) v[i * RS + k] = ok ? irow[slot_pos<N, T, RS>(t, i, k)] : make_float2(0.f, 0.f);
      kick_row<N, FWD>(v, phi[half], T6, a, rg, r, b, ok, psi + b * rg.bstride + (long long)r * rg.pitch, buf, tw, t);
    }
  }
}

template <int N, bool FWD>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_kick(const float2* psi_in, float2* psi, const float2* __restrict__ H, RowGeom rg, long long hpitch,
          long long hbstride, const float4* __restrict__ twg, KickArgs a, XWork w) {
  // psi_in == psi runs in place; a separate psi_in keeps the input state
  WDM_XPASS_PROLOGUE
  (void)nunits;
  (void)t;
  xw_kick_units<N, FWD>(psi_in, psi, H, rg, hpitch, hbstride, a, w,
                        XSlice{(long long)blockIdx.x * C::WARPS + warp, wstride, tw, buf});
}

// ----------------------------------------------------------------------------
// P5: psi x-inverse (+mask) of rows A and B, rho = |psi|^2 (+rho_b) - shift,
// packed R2C of (rho_A, rho_B) -> H rows A and B
// ----------------------------------------------------------------------------
// The part of a P5 row after its inverse transform: v holds psi row r in real
// space at radix-RS slots; mask it and store it back to `row` (write_psi), then
// form rho - shift into rho0 (half 0) or the packed z (half 1).  rb: the
// baryon density row or null.
template <int N, bool CEN>
__device__ __forceinline__ void rho_row_post(float2* v, const RhoArgs& a, const RowGeom& rg, int r, bool ok,
                                             float2* row, const float* rb, float shift, int half, float* rho0,
                                             float2* z, int t, CentreAcc& ca) {
  constexpr int T = XCfg<N>::T;
  constexpr int RS = RadInfo<typename XPlan<N>::Fwd>::last;
  if (a.write_psi) {
    if (a.mx) {
      const int y = r % rg.ny, zz = r / rg.ny;
      const float myz = ok ? a.my[y] * a.mz[zz] : 0.f;
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k) v[i * RS + k] = cscale(v[i * RS + k], myz * a.mx[slot_pos<N, T, RS>(t, i, k)]);
    }
    store_row<N, RS>(row, v, ok, t);
  }
  // The density is formed in place (rho0 for row A, the y parts of z for
  // row B), each optional step tested once for the row's points.
  constexpr int NQ = N / T;
  auto d = [&](int q) -> float& { return half == 0 ? rho0[q] : z[q].y; };
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    if (half != 0) z[q].x = rho0[q];
    d(q) = fmaf(v[q].x, v[q].x, v[q].y * v[q].y);
  }
  if (ok && a.nonfinite) {
    bool bad = false;
#pragma unroll
    for (int q = 0; q < NQ; ++q) bad |= !isfinite(d(q));
    if (bad) *a.nonfinite = 1;
  }
  if constexpr (CEN) {
#pragma unroll
    for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
      for (int k = 0; k < RS; ++k) {
        const int x = slot_pos<N, T, RS>(t, i, k);
        ca.add(d(i * RS + k), (unsigned)r * (unsigned)N + (unsigned)x, x, half);
      }
  }
  if (rb && ok) {
#pragma unroll
    for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
      for (int k = 0; k < RS; ++k) d(i * RS + k) += rb[slot_pos<N, T, RS>(t, i, k)];
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) d(q) -= shift;
}

// One row of P5: v holds psi row r (write_psi: x-spectral at radix-R1 slots,
// else real space at radix-RS slots).  Inverts it (write_psi), then
// rho_row_post.
template <int N, bool CEN>
__device__ __forceinline__ void inv_rho_row(float2* v, const RhoArgs& a, const RowGeom& rg, int r, bool ok,
                                            float2* row, const float* rb, float shift, int half, float* rho0,
                                            float2* z, float2* buf, const float4* tw, int t, CentreAcc& ca) {
  using C = XCfg<N>;
  if (a.write_psi) run_wstages<N, C::T, C::NP, true>(typename XPlan<N>::Fwd{}, v, buf, tw, t);
  rho_row_post<N, CEN>(v, a, rg, r, ok, row, rb, shift, half, rho0, z, t, ca);
}

template <int N, bool CEN>
__device__ __forceinline__ void xw_inv_rho_units(float2* __restrict__ psi, float2* __restrict__ H, const RowGeom& rg,
                                                 long long hpitch, long long hbstride, const RhoArgs& a,
                                                 const XWork& w, const XSlice& sl) {
  using C = XCfg<N>;
  constexpr int T = C::T;
  using Rad = typename XPlan<N>::Fwd;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  const int lane = threadIdx.x & 31, g = lane / T, t = lane % T;
  const float4* tw = sl.tw;
  float2* buf = sl.buf;
  const long long nunits = w.units(C::GROUPS);
  CentreSum cs;
  cs.reset(-1);
  for (long long u = sl.u0; u < nunits; u += sl.ustride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
    const float shift = a.shift ? a.shift[b] : 0.f;
    float rho0[N / T];  // row A density at radix-RS slots
    float2 z[N / T];    // packed (rho_A, rho_B) at radix-RS slots
    float2 v[N / T];
    CentreAcc ca;
    ca.reset();
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int r = ra + half;
      float2* row = psi + b * rg.bstride + (long long)r * rg.pitch;
      if (a.write_psi) {
#pragma unroll
        for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
          for (int k = 0; k < R1; ++k) v[i * R1 + k] = ok ? row[slot_pos<N, T, R1>(t, i, k)] : make_float2(0.f, 0.f);
      } else {
#pragma unroll
        for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
          for (int k = 0; k < RS; ++k) v[i * RS + k] = ok ? row[slot_pos<N, T, RS>(t, i, k)] : make_float2(0.f, 0.f);
      }
      const bool rb_row = a.rho_b && (!a.rb_rows || a.rb_rows[r]);  // rows without baryon mass are zero
      const float* rb = rb_row ? a.rho_b + b * a.rb_bstride + (long long)r * rg.pitch : nullptr;
      inv_rho_row<N, CEN>(v, a, rg, r, ok, row, rb, shift, half, rho0, z, buf, tw, t, ca);
    }
    if constexpr (CEN) centre_pair_done<N>(a, rg, ca, cs, b, ra, ok, t);
    reorder<N, T, RS, R1>(z, v);
    run_wstages<N, T, C::NP, false>(Rad{}, v, buf, tw, t);
    float2* hrow = H + b * hbstride + ra * hpitch;
    store_packed_half<N, T, RS>(v, buf, hrow, hrow + hpitch, ok, t);
  }
  if (CEN && t == 0) cs.flush(a.centre);
}

// CEN: also accumulate the density maximum and moments for the tide's frame
// (RhoArgs::centre), a compile-time choice so that the pass without it keeps
// its registers and instructions.
template <int N, bool CEN>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_inv_rho(float2* __restrict__ psi, float2* __restrict__ H, RowGeom rg, long long hpitch, long long hbstride,
             const float4* __restrict__ twg, RhoArgs a, XWork w) {
  WDM_XPASS_PROLOGUE
  (void)nunits;
  (void)t;
  xw_inv_rho_units<N, CEN>(psi, H, rg, hpitch, hbstride, a, w,
                           XSlice{(long long)blockIdx.x * C::WARPS + warp, wstride, tw, buf});
}

// Plain C2C x pass (rows processed pairwise, scaled output).
template <int N, bool INV>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_fft(float2* __restrict__ data, RowGeom rg, const float4* __restrict__ twg, float scale, XWork w) {
  WDM_XPASS_PROLOGUE
  for (long long u = (long long)blockIdx.x * C::WARPS + warp; u < nunits; u += wstride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float2* row = data + b * rg.bstride + (long long)(ra + half) * rg.pitch;
      float2 v[N / T];
#pragma unroll
      for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
        for (int k = 0; k < R1; ++k) v[i * R1 + k] = ok ? row[slot_pos<N, T, R1>(t, i, k)] : make_float2(0.f, 0.f);
      run_wstages<N, T, C::NP, INV>(Rad{}, v, buf, tw, t);
      if (ok)
#pragma unroll
        for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
          for (int k = 0; k < RS; ++k) row[slot_pos<N, T, RS>(t, i, k)] = cscale(v[i * RS + k], scale);
    }
  }
}

// Phi rows (real) from H: packed C2R only.
template <int N>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_c2r(const float2* __restrict__ H, float* __restrict__ out, RowGeom rg, long long hpitch, long long hbstride,
         const float4* __restrict__ twg, XWork w) {
  WDM_XPASS_PROLOGUE
  for (long long u = (long long)blockIdx.x * C::WARPS + warp; u < nunits; u += wstride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
    const float2* hrow = H + b * hbstride + ra * hpitch;
    float2 v[N / T];
    load_packed_half<N, T, R1>(v, hrow, hrow + hpitch, ok, t);
    run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);
    if (!ok) continue;
    float* oa = out + b * rg.bstride + (long long)ra * rg.pitch;
#pragma unroll
    for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
      for (int k = 0; k < RS; ++k) {
        const int x = slot_pos<N, T, RS>(t, i, k);
        oa[x] = v[i * RS + k].x;
        oa[rg.pitch + x] = v[i * RS + k].y;
      }
  }
}

// Real rows -> H (packed R2C) from a float field, minus a per-item shift.
template <int N>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_r2c(const float* __restrict__ in, float2* __restrict__ H, RowGeom rg, long long hpitch, long long hbstride,
         const float4* __restrict__ twg, const float* __restrict__ shift_b, XWork w) {
  WDM_XPASS_PROLOGUE
  for (long long u = (long long)blockIdx.x * C::WARPS + warp; u < nunits; u += wstride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
    const float shift = shift_b ? shift_b[b] : 0.f;
    const float* ia = in + b * rg.bstride + (long long)ra * rg.pitch;
    float2 v[N / T];
#pragma unroll
    for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
      for (int k = 0; k < R1; ++k) {
        const int x = slot_pos<N, T, R1>(t, i, k);
        v[i * R1 + k] = ok ? make_float2(ia[x] - shift, ia[rg.pitch + x] - shift) : make_float2(0.f, 0.f);
      }
    run_wstages<N, T, C::NP, false>(Rad{}, v, buf, tw, t);
    float2* hrow = H + b * hbstride + ra * hpitch;
    store_packed_half<N, T, RS>(v, buf, hrow, hrow + hpitch, ok, t);
  }
}

// ----------------------------------------------------------------------------
// Adjoint passes.  For a kick psi+ = exp(-i th) psi (th = dt_k (Phi + V + tide +
// kappa |psi|^2)) the adjoint of lam+ is
//   lam = exp(i th) lam+ + 2 (G mu + kappa mu) psi,  mu = dt_k Im(conj(lam+) psi+),
// with G the Poisson operator; a tidal amplitude a (tide = a D) adds
// dL/da += sum mu (1/2 x^T D x).  A1 does the x-inverse of lam, the pointwise
// part and the packed R2C of mu; A5 adds 2 G(mu) psi after the Poisson solve,
// the absorbing mask and (FWD) the x-forward transform of the drift adjoint.
// ----------------------------------------------------------------------------
struct AdjArgs {
  const float2* pre;      // pre-kick state psi [batch][nz][ny][nx] (real space)
  const float* D6;        // tidal direction (xx, yy, zz, xy, xz, yz) or null
  double* damp;           // [batch] accumulators of dL/da
  const float* mx;        // absorbing-mask tables (A5, null: none)
  const float* my;
  const float* mz;
};

// Pointwise part of the adjoint kick for row r, shared by the direct and the
// staged kernel: v holds lam+ at the radix-RS slots, phi the potential there
// and pre_at(q, x) the pre-kick state at slot q (position x).  Stores the new
// lam row (when ok), keeps mu of row A in mu0 and packs (mu_A, mu_B) into z
// at row B, and adds the tidal-amplitude term of the row to damp.
template <int N, class PreAt>
__device__ __forceinline__ void adj_kick_points(const float2* v, const float* phi, PreAt pre_at, const float* vrow,
                                                const float* T6, const KickArgs& a, const AdjArgs& j,
                                                const RowGeom& rg, int r, bool ok, float2* row, int half, float* mu0,
                                                float2* z, float& damp, int t) {
  using C = XCfg<N>;
  constexpr int T = C::T;
  constexpr int RS = RadInfo<typename XPlan<N>::Fwd>::last;
  const int y = r % rg.ny, zc = r / rg.ny;
  const float fy = a.y0 + a.dy * y, fz = a.z0 + a.dz * zc;
  const float cyz = 0.5f * T6[1] * fy * fy + T6[5] * fy * fz + 0.5f * T6[2] * fz * fz;
  const float lin = T6[3] * fy + T6[4] * fz;
  float dyz = 0.f, dlin = 0.f;
  if (j.D6) {
    dyz = 0.5f * j.D6[1] * fy * fy + j.D6[5] * fy * fz + 0.5f * j.D6[2] * fz * fz;
    dlin = j.D6[3] * fy + j.D6[4] * fz;
  }
#pragma unroll
  for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
    for (int k = 0; k < RS; ++k) {
      const int q = i * RS + k;
      const int x = slot_pos<N, T, RS>(t, i, k);
      const float2 pre = pre_at(q, x);
      const float fx = a.x0 + a.dx * x;
      float pot = phi[q];
      if (a.tidal) pot += fmaf(fx, fmaf(0.5f * T6[0], fx, lin), cyz);
      if (a.kerr != 0.f) pot = fmaf(a.kerr, fmaf(pre.x, pre.x, pre.y * pre.y), pot);  // as kick_points
      if (vrow && ok) pot += vrow[x];
      // mu = dt Im(conj(lam+) psi+) with psi+ = exp(-i th) pre equals
      // dt Im(conj(exp(+i th) lam+) pre): the rotated lam serves both
      float2 ln = kick_by<true>(v[q], kick_factor(pot, a), a);  // exp(+i th) lam+
      const float mu = a.dt_hi * (ln.x * pre.y - ln.y * pre.x);
      if (a.kerr != 0.f) {
        ln.x = fmaf(2.f * a.kerr * mu, pre.x, ln.x);
        ln.y = fmaf(2.f * a.kerr * mu, pre.y, ln.y);
      }
      if (j.D6) damp = fmaf(mu, fmaf(fx, fmaf(0.5f * j.D6[0], fx, dlin), dyz), damp);
      if (ok) row[x] = ln;
      if (half == 0)
        mu0[q] = mu;
      else
        z[q] = make_float2(mu0[q], mu);
    }
}

template <int N>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_adj_kick(float2* __restrict__ lam, const float2* __restrict__ H, float2* __restrict__ Hmu, RowGeom rg,
              long long hpitch, long long hbstride, const float4* __restrict__ twg, KickArgs a, AdjArgs j, XWork w) {
  WDM_XPASS_PROLOGUE
  // With at most WDM_ADJ_PF points per lane the lam and pre rows of the pair
  // fit in registers: row A's are loaded before the potential transform, row
  // B's after it, so the warp does not wait on them one by one.
  constexpr bool PF = N / T <= WDM_ADJ_PF;
  constexpr int PN = PF ? N / T : 1;
  for (long long u = (long long)blockIdx.x * C::WARPS + warp; u < nunits; u += wstride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
    const float2* hrow = H + b * hbstride + ra * hpitch;
    float2 v[N / T];
    // potential rows of the pair, at the radix-RS slots
    load_packed_half<N, T, R1>(v, hrow, hrow + hpitch, ok, t);
    // lam rows at the radix-R1 slots, pre rows at the radix-RS slots
    float2 lpf[2][PN], ppf[2][PN];
    auto prefetch = [&](int half) {
      const float2* row = lam + b * rg.bstride + (long long)(ra + half) * rg.pitch;
      const float2* prow = j.pre + b * rg.bstride + (long long)(ra + half) * rg.pitch;
#pragma unroll
      for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
        for (int k = 0; k < R1; ++k)
          lpf[half][i * R1 + k] = ok ? row[slot_pos<N, T, R1>(t, i, k)] : make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k)
          ppf[half][i * RS + k] = ok ? prow[slot_pos<N, T, RS>(t, i, k)] : make_float2(0.f, 0.f);
    };
    if constexpr (PF) prefetch(0);
    run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);
    float phi[2][N / T];
#pragma unroll
    for (int q = 0; q < N / T; ++q) {
      phi[0][q] = v[q].x;
      phi[1][q] = v[q].y;
    }
    if constexpr (PF) prefetch(1);
    float T6[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) T6[q] = a.T6b ? a.T6b[b * 6 + q] : a.T6[q];
    float mu0[N / T];
    float2 z[N / T];
    float damp = 0.f;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int r = ra + half;
      float2* row = lam + b * rg.bstride + (long long)r * rg.pitch;
      const float2* prow = j.pre + b * rg.bstride + (long long)r * rg.pitch;
      const float* vrow = a.V ? a.V + b * a.v_bstride + (long long)r * rg.pitch : nullptr;
      if constexpr (PF) {
#pragma unroll
        for (int q = 0; q < N / T; ++q) v[q] = lpf[half][q];
      } else {
#pragma unroll
        for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
          for (int k = 0; k < R1; ++k) v[i * R1 + k] = ok ? row[slot_pos<N, T, R1>(t, i, k)] : make_float2(0.f, 0.f);
      }
      run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);  // lam+ in real space, radix-RS slots
      auto pre_at = [&](int q, int x) {
        if constexpr (PF)
          return ppf[half][q];
        else
          return ok ? prow[x] : make_float2(0.f, 0.f);
      };
      adj_kick_points<N>(v, phi[half], pre_at, vrow, T6, a, j, rg, r, ok, row, half, mu0, z, damp, t);
    }
    reorder<N, T, RS, R1>(z, v);
    run_wstages<N, T, C::NP, false>(Rad{}, v, buf, tw, t);
    float2* hm = Hmu + b * hbstride + ra * hpitch;
    store_packed_half<N, T, RS>(v, buf, hm, hm + hpitch, ok, t);
    if (j.D6) {
      // sum over the T lanes of this group only (groups of one warp may hold
      // rows of different batch items)
#pragma unroll
      for (int off = T / 2; off > 0; off >>= 1) damp += __shfl_down_sync(0xffffffffu, damp, off, T);
      if (t == 0 && ok) atomicAdd(j.damp + b, (double)damp);
    }
  }
}

template <int N, bool FWD>
__global__ void __launch_bounds__(XCfg<N>::NT, WDM_X_MINB)
k_xw_adj_apply(float2* __restrict__ lam, const float2* __restrict__ Hmu, RowGeom rg, long long hpitch,
               long long hbstride, const float4* __restrict__ twg, AdjArgs j, XWork w) {
  WDM_XPASS_PROLOGUE
  for (long long u = (long long)blockIdx.x * C::WARPS + warp; u < nunits; u += wstride) {
    const long long pp = u * C::GROUPS + g;
    const bool ok = pp < (long long)w.pairs_per_item * w.batch;
    const int b = ok ? (int)(pp / w.pairs_per_item) : 0;
    const int ra = ok ? 2 * (int)(pp - (long long)b * w.pairs_per_item) : 0;
    const float2* hrow = Hmu + b * hbstride + ra * hpitch;
    float2 v[N / T];
    load_packed_half<N, T, R1>(v, hrow, hrow + hpitch, ok, t);
    run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);  // G mu of rows A, B at radix-RS slots
    float gmu[2][N / T];
#pragma unroll
    for (int q = 0; q < N / T; ++q) {
      gmu[0][q] = v[q].x;
      gmu[1][q] = v[q].y;
    }
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int r = ra + half;
      float2* row = lam + b * rg.bstride + (long long)r * rg.pitch;
      const float2* prow = j.pre + b * rg.bstride + (long long)r * rg.pitch;
      const float myz = j.mx ? j.my[r % rg.ny] * j.mz[r / rg.ny] : 1.f;
      float2 zz[N / T];
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k) {
          const int q = i * RS + k;
          const int x = slot_pos<N, T, RS>(t, i, k);
          float2 l = ok ? row[x] : make_float2(0.f, 0.f);
          const float2 pre = ok ? prow[x] : make_float2(0.f, 0.f);
          l.x = fmaf(2.f * gmu[half][q], pre.x, l.x);
          l.y = fmaf(2.f * gmu[half][q], pre.y, l.y);
          if (FWD && j.mx) l = cscale(l, myz * j.mx[x]);  // the mask precedes every kick but the first
          zz[q] = l;
        }
      if constexpr (FWD) {
        reorder<N, T, RS, R1>(zz, v);
        run_wstages<N, T, C::NP, false>(Rad{}, v, buf, tw, t);
        if (ok)
#pragma unroll
          for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
            for (int k = 0; k < RS; ++k) row[slot_pos<N, T, RS>(t, i, k)] = v[i * RS + k];
      } else {
        if (ok)
#pragma unroll
          for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
            for (int k = 0; k < RS; ++k) row[slot_pos<N, T, RS>(t, i, k)] = zz[i * RS + k];
      }
    }
  }
}

// WDM_XPASS_PROLOGUE stays defined for the staged kernels (xpass_staged.cuh)

}  // namespace wdm
