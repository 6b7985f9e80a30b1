// x passes with their input rows staged in shared memory by 1-D bulk copies.
//
// The direct kernels (xpass_warp.cuh) load each row into registers when they
// reach it, so a warp waits on global memory three times per row pair (the
// potential rows, then psi row A, then psi row B) with nothing else to do.
// Here every warp owns two slots: slot A for the half-spectrum rows (kick) or
// the baryon density rows (density pass), slot B for the psi rows of a whole
// unit (the GROUPS row pairs of one warp).  As soon as a slot's rows are in
// registers the warp's lane 0 issues the bulk copies of the same rows of its
// next unit into it, so those copies run under the transforms of the current
// unit.  Each row is one copy into a slot row whose pitch is padded by 16
// bytes, so that the lane groups of a warp read different banks.  At N = 384
// the kernels run 3 CTAs of 4 warps per SM with up to 170 registers per
// thread (XStageCap).  Every wait is bounded: a warp that gives up records
// WDM_DEVERR_TMA_WAIT, drains its copies (bounded) and exits.
#pragma once
#include "xpass_warp.cuh"

namespace wdm {
// Largest number of resident CTAs per SM the staged kernels of size N are
// compiled for (registers per thread = 65536 / (128 threads x that number));
// WDM_XS_MINB_CAP overrides it for every size.  At N = 384 the shared memory
// allows 4, but the kick compiled for 4 (122 registers) issued 6% more
// instructions and measured 0.353 ms against 0.337 ms for 3 CTAs of up to
// 170 registers.
template <int N>
struct XStageCap {
  static constexpr int value = 4;
};
template <>
struct XStageCap<384> {
  static constexpr int value = 3;
};
}  // namespace wdm
#ifdef WDM_XS_MINB_CAP
#define WDM_XS_CAP(N) WDM_XS_MINB_CAP
#else
#define WDM_XS_CAP(N) XStageCap<N>::value
#endif
// 1: the staged density pass transforms the two rows of a pair side by side
#ifndef WDM_XS_PAIR
#define WDM_XS_PAIR 1
#endif

namespace wdm {

template <int N>
struct XStage {
  using C = XCfg<N>;
  static constexpr int G = C::GROUPS;
  static constexpr int ROWS = 2 * G;    // rows of one warp unit
  static constexpr int HP = N / 2 + 2;  // H row pitch in global memory: nx/2 + 1 rounded up to even
  static constexpr int PSI_P = N + 2;   // staged psi row pitch (float2)
  static constexpr int H_P = HP + 2;    // staged H row pitch (float2)
  static constexpr int RB_P = N + 4;    // staged density row pitch (float)
  static constexpr size_t A_BYTES = sizeof(float2) * ROWS * H_P;
  static constexpr size_t B_BYTES = sizeof(float2) * ROWS * PSI_P;
  static_assert(sizeof(float) * ROWS * RB_P <= A_BYTES, "density rows fit slot A");
  static constexpr size_t WARP_BYTES = A_BYTES + B_BYTES;
  static constexpr size_t BASE = C::SMEM;  // after the twiddle tables and exchange buffers
  static constexpr size_t SMEM = BASE + C::WARPS * WARP_BYTES + C::WARPS * 2 * sizeof(uint64_t);
  // resident CTAs per SM the shared memory allows (at most XStageCap), for
  // the register budget
  static constexpr int CAP = WDM_XS_CAP(N);
  static constexpr int MINB_RAW = (int)((228u * 1024u) / (SMEM + 1024u));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > CAP ? CAP : MINB_RAW);
  static_assert(BASE % 16 == 0 && A_BYTES % 16 == 0 && B_BYTES % 16 == 0, "16-byte aligned slots");
  static_assert(2 * PSI_P >= C::NP, "a pair's psi rows hold one exchange buffer");
};

// Copy `nrows` rows of `row_elems` elements (pitch src_pitch) to a slot with
// row pitch dst_pitch, all completing on `bar` (one lane).
template <typename E>
__device__ __forceinline__ void stage_rows(E* dst, int dst_pitch, const E* src, long long src_pitch, int row_elems,
                                           int nrows, uint64_t* bar) {
  const unsigned rb = (unsigned)(row_elems * sizeof(E));
  mbar_expect_tx(bar, rb * (unsigned)nrows);
  for (int r = 0; r < nrows; ++r) bulk_g2s(dst + r * dst_pitch, src + r * src_pitch, rb, bar);
}

// Bounded wait, uniform over the warp.
__device__ __forceinline__ bool xwait(uint64_t* bar, unsigned parity) {
  return __all_sync(0xffffffffu, mbar_wait_bounded(bar, parity));
}

// The slot's rows are in registers: order those reads before the next copy.
__device__ __forceinline__ void xrelease() {
  fence_proxy_async_smem();
  __syncwarp();
}

// The adjoint kick stages a third slot, the pre-kick rows, after slot B; its
// lam and pre rows complete on the one barrier of slot B.
template <int N>
struct XStageAdj : XStage<N> {
  using B = XStage<N>;
  static constexpr size_t WARP_BYTES = B::A_BYTES + 2 * B::B_BYTES;
  static constexpr size_t SMEM = B::BASE + B::C::WARPS * WARP_BYTES + B::C::WARPS * 2 * sizeof(uint64_t);
  static constexpr int MINB_RAW = (int)((228u * 1024u) / (SMEM + 1024u));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > B::CAP ? B::CAP : MINB_RAW);
};

#define WDM_XSTAGE_PROLOGUE WDM_XSTAGE_PROLOGUE_T(XStage<N>)
#define WDM_XSTAGE_PROLOGUE_T(ST)                                                                    \
  using S = ST;                                                                                      \
  unsigned char* sraw = reinterpret_cast<unsigned char*>(smem);                                      \
  unsigned char* wslots = sraw + S::BASE + (size_t)warp * S::WARP_BYTES;                             \
  float2* slotA = reinterpret_cast<float2*>(wslots);                                                 \
  float2* slotB = reinterpret_cast<float2*>(wslots + S::A_BYTES);                                    \
  uint64_t* xbar = reinterpret_cast<uint64_t*>(sraw + S::BASE + (size_t)C::WARPS * S::WARP_BYTES) + 2 * warp; \
  if (lane == 0) {                                                                                   \
    mbar_init(&xbar[0], 1);                                                                          \
    mbar_init(&xbar[1], 1);                                                                          \
    mbar_fence_init();                                                                               \
  }                                                                                                  \
  __syncwarp();                                                                                      \
  const int ppi = w.pairs_per_item;                                                                  \
  unsigned pend = 0, ph = 0; /* bit s: slot s has copies in flight / parity of its next phase */

// Wait for slot s (bounded, warp-uniform); false: give up.
#define WDM_XSTAGE_WAIT(s) \
  (xwait(&xbar[(s)], (ph >> (s)) & 1u) ? (ph ^= 1u << (s), pend &= ~(1u << (s)), true) : false)

// Give up: record the error, drain this warp's copies (bounded), leave.
#define WDM_XSTAGE_FAIL(errp)                                                        \
  do {                                                                               \
    if (lane == 0 && (errp)) atomicOr((errp), WDM_DEVERR_TMA_WAIT);                  \
    bool drained = true;                                                             \
    for (int s_ = 0; s_ < 2; ++s_)                                                   \
      if (pend & (1u << s_)) drained = xwait(&xbar[s_], (ph >> s_) & 1u) && drained; \
    if (lane == 0 && (errp) && !drained) atomicOr((errp), WDM_DEVERR_TMA_DRAIN);     \
    return;                                                                          \
  } while (0)

// first batch item and row of warp unit u (a unit never straddles two items:
// the launcher requires GROUPS to divide the row pairs of an item)
__device__ __forceinline__ void unit_rows(long long u, int groups, int ppi, int* b, int* ra) {
  const long long pp0 = u * groups;
  *b = (int)(pp0 / ppi);
  *ra = 2 * (int)(pp0 - (long long)(*b) * ppi);
}

// P1 (staged): Phi rows from H, kick, forward x transform (FWD) or not.
template <int N, bool FWD>
__global__ void __launch_bounds__(XCfg<N>::NT, XStage<N>::MINB)
k_xs_kick(const float2* psi_in, float2* psi, const float2* __restrict__ H, RowGeom rg, long long hpitch,
          long long hbstride, const float4* __restrict__ twg, KickArgs a, XWork w) {
  WDM_XPASS_PROLOGUE
  WDM_XSTAGE_PROLOGUE
  auto issue_h = [&](long long u) {
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    stage_rows(slotA, S::H_P, H + b * hbstride + ra * hpitch, hpitch, S::HP, S::ROWS, &xbar[0]);
  };
  auto issue_p = [&](long long u) {
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    stage_rows(slotB, S::PSI_P, psi_in + b * rg.bstride + ra * rg.pitch, rg.pitch, N, S::ROWS, &xbar[1]);
  };
  long long u = (long long)blockIdx.x * C::WARPS + warp;
  if (u < nunits) {
    if (lane == 0) {
      issue_h(u);
      issue_p(u);
    }
    pend = 3u;
  }
  for (; u < nunits; u += wstride) {
    const long long un = u + wstride;
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    ra += 2 * g;  // this lane group's pair
    if (!WDM_XSTAGE_WAIT(0)) WDM_XSTAGE_FAIL(a.err);
    float2 v[N / T];
    load_packed_half<N, T, R1>(v, slotA + (2 * g) * S::H_P, slotA + (2 * g + 1) * S::H_P, true, t);
    xrelease();
    if (un < nunits) {
      if (lane == 0) issue_h(un);
      pend |= 1u;
    }
    run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);  // ends with radix RS
    float phi[2][N / T];
#pragma unroll
    for (int q = 0; q < N / T; ++q) {
      phi[0][q] = v[q].x;
      phi[1][q] = v[q].y;
    }
    float T6[10];
    kick_tidal<N>(T6, a, rg, b);
    auto release_b = [&]() {
      xrelease();
      if (un < nunits) {
        if (lane == 0) issue_p(un);
        pend |= 2u;
      }
    };
    if constexpr (FWD) {
      // One row per iteration of a loop that is not unrolled: half the code
      // of an unrolled pair (70 against 99 KB at N = 384), so that more of
      // the loop stays in the instruction cache.  At N = 384 this measured
      // 0.382 ms against 0.384 for both rows side by side (one twiddle load
      // for both, as the density pass does).
      float phr[N / T];  // the potential of the row in hand
#pragma unroll
      for (int q = 0; q < N / T; ++q) phr[q] = phi[0][q];
      if (!WDM_XSTAGE_WAIT(1)) WDM_XSTAGE_FAIL(a.err);
#pragma unroll 1
      for (int half = 0; half < 2; ++half) {
        const float2* srow = slotB + (2 * g + half) * S::PSI_P;
#pragma unroll
        for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
          for (int k = 0; k < RS; ++k) v[i * RS + k] = srow[slot_pos<N, T, RS>(t, i, k)];
        if (half == 1) release_b();
        const int r = ra + half;
        kick_row<N, true>(v, phr, T6, a, rg, r, b, true, psi + b * rg.bstride + (long long)r * rg.pitch, buf, tw, t);
#pragma unroll
        for (int q = 0; q < N / T; ++q) phr[q] = phi[1][q];
      }
    } else {
      // The closing half kick (no transform): both rows at once, slot B
      // released as soon as they are in registers.
      if (!WDM_XSTAGE_WAIT(1)) WDM_XSTAGE_FAIL(a.err);
      float2 vb[N / T];
      const float2* sb = slotB + (2 * g) * S::PSI_P;
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k) {
          v[i * RS + k] = sb[slot_pos<N, T, RS>(t, i, k)];
          vb[i * RS + k] = sb[S::PSI_P + slot_pos<N, T, RS>(t, i, k)];
        }
      release_b();
      kick_points<N, RS>(v, phi[0], T6, a, rg, ra, b, true, t);
      kick_points<N, RS>(vb, phi[1], T6, a, rg, ra + 1, b, true, t);
      float2* rowa = psi + b * rg.bstride + (long long)ra * rg.pitch;
      store_row<N, RS>(rowa, v, true, t);
      store_row<N, RS>(rowa + rg.pitch, vb, true, t);
    }
  }
}

// P5 (staged): psi x-inverse (+mask), rho = |psi|^2 (+rho_b) - shift, packed R2C -> H
// (CEN: with the density maximum and moments for the tide's frame).
template <int N, bool CEN>
__global__ void __launch_bounds__(XCfg<N>::NT, XStage<N>::MINB)
k_xs_inv_rho(float2* __restrict__ psi, float2* __restrict__ H, RowGeom rg, long long hpitch, long long hbstride,
             const float4* __restrict__ twg, RhoArgs a, XWork w) {
  WDM_XPASS_PROLOGUE
  WDM_XSTAGE_PROLOGUE
  float* rbslot = reinterpret_cast<float*>(slotA);
  auto issue_p = [&](long long u) {
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    stage_rows(slotB, S::PSI_P, psi + b * rg.bstride + ra * rg.pitch, rg.pitch, N, S::ROWS, &xbar[1]);
  };
  const bool with_rb = a.rho_b != nullptr;
  // Bit r: row r of unit uu holds baryon mass (every row without flags).  The
  // flags are read a unit ahead, so that their latency hides under the work
  // of a unit instead of stalling the copies and the density.
  auto rb_mask = [&](long long uu) -> unsigned {
    if (!with_rb) return 0u;
    if (!a.rb_rows) return S::ROWS >= 32 ? ~0u : (1u << (S::ROWS & 31)) - 1u;
    int b, ra0;
    unit_rows(uu, C::GROUPS, ppi, &b, &ra0);
    unsigned m = 0;
#pragma unroll
    for (int r = 0; r < S::ROWS; ++r) m |= (a.rb_rows[ra0 + r] ? 1u : 0u) << r;
    return m;
  };
  // only the rows flagged as holding baryon mass are copied (a phase with no
  // copy completes on the arrival alone)
  auto issue_r = [&](long long u, unsigned m) {
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    const float* src = a.rho_b + b * a.rb_bstride + ra * rg.pitch;
    mbar_expect_tx(&xbar[0], (unsigned)__popc(m) * (unsigned)(N * sizeof(float)));
    for (int r = 0; r < S::ROWS; ++r)
      if ((m >> r) & 1u) bulk_g2s(rbslot + r * S::RB_P, src + r * rg.pitch, (unsigned)(N * sizeof(float)), &xbar[0]);
  };
  CentreSum cs;
  cs.reset(-1);
  long long u = (long long)blockIdx.x * C::WARPS + warp;
  unsigned mcur = u < nunits ? rb_mask(u) : 0u;
  if (u < nunits) {
    if (lane == 0) {
      issue_p(u);
      if (with_rb) issue_r(u, mcur);
    }
    pend = with_rb ? 3u : 2u;
  }
  for (; u < nunits; u += wstride) {
    const long long un = u + wstride;
    const unsigned mnext = un < nunits ? rb_mask(un) : 0u;
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    ra += 2 * g;
    const float shift = a.shift ? a.shift[b] : 0.f;
    float rho0[N / T];  // row A density at radix-RS slots
    float2 z[N / T];    // packed (rho_A, rho_B) at radix-RS slots
    float2 v[N / T];
    CentreAcc ca;
    ca.reset();
    if (!WDM_XSTAGE_WAIT(1)) WDM_XSTAGE_FAIL(a.err);
    auto release_p = [&]() {
      xrelease();
      if (un < nunits) {
        if (lane == 0) issue_p(un);
        pend |= 2u;
      }
    };
    auto release_r = [&]() {
      xrelease();
      if (un < nunits) {
        if (lane == 0) issue_r(un, mnext);
        pend |= 1u;
      }
    };
    auto rb_of = [&](int half) -> const float* {
      return ((mcur >> (2 * g + half)) & 1u) ? rbslot + (2 * g + half) * S::RB_P : nullptr;
    };
    const bool paired = WDM_XS_PAIR && a.write_psi;
    if (paired) {
      // Both rows inverted side by side, row B exchanging through slot B
      // (its rows are in registers by then); the next psi copy follows.
      float2 vb[N / T];
      float2* sb = slotB + (2 * g) * S::PSI_P;
#pragma unroll
      for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
        for (int k = 0; k < R1; ++k) {
          v[i * R1 + k] = sb[slot_pos<N, T, R1>(t, i, k)];
          vb[i * R1 + k] = sb[S::PSI_P + slot_pos<N, T, R1>(t, i, k)];
        }
      run_wstages2<N, T, C::NP, true>(Rad{}, v, vb, buf, sb, tw, t);
      release_p();
      if (with_rb && !WDM_XSTAGE_WAIT(0)) WDM_XSTAGE_FAIL(a.err);
      float2* rowa = psi + b * rg.bstride + (long long)ra * rg.pitch;
      rho_row_post<N, CEN>(v, a, rg, ra, true, rowa, rb_of(0), shift, 0, rho0, z, t, ca);
      rho_row_post<N, CEN>(vb, a, rg, ra + 1, true, rowa + rg.pitch, rb_of(1), shift, 1, rho0, z, t, ca);
      if (with_rb) release_r();
    } else {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const float2* srow = slotB + (2 * g + half) * S::PSI_P;
      if (a.write_psi) {
#pragma unroll
        for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
          for (int k = 0; k < R1; ++k) v[i * R1 + k] = srow[slot_pos<N, T, R1>(t, i, k)];
      } else {
#pragma unroll
        for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
          for (int k = 0; k < RS; ++k) v[i * RS + k] = srow[slot_pos<N, T, RS>(t, i, k)];
      }
      if (half == 1) release_p();
      if (half == 0 && with_rb && !WDM_XSTAGE_WAIT(0)) WDM_XSTAGE_FAIL(a.err);
      const int r = ra + half;
      inv_rho_row<N, CEN>(v, a, rg, r, true, psi + b * rg.bstride + (long long)r * rg.pitch, rb_of(half), shift,
                          half, rho0, z, buf, tw, t, ca);
      if (half == 1 && with_rb) release_r();
    }
    }
    if constexpr (CEN) centre_pair_done<N>(a, rg, ca, cs, b, ra, true, t);
    mcur = mnext;
    reorder<N, T, RS, R1>(z, v);
    run_wstages<N, T, C::NP, false>(Rad{}, v, buf, tw, t);
    float2* hrow = H + b * hbstride + ra * hpitch;
    store_packed_half<N, T, RS>(v, buf, hrow, hrow + hpitch, true, t);
  }
  if (CEN && t == 0) cs.flush(a.centre);
}

// Adjoint kick (staged): the arithmetic of k_xw_adj_kick, with the H rows in
// slot A and the lam and pre rows of the unit in slots B and C, all copied
// one unit ahead.  The updated lam rows and the packed mu spectrum are stored
// straight to global memory.
template <int N>
__global__ void __launch_bounds__(XCfg<N>::NT, XStageAdj<N>::MINB)
k_xs_adj_kick(float2* __restrict__ lam, const float2* __restrict__ H, float2* __restrict__ Hmu, RowGeom rg,
              long long hpitch, long long hbstride, const float4* __restrict__ twg, KickArgs a, AdjArgs j,
              XWork w) {
  WDM_XPASS_PROLOGUE
  WDM_XSTAGE_PROLOGUE_T(XStageAdj<N>)
  float2* slotC = slotB + S::ROWS * S::PSI_P;
  auto issue_h = [&](long long u) {
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    stage_rows(slotA, S::H_P, H + b * hbstride + ra * hpitch, hpitch, S::HP, S::ROWS, &xbar[0]);
  };
  auto issue_lp = [&](long long u) {
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    const unsigned rb = (unsigned)(N * sizeof(float2));
    const long long o = b * rg.bstride + ra * rg.pitch;
    mbar_expect_tx(&xbar[1], 2u * rb * (unsigned)S::ROWS);
    for (int r = 0; r < S::ROWS; ++r) {
      bulk_g2s(slotB + r * S::PSI_P, lam + o + r * rg.pitch, rb, &xbar[1]);
      bulk_g2s(slotC + r * S::PSI_P, j.pre + o + r * rg.pitch, rb, &xbar[1]);
    }
  };
  long long u = (long long)blockIdx.x * C::WARPS + warp;
  if (u < nunits) {
    if (lane == 0) {
      issue_h(u);
      issue_lp(u);
    }
    pend = 3u;
  }
  for (; u < nunits; u += wstride) {
    const long long un = u + wstride;
    int b, ra;
    unit_rows(u, C::GROUPS, ppi, &b, &ra);
    ra += 2 * g;  // this lane group's pair
    if (!WDM_XSTAGE_WAIT(0)) WDM_XSTAGE_FAIL(a.err);
    float2 v[N / T];
    load_packed_half<N, T, R1>(v, slotA + (2 * g) * S::H_P, slotA + (2 * g + 1) * S::H_P, true, t);
    xrelease();
    if (un < nunits) {
      if (lane == 0) issue_h(un);
      pend |= 1u;
    }
    run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);
    float phi[2][N / T];
#pragma unroll
    for (int q = 0; q < N / T; ++q) {
      phi[0][q] = v[q].x;
      phi[1][q] = v[q].y;
    }
    float T6[10];
    kick_tidal<N>(T6, a, rg, b);
    float mu0[N / T];
    float2 z[N / T];
    float damp = 0.f;
    if (!WDM_XSTAGE_WAIT(1)) WDM_XSTAGE_FAIL(a.err);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int r = ra + half;
      const float2* lrow = slotB + (2 * g + half) * S::PSI_P;
      const float2* prow = slotC + (2 * g + half) * S::PSI_P;
      float2* row = lam + b * rg.bstride + (long long)r * rg.pitch;
      const float* vrow = a.V ? a.V + b * a.v_bstride + (long long)r * rg.pitch : nullptr;
#pragma unroll
      for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
        for (int k = 0; k < R1; ++k) v[i * R1 + k] = lrow[slot_pos<N, T, R1>(t, i, k)];
      run_wstages<N, T, C::NP, true>(Rad{}, v, buf, tw, t);  // lam+ in real space, radix-RS slots
      auto pre_at = [&](int, int x) { return prow[x]; };
      adj_kick_points<N>(v, phi[half], pre_at, vrow, T6, a, j, rg, r, true, row, half, mu0, z, damp, t);
      if (half == 1) {
        xrelease();
        if (un < nunits) {
          if (lane == 0) issue_lp(un);
          pend |= 2u;
        }
      }
    }
    reorder<N, T, RS, R1>(z, v);
    run_wstages<N, T, C::NP, false>(Rad{}, v, buf, tw, t);
    float2* hm = Hmu + b * hbstride + ra * hpitch;
    store_packed_half<N, T, RS>(v, buf, hm, hm + hpitch, true, t);
    if (j.D6) {
#pragma unroll
      for (int off = T / 2; off > 0; off >>= 1) damp += __shfl_down_sync(0xffffffffu, damp, off, T);
      if (t == 0) atomicAdd(j.damp + b, (double)damp);
    }
  }
}

#undef WDM_XSTAGE_FAIL
#undef WDM_XSTAGE_WAIT
#undef WDM_XSTAGE_PROLOGUE_T
#undef WDM_XSTAGE_PROLOGUE
#undef WDM_XPASS_PROLOGUE

}  // namespace wdm
