// Launchers of the pass kernels for one axis length N (included by sizes_*.cu).
#pragma once
#include <atomic>
#include <cmath>
#include "kernel_set.h"
#include "xpass_warp.cuh"

namespace wdm {

// Launch settings are device properties: each is found once per device (the
// current one at the launch) and kept in a slot per device ordinal.
constexpr int MAX_DEVICES = 64;

static int current_device() {
  int dev = 0;
  cudaGetDevice(&dev);
  return dev >= 0 && dev < MAX_DEVICES ? dev : 0;
}

// Opt a kernel in to more than 48 KB of dynamic shared memory, once per device.
template <auto K>
static cudaError_t prep_once(size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  // 0: not yet, 1: done, 2 + e: failed with cudaError_t e
  static std::atomic<int> state[MAX_DEVICES];
  std::atomic<int>& st = state[current_device()];
  int v = st.load(std::memory_order_acquire);
  if (v == 0) {
    const cudaError_t e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    v = e == cudaSuccess ? 1 : 2 + (int)e;
    st.store(v, std::memory_order_release);
  }
  return v == 1 ? cudaSuccess : (cudaError_t)(v - 2);
}

// SMs of the current device.
static int sm_count() {
  static std::atomic<int> n[MAX_DEVICES];
  const int dev = current_device();
  int v = n[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    v = v > 0 ? v : 1;
    n[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// Resident CTAs per SM of a kernel at its block size and shared memory, on the
// current device (each call site passes one fixed size).
template <auto K>
static int resident_ctas(int threads, size_t smem) {
  static std::atomic<int> n[MAX_DEVICES];
  std::atomic<int>& slot = n[current_device()];
  int v = slot.load(std::memory_order_relaxed);
  if (v == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, K, threads, smem);
    v = v > 0 ? v : 1;
    slot.store(v, std::memory_order_relaxed);
  }
  return v;
}

template <int N>
struct Launch {
  static constexpr int NT = threads_for<N>();

  // Tensor map of the lines of g (null view: false).
  static bool line_map(CUtensorMap* map, const float2* data, const LineGeom& g, int batch) {
    using TT = TmaTile<N>;
    if (g.axis != 1 && g.axis != 2) return false;
    if (g.nxa < LINES || g.rows <= 0) return false;  // the box stays inside the tensor along x
    const uint64_t e = sizeof(float2);
    uint64_t dims[4], strides[3];
    uint32_t box[4];
    dims[0] = (uint64_t)g.nxa;
    dims[3] = (uint64_t)batch;
    strides[0] = (uint64_t)g.pitch * e;
    strides[2] = (uint64_t)g.bstride * e;
    if (g.axis == 1) {  // [batch][rows][N][pitch]
      dims[1] = N;
      dims[2] = (uint64_t)g.rows;
      strides[1] = (uint64_t)g.pitch * N * e;
      box[0] = LINES, box[1] = TT::BOXP, box[2] = 1, box[3] = 1;
    } else {  // [batch][N][rows][pitch]
      dims[1] = (uint64_t)g.rows;
      dims[2] = N;
      strides[1] = (uint64_t)g.pitch * g.rows * e;
      box[0] = LINES, box[1] = 1, box[2] = TT::BOXP, box[3] = 1;
    }
    return encode_map_c64(map, data, dims, strides, box);
  }

  // Tensor map of the edge tiles of g (the last column when nxa = 16 m + 1,
  // 8 rows per tile; k_lfft_tma): the lines' axis outermost, a box of 2
  // columns x 8 rows x BOXP points starting at column nxa - 1, whose x offset
  // (nxa - 1) * 8 bytes must be a multiple of 16.  false: no edge tiles.
  static bool edge_map(CUtensorMap* map, const float2* data, const LineGeom& g, int batch) {
    using TT = TmaTile<N>;
    if (g.axis != 1 && g.axis != 2) return false;
    if (g.nxa % LINES != 1 || g.nxa < LINES || (g.nxa - 1) % 2 != 0 || g.rows <= 0 || g.rows % 8 != 0) return false;
    const uint64_t e = sizeof(float2);
    uint64_t dims[4] = {(uint64_t)g.nxa, (uint64_t)g.rows, (uint64_t)N, (uint64_t)batch};
    uint64_t strides[3];
    if (g.axis == 1) {  // rows (z) at pitch * N, points (y) at pitch
      strides[0] = (uint64_t)g.pitch * N * e;
      strides[1] = (uint64_t)g.pitch * e;
    } else {  // rows (y) at pitch, points (z) at pitch * rows
      strides[0] = (uint64_t)g.pitch * e;
      strides[1] = (uint64_t)g.pitch * g.rows * e;
    }
    strides[2] = (uint64_t)g.bstride * e;
    const uint32_t box[4] = {2, 8, (uint32_t)TT::BOXP, 1};
    return encode_map_c64(map, data, dims, strides, box);
  }

  template <int MODE, bool LATE, class Op>
  static cudaError_t ltma_launch(float2* data, const CUtensorMap& map, const CUtensorMap& emap, const LineGeom& ge,
                                 const float4* tw, const Op& op, int batch, cudaStream_t st) {
    constexpr size_t SMEM = ltma_smem_bytes<N, MODE>();
    cudaError_t e;
    if ((e = prep_once<k_lfft_tma<N, MODE, Op, LATE>>(SMEM)) != cudaSuccess) return e;
    const int tx = ge.edge ? ge.nxa / LINES : (ge.nxa + LINES - 1) / LINES;
    const long long tiles = ((long long)ge.rows * tx + ge.edge) * batch;
    const long long cap = (long long)resident_ctas<k_lfft_tma<N, MODE, Op, LATE>>(NT, SMEM) * sm_count();
    const unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
    k_lfft_tma<N, MODE, Op, LATE><<<grid, NT, SMEM, st>>>(data, map, emap, ge, tw, op, batch);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }

  // persistent line pass: one wave of resident CTAs walking all tiles
  template <int MODE, class Op>
  static cudaError_t lpipe(float2* data, const LineGeom& g, const float4* tw, const Op& op, int batch,
                           cudaStream_t st) {
    if (g.nlines <= 0 || batch <= 0) return cudaSuccess;
#if !defined(WDM_LINE_PIPELINE) && !defined(WDM_LINE_TILE)
    {
      CUtensorMap map, emap;
      if (g.impl == LINE_IMPL_TMA && line_map(&map, data, g, batch)) {
        LineGeom ge = g;
        ge.edge = 0;
#ifndef WDM_NO_EDGE_TILES
        if (edge_map(&emap, data, g, batch)) ge.edge = g.rows / 8;
#endif
        if (!ge.edge) emap = map;  // not read
        // The next tile's copy goes out late (k_lfft_tma) in the fused z
        // passes, which are bound by instruction issue, and in the y passes
        // of a half spectrum (the ones with edge tiles); early in the y passes
        // of psi, which are bound by memory.  Measured at 384^3 against early
        // everywhere: the z passes 0.8-1.1% faster, the half-spectrum y
        // passes 1.3-3% faster; late everywhere made the psi y passes 0.7-1.3%
        // slower.
        if constexpr (MODE == 2) {
          return ltma_launch<MODE, true>(data, map, emap, ge, tw, op, batch, st);
        } else {
#ifndef WDM_TMA_EARLY_HALF_Y  // tuning variant: early in every y pass
          if (ge.edge) return ltma_launch<MODE, true>(data, map, emap, ge, tw, op, batch, st);
#endif
          return ltma_launch<MODE, false>(data, map, emap, ge, tw, op, batch, st);
        }
      }
    }
#endif
#ifndef WDM_LINE_PIPELINE
    return ltile<MODE>(data, g, tw, op, batch, st);
#else
    constexpr size_t SMEM = lpipe_smem_bytes<N, MODE>();
    cudaError_t e;
    if ((e = prep_once<k_lfft_pipe<N, MODE, Op>>(SMEM)) != cudaSuccess) return e;
    const long long tiles = (long long)((g.nlines + LINES - 1) / LINES) * batch;
    const long long cap = (long long)resident_ctas<k_lfft_pipe<N, MODE, Op>>(NT, SMEM) * sm_count();
    const unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
    k_lfft_pipe<N, MODE, Op><<<grid, NT, SMEM, st>>>(data, g, tw, op, batch);
    ++tl_kernel_launches;
    return cudaGetLastError();
#endif
  }

  // one register tile of LINES lines per CTA (lines may straddle rows)
  template <int MODE, class Op>
  static cudaError_t ltile(float2* data, const LineGeom& g, const float4* tw, const Op& op, int batch,
                           cudaStream_t st) {
    constexpr size_t SMEM = ltile_smem_bytes<N, MODE>();
    cudaError_t e;
    if ((e = prep_once<k_lfft_tile<N, MODE, Op>>(SMEM)) != cudaSuccess) return e;
    k_lfft_tile<N, MODE, Op><<<dim3((g.nlines + LINES - 1) / LINES, batch), NT, SMEM, st>>>(data, g, tw, op);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }

  static cudaError_t lfft(float2* data, const LineGeom& g, const float4* tw, bool inv, int batch, cudaStream_t st) {
    return inv ? lpipe<1>(data, g, tw, NoOp{}, batch, st) : lpipe<0>(data, g, tw, NoOp{}, batch, st);
  }
  static cudaError_t lfft_drift(float2* data, const LineGeom& g, const float4* tw, const DriftOp& op, int batch,
                                cudaStream_t st) {
    return lpipe<2>(data, g, tw, op, batch, st);
  }
  static cudaError_t lfft_poisson(float2* data, const LineGeom& g, const float4* tw, const PoissonOp& op, int batch,
                                  cudaStream_t st) {
    return lpipe<2>(data, g, tw, op, batch, st);
  }
  // x passes: lane group per row pair, grid-stride over warp units
  static constexpr int XNT = XCfg<N>::NT;
  static constexpr size_t XSMEM = XCfg<N>::SMEM;
  static dim3 grid_x(const RowGeom& rg, int batch, XWork* w) {
    w->pairs_per_item = rg.nrows / 2;
    w->batch = batch;
    const long long pairs = (long long)w->pairs_per_item * batch;
    const long long units = (pairs + XCfg<N>::GROUPS - 1) / XCfg<N>::GROUPS;
    long long ctas = (units + XCfg<N>::WARPS - 1) / XCfg<N>::WARPS;
    const long long cap = 152LL * 6;
    return dim3((unsigned)(ctas < cap ? ctas : cap));
  }
  static cudaError_t xfft(float2* data, const RowGeom& rg, const float4* tw, bool inv, float scale, int batch,
                          cudaStream_t st) {
    cudaError_t e;
    XWork w;
    const dim3 gr = grid_x(rg, batch, &w);
    if (inv) {
      if ((e = prep_once<k_xw_fft<N, true>>(XSMEM)) != cudaSuccess) return e;
      k_xw_fft<N, true><<<gr, XNT, XSMEM, st>>>(data, rg, tw, scale, w);
      ++tl_kernel_launches;
    } else {
      if ((e = prep_once<k_xw_fft<N, false>>(XSMEM)) != cudaSuccess) return e;
      k_xw_fft<N, false><<<gr, XNT, XSMEM, st>>>(data, rg, tw, scale, w);
      ++tl_kernel_launches;
    }
    return cudaGetLastError();
  }
  // Staged x passes: the layout conditions of their bulk copies.  Rows of
  // 16-byte multiples at 16-byte aligned addresses (the half spectrum with the
  // even pitch nx/2 + 2), and units of GROUPS row pairs inside one batch item.
  using XS = XStage<N>;
  static bool x_staged_ok(const RowGeom& rg, long long hpitch, const void* p0, const void* p1, const void* p2) {
    // the staged copies take XS::HP entries of an H row (the pitch may be wider, and even)
    if (rg.impl != X_IMPL_STAGED || hpitch < XS::HP || hpitch % 2 != 0 || rg.pitch != N) return false;
    if ((rg.nrows / 2) % XCfg<N>::GROUPS != 0 || rg.nrows % 2 != 0) return false;
    for (const void* p : {p0, p1, p2})
      if (reinterpret_cast<uintptr_t>(p) % 16) return false;
    return true;
  }
  template <auto K>
  static dim3 grid_xs(const RowGeom& rg, int batch, XWork* w, size_t smem = XS::SMEM) {
    w->pairs_per_item = rg.nrows / 2;
    w->batch = batch;
    const long long units = (long long)w->pairs_per_item * batch / XCfg<N>::GROUPS;
    const long long ctas = (units + XCfg<N>::WARPS - 1) / XCfg<N>::WARPS;
    const long long cap = (long long)resident_ctas<K>(XNT, smem) * sm_count();
    return dim3((unsigned)(ctas < cap ? ctas : cap));
  }
  template <bool CEN>
  static cudaError_t x_inv_rho_t(float2* psi, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                                 const float4* tw, const RhoArgs& a, int batch, cudaStream_t st) {
    cudaError_t e;
    XWork w;
    if (x_staged_ok(rg, hpitch, psi, H, a.rho_b) && (!a.rho_b || (a.rb_bstride * 4) % 16 == 0)) {
      constexpr auto K = k_xs_inv_rho<N, CEN>;
      if ((e = prep_once<K>(XS::SMEM)) != cudaSuccess) return e;
      const dim3 gr = grid_xs<K>(rg, batch, &w);
      K<<<gr, XNT, XS::SMEM, st>>>(psi, H, rg, hpitch, hbstride, tw, a, w);
      ++tl_kernel_launches;
      return cudaGetLastError();
    }
    const dim3 gr = grid_x(rg, batch, &w);
    if ((e = prep_once<k_xw_inv_rho<N, CEN>>(XSMEM)) != cudaSuccess) return e;
    k_xw_inv_rho<N, CEN><<<gr, XNT, XSMEM, st>>>(psi, H, rg, hpitch, hbstride, tw, a, w);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }
  static cudaError_t x_inv_rho(float2* psi, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                               const float4* tw, const RhoArgs& a, int batch, cudaStream_t st) {
    return a.centre ? x_inv_rho_t<true>(psi, H, rg, hpitch, hbstride, tw, a, batch, st)
                    : x_inv_rho_t<false>(psi, H, rg, hpitch, hbstride, tw, a, batch, st);
  }
  template <bool FWD>
  static cudaError_t x_kick_t(const float2* psi_in, float2* psi, const float2* H, const RowGeom& rg, long long hpitch,
                              long long hbstride, const float4* tw, const KickArgs& a, int batch, cudaStream_t st) {
    cudaError_t e;
    XWork w;
    if (x_staged_ok(rg, hpitch, psi_in, psi, H)) {
      constexpr auto K = k_xs_kick<N, FWD>;
      if ((e = prep_once<K>(XS::SMEM)) != cudaSuccess) return e;
      const dim3 gr = grid_xs<K>(rg, batch, &w);
      K<<<gr, XNT, XS::SMEM, st>>>(psi_in, psi, H, rg, hpitch, hbstride, tw, a, w);
      ++tl_kernel_launches;
      return cudaGetLastError();
    }
    const dim3 gr = grid_x(rg, batch, &w);
    if ((e = prep_once<k_xw_kick<N, FWD>>(XSMEM)) != cudaSuccess) return e;
    k_xw_kick<N, FWD><<<gr, XNT, XSMEM, st>>>(psi_in, psi, H, rg, hpitch, hbstride, tw, a, w);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }
  static cudaError_t x_kick(const float2* psi_in, float2* psi, const float2* H, const RowGeom& rg, long long hpitch,
                            long long hbstride, const float4* tw, const KickArgs& a, bool fwd, int batch,
                            cudaStream_t st) {
    return fwd ? x_kick_t<true>(psi_in, psi, H, rg, hpitch, hbstride, tw, a, batch, st)
               : x_kick_t<false>(psi_in, psi, H, rg, hpitch, hbstride, tw, a, batch, st);
  }
  static cudaError_t x_c2r(const float2* H, float* out, const RowGeom& rg, long long hpitch, long long hbstride,
                           const float4* tw, int batch, cudaStream_t st) {
    cudaError_t e;
    XWork w;
    const dim3 gr = grid_x(rg, batch, &w);
    if ((e = prep_once<k_xw_c2r<N>>(XSMEM)) != cudaSuccess) return e;
    k_xw_c2r<N><<<gr, XNT, XSMEM, st>>>(H, out, rg, hpitch, hbstride, tw, w);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }
  static cudaError_t x_r2c(const float* in, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                           const float4* tw, const float* shift, int batch, cudaStream_t st) {
    cudaError_t e;
    XWork w;
    const dim3 gr = grid_x(rg, batch, &w);
    if ((e = prep_once<k_xw_r2c<N>>(XSMEM)) != cudaSuccess) return e;
    k_xw_r2c<N><<<gr, XNT, XSMEM, st>>>(in, H, rg, hpitch, hbstride, tw, shift, w);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }
  // host: the four stage-major twiddle tables of this axis length (TW_TABLES x N)
  static void fill_twiddles(float4* out) {
    auto make = [](long long m) {
      const double a = -2.0 * 3.14159265358979323846 * (double)m / (double)N;
      return pack_twiddle(std::cos(a), std::sin(a));
    };
    for (int q = 0; q < TW_TABLES * N; ++q) out[q] = make_float4(1.f, 0.f, 0.f, 0.f);
    using LF = typename Plan<N>::Fwd;
    using XF = typename XPlan<N>::Fwd;
    fill_stage_twiddles<N>(LF{}, out + TW_LINE_FWD * N, make);
    fill_stage_twiddles<N>(typename Reverse<LF>::type{}, out + TW_LINE_REV * N, make);
    fill_stage_twiddles<N>(XF{}, out + TW_X_FWD * N, make);
    fill_stage_twiddles<N>(typename Reverse<XF>::type{}, out + TW_X_REV * N, make);
  }
  static cudaError_t adj_kick(float2* lam, const float2* H, float2* Hmu, const RowGeom& rg, long long hpitch,
                              long long hbstride, const float4* tw, const KickArgs& a, const AdjArgs& j, int batch,
                              cudaStream_t st) {
    cudaError_t e;
    XWork w;
    // staged where its three slots still leave 3 or more CTAs per SM
    using XA = XStageAdj<N>;
    if constexpr (XA::MINB_RAW >= 3) {
      if (x_staged_ok(rg, hpitch, lam, H, j.pre)) {
        constexpr auto K = k_xs_adj_kick<N>;
        if ((e = prep_once<K>(XA::SMEM)) != cudaSuccess) return e;
        const dim3 gr = grid_xs<K>(rg, batch, &w, XA::SMEM);
        K<<<gr, XNT, XA::SMEM, st>>>(lam, H, Hmu, rg, hpitch, hbstride, tw, a, j, w);
        ++tl_kernel_launches;
        return cudaGetLastError();
      }
    }
    const dim3 gr = grid_x(rg, batch, &w);
    if ((e = prep_once<k_xw_adj_kick<N>>(XSMEM)) != cudaSuccess) return e;
    k_xw_adj_kick<N><<<gr, XNT, XSMEM, st>>>(lam, H, Hmu, rg, hpitch, hbstride, tw, a, j, w);
    ++tl_kernel_launches;
    return cudaGetLastError();
  }
  static cudaError_t adj_apply(float2* lam, const float2* Hmu, const RowGeom& rg, long long hpitch, long long hbstride,
                               const float4* tw, const AdjArgs& j, bool fwd, int batch, cudaStream_t st) {
    cudaError_t e;
    XWork w;
    const dim3 gr = grid_x(rg, batch, &w);
    if (fwd) {
      if ((e = prep_once<k_xw_adj_apply<N, true>>(XSMEM)) != cudaSuccess) return e;
      k_xw_adj_apply<N, true><<<gr, XNT, XSMEM, st>>>(lam, Hmu, rg, hpitch, hbstride, tw, j, w);
      ++tl_kernel_launches;
    } else {
      if ((e = prep_once<k_xw_adj_apply<N, false>>(XSMEM)) != cudaSuccess) return e;
      k_xw_adj_apply<N, false><<<gr, XNT, XSMEM, st>>>(lam, Hmu, rg, hpitch, hbstride, tw, j, w);
      ++tl_kernel_launches;
    }
    return cudaGetLastError();
  }
  static const KernelSet* set() {
    static const KernelSet ks = {N,          &lfft,  &lfft_drift,    &lfft_poisson, &xfft,     &x_inv_rho,
                                 &x_kick,    &x_c2r, &x_r2c,         &fill_twiddles, &adj_kick, &adj_apply};
    return &ks;
  }
};

}  // namespace wdm

#define WDM_INSTANTIATE(N) \
  namespace wdm {          \
  const KernelSet* ks_##N() { return Launch<N>::set(); } \
  }
