// Launchers of the pass kernels for one axis length N (included by sizes_*.cu).
#pragma once
#include "kernel_set.h"

namespace wdm {

// Opt a kernel in to more than 48 KB of dynamic shared memory, once per process.
template <auto K>
static cudaError_t prep_once(size_t smem) {
  static const cudaError_t e =
      smem > 48 * 1024 ? cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) : cudaSuccess;
  return e;
}

template <int N>
struct Launch {
  static constexpr int NT = threads_for<N>();
  static constexpr size_t SM = smem_bytes<N>();

  static dim3 grid_lines(int nlines, int batch) { return dim3((nlines + LINES - 1) / LINES, batch); }

  static cudaError_t lfft(float2* data, const LineGeom& g, const float2* tw, bool inv, int batch, cudaStream_t st) {
    if (g.nlines <= 0) return cudaSuccess;
    cudaError_t e;
    if (inv) {
      if ((e = prep_once<k_lfft<N, true>>(SM)) != cudaSuccess) return e;
      k_lfft<N, true><<<grid_lines(g.nlines, batch), NT, SM, st>>>(data, g, tw);
    } else {
      if ((e = prep_once<k_lfft<N, false>>(SM)) != cudaSuccess) return e;
      k_lfft<N, false><<<grid_lines(g.nlines, batch), NT, SM, st>>>(data, g, tw);
    }
    return cudaGetLastError();
  }
  static cudaError_t lfft_drift(float2* data, const LineGeom& g, const float2* tw, const DriftOp& op, int batch,
                                cudaStream_t st) {
    cudaError_t e;
    if ((e = prep_once<k_lfft_mid<N, DriftOp>>(SM)) != cudaSuccess) return e;
    k_lfft_mid<N, DriftOp><<<grid_lines(g.nlines, batch), NT, SM, st>>>(data, g, tw, op);
    return cudaGetLastError();
  }
  static cudaError_t lfft_poisson(float2* data, const LineGeom& g, const float2* tw, const PoissonOp& op, int batch,
                                  cudaStream_t st) {
    cudaError_t e;
    if ((e = prep_once<k_lfft_mid<N, PoissonOp>>(SM)) != cudaSuccess) return e;
    k_lfft_mid<N, PoissonOp><<<grid_lines(g.nlines, batch), NT, SM, st>>>(data, g, tw, op);
    return cudaGetLastError();
  }
  static cudaError_t xfft(float2* data, const RowGeom& rg, const float2* tw, bool inv, float scale, int batch,
                          cudaStream_t st) {
    cudaError_t e;
    if (inv) {
      if ((e = prep_once<k_xfft<N, true>>(SM)) != cudaSuccess) return e;
      k_xfft<N, true><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(data, rg, tw, scale);
    } else {
      if ((e = prep_once<k_xfft<N, false>>(SM)) != cudaSuccess) return e;
      k_xfft<N, false><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(data, rg, tw, scale);
    }
    return cudaGetLastError();
  }
  static cudaError_t x_inv_rho(float2* psi, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                               const float2* tw, const RhoArgs& a, int batch, cudaStream_t st) {
    cudaError_t e;
    if ((e = prep_once<k_x_inv_rho<N>>(SM)) != cudaSuccess) return e;
    k_x_inv_rho<N><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(psi, H, rg, hpitch, hbstride, tw, a);
    return cudaGetLastError();
  }
  static cudaError_t x_kick(float2* psi, const float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                            const float2* tw, const KickArgs& a, bool fwd, int batch, cudaStream_t st) {
    cudaError_t e;
    if (fwd) {
      if ((e = prep_once<k_x_kick<N, true>>(SM)) != cudaSuccess) return e;
      k_x_kick<N, true><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(psi, H, rg, hpitch, hbstride, tw, a);
    } else {
      if ((e = prep_once<k_x_kick<N, false>>(SM)) != cudaSuccess) return e;
      k_x_kick<N, false><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(psi, H, rg, hpitch, hbstride, tw, a);
    }
    return cudaGetLastError();
  }
  static cudaError_t x_c2r(const float2* H, float* out, const RowGeom& rg, long long hpitch, long long hbstride,
                           const float2* tw, int batch, cudaStream_t st) {
    cudaError_t e;
    if ((e = prep_once<k_x_c2r<N>>(SM)) != cudaSuccess) return e;
    k_x_c2r<N><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(H, out, rg, hpitch, hbstride, tw);
    return cudaGetLastError();
  }
  static cudaError_t x_r2c(const float* in, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                           const float2* tw, int batch, cudaStream_t st) {
    cudaError_t e;
    if ((e = prep_once<k_x_r2c<N>>(SM)) != cudaSuccess) return e;
    k_x_r2c<N><<<grid_lines(rg.nrows, batch), NT, SM, st>>>(in, H, rg, hpitch, hbstride, tw);
    return cudaGetLastError();
  }
  static const KernelSet* set() {
    static const KernelSet ks = {N, &lfft, &lfft_drift, &lfft_poisson, &xfft, &x_inv_rho, &x_kick, &x_c2r, &x_r2c};
    return &ks;
  }
};

}  // namespace wdm

#define WDM_INSTANTIATE(N) \
  namespace wdm {          \
  const KernelSet* ks_##N() { return Launch<N>::set(); } \
  }
