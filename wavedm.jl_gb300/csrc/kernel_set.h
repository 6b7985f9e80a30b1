// Per-axis-length table of launchers for the pass kernels.  Each supported
// length N is compiled in one of the sizes_*.cu translation units (so the
// build parallelises) and exposes wdm_ks_<N>().
#pragma once
#include <cuda_runtime.h>
#include "xpass_staged.cuh"

namespace wdm {

// Kernels launched by this host thread through the KernelSet launchers (a
// pass may take more than one launch); the API layer counts launches from it.
extern thread_local long long tl_kernel_launches;

struct KernelSet {
  int n;
  // strided lines (y or z axis), C2C in place
  cudaError_t (*lfft)(float2* data, const LineGeom& g, const float4* tw, bool inv, int batch, cudaStream_t st);
  cudaError_t (*lfft_drift)(float2* data, const LineGeom& g, const float4* tw, const DriftOp& op, int batch,
                            cudaStream_t st);
  cudaError_t (*lfft_poisson)(float2* data, const LineGeom& g, const float4* tw, const PoissonOp& op, int batch,
                              cudaStream_t st);
  // contiguous rows (x axis)
  cudaError_t (*xfft)(float2* data, const RowGeom& rg, const float4* tw, bool inv, float scale, int batch,
                      cudaStream_t st);
  cudaError_t (*x_inv_rho)(float2* psi, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                           const float4* tw, const RhoArgs& a, int batch, cudaStream_t st);
  cudaError_t (*x_kick)(const float2* psi_in, float2* psi, const float2* H, const RowGeom& rg, long long hpitch,
                        long long hbstride,
                        const float4* tw, const KickArgs& a, bool fwd, int batch, cudaStream_t st);
  cudaError_t (*x_c2r)(const float2* H, float* out, const RowGeom& rg, long long hpitch, long long hbstride,
                       const float4* tw, int batch, cudaStream_t st);
  cudaError_t (*x_r2c)(const float* in, float2* H, const RowGeom& rg, long long hpitch, long long hbstride,
                       const float4* tw, const float* shift, int batch, cudaStream_t st);
  // host: fill the TW_TABLES x n stage-major twiddle tables of this axis length
  void (*fill_twiddles)(float4* out);
  // adjoint x passes (xpass_warp.cuh)
  cudaError_t (*adj_kick)(float2* lam, const float2* H, float2* Hmu, const RowGeom& rg, long long hpitch,
                          long long hbstride, const float4* tw, const KickArgs& a, const AdjArgs& j, int batch,
                          cudaStream_t st);
  cudaError_t (*adj_apply)(float2* lam, const float2* Hmu, const RowGeom& rg, long long hpitch, long long hbstride,
                           const float4* tw, const AdjArgs& j, bool fwd, int batch, cudaStream_t st);
};

const KernelSet* kernels_for(int n);

}  // namespace wdm
