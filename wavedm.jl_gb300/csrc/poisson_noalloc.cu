// wdm_poisson_noalloc: the Poisson solve of wdm_poisson without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Everything the solve needs beyond its input and output lives in one
// file-scope device array, g_noalloc_scratch (NOALLOC_BYTES, about 8.3 MiB,
// held by every GPU that loads the library until the process exits):
//   the density half spectrum   (nx/2+1) ny nz complex64, at most NOALLOC_MAX_HALF
//   the twiddle tables          3 axes x 4 tables x 512 (hi, lo) pairs
//   the k^2 tables              3 axes x 512 floats
//   the mean-shift cells        one double sum, one float shift
// The tables are rebuilt by a kernel on every call and the sum is cleared
// before use, so a call never depends on what an earlier call left there.
// All calls share the array: calls whose work overlaps on the GPU (on two
// streams, or from two host threads) race on it and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/wavedm.h"
#include "aux_kernels.cuh"
#include "kernel_set.h"
#include "xpass_warp.cuh"

void wdm_set_global_error(const std::string& msg);

namespace {

using namespace wdm;

constexpr long long NOALLOC_MAX_HALF = 65LL * 128 * 128;  // (nx/2+1) ny nz of a 128^3 grid
constexpr int NOALLOC_MAX_AXIS = 512;
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t OFF_H = 0;
constexpr size_t OFF_TW = OFF_H + align256(sizeof(float2) * NOALLOC_MAX_HALF);
constexpr size_t OFF_K2 = OFF_TW + align256(sizeof(float4) * 3 * TW_TABLES * NOALLOC_MAX_AXIS);
constexpr size_t OFF_SUM = OFF_K2 + align256(sizeof(float) * 3 * NOALLOC_MAX_AXIS);
constexpr size_t OFF_SHIFT = OFF_SUM + 256;
constexpr size_t NOALLOC_BYTES = OFF_SHIFT + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Per-device address of g_noalloc_scratch (host code may not use the symbol
// itself as a device pointer).  Filled on the first call on each device.
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char* g_dev_ptr[MAX_DEVICES] = {};

wdm_status scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    wdm_set_global_error(std::string("wdm_poisson_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return WDM_ERR_CUDA;
  }
  if (dev < 0 || dev >= MAX_DEVICES) {
    wdm_set_global_error("wdm_poisson_noalloc: device index out of range");
    return WDM_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_dev_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      wdm_set_global_error(std::string("wdm_poisson_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return WDM_ERR_CUDA;
    }
    g_dev_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_dev_ptr[dev];
  return WDM_OK;
}

// W_N^m as an FP32 (hi, lo) pair from the FP64 value (pack_twiddle layout).
__device__ float4 twiddle_entry(long long m, int n) {
  double s, c;
  sincospi(-2.0 * (double)m / (double)n, &s, &c);
  return pack_twiddle(c, s);
}

// Entry idx of the stage-major table of a radix order (same layout as
// fill_stage_twiddles on the host).
template <int N, int... Rs>
__device__ float4 stage_entry(Radices<Rs...>, int idx) {
  const int rad[] = {Rs...};
  int ns = 1, off = 0;
  for (int s = 0; s < (int)sizeof...(Rs); ++s) {
    const int R = rad[s];
    const int cnt = ns * (R - 1);
    if (idx < off + cnt) {
      const int jm = (idx - off) / (R - 1), k = (idx - off) % (R - 1) + 1;
      return twiddle_entry((long long)k * jm * (N / (ns * R)), N);
    }
    off += cnt;
    ns *= R;
  }
  return make_float4(1.f, 0.f, 0.f, 0.f);
}

template <int N>
__global__ void k_fill_twiddles(float4* out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= TW_TABLES * N) return;
  const int table = q / N, idx = q % N;
  using LF = typename Plan<N>::Fwd;
  using XF = typename XPlan<N>::Fwd;
  float4 v;
  if (table == TW_LINE_FWD) v = stage_entry<N>(LF{}, idx);
  else if (table == TW_LINE_REV) v = stage_entry<N>(typename Reverse<LF>::type{}, idx);
  else if (table == TW_X_FWD) v = stage_entry<N>(XF{}, idx);
  else v = stage_entry<N>(typename Reverse<XF>::type{}, idx);
  out[q] = v;
}

// k^2 of FFT index m on an axis of n points and period L (fftfreq order)
__global__ void k_fill_k2(float* out, int n, double L) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const int s = (m < (n + 1) / 2) ? m : m - n;
  const double k = 2.0 * 3.14159265358979323846 * s / L;
  out[m] = (float)(k * k);
}

cudaError_t fill_twiddles_dev(int n, float4* out, cudaStream_t st) {
  const int threads = 128, blocks = (TW_TABLES * n + threads - 1) / threads;
  switch (n) {
#define WDM_TW_CASE(N_) \
  case N_: k_fill_twiddles<N_><<<blocks, threads, 0, st>>>(out); break;
    WDM_TW_CASE(8) WDM_TW_CASE(12) WDM_TW_CASE(16) WDM_TW_CASE(24) WDM_TW_CASE(32) WDM_TW_CASE(48)
    WDM_TW_CASE(64) WDM_TW_CASE(96) WDM_TW_CASE(128) WDM_TW_CASE(192) WDM_TW_CASE(256) WDM_TW_CASE(384)
    WDM_TW_CASE(512)
#undef WDM_TW_CASE
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

wdm_status fail_noalloc(wdm_status s, const std::string& msg) {
  wdm_set_global_error("wdm_poisson_noalloc: " + msg);
  return s;
}

}  // namespace

extern "C" wdm_status wdm_poisson_noalloc(const float* rho, float* phi, int32_t nx, int32_t ny, int32_t nz,
                                          double lx, double ly, double lz, double poisson_coeff, void* stream) {
  if (!rho || !phi) return fail_noalloc(WDM_ERR_INVALID, "null rho/phi");
  const int n[3] = {nx, ny, nz};
  const KernelSet* ks[3];
  for (int a = 0; a < 3; ++a) {
    ks[a] = kernels_for(n[a]);
    if (!ks[a]) return fail_noalloc(WDM_ERR_UNSUPPORTED, "axis length " + std::to_string(n[a]) + " has no FFT plan");
  }
  if (!(lx > 0 && ly > 0 && lz > 0)) return fail_noalloc(WDM_ERR_INVALID, "box lengths must be > 0");
  const int nxh = nx / 2 + 1;
  const long long nhalf = (long long)nxh * ny * nz;
  if (nhalf > NOALLOC_MAX_HALF)
    return fail_noalloc(WDM_ERR_INVALID, "grid too large for the static scratch: (nx/2+1)*ny*nz = " +
                                             std::to_string(nhalf) + " > " + std::to_string(NOALLOC_MAX_HALF) +
                                             " (a 128^3 grid); use wdm_poisson");
  unsigned char* base = nullptr;
  wdm_status s = scratch_on_current_device(&base);
  if (s != WDM_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2* H = reinterpret_cast<float2*>(base + OFF_H);
  float4* tw[3];
  float* k2[3];
  for (int a = 0; a < 3; ++a) {
    tw[a] = reinterpret_cast<float4*>(base + OFF_TW) + (size_t)a * TW_TABLES * NOALLOC_MAX_AXIS;
    k2[a] = reinterpret_cast<float*>(base + OFF_K2) + (size_t)a * NOALLOC_MAX_AXIS;
  }
  double* sums = reinterpret_cast<double*>(base + OFF_SUM);
  float* shift = reinterpret_cast<float*>(base + OFF_SHIFT);
  const double L[3] = {lx, ly, lz};
  cudaError_t e = cudaSuccess;
  for (int a = 0; a < 3 && e == cudaSuccess; ++a) {
    e = fill_twiddles_dev(n[a], tw[a], st);
    if (e == cudaSuccess) {
      k_fill_k2<<<(n[a] + 127) / 128, 128, 0, st>>>(k2[a], n[a], L[a]);
      e = cudaGetLastError();
    }
  }
  const long long ncell = (long long)nx * ny * nz;
  RowGeom rg;
  rg.nrows = ny * nz;
  rg.ny = ny;
  rg.pitch = nx;
  rg.bstride = ncell;
  LineGeom gy;
  gy.nlines = nxh * nz;
  gy.nxa = nxh;
  gy.outer = (long long)ny * nxh;
  gy.pstride = nxh;
  gy.bstride = nhalf;
  LineGeom gz;
  gz.nlines = nxh * ny;
  gz.nxa = nxh;
  gz.outer = nxh;
  gz.pstride = (long long)ny * nxh;
  gz.bstride = nhalf;
  PoissonOp po;
  po.kx2 = k2[0];
  po.ky2 = k2[1];
  po.kz2 = k2[2];
  po.coef = (float)(-poisson_coeff / ((double)nx * ny * nz));
  if (e == cudaSuccess) e = launch_mean_shift(rho, false, ncell, 1, sums, shift, 0.0, st);
  if (e == cudaSuccess) e = ks[0]->x_r2c(rho, H, rg, nxh, nhalf, tw[0], shift, 1, st);
  if (e == cudaSuccess) e = ks[1]->lfft(H, gy, tw[1], false, 1, st);
  if (e == cudaSuccess) e = ks[2]->lfft_poisson(H, gz, tw[2], po, 1, st);
  if (e == cudaSuccess) e = ks[1]->lfft(H, gy, tw[1], true, 1, st);
  if (e == cudaSuccess) e = ks[0]->x_c2r(H, phi, rg, nxh, nhalf, tw[0], 1, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_noalloc(WDM_ERR_CUDA, cudaGetErrorString(e));
  return WDM_OK;
}
