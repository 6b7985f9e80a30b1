// Persistent ensemble step (k_ensemble): the passes of every member context,
// of every step of a call, in one cooperative launch.
//
// The grid is exactly the CTAs that fit on the GPU at once (cooperative
// launch), 8 warps each.  A pass is one phase: every CTA works through its
// share of every member's units (warp units of the x passes, tiles of 16 lines
// of the line passes), one member after another with no barrier between
// members, so the small grids of one size fill the machine together with the
// others instead of one after another.  Phases are separated by a grid-wide
// barrier whose waits are bounded: a CTA that has waited WAIT_LIMIT_NS (or
// WAIT_MAX_POLLS polls) records WDM_DEVERR_BARRIER, raises the abort word and
// leaves, and every other CTA leaves at its next barrier, so the launch always
// ends.  Members keep their buffers; the pass bodies are those of the direct
// x passes and of the line passes (xw_kick_units, xw_inv_rho_units, and
// lfft_pipe_run, which prefetches tiles by cp.async), all with the arithmetic of
// the per-pass launches, so a step equals those launches bit for bit.
#include "ensemble.cuh"

#include <algorithm>

#include "../../include/wavedm.h"

namespace wdm {
namespace {

constexpr int ENS_WARPS = ENS_THREADS / 32;

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier number `epoch` (1, 2, ... within a launch).  The CTA's
// writes before it are visible to every CTA after it.  false: the wait was
// abandoned (here or by another CTA); the caller leaves the kernel.
__device__ bool ens_grid_sync(unsigned* words, unsigned epoch, int* err) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    red_release_add(words, 1u);
    const unsigned target = epoch * gridDim.x;
    int ok = 1;
    if (ld_acquire(words) < target) {
      const unsigned long long t0 = globaltimer_ns();
      for (unsigned i = 1;; ++i) {
        if (ld_acquire(words) >= target) break;
        if (ld_acquire(words + 1) != 0u) {
          ok = 0;
          break;
        }
        if (i >= WAIT_MAX_POLLS || ((i & 255u) == 0 && globaltimer_ns() - t0 > WAIT_LIMIT_NS)) {
          if (err) atomicOr(err, WDM_DEVERR_BARRIER);
          atomicExch(words + 1, 1u);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// ---------------------------------------------------------------------------
// pass bodies for one member, over the virtual block vb of vg
// ---------------------------------------------------------------------------
template <int N>
constexpr size_t x_smem() {
  return sizeof(float2) * (2 * (size_t)N + (size_t)ENS_WARPS * XCfg<N>::GROUPS * XCfg<N>::NP);
}

template <int N, int NTAB>
constexpr size_t line_smem() {
  return sizeof(float2) * (2 * (size_t)NTAB * N + (size_t)(ENS_THREADS / threads_for<N>()) * 2 * N * LBUF);
}

template <int N, bool FWD>
__device__ __noinline__ void x_kick(const EnsMember& m, const KickArgs& a, unsigned char* sm, int vb, int vg) {
  using C = XCfg<N>;
  float4* tw = reinterpret_cast<float4*>(sm);
  load_twiddles(tw, m.twx + TW_X_FWD * N, N);
  __syncthreads();
  const int warp = threadIdx.x >> 5, g = (threadIdx.x & 31) / C::T;
  float2* buf = reinterpret_cast<float2*>(sm) + 2 * N + (size_t)(warp * C::GROUPS + g) * C::NP;
  const XWork w{m.rows.nrows / 2, m.batch};
  const XSlice sl{(long long)vb * ENS_WARPS + warp, (long long)vg * ENS_WARPS, tw, buf};
  xw_kick_units<N, FWD>(m.psi, m.psi, m.H, m.rows, m.hpitch, m.nhalf, a, w, sl);
  __syncthreads();
}

template <int N>
__device__ __noinline__ void x_rho(const EnsMember& m, unsigned char* sm, int vb, int vg) {
  using C = XCfg<N>;
  float4* tw = reinterpret_cast<float4*>(sm);
  load_twiddles(tw, m.twx + TW_X_FWD * N, N);
  __syncthreads();
  const int warp = threadIdx.x >> 5, g = (threadIdx.x & 31) / C::T;
  float2* buf = reinterpret_cast<float2*>(sm) + 2 * N + (size_t)(warp * C::GROUPS + g) * C::NP;
  const XWork w{m.rows.nrows / 2, m.batch};
  const XSlice sl{(long long)vb * ENS_WARPS + warp, (long long)vg * ENS_WARPS, tw, buf};
  if (m.rho.centre) xw_inv_rho_units<N, true>(m.psi, m.H, m.rows, m.hpitch, m.nhalf, m.rho, w, sl);
  else xw_inv_rho_units<N, false>(m.psi, m.H, m.rows, m.hpitch, m.nhalf, m.rho, w, sl);
  __syncthreads();
}

// Line pass: the CTA's threads form SUB groups of threads_for<N>() that take
// SUB consecutive tiles per round, each group prefetching its next tile by
// cp.async into its own double buffer (lfft_pipe_run; all groups reach the
// same barriers).
template <int N, int MODE, class Op>
__device__ __noinline__ void lines(float2* data, const LineGeom& g, const float4* twg, const Op& op, int batch,
                                   unsigned char* sm, int vb, int vg) {
  constexpr int NTAB = MODE == 2 ? 2 : 1;
  constexpr int NT = threads_for<N>();
  constexpr int SUB = ENS_THREADS / NT;
  static_assert(SUB * NT == ENS_THREADS, "tile groups fill the CTA");
  float4* tw = reinterpret_cast<float4*>(sm);
  load_twiddles(tw, twg + TW_LINE_FWD * N, NTAB * N);  // visible after the first round's barrier
  const int sub = threadIdx.x / NT, tid = threadIdx.x % NT;
  float2* bufs = reinterpret_cast<float2*>(sm) + 2 * NTAB * N + (size_t)sub * 2 * N * LBUF;
  lfft_pipe_run<N, MODE, Op>(data, g, tw, op, batch, bufs, tid, (long long)vb * SUB, (long long)vg * SUB, sub);
  __syncthreads();
}

#define WDM_ENS_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128)

__device__ void pass_x_kick(const EnsMember& m, const KickArgs& a, bool fwd, unsigned char* sm, int vb, int vg) {
  switch (m.nx) {
#define WDM_CASE(N_)                            \
  case N_:                                      \
    if (fwd) x_kick<N_, true>(m, a, sm, vb, vg);  \
    else x_kick<N_, false>(m, a, sm, vb, vg);     \
    break;
    WDM_ENS_SIZES(WDM_CASE)
#undef WDM_CASE
  }
}

__device__ void pass_x_rho(const EnsMember& m, unsigned char* sm, int vb, int vg) {
  switch (m.nx) {
#define WDM_CASE(N_) \
  case N_: x_rho<N_>(m, sm, vb, vg); break;
    WDM_ENS_SIZES(WDM_CASE)
#undef WDM_CASE
  }
}

template <int MODE, class Op>
__device__ void pass_lines(int n, float2* data, const LineGeom& g, const float4* tw, const Op& op, int batch,
                           unsigned char* sm, int vb, int vg) {
  switch (n) {
#define WDM_CASE(N_) \
  case N_: lines<N_, MODE, Op>(data, g, tw, op, batch, sm, vb, vg); break;
    WDM_ENS_SIZES(WDM_CASE)
#undef WDM_CASE
  }
}

// The tide's frame of item b of a member for its next kick (the frame words
// of the last density pass; the kicks' tensor is constant during a call).
__device__ void member_frame(const EnsMember& m, int b) {
  const KickArgs& a = m.kick_full;
  float T6[6];
  for (int q = 0; q < 6; ++q) T6[q] = a.T6b ? a.T6b[6 * b + q] : a.T6[q];
  const double x0[3] = {a.x0, a.y0, a.z0}, d[3] = {a.dx, a.dy, a.dz};
  tide_frame_of(m.frame + 4 * b, T6, m.centre + (long long)CENTRE_WORDS * b, m.centre_mode, m.nx, m.ny, x0, d);
}

// Pass p (0..7: P1..P8 of the step; 8: the closing half kick) of one member.
__device__ void member_pass(const EnsMember& m, int p, int s, int mode, unsigned char* sm, int vb, int vg) {
  switch (p) {
    case 0: {
      const bool full = mode == WDM_STEP_LIE || (mode == WDM_STEP_STRANG && s > 0);  // interior half kicks merged
      pass_x_kick(m, full ? m.kick_full : m.kick_half, true, sm, vb, vg);
      break;
    }
    case 1: pass_lines<0>(m.ny, m.psi, m.ly_psi, m.twy, NoOp{}, m.batch, sm, vb, vg); break;
    case 2: pass_lines<2>(m.nz, m.psi, m.lz_psi, m.twz, m.drift, m.batch, sm, vb, vg); break;
    case 3: pass_lines<1>(m.ny, m.psi, m.ly_psi, m.twy, NoOp{}, m.batch, sm, vb, vg); break;
    case 4: pass_x_rho(m, sm, vb, vg); break;
    case 5: pass_lines<0>(m.ny, m.H, m.ly_h, m.twy, NoOp{}, m.batch, sm, vb, vg); break;
    case 6: pass_lines<2>(m.nz, m.H, m.lz_h, m.twz, m.poisson, m.batch, sm, vb, vg); break;
    case 7: pass_lines<1>(m.ny, m.H, m.ly_h, m.twy, NoOp{}, m.batch, sm, vb, vg); break;
    default: pass_x_kick(m, m.kick_half, false, sm, vb, vg); break;
  }
}

__global__ void __launch_bounds__(ENS_THREADS, 2)
k_ensemble(const EnsMember* __restrict__ mem, int nmem, int nsteps, int mode, unsigned* words, int* err) {
  extern __shared__ __align__(16) unsigned char esm[];
  const int vg = gridDim.x;
  unsigned epoch = 0;
  for (int s = 0; s < nsteps; ++s) {
    for (int p = 0; p < 8; ++p) {
      // the tide-frame words the density pass (p = 4) fills start at zero (the
      // frames of phase 0's kicks came from them before the last barrier), and
      // the frames of the next kicks come from the filled words in phase 7
      if (p == 3 && blockIdx.x == 0)
        for (int m = 0; m < nmem; ++m)
          if (mem[m].centre)
            for (int i = threadIdx.x; i < CENTRE_WORDS * mem[m].batch; i += blockDim.x) mem[m].centre[i] = 0ull;
      if (p == 7 && blockIdx.x == 0)
        for (int m = 0; m < nmem; ++m)
          if (mem[m].centre)
            for (int b = threadIdx.x; b < mem[m].batch; b += blockDim.x) member_frame(mem[m], b);
      for (int m = 0; m < nmem; ++m) member_pass(mem[m], p, s, mode, esm, (blockIdx.x + mem[m].rot) % vg, vg);
      if (!ens_grid_sync(words, ++epoch, err)) return;
    }
  }
  if (mode == WDM_STEP_STRANG)
    for (int m = 0; m < nmem; ++m) member_pass(mem[m], 8, nsteps, mode, esm, (blockIdx.x + mem[m].rot) % vg, vg);
}

size_t smem_for_axis(int n, int kind) {  // kind 0: x pass, 1: y lines, 2: z lines (two tables)
  switch (n) {
#define WDM_CASE(N_) \
  case N_: return kind == 0 ? x_smem<N_>() : (kind == 1 ? line_smem<N_, 1>() : line_smem<N_, 2>());
    WDM_ENS_SIZES(WDM_CASE)
#undef WDM_CASE
  }
  return 0;
}

__global__ void k_tide_frame(const unsigned long long* __restrict__ words, KickArgs a, int mode, int nx, int ny,
                             int batch, float* __restrict__ frame) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < batch; b += gridDim.x * blockDim.x) {
    float T6[6];
    for (int q = 0; q < 6; ++q) T6[q] = a.T6b ? a.T6b[6 * b + q] : a.T6[q];
    const double x0[3] = {a.x0, a.y0, a.z0}, d[3] = {a.dx, a.dy, a.dz};
    tide_frame_of(frame + 4 * b, T6, words + (long long)CENTRE_WORDS * b, mode, nx, ny, x0, d);
  }
}

}  // namespace

cudaError_t launch_tide_frame(const unsigned long long* words, const KickArgs& a, int mode, int nx, int ny, int batch,
                              float* frame, cudaStream_t st) {
  k_tide_frame<<<(batch + 127) / 128, 128, 0, st>>>(words, a, mode, nx, ny, batch, frame);
  ++tl_kernel_launches;
  return cudaGetLastError();
}

bool ens_size_supported(int n) {
  switch (n) {
#define WDM_CASE(N_) case N_:
    WDM_ENS_SIZES(WDM_CASE)
#undef WDM_CASE
    return true;
  }
  return false;
}

size_t ens_smem_bytes(const int* nx, const int* ny, const int* nz, int nmem) {
  size_t s = 0;
  for (int i = 0; i < nmem; ++i) {
    s = std::max(s, smem_for_axis(nx[i], 0));
    s = std::max(s, smem_for_axis(ny[i], 1));
    s = std::max(s, smem_for_axis(nz[i], 2));
  }
  return s;
}

int ens_grid(size_t smem) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (smem > 48 * 1024 && cudaFuncSetAttribute(k_ensemble, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                              cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ensemble, ENS_THREADS, smem) != cudaSuccess) return 0;
  return per * sms;
}

cudaError_t ens_launch(const EnsMember* mem, int nmem, int nsteps, int mode, unsigned* words, int* err, size_t smem,
                       int grid, cudaStream_t st) {
  void* args[] = {(void*)&mem, (void*)&nmem, (void*)&nsteps, (void*)&mode, (void*)&words, (void*)&err};
  ++tl_kernel_launches;
  return cudaLaunchCooperativeKernel((const void*)k_ensemble, dim3(grid), dim3(ENS_THREADS), args, smem, st);
}

}  // namespace wdm
