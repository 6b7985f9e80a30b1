// Persistent ensemble step: every pass of every member (contexts of several
// grid sizes, each with `batch` halos) in one cooperative launch.
#pragma once
#include <cuda_runtime.h>

#include "kernel_set.h"

namespace wdm {

// One member context as the persistent kernel sees it (filled on the host,
// kept in device memory).  The kernel runs the pass bodies of the direct x
// passes and the register-tile line passes, the same arithmetic as those
// launches, so its results equal the per-pass launches of that schedule bit
// for bit.
struct EnsMember {
  int nx, ny, nz, batch;
  float2* psi;
  float2* H;
  long long hpitch, nhalf;
  const float4* twx;
  const float4* twy;
  const float4* twz;
  RowGeom rows;
  LineGeom ly_psi, lz_psi, ly_h, lz_h;
  KickArgs kick_half, kick_full;  // kicks of dt/2 and dt
  RhoArgs rho;
  DriftOp drift;
  PoissonOp poisson;
  unsigned long long* centre;     // tide-frame words to zero before each density pass (or null)
  float* frame;                   // the tide's frame per item, made from them for the next kick
  int centre_mode;                // 1 or 2 (wdm_tide_centering)
  int rot;                        // first virtual block of this member (spreads the members' tails)
};

// Device words of one launch: [0] the barrier count, [1] the abort flag (set
// by a CTA that gave up a barrier wait; the others then leave too).
enum { ENS_SYNC_WORDS = 2 };
// Error bit of an abandoned barrier wait (in the first member's error word).
enum { WDM_DEVERR_BARRIER = 4 };
constexpr int ENS_THREADS = 256;

// The tide's frame (tide_frame_of) of every batch item for the next kick with
// arguments a: one small launch after the density pass that filled `words`.
cudaError_t launch_tide_frame(const unsigned long long* words, const KickArgs& a, int mode, int nx, int ny, int batch,
                              float* frame, cudaStream_t st);

// Axis lengths the persistent kernel is built for.
bool ens_size_supported(int n);
// Dynamic shared memory the kernel needs for members with these axis lengths.
size_t ens_smem_bytes(const int* nx, const int* ny, const int* nz, int nmem);
// Co-resident CTAs of the kernel on the current device at that shared memory.
int ens_grid(size_t smem);
// nsteps steps (mode: wdm_step_mode) of all members; words: ENS_SYNC_WORDS
// zeroed device words; err: the error word for an abandoned barrier.
cudaError_t ens_launch(const EnsMember* mem, int nmem, int nsteps, int mode, unsigned* words, int* err,
                       size_t smem, int grid, cudaStream_t st);

}  // namespace wdm
