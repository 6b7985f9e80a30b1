// Auxiliary kernels: density output, FP64 diagnostics reductions, CIC.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace wdm {

// CIC particle: base cell (wrapped into the grid) and fractional offsets in
// [0, 1) along each axis, built in FP64 on the host; m = mass / dV.
struct CicParticle {
  int i[3];
  float f[3];
  float m;
};

enum {
  RED_MASS = 0,  // sum rho
  RED_MAX,       // max rho
  RED_ARG,       // flat index of the max
  RED_MX,        // sum rho x
  RED_MY,
  RED_MZ,
  RED_W,         // sum rho Phi over interior cells
  RED_K,         // sum (rho v)^2 / rho over interior cells
  RED_Q,         // sum |grad sqrt rho|^2 over interior cells
  RED_PX,        // sum rho v (= Im(conj(psi) grad psi)) over interior cells
  RED_PY,
  RED_PZ,
  RED_PHIMAX,    // max |Phi|
  RED_SW,        // z-slice zmid: sum rho, sum rho r, sum rho r^2 (r from the coordinate origin)
  RED_SWR,
  RED_SWR2,
  RED_FIELDS
};
// fields combined by max rather than by sum (RED_ARG travels with RED_MAX)
__host__ __device__ constexpr bool red_is_max(int q) { return q == RED_MAX || q == RED_ARG || q == RED_PHIMAX; }

struct RedGeom {
  int nx, ny, nz;
  double dx, dy, dz, x0, y0, z0;
  int zmid;  // z index of the slice the RED_SW* sums cover
};

// Lagrangian radii: per squared cell distance key = di^2 + dj^2 + dk^2 from
// cell (cx, cy, cz), the FP64 sum of rho over the cells at that distance;
// then, for up to RADII_KEYS keys, the smallest nonzero rho (as the bits of a
// positive double) over their cells.
constexpr int RADII_KEYS = 16;
struct RadiiKeys {
  long long k[RADII_KEYS];
  int n;
};
cudaError_t launch_radii_hist(const float2* psi, int nx, int ny, int nz, int cx, int cy, int cz, double* wsum,
                              cudaStream_t st);
cudaError_t launch_radii_min(const float2* psi, int nx, int ny, int nz, int cx, int cy, int cz, const RadiiKeys& keys,
                             unsigned long long* wmin, cudaStream_t st);

cudaError_t launch_abs2(const float2* psi, float* out, long long n, cudaStream_t st);
// Adjoint seed of L = sum (|psi|^2 - rho_t)^2 dV: lam = 4 (|psi|^2 - rho_t) psi dV,
// loss[b] += sum (|psi|^2 - rho_t)^2 dV (FP64), per batch item of n cells.
cudaError_t launch_adj_seed(const float2* psi, const float* rho_t, float2* lam, long long n, int batch, double dV,
                            double* loss, cudaStream_t st);
// bounded mbarrier wait that runs out (self-test): out[0] error bits, out[1] ns waited
cudaError_t launch_bounded_wait_probe(unsigned long long limit_ns, unsigned long long* out, cudaStream_t st);
// out[2i], out[2i+1] = series sin, cos of h[i] (wdm_math.cuh), for self-tests
cudaError_t launch_sincos_half(const float* h, float* out, long long n, cudaStream_t st);
// shift[b] = mean over item b of |data|^2 (complex_in) or of data (float), + add
cudaError_t launch_mean_shift(const void* data, bool complex_in, long long n, int batch, double* sums, float* shift,
                              double add, cudaStream_t st);
cudaError_t launch_reduce(const float2* psi, const float* phi, const RedGeom& g, double* partials, int nblocks,
                          int batch, cudaStream_t st);
// CIC deposit of the particles into rho, which must be zero; rows (ny * nz
// ints, may be null) flags the x rows that hold deposited mass.  The deposit
// of static particles is kept: every density pass reads its flagged rows, and
// it is cleared only when the particles change.
cudaError_t launch_cic_deposit(float* rho, const CicParticle* p, long long n, int nx, int ny, int nz, int* rows,
                               cudaStream_t st);
cudaError_t launch_cic_interp(const float* field, const CicParticle* p, long long n, int nx, int ny, int nz,
                              double* out, cudaStream_t st);

}  // namespace wdm
