// Auxiliary kernels: density output, FP64 diagnostics reductions, CIC.
#include "aux_kernels.cuh"
#include "tma.cuh"
#include "wdm_math.cuh"

namespace wdm {

__global__ void k_sincos_half(const float* __restrict__ h, float* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s, c;
    sincos_half(h[i], &s, &c);
    out[2 * i] = s;
    out[2 * i + 1] = c;
  }
}

__global__ void k_adj_seed(const float2* __restrict__ psi, const float* __restrict__ rho_t, float2* __restrict__ lam,
                           long long n, double dV, double* __restrict__ loss) {
  const long long off = blockIdx.y * n;
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 p = psi[off + i];
    const float d = p.x * p.x + p.y * p.y - rho_t[off + i];
    const float s = (float)(4.0 * dV) * d;
    lam[off + i] = make_float2(s * p.x, s * p.y);
    acc += (double)d * d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    atomicAdd(loss + blockIdx.y, s * dV);
  }
}

cudaError_t launch_adj_seed(const float2* psi, const float* rho_t, float2* lam, long long n, int batch, double dV,
                            double* loss, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 608) blocks = 608;
  k_adj_seed<<<dim3((unsigned)blocks, batch), 256, 0, st>>>(psi, rho_t, lam, n, dV, loss);
  return cudaGetLastError();
}

// One CTA waits on an mbarrier phase that nothing completes (no arrival, no
// copy), through the same bounded wait the TMA line passes use; it records
// WDM_DEVERR_TMA_WAIT in out[0] and the nanoseconds it waited in out[1].
__global__ void k_bounded_wait_probe(unsigned long long limit_ns, unsigned long long* out) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const unsigned long long t0 = globaltimer_ns();
  const bool landed = mbar_wait_bounded(&bar, 0u, limit_ns);
  const bool all = __syncthreads_and(landed);
  if (threadIdx.x == 0) {
    out[0] = all ? 0ull : (unsigned long long)WDM_DEVERR_TMA_WAIT;
    out[1] = globaltimer_ns() - t0;
  }
}

cudaError_t launch_bounded_wait_probe(unsigned long long limit_ns, unsigned long long* out, cudaStream_t st) {
  k_bounded_wait_probe<<<1, 128, 0, st>>>(limit_ns, out);
  return cudaGetLastError();
}

cudaError_t launch_sincos_half(const float* h, float* out, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long b = (n + 255) / 256;
  k_sincos_half<<<(unsigned)(b < 4096 ? b : 4096), 256, 0, st>>>(h, out, n);
  return cudaGetLastError();
}

__global__ void k_abs2(const float2* __restrict__ psi, float* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 v = psi[i];
    out[i] = v.x * v.x + v.y * v.y;
  }
}

cudaError_t launch_abs2(const float2* psi, float* out, long long n, cudaStream_t st) {
  const int blocks = (int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
  k_abs2<<<blocks, 256, 0, st>>>(psi, out, n);
  return cudaGetLastError();
}

// One block partial per (block, batch item): RED_FIELDS doubles.  The sums
// restate src/visualization/runtime.jl:210-238 (interior cells, second-order
// central differences) and src/simulation_main.jl:652 (total mass).
constexpr int RED_THREADS = 128;

// Per-thread running sum as an unevaluated float pair hi + lo (Knuth's
// two-sum moves every rounding error of hi into lo).  A thread adds a few
// hundred terms, so hi + lo carries the sum to about 2^-44 relative: FP64
// accuracy for the totals without FP64 arithmetic per cell, which this GPU
// runs at a small fraction of its FP32 rate.
struct FAcc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float s = hi + v;
    const float bb = s - hi;
    lo += (hi - (s - bb)) + (v - bb);
    hi = s;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__global__ void __launch_bounds__(RED_THREADS)
k_reduce(const float2* __restrict__ psi_all, const float* __restrict__ phi_all, RedGeom g,
         double* __restrict__ partials) {
  const long long nxy = (long long)g.nx * g.ny;
  const long long n = nxy * g.nz;
  const float2* psi = psi_all + blockIdx.y * n;
  const float* phi = phi_all + blockIdx.y * n;
  FAcc mass, mx, my, mz, wp, kk, q, px, py, pz;
  float best_hi = -1.f, best_lo = 0.f, phimax = 0.f;
  long long best_i = 0;
  double sw = 0.0, swr = 0.0, swr2 = 0.0;  // one z-slice only: FP64 is cheap there
  const float fi2dx = (float)(0.5 / g.dx), fi2dy = (float)(0.5 / g.dy), fi2dz = (float)(0.5 / g.dz);
  const float fx0 = (float)g.x0, fy0 = (float)g.y0, fz0 = (float)g.z0;
  const float fdx = (float)g.dx, fdy = (float)g.dy, fdz = (float)g.dz;
  // rows (y, z) over the blocks, x over the threads: one index division per row
  const long long nrows = (long long)g.ny * g.nz;
  for (long long row = blockIdx.x; row < nrows; row += gridDim.x)
  for (int x = threadIdx.x; x < g.nx; x += blockDim.x) {
    const int z = (int)(row / g.ny);
    const int y = (int)(row - (long long)z * g.ny);
    const long long i = row * g.nx + x;
    const float2 p = psi[i];
    // rho = p.x^2 + p.y^2 exactly as (rs, rt): two-product of each square, two-sum of the pair
    const float a = p.x * p.x, b = p.y * p.y;
    const float ea = fmaf(p.x, p.x, -a), eb = fmaf(p.y, p.y, -b);
    const float rs = a + b;
    const float bb = rs - a;
    const float rt = ((a - (rs - bb)) + (b - bb)) + (ea + eb);
    mass.add(rs);
    mass.lo += rt;
    mx.add(rs * fmaf(fdx, (float)x, fx0));
    my.add(rs * fmaf(fdy, (float)y, fy0));
    mz.add(rs * fmaf(fdz, (float)z, fz0));
    if (rs > best_hi || (rs == best_hi && rt > best_lo)) {
      best_hi = rs;
      best_lo = rt;
      best_i = i;
    }
    const float ph = phi[i];
    phimax = fmaxf(phimax, fabsf(ph));
    if (z == g.zmid) {
      const double rho = (double)rs + (double)rt;
      const double fx = g.x0 + g.dx * x, fy = g.y0 + g.dy * y, fz = g.z0 + g.dz * z;
      const double r2 = fx * fx + fy * fy + fz * fz;
      sw += rho;
      swr += rho * sqrt(r2);
      swr2 += rho * r2;
    }
    if (x > 0 && x < g.nx - 1 && y > 0 && y < g.ny - 1 && z > 0 && z < g.nz - 1) {
      // per-cell terms in FP32 (the reference forms them from its FP32 psi too)
      wp.add(rs * ph);
      const float2 xp = psi[i + 1], xm = psi[i - 1];
      const float2 yp = psi[i + g.nx], ym = psi[i - g.nx];
      const float2 zp = psi[i + nxy], zm = psi[i - nxy];
      // rho v = Im(conj(psi) grad psi)
      const float gxr = (xp.x - xm.x) * fi2dx, gxi = (xp.y - xm.y) * fi2dx;
      const float gyr = (yp.x - ym.x) * fi2dy, gyi = (yp.y - ym.y) * fi2dy;
      const float gzr = (zp.x - zm.x) * fi2dz, gzi = (zp.y - zm.y) * fi2dz;
      const float jx = fmaf(p.x, gxi, -p.y * gxr);
      const float jy = fmaf(p.x, gyi, -p.y * gyr);
      const float jz = fmaf(p.x, gzi, -p.y * gzr);
      px.add(jx);
      py.add(jy);
      pz.add(jz);
      if (rs > 0.f) kk.add(fmaf(jx, jx, fmaf(jy, jy, jz * jz)) / rs);
      auto mag = [](float2 v) { return sqrtf(fmaf(v.x, v.x, v.y * v.y)); };
      const float ax = (mag(xp) - mag(xm)) * fi2dx;
      const float ay = (mag(yp) - mag(ym)) * fi2dy;
      const float az = (mag(zp) - mag(zm)) * fi2dz;
      q.add(fmaf(ax, ax, fmaf(ay, ay, az * az)));
    }
  }
  double acc[RED_FIELDS];
  acc[RED_MASS] = mass.value();
  acc[RED_MAX] = best_hi < 0.f ? -1.0 : (double)best_hi + (double)best_lo;
  acc[RED_ARG] = (double)best_i;
  acc[RED_MX] = mx.value();
  acc[RED_MY] = my.value();
  acc[RED_MZ] = mz.value();
  acc[RED_W] = wp.value();
  acc[RED_K] = kk.value();
  acc[RED_Q] = q.value();
  acc[RED_PX] = px.value();
  acc[RED_PY] = py.value();
  acc[RED_PZ] = pz.value();
  acc[RED_PHIMAX] = (double)phimax;
  acc[RED_SW] = sw;
  acc[RED_SWR] = swr;
  acc[RED_SWR2] = swr2;
  // block reduction (warp shuffles, then one warp over the warp results)
  __shared__ double sh[RED_THREADS / 32][RED_FIELDS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int q = 0; q < RED_FIELDS; ++q) {
      const double o = __shfl_down_sync(0xffffffffu, acc[q], off);
      if (q == RED_PHIMAX) acc[q] = fmax(acc[q], o);
      if (red_is_max(q)) continue;
      acc[q] += o;
    }
    const double om = __shfl_down_sync(0xffffffffu, acc[RED_MAX], off);
    const double oa = __shfl_down_sync(0xffffffffu, acc[RED_ARG], off);
    if (om > acc[RED_MAX] || (om == acc[RED_MAX] && oa < acc[RED_ARG])) {
      acc[RED_MAX] = om;
      acc[RED_ARG] = oa;
    }
  }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < RED_FIELDS; ++q) sh[w][q] = acc[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[RED_FIELDS];
#pragma unroll
    for (int q = 0; q < RED_FIELDS; ++q) r[q] = sh[0][q];
    for (int k = 1; k < RED_THREADS / 32; ++k) {
      for (int q = 0; q < RED_FIELDS; ++q)
        if (!red_is_max(q)) r[q] += sh[k][q];
      r[RED_PHIMAX] = fmax(r[RED_PHIMAX], sh[k][RED_PHIMAX]);
      if (sh[k][RED_MAX] > r[RED_MAX] || (sh[k][RED_MAX] == r[RED_MAX] && sh[k][RED_ARG] < r[RED_ARG])) {
        r[RED_MAX] = sh[k][RED_MAX];
        r[RED_ARG] = sh[k][RED_ARG];
      }
    }
    double* o = partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * RED_FIELDS;
    for (int q = 0; q < RED_FIELDS; ++q) o[q] = r[q];
  }
}

cudaError_t launch_reduce(const float2* psi, const float* phi, const RedGeom& g, double* partials, int nblocks,
                          int batch, cudaStream_t st) {
  k_reduce<<<dim3(nblocks, batch), RED_THREADS, 0, st>>>(psi, phi, g, partials);
  return cudaGetLastError();
}

// Weights of the distances from the density maximum (the weighted quantiles of
// src/simulation_main.jl:641-650), keyed by the squared distance in cells.  A
// thread takes one offset (a, b, c) >= 0 and sums the up to eight cells at
// (cx +- a, cy +- b, cz +- c) inside the grid, which share the key
// a^2 + b^2 + c^2, so a centred halo needs one atomic add per eight cells.
__global__ void k_radii_hist(const float2* __restrict__ psi, int nx, int ny, int nz, int cx, int cy, int cz, int da,
                             int db, int dc, double* __restrict__ wsum) {
  const int nbc = db * dc;
  for (int bc = blockIdx.x; bc < nbc; bc += gridDim.x)
  for (int a = threadIdx.x; a < da; a += blockDim.x) {
    const int c = bc / db;
    const int b = bc - c * db;
    double s = 0.0;
    for (int sz = 0; sz < (c ? 2 : 1); ++sz) {
      const int zz = sz ? cz - c : cz + c;
      if (zz < 0 || zz >= nz) continue;
      for (int sy = 0; sy < (b ? 2 : 1); ++sy) {
        const int yy = sy ? cy - b : cy + b;
        if (yy < 0 || yy >= ny) continue;
        const long long row = ((long long)zz * ny + yy) * nx;
        for (int sx = 0; sx < (a ? 2 : 1); ++sx) {
          const int xx = sx ? cx - a : cx + a;
          if (xx < 0 || xx >= nx) continue;
          const float2 p = psi[row + xx];
          s += (double)p.x * p.x + (double)p.y * p.y;
        }
      }
    }
    if (s > 0.0) atomicAdd(&wsum[(long long)a * a + (long long)b * b + (long long)c * c], s);
  }
}

cudaError_t launch_radii_hist(const float2* psi, int nx, int ny, int nz, int cx, int cy, int cz, double* wsum,
                              cudaStream_t st) {
  const int da = (cx > nx - 1 - cx ? cx : nx - 1 - cx) + 1;
  const int db = (cy > ny - 1 - cy ? cy : ny - 1 - cy) + 1;
  const int dc = (cz > nz - 1 - cz ? cz : nz - 1 - cz) + 1;
  const int rows = db * dc;
  k_radii_hist<<<(unsigned)(rows < 152 * 32 ? rows : 152 * 32), 128, 0, st>>>(psi, nx, ny, nz, cx, cy, cz, da, db, dc,
                                                                              wsum);
  return cudaGetLastError();
}

// Smallest nonzero weight (bits of a positive double) among the cells whose
// key is one of keys.k[0..n): the few groups the quantiles fall in.
__global__ void k_radii_min(const float2* __restrict__ psi, int nx, int ny, int nz, int cx, int cy, int cz,
                            RadiiKeys keys, unsigned long long* __restrict__ wmin) {
  const int nrows = ny * nz;
  for (int row = blockIdx.x; row < nrows; row += gridDim.x)
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    const int z = row / ny;
    const int y = row - z * ny;
    const long long i = (long long)row * nx + x;
    const long long ddx = x - cx, ddy = y - cy, ddz = z - cz;
    const long long key = ddx * ddx + ddy * ddy + ddz * ddz;
    for (int j = 0; j < keys.n; ++j)
      if (key == keys.k[j]) {
        const float2 p = psi[i];
        const double rho = (double)p.x * p.x + (double)p.y * p.y;
        if (rho > 0.0) atomicMin(&wmin[j], (unsigned long long)__double_as_longlong(rho));
      }
  }
}

cudaError_t launch_radii_min(const float2* psi, int nx, int ny, int nz, int cx, int cy, int cz, const RadiiKeys& keys,
                             unsigned long long* wmin, cudaStream_t st) {
  const int rows = ny * nz;
  k_radii_min<<<(unsigned)(rows < 152 * 32 ? rows : 152 * 32), 128, 0, st>>>(psi, nx, ny, nz, cx, cy, cz, keys, wmin);
  return cudaGetLastError();
}

__device__ __forceinline__ long long cic_cell(int ix, int iy, int iz, int nx, int ny, int nz) {
  ix = ix >= nx ? ix - nx : ix;
  iy = iy >= ny ? iy - ny : iy;
  iz = iz >= nz ? iz - nz : iz;
  return ((long long)iz * ny + iy) * nx + ix;
}

// rows (ny * nz flags, may be null): set to 1 for every x row a particle touches
__global__ void k_cic_deposit(float* __restrict__ rho, const CicParticle* __restrict__ p, long long n, int nx, int ny,
                              int nz, int* __restrict__ rows) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const CicParticle a = p[q];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int ox = c & 1, oy = (c >> 1) & 1, oz = c >> 2;
    const float w = (ox ? a.f[0] : 1.f - a.f[0]) * (oy ? a.f[1] : 1.f - a.f[1]) * (oz ? a.f[2] : 1.f - a.f[2]);
    const long long cell = cic_cell(a.i[0] + ox, a.i[1] + oy, a.i[2] + oz, nx, ny, nz);
    atomicAdd(rho + cell, a.m * w);
    if (rows && c % 2 == 0) rows[cell / nx] = 1;
  }
}

__global__ void k_cic_interp(const float* __restrict__ f, const CicParticle* __restrict__ p, long long n, int nx,
                             int ny, int nz, double* __restrict__ out) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const CicParticle a = p[q];
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int ox = c & 1, oy = (c >> 1) & 1, oz = c >> 2;
    const double w = (double)(ox ? a.f[0] : 1.f - a.f[0]) * (oy ? a.f[1] : 1.f - a.f[1]) * (oz ? a.f[2] : 1.f - a.f[2]);
    s += w * f[cic_cell(a.i[0] + ox, a.i[1] + oy, a.i[2] + oz, nx, ny, nz)];
  }
  out[q] = s;
}

cudaError_t launch_cic_deposit(float* rho, const CicParticle* p, long long n, int nx, int ny, int nz, int* rows,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_cic_deposit<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rho, p, n, nx, ny, nz, rows);
  return cudaGetLastError();
}

cudaError_t launch_cic_interp(const float* field, const CicParticle* p, long long n, int nx, int ny, int nz,
                              double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_cic_interp<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(field, p, n, nx, ny, nz, out);
  return cudaGetLastError();
}

}  // namespace wdm

namespace wdm {

// Mean of |psi|^2 (complex input) or of a float field, per batch item, as a
// float shift: FP64 block partial sums, FP64 atomics into sums[b] (zeroed by
// the launcher), then shift[b] = sums[b] / n + add.
template <bool COMPLEX>
__global__ void k_block_sum(const void* __restrict__ data, long long n, double* __restrict__ sums) {
  // per-thread FP32 partial sums (the shift only needs to be near the mean:
  // any value is exact), FP64 from the warp reduction on
  float accf = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if constexpr (COMPLEX) {
      const float2 v = static_cast<const float2*>(data)[blockIdx.y * n + i];
      accf = fmaf(v.x, v.x, fmaf(v.y, v.y, accf));
    } else {
      accf += static_cast<const float*>(data)[blockIdx.y * n + i];
    }
  }
  double acc = accf;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    atomicAdd(sums + blockIdx.y, s);
  }
}

__global__ void k_finalize_shift(const double* __restrict__ sums, float* __restrict__ shift, int batch, double inv_n,
                                 double add) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) shift[b] = (float)(sums[b] * inv_n + add);
}

cudaError_t launch_mean_shift(const void* data, bool complex_in, long long n, int batch, double* sums, float* shift,
                              double add, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sums, 0, sizeof(double) * batch, st);
  if (e != cudaSuccess) return e;
  long long blocks = (n + 255) / 256;
  if (blocks > 304) blocks = 304;
  if (complex_in) k_block_sum<true><<<dim3((unsigned)blocks, batch), 256, 0, st>>>(data, n, sums);
  else k_block_sum<false><<<dim3((unsigned)blocks, batch), 256, 0, st>>>(data, n, sums);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_finalize_shift<<<(batch + 127) / 128, 128, 0, st>>>(sums, shift, batch, 1.0 / (double)n, add);
  return cudaGetLastError();
}

}  // namespace wdm
