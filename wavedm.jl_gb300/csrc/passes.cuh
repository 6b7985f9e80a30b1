// Pass kernels of the split-step KDK step.
//
// Storage (x fastest, the C-order view of Julia's psi[x, y, z]):
//   psi  complex64 [nz][ny][nx]        the wavefunction; every pass runs in place
//   H    complex64 [nz][ny][nxh]       nxh = nx/2 + 1: the density / potential
//                                      half spectrum along x (Hermitian in kx)
// One KDK step is eight launches, each one read + one write of its array:
//   P1 k_x_kick_fwd   H -> Phi rows (C2R), psi <- exp(-i dt Phi) psi, x-FFT fwd
//   P2 k_lfft<fwd>    psi, y axis
//   P3 k_lfft_mid     psi, z axis: fwd, exp(-i k^2 dt/2)/(nx ny nz), inverse
//   P4 k_lfft<inv>    psi, y axis
//   P5 k_x_inv_rho    psi x-FFT inverse (+ absorbing mask), rho = |psi|^2 (+ rho_b),
//                     rho rows R2C -> H
//   P6 k_lfft<fwd>    H, y axis
//   P7 k_lfft_mid     H, z axis: fwd, -c/(k^2 nx ny nz), inverse
//   P8 k_lfft<inv>    H, y axis
#pragma once
#include "fft_engine.cuh"

namespace wdm {

constexpr int LINES = 16;        // lines per CTA
constexpr int LPITCH = LINES + 1; // shared-memory pitch (in float2) between points

template <int N>
__host__ __device__ constexpr int threads_for() { return Plan<N>::T * LINES; }

template <int N>
__host__ __device__ constexpr int min_blocks() { return threads_for<N>() >= 512 ? 1 : 512 / threads_for<N>(); }

template <int N>
__host__ __device__ constexpr size_t smem_bytes() { return sizeof(float2) * (size_t)(N + N * LPITCH); }

struct LineGeom {
  int nlines;         // lines per batch item
  int nxa;            // lines that are contiguous along x
  long long outer;    // element stride between successive groups of nxa lines
  long long pstride;  // element stride between points of one line
  long long bstride;  // element stride between batch items
};

struct RowGeom {
  int nrows;          // rows per batch item (ny * nz)
  int ny;             // rows per z plane
  long long pitch;    // element stride between rows
  long long bstride;  // element stride between batch items
};

__device__ __forceinline__ long long line_base(const LineGeom& g, int line) {
  return (long long)(line / g.nxa) * g.outer + (line % g.nxa);
}

// ----------------------------------------------------------------------------
// k-space operators applied between the forward and inverse transforms of a
// fused pass.  `line` indexes (mx + nxa * my), `pos` is mz, `b` the batch item.
// ----------------------------------------------------------------------------
struct DriftOp {
  // precise form: separable phase tables exp(-i k_a^2 dt/2) built in FP64; the
  // z table also carries 1/(nx ny nz).
  const float2* cx;
  const float2* cy;
  const float2* cz;
  // plain form: k_a^2 tables and the FP32 phase k^2 dt/2
  const float* kx2;
  const float* ky2;
  const float* kz2;
  float half_dt;
  float scale;
  int nxa;
  int precise;
  long long tab_bstride;  // per-batch-item stride of the phase tables (0 = shared)
  __device__ __forceinline__ float2 operator()(float2 v, int line, int pos, int b) const {
    const int mx = line % nxa, my = line / nxa;
    if (precise) {
      const long long o = b * tab_bstride;
      float2 f = cmul(cmul(cx[o + mx], cy[o + my]), cz[o + pos]);
      return cmul(v, f);
    }
    const float th = (kx2[mx] + ky2[my] + kz2[pos]) * half_dt;
    float s, c;
    sincosf(th, &s, &c);
    return cmul(v, make_float2(c * scale, -s * scale));
  }
};

struct PoissonOp {
  const float* kx2;
  const float* ky2;
  const float* kz2;
  float coef;  // -c / (nx ny nz)
  int nxa;
  __device__ __forceinline__ float2 operator()(float2 v, int line, int pos, int) const {
    const int mx = line % nxa, my = line / nxa;
    const float k2 = kx2[mx] + ky2[my] + kz2[pos];
    const float f = (k2 > 0.f) ? coef / k2 : 0.f;
    return make_float2(v.x * f, v.y * f);
  }
};

// ----------------------------------------------------------------------------
// strided-line passes (y or z axis)
// ----------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void lines_load(float2* v, const float2* base, long long ps, bool ok, int t) {
  using P = Plan<N>;
  constexpr int T = P::T, R1 = RadInfo<typename P::Fwd>::first;
#pragma unroll
  for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
    for (int k = 0; k < R1; ++k)
      v[i * R1 + k] = ok ? base[(long long)slot_pos<N, T, R1>(t, i, k) * ps] : make_float2(0.f, 0.f);
}

template <int N, int R>
__device__ __forceinline__ void lines_store(const float2* v, float2* base, long long ps, bool ok, int t) {
  constexpr int T = Plan<N>::T;
  if (!ok) return;
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) base[(long long)slot_pos<N, T, R>(t, i, k) * ps] = v[i * R + k];
}

template <int N, bool INV>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_lfft(float2* __restrict__ data, LineGeom g, const float2* __restrict__ twg) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int line = blockIdx.x * LINES + l;
  const bool ok = line < g.nlines;
  float2* base = data + blockIdx.y * g.bstride + (ok ? line_base(g, line) : 0);
  float2 v[N / T];
  lines_load<N>(v, base, g.pstride, ok, t);
  __syncthreads();
  run_stages<N, T, LPITCH, INV>(Rad{}, v, s, tw, t, l);
  lines_store<N, RadInfo<Rad>::last>(v, base, g.pstride, ok, t);
}

template <int N, class Op>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_lfft_mid(float2* __restrict__ data, LineGeom g, const float2* __restrict__ twg, Op op) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  using Rev = typename Reverse<Rad>::type;
  constexpr int RS = RadInfo<Rad>::last;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int line = blockIdx.x * LINES + l;
  const bool ok = line < g.nlines;
  float2* base = data + blockIdx.y * g.bstride + (ok ? line_base(g, line) : 0);
  float2 v[N / T];
  lines_load<N>(v, base, g.pstride, ok, t);
  __syncthreads();
  run_stages<N, T, LPITCH, false>(Rad{}, v, s, tw, t, l);
  const int lc = ok ? line : 0;
#pragma unroll
  for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
    for (int k = 0; k < RS; ++k)
      v[i * RS + k] = op(v[i * RS + k], lc, slot_pos<N, T, RS>(t, i, k), blockIdx.y);
  run_stages<N, T, LPITCH, true>(Rev{}, v, s, tw, t, l);
  lines_store<N, RadInfo<Rev>::last>(v, base, g.pstride, ok, t);
}

// ----------------------------------------------------------------------------
// x-axis (contiguous rows) passes: coalesced row tiles staged through s
// ----------------------------------------------------------------------------
// s[x * LPITCH + rl] <- f(row, x, data[row * pitch + x]) for the CTA's rows.
template <int N, class F>
__device__ __forceinline__ void tile_load(float2* s, const float2* __restrict__ g, int r0, int nrows,
                                          long long pitch, F f) {
  constexpr int NT = threads_for<N>();
  constexpr int TOT = LINES * N;
#pragma unroll 4
  for (int e = threadIdx.x; e < TOT; e += NT) {
    const int rl = e / N, x = e - rl * N;
    const int r = r0 + rl;
    float2 val = make_float2(0.f, 0.f);
    if (r < nrows) val = f(r, x, g[(long long)r * pitch + x]);
    s[x * LPITCH + rl] = val;
  }
}

template <int N, class F>
__device__ __forceinline__ void tile_store(const float2* s, float2* __restrict__ g, int r0, int nrows,
                                           long long pitch, F f) {
  constexpr int NT = threads_for<N>();
  constexpr int TOT = LINES * N;
#pragma unroll 4
  for (int e = threadIdx.x; e < TOT; e += NT) {
    const int rl = e / N, x = e - rl * N;
    const int r = r0 + rl;
    if (r < nrows) g[(long long)r * pitch + x] = f(r, x, s[x * LPITCH + rl]);
  }
}

// write register slots positioned for radix R into s
template <int N, int R>
__device__ __forceinline__ void regs_to_smem(float2* s, const float2* v, int t, int l) {
  constexpr int T = Plan<N>::T;
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) s[slot_pos<N, T, R>(t, i, k) * LPITCH + l] = v[i * R + k];
}

template <int N, int R>
__device__ __forceinline__ void smem_to_regs(const float2* s, float2* v, int t, int l) {
  constexpr int T = Plan<N>::T;
#pragma unroll
  for (int i = 0; i < N / (R * T); ++i)
#pragma unroll
    for (int k = 0; k < R; ++k) v[i * R + k] = s[slot_pos<N, T, R>(t, i, k) * LPITCH + l];
}

struct Ident {
  __device__ __forceinline__ float2 operator()(int, int, float2 v) const { return v; }
};
struct Scale {
  float s;
  __device__ __forceinline__ float2 operator()(int, int, float2 v) const { return make_float2(v.x * s, v.y * s); }
};

template <int N, bool INV>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_xfft(float2* __restrict__ data, RowGeom rg, const float2* __restrict__ twg, float scale) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int r0 = blockIdx.x * LINES;
  float2* d = data + blockIdx.y * rg.bstride;
  tile_load<N>(s, d, r0, rg.nrows, rg.pitch, Ident{});
  __syncthreads();
  float2 v[N / T];
  smem_to_regs<N, RadInfo<Rad>::first>(s, v, t, l);
  run_stages<N, T, LPITCH, INV>(Rad{}, v, s, tw, t, l);
  __syncthreads();
  regs_to_smem<N, RadInfo<Rad>::last>(s, v, t, l);
  __syncthreads();
  tile_store<N>(s, d, r0, rg.nrows, rg.pitch, Scale{scale});
}

// ----------------------------------------------------------------------------
// real rows <-> half spectra.  Rows (2m, 2m+1) of a CTA tile are packed as the
// complex line z_m = a + i b; its DFT Z gives A[k] = (Z[k] + conj Z[N-k])/2 and
// B[k] = (Z[k] - conj Z[N-k])/(2i) for k = 0..N/2 (forward), and the inverse
// packs Z[k] = A[k] + i B[k] with A[N-k] = conj A[k] (inverse).
// ----------------------------------------------------------------------------
// Hermitian split of the packed spectra in s (lines m < LINES/2) into H rows.
template <int N>
__device__ __forceinline__ void store_half_rows(const float2* s, float2* __restrict__ H, int r0, int nrows,
                                                long long hpitch) {
  constexpr int NT = threads_for<N>();
  constexpr int NH = N / 2 + 1;
  constexpr int TOT = LINES * NH;
  for (int e = threadIdx.x; e < TOT; e += NT) {
    const int rl = e / NH, k = e - rl * NH;
    const int r = r0 + rl;
    if (r >= nrows) continue;
    const int m = rl >> 1;
    const float2 zk = s[k * LPITCH + m];
    const float2 zn = s[((N - k) % N) * LPITCH + m];
    float2 out;
    if ((rl & 1) == 0) {
      out = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
    } else {
      // (Z[k] - conj Z[N-k]) / (2i)
      const float dx = zk.x - zn.x, dy = zk.y + zn.y;
      out = make_float2(0.5f * dy, -0.5f * dx);
    }
    H[(long long)r * hpitch + k] = out;
  }
}

// Pack H rows (pairs) into full-length complex lines m < LINES/2 of s.
template <int N>
__device__ __forceinline__ void load_half_rows(float2* s, const float2* __restrict__ H, int r0, int nrows,
                                               long long hpitch) {
  constexpr int NT = threads_for<N>();
  constexpr int NH = N / 2 + 1;
  constexpr int TOT = (LINES / 2) * NH;
  for (int e = threadIdx.x; e < TOT; e += NT) {
    const int m = e / NH, k = e - m * NH;
    const int ra = r0 + 2 * m;
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (ra < nrows) a = H[(long long)ra * hpitch + k];
    if (ra + 1 < nrows) b = H[(long long)(ra + 1) * hpitch + k];
    // Z[k] = A[k] + i B[k]
    s[k * LPITCH + m] = make_float2(a.x - b.y, a.y + b.x);
    if (k > 0 && k < N / 2) {
      // Z[N-k] = conj(A[k]) + i conj(B[k])
      s[(N - k) * LPITCH + m] = make_float2(a.x + b.y, b.x - a.y);
    }
  }
}

// ----------------------------------------------------------------------------
// P5: psi x-inverse (+mask), rho = |psi|^2 (+rho_b), rho R2C rows -> H
// ----------------------------------------------------------------------------
struct RhoArgs {
  const float* mx;   // separable absorbing-mask tables (null: no mask)
  const float* my;
  const float* mz;
  const float* rho_b;  // baryon density [nz][ny][nx] (null: none)
  long long rb_bstride;
  int write_psi;     // 0: density only (psi is already in real space, left untouched)
  int* nonfinite;    // set to 1 when any density value is NaN/Inf (null: unchecked)
};

template <int N>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_x_inv_rho(float2* __restrict__ psi, float2* __restrict__ H, RowGeom rg, long long hpitch, long long hbstride,
            const float2* __restrict__ twg, RhoArgs a) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  constexpr int RS = RadInfo<Rad>::last, R1 = RadInfo<Rad>::first;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int r0 = blockIdx.x * LINES;
  float2* d = psi + blockIdx.y * rg.bstride;
  float2* h = H + blockIdx.y * hbstride;
  tile_load<N>(s, d, r0, rg.nrows, rg.pitch, Ident{});
  __syncthreads();
  float2 v[N / T];
  int pR;  // radix of the register positions held in v
  if (a.write_psi) {
    smem_to_regs<N, R1>(s, v, t, l);
    run_stages<N, T, LPITCH, true>(Rad{}, v, s, tw, t, l);
    pR = RS;
    if (a.mx) {
      const int r = r0 + l;
      const int y = r % rg.ny, z = r / rg.ny;
      const float myz = (r < rg.nrows) ? a.my[y] * a.mz[z] : 0.f;
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k) v[i * RS + k] = cscale(v[i * RS + k], myz * a.mx[slot_pos<N, T, RS>(t, i, k)]);
    }
    __syncthreads();
    regs_to_smem<N, RS>(s, v, t, l);
    __syncthreads();
    tile_store<N>(s, d, r0, rg.nrows, rg.pitch, Ident{});
  } else {
    smem_to_regs<N, RS>(s, v, t, l);
    pR = RS;
  }
  (void)pR;
  // rho of the rows into packed lines: s float view, complex slot m = l/2, part l&1
  __syncthreads();
  float* sf = reinterpret_cast<float*>(s);
#pragma unroll
  for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
    for (int k = 0; k < RS; ++k) {
      const float2 q = v[i * RS + k];
      const float rho = q.x * q.x + q.y * q.y;
      if (a.nonfinite && !isfinite(rho)) *a.nonfinite = 1;
      sf[(slot_pos<N, T, RS>(t, i, k) * LPITCH + (l >> 1)) * 2 + (l & 1)] = rho;
    }
  if (a.rho_b) {
    __syncthreads();
    const float* rb = a.rho_b + blockIdx.y * a.rb_bstride;
    constexpr int NT = threads_for<N>();
    for (int e = threadIdx.x; e < LINES * N; e += NT) {
      const int rl = e / N, x = e - rl * N;
      const int r = r0 + rl;
      if (r < rg.nrows) sf[(x * LPITCH + (rl >> 1)) * 2 + (rl & 1)] += rb[(long long)r * rg.pitch + x];
    }
  }
  __syncthreads();
  smem_to_regs<N, R1>(s, v, t, l);
  run_stages<N, T, LPITCH, false>(Rad{}, v, s, tw, t, l);
  __syncthreads();
  regs_to_smem<N, RS>(s, v, t, l);
  __syncthreads();
  store_half_rows<N>(s, h, r0, rg.nrows, hpitch);
}

// ----------------------------------------------------------------------------
// P1: Phi rows from H (C2R), kick, then (optionally) the forward x-FFT
// ----------------------------------------------------------------------------
struct KickArgs {
  float dt_hi, dt_lo;    // kick time step as a float pair (dt = hi + lo)
  float T6[6];           // tidal tensor (xx, yy, zz, xy, xz, yz); used if tidal != 0
  const float* T6b;      // per-batch-item tidal tensors [b][6] (overrides T6 when non-null)
  int tidal;
  float x0, y0, z0;      // coordinate of cell 0 along each axis
  float dx, dy, dz;
  float kerr;            // kappa |psi|^2 local potential
  const float* V;        // static potential [nz][ny][nx] or null
  long long v_bstride;
  int precise;           // reduce the phase modulo 2 pi in float-float before sincos
};

__device__ __forceinline__ float2 phase_factor(float pot, const KickArgs& a) {
  float s, c;
  if (a.precise) {
    // theta = pot * dt as an unevaluated float pair, reduced by 2 pi (Cody-Waite
    // with a two-term 2 pi), then one float sincos on |r| <= pi.
    const float th = pot * a.dt_hi;
    const float te = fmaf(pot, a.dt_hi, -th) + pot * a.dt_lo;
    const float n = rintf(th * 0.15915494309189535f);
    const float r = fmaf(-n, 6.28318548202514648f, th) + fmaf(-n, -1.7484555e-07f, te);
    sincosf(r, &s, &c);
  } else {
    sincosf(pot * a.dt_hi, &s, &c);
  }
  return make_float2(c, -s);
}

template <int N, bool FWD>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_x_kick(float2* __restrict__ psi, const float2* __restrict__ H, RowGeom rg, long long hpitch, long long hbstride,
         const float2* __restrict__ twg, KickArgs a) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  using Rev = typename Reverse<Rad>::type;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int r0 = blockIdx.x * LINES;
  float2* d = psi + blockIdx.y * rg.bstride;
  const float2* h = H + blockIdx.y * hbstride;
  // Phi rows: packed inverse transform; the reversed plan ends with radix R1,
  // so the values land at the register slots the psi tile is read from.
  load_half_rows<N>(s, h, r0, rg.nrows, hpitch);
  __syncthreads();
  float2 v[N / T];
  smem_to_regs<N, RS>(s, v, t, l);
  run_stages<N, T, LPITCH, true>(Rev{}, v, s, tw, t, l);
  float phi[N / T];
  {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned src = (lane & ~15u) | ((unsigned)l >> 1);
#pragma unroll
    for (int q = 0; q < N / T; ++q) {
      const float px = __shfl_sync(0xffffffffu, v[q].x, src);
      const float py = __shfl_sync(0xffffffffu, v[q].y, src);
      phi[q] = (l & 1) ? py : px;
    }
  }
  __syncthreads();
  // psi tile; the static potential (if any) is applied here with coalesced reads
  if (a.V) {
    const float* V = a.V + blockIdx.y * a.v_bstride;
    const KickArgs& aa = a;
    tile_load<N>(s, d, r0, rg.nrows, rg.pitch, [&](int r, int x, float2 val) {
      return cmul(val, phase_factor(V[(long long)r * rg.pitch + x], aa));
    });
  } else {
    tile_load<N>(s, d, r0, rg.nrows, rg.pitch, Ident{});
  }
  __syncthreads();
  smem_to_regs<N, R1>(s, v, t, l);
  {
    const int r = min(r0 + l, rg.nrows - 1);
    const int y = r % rg.ny, z = r / rg.ny;
    const float fy = a.y0 + a.dy * y, fz = a.z0 + a.dz * z;
    float T6[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) T6[q] = a.T6b ? a.T6b[blockIdx.y * 6 + q] : a.T6[q];
    // 1/2 x^T T x = 1/2 Txx x^2 + Txy x y + Txz x z + (1/2 Tyy y^2 + Tyz y z + 1/2 Tzz z^2)
    const float cyz = 0.5f * T6[1] * fy * fy + T6[5] * fy * fz + 0.5f * T6[2] * fz * fz;
    const float lin = T6[3] * fy + T6[4] * fz;
#pragma unroll
    for (int i = 0; i < N / (R1 * T); ++i)
#pragma unroll
      for (int k = 0; k < R1; ++k) {
        const int q = i * R1 + k;
        float pot = phi[q];
        if (a.tidal) {
          const float fx = a.x0 + a.dx * slot_pos<N, T, R1>(t, i, k);
          pot += fmaf(fx, fmaf(0.5f * T6[0], fx, lin), cyz);
        }
        if (a.kerr != 0.f) pot += a.kerr * (v[q].x * v[q].x + v[q].y * v[q].y);
        v[q] = cmul(v[q], phase_factor(pot, a));
      }
  }
  if constexpr (FWD) {
    run_stages<N, T, LPITCH, false>(Rad{}, v, s, tw, t, l);
    __syncthreads();
    regs_to_smem<N, RS>(s, v, t, l);
  } else {
    __syncthreads();
    regs_to_smem<N, R1>(s, v, t, l);
  }
  __syncthreads();
  tile_store<N>(s, d, r0, rg.nrows, rg.pitch, Ident{});
}

// Phi rows (real) from H: C2R x pass only (diagnostic output of the potential).
template <int N>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_x_c2r(const float2* __restrict__ H, float* __restrict__ out, RowGeom rg, long long hpitch, long long hbstride,
        const float2* __restrict__ twg) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int r0 = blockIdx.x * LINES;
  load_half_rows<N>(s, H + blockIdx.y * hbstride, r0, rg.nrows, hpitch);
  __syncthreads();
  float2 v[N / T];
  smem_to_regs<N, R1>(s, v, t, l);
  run_stages<N, T, LPITCH, true>(Rad{}, v, s, tw, t, l);
  __syncthreads();
  regs_to_smem<N, RS>(s, v, t, l);
  __syncthreads();
  float* o = out + blockIdx.y * rg.bstride;
  constexpr int NT = threads_for<N>();
  for (int e = threadIdx.x; e < LINES * N; e += NT) {
    const int rl = e / N, x = e - rl * N;
    const int r = r0 + rl;
    if (r >= rg.nrows) continue;
    const float2 z = s[x * LPITCH + (rl >> 1)];
    o[(long long)r * rg.pitch + x] = (rl & 1) ? z.y : z.x;
  }
}

// Real rows -> H (R2C x pass) from a float field (standalone Poisson input).
template <int N>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_x_r2c(const float* __restrict__ in, float2* __restrict__ H, RowGeom rg, long long hpitch, long long hbstride,
        const float2* __restrict__ twg) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + N;
  load_twiddles<N>(tw, twg);
  const int l = threadIdx.x % LINES, t = threadIdx.x / LINES;
  const int r0 = blockIdx.x * LINES;
  const float* src = in + blockIdx.y * rg.bstride;
  float* sf = reinterpret_cast<float*>(s);
  constexpr int NT = threads_for<N>();
  for (int e = threadIdx.x; e < LINES * N; e += NT) {
    const int rl = e / N, x = e - rl * N;
    const int r = r0 + rl;
    sf[(x * LPITCH + (rl >> 1)) * 2 + (rl & 1)] = (r < rg.nrows) ? src[(long long)r * rg.pitch + x] : 0.f;
  }
  __syncthreads();
  float2 v[N / T];
  smem_to_regs<N, R1>(s, v, t, l);
  run_stages<N, T, LPITCH, false>(Rad{}, v, s, tw, t, l);
  __syncthreads();
  regs_to_smem<N, RS>(s, v, t, l);
  __syncthreads();
  store_half_rows<N>(s, H + blockIdx.y * hbstride, r0, rg.nrows, hpitch);
}

}  // namespace wdm
