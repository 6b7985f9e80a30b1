// Pass kernels of the split-step KDK step.
//
// Storage (x fastest, the C-order view of Julia's psi[x, y, z]):
//   psi  complex64 [nz][ny][nx]        the wavefunction; every pass runs in place
//   H    complex64 [nz][ny][hpitch]    the density / potential half spectrum
//                                      along x (nx/2 + 1 columns, Hermitian in
//                                      kx; hpitch: that rounded up to even)
// One KDK step is eight launches, each one read + one write of its array (the
// line passes are k_lfft_tma, or k_lfft_tile; the x passes the staged k_xs_*
// kernels of xpass_staged.cuh, or the direct k_xw_* kernels of xpass_warp.cuh):
//   P1 kick       H -> Phi rows (C2R), psi <- exp(-i dt Phi) psi, x-FFT fwd
//   P2 line <0>   psi, y axis
//   P3 line <2>   psi, z axis: fwd, exp(-i k^2 dt/2)/(nx ny nz) (DriftOp), inverse
//   P4 line <1>   psi, y axis
//   P5 inv_rho    psi x-FFT inverse (+ absorbing mask), rho = |psi|^2 (+ rho_b),
//                 rho rows R2C -> H
//   P6 line <0>   H, y axis
//   P7 line <2>   H, z axis: fwd, -c/(k^2 nx ny nz) (PoissonOp), inverse
//   P8 line <1>   H, y axis
#pragma once
#include "fft_engine.cuh"
#include "tma.cuh"
#include "wdm_math.cuh"

namespace wdm {

constexpr int LINES = 16;        // lines per CTA
constexpr int LPITCH = LINES + 1; // shared-memory pitch (in float2) between points

template <int N>
__host__ __device__ constexpr int threads_for() { return Plan<N>::T * LINES; }

template <int N>
__host__ __device__ constexpr int min_blocks() {
#ifdef WDM_LINE_THREADS_PER_SM
  return threads_for<N>() >= WDM_LINE_THREADS_PER_SM ? 1 : WDM_LINE_THREADS_PER_SM / threads_for<N>();
#else
  return threads_for<N>() >= 512 ? 1 : 512 / threads_for<N>();
#endif
}

template <int N>
__host__ __device__ constexpr size_t smem_bytes() { return sizeof(float2) * (size_t)(2 * N + N * LPITCH); }

// fused forward/op/inverse line pass: both twiddle tables
template <int N>
__host__ __device__ constexpr size_t smem_bytes_mid() { return sizeof(float2) * (size_t)(4 * N + N * LPITCH); }

struct LineGeom {
  int nlines;         // lines per batch item
  int nxa;            // lines that are contiguous along x
  long long outer;    // element stride between successive groups of nxa lines
  long long pstride;  // element stride between points of one line
  long long bstride;  // element stride between batch items
  // tensor-map view for the TMA-fed pass: the array is [batch][d2][d1][pitch]
  // with the lines along d1 (axis 1) or d2 (axis 2); `rows` counts the other
  // of d1/d2, so a batch item holds rows * ceil(nxa / LINES) tiles
  int axis = 0;          // 1: lines along y, 2: lines along z, 0: no tensor-map view
  int rows = 0;          // groups of nxa lines per batch item
  long long pitch = 0;   // element stride along y (row pitch)
  int* err = nullptr;    // device-visible error word (bounded waits), may be null
  int x0 = 0;            // x column of the first line (k-space operators see mx = x0 + column)
  int impl = 0;          // LINE_IMPL_TMA or LINE_IMPL_TILE (chosen per pass by the autotuner)
  // TMA pass only: edge tiles per batch item for the last column when
  // nxa = 16 m + 1 (the kx = N/2 column of a half spectrum), 0: none.  The
  // rows' full tiles then cover columns 0 .. 16 m - 1, and each edge tile
  // holds the last column of 8 rows (filled in by the launcher).
  int edge = 0;
};

// Implementations of a line pass: the TMA-fed persistent pass (used where the
// array has a tensor-map view) and the one-register-tile-per-CTA pass.
enum { LINE_IMPL_TMA = 0, LINE_IMPL_TILE = 1 };

struct RowGeom {
  int nrows;          // rows per batch item (ny * nz)
  int ny;             // rows per z plane
  long long pitch;    // element stride between rows
  long long bstride;  // element stride between batch items
  int impl = 0;       // X_IMPL_STAGED or X_IMPL_DIRECT for the kick and density passes
};

// Implementations of the kick and density x passes: rows staged in shared
// memory by bulk copies one unit ahead (where the layout allows), or loaded
// straight into registers.
enum { X_IMPL_STAGED = 0, X_IMPL_DIRECT = 1 };

__device__ __forceinline__ long long line_base(const LineGeom& g, int line) {
  return (long long)(line / g.nxa) * g.outer + (line % g.nxa);
}

// ----------------------------------------------------------------------------
// k-space operators applied between the forward and inverse transforms of a
// fused pass at mode (mx, my, pos = mz) of batch item b.
// ----------------------------------------------------------------------------
// Exact error of the FP32 sum s = a + b (Knuth two-sum).
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
  const float bb = s - a;
  return (a - (s - bb)) + (b - bb);
}

struct DriftOp {
  // precise form: the factor exp(-i (kx^2 + ky^2 + kz^2) dt/2) / (nx ny nz)
  // separates into a factor per z line and one per mode along the line.
  // cxy[my * nxy + mx] = exp(-i (kx^2 + ky^2) dt/2) / (nx ny nz) and
  // cz[mz] = exp(-i kz^2 dt/2) are built in FP64 (phases reduced mod 2 pi in
  // double) and kept as FP32 (hi, lo) pairs in the twiddle layout
  // (pack_twiddle); a point takes two compensated complex products
  // (twiddle_mul), so each factor acts with its FP64 modulus and phase and
  // only the two roundings of the product remain, unbiased from point to
  // point and step to step.  A plain FP32 table would instead repeat one
  // fixed rounding of |factor| over whole planes of modes every step, which
  // shows up as a mass drift.
  const float4* cxy;
  const float4* cz;
  int nxy;                // row length of cxy (nx)
  int rot;                // cz holds entries flagged as rotated (sin = +-1/2)
  // plain form: k_a^2 tables and the FP32 phase k^2 dt/2
  const float* kx2;
  const float* ky2;
  const float* kz2;
  float half_dt;
  float scale;
  float sign;             // +1: exp(-i k^2 dt/2); -1: its conjugate (the drift adjoint)
  int precise;
  static constexpr bool TABLE = false;
  static constexpr bool FORMS = true;  // the precise / plain choice is made once per line (op_points)
  // ROT: cz may hold flagged entries (rot != 0)
  template <bool PRECISE, bool ROT>
  __device__ __forceinline__ float2 at(float2 v, int mx, int my, int pos) const {
    if constexpr (PRECISE) {
      const bool conj = sign < 0.f;
      const float4 wz = cz[pos];
      const float4 wxy = cxy[(long long)my * nxy + mx];
      const float2 u = twiddle_mul<ROT>(v, wz, conj);
      return twiddle_mul<false>(u, wxy, conj);
    }
    const float th = sign * (kx2[mx] + ky2[my] + kz2[pos]) * half_dt;
    const float2 sc = sincos_plain(th);
    return cmul(v, make_float2(sc.y * scale, -sc.x * scale));
  }
  __device__ __forceinline__ float2 operator()(float2 v, int mx, int my, int pos, int) const {
    return precise ? (rot ? at<true, true>(v, mx, my, pos) : at<true, false>(v, mx, my, pos))
                   : at<false, false>(v, mx, my, pos);
  }
};

struct PoissonOp {
  static constexpr bool FORMS = false;
  const float* kx2;
  const float* ky2;
  const float* kz2;
  float coef;  // -c / (nx ny nz)
  __device__ __forceinline__ float2 operator()(float2 v, int mx, int my, int pos, int) const {
    return scaled(v, kx2[mx] + ky2[my] + kz2[pos]);
  }
  // The TMA line pass stages kz2 (the table along its lines) in shared memory
  // once per CTA: read from global memory between the two transforms of every
  // point, with nothing to hide its latency, it was the pass's main stall.
  static constexpr bool TABLE = true;
  __device__ __forceinline__ float table_entry(int pos) const { return kz2[pos]; }
  __device__ __forceinline__ float2 with_table(float2 v, int mx, int my, int pos, const float* tab) const {
    return scaled(v, kx2[mx] + ky2[my] + tab[pos]);
  }
  // -c / k^2 by CUDA's fast division (__fdividef: at most 2 ulp; k^2 lies far
  // inside its range).  The IEEE division's slow-path branch at every point
  // kept the compiler from interleaving the points of a line: the H z pass
  // took 0.164 ms with it and 0.148 ms with __fdividef at 384^3 (coef times
  // __frcp_rn(k^2): 0.166 ms).  The potential's relative rounding of 2.4e-7
  // is of the order of the FP32 transforms' own.
  __device__ __forceinline__ float2 scaled(float2 v, float k2) const {
#if defined(WDM_POISSON_IEEE_DIV)
    const float f = (k2 > 0.f) ? coef / k2 : 0.f;
#else
    const float f = (k2 > 0.f) ? __fdividef(coef, k2) : 0.f;
#endif
    return make_float2(v.x * f, v.y * f);
  }
};

// The k-space operator at every point of one line held at radix-RS slots
// (mode (mx, my, pos) of batch item b): from the table staged in shared memory
// (TAB, for operators that have one), or with a runtime form tested once for
// the line's points.
template <bool A, bool B>
struct BoolPair {
  static constexpr bool first = A, second = B;
};

template <int N, int T, int RS, bool TAB, class Op>
__device__ __forceinline__ void op_points(const Op& op, float2* v, int mx, int my, int t, int b, const float* tab) {
  if constexpr (TAB && Op::TABLE) {
#pragma unroll
    for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
      for (int k = 0; k < RS; ++k) v[i * RS + k] = op.with_table(v[i * RS + k], mx, my, slot_pos<N, T, RS>(t, i, k), tab);
  } else if constexpr (Op::FORMS) {
    auto line = [&](auto form) {
      constexpr bool P = decltype(form)::first, R = decltype(form)::second;
#pragma unroll
      for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
        for (int k = 0; k < RS; ++k)
          v[i * RS + k] = op.template at<P, R>(v[i * RS + k], mx, my, slot_pos<N, T, RS>(t, i, k));
    };
    if (!op.precise) line(BoolPair<false, false>{});
    else if (op.rot) line(BoolPair<true, true>{});
    else line(BoolPair<true, false>{});
  } else {
#pragma unroll
    for (int i = 0; i < N / (RS * T); ++i)
#pragma unroll
      for (int k = 0; k < RS; ++k) v[i * RS + k] = op(v[i * RS + k], mx, my, slot_pos<N, T, RS>(t, i, k), b);
  }
}

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

// Persistent, double-buffered line pass.  Each CTA walks tiles of LINES lines
// (grid-stride over all batch items).  While tile i is transformed in
// registers (its exchanges reuse the buffer it arrived in), the cp.async copy
// of tile i+1 into the other buffer is in flight, so the loads of a CTA never
// wait behind its own arithmetic.  Thread (t, l) copies exactly the points
// t + T m of line l that its first stage reads; 16 lanes of a half-warp copy
// 16 neighbouring lines at one point, i.e. 128 contiguous bytes when the lines
// are contiguous along x.
// MODE: 0 forward, 1 inverse, 2 forward / op / inverse (fused k-space step).
constexpr int LBUF = LINES;  // pitch of a tile buffer: point-major, one slot per line

template <int N, int MODE>
__host__ __device__ constexpr size_t lpipe_smem_bytes() {
  return sizeof(float4) * (MODE == 2 ? 2 : 1) * N + 2 * sizeof(float2) * (size_t)N * LBUF;
}

template <int N>
__device__ __forceinline__ void lines_issue(float2* buf, const LineGeom& g, float2* data, long long tile,
                                            int tiles_per_item, int t, int l) {
  constexpr int T = Plan<N>::T;
  const int b = (int)(tile / tiles_per_item);
  const int line = (int)(tile - (long long)b * tiles_per_item) * LINES + l;
  if (line >= g.nlines) return;
  const float2* base = data + b * g.bstride + line_base(g, line);
#pragma unroll
  for (int m = 0; m < N / T; ++m) {
    const int p = t + T * m;
    cp_async8(buf + p * LBUF + l, base + (long long)p * g.pstride);
  }
}

// The tiles base + sub, base + step + sub, ... (tile numbers over all batch
// items) by the threads tid < threads_for<N>() of one group, with the group's
// double buffer bufs (2 N LBUF entries) and the twiddle tables at tw: the
// cp.async copy of the group's next tile is in flight while its current one is
// transformed.  Every thread of the CTA runs the same rounds (a group without
// a tile in a round computes on stale data and stores nothing), so the CTA's
// barriers line up; the arithmetic is that of lfft_tile_one.
template <int N, int MODE, class Op>
__device__ __forceinline__ void lfft_pipe_run(float2* __restrict__ data, const LineGeom& g, const float4* tw,
                                              const Op& op, int batch, float2* bufs, int tid, long long base,
                                              long long step, int sub) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  using Rev = typename Reverse<Rad>::type;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  const int l = tid % LINES, t = tid / LINES;
  const int tiles_per_item = (g.nlines + LINES - 1) / LINES;
  const long long total = (long long)tiles_per_item * batch;
  if (base + sub < total) lines_issue<N>(bufs, g, data, base + sub, tiles_per_item, t, l);
  cp_async_commit();
  int cur = 0;
  for (; base < total; base += step) {
    const long long tile = base + sub, nxt = tile + step;
    if (nxt < total) lines_issue<N>(bufs + (cur ^ 1) * N * LBUF, g, data, nxt, tiles_per_item, t, l);
    cp_async_commit();
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    __syncthreads();
    float2* s = bufs + cur * N * LBUF;
    const bool have = tile < total;
    const int b = have ? (int)(tile / tiles_per_item) : 0;
    const int line = have ? (int)(tile - (long long)b * tiles_per_item) * LINES + l : g.nlines;
    const bool ok = line < g.nlines;
    float2 v[N / T];
    stage_read<N, T, R1, LBUF>(s, v, t, l);
    if constexpr (MODE == 1) {
      run_stages<N, T, LBUF, true>(Rad{}, v, s, tw, t, l);
    } else {
      run_stages<N, T, LBUF, false>(Rad{}, v, s, tw, t, l);
    }
    float2* gbase = data + b * g.bstride + (ok ? line_base(g, line) : 0);
    if constexpr (MODE == 2) {
      const int lc = ok ? line : 0;
      const int mx = g.x0 + lc % g.nxa, my = lc / g.nxa;
      op_points<N, T, RS, false>(op, v, mx, my, t, b, nullptr);
      run_stages<N, T, LBUF, true>(Rev{}, v, s, tw + N, t, l);
      lines_store<N, RadInfo<Rev>::last>(v, gbase, g.pstride, ok, t);
    } else {
      lines_store<N, RS>(v, gbase, g.pstride, ok, t);
    }
    __syncthreads();  // the exchanges in s are done before s receives the round after next
    cur ^= 1;
  }
  cp_async_wait_all();
}

template <int N, int MODE, class Op>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_lfft_pipe(float2* __restrict__ data, LineGeom g, const float4* __restrict__ twg, Op op, int batch) {
  extern __shared__ float2 smem[];
  float4* tw = reinterpret_cast<float4*>(smem);  // line fwd [| line rev] tables
  constexpr int NTAB = MODE == 2 ? 2 : 1;
  load_twiddles(tw, twg + TW_LINE_FWD * N, NTAB * N);  // visible after the first round's barrier
  lfft_pipe_run<N, MODE, Op>(data, g, tw, op, batch, smem + 2 * NTAB * N, threadIdx.x, blockIdx.x, gridDim.x, 0);
}

struct NoOp {
  static constexpr bool TABLE = false;
  static constexpr bool FORMS = false;
  __device__ __forceinline__ float2 operator()(float2 v, int, int, int, int) const { return v; }
};

// One tile of LINES lines, loaded straight into registers (every point of the
// tile in flight at once) and stored straight from them: lines line0 ..
// line0 + LINES - 1 of batch item b, by threads tid = 0 .. threads_for<N>() - 1
// (all of which, and any other threads of the CTA, reach the same barriers),
// with the twiddle tables already in shared memory at tw and the exchange
// buffer s (N * LPITCH entries).
template <int N, int MODE, class Op>
__device__ __forceinline__ void lfft_tile_one(float2* __restrict__ data, const LineGeom& g, const float4* tw,
                                              const Op& op, int line0, int b, float2* s, int tid) {
  using P = Plan<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  using Rev = typename Reverse<Rad>::type;
  constexpr int RS = RadInfo<Rad>::last;
  const int l = tid % LINES, t = tid / LINES;
  const int line = line0 + l;
  const bool ok = line < g.nlines;
  float2* base = data + b * g.bstride + (ok ? line_base(g, line) : 0);
  float2 v[N / T];
  lines_load<N>(v, base, g.pstride, ok, t);
  __syncthreads();
  if constexpr (MODE == 1) {
    run_stages<N, T, LPITCH, true>(Rad{}, v, s, tw, t, l);
  } else {
    run_stages<N, T, LPITCH, false>(Rad{}, v, s, tw, t, l);
  }
  if constexpr (MODE == 2) {
    const int lc = ok ? line : 0;
    const int mx = g.x0 + lc % g.nxa, my = lc / g.nxa;
    op_points<N, T, RS, false>(op, v, mx, my, t, b, nullptr);
    run_stages<N, T, LPITCH, true>(Rev{}, v, s, tw + N, t, l);
    lines_store<N, RadInfo<Rev>::last>(v, base, g.pstride, ok, t);
  } else {
    lines_store<N, RS>(v, base, g.pstride, ok, t);
  }
}

// One tile of LINES lines per CTA (lfft_tile_one); the hardware overlaps one
// resident CTA's loads with another's arithmetic.  This is the line pass where
// the array has no tensor-map view (or the autotuner prefers it); the
// persistent cp.async pipeline above is kept behind WDM_LINE_PIPELINE for
// tuning.
template <int N, int MODE, class Op>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks<N>())
k_lfft_tile(float2* __restrict__ data, LineGeom g, const float4* __restrict__ twg, Op op) {
  constexpr int NTAB = MODE == 2 ? 2 : 1;
  extern __shared__ float2 smem[];
  float4* tw = reinterpret_cast<float4*>(smem);  // line fwd [| line rev] tables
  float2* s = smem + 2 * NTAB * N;
  load_twiddles(tw, twg + TW_LINE_FWD * N, NTAB * N);
  lfft_tile_one<N, MODE, Op>(data, g, tw, op, blockIdx.x * LINES, blockIdx.y, s, threadIdx.x);
}

template <int N, int MODE>
__host__ __device__ constexpr size_t ltile_smem_bytes() {
  return sizeof(float2) * (size_t)(2 * (MODE == 2 ? 2 : 1) * N + N * LPITCH);
}

// TMA-fed persistent line pass.  A tile is LINES lines that are neighbours
// along x (one 128-byte row of the box per point), so the box lands in shared
// memory as a dense [N][LINES] array: the layout stage_read expects with a
// pitch of LINES, conflict-free because each half-warp touches one 128-byte
// row.  Each CTA keeps two tile slots: the bulk tensor copy of its next tile
// is in flight while the current one is transformed in place in its own slot
// and stored from registers, so the loads are never behind the arithmetic.
// One thread issues the copies; every wait on a slot's mbarrier is bounded,
// and a CTA that gives up records WDM_DEVERR_TMA_WAIT, drains its copies
// (bounded again) and exits.
template <int N>
struct TmaTile {
  static constexpr int BOXP = N <= 256 ? N : N / 2;  // points per box (box extents are <= 256)
  static constexpr int NBOX = N / BOXP;
  static constexpr unsigned BYTES = (unsigned)(N * LINES * sizeof(float2));
};

template <int N, int MODE>
__host__ __device__ constexpr size_t ltma_smem_bytes() {
  // two tile slots, the twiddle table(s), two mbarriers (, an operator table)
  return 2 * (size_t)TmaTile<N>::BYTES + sizeof(float4) * (MODE == 2 ? 2 : 1) * N + 2 * sizeof(uint64_t) +
         (MODE == 2 ? sizeof(float) * N : 0);
}

// Edge tiles: the map `emap` views the array with the lines' axis outermost
// and a box of 2 columns x 8 rows x BOXP points, so that the box lands as
// [point][row][column], the [N][LINES] layout of a full tile with line
// l = 2 row + column.  The box starts at the last column, x = nxa - 1; its
// second column lies past the tensor, is filled with zeros and never stored.
// A tile's per-item number: rows * tx full tiles, then g.edge edge tiles.
template <int N>
__device__ __forceinline__ void ltma_issue(const CUtensorMap* map, const CUtensorMap* emap, float2* slot,
                                           uint64_t* bar, const LineGeom& g, long long tile, int tx) {
  using TT = TmaTile<N>;
  const long long per_item = (long long)g.rows * tx + g.edge;
  const int b = (int)(tile / per_item);
  const int rem = (int)(tile - (long long)b * per_item);
  mbar_expect_tx(bar, TT::BYTES);
  if (rem >= g.rows * tx) {
    const int e = rem - g.rows * tx;
#pragma unroll
    for (int q = 0; q < TT::NBOX; ++q) tma_load_4d(slot + q * TT::BOXP * LINES, emap, bar, g.nxa - 1, 8 * e, q * TT::BOXP, b);
    return;
  }
  const int row = rem / tx, x0 = (rem - row * tx) * LINES;
#pragma unroll
  for (int q = 0; q < TT::NBOX; ++q) {
    if (g.axis == 1)
      tma_load_4d(slot + q * TT::BOXP * LINES, map, bar, x0, q * TT::BOXP, row, b);
    else
      tma_load_4d(slot + q * TT::BOXP * LINES, map, bar, x0, row, q * TT::BOXP, b);
  }
}

template <int N>
__host__ __device__ constexpr int ltma_min_blocks() {
  return ltma_smem_bytes<N, 2>() * 2 <= 220 * 1024 ? (threads_for<N>() * 2 <= 1024 ? 2 : 1) : 1;
}

template <int N, int MODE, class Op, bool LATE>
__global__ void __launch_bounds__(threads_for<N>(), ltma_min_blocks<N>())
k_lfft_tma(float2* __restrict__ data, const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap emap,
           LineGeom g, const float4* __restrict__ twg, Op op, int batch) {
  using P = Plan<N>;
  using TT = TmaTile<N>;
  constexpr int T = P::T;
  using Rad = typename P::Fwd;
  using Rev = typename Reverse<Rad>::type;
  constexpr int R1 = RadInfo<Rad>::first, RS = RadInfo<Rad>::last;
  constexpr int NTAB = MODE == 2 ? 2 : 1;
  extern __shared__ __align__(1024) unsigned char lsm[];
  float2* slots = reinterpret_cast<float2*>(lsm);
  float4* tw = reinterpret_cast<float4*>(lsm + 2 * TT::BYTES);
  uint64_t* bar = reinterpret_cast<uint64_t*>(lsm + 2 * TT::BYTES + sizeof(float4) * NTAB * N);
  float* optab = reinterpret_cast<float*>(bar + 2);  // N entries (MODE 2)
  const int tid = threadIdx.x;
  const int l = tid % LINES, t = tid / LINES;
  // When the copy of the next tile goes out (LATE, chosen by the launcher).
  // Early: before the wait for the current tile, so that two copies are in
  // flight during the wait, and a barrier closes every tile so that the copy
  // after next may overwrite its slot.  Late: after the current tile's first
  // barrier, by which every thread has finished the other slot's tile, which
  // saves the closing barrier.
  // tiles of 16 columns; when 16 does not divide nxa the last tile of a row
  // reaches past the tensor (zero-filled by the copy, not stored), unless the
  // last column goes to edge tiles
  const int tx = g.edge ? g.nxa / LINES : (g.nxa + LINES - 1) / LINES;
  const long long per_item = (long long)g.rows * tx + g.edge;
  const long long total = per_item * batch;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  load_twiddles(tw, twg + TW_LINE_FWD * N, NTAB * N);
  if constexpr (MODE == 2 && Op::TABLE)
    for (int i = tid; i < N; i += blockDim.x) optab[i] = op.table_entry(i);
  __syncthreads();
  long long tile = blockIdx.x;
  if (tid == 0 && tile < total) ltma_issue<N>(&map, &emap, slots, &bar[0], g, tile, tx);
  unsigned pending = tile < total ? 1u : 0u;  // bit s: slot s has a copy in flight
  for (int it = 0; tile < total; tile += gridDim.x, ++it) {
    const int cur = it & 1;
    const unsigned par = (unsigned)(it >> 1) & 1u;  // slot cur's k-th use completes phase k
    const long long nxt = tile + gridDim.x;
    if (!LATE && nxt < total) {
      if (tid == 0) ltma_issue<N>(&map, &emap, slots + (cur ^ 1) * N * LINES, &bar[cur ^ 1], g, nxt, tx);
      pending |= 1u << (cur ^ 1);
    }
    const bool landed = mbar_wait_bounded(&bar[cur], par);
    if constexpr (LATE) fence_proxy_async_smem();  // this thread is done with the other slot's last tile
    if (!__syncthreads_and(landed)) {
      if (tid == 0 && g.err) atomicOr(g.err, WDM_DEVERR_TMA_WAIT);
      // drain: the slot that timed out and the look-ahead copy, each bounded
      const bool d0 = mbar_wait_bounded(&bar[cur], par);
      const bool d1 = !((pending >> (cur ^ 1)) & 1u) || mbar_wait_bounded(&bar[cur ^ 1], (unsigned)((it + 1) >> 1) & 1u);
      if (tid == 0 && g.err && !(d0 && d1)) atomicOr(g.err, WDM_DEVERR_TMA_DRAIN);
      return;
    }
    pending &= ~(1u << cur);
    if (LATE && nxt < total) {
      if (tid == 0) ltma_issue<N>(&map, &emap, slots + (cur ^ 1) * N * LINES, &bar[cur ^ 1], g, nxt, tx);
      pending |= 1u << (cur ^ 1);
    }
    float2* s = slots + cur * N * LINES;
    const int b = (int)(tile / per_item);
    const int rem = (int)(tile - (long long)b * per_item);
    const bool edge = rem >= g.rows * tx;
    const int row = edge ? 8 * (rem - g.rows * tx) + (l >> 1) : rem / tx;
    const int x = edge ? g.nxa - 1 + (l & 1) : (rem - row * tx) * LINES + l;
    const bool ok = x < g.nxa;
    const int mx = ok ? x : 0;
    float2* base = data + b * g.bstride + (long long)row * g.outer + mx;
    float2 v[N / T];
    stage_read<N, T, R1, LINES>(s, v, t, l);
    if constexpr (MODE == 1) {
      run_stages<N, T, LINES, true>(Rad{}, v, s, tw, t, l);
    } else {
      run_stages<N, T, LINES, false>(Rad{}, v, s, tw, t, l);
    }
    if constexpr (MODE == 2) {
      op_points<N, T, RS, true>(op, v, g.x0 + mx, row, t, b, optab);
      run_stages<N, T, LINES, true>(Rev{}, v, s, tw + N, t, l);
      lines_store<N, RadInfo<Rev>::last>(v, base, g.pstride, ok, t);
    } else {
      lines_store<N, RS>(v, base, g.pstride, ok, t);
    }
    if constexpr (!LATE) {
      // the slot's generic reads and writes are done before the copy of
      // tile + 2 gridDim overwrites it
      fence_proxy_async_smem();
      __syncthreads();
    }
  }
}

// ----------------------------------------------------------------------------
// Arguments of the fused x passes (xpass_warp.cuh)
// ----------------------------------------------------------------------------
struct RhoArgs {
  const float* mx;   // separable absorbing-mask tables (null: no mask)
  const float* my;
  const float* mz;
  const float* rho_b;  // baryon density [nz][ny][nx] (null: none)
  long long rb_bstride;
  // ny*nz flags of the rows of rho_b that hold mass (null: every row); the
  // other rows are zero and are not read
  const int* rb_rows = nullptr;
  int write_psi;     // 0: density only (psi is already in real space, left untouched)
  int* nonfinite;    // set to 1 when any density value is NaN/Inf (null: unchecked)
  int* err = nullptr;  // error word of abandoned waits of the staged pass (may be null)
  // Per-batch-item constant subtracted from rho before the transform (an
  // estimate of its mean).  Only the k = 0 mode changes, which the Poisson
  // solve drops, so any value is exact; a value near the mean keeps the FP32
  // transform's rounding relative to rho - <rho> instead of rho.
  const float* shift;
  // Non-null: accumulate the density maximum and moments of |psi|^2 into these
  // zeroed words ([batch][CENTRE_WORDS]) for the tide frame of the next kick.
  unsigned long long* centre = nullptr;
};

// ----------------------------------------------------------------------------
// Arguments of the kick passes
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
  int* err = nullptr;    // error word of abandoned waits of the staged pass (may be null)
  // Frame of the tide (used when tidal != 0): null keeps 1/2 x^T T x about the
  // box centre; otherwise 4 floats per batch item, the coordinates of cell 0
  // in the tide's frame and a constant added to the tide (tide_frame_of).
  const float* frame = nullptr;
};

// Per-batch-item words a density pass accumulates for the tide frame: [0] the
// density maximum packed as (float bits of rho) << 32 | (0xffffffff - flat
// cell index), so that the largest word is the largest rho at its first cell
// in memory order; [1..4] the FP64 sums of rho, rho i, rho j, rho k over the
// item (i, j, k the cell indices along x, y, z).  rho = |psi|^2, without the
// baryon density.  Zeroed before every density pass that fills them.
enum { CENTRE_WORDS = 5 };

// The tide's frame for one batch item from the words of the last density pass
// (CentreWords) and its tidal tensor T6.  x_c is the centre of the cell of the
// density maximum and <x> the density-weighted mean position; for the
// quadratic tide Phi(x) = 1/2 x^T T x:
//   mode 1: Phi(x) - Phi(x_c), the potential src/physics/tidal_fields.jl:114
//     leaves (its gradient cancellation, :115 and :126-146, rebinds the
//     function's local argument and does not change the caller's potential);
//   mode 2: Phi(x) - Phi(x_c) - grad Phi(x_c).(x - <x>), what that
//     cancellation computes: = 1/2 (x - x_c)^T T (x - x_c) + (T x_c).(<x> - x_c).
// out: the coordinates of cell 0 in the frame (x0, y0, z0) and the constant,
// from FP64 arithmetic; x0, d: cell 0's coordinates and the spacings.
__device__ inline void tide_frame_of(float* out, const float* T6, const unsigned long long* w, int mode, int nx,
                                     int ny, const double* x0, const double* d) {
  const unsigned flat = 0xffffffffu - (unsigned)(w[0] & 0xffffffffull);
  const unsigned ix = flat % (unsigned)nx, iy = (flat / (unsigned)nx) % (unsigned)ny;
  const unsigned iz = flat / ((unsigned)nx * (unsigned)ny);
  const double xc = x0[0] + d[0] * ix, yc = x0[1] + d[1] * iy, zc = x0[2] + d[2] * iz;
  const double txx = T6[0], tyy = T6[1], tzz = T6[2], txy = T6[3], txz = T6[4], tyz = T6[5];
  const double gx = txx * xc + txy * yc + txz * zc;
  const double gy = txy * xc + tyy * yc + tyz * zc;
  const double gz = txz * xc + tyz * yc + tzz * zc;
  if (mode == 1) {
    out[0] = (float)x0[0];
    out[1] = (float)x0[1];
    out[2] = (float)x0[2];
    out[3] = (float)(-0.5 * (xc * gx + yc * gy + zc * gz));
    return;
  }
  const double s0 = __longlong_as_double((long long)w[1]);
  const double inv = s0 > 0.0 ? 1.0 / s0 : 0.0;
  const double mx = x0[0] + d[0] * (__longlong_as_double((long long)w[2]) * inv);
  const double my = x0[1] + d[1] * (__longlong_as_double((long long)w[3]) * inv);
  const double mz = x0[2] + d[2] * (__longlong_as_double((long long)w[4]) * inv);
  out[0] = (float)(-d[0] * ix);
  out[1] = (float)(-d[1] * iy);
  out[2] = (float)(-d[2] * iz);
  out[3] = (float)(gx * (mx - xc) + gy * (my - yc) + gz * (mz - zc));
}


// psi * exp(-i dt pot).
// Plain form: one FP32 sincos of pot*dt.
// Precise form: theta = pot*dt as an unevaluated float pair, reduced by 2 pi
// (Cody-Waite with a two-term 2 pi) to |r| <= pi, then applied as
// psi + psi (exp(-i r) - 1) with exp(-i r) - 1 = (-2 sin^2(r/2), -sin r) from the
// series sin/cos of r/2 (wdm_math.cuh): accurate relative to |exp(-i r) - 1|, so
// small kicks do not carry the fixed modulus error of a cosine rounded near 1.
// kick_factor gives the phase factor once, so that a caller applying the same
// kick to two states (the adjoint: psi and lam) evaluates it once:
// exp(-i r) - 1 in the precise form, exp(-i th) in the plain form.
// The _t forms take the form as a compile-time flag, so that a caller can
// test a.precise once for many points.
template <bool PRECISE>
__device__ __forceinline__ float2 kick_factor_t(float pot, const KickArgs& a) {
  if constexpr (PRECISE) {
    const float th = pot * a.dt_hi;
    const float te = fmaf(pot, a.dt_hi, -th) + pot * a.dt_lo;
    const float n = rintf(th * 0.15915494309189535f);
    const float r = fmaf(-n, 6.28318548202514648f, th) + fmaf(-n, -1.7484555e-07f, te);
    return expm1_neg_i(r);  // (cos r - 1, -sin r)
  }
  const float2 sc = sincos_plain(pot * a.dt_hi);
  return make_float2(sc.y, -sc.x);
}

__device__ __forceinline__ float2 kick_factor(float pot, const KickArgs& a) {
  if (a.precise) return kick_factor_t<true>(pot, a);
  return kick_factor_t<false>(pot, a);
}

// v exp(-i th), or v exp(+i th) (CONJ), from the factor of kick_factor.  In
// the precise form the conjugate factor is bit for bit the factor of -pot (the
// reduction and the series are odd/even in th), so CONJ is a kick by -pot.
template <bool PRECISE, bool CONJ = false>
__device__ __forceinline__ float2 kick_by_t(float2 v, float2 e) {
  if (CONJ) e.y = -e.y;
  if constexpr (PRECISE) return make_float2(v.x + (v.x * e.x - v.y * e.y), v.y + (v.x * e.y + v.y * e.x));
  return cmul(v, e);
}

template <bool CONJ = false>
__device__ __forceinline__ float2 kick_by(float2 v, float2 e, const KickArgs& a) {
  if (a.precise) return kick_by_t<true, CONJ>(v, e);
  return kick_by_t<false, CONJ>(v, e);
}

__device__ __forceinline__ float2 apply_kick(float2 v, float pot, const KickArgs& a) {
  return kick_by(v, kick_factor(pot, a), a);
}

}  // namespace wdm
