// C-ABI of libwavedm: context, tables, step orchestration, diagnostics, CIC.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/wavedm.h"
#include "aux_kernels.cuh"
#include "ensemble.cuh"
#include "kernel_set.h"

namespace wdm {
thread_local long long tl_kernel_launches = 0;

const KernelSet* ks_8();
const KernelSet* ks_12();
const KernelSet* ks_16();
const KernelSet* ks_24();
const KernelSet* ks_32();
const KernelSet* ks_48();
const KernelSet* ks_64();
const KernelSet* ks_96();
const KernelSet* ks_128();
const KernelSet* ks_192();
const KernelSet* ks_256();
const KernelSet* ks_384();
const KernelSet* ks_512();

const KernelSet* kernels_for(int n) {
  switch (n) {
    case 8: return ks_8();
    case 12: return ks_12();
    case 16: return ks_16();
    case 24: return ks_24();
    case 32: return ks_32();
    case 48: return ks_48();
    case 64: return ks_64();
    case 96: return ks_96();
    case 128: return ks_128();
    case 192: return ks_192();
    case 256: return ks_256();
    case 384: return ks_384();
    case 512: return ks_512();
    default: return nullptr;
  }
}
}  // namespace wdm

using namespace wdm;

static std::string g_create_error;

// Message returned by wdm_last_error(NULL) for entry points without a context.
void wdm_set_global_error(const std::string& msg) { g_create_error = msg; }

// Passes of the pipeline, for launch counting and per-pass event timing.
enum Pass {
  P_KICK_FWD = 0,  // P1: Phi C2R + kick + psi x-FFT
  P_PSI_Y_FWD,     // P2
  P_PSI_Z_DRIFT,   // P3
  P_PSI_Y_INV,     // P4
  P_X_INV_RHO,     // P5: psi x-iFFT (+mask) + density R2C
  P_H_Y_FWD,       // P6
  P_H_Z_POISSON,   // P7
  P_H_Y_INV,       // P8
  P_KICK,          // final half kick (no FFT)
  P_DENSITY,       // density R2C of real-space psi (start of a run)
  P_CIC_DEPOSIT,
  P_X_FFT,         // plain x-FFT (wdm_drift)
  P_PHI_OUT,       // Phi C2R to a real field
  P_ADJ_KICK,      // adjoint kick: lam x-iFFT, exp(+i th) lam, mu R2C
  P_ADJ_POISSON,   // Poisson solve of mu (H y, z, y)
  P_ADJ_APPLY,     // lam += 2 G(mu) psi (+mask), x-FFT
  NPASS
};
static const char* const PASS_NAMES[NPASS] = {
    "kick_xfft_fwd", "psi_y_fwd", "psi_z_drift", "psi_y_inv", "psi_x_inv_rho", "rho_y_fwd", "rho_z_poisson",
    "phi_y_inv",     "kick_final", "rho_density", "cic_deposit", "psi_x_fwd", "phi_x_c2r",
    "adj_kick",   "adj_poisson", "adj_apply"};

struct Profiler {
  bool on = false;
  uint64_t mask = ~0ull;  // passes bracketed by events while on (bit p: pass p)
  std::vector<cudaEvent_t> pool;
  struct Rec {
    int pass;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  int64_t launches[NPASS] = {0};
  double ms[NPASS] = {0};
};

// Line passes the autotuner chooses an implementation for.
// (the x passes' choice is X_IMPL_STAGED / X_IMPL_DIRECT, the line passes' LINE_IMPL_TMA / LINE_IMPL_TILE;
// 0 is the preferred implementation of each)
// (LP_X_RHO_B: the density pass with a baryon density to add, which the staged
// pass prefetches and the direct pass loads after its transform)
enum { LP_PSI_Y = 0, LP_PSI_Z = 1, LP_H_Y = 2, LP_H_Z = 3, LP_X_KICK = 4, LP_X_RHO = 5, LP_X_RHO_B = 6, LP_COUNT = 7 };

struct wdm_ctx {
  wdm_desc d{};
  int nxh = 0;           // half-spectrum columns (nx/2 + 1)
  int hpitch = 0;        // H row pitch: nxh rounded up to even, so rows are 16-byte
                         // aligned and H has a tensor-map view for the TMA line passes
  long long ncell = 0;   // cells per batch item
  long long nhalf = 0;   // H entries per batch item (hpitch * ny * nz, the batch stride)
  cudaStream_t st = nullptr;
  const KernelSet *kx = nullptr, *ky = nullptr, *kz = nullptr;
  double dx = 0, dy = 0, dz = 0, x0 = 0, y0 = 0, z0 = 0;
  // device buffers
  float2* psi = nullptr;
  float2* H = nullptr;
  float4 *twx = nullptr, *twy = nullptr, *twz = nullptr;  // (hi, lo) twiddles
  float *kx2 = nullptr, *ky2 = nullptr, *kz2 = nullptr;
  float4 *cxy = nullptr, *cz = nullptr;  // precise drift factors per z line / per kz (cached per dt)
  int drift_rot = 0;                      // cz holds rotated (flagged) entries
  double tab_dt = NAN;
  float *mx = nullptr, *my = nullptr, *mz = nullptr;     // absorbing mask tables (cached per dt)
  double mask_dt = NAN;
  float* V = nullptr;
  float* rho_b = nullptr;
  int* rb_rows = nullptr;           // ny*nz flags: x rows holding deposited baryon mass
  CicParticle* parts = nullptr;
  long long nparts = 0;
  float* T6b = nullptr;             // per-batch-item tidal tensors
  std::vector<double> tide;         // host schedule rows of 6
  int tide_on = 0;
  // clock of the schedule: row s is the tensor at time tide_t0 + s tide_dt
  // (tide_dt == 0: no clock, row s belongs to kick s of each wdm_step call)
  double tide_t0 = 0.0, tide_dt = 0.0;
  // frame of the tide (wdm_tidal_centering) and the words the density passes
  // leave for it ([batch][CENTRE_WORDS], allocated when a frame is chosen)
  int tide_centre = 0;
  unsigned long long* centre = nullptr;
  float* frame = nullptr;           // [batch][4] the tide's frame of the next kick
  int* flag = nullptr;              // device words: [0] non-finite psi, [1] abandoned-wait bits
  float* scratch_f = nullptr;       // float field scratch [batch][ncell]
  float2* scratch_h = nullptr;      // half-spectrum scratch
  double* red = nullptr;            // reduction partials
  int red_blocks = 0;
  double* sums = nullptr;           // [batch] FP64 sums for the density shift
  float* shift = nullptr;           // [batch] estimate of <rho> subtracted before the R2C (psi path)
  float* shift_in = nullptr;        // [batch] mean of a wdm_poisson input
  double rho_b_mean = 0.0;          // mean baryon density (static particles)
  int have_psi = 0;
  int phi_valid = 0;
  int64_t launch_count = 0;
  // autotuned implementation of each line pass (LP_*) and the candidate timings
  int line_impl[LP_COUNT] = {0, 0, 0, 0, 0, 0, 0};
  double line_ms[LP_COUNT][2] = {{-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}};
  // adjoint buffers (allocated on first use)
  float2* lam = nullptr;            // adjoint state [batch][ncell]
  float2* Hmu = nullptr;            // half spectrum of mu
  float* rho_t = nullptr;           // target density
  float* D6 = nullptr;              // tidal direction
  double* adj_acc = nullptr;        // [2 batch]: loss, dL/da
  std::vector<float2*> ck_psi, ck_H, slot_psi, slot_H;  // checkpoints / segment states (set 0)
  std::vector<float2*> slot2_psi, slot2_H;              // segment states, set 1
  cudaStream_t st_rec = nullptr;    // adjoint: recompute of the next segment, beside the reverse sweep
  cudaEvent_t ev_ck = nullptr, ev_rec[2] = {nullptr, nullptr}, ev_bwd[2] = {nullptr, nullptr};
  // baryons: the CIC deposit of the current particles is in rho_b.  The
  // particles are static (src/simulation_main.jl:248-261 computes their
  // potential once, before the loop), so the deposit is made once per
  // particle set and every density pass reads it.
  int rb_ready = 0;
  // diagnostics: radii histogram and minimum words (allocated on first use)
  double* diag_wsum = nullptr;
  unsigned long long* diag_wmin = nullptr;
  long long version = 0;            // bumped by every set_* call that a captured graph bakes in
  struct wdm_group* self_group = nullptr;  // single-member group of wdm_step_graph
  Profiler prof;
  std::string err;
};

static cudaEvent_t prof_event(wdm_ctx* c) {
  if (!c->prof.pool.empty()) {
    cudaEvent_t e = c->prof.pool.back();
    c->prof.pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Collect finished event pairs into the per-pass totals.
static cudaError_t prof_flush(wdm_ctx* c) {
  if (c->prof.pending.empty()) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return e;
  for (auto& r : c->prof.pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) c->prof.ms[r.pass] += ms;
    c->prof.launches[r.pass] += 1;
    c->prof.pool.push_back(r.a);
    c->prof.pool.push_back(r.b);
  }
  c->prof.pending.clear();
  return cudaSuccess;
}

// Run one pass launch: counted always, bracketed by events when profiling.
// A launcher outside the KernelSet (the auxiliary kernels) counts as one.
template <class F>
static cudaError_t counted(wdm_ctx* c, F launch) {
  const long long l0 = tl_kernel_launches;
  const cudaError_t e = launch();
  const long long n = tl_kernel_launches - l0;
  c->launch_count += n > 0 ? n : 1;
  return e;
}

template <class F>
static cudaError_t run_pass(wdm_ctx* c, int pass, F launch) {
  if (!c->prof.on || !((c->prof.mask >> pass) & 1ull)) return counted(c, launch);
  cudaEvent_t a = prof_event(c), b = prof_event(c);
  cudaEventRecord(a, c->st);
  cudaError_t e = counted(c, launch);
  cudaEventRecord(b, c->st);
  c->prof.pending.push_back({pass, a, b});
  if (c->prof.pending.size() > 4096) {
    cudaError_t f = prof_flush(c);
    if (e == cudaSuccess) e = f;
  }
  return e;
}

// Algorithmic bytes of one launch of a pass: every operand read once and
// written once (complex64 8 B, float 4 B), all batch items.
static double pass_bytes(const wdm_ctx* c, int p) {
  const double B = c->d.batch, nc = (double)c->ncell * B, nh = (double)c->nxh * c->d.ny * c->d.nz * B;
  switch (p) {
    case P_KICK_FWD:
    case P_KICK: return 16.0 * nc + 8.0 * nh + (c->V ? 4.0 * nc : 0.0);
    case P_PSI_Y_FWD:
    case P_PSI_Z_DRIFT:
    case P_PSI_Y_INV:
    case P_X_FFT: return 16.0 * nc;
    case P_X_INV_RHO: return 16.0 * nc + 8.0 * nh + (c->nparts ? 4.0 * c->ncell : 0.0);
    case P_DENSITY: return 8.0 * nc + 8.0 * nh + (c->nparts ? 4.0 * c->ncell : 0.0);
    case P_H_Y_FWD:
    case P_H_Z_POISSON:
    case P_H_Y_INV: return 16.0 * nh;
    case P_CIC_DEPOSIT: return (double)c->nparts * (sizeof(CicParticle) + 8 * 2 * sizeof(float));
    case P_PHI_OUT: return 8.0 * nh + 4.0 * nc;
    case P_ADJ_KICK: return 24.0 * nc + 16.0 * nh;   // lam in/out, pre-kick psi, H in, mu spectrum out
    case P_ADJ_POISSON: return 3.0 * 16.0 * nh;
    case P_ADJ_APPLY: return 24.0 * nc + 8.0 * nh;   // lam in/out, pre-kick psi, G(mu) in
    default: return 0.0;
  }
}

// --------------------------------------------------------------------------
// helpers
// --------------------------------------------------------------------------
static wdm_status fail(wdm_ctx* c, wdm_status s, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return s;
}

static wdm_status cuda_fail(wdm_ctx* c, cudaError_t e, const char* what) {
  return fail(c, WDM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define WDM_CU(c, call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail((c), e_, #call); \
  } while (0)

// Host-side fault injection (no GPU fault): WDM_FAULT=nonfinite makes the
// finite check report a non-finite density; WDM_FAULT=alloc makes every device
// allocation fail, and WDM_FAULT=alloc:N only the N-th one counted since the
// variable took its present value (so a context creation can fail half way).
static bool fault_injected(const char* what) {
  const char* f = std::getenv("WDM_FAULT");
  return f && std::strstr(f, what) != nullptr;
}

static std::mutex g_fault_mu;
static std::string g_fault_value;
static long long g_fault_allocs = 0;

static bool alloc_fault_injected() {
  const char* f = std::getenv("WDM_FAULT");
  if (!f) return false;
  const char* a = std::strstr(f, "alloc");
  if (!a) return false;
  std::lock_guard<std::mutex> lock(g_fault_mu);
  if (g_fault_value != f) {
    g_fault_value = f;
    g_fault_allocs = 0;
  }
  ++g_fault_allocs;
  if (a[5] != ':') return true;
  return g_fault_allocs == std::atoll(a + 6);
}

template <class T>
static wdm_status dalloc(wdm_ctx* c, T** p, size_t count) {
  if (alloc_fault_injected()) {
    *p = nullptr;
    return fail(c, WDM_ERR_ALLOC, "injected allocation failure (WDM_FAULT=alloc)");
  }
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T) + 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(c, WDM_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return WDM_OK;
}

#define WDM_TRY(x)                    \
  do {                                \
    wdm_status s_ = (x);              \
    if (s_ != WDM_OK) return s_;      \
  } while (0)

static void axis_geom(int n, double L, int conv, double* d, double* x0) {
  if (conv == WDM_GRID_REFERENCE) {
    *d = L / (n - 1);
    *x0 = -L / 2;
  } else {
    *d = L / n;
    *x0 = -L / 2;
  }
}

// angular wavenumber of FFT index m on an axis of n points and period L
static double kval(int m, int n, double L) {
  const int s = (m < (n + 1) / 2) ? m : m - n;  // fftfreq order: 0..ceil(n/2)-1, -floor(n/2)..-1
  return 2.0 * M_PI * s / L;
}

// The four stage-major (hi, lo) twiddle tables of an axis (TW_TABLES x n).
static wdm_status upload_twiddles(wdm_ctx* c, float4** dst, const KernelSet* ks) {
  const int n = ks->n;
  std::vector<float4> h((size_t)TW_TABLES * n);
  ks->fill_twiddles(h.data());
  WDM_TRY(dalloc(c, dst, h.size()));
  WDM_CU(c, cudaMemcpy(*dst, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice));
  return WDM_OK;
}

static wdm_status upload_k2(wdm_ctx* c, float** dst, int n, double L) {
  std::vector<float> h(n);
  for (int m = 0; m < n; ++m) {
    const double k = kval(m, n, L);
    h[m] = (float)(k * k);
  }
  WDM_TRY(dalloc(c, dst, n));
  WDM_CU(c, cudaMemcpy(*dst, h.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  return WDM_OK;
}

// Drift factors of the precise form, in FP64 with the phases reduced mod 2 pi
// in double: cxy[my][mx] = exp(-i (kx^2 + ky^2) dt/2) / (nx ny nz) and
// cz[mz] = exp(-i kz^2 dt/2), each kept as an FP32 (hi, lo) pair
// (pack_twiddle).
static wdm_status ensure_drift_tables(wdm_ctx* c, double dt) {
  if (c->tab_dt == dt) return WDM_OK;
  const int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
  auto phase = [&](int m, int n, double L) {
    const double k = kval(m, n, L);
    return std::fmod(0.5 * k * k * dt, 2.0 * M_PI);
  };
  std::vector<double> thx(nx), thy(ny);
  for (int m = 0; m < nx; ++m) thx[m] = phase(m, nx, c->d.lx);
  for (int m = 0; m < ny; ++m) thy[m] = phase(m, ny, c->d.ly);
  const double scale = 1.0 / ((double)nx * ny * nz);
  std::vector<float4> hxy((size_t)nx * ny), hz(nz);
  for (int my = 0; my < ny; ++my)
    for (int mx = 0; mx < nx; ++mx) {
      const double th = std::fmod(thx[mx] + thy[my], 2.0 * M_PI);
      hxy[(size_t)my * nx + mx] = pack_twiddle(scale * std::cos(th), -scale * std::sin(th));
    }
  int rot = 0;
  for (int m = 0; m < nz; ++m) {
    const double th = phase(m, nz, c->d.lz);
    hz[m] = pack_twiddle(std::cos(th), -std::sin(th));
    unsigned bits;
    std::memcpy(&bits, &hz[m].w, sizeof(bits));
    rot |= (int)(bits & 1u);
  }
  WDM_CU(c, cudaMemcpyAsync(c->cxy, hxy.data(), hxy.size() * sizeof(float4), cudaMemcpyHostToDevice, c->st));
  WDM_CU(c, cudaMemcpyAsync(c->cz, hz.data(), hz.size() * sizeof(float4), cudaMemcpyHostToDevice, c->st));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  c->drift_rot = rot;
  c->tab_dt = dt;
  return WDM_OK;
}

// Absorbing mask exp(-alpha dt (6 - tanh((x+X)/w) + tanh((x-X)/w) - ...)) of
// src/solver/fft_operators.jl:22-27 factorises into one table per axis:
// m_a(x) = exp(-alpha dt (2 - tanh((x+X)/w) + tanh((x-X)/w))), w = X/50.
static wdm_status ensure_mask_tables(wdm_ctx* c, double dt) {
  if (c->d.absorb_alpha == 0.0 || c->mask_dt == dt) return WDM_OK;
  const int n[3] = {c->d.nx, c->d.ny, c->d.nz};
  const double L[3] = {c->d.lx, c->d.ly, c->d.lz};
  const double d[3] = {c->dx, c->dy, c->dz};
  const double o[3] = {c->x0, c->y0, c->z0};
  float* dst[3] = {c->mx, c->my, c->mz};
  for (int a = 0; a < 3; ++a) {
    const double X = L[a] / 2, w = X / 50;
    std::vector<float> h(n[a]);
    for (int i = 0; i < n[a]; ++i) {
      const double x = o[a] + d[a] * i;
      h[i] = (float)std::exp(-c->d.absorb_alpha * dt * (2.0 - std::tanh((x + X) / w) + std::tanh((x - X) / w)));
    }
    WDM_CU(c, cudaMemcpyAsync(dst[a], h.data(), n[a] * sizeof(float), cudaMemcpyHostToDevice, c->st));
    WDM_CU(c, cudaStreamSynchronize(c->st));
  }
  c->mask_dt = dt;
  return WDM_OK;
}

static RowGeom rows_psi(const wdm_ctx* c) {
  RowGeom r;
  r.nrows = c->d.ny * c->d.nz;
  r.ny = c->d.ny;
  r.pitch = c->d.nx;
  r.bstride = c->ncell;
  return r;
}

// The rows of psi for the tuned x pass `kind` (LP_X_KICK, LP_X_RHO or LP_X_RHO_B).
static RowGeom rows_psi(const wdm_ctx* c, int kind) {
  RowGeom r = rows_psi(c);
  r.impl = c->line_impl[kind];
  return r;
}

// Lines along y (or z) of an array [batch][nz][ny][pitch] whose first xext
// entries of a row are data.
static LineGeom lines_y(const wdm_ctx* c, int xext, long long pitch, long long bstride) {
  LineGeom g;
  g.nlines = xext * c->d.nz;
  g.nxa = xext;
  g.outer = (long long)c->d.ny * pitch;
  g.pstride = pitch;
  g.bstride = bstride;
  g.axis = 1;
  g.rows = c->d.nz;
  g.pitch = pitch;
  g.err = c->flag + 1;
  g.impl = c->line_impl[xext == c->nxh ? LP_H_Y : LP_PSI_Y];
  return g;
}

static LineGeom lines_z(const wdm_ctx* c, int xext, long long pitch, long long bstride) {
  LineGeom g;
  g.nlines = xext * c->d.ny;
  g.nxa = xext;
  g.outer = pitch;
  g.pstride = (long long)c->d.ny * pitch;
  g.bstride = bstride;
  g.axis = 2;
  g.rows = c->d.ny;
  g.pitch = pitch;
  g.err = c->flag + 1;
  g.impl = c->line_impl[xext == c->nxh ? LP_H_Z : LP_PSI_Z];
  return g;
}

// --------------------------------------------------------------------------
// pipeline pieces
// --------------------------------------------------------------------------
// density (+baryons) of psi -> H, then the Poisson solve on H (P5..P8).
// The CIC deposit of the current particles into rho_b (zero before it), made
// once per particle set.
static wdm_status ensure_deposit(wdm_ctx* c) {
  if (c->nparts == 0 || c->rb_ready) return WDM_OK;
  cudaError_t e = run_pass(c, P_CIC_DEPOSIT, [&] {
    return launch_cic_deposit(c->rho_b, c->parts, c->nparts, c->d.nx, c->d.ny, c->d.nz, c->rb_rows, c->st);
  });
  if (e != cudaSuccess) return cuda_fail(c, e, "cic deposit");
  c->rb_ready = 1;
  return WDM_OK;
}

// Density pass (P5) and Poisson solve (P6-P8).  write_psi != 0: psi holds
// x-spectral data (after P4); the pass inverts it first (with the absorbing
// mask) and writes real-space psi back.  With baryons, P5 adds the kept
// deposit (only the rows it flags are read).
static wdm_status density_poisson(wdm_ctx* c, int write_psi, double dt_mask) {
  const int B = c->d.batch;
  if (c->nparts > 0) WDM_TRY(ensure_deposit(c));
  RhoArgs ra{};
  const bool mask = write_psi && c->d.absorb_alpha != 0.0;
  if (mask) WDM_TRY(ensure_mask_tables(c, dt_mask));
  ra.mx = mask ? c->mx : nullptr;
  ra.my = mask ? c->my : nullptr;
  ra.mz = mask ? c->mz : nullptr;
  ra.rho_b = c->nparts > 0 ? c->rho_b : nullptr;
  ra.rb_rows = c->nparts > 0 ? c->rb_rows : nullptr;
  ra.rb_bstride = 0;
  ra.write_psi = write_psi;
  ra.nonfinite = c->flag;
  ra.shift = c->shift;
  ra.err = c->flag + 1;
  if (c->tide_centre && c->tide_on) {
    WDM_CU(c, cudaMemsetAsync(c->centre, 0, sizeof(unsigned long long) * CENTRE_WORDS * B, c->st));
    ra.centre = c->centre;
  }
  cudaError_t e = run_pass(c, write_psi ? P_X_INV_RHO : P_DENSITY, [&] {
    return c->kx->x_inv_rho(c->psi, c->H, rows_psi(c, c->nparts > 0 ? LP_X_RHO_B : LP_X_RHO), c->hpitch, c->nhalf,
                            c->twx, ra, B, c->st);
  });
  if (e != cudaSuccess) return cuda_fail(c, e, "x_inv_rho");
  if ((e = run_pass(c, P_H_Y_FWD, [&] { return c->ky->lfft(c->H, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, false, B, c->st); })) !=
      cudaSuccess)
    return cuda_fail(c, e, "H y fwd");
  PoissonOp po;
  po.kx2 = c->kx2;
  po.ky2 = c->ky2;
  po.kz2 = c->kz2;
  po.coef = (float)(-c->d.poisson_coeff / ((double)c->d.nx * c->d.ny * c->d.nz));
  if ((e = run_pass(c, P_H_Z_POISSON,
                    [&] { return c->kz->lfft_poisson(c->H, lines_z(c, c->nxh, c->hpitch, c->nhalf), c->twz, po, B, c->st); })) !=
      cudaSuccess)
    return cuda_fail(c, e, "H z poisson");
  if ((e = run_pass(c, P_H_Y_INV, [&] { return c->ky->lfft(c->H, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, true, B, c->st); })) !=
      cudaSuccess)
    return cuda_fail(c, e, "H y inv");
  c->phi_valid = 1;
  return WDM_OK;
}

static void split_dt(double dt, float* hi, float* lo) {
  *hi = (float)dt;
  *lo = (float)(dt - (double)*hi);
}

static KickArgs kick_args(const wdm_ctx* c, double dt, int sched_row) {
  KickArgs a{};
  split_dt(dt, &a.dt_hi, &a.dt_lo);
  a.T6b = nullptr;
  a.tidal = 0;
  if (c->tide_on == 2) {
    a.T6b = c->T6b;
    a.tidal = 1;
  } else if (c->tide_on == 1) {
    const int nrow = (int)(c->tide.size() / 6);
    const int r = sched_row < nrow ? sched_row : nrow - 1;
    for (int q = 0; q < 6; ++q) a.T6[q] = (float)c->tide[6 * r + q];
    a.tidal = 1;
  }
  a.x0 = (float)c->x0;
  a.y0 = (float)c->y0;
  a.z0 = (float)c->z0;
  a.dx = (float)c->dx;
  a.dy = (float)c->dy;
  a.dz = (float)c->dz;
  a.kerr = (float)c->d.kerr;
  a.V = c->V;
  a.v_bstride = c->ncell;
  a.precise = c->d.phase_mode == WDM_PHASE_PRECISE;
  a.err = c->flag + 1;
  if (c->tide_centre && a.tidal) a.frame = c->frame;
  return a;
}

// Schedule row of the kick at time t that is kick s of a call: with a clock
// the row whose time is nearest to t, without one row s.  A one-row schedule
// is a constant tide (row 0 at every time).
static int tide_row(const wdm_ctx* c, double t, int s) {
  if (c->tide.size() <= 6) return 0;
  if (c->tide_dt > 0.0) return (int)std::floor((t - c->tide_t0) / c->tide_dt + 0.5);
  return s;
}

// The kicks at times t0 + s dt, s = 0 .. nkicks-1, of one call all have a row.
static wdm_status check_tide_rows(wdm_ctx* c, double t0, double dt, int nkicks, const char* who) {
  if (c->tide_on != 1 || nkicks <= 0) return WDM_OK;
  const int nrow = (int)(c->tide.size() / 6);
  if (nrow == 1) return WDM_OK;
  for (int s : {0, nkicks - 1}) {
    const int r = tide_row(c, t0 + s * dt, s);
    if (r < 0 || r >= nrow) {
      if (c->tide_dt > 0.0)
        return fail(c, WDM_ERR_INVALID, std::string(who) + ": the kick at t = " + std::to_string(t0 + s * dt) +
                                            " falls outside the tidal schedule (" + std::to_string(nrow) +
                                            " rows from t = " + std::to_string(c->tide_t0) + " every " +
                                            std::to_string(c->tide_dt) + ")");
      return fail(c, WDM_ERR_INVALID, std::string(who) + ": tidal schedule has " + std::to_string(nrow) +
                                          " rows, the call needs " + std::to_string(nkicks) + " (or exactly 1)");
    }
  }
  return WDM_OK;
}

// Kick of psi (in place), or of psi_in into c->psi when psi_in is given.  A
// tide anchored at the density maximum first gets its frame from the words of
// the last density pass.
static wdm_status kick(wdm_ctx* c, double dt, int sched_row, bool fwd, const float2* psi_in = nullptr) {
  KickArgs a = kick_args(c, dt, sched_row);
  if (a.frame) {
    cudaError_t e = counted(c, [&] {
      return launch_tide_frame(c->centre, a, c->tide_centre, c->d.nx, c->d.ny, c->d.batch, c->frame, c->st);
    });
    if (e != cudaSuccess) return cuda_fail(c, e, "tide frame");
  }
  const float2* in = psi_in ? psi_in : c->psi;
  cudaError_t e = run_pass(c, fwd ? P_KICK_FWD : P_KICK, [&] {
    return c->kx->x_kick(in, c->psi, c->H, rows_psi(c, LP_X_KICK), c->hpitch, c->nhalf, c->twx, a, fwd, c->d.batch, c->st);
  });
  if (e != cudaSuccess) return cuda_fail(c, e, "x_kick");
  return WDM_OK;
}

// P2..P4 on x-spectral data (psi, or `data` when given): y fwd, z fwd * drift
// phase * inverse, y inverse.  sign = -1 applies the conjugate phase (the
// drift adjoint).
static wdm_status drift_yz(wdm_ctx* c, double dt, float sign = 1.f, float2* data = nullptr) {
  const int B = c->d.batch;
  float2* psi = data ? data : c->psi;
  DriftOp op{};
  op.sign = sign;
  const bool precise = c->d.phase_mode == WDM_PHASE_PRECISE;
  if (precise) WDM_TRY(ensure_drift_tables(c, dt));
  op.cxy = c->cxy;
  op.cz = c->cz;
  op.nxy = c->d.nx;
  op.rot = c->drift_rot;
  op.kx2 = c->kx2;
  op.ky2 = c->ky2;
  op.kz2 = c->kz2;
  op.half_dt = (float)(0.5 * dt);
  op.scale = (float)(1.0 / ((double)c->d.nx * c->d.ny * c->d.nz));
  op.precise = precise;
  cudaError_t e;
  if ((e = run_pass(c, P_PSI_Y_FWD,
                    [&] { return c->ky->lfft(psi, lines_y(c, c->d.nx, c->d.nx, c->ncell), c->twy, false, B, c->st); })) !=
      cudaSuccess)
    return cuda_fail(c, e, "psi y fwd");
  if ((e = run_pass(c, P_PSI_Z_DRIFT,
                    [&] { return c->kz->lfft_drift(psi, lines_z(c, c->d.nx, c->d.nx, c->ncell), c->twz, op, B, c->st); })) !=
      cudaSuccess)
    return cuda_fail(c, e, "psi z drift");
  if ((e = run_pass(c, P_PSI_Y_INV,
                    [&] { return c->ky->lfft(psi, lines_y(c, c->d.nx, c->d.nx, c->ncell), c->twy, true, B, c->st); })) !=
      cudaSuccess)
    return cuda_fail(c, e, "psi y inv");
  return WDM_OK;
}

static wdm_status sync_and_check(wdm_ctx* c) {
  WDM_CU(c, cudaStreamSynchronize(c->st));
  int flag[2] = {0, 0};
  WDM_CU(c, cudaMemcpy(flag, c->flag, 2 * sizeof(int), cudaMemcpyDeviceToHost));
  if (flag[1])
    return fail(c, WDM_ERR_CUDA,
                "a line pass abandoned a bounded wait for its TMA tile (device error bits " +
                    std::to_string(flag[1]) + "); psi is stale until wdm_set_psi");
  if (fault_injected("nonfinite")) flag[0] = 1;
  if (flag[0]) return fail(c, WDM_ERR_NONFINITE, "psi became non-finite (NaN/Inf density)");
  return WDM_OK;
}

static wdm_status need_psi(wdm_ctx* c) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  if (!c->have_psi) return fail(c, WDM_ERR_STATE, "psi has not been set (call wdm_set_psi first)");
  return WDM_OK;
}

static wdm_status copy_in(wdm_ctx* c, void* dst, const void* src, size_t bytes, int where) {
  if (!src) return fail(c, WDM_ERR_INVALID, "null input pointer");
  if (where != WDM_HOST && where != WDM_DEVICE) return fail(c, WDM_ERR_INVALID, "where must be WDM_HOST or WDM_DEVICE");
  WDM_CU(c, cudaMemcpyAsync(dst, src, bytes, where == WDM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                            c->st));
  return WDM_OK;
}

static wdm_status copy_out(wdm_ctx* c, void* dst, const void* src, size_t bytes, int where) {
  if (!dst) return fail(c, WDM_ERR_INVALID, "null output pointer");
  if (where != WDM_HOST && where != WDM_DEVICE) return fail(c, WDM_ERR_INVALID, "where must be WDM_HOST or WDM_DEVICE");
  WDM_CU(c, cudaMemcpyAsync(dst, src, bytes, where == WDM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                            c->st));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  return WDM_OK;
}

static wdm_status ensure_scratch(wdm_ctx* c) {
  if (!c->scratch_f) WDM_TRY(dalloc(c, &c->scratch_f, (size_t)c->ncell * c->d.batch));
  if (!c->scratch_h) WDM_TRY(dalloc(c, &c->scratch_h, (size_t)c->nhalf * c->d.batch));
  return WDM_OK;
}

// shift[b] = <|psi_b|^2> + mean baryon density: the constant removed from rho
// before its transform (exact for any value: only k = 0 changes).
static wdm_status update_shift(wdm_ctx* c) {
  cudaError_t e = launch_mean_shift(c->psi, true, c->ncell, c->d.batch, c->sums, c->shift, c->rho_b_mean, c->st);
  if (e != cudaSuccess) return cuda_fail(c, e, "mean shift");
  return WDM_OK;
}

// --------------------------------------------------------------------------
// C ABI
// --------------------------------------------------------------------------
extern "C" {

int32_t wdm_version(void) { return 1; }

int32_t wdm_size_supported(int32_t n) { return kernels_for(n) != nullptr ? 1 : 0; }

const char* wdm_last_error(const wdm_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

void* wdm_stream(wdm_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }

wdm_status wdm_destroy(wdm_ctx* c) {
  if (!c) return WDM_OK;
  if (c->self_group) wdm_group_destroy(c->self_group);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->st_rec) cudaStreamSynchronize(c->st_rec);
  void* bufs[] = {c->psi, c->H,  c->twx, c->twy, c->twz, c->kx2, c->ky2,       c->kz2,       c->cxy,
                  c->cz,  c->mx, c->my,  c->mz,  c->V,   c->rho_b, c->rb_rows, c->parts, c->T6b, c->flag, c->scratch_f,
                  c->scratch_h, c->red, c->sums, c->shift, c->shift_in};
  for (void* p : bufs)
    if (p) cudaFree(p);
  void* adj[] = {c->lam, c->Hmu, c->rho_t, c->D6, c->adj_acc, c->diag_wsum, c->diag_wmin, c->centre, c->frame};
  for (void* p : adj)
    if (p) cudaFree(p);
  for (auto* v : {&c->ck_psi, &c->ck_H, &c->slot_psi, &c->slot_H, &c->slot2_psi, &c->slot2_H})
    for (float2* p : *v)
      if (p) cudaFree(p);
  if (c->st_rec) cudaStreamDestroy(c->st_rec);
  for (cudaEvent_t e : {c->ev_ck, c->ev_rec[0], c->ev_rec[1], c->ev_bwd[0], c->ev_bwd[1]})
    if (e) cudaEventDestroy(e);
  for (auto& r : c->prof.pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : c->prof.pool) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return WDM_OK;
}

// --------------------------------------------------------------------------
// Line-pass autotuner
// --------------------------------------------------------------------------
// Each line pass (psi and H, along y and z) has two implementations, the
// TMA-fed persistent pass and the register-tile pass, and the kick and
// density x passes two, rows staged by bulk copies or loaded directly.  Which
// is faster depends on the axis length, the width of the rows (the odd
// nx/2 + 1 of H leaves a mostly empty last 16-line tile), the batch and the
// occupancy the staging slots leave, so a new context times both of every
// pass on its own buffers (zeroed; the fused z passes with the Poisson
// operator, the kick with a small time step) and keeps the faster, preferring
// implementation 0 within 3%.  Choices are kept per (device, nx, ny, nz,
// batch); WDM_LINE_IMPL=tma|tile and WDM_X_IMPL=staged|direct force them.
using TuneKey = std::tuple<int, int, int, int, int>;
struct TuneVal {
  int impl[LP_COUNT];
  double ms[LP_COUNT][2];
};
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneVal> g_tune_cache;

// Implementations forced through the environment (after tuning; not cached).
static void forced_impls(wdm_ctx* c) {
  if (const char* env = std::getenv("WDM_LINE_IMPL")) {
    if (!std::strcmp(env, "tma") || !std::strcmp(env, "tile"))
      for (int k = LP_PSI_Y; k <= LP_H_Z; ++k) c->line_impl[k] = std::strcmp(env, "tma") ? LINE_IMPL_TILE : LINE_IMPL_TMA;
  }
  if (const char* env = std::getenv("WDM_X_IMPL")) {
    if (!std::strcmp(env, "staged") || !std::strcmp(env, "direct"))
      for (int k = LP_X_KICK; k <= LP_X_RHO_B; ++k)
        c->line_impl[k] = std::strcmp(env, "staged") ? X_IMPL_DIRECT : X_IMPL_STAGED;
  }
}

static wdm_status tune_passes_timed(wdm_ctx* c);

// WDM_SCHEDULE="a,b,c,d,e,f,g": the whole schedule (psi-y, psi-z, H-y, H-z as
// tma|tile; kick, density, density with baryons as staged|direct), no timing
// (e.g. under a profiler).
static bool schedule_from_env(wdm_ctx* c) {
  const char* env = std::getenv("WDM_SCHEDULE");
  if (!env) return false;
  static const char* const names[2][2] = {{"tma", "tile"}, {"staged", "direct"}};
  int impl[LP_COUNT];
  std::string s(env);
  size_t pos = 0;
  for (int k = 0; k < LP_COUNT; ++k) {
    const size_t end = s.find(',', pos);
    const std::string tok = s.substr(pos, end == std::string::npos ? std::string::npos : end - pos);
    const int kind = k < LP_X_KICK ? 0 : 1;
    if (tok == names[kind][0]) impl[k] = 0;
    else if (tok == names[kind][1]) impl[k] = 1;
    else return false;
    if (end == std::string::npos && k + 1 < LP_COUNT) return false;
    pos = end + 1;
  }
  std::memcpy(c->line_impl, impl, sizeof(impl));
  return true;
}

static wdm_status tune_passes(wdm_ctx* c) {
  if (schedule_from_env(c)) return WDM_OK;
  WDM_TRY(tune_passes_timed(c));
  forced_impls(c);
  return WDM_OK;
}

static wdm_status tune_passes_timed(wdm_ctx* c) {
  int dev = 0;
  WDM_CU(c, cudaGetDevice(&dev));
  const TuneKey key{dev, c->d.nx, c->d.ny, c->d.nz, c->d.batch};
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto hit = g_tune_cache.find(key);
  if (hit != g_tune_cache.end()) {
    std::memcpy(c->line_impl, hit->second.impl, sizeof(c->line_impl));
    std::memcpy(c->line_ms, hit->second.ms, sizeof(c->line_ms));
    return WDM_OK;
  }
  const int B = c->d.batch;
  WDM_CU(c, cudaMemsetAsync(c->psi, 0, sizeof(float2) * c->ncell * B, c->st));
  WDM_CU(c, cudaMemsetAsync(c->H, 0, sizeof(float2) * c->nhalf * B, c->st));
  PoissonOp po;
  po.kx2 = c->kx2;
  po.ky2 = c->ky2;
  po.kz2 = c->kz2;
  po.coef = 1.f;
  const KickArgs ka = kick_args(c, 1e-3, 0);
  RhoArgs ra{};
  ra.write_psi = 1;
  ra.nonfinite = c->flag;
  ra.shift = c->shift;
  ra.err = c->flag + 1;
  auto run = [&](int k) -> cudaError_t {
    switch (k) {
      case LP_PSI_Y: return c->ky->lfft(c->psi, lines_y(c, c->d.nx, c->d.nx, c->ncell), c->twy, false, B, c->st);
      case LP_PSI_Z: return c->kz->lfft_poisson(c->psi, lines_z(c, c->d.nx, c->d.nx, c->ncell), c->twz, po, B, c->st);
      case LP_H_Y: return c->ky->lfft(c->H, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, false, B, c->st);
      case LP_H_Z: return c->kz->lfft_poisson(c->H, lines_z(c, c->nxh, c->hpitch, c->nhalf), c->twz, po, B, c->st);
      case LP_X_KICK:
        return c->kx->x_kick(c->psi, c->psi, c->H, rows_psi(c, LP_X_KICK), c->hpitch, c->nhalf, c->twx, ka, true, B,
                             c->st);
      case LP_X_RHO: return c->kx->x_inv_rho(c->psi, c->H, rows_psi(c, LP_X_RHO), c->hpitch, c->nhalf, c->twx, ra, B, c->st);
      default: {
        // a stand-in baryon density: the zeroed psi buffer, read as floats
        RhoArgs rb = ra;
        rb.rho_b = reinterpret_cast<const float*>(c->psi);
        return c->kx->x_inv_rho(c->psi, c->H, rows_psi(c, LP_X_RHO_B), c->hpitch, c->nhalf, c->twx, rb, B, c->st);
      }
    }
  };
  cudaEvent_t e0, e1;
  WDM_CU(c, cudaEventCreate(&e0));
  WDM_CU(c, cudaEventCreate(&e1));
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < LP_COUNT && e == cudaSuccess; ++k) {
    for (int impl = 0; impl <= 1 && e == cudaSuccess; ++impl) {
      c->line_impl[k] = impl;
      double best = 1e30;
      for (int r = 0; r < 4 && e == cudaSuccess; ++r) {  // the first run is a warm-up
        if ((e = cudaEventRecord(e0, c->st)) != cudaSuccess || (e = run(k)) != cudaSuccess ||
            (e = cudaEventRecord(e1, c->st)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess)
          break;
        float ms = 0.f;
        if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
        if (r > 0 && ms < best) best = ms;
      }
      c->line_ms[k][impl] = best;
    }
    c->line_impl[k] = c->line_ms[k][1] < 0.97 * c->line_ms[k][0] ? 1 : 0;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(c, e, "line-pass autotuner");
  TuneVal v;
  std::memcpy(v.impl, c->line_impl, sizeof(v.impl));
  std::memcpy(v.ms, c->line_ms, sizeof(v.ms));
  g_tune_cache[key] = v;
  return WDM_OK;
}

wdm_status wdm_get_line_schedule(const wdm_ctx* c, int32_t* impl, double* ms) {
  if (!c || !impl || !ms) return fail(nullptr, WDM_ERR_INVALID, "wdm_get_line_schedule: null argument");
  for (int k = 0; k < LP_COUNT; ++k) {
    impl[k] = c->line_impl[k];
    ms[2 * k] = c->line_ms[k][0];
    ms[2 * k + 1] = c->line_ms[k][1];
  }
  return WDM_OK;
}

wdm_status wdm_create(const wdm_desc* d, wdm_ctx** out) {
  if (!d || !out) return fail(nullptr, WDM_ERR_INVALID, "wdm_create: null argument");
  *out = nullptr;
  const int n[3] = {d->nx, d->ny, d->nz};
  for (int a = 0; a < 3; ++a)
    if (!kernels_for(n[a]))
      return fail(nullptr, WDM_ERR_UNSUPPORTED,
                  "wdm_create: axis length " + std::to_string(n[a]) +
                      " has no FFT plan (supported: 8 12 16 24 32 48 64 96 128 192 256 384 512)");
  if (!(d->lx > 0 && d->ly > 0 && d->lz > 0)) return fail(nullptr, WDM_ERR_INVALID, "wdm_create: box lengths must be > 0");
  if (d->batch < 1) return fail(nullptr, WDM_ERR_INVALID, "wdm_create: batch must be >= 1");
  if (d->convention != WDM_GRID_PERIODIC && d->convention != WDM_GRID_REFERENCE)
    return fail(nullptr, WDM_ERR_INVALID, "wdm_create: unknown grid convention");
  if (d->phase_mode != WDM_PHASE_PLAIN && d->phase_mode != WDM_PHASE_PRECISE)
    return fail(nullptr, WDM_ERR_INVALID, "wdm_create: unknown phase mode");
  const long long ncell = (long long)d->nx * d->ny * d->nz;
  if (ncell * d->batch > (1LL << 31) - 1) return fail(nullptr, WDM_ERR_UNSUPPORTED, "wdm_create: batch*cells exceeds 2^31");
  wdm_ctx* c = new wdm_ctx();
  c->d = *d;
  c->nxh = d->nx / 2 + 1;
  c->ncell = ncell;
  c->hpitch = c->nxh + (c->nxh & 1);
#ifdef WDM_HPITCH_ALIGN
  // tuning variant: rows of H start on WDM_HPITCH_ALIGN-element boundaries
  c->hpitch = (c->nxh + WDM_HPITCH_ALIGN - 1) / WDM_HPITCH_ALIGN * WDM_HPITCH_ALIGN;
#endif
  c->nhalf = (long long)c->hpitch * d->ny * d->nz;
  c->kx = kernels_for(d->nx);
  c->ky = kernels_for(d->ny);
  c->kz = kernels_for(d->nz);
  axis_geom(d->nx, d->lx, d->convention, &c->dx, &c->x0);
  axis_geom(d->ny, d->ly, d->convention, &c->dy, &c->y0);
  axis_geom(d->nz, d->lz, d->convention, &c->dz, &c->z0);
  wdm_status s = WDM_OK;
  auto bail = [&](wdm_status st) {
    g_create_error = c->err;
    wdm_destroy(c);
    return st;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cuda_fail(c, e, "cudaStreamCreate");
    return bail(WDM_ERR_CUDA);
  }
  const size_t B = (size_t)d->batch;
  if ((s = dalloc(c, &c->psi, B * ncell)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->H, B * c->nhalf)) != WDM_OK) return bail(s);
  if ((s = upload_twiddles(c, &c->twx, c->kx)) != WDM_OK) return bail(s);
  if ((s = upload_twiddles(c, &c->twy, c->ky)) != WDM_OK) return bail(s);
  if ((s = upload_twiddles(c, &c->twz, c->kz)) != WDM_OK) return bail(s);
  if ((s = upload_k2(c, &c->kx2, d->nx, d->lx)) != WDM_OK) return bail(s);
  if ((s = upload_k2(c, &c->ky2, d->ny, d->ly)) != WDM_OK) return bail(s);
  if ((s = upload_k2(c, &c->kz2, d->nz, d->lz)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->cxy, (size_t)d->nx * d->ny)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->cz, d->nz)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->mx, d->nx)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->my, d->ny)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->mz, d->nz)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->flag, 2)) != WDM_OK) return bail(s);
  if ((e = cudaMemsetAsync(c->flag, 0, 2 * sizeof(int), c->st)) != cudaSuccess) {
    cuda_fail(c, e, "memset flag");
    return bail(WDM_ERR_CUDA);
  }
  c->red_blocks = 4 * 152;
  if ((s = dalloc(c, &c->red, B * c->red_blocks * RED_FIELDS)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->sums, B)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->shift, B)) != WDM_OK) return bail(s);
  if ((s = dalloc(c, &c->shift_in, B)) != WDM_OK) return bail(s);
  if ((e = cudaMemsetAsync(c->shift, 0, sizeof(float) * B, c->st)) != cudaSuccess) {
    cuda_fail(c, e, "memset shift");
    return bail(WDM_ERR_CUDA);
  }
  if ((s = tune_passes(c)) != WDM_OK) return bail(s);
  if ((e = cudaStreamSynchronize(c->st)) != cudaSuccess) {
    cuda_fail(c, e, "sync");
    return bail(WDM_ERR_CUDA);
  }
  *out = c;
  return WDM_OK;
}

wdm_status wdm_set_psi(wdm_ctx* c, const void* psi, int32_t where) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  WDM_TRY(copy_in(c, c->psi, psi, sizeof(float2) * c->ncell * c->d.batch, where));
  WDM_CU(c, cudaMemsetAsync(c->flag, 0, 2 * sizeof(int), c->st));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  WDM_TRY(update_shift(c));
  c->have_psi = 1;
  c->phi_valid = 0;
  return WDM_OK;
}

wdm_status wdm_get_psi(wdm_ctx* c, void* psi, int32_t where) {
  WDM_TRY(need_psi(c));
  return copy_out(c, psi, c->psi, sizeof(float2) * c->ncell * c->d.batch, where);
}

wdm_status wdm_get_rho(wdm_ctx* c, float* rho, int32_t where) {
  WDM_TRY(need_psi(c));
  WDM_TRY(ensure_scratch(c));
  cudaError_t e = launch_abs2(c->psi, c->scratch_f, c->ncell * c->d.batch, c->st);
  if (e != cudaSuccess) return cuda_fail(c, e, "abs2");
  return copy_out(c, rho, c->scratch_f, sizeof(float) * c->ncell * c->d.batch, where);
}

static wdm_status phi_real(wdm_ctx* c) {
  WDM_TRY(ensure_scratch(c));
  if (!c->phi_valid) WDM_TRY(density_poisson(c, 0, 0.0));
  cudaError_t e = run_pass(c, P_PHI_OUT, [&] {
    return c->kx->x_c2r(c->H, c->scratch_f, rows_psi(c), c->hpitch, c->nhalf, c->twx, c->d.batch, c->st);
  });
  if (e != cudaSuccess) return cuda_fail(c, e, "x_c2r");
  return WDM_OK;
}

wdm_status wdm_get_phi(wdm_ctx* c, float* phi, int32_t where) {
  WDM_TRY(need_psi(c));
  WDM_TRY(phi_real(c));
  return copy_out(c, phi, c->scratch_f, sizeof(float) * c->ncell * c->d.batch, where);
}

wdm_status wdm_set_static_potential(wdm_ctx* c, const float* V, int32_t where) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  c->version++;
  if (!V) {
    if (c->V) cudaFree(c->V);
    c->V = nullptr;
    return WDM_OK;
  }
  if (!c->V) WDM_TRY(dalloc(c, &c->V, (size_t)c->ncell * c->d.batch));
  WDM_TRY(copy_in(c, c->V, V, sizeof(float) * c->ncell * c->d.batch, where));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  return WDM_OK;
}

wdm_status wdm_set_tidal(wdm_ctx* c, const double* sched, int32_t nsched, int32_t per_item) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  c->version++;
  if (nsched < 0) return fail(c, WDM_ERR_INVALID, "nsched < 0");
  c->tide_t0 = 0.0;
  c->tide_dt = 0.0;
  if (nsched == 0) {
    c->tide_on = 0;
    c->tide.clear();
    return WDM_OK;
  }
  if (!sched) return fail(c, WDM_ERR_INVALID, "null tidal schedule");
  if (per_item) {
    if (nsched != c->d.batch) return fail(c, WDM_ERR_INVALID, "per-item tidal tensors need nsched == batch");
    if (!c->T6b) WDM_TRY(dalloc(c, &c->T6b, (size_t)6 * c->d.batch));
    std::vector<float> h((size_t)6 * nsched);
    for (size_t i = 0; i < h.size(); ++i) h[i] = (float)sched[i];
    WDM_CU(c, cudaMemcpyAsync(c->T6b, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->st));
    WDM_CU(c, cudaStreamSynchronize(c->st));
    c->tide_on = 2;
  } else {
    c->tide.assign(sched, sched + (size_t)6 * nsched);
    c->tide_on = 1;
  }
  return WDM_OK;
}

wdm_status wdm_set_tidal_clock(wdm_ctx* c, double t_first, double t_step) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  if (!std::isfinite(t_first) || !std::isfinite(t_step) || t_step < 0.0)
    return fail(c, WDM_ERR_INVALID, "wdm_set_tidal_clock: t_first must be finite and t_step finite and >= 0");
  if (c->tide_on != 1 && t_step > 0.0)
    return fail(c, WDM_ERR_STATE, "wdm_set_tidal_clock: set a schedule of shared rows with wdm_set_tidal first");
  c->version++;
  c->tide_t0 = t_first;
  c->tide_dt = t_step;
  return WDM_OK;
}

wdm_status wdm_set_tidal_centering(wdm_ctx* c, int32_t mode) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  if (mode != WDM_TIDE_BOX_CENTRE && mode != WDM_TIDE_REFERENCE && mode != WDM_TIDE_DENSITY_MAX)
    return fail(c, WDM_ERR_INVALID, "wdm_set_tidal_centering: unknown mode");
  if (mode != WDM_TIDE_BOX_CENTRE && !c->centre) {
    WDM_TRY(dalloc(c, &c->frame, (size_t)4 * c->d.batch));
    WDM_TRY(dalloc(c, &c->centre, (size_t)CENTRE_WORDS * c->d.batch));
    WDM_CU(c, cudaMemsetAsync(c->centre, 0, sizeof(unsigned long long) * CENTRE_WORDS * c->d.batch, c->st));
    WDM_CU(c, cudaStreamSynchronize(c->st));
  }
  c->version++;
  c->tide_centre = mode;
  c->phi_valid = 0;  // the next kick needs a density pass that fills the words
  return WDM_OK;
}

wdm_status wdm_set_particles(wdm_ctx* c, const double* pos, const double* mass, int64_t n) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  c->version++;
  if (n < 0) return fail(c, WDM_ERR_INVALID, "n < 0");
  if (n > 0 && c->d.batch != 1) return fail(c, WDM_ERR_UNSUPPORTED, "baryon particles need batch == 1");
  if (c->parts) cudaFree(c->parts);
  c->parts = nullptr;
  c->nparts = 0;
  if (c->rb_ready) {  // clear the deposit of the old particles
    WDM_CU(c, cudaMemsetAsync(c->rho_b, 0, sizeof(float) * c->ncell, c->st));
    WDM_CU(c, cudaMemsetAsync(c->rb_rows, 0, sizeof(int) * c->d.ny * c->d.nz, c->st));
    c->rb_ready = 0;
  }
  if (n == 0) {  // no baryons from now on: the potential and the density shift lose them too
    c->rho_b_mean = 0.0;
    if (c->have_psi) WDM_TRY(update_shift(c));
    c->phi_valid = 0;
    return WDM_OK;
  }
  if (!pos || !mass) return fail(c, WDM_ERR_INVALID, "null particle arrays");
  if (!c->rho_b) {
    WDM_TRY(dalloc(c, &c->rho_b, (size_t)c->ncell));
    WDM_CU(c, cudaMemsetAsync(c->rho_b, 0, sizeof(float) * c->ncell, c->st));
  }
  if (!c->rb_rows) {
    WDM_TRY(dalloc(c, &c->rb_rows, (size_t)c->d.ny * c->d.nz));
    WDM_CU(c, cudaMemsetAsync(c->rb_rows, 0, sizeof(int) * c->d.ny * c->d.nz, c->st));
  }
  // cell index and fractions in FP64 on the host (particles are static)
  std::vector<CicParticle> h((size_t)n);
  const double d[3] = {c->dx, c->dy, c->dz};
  const double o[3] = {c->x0, c->y0, c->z0};
  const int nn[3] = {c->d.nx, c->d.ny, c->d.nz};
  const double dV = c->dx * c->dy * c->dz;
  for (int64_t p = 0; p < n; ++p) {
    for (int a = 0; a < 3; ++a) {
      const double u = (pos[3 * p + a] - o[a]) / d[a];
      const double fl = std::floor(u);
      long long i0 = (long long)fl % nn[a];
      if (i0 < 0) i0 += nn[a];
      h[p].i[a] = (int)i0;
      h[p].f[a] = (float)(u - fl);
    }
    h[p].m = (float)(mass[p] / dV);
  }
  WDM_TRY(dalloc(c, &c->parts, (size_t)n));
  WDM_CU(c, cudaMemcpyAsync(c->parts, h.data(), sizeof(CicParticle) * n, cudaMemcpyHostToDevice, c->st));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  c->nparts = n;
  double msum = 0.0;
  for (int64_t p = 0; p < n; ++p) msum += mass[p];
  c->rho_b_mean = msum / ((double)c->ncell * dV);
  if (c->have_psi) WDM_TRY(update_shift(c));
  c->phi_valid = 0;
  return WDM_OK;
}

static wdm_status step_impl(wdm_ctx* c, int32_t nsteps, double dt, double t0, int32_t mode) {
  WDM_TRY(need_psi(c));
  if (nsteps < 0) return fail(c, WDM_ERR_INVALID, "nsteps < 0");
  if (!(std::isfinite(dt))) return fail(c, WDM_ERR_INVALID, "dt is not finite");
  if (mode != WDM_STEP_STRANG && mode != WDM_STEP_REFERENCE_LOOP && mode != WDM_STEP_LIE)
    return fail(c, WDM_ERR_INVALID, "unknown step mode");
  if (!std::isfinite(t0)) return fail(c, WDM_ERR_INVALID, "t0 is not finite");
  // kick s runs at time t0 + s dt (the Strang step's closing half kick is kick nsteps)
  if (nsteps == 0) return WDM_OK;
  WDM_TRY(check_tide_rows(c, t0, dt, nsteps + 1, "wdm_step"));
  if (!c->phi_valid) WDM_TRY(density_poisson(c, 0, dt));
  for (int s = 0; s < nsteps; ++s) {
    double kdt;
    if (mode == WDM_STEP_STRANG) kdt = (s == 0) ? 0.5 * dt : dt;  // interior half kicks merged
    else if (mode == WDM_STEP_REFERENCE_LOOP) kdt = 0.5 * dt;
    else kdt = dt;
    WDM_TRY(kick(c, kdt, tide_row(c, t0 + s * dt, s), true));
    WDM_TRY(drift_yz(c, dt));
    WDM_TRY(density_poisson(c, 1, dt));
  }
  if (mode == WDM_STEP_STRANG) WDM_TRY(kick(c, 0.5 * dt, tide_row(c, t0 + nsteps * dt, nsteps), false));
  return WDM_OK;
}

wdm_status wdm_step_async(wdm_ctx* c, int32_t nsteps, double dt, double t0, int32_t mode) {
  return step_impl(c, nsteps, dt, t0, mode);
}

wdm_status wdm_step(wdm_ctx* c, int32_t nsteps, double dt, double t0, int32_t mode) {
  WDM_TRY(step_impl(c, nsteps, dt, t0, mode));
  return sync_and_check(c);
}

wdm_status wdm_kick(wdm_ctx* c, double dt, double t) {
  WDM_TRY(need_psi(c));
  if (!std::isfinite(dt) || !std::isfinite(t)) return fail(c, WDM_ERR_INVALID, "wdm_kick: dt and t must be finite");
  if (c->tide_on == 1 && c->tide.size() > 6 && !(c->tide_dt > 0.0))
    return fail(c, WDM_ERR_STATE,
                "wdm_kick: the tidal schedule has several rows but no clock (wdm_set_tidal_clock), so time t "
                "selects no row");
  WDM_TRY(check_tide_rows(c, t, 0.0, 1, "wdm_kick"));
  if (!c->phi_valid) WDM_TRY(density_poisson(c, 0, 0.0));
  WDM_TRY(kick(c, dt, tide_row(c, t, 0), false));
  return sync_and_check(c);
}

wdm_status wdm_drift(wdm_ctx* c, double dt) {
  WDM_TRY(need_psi(c));
  cudaError_t e = run_pass(c, P_X_FFT, [&] { return c->kx->xfft(c->psi, rows_psi(c), c->twx, false, 1.0f, c->d.batch, c->st); });
  if (e != cudaSuccess) return cuda_fail(c, e, "x fwd");
  WDM_TRY(drift_yz(c, dt));
  WDM_TRY(density_poisson(c, 1, dt));
  return sync_and_check(c);
}

wdm_status wdm_poisson(wdm_ctx* c, const float* rho, float* phi, int32_t where) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  WDM_TRY(ensure_scratch(c));
  const int B = c->d.batch;
  const size_t bytes = sizeof(float) * c->ncell * B;
  const float* in = rho;
  if (where == WDM_HOST) {
    WDM_TRY(copy_in(c, c->scratch_f, rho, bytes, WDM_HOST));
    in = c->scratch_f;
  } else if (where != WDM_DEVICE) {
    return fail(c, WDM_ERR_INVALID, "where must be WDM_HOST or WDM_DEVICE");
  }
  if (!in || !phi) return fail(c, WDM_ERR_INVALID, "null rho/phi");
  cudaError_t e;
  if ((e = launch_mean_shift(in, false, c->ncell, B, c->sums, c->shift_in, 0.0, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "mean");
  if ((e = c->kx->x_r2c(in, c->scratch_h, rows_psi(c), c->hpitch, c->nhalf, c->twx, c->shift_in, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "x r2c");
  if ((e = c->ky->lfft(c->scratch_h, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, false, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "y fwd");
  PoissonOp po;
  po.kx2 = c->kx2;
  po.ky2 = c->ky2;
  po.kz2 = c->kz2;
  po.coef = (float)(-c->d.poisson_coeff / ((double)c->d.nx * c->d.ny * c->d.nz));
  if ((e = c->kz->lfft_poisson(c->scratch_h, lines_z(c, c->nxh, c->hpitch, c->nhalf), c->twz, po, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "z poisson");
  if ((e = c->ky->lfft(c->scratch_h, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, true, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "y inv");
  float* dst = where == WDM_HOST ? c->scratch_f : phi;
  if ((e = c->kx->x_c2r(c->scratch_h, dst, rows_psi(c), c->hpitch, c->nhalf, c->twx, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "x c2r");
  if (where == WDM_HOST) return copy_out(c, phi, c->scratch_f, bytes, WDM_HOST);
  WDM_CU(c, cudaStreamSynchronize(c->st));
  return WDM_OK;
}

wdm_status wdm_fft3d(wdm_ctx* c, void* data, int32_t dir) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  if (!data) return fail(c, WDM_ERR_INVALID, "null data");
  if (dir != -1 && dir != 1) return fail(c, WDM_ERR_INVALID, "dir must be -1 or +1");
  const bool inv = dir == 1;
  const int B = c->d.batch;
  float2* p = (float2*)data;
  cudaError_t e;
  if ((e = c->kx->xfft(p, rows_psi(c), c->twx, inv, 1.0f, B, c->st)) != cudaSuccess) return cuda_fail(c, e, "x");
  if ((e = c->ky->lfft(p, lines_y(c, c->d.nx, c->d.nx, c->ncell), c->twy, inv, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "y");
  if ((e = c->kz->lfft(p, lines_z(c, c->d.nx, c->d.nx, c->ncell), c->twz, inv, B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "z");
  WDM_CU(c, cudaStreamSynchronize(c->st));
  return WDM_OK;
}

// The per-item FP64 reduction of psi and Phi (k_reduce), block partials
// combined on the host: r[b] holds the RED_* fields of batch item b.
static wdm_status reduce_items(wdm_ctx* c, std::vector<std::array<double, RED_FIELDS>>& r) {
  WDM_TRY(phi_real(c));
  RedGeom g;
  g.nx = c->d.nx;
  g.ny = c->d.ny;
  g.nz = c->d.nz;
  g.dx = c->dx;
  g.dy = c->dy;
  g.dz = c->dz;
  g.x0 = c->x0;
  g.y0 = c->y0;
  g.z0 = c->z0;
  g.zmid = c->d.nz / 2 - 1 > 0 ? c->d.nz / 2 - 1 : 0;  // the slice div(end, 2) of a 1-based z axis
  cudaError_t e = launch_reduce(c->psi, c->scratch_f, g, c->red, c->red_blocks, c->d.batch, c->st);
  if (e != cudaSuccess) return cuda_fail(c, e, "reduce");
  std::vector<double> h((size_t)c->red_blocks * RED_FIELDS * c->d.batch);
  WDM_CU(c, cudaMemcpyAsync(h.data(), c->red, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  r.assign((size_t)c->d.batch, {});
  for (int b = 0; b < c->d.batch; ++b) {
    std::array<double, RED_FIELDS>& acc = r[(size_t)b];
    acc.fill(0.0);
    acc[RED_MAX] = -1.0;
    for (int k = 0; k < c->red_blocks; ++k) {
      const double* p = &h[((size_t)b * c->red_blocks + k) * RED_FIELDS];
      for (int q = 0; q < RED_FIELDS; ++q)
        if (!red_is_max(q)) acc[q] += p[q];
      acc[RED_PHIMAX] = std::max(acc[RED_PHIMAX], p[RED_PHIMAX]);
      if (p[RED_MAX] > acc[RED_MAX] || (p[RED_MAX] == acc[RED_MAX] && p[RED_ARG] < acc[RED_ARG])) {
        acc[RED_MAX] = p[RED_MAX];
        acc[RED_ARG] = p[RED_ARG];
      }
    }
  }
  return WDM_OK;
}

// The ten fields of wdm_reduce from one item's RED_* sums.
static void reduce_fields(const wdm_ctx* c, const std::array<double, RED_FIELDS>& acc, double* o) {
  const double dV = c->dx * c->dy * c->dz;
  const double m = acc[RED_MASS];
  o[0] = m * dV;
  o[1] = acc[RED_MAX];
  o[2] = acc[RED_ARG];
  o[3] = m > 0 ? acc[RED_MX] / m : 0.0;
  o[4] = m > 0 ? acc[RED_MY] / m : 0.0;
  o[5] = m > 0 ? acc[RED_MZ] / m : 0.0;
  const double W = -0.5 * acc[RED_W] * dV;
  const double K = 0.5 * acc[RED_K] * dV;
  const double Q = 0.5 * acc[RED_Q] * dV;
  o[6] = W;
  o[7] = K;
  o[8] = Q;
  o[9] = 2 * K + 2 * Q - W;
}

wdm_status wdm_reduce(wdm_ctx* c, double* out) {
  WDM_TRY(need_psi(c));
  if (!out) return fail(c, WDM_ERR_INVALID, "null output");
  std::vector<std::array<double, RED_FIELDS>> r;
  WDM_TRY(reduce_items(c, r));
  for (int b = 0; b < c->d.batch; ++b) reduce_fields(c, r[(size_t)b], out + 10 * b);
  return WDM_OK;
}

// Weighted quantiles over groups of equal values, the groups ascending in
// value.  Restates the weighted quantile of StatsBase 0.34 (`quantile(v,
// w::AbstractWeights, p)` for weights other than FrequencyWeights, as
// src/simulation_main.jl:641 calls it): elements sorted by (value, weight);
// h = p (sum w - w_1) + w_1; the first element k with cumulative weight S_k > h
// gives v_{k-1} + (h - S_{k-1}) / (S_k - S_{k-1}) (v_k - v_{k-1}) (v_0 = 0, S_0 = 0);
// no such element gives the largest value.  Inside a group the first element
// is its smallest weight: a crossing there interpolates from the previous
// group's value, a crossing at any later element returns the group's value.
// Groups of zero total weight are skipped (zero weights take no part).
// Cumulative sums are FP64.
struct GroupCum {
  std::vector<int64_t> idx;  // nonempty groups, ascending
  std::vector<double> S;     // cumulative weight through each
  explicit GroupCum(const double* wsum, int64_t ng) {
    double acc = 0.0;
    for (int64_t g = 0; g < ng; ++g)
      if (wsum[g] > 0.0) {
        idx.push_back(g);
        S.push_back(acc += wsum[g]);
      }
  }
  // position in idx of the first group whose cumulative weight exceeds h (idx.size(): none)
  size_t find(double h) const { return (size_t)(std::upper_bound(S.begin(), S.end(), h) - S.begin()); }
  double h(double p, double w1) const { return p * (S.back() - w1) + w1; }
};

// value(g) and wmin(g): a group's value and smallest element weight; only
// the first group, the groups the quantiles fall in and their predecessors
// are asked for.
extern "C++" {
template <class Value, class Wmin>
static void grouped_quantiles(const GroupCum& gc, Value value, Wmin wmin, const double* p, int np, double* out) {
  if (gc.idx.empty()) {
    for (int i = 0; i < np; ++i) out[i] = NAN;
    return;
  }
  const double w1 = wmin(gc.idx[0]);
  for (int i = 0; i < np; ++i) {
    const double h = gc.h(p[i], w1);
    const size_t k = gc.find(h);
    if (k >= gc.idx.size()) {
      out[i] = value(gc.idx.back());
      continue;
    }
    const double Sprev = k ? gc.S[k - 1] : 0.0, vprev = k ? value(gc.idx[k - 1]) : 0.0;
    const double m = wmin(gc.idx[k]);
    const double v = value(gc.idx[k]);
    out[i] = (h < Sprev + m) ? vprev + (h - Sprev) / m * (v - vprev) : v;
  }
}
}  // extern "C++"

wdm_status wdm_weighted_quantiles_grouped(const double* value, const double* wsum, const double* wmin, int64_t ngroups,
                                          const double* p, int32_t np, double* out) {
  if (ngroups < 0 || np < 0 || (ngroups > 0 && (!value || !wsum || !wmin)) || (np > 0 && (!p || !out)))
    return fail(nullptr, WDM_ERR_INVALID, "wdm_weighted_quantiles_grouped: bad arguments");
  for (int64_t g = 1; g < ngroups; ++g)
    if (!(value[g] > value[g - 1]))
      return fail(nullptr, WDM_ERR_INVALID, "wdm_weighted_quantiles_grouped: values must ascend strictly");
  const GroupCum gc(wsum, ngroups);
  grouped_quantiles(
      gc, [&](int64_t g) { return value[g]; }, [&](int64_t g) { return wmin[g]; }, p, np, out);
  return WDM_OK;
}

wdm_status wdm_diagnostics(wdm_ctx* c, double* out) {
  WDM_TRY(need_psi(c));
  if (!out) return fail(c, WDM_ERR_INVALID, "null output");
  std::vector<std::array<double, RED_FIELDS>> r;
  WDM_TRY(reduce_items(c, r));
  const int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
  // the radii need equal spacings: squared distances are then dx^2 times an integer key
  const double tol = 1e-12 * c->dx;
  const bool cubic = std::fabs(c->dx - c->dy) <= tol && std::fabs(c->dx - c->dz) <= tol;
  const int64_t nkeys = (int64_t)(nx - 1) * (nx - 1) + (int64_t)(ny - 1) * (ny - 1) + (int64_t)(nz - 1) * (nz - 1) + 1;
  std::vector<double> hs;
  if (cubic) {
    // the histogram (nkeys doubles) and the minimum words live with the context
    if (!c->diag_wsum) WDM_TRY(dalloc(c, &c->diag_wsum, (size_t)nkeys));
    if (!c->diag_wmin) WDM_TRY(dalloc(c, &c->diag_wmin, (size_t)RADII_KEYS));
    hs.resize((size_t)nkeys);
  }
  double* wsum = c->diag_wsum;
  unsigned long long* wmin = c->diag_wmin;
  static const double P[9] = {0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9};
  wdm_status s = WDM_OK;
  for (int b = 0; b < c->d.batch && s == WDM_OK; ++b) {
    const auto& acc = r[(size_t)b];
    double* o = out + (size_t)WDM_DIAG_FIELDS * b;
    reduce_fields(c, acc, o);
    const double dV = c->dx * c->dy * c->dz;
    o[10] = acc[RED_PX] * dV;
    o[11] = acc[RED_PY] * dV;
    o[12] = acc[RED_PZ] * dV;
    o[13] = acc[RED_PHIMAX];
    o[14] = std::sqrt(acc[RED_MAX]);
    o[15] = 2.0 * c->dx * c->dx / M_PI;
    o[16] = o[13] > 0 ? 2.0 * M_PI / o[13] : INFINITY;
    o[17] = (c->d.kerr != 0.0 && o[14] > 0) ? 2.0 * M_PI / std::fabs(c->d.kerr) / o[14] : INFINITY;
    const double sw = acc[RED_SW];
    if (sw > 0) {
      const double mean = acc[RED_SWR] / sw;
      o[18] = std::sqrt(std::max(0.0, acc[RED_SWR2] / sw - mean * mean));
    } else {
      o[18] = NAN;
    }
    if (!cubic) {
      for (int i = 0; i < 9; ++i) o[19 + i] = NAN;
      continue;
    }
    const long long arg = (long long)acc[RED_ARG];
    const int cz = (int)(arg / ((long long)nx * ny)), rem = (int)(arg - (long long)cz * nx * ny);
    const int cy = rem / nx, cx = rem - cy * nx;
    // pass 1: the weight of every distance
    cudaError_t e = cudaMemsetAsync(wsum, 0, sizeof(double) * nkeys, c->st);
    const float2* pb = c->psi + (size_t)b * c->ncell;
    if (e == cudaSuccess) e = launch_radii_hist(pb, nx, ny, nz, cx, cy, cz, wsum, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hs.data(), wsum, sizeof(double) * nkeys, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    // pass 2: the smallest element weight of the distance 0 (w_1) and of the
    // groups the quantiles fall in, the only ones the quantile reads
    RadiiKeys keys{};
    keys.k[keys.n++] = 0;
    const GroupCum gc(hs.data(), e == cudaSuccess ? nkeys : 0);
    if (!gc.idx.empty())
      for (int i = 0; i < 9; ++i) {
        const size_t k = gc.find(gc.h(P[i], acc[RED_MAX]));  // w_1 is the maximum's weight
        if (k >= gc.idx.size()) continue;
        const long long key = gc.idx[k];
        if (std::find(keys.k, keys.k + keys.n, key) == keys.k + keys.n && keys.n < RADII_KEYS) keys.k[keys.n++] = key;
      }
    unsigned long long m[RADII_KEYS];
    if (e == cudaSuccess) e = cudaMemsetAsync(wmin, 0xff, sizeof(unsigned long long) * RADII_KEYS, c->st);
    if (e == cudaSuccess) e = launch_radii_min(pb, nx, ny, nz, cx, cy, cz, keys, wmin, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m, wmin, sizeof(m), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
      s = cuda_fail(c, e, "diagnostics histogram");
      break;
    }
    c->launch_count += 2;
    const double dx = c->dx;
    auto value = [dx](int64_t g) { return dx * std::sqrt((double)g); };
    auto wmin_of = [&](int64_t g) {
      for (int j = 0; j < keys.n; ++j)
        if (keys.k[j] == g) {
          double v;
          std::memcpy(&v, &m[j], sizeof(v));
          return v;
        }
      return (double)INFINITY;  // not a group the quantiles fall in
    };
    grouped_quantiles(gc, value, wmin_of, P, 9, o + 19);
  }
  return s;
}

wdm_status wdm_interpolate_phi(wdm_ctx* c, const double* pos, int64_t n, double* out) {
  WDM_TRY(need_psi(c));
  if (n < 0 || (n > 0 && (!pos || !out))) return fail(c, WDM_ERR_INVALID, "bad particle arrays");
  if (n == 0) return WDM_OK;
  if (c->d.batch != 1) return fail(c, WDM_ERR_UNSUPPORTED, "interpolation needs batch == 1");
  WDM_TRY(phi_real(c));
  std::vector<CicParticle> h((size_t)n);
  const double d[3] = {c->dx, c->dy, c->dz};
  const double o[3] = {c->x0, c->y0, c->z0};
  const int nn[3] = {c->d.nx, c->d.ny, c->d.nz};
  for (int64_t p = 0; p < n; ++p) {
    for (int a = 0; a < 3; ++a) {
      const double u = (pos[3 * p + a] - o[a]) / d[a];
      const double fl = std::floor(u);
      long long i0 = (long long)fl % nn[a];
      if (i0 < 0) i0 += nn[a];
      h[p].i[a] = (int)i0;
      h[p].f[a] = (float)(u - fl);
    }
    h[p].m = 1.f;
  }
  CicParticle* dp = nullptr;
  double* dout = nullptr;
  WDM_TRY(dalloc(c, &dp, (size_t)n));
  wdm_status s = dalloc(c, &dout, (size_t)n);
  if (s != WDM_OK) {
    cudaFree(dp);
    return s;
  }
  cudaError_t e = cudaMemcpyAsync(dp, h.data(), sizeof(CicParticle) * n, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = launch_cic_interp(c->scratch_f, dp, n, c->d.nx, c->d.ny, c->d.nz, dout, c->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(dp);
  cudaFree(dout);
  if (e != cudaSuccess) return cuda_fail(c, e, "interpolate");
  return WDM_OK;
}

wdm_status wdm_selftest_sincos(const float* h, float* out, int64_t n) {
  if (!h || !out || n < 0) return fail(nullptr, WDM_ERR_INVALID, "wdm_selftest_sincos: bad arguments");
  cudaError_t e = launch_sincos_half(h, out, n, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail(nullptr, WDM_ERR_CUDA, std::string("wdm_selftest_sincos: ") + cudaGetErrorString(e));
  return WDM_OK;
}

wdm_status wdm_selftest_bounded_wait(int64_t limit_ns, int32_t* bits, int64_t* waited_ns) {
  if (!bits || !waited_ns || limit_ns < 0 || limit_ns > 10000000000LL)
    return fail(nullptr, WDM_ERR_INVALID, "wdm_selftest_bounded_wait: bad arguments (limit 0..1e10 ns)");
  unsigned long long* d = nullptr;
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMalloc((void**)&d, sizeof(h));
  if (e == cudaSuccess) e = launch_bounded_wait_probe((unsigned long long)limit_ns, d, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess)
    return fail(nullptr, WDM_ERR_CUDA, std::string("wdm_selftest_bounded_wait: ") + cudaGetErrorString(e));
  *bits = (int32_t)h[0];
  *waited_ns = (int64_t)h[1];
  return WDM_OK;
}

int32_t wdm_num_passes(void) { return NPASS; }

const char* wdm_pass_name(int32_t p) { return (p >= 0 && p < NPASS) ? PASS_NAMES[p] : ""; }

int64_t wdm_launch_count(const wdm_ctx* c) { return c ? c->launch_count : 0; }

wdm_status wdm_set_profiling(wdm_ctx* c, int32_t on) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  WDM_CU(c, prof_flush(c));
  for (int p = 0; p < NPASS; ++p) {
    c->prof.launches[p] = 0;
    c->prof.ms[p] = 0.0;
  }
  c->prof.on = on != 0;
  return WDM_OK;
}

wdm_status wdm_set_profile_mask(wdm_ctx* c, uint64_t mask) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  c->prof.mask = mask;
  return WDM_OK;
}

wdm_status wdm_get_profile(wdm_ctx* c, int64_t* launches, double* ms, double* bytes) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  WDM_CU(c, prof_flush(c));
  for (int p = 0; p < NPASS; ++p) {
    if (launches) launches[p] = c->prof.launches[p];
    if (ms) ms[p] = c->prof.ms[p];
    if (bytes) bytes[p] = pass_bytes(c, p);
  }
  return WDM_OK;
}

wdm_status wdm_check_finite(wdm_ctx* c, int32_t* finite) {
  WDM_TRY(need_psi(c));
  if (!finite) return fail(c, WDM_ERR_INVALID, "null output");
  WDM_CU(c, cudaStreamSynchronize(c->st));
  int flag = 0;
  WDM_CU(c, cudaMemcpy(&flag, c->flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (fault_injected("nonfinite")) flag = 1;
  *finite = flag ? 0 : 1;
  return WDM_OK;
}

// --------------------------------------------------------------------------
// Adjoint of a Strang run (checkpointed)
// --------------------------------------------------------------------------
// A Strang run of N steps is N+1 kicks at the boundaries b = 0..N (dt/2, dt,
// ..., dt, dt/2; consecutive half kicks see the same density and merge) and N
// drifts.  s_b is the state just before the kick of boundary b; the forward
// pass keeps (s_b, H_b) every ck steps, the reverse sweep recomputes the
// states of one segment at a time and runs the adjoint kick (A1, Poisson of mu,
// A5) and the adjoint drift (conjugate phase) boundary by boundary.
static wdm_status ensure_pairs(wdm_ctx* c, std::vector<float2*>& ps, std::vector<float2*>& hs, size_t n) {
  const size_t B = (size_t)c->d.batch;
  while (ps.size() < n) {
    float2 *p = nullptr, *h = nullptr;
    WDM_TRY(dalloc(c, &p, B * c->ncell));
    ps.push_back(p);
    wdm_status s = dalloc(c, &h, B * c->nhalf);
    if (s != WDM_OK) return s;
    hs.push_back(h);
  }
  return WDM_OK;
}

static wdm_status copy_pair(wdm_ctx* c, float2* dp, float2* dh, const float2* sp, const float2* sh) {
  const size_t B = (size_t)c->d.batch;
  WDM_CU(c, cudaMemcpyAsync(dp, sp, sizeof(float2) * B * c->ncell, cudaMemcpyDeviceToDevice, c->st));
  WDM_CU(c, cudaMemcpyAsync(dh, sh, sizeof(float2) * B * c->nhalf, cudaMemcpyDeviceToDevice, c->st));
  return WDM_OK;
}

// one boundary of the forward run: kick of boundary b, drift, density and Poisson
static wdm_status forward_boundary(wdm_ctx* c, int b, double dt) {
  WDM_TRY(kick(c, b == 0 ? 0.5 * dt : dt, tide_row(c, b * dt, b), true));
  WDM_TRY(drift_yz(c, dt));
  return density_poisson(c, 1, dt);
}

// The same boundary out of place: (psi_in, H_in) = s_b -> (psi_out, H_out) = s_{b+1}.
// Keeps every state of a segment without copies.
static wdm_status forward_boundary_to(wdm_ctx* c, int b, double dt, const float2* psi_in, float2* H_in,
                                      float2* psi_out, float2* H_out) {
  float2* keep_psi = c->psi;
  float2* keep_H = c->H;
  c->psi = psi_out;
  c->H = H_in;
  wdm_status s = kick(c, b == 0 ? 0.5 * dt : dt, tide_row(c, b * dt, b), true, psi_in);
  if (s == WDM_OK) s = drift_yz(c, dt);
  c->H = H_out;
  if (s == WDM_OK) s = density_poisson(c, 1, dt);
  c->psi = keep_psi;
  c->H = keep_H;
  return s;
}

static wdm_status adjoint_impl(wdm_ctx* c, int nsteps, double dt, int ck, const float* rho_target, int where_t,
                               const double* tidal_dir, void* grad, int where_g, double* loss, double* damp) {
  WDM_TRY(need_psi(c));
  if (nsteps < 1 || ck < 1) return fail(c, WDM_ERR_INVALID, "wdm_adjoint: nsteps and ckpt_every must be >= 1");
  if (!rho_target || !grad || !loss) return fail(c, WDM_ERR_INVALID, "wdm_adjoint: null argument");
  WDM_TRY(check_tide_rows(c, 0.0, dt, nsteps + 1, "wdm_adjoint"));
  if (c->tide_centre && c->tide_on)
    return fail(c, WDM_ERR_UNSUPPORTED, "wdm_adjoint: the tide about the density maximum is not differentiated "
                                        "(use WDM_TIDE_BOX_CENTRE)");
  const int B = c->d.batch;
  const size_t nc = (size_t)B * c->ncell, nh = (size_t)B * c->nhalf;
  if (!c->lam) WDM_TRY(dalloc(c, &c->lam, nc));
  if (!c->Hmu) WDM_TRY(dalloc(c, &c->Hmu, nh));
  if (!c->rho_t) WDM_TRY(dalloc(c, &c->rho_t, nc));
  if (!c->D6) WDM_TRY(dalloc(c, &c->D6, 6));
  if (!c->adj_acc) WDM_TRY(dalloc(c, &c->adj_acc, (size_t)2 * B));
  const int nck = nsteps / ck + 1;
  const int last_seg = (nsteps - 1) / ck, jl0 = last_seg * ck;
  // Segment s keeps its states in slot set s % 2.  The recompute of segment
  // s - 1 (on st_rec) then runs beside the reverse sweep of segment s (on the
  // context stream): each alone leaves most of the GPU idle at small grids.
  WDM_TRY(ensure_pairs(c, c->ck_psi, c->ck_H, (size_t)nck));
  WDM_TRY(ensure_pairs(c, c->slot_psi, c->slot_H, (size_t)ck + 1));
  if (last_seg > 0) {
    WDM_TRY(ensure_pairs(c, c->slot2_psi, c->slot2_H, (size_t)ck + 1));
    if (!c->st_rec) WDM_CU(c, cudaStreamCreateWithFlags(&c->st_rec, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&c->ev_ck, &c->ev_rec[0], &c->ev_rec[1], &c->ev_bwd[0], &c->ev_bwd[1]})
      if (!*e) WDM_CU(c, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  // on every way out, later work on the context stream waits for st_rec (on an
  // early error return it may still hold recomputes that use the scratch buffers)
  struct Join {
    wdm_ctx* c;
    ~Join() {
      if (c->st_rec && cudaEventRecord(c->ev_ck, c->st_rec) == cudaSuccess) cudaStreamWaitEvent(c->st, c->ev_ck, 0);
    }
  } join{c};
  std::vector<float2*>* set_psi[2] = {&c->slot_psi, &c->slot2_psi};
  std::vector<float2*>* set_H[2] = {&c->slot_H, &c->slot2_H};
  WDM_TRY(copy_in(c, c->rho_t, rho_target, sizeof(float) * nc, where_t));
  if (tidal_dir) {
    float d6[6];
    for (int q = 0; q < 6; ++q) d6[q] = (float)tidal_dir[q];
    WDM_CU(c, cudaMemcpyAsync(c->D6, d6, sizeof(d6), cudaMemcpyHostToDevice, c->st));
  }
  WDM_CU(c, cudaMemsetAsync(c->adj_acc, 0, sizeof(double) * 2 * B, c->st));
  if (c->d.phase_mode == WDM_PHASE_PRECISE) WDM_TRY(ensure_drift_tables(c, dt));
  if (c->d.absorb_alpha != 0.0) WDM_TRY(ensure_mask_tables(c, dt));
  if (!c->phi_valid) WDM_TRY(density_poisson(c, 0, dt));
  // forward: checkpoints of (s_b, H_b) at b = 0, ck, 2 ck, ...; the states of
  // the last segment go straight into its slots (no recompute needed for it)
  // state s_b of the segment starting at j0: the checkpoint or a slot of its set
  auto st_psi = [&](int seg, int b) {
    return b == seg * ck ? c->ck_psi[seg] : (*set_psi[seg & 1])[b - seg * ck];
  };
  auto st_H = [&](int seg, int b) { return b == seg * ck ? c->ck_H[seg] : (*set_H[seg & 1])[b - seg * ck]; };
  WDM_TRY(copy_pair(c, c->ck_psi[0], c->ck_H[0], c->psi, c->H));
  for (int b = 0; b < jl0; ++b) {
    WDM_TRY(forward_boundary(c, b, dt));
    if ((b + 1) % ck == 0) WDM_TRY(copy_pair(c, c->ck_psi[(b + 1) / ck], c->ck_H[(b + 1) / ck], c->psi, c->H));
  }
  for (int b = jl0; b < nsteps; ++b)
    WDM_TRY(forward_boundary_to(c, b, dt, st_psi(last_seg, b), st_H(last_seg, b), st_psi(last_seg, b + 1),
                                st_H(last_seg, b + 1)));
  {  // psi_N = final half kick of s_N, into the context's psi (psi_0 is kept in ck[0])
    float2* keep_H = c->H;
    c->H = st_H(last_seg, nsteps);
    wdm_status s = kick(c, 0.5 * dt, tide_row(c, nsteps * dt, nsteps), false, st_psi(last_seg, nsteps));
    c->H = keep_H;
    WDM_TRY(s);
  }
  cudaError_t e = launch_adj_seed(c->psi, c->rho_t, c->lam, c->ncell, B, c->dx * c->dy * c->dz, c->adj_acc, c->st);
  if (e != cudaSuccess) return cuda_fail(c, e, "adjoint seed");
  if ((e = c->kx->xfft(c->lam, rows_psi(c), c->twx, false, (float)(1.0 / c->d.nx), B, c->st)) != cudaSuccess)
    return cuda_fail(c, e, "adjoint x fwd");
  AdjArgs j{};
  j.D6 = tidal_dir ? c->D6 : nullptr;
  j.damp = c->adj_acc + B;
  const bool mask = c->d.absorb_alpha != 0.0;
  j.mx = mask ? c->mx : nullptr;
  j.my = mask ? c->my : nullptr;
  j.mz = mask ? c->mz : nullptr;
  PoissonOp po;
  po.kx2 = c->kx2;
  po.ky2 = c->ky2;
  po.kz2 = c->kz2;
  po.coef = (float)(-c->d.poisson_coeff / ((double)c->d.nx * c->d.ny * c->d.nz));
  // recompute s_{j0+1..j1} of segment seg into its slots, out of place, on st_rec
  auto recompute = [&](int seg) -> wdm_status {
    const int j0 = seg * ck, j1 = std::min(j0 + ck, nsteps);
    cudaStream_t keep = c->st;
    c->st = c->st_rec;
    wdm_status s = WDM_OK;
    for (int b = j0; b < j1 && s == WDM_OK; ++b)
      s = forward_boundary_to(c, b, dt, st_psi(seg, b), st_H(seg, b), st_psi(seg, b + 1), st_H(seg, b + 1));
    cudaError_t er = cudaSuccess;
    if (s == WDM_OK) er = cudaEventRecord(c->ev_rec[seg & 1], c->st_rec);
    c->st = keep;
    if (er != cudaSuccess) return cuda_fail(c, er, "adjoint recompute event");
    return s;
  };
  if (last_seg > 0) {
    // recomputes start from the checkpoints of the forward run above
    WDM_CU(c, cudaEventRecord(c->ev_ck, c->st));
    WDM_CU(c, cudaStreamWaitEvent(c->st_rec, c->ev_ck, 0));
    WDM_TRY(recompute(last_seg - 1));
  }
  for (int seg = last_seg; seg >= 0; --seg) {
    const int j0 = seg * ck, j1 = std::min(j0 + ck, nsteps);
    if (seg != last_seg) {
      WDM_CU(c, cudaStreamWaitEvent(c->st, c->ev_rec[seg & 1], 0));  // this segment's states
      if (seg > 0) {
        // segment seg - 1 reuses the slots of segment seg + 1, whose sweep is done
        WDM_CU(c, cudaStreamWaitEvent(c->st_rec, c->ev_bwd[(seg + 1) & 1], 0));
        WDM_TRY(recompute(seg - 1));
      }
    }
    const int blo = (j0 == 0) ? 0 : j0 + 1;
    for (int b = j1; b >= blo; --b) {
      const double dtk = (b == 0 || b == nsteps) ? 0.5 * dt : dt;
      KickArgs ka = kick_args(c, dtk, tide_row(c, b * dt, b));
      j.pre = st_psi(seg, b);
      const float2* Hb = st_H(seg, b);
      // the adjoint kick follows the kick pass's implementation (staged or direct)
      if ((e = run_pass(c, P_ADJ_KICK, [&] {
             return c->kx->adj_kick(c->lam, Hb, c->Hmu, rows_psi(c, LP_X_KICK), c->hpitch, c->nhalf, c->twx, ka, j,
                                    B, c->st);
           })) != cudaSuccess)
        return cuda_fail(c, e, "adjoint kick");
      if ((e = run_pass(c, P_ADJ_POISSON, [&] {
             cudaError_t f;
             if ((f = c->ky->lfft(c->Hmu, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, false, B, c->st)) !=
                     cudaSuccess ||
                 (f = c->kz->lfft_poisson(c->Hmu, lines_z(c, c->nxh, c->hpitch, c->nhalf), c->twz, po, B, c->st)) !=
                     cudaSuccess)
               return f;
             return c->ky->lfft(c->Hmu, lines_y(c, c->nxh, c->hpitch, c->nhalf), c->twy, true, B, c->st);
           })) != cudaSuccess)
        return cuda_fail(c, e, "adjoint Poisson");
      if ((e = run_pass(c, P_ADJ_APPLY, [&] {
             return c->kx->adj_apply(c->lam, c->Hmu, rows_psi(c), c->hpitch, c->nhalf, c->twx, j, b > 0, B, c->st);
           })) != cudaSuccess)
        return cuda_fail(c, e, "adjoint apply");
      if (b > 0) WDM_TRY(drift_yz(c, dt, -1.f, c->lam));
    }
    if (seg >= 2) WDM_CU(c, cudaEventRecord(c->ev_bwd[seg & 1], c->st));  // its slots may be reused
  }
  // leave the context at psi_0 with its potential
  WDM_TRY(copy_pair(c, c->psi, c->H, c->ck_psi[0], c->ck_H[0]));
  c->phi_valid = 1;
  WDM_TRY(copy_out(c, grad, c->lam, sizeof(float2) * nc, where_g));
  std::vector<double> acc((size_t)2 * B);
  WDM_CU(c, cudaMemcpy(acc.data(), c->adj_acc, sizeof(double) * 2 * B, cudaMemcpyDeviceToHost));
  for (int b = 0; b < B; ++b) {
    loss[b] = acc[b];
    if (damp) damp[b] = acc[B + b];
  }
  return sync_and_check(c);
}

extern "C" wdm_status wdm_adjoint(wdm_ctx* c, int32_t nsteps, double dt, int32_t ckpt_every, const float* rho_target,
                                  int32_t where_target, const double* tidal_dir, void* grad, int32_t where_grad,
                                  double* loss, double* dloss_damp) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  return adjoint_impl(c, nsteps, dt, ckpt_every, rho_target, where_target, tidal_dir, grad, where_grad, loss,
                      dloss_damp);
}

// --------------------------------------------------------------------------
// CUDA-graph replay of whole step sequences, for one context or an ensemble
// --------------------------------------------------------------------------
struct wdm_group {
  std::vector<wdm_ctx*> m;
  cudaStream_t st = nullptr;
  struct Entry {
    int nsteps, mode, sched;
    std::vector<double> dts;
    std::vector<long long> versions;
    cudaGraphExec_t exec;
    int64_t launches;
  };
  std::vector<Entry> cache;
  int64_t launches = 0;
  // schedule: GROUP_GRAPH (the members' pass launches in one captured graph),
  // GROUP_PERSISTENT (one cooperative launch of k_ensemble per call) or
  // GROUP_STREAMS (the pass launches of each member on a stream of its own,
  // forked from and joined to the group's stream inside the graph);
  // chosen by timing both on the first call (see choose_schedule)
  int sched = -1;
  double sched_ms[3] = {-1.0, -1.0, -1.0};
  std::vector<cudaStream_t> fork;     // GROUP_STREAMS: one stream per member
  std::vector<cudaEvent_t> ev_join;   // and its join event
  cudaEvent_t ev_fork = nullptr;
  // the persistent kernel's member table on the device, for (dts, mode, versions)
  EnsMember* dmem = nullptr;
  unsigned* dwords = nullptr;
  std::vector<double> dmem_dts;
  std::vector<long long> dmem_versions;
  int dmem_mode = -1;
  size_t ens_smem = 0;
  int ens_grid = 0;
};
enum { GROUP_GRAPH = 0, GROUP_PERSISTENT = 1, GROUP_STREAMS = 2, GROUP_NSCHED = 3 };

// Everything a captured step sequence must not do inside the capture (table
// uploads with a host sync, the first potential) is done here, eagerly.
static wdm_status prepare_capture(wdm_ctx* c, double dt) {
  WDM_TRY(need_psi(c));
  if (c->d.phase_mode == WDM_PHASE_PRECISE) WDM_TRY(ensure_drift_tables(c, dt));
  if (c->d.absorb_alpha != 0.0) WDM_TRY(ensure_mask_tables(c, dt));
  if (!c->phi_valid) WDM_TRY(density_poisson(c, 0, dt));
  // the deposit is made once per particle set, here, so a captured sequence
  // holds none
  WDM_TRY(ensure_deposit(c));
  WDM_CU(c, cudaStreamSynchronize(c->st));
  return WDM_OK;
}

static wdm_status group_fail(wdm_status s, const std::string& msg) { return fail(nullptr, s, msg); }

wdm_status wdm_group_create(wdm_ctx* const* members, int32_t n, wdm_group** out) {
  if (!members || n <= 0 || !out) return group_fail(WDM_ERR_INVALID, "wdm_group_create: bad arguments");
  *out = nullptr;
  wdm_group* g = new wdm_group();
  for (int i = 0; i < n; ++i) {
    if (!members[i]) {
      delete g;
      return group_fail(WDM_ERR_INVALID, "wdm_group_create: null member");
    }
    g->m.push_back(members[i]);
  }
  cudaError_t e = cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete g;
    return group_fail(WDM_ERR_CUDA, std::string("wdm_group_create: ") + cudaGetErrorString(e));
  }
  *out = g;
  return WDM_OK;
}

wdm_status wdm_group_destroy(wdm_group* g) {
  if (!g) return WDM_OK;
  if (g->st) cudaStreamSynchronize(g->st);
  for (auto& en : g->cache) cudaGraphExecDestroy(en.exec);
  if (g->dmem) cudaFree(g->dmem);
  if (g->dwords) cudaFree(g->dwords);
  for (cudaStream_t f : g->fork) cudaStreamDestroy(f);
  for (cudaEvent_t e : g->ev_join) cudaEventDestroy(e);
  if (g->ev_fork) cudaEventDestroy(g->ev_fork);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return WDM_OK;
}

int64_t wdm_group_launch_count(const wdm_group* g) { return g ? g->launches : 0; }

// The persistent kernel covers members whose axis lengths it is built for,
// without baryon particles and with a tide that is constant during the call.
static bool persistent_ok(const wdm_group* g) {
  for (const wdm_ctx* c : g->m) {
    if (!ens_size_supported(c->d.nx) || !ens_size_supported(c->d.ny) || !ens_size_supported(c->d.nz)) return false;
    if (c->tide_on == 1 && c->tide.size() > 6) return false;
  }
  return true;
}

// Member table of the persistent kernel for these time steps and mode: the
// arguments of the direct x passes and the register-tile line passes that the
// pass launches of step_impl would get.
static wdm_status build_members(wdm_group* g, const std::vector<double>& dt, int mode,
                                const std::vector<long long>& ver) {
  if (g->dmem && g->dmem_dts == dt && g->dmem_mode == mode && g->dmem_versions == ver) return WDM_OK;
  const int n = (int)g->m.size();
  std::vector<EnsMember> h((size_t)n);
  std::vector<int> nx(n), ny(n), nz(n);
  for (int i = 0; i < n; ++i) {
    wdm_ctx* c = g->m[i];
    EnsMember& e = h[i];
    e.nx = nx[i] = c->d.nx;
    e.ny = ny[i] = c->d.ny;
    e.nz = nz[i] = c->d.nz;
    e.batch = c->d.batch;
    e.psi = c->psi;
    e.H = c->H;
    e.hpitch = c->hpitch;
    e.nhalf = c->nhalf;
    e.twx = c->twx;
    e.twy = c->twy;
    e.twz = c->twz;
    e.rows = rows_psi(c);
    e.rows.impl = X_IMPL_DIRECT;
    e.ly_psi = lines_y(c, c->d.nx, c->d.nx, c->ncell);
    e.lz_psi = lines_z(c, c->d.nx, c->d.nx, c->ncell);
    e.ly_h = lines_y(c, c->nxh, c->hpitch, c->nhalf);
    e.lz_h = lines_z(c, c->nxh, c->hpitch, c->nhalf);
    e.kick_half = kick_args(c, 0.5 * dt[i], 0);
    e.kick_full = kick_args(c, dt[i], 0);
    RhoArgs ra{};
    const bool mask = c->d.absorb_alpha != 0.0;
    ra.mx = mask ? c->mx : nullptr;
    ra.my = mask ? c->my : nullptr;
    ra.mz = mask ? c->mz : nullptr;
    ra.rho_b = c->nparts > 0 ? c->rho_b : nullptr;  // the kept deposit (prepare_capture made it)
    ra.rb_rows = c->nparts > 0 ? c->rb_rows : nullptr;
    ra.write_psi = 1;
    ra.nonfinite = c->flag;
    ra.shift = c->shift;
    ra.err = c->flag + 1;
    e.centre = (c->tide_centre && c->tide_on) ? c->centre : nullptr;
    e.frame = e.centre ? c->frame : nullptr;
    e.centre_mode = c->tide_centre;
    ra.centre = e.centre;
    e.rho = ra;
    DriftOp op{};
    op.sign = 1.f;
    op.cxy = c->cxy;
    op.cz = c->cz;
    op.nxy = c->d.nx;
    op.rot = c->drift_rot;
    op.kx2 = c->kx2;
    op.ky2 = c->ky2;
    op.kz2 = c->kz2;
    op.half_dt = (float)(0.5 * dt[i]);
    op.scale = (float)(1.0 / ((double)c->d.nx * c->d.ny * c->d.nz));
    op.precise = c->d.phase_mode == WDM_PHASE_PRECISE;
    e.drift = op;
    PoissonOp po;
    po.kx2 = c->kx2;
    po.ky2 = c->ky2;
    po.kz2 = c->kz2;
    po.coef = (float)(-c->d.poisson_coeff / ((double)c->d.nx * c->d.ny * c->d.nz));
    e.poisson = po;
  }
  if (!g->dwords && cudaMalloc((void**)&g->dwords, sizeof(unsigned) * ENS_SYNC_WORDS) != cudaSuccess)
    return group_fail(WDM_ERR_ALLOC, "wdm_group_step: cudaMalloc of the barrier words failed");
  if (!g->dmem && cudaMalloc((void**)&g->dmem, sizeof(EnsMember) * n) != cudaSuccess)
    return group_fail(WDM_ERR_ALLOC, "wdm_group_step: cudaMalloc of the member table failed");
  g->ens_smem = ens_smem_bytes(nx.data(), ny.data(), nz.data(), n);
  g->ens_grid = ens_grid(g->ens_smem);
  if (g->ens_grid <= 0) return group_fail(WDM_ERR_CUDA, "wdm_group_step: the persistent kernel does not fit");
  for (int i = 0; i < n; ++i) h[i].rot = (int)(((long long)i * g->ens_grid) / n);
  cudaError_t e = cudaMemcpyAsync(g->dmem, h.data(), sizeof(EnsMember) * n, cudaMemcpyHostToDevice, g->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->st);
  if (e != cudaSuccess) return group_fail(WDM_ERR_CUDA, std::string("wdm_group_step: member table: ") + cudaGetErrorString(e));
  g->dmem_dts = dt;
  g->dmem_mode = mode;
  g->dmem_versions = ver;
  return WDM_OK;
}

// Enqueue one call on the group's stream under schedule `sched`: the captured
// graph of the members' pass launches, or the graph of one persistent launch
// (its barrier words cleared first).  Graphs are captured once per (nsteps,
// mode, dts, member state, schedule) and replayed.
static wdm_status group_launch(wdm_group* g, int32_t nsteps, const std::vector<double>& dt,
                               const std::vector<long long>& ver, int32_t mode, int sched) {
  const size_t n = g->m.size();
  if (sched == GROUP_PERSISTENT) WDM_TRY(build_members(g, dt, mode, ver));
  if (sched == GROUP_STREAMS && g->fork.size() < n) {
    if (!g->ev_fork && cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming) != cudaSuccess)
      return group_fail(WDM_ERR_CUDA, "wdm_group_step: cudaEventCreate failed");
    while (g->fork.size() < n) {
      cudaStream_t f = nullptr;
      cudaEvent_t ev = nullptr;
      if (cudaStreamCreateWithFlags(&f, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        if (f) cudaStreamDestroy(f);
        return group_fail(WDM_ERR_CUDA, "wdm_group_step: stream or event creation failed");
      }
      g->fork.push_back(f);
      g->ev_join.push_back(ev);
    }
  }
  wdm_group::Entry* hit = nullptr;
  for (auto& en : g->cache)
    if (en.nsteps == nsteps && en.mode == mode && en.sched == sched && en.dts == dt && en.versions == ver) hit = &en;
  if (!hit) {
    if (g->cache.size() >= 8) {
      cudaGraphExecDestroy(g->cache.front().exec);
      g->cache.erase(g->cache.begin());
    }
    cudaError_t e = cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return group_fail(WDM_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(e));
    int64_t launches = 0;
    wdm_status bad = WDM_OK;
    std::string why;
    if (sched == GROUP_PERSISTENT) {
      wdm_ctx* c0 = g->m[0];
      const long long l0 = tl_kernel_launches;
      e = cudaMemsetAsync(g->dwords, 0, sizeof(unsigned) * ENS_SYNC_WORDS, g->st);
      // the frames of the first kicks (later ones are made inside the launch)
      for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
        wdm_ctx* c = g->m[i];
        if (c->tide_centre && c->tide_on)
          e = launch_tide_frame(c->centre, kick_args(c, dt[i], 0), c->tide_centre, c->d.nx, c->d.ny, c->d.batch,
                                c->frame, g->st);
      }
      if (e == cudaSuccess)
        e = ens_launch(g->dmem, (int)n, nsteps, mode, g->dwords, c0->flag + 1, g->ens_smem, g->ens_grid, g->st);
      launches = tl_kernel_launches - l0;
      if (e != cudaSuccess) {
        bad = WDM_ERR_CUDA;
        why = std::string("persistent launch: ") + cudaGetErrorString(e);
      }
    } else {
      const bool streams = sched == GROUP_STREAMS;
      if (streams && (e = cudaEventRecord(g->ev_fork, g->st)) != cudaSuccess) {
        bad = WDM_ERR_CUDA;
        why = std::string("fork: ") + cudaGetErrorString(e);
      }
      for (size_t i = 0; i < n && bad == WDM_OK; ++i) {
        wdm_ctx* c = g->m[i];
        cudaStream_t own = c->st;
        const bool prof = c->prof.on;
        const int64_t l0 = c->launch_count;
        c->st = streams ? g->fork[i] : g->st;
        c->prof.on = false;
        if (streams && (e = cudaStreamWaitEvent(c->st, g->ev_fork, 0)) != cudaSuccess) {
          bad = WDM_ERR_CUDA;
          why = std::string("fork: ") + cudaGetErrorString(e);
        }
        if (bad == WDM_OK) {
          bad = step_impl(c, nsteps, dt[i], 0.0, mode);
          if (bad != WDM_OK) why = c->err;
        }
        if (bad == WDM_OK && streams &&
            ((e = cudaEventRecord(g->ev_join[i], c->st)) != cudaSuccess ||
             (e = cudaStreamWaitEvent(g->st, g->ev_join[i], 0)) != cudaSuccess)) {
          bad = WDM_ERR_CUDA;
          why = std::string("join: ") + cudaGetErrorString(e);
        }
        launches += c->launch_count - l0;
        c->launch_count = l0;  // counted when the graph runs
        c->st = own;
        c->prof.on = prof;
      }
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(g->st, &graph);
    if (bad != WDM_OK || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      if (bad != WDM_OK) return group_fail(bad, "wdm_group_step: capture: " + why);
      return group_fail(WDM_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return group_fail(WDM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    g->cache.push_back({nsteps, mode, sched, dt, ver, exec, launches});
    hit = &g->cache.back();
  }
  cudaError_t e = cudaGraphLaunch(hit->exec, g->st);
  if (e != cudaSuccess) return group_fail(WDM_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
  g->launches += hit->launches;
  for (size_t i = 0; i < n; ++i) g->m[i]->launch_count += hit->launches / (int64_t)n;
  return WDM_OK;
}

// Time the schedules on the members' own state (saved first and put back
// after each timing), two steps each after a warm-up call, and keep the
// fastest (the graph of pass launches unless another is faster by more than
// 3%).  The persistent kernel is timed only for the groups it covers.
// WDM_GROUP_SCHEDULE=graph|persistent|streams forces the choice.
static wdm_status choose_schedule(wdm_group* g, const std::vector<double>& dt, const std::vector<long long>& ver,
                                  int32_t mode) {
  if (const char* env = std::getenv("WDM_GROUP_SCHEDULE")) {
    if (!std::strcmp(env, "graph")) {
      g->sched = GROUP_GRAPH;
      return WDM_OK;
    }
    if (!std::strcmp(env, "streams")) {
      g->sched = GROUP_STREAMS;
      return WDM_OK;
    }
    if (!std::strcmp(env, "persistent")) {
      if (!persistent_ok(g)) return group_fail(WDM_ERR_UNSUPPORTED, "WDM_GROUP_SCHEDULE=persistent: a member's "
                                                                   "size or options are not covered by the persistent kernel");
      g->sched = GROUP_PERSISTENT;
      return WDM_OK;
    }
  }
  const bool pers = persistent_ok(g);
  const size_t n = g->m.size();
  std::vector<float2*> keep(2 * n, nullptr);
  auto release = [&]() {
    for (float2* p : keep)
      if (p) cudaFree(p);
  };
  for (size_t i = 0; i < n; ++i) {
    wdm_ctx* c = g->m[i];
    const size_t np = (size_t)c->ncell * c->d.batch, nh = (size_t)c->nhalf * c->d.batch;
    if (cudaMalloc((void**)&keep[2 * i], sizeof(float2) * np) != cudaSuccess ||
        cudaMalloc((void**)&keep[2 * i + 1], sizeof(float2) * nh) != cudaSuccess) {
      release();
      g->sched = GROUP_GRAPH;  // no room to time both: keep the launches
      cudaGetLastError();
      return WDM_OK;
    }
    cudaMemcpyAsync(keep[2 * i], c->psi, sizeof(float2) * np, cudaMemcpyDeviceToDevice, g->st);
    cudaMemcpyAsync(keep[2 * i + 1], c->H, sizeof(float2) * nh, cudaMemcpyDeviceToDevice, g->st);
  }
  // the tide-frame words of the last density pass belong to the saved state too
  std::vector<std::vector<unsigned long long>> words(n);
  cudaStreamSynchronize(g->st);
  for (size_t i = 0; i < n; ++i)
    if (g->m[i]->centre) {
      words[i].resize((size_t)CENTRE_WORDS * g->m[i]->d.batch);
      cudaMemcpy(words[i].data(), g->m[i]->centre, sizeof(unsigned long long) * words[i].size(), cudaMemcpyDeviceToHost);
    }
  auto restore = [&]() {
    for (size_t i = 0; i < n; ++i) {
      wdm_ctx* c = g->m[i];
      cudaMemcpyAsync(c->psi, keep[2 * i], sizeof(float2) * c->ncell * c->d.batch, cudaMemcpyDeviceToDevice, g->st);
      cudaMemcpyAsync(c->H, keep[2 * i + 1], sizeof(float2) * c->nhalf * c->d.batch, cudaMemcpyDeviceToDevice, g->st);
      if (!words[i].empty())
        cudaMemcpyAsync(c->centre, words[i].data(), sizeof(unsigned long long) * words[i].size(),
                        cudaMemcpyHostToDevice, g->st);
    }
    cudaStreamSynchronize(g->st);
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  wdm_status st = WDM_OK;
  for (int sch = 0; sch < GROUP_NSCHED && st == WDM_OK; ++sch) {
    if (sch == GROUP_PERSISTENT && !pers) continue;
    st = group_launch(g, 2, dt, ver, mode, sch);  // warm-up (and capture)
    restore();
    if (st != WDM_OK) break;
    cudaEventRecord(e0, g->st);
    st = group_launch(g, 2, dt, ver, mode, sch);
    cudaEventRecord(e1, g->st);
    restore();
    if (st != WDM_OK) break;
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      st = group_fail(WDM_ERR_CUDA, "wdm_group_step: schedule timing failed");
      break;
    }
    g->sched_ms[sch] = ms;
  }
  cudaStreamSynchronize(g->st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  release();
  if (st != WDM_OK) return st;
  for (wdm_ctx* c : g->m) {  // the timing runs must leave no error bits behind
    cudaMemsetAsync(c->flag, 0, 2 * sizeof(int), g->st);
  }
  cudaStreamSynchronize(g->st);
  int best = GROUP_GRAPH;
  for (int sch = 1; sch < GROUP_NSCHED; ++sch)
    if (g->sched_ms[sch] > 0.0 && g->sched_ms[sch] < 0.97 * g->sched_ms[GROUP_GRAPH] &&
        g->sched_ms[sch] < g->sched_ms[best])
      best = sch;
  g->sched = best;
  return WDM_OK;
}

// Launch nsteps steps of every member on the group's stream without waiting.
static wdm_status group_enqueue(wdm_group* g, int32_t nsteps, const double* dts, int32_t mode) {
  if (!g || !dts || nsteps < 0) return group_fail(WDM_ERR_INVALID, "wdm_group_step: bad arguments");
  if (mode != WDM_STEP_STRANG && mode != WDM_STEP_REFERENCE_LOOP && mode != WDM_STEP_LIE)
    return group_fail(WDM_ERR_INVALID, "wdm_group_step: unknown step mode");
  if (nsteps == 0) return WDM_OK;
  const size_t n = g->m.size();
  std::vector<double> dt(dts, dts + n);
  std::vector<long long> ver(n);
  for (size_t i = 0; i < n; ++i) {
    const wdm_ctx* c = g->m[i];
    if (c->tide_on == 1 && c->tide.size() > 6 && c->tide_dt > 0.0)
      return group_fail(WDM_ERR_STATE, "wdm_group_step: member " + std::to_string(i) +
                                           " has a clocked tidal schedule of several rows; a replayed graph "
                                           "cannot follow the time (use wdm_step)");
    wdm_status s = prepare_capture(g->m[i], dt[i]);
    if (s != WDM_OK) return group_fail(s, "wdm_group_step: member " + std::to_string(i) + ": " + g->m[i]->err);
    ver[i] = g->m[i]->version;
  }
  if (g->sched < 0 || (g->sched == GROUP_PERSISTENT && !persistent_ok(g))) WDM_TRY(choose_schedule(g, dt, ver, mode));
  return group_launch(g, nsteps, dt, ver, mode, g->sched);
}

wdm_status wdm_group_schedule(const wdm_group* g, int32_t* sched, double* ms) {
  if (!g || !sched) return group_fail(WDM_ERR_INVALID, "wdm_group_schedule: null argument");
  *sched = g->sched;
  if (ms)
    for (int k = 0; k < GROUP_NSCHED; ++k) ms[k] = g->sched_ms[k];
  return WDM_OK;
}

wdm_status wdm_group_step(wdm_group* g, int32_t nsteps, const double* dts, int32_t mode) {
  WDM_TRY(group_enqueue(g, nsteps, dts, mode));
  if (nsteps == 0) return WDM_OK;
  cudaError_t e = cudaStreamSynchronize(g->st);
  if (e != cudaSuccess) return group_fail(WDM_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
  for (size_t i = 0; i < g->m.size(); ++i) {
    wdm_status s = sync_and_check(g->m[i]);
    if (s != WDM_OK) return group_fail(s, "wdm_group_step: member " + std::to_string(i) + ": " + g->m[i]->err);
  }
  return WDM_OK;
}

wdm_status wdm_group_step_async(wdm_group* g, int32_t nsteps, const double* dts, int32_t mode) {
  return group_enqueue(g, nsteps, dts, mode);
}

void* wdm_group_stream(const wdm_group* g) { return g ? (void*)g->st : nullptr; }

wdm_status wdm_step_graph(wdm_ctx* c, int32_t nsteps, double dt, int32_t mode) {
  if (!c) return fail(nullptr, WDM_ERR_INVALID, "null context");
  if (!c->self_group) {
    wdm_ctx* self = c;
    wdm_status s = wdm_group_create(&self, 1, &c->self_group);
    if (s != WDM_OK) return fail(c, s, wdm_last_error(nullptr));
  }
  wdm_status s = wdm_group_step(c->self_group, nsteps, &dt, mode);
  if (s != WDM_OK) return fail(c, s, wdm_last_error(nullptr));
  return WDM_OK;
}

}  // extern "C"
