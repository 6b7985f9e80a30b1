/*
 * libwavedm -- GB300 (sm_103a) split-step Fourier kick-drift-kick step for the
 * Schroedinger-Poisson equation, behind a plain C ABI.
 *
 * Every entry point returns a wdm_status; wdm_last_error() gives the message of
 * the last failure on a context (or the last create failure when ctx is NULL).
 * The context owns every device buffer and one CUDA stream; host buffers passed
 * in are borrowed for the duration of the call only.  Calls on one context are
 * not thread safe (one context per host thread).  A call returns after its work
 * is complete on the GPU unless its name ends in _async.
 *
 * Arrays are C order [nz][ny][nx] (x fastest), which is the memory order of the
 * reference's column-major Julia arrays psi[x, y, z]: a Julia Array{ComplexF32,3}
 * or CuArray{ComplexF32,3} is passed as is.
 *
 * Reference interfaces replaced (paths inside the WaveDM.jl project):
 *   apply_kick_step!          src/solver/KDK.jl:37-77        -> wdm_kick
 *   apply_drift_step!         src/solver/KDK.jl:88-101       -> wdm_drift
 *   setup_fft_operators       src/solver/fft_operators.jl:8-15 -> built inside wdm_drift / wdm_step
 *   setup_absorption_boundary src/solver/fft_operators.jl:22-27 -> wdm_desc.absorb_alpha
 *   compute_gravitational_potential src/solver/gravity.jl:7-35 -> wdm_get_phi
 *   parallel_poisson / _poisson_gpu src/parallel_poisson.jl:36-68 -> wdm_poisson
 *   SPE3D_waveDM loop body    src/simulation_main.jl:536-559 -> wdm_step
 *   add_tidal_potential!      src/physics/tidal_fields.jl:64-118 -> wdm_set_tidal
 *   total mass / virial sums  src/simulation_main.jl:652, src/visualization/runtime.jl:210-238 -> wdm_reduce
 *   loop diagnostics (findmax, radii quantiles, R, momentum) and compute_timestep limits
 *                             src/simulation_main.jl:551-558,641-653, src/physics/poisson.jl:35-50 -> wdm_diagnostics
 */
#ifndef WAVEDM_H
#define WAVEDM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  WDM_OK = 0,
  WDM_ERR_INVALID = 1,      /* bad argument (null pointer, size, mode)            */
  WDM_ERR_UNSUPPORTED = 2,  /* grid size without an FFT plan, option not built    */
  WDM_ERR_CUDA = 3,         /* a CUDA runtime call failed                         */
  WDM_ERR_ALLOC = 4,        /* device allocation failed                           */
  WDM_ERR_NONFINITE = 5,    /* psi or Phi holds NaN/Inf after a step              */
  WDM_ERR_STATE = 6         /* call out of order (e.g. no psi set yet)            */
} wdm_status;

typedef enum { WDM_HOST = 0, WDM_DEVICE = 1 } wdm_where;

typedef enum {
  WDM_STEP_STRANG = 0,         /* K(dt/2) D(dt) [mask] K(dt/2), docs/src/algorithms.md:120-142 */
  WDM_STEP_REFERENCE_LOOP = 1, /* K(dt/2) D(dt) [mask]: the literal loop, simulation_main.jl:538-547 */
  WDM_STEP_LIE = 2             /* K(dt) D(dt) [mask]: KDK_flag = false                       */
} wdm_step_mode;

typedef enum {
  WDM_GRID_PERIODIC = 0,  /* x_i = -L/2 + i L/N, k = 2 pi m / L                           */
  WDM_GRID_REFERENCE = 1  /* x = LinRange(-L/2, L/2, N) (poisson.jl:8-15), k = 2 pi m / L  */
} wdm_grid_convention;

typedef enum {
  WDM_PHASE_PLAIN = 0,    /* FP32 phases k^2 dt/2 and Phi dt                               */
  WDM_PHASE_PRECISE = 1   /* FP64-built separable drift tables; kick phase reduced mod 2 pi
                             in float-float before the FP32 sincos                          */
} wdm_phase_mode;

typedef struct {
  int32_t nx, ny, nz;          /* grid points per axis: each 2^a 3^b with a plan (8..512)   */
  double lx, ly, lz;           /* full box lengths                                          */
  int32_t convention;          /* wdm_grid_convention                                       */
  double poisson_coeff;        /* c in lap Phi = c (rho - <rho>): 4 pi G (4pi in the reference, gravity.jl:23) */
  double kerr;                 /* kappa of the local potential kappa |psi|^2 (0: off)       */
  double absorb_alpha;         /* absorbing-mask coefficient (0: no mask), fft_operators.jl:22-27 */
  int32_t phase_mode;          /* wdm_phase_mode                                            */
  int32_t batch;               /* independent halos of this size advanced together (>= 1)  */
} wdm_desc;

typedef struct wdm_ctx wdm_ctx;

/* lifecycle ---------------------------------------------------------------- */
wdm_status wdm_create(const wdm_desc* desc, wdm_ctx** out);
wdm_status wdm_destroy(wdm_ctx* ctx);
const char* wdm_last_error(const wdm_ctx* ctx);
int32_t wdm_version(void);
/* 1 when an FFT plan exists for n (2^a 3^b in [8, 512]) */
int32_t wdm_size_supported(int32_t n);

/* state --------------------------------------------------------------------- */
/* psi: complex64 (interleaved float pairs) [batch][nz][ny][nx] */
wdm_status wdm_set_psi(wdm_ctx* ctx, const void* psi, int32_t where);
wdm_status wdm_get_psi(wdm_ctx* ctx, void* psi, int32_t where);
/* rho = |psi|^2 and the total potential Phi (gravity only, no V/tide), float32 */
wdm_status wdm_get_rho(wdm_ctx* ctx, float* rho, int32_t where);
wdm_status wdm_get_phi(wdm_ctx* ctx, float* phi, int32_t where);
/* static external potential V [batch][nz][ny][nx] float32; NULL clears it */
wdm_status wdm_set_static_potential(wdm_ctx* ctx, const float* V, int32_t where);
/* tidal tensor 1/2 x^T T x about the box centre, T = (xx, yy, zz, xy, xz, yz),
 * replacing the tide add_tidal_potential! evaluates at time t[i]
 * (src/physics/tidal_fields.jl:64-118).
 * schedule: nsched rows of 6 doubles.  Without a clock (the state after this
 * call) row s is used by kick s of every following wdm_step call, the kick at
 * time t0 + s*dt, whatever t0 is; a single row is a constant tide.
 * per_item != 0: one constant row per batch item (nsched == batch).
 * nsched == 0 turns the tide off.  Either form clears the clock. */
wdm_status wdm_set_tidal(wdm_ctx* ctx, const double* schedule, int32_t nsched, int32_t per_item);
/* Gives the shared-row schedule of wdm_set_tidal a clock: row s is the tensor
 * at time t_first + s*t_step.  Every kick then uses the row nearest to its own
 * time (wdm_step: t0 + s*dt; wdm_kick: t; wdm_adjoint: s*dt from t = 0), and a
 * call whose kicks fall outside the rows returns WDM_ERR_INVALID.  t_step == 0
 * removes the clock.  A clocked schedule of several rows cannot be replayed by
 * wdm_step_graph or a group (their graphs do not follow the time):
 * WDM_ERR_STATE.  No counterpart in the reference, whose tide is a function
 * of t evaluated on the host every step. */
wdm_status wdm_set_tidal_clock(wdm_ctx* ctx, double t_first, double t_step);
/* Where the tide is anchored, replacing the treatment of the tidal potential
 * at the density maximum in add_tidal_potential! (src/physics/tidal_fields.jl:114-146).
 * x_c is the centre of the cell of the largest |psi|^2 (the first such cell in
 * memory order, as findmax picks it; baryons not included) and <x> the
 * |psi|^2-weighted mean position, both taken by the density pass before each
 * kick.  For Phi(x) = 1/2 x^T T x about the box centre:
 *   WDM_TIDE_BOX_CENTRE  Phi(x) (the default);
 *   WDM_TIDE_REFERENCE   Phi(x) - Phi(x_c): the potential the reference's code
 *                        leaves (tidal_fields.jl:114).  Its gradient
 *                        cancellation (:115, :126-146) assigns to its local
 *                        argument and discards the result, so the caller's
 *                        potential keeps its gradient;
 *   WDM_TIDE_DENSITY_MAX Phi(x) - Phi(x_c) - grad Phi(x_c).(x - <x>): the value and
 *                        gradient removed at x_c as that cancellation computes
 *                        them, = 1/2 (x-x_c)^T T (x-x_c) + (T x_c).(<x> - x_c).
 * Modes 0 and 1 differ by a uniform potential (a global phase of psi).
 * wdm_adjoint refuses modes 1 and 2 (WDM_ERR_UNSUPPORTED). */
typedef enum { WDM_TIDE_BOX_CENTRE = 0, WDM_TIDE_REFERENCE = 1, WDM_TIDE_DENSITY_MAX = 2 } wdm_tide_centering;
wdm_status wdm_set_tidal_centering(wdm_ctx* ctx, int32_t mode);
/* static baryon particles (positions [n][3] and masses [n], doubles): their
 * CIC deposit is made once, at the next density pass, and added to the density
 * of every Poisson solve until the next call; n == 0 removes them.  The call
 * invalidates the potential, which the next kick or step recomputes. */
wdm_status wdm_set_particles(wdm_ctx* ctx, const double* pos, const double* mass, int64_t n);

/* the path ------------------------------------------------------------------ */
/* nsteps steps of size dt from time t0: kick s runs at time t0 + s*dt (the
 * Strang step's closing half kick is kick nsteps), which selects its tidal
 * row when the schedule has a clock (wdm_set_tidal_clock) */
wdm_status wdm_step(wdm_ctx* ctx, int32_t nsteps, double dt, double t0, int32_t mode);
wdm_status wdm_step_async(wdm_ctx* ctx, int32_t nsteps, double dt, double t0, int32_t mode);
/* wdm_step through a CUDA graph: the launches of nsteps steps are captured once
 * per (nsteps, dt, mode, state) and replayed; returns when the steps are done.
 * Every replay uses tidal rows 0..nsteps of an unclocked schedule. */
wdm_status wdm_step_graph(wdm_ctx* ctx, int32_t nsteps, double dt, int32_t mode);

/* ensembles: contexts of different grid sizes (each holding `batch` halos of
 * its size) advanced together; their steps are captured into one CUDA graph on
 * one stream and replayed as a single graph launch per call.  Member contexts
 * stay owned by the caller and must outlive the group. */
typedef struct wdm_group wdm_group;
wdm_status wdm_group_create(wdm_ctx* const* members, int32_t n, wdm_group** out);
wdm_status wdm_group_destroy(wdm_group* g);
/* nsteps steps of every member, member i with time step dts[i] */
wdm_status wdm_group_step(wdm_group* g, int32_t nsteps, const double* dts, int32_t mode);
/* the same, returning once the graph is enqueued on the group's stream (check
 * the members with wdm_check_finite after synchronising the stream) */
wdm_status wdm_group_step_async(wdm_group* g, int32_t nsteps, const double* dts, int32_t mode);
/* How the group runs a call, chosen on its first call by timing the
 * candidates on the members' own state (saved and put back):
 *   0  the members' pass launches, captured into one CUDA graph, one member
 *      after another on the group's stream;
 *   1  one persistent cooperative kernel for all passes of all members and
 *      steps, a device-wide barrier between passes (its waits bounded: an
 *      abandoned one is reported as WDM_ERR_CUDA), replayed from a graph.
 *      It covers members with axis lengths 16..128 without baryon particles
 *      and with a tide that is constant during the call (timed only then);
 *   2  the members' pass launches in one graph, each member on a stream of
 *      its own forked from the group's stream, so that the sizes run
 *      concurrently.
 * sched: the choice (-1 before the first call); ms[0..2]: the timed
 * milliseconds of two steps under each (-1 when not timed).  The environment
 * variable WDM_GROUP_SCHEDULE=graph|persistent|streams forces the choice. */
wdm_status wdm_group_schedule(const wdm_group* g, int32_t* sched, double* ms);
/* the group's cudaStream_t */
void* wdm_group_stream(const wdm_group* g);
/* kernel launches executed by the group's graph replays so far */
int64_t wdm_group_launch_count(const wdm_group* g);

/* apply_kick_step!: Phi from |psi|^2, psi <- exp(-i dt (Phi + V + tide(t))) psi.
 * tide(t) is the clocked schedule's row nearest to t, or the single row of a
 * constant tide; an unclocked schedule of several rows gives WDM_ERR_STATE. */
wdm_status wdm_kick(wdm_ctx* ctx, double dt, double t);
/* apply_drift_step!: psi <- mask * ifft(exp(-i k^2 dt/2) fft(psi)) */
wdm_status wdm_drift(wdm_ctx* ctx, double dt);
/* parallel_poisson: phi = Poisson(rho) with lap phi = coeff (rho - <rho>), float32
 * [batch][nz][ny][nx] in and out (host or device pointers) */
wdm_status wdm_poisson(wdm_ctx* ctx, const float* rho, float* phi, int32_t where);
/* in-place 3D C2C FFT of a complex64 device array (dir = -1 forward, +1 inverse, unnormalised) */
wdm_status wdm_fft3d(wdm_ctx* ctx, void* data_dev, int32_t dir);
/* The same Poisson solve as wdm_poisson for one device-resident grid, for callers
 * that cannot allocate device memory: code running under a host runtime that owns
 * the GPU's memory pool and allows no allocation outside it (for example a Julia
 * CUDA.jl process with a memory limit), or a time-critical loop in which the
 * implicit device synchronisation of cudaMalloc/cudaFree would stall other work.
 * It needs no context and calls no cudaMalloc, cudaFree or other allocating
 * routine.  Its scratch is one static device array of about 8.3 MiB that every
 * GPU loading the library holds until the process exits; grids are limited to
 * (nx/2+1)*ny*nz <= 1,064,960 (a 128^3 grid), larger ones return
 * WDM_ERR_INVALID.  rho and phi are float32 device pointers [nz][ny][nx]; stream is
 * a cudaStream_t (NULL: the default stream).  The call synchronises that stream
 * before it returns, so phi is ready on return, and for the same reason no call
 * can be made while the stream is being captured into a CUDA graph.  All calls
 * share the array: calls whose work overlaps on the GPU race and must be
 * serialised by the caller.
 * It builds its twiddle tables on the device (FP64 sincospi) where wdm_poisson
 * builds them on the host, and it always takes the register-tile line passes
 * and the direct x passes, so its phi agrees with wdm_poisson's to FP32
 * rounding, not bit for bit.
 * Errors are reported through wdm_last_error(NULL).
 * No counterpart in the reference: it is an addition of this library. */
wdm_status wdm_poisson_noalloc(const float* rho_dev, float* phi_dev, int32_t nx, int32_t ny, int32_t nz,
                               double lx, double ly, double lz, double poisson_coeff, void* stream);

/* differentiation ------------------------------------------------------------ */
/* Adjoint of nsteps Strang steps from the context's psi_0 (left unchanged) for
 * L = sum (|psi_N|^2 - rho_target)^2 dV per batch item.  Outputs:
 *   grad       complex64 [batch][nz][ny][nx]: dL/dRe psi_0 + i dL/dIm psi_0
 *   loss       L per batch item (doubles)
 *   dloss_damp dL/da per batch item when tidal_dir (6 doubles) is given, for a
 *              tide equal to a * tidal_dir (as set with wdm_set_tidal); may be NULL
 * psi is checkpointed every ckpt_every steps and recomputed between checkpoints
 * (memory: (nsteps/ckpt_every + ckpt_every + 2) copies of psi and its half
 * spectrum).  rho_target is float32 on host or device (where_target); grad is
 * written to host or device memory (where_grad).  No counterpart in the
 * reference (it has no differentiation); the gradient is exact for the
 * discrete run, FP32 rounding aside. */
wdm_status wdm_adjoint(wdm_ctx* ctx, int32_t nsteps, double dt, int32_t ckpt_every, const float* rho_target,
                       int32_t where_target, const double* tidal_dir, void* grad, int32_t where_grad, double* loss,
                       double* dloss_damp);

/* diagnostics --------------------------------------------------------------- */
/* out[0..9] (per batch item, 10 doubles each): mass, rho_max, argmax (flat index),
 * centre of mass x, y, z, and the virial sums VirialPotential, TotalKineticE,
 * TotalQuantumE, Virial = 2K + 2Q - VirialPotential */
wdm_status wdm_reduce(wdm_ctx* ctx, double* out);
/* The per-step loop diagnostics of src/simulation_main.jl:551-558,641-653 and
 * the timestep limits of compute_timestep (src/physics/poisson.jl:35-50),
 * computed on the device so the loop needs no psi download.
 * out[WDM_DIAG_FIELDS * b + k] for batch item b:
 *   0..9   the wdm_reduce fields;
 *   10..12 MomentumX/Y/Z = sum rho v dV over interior cells
 *          (src/visualization/runtime.jl:229-231, code units);
 *   13     max |Phi| (gravity with baryons; the tidal term is not included);
 *   14     max |psi|;
 *   15..17 the limits 2 dx^2 / pi, 2 pi / max|Phi|, 2 pi / (|kappa| max|psi|)
 *          (infinity where a denominator is zero);
 *   18     R: weighted standard deviation (uncorrected, weights |psi|^2) of
 *          the distance from the coordinate origin over the z-slice nz/2 - 1
 *          (0-based; the reference's r[:, :, div(end, 2)]);
 *   19..27 radii at p = 0.1, 0.2, ..., 0.9: weighted quantiles of the distance
 *          from the density maximum with weights rho (the StatsBase weighted
 *          quantile, FP64 cumulative sums; needs dx == dy == dz, else NaN). */
#define WDM_DIAG_FIELDS 28
wdm_status wdm_diagnostics(wdm_ctx* ctx, double* out);
/* The weighted quantile behind the radii, on values grouped by equal value:
 * groups ascending strictly in value[], with the total weight wsum[] and the
 * smallest element weight wmin[] of each group (empty groups: wsum 0).
 * Host-only; the grouped form of StatsBase's quantile(v, w, p). */
wdm_status wdm_weighted_quantiles_grouped(const double* value, const double* wsum, const double* wmin, int64_t ngroups,
                                          const double* p, int32_t np, double* out);
/* CIC interpolation of Phi (gravity) at n positions [n][3] -> out[n] (doubles, host) */
wdm_status wdm_interpolate_phi(wdm_ctx* ctx, const double* pos, int64_t n, double* out);
/* 1 if the last checked step left psi finite */
wdm_status wdm_check_finite(wdm_ctx* ctx, int32_t* finite);
/* CUDA stream the context runs on (a cudaStream_t) */
void* wdm_stream(wdm_ctx* ctx);

/* profiling ------------------------------------------------------------------ */
/* per-pass GPU time: with on != 0 every pass launch is bracketed by CUDA events
 * on the context stream (off by default; turning it on clears the totals) */
wdm_status wdm_set_profiling(wdm_ctx* ctx, int32_t on);
/* which passes profiling brackets with events: bit p for pass p (default all).
 * Bracketing only the pass of interest keeps the event overhead of the others
 * out of a timed run. */
wdm_status wdm_set_profile_mask(wdm_ctx* ctx, uint64_t mask);
/* for pass p < WDM_NPASS: launches, summed milliseconds and algorithmic bytes
 * (one read + one write of every operand) of one launch, since profiling on */
wdm_status wdm_get_profile(wdm_ctx* ctx, int64_t* launches, double* ms, double* bytes_per_launch);
/* Pass schedule chosen by the autotuner when the context was created, for the
 * passes psi-y, psi-z, H-y, H-z (line passes: impl 0 = TMA-fed persistent
 * pass, 1 = register-tile pass), the kick, the density pass and the density
 * pass with baryons (x passes: impl 0 = rows staged by bulk copies, 1 = rows
 * loaded directly), in that order; ms[2k], ms[2k+1] the best timed
 * milliseconds of implementations 0 and 1.  The environment variables
 * WDM_SCHEDULE (all seven, comma separated), WDM_LINE_IMPL=tma|tile and
 * WDM_X_IMPL=staged|direct override the choice. */
wdm_status wdm_get_line_schedule(const wdm_ctx* ctx, int32_t impl[7], double ms[14]);
/* number of passes and the name of pass p */
int32_t wdm_num_passes(void);
const char* wdm_pass_name(int32_t p);
/* kernel launches issued by this context since creation */
int64_t wdm_launch_count(const wdm_ctx* ctx);

/* self-test ------------------------------------------------------------------ */
/* out[2i], out[2i+1] = sin, cos of h[i] (|h| <= pi/2) as evaluated by the series
 * the precise phase form uses; device pointers, n values. */
wdm_status wdm_selftest_sincos(const float* h_dev, float* out_dev, int64_t n);
/* Runs one CTA that waits on an mbarrier nothing completes, through the bounded
 * wait of the TMA-fed passes with a limit of limit_ns nanoseconds.  On return
 * *bits holds the error bits the kernel recorded (1: wait abandoned) and
 * *waited_ns how long it waited; the device stays usable. */
wdm_status wdm_selftest_bounded_wait(int64_t limit_ns, int32_t* bits, int64_t* waited_ns);

#ifdef __cplusplus
}
#endif
#endif
