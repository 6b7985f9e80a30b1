# Julia bindings of libwavedm for WaveDM.jl's gpu=true path.
#
# ccall wrappers over include/wavedm.h plus the drop-in replacements of the
# operators the SPE3D_waveDM loop calls on the GPU (src/solver/KDK.jl,
# src/parallel_poisson.jl), and a ChainRulesCore.rrule for the checkpointed
# adjoint.  Arrays are passed as they are: a CuArray{ComplexF32,3} psi[x, y, z]
# (column major, x fastest) is the [nz][ny][nx] C-order layout of the library.
module WaveDMGB300

using CUDA
using ChainRulesCore

const libwavedm = get(ENV, "WDM_LIB_PATH", joinpath(@__DIR__, "..", "libwavedm.so"))

const WDM_HOST, WDM_DEVICE = Int32(0), Int32(1)
const WDM_STEP_STRANG, WDM_STEP_REFERENCE_LOOP, WDM_STEP_LIE = Int32(0), Int32(1), Int32(2)
const WDM_GRID_PERIODIC, WDM_GRID_REFERENCE = Int32(0), Int32(1)
const WDM_PHASE_PLAIN, WDM_PHASE_PRECISE = Int32(0), Int32(1)

# same field order and types as wdm_desc; Julia lays isbits structs out with C alignment
struct WdmDesc
    nx::Int32; ny::Int32; nz::Int32
    lx::Float64; ly::Float64; lz::Float64
    convention::Int32
    poisson_coeff::Float64
    kerr::Float64
    absorb_alpha::Float64
    phase_mode::Int32
    batch::Int32
end

struct WdmError <: Exception
    status::Int32
    msg::String
end

lasterror(h) = unsafe_string(ccall((:wdm_last_error, libwavedm), Cstring, (Ptr{Cvoid},), h))
check(st, h=C_NULL) = st == 0 ? nothing : throw(WdmError(st, lasterror(h)))

mutable struct Context
    h::Ptr{Cvoid}
    dims::NTuple{3,Int}
    function Context(Nx, Ny, Nz, Lx, Ly, Lz; convention=WDM_GRID_REFERENCE, poisson_coeff=4π, kerr=0.0,
                     absorb_coeff=0.0, phase_mode=WDM_PHASE_PRECISE, batch=1)
        d = Ref(WdmDesc(Nx, Ny, Nz, Lx, Ly, Lz, convention, poisson_coeff, kerr, absorb_coeff, phase_mode, batch))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:wdm_create, libwavedm), Int32, (Ref{WdmDesc}, Ref{Ptr{Cvoid}}), d, h))
        c = new(h[], (Nx, Ny, Nz))
        finalizer(x -> ccall((:wdm_destroy, libwavedm), Int32, (Ptr{Cvoid},), x.h), c)
        c
    end
end

set_psi!(c::Context, psi::CuArray{ComplexF32,3}) =
    check(ccall((:wdm_set_psi, libwavedm), Int32, (Ptr{Cvoid}, CuPtr{ComplexF32}, Int32), c.h, psi, WDM_DEVICE), c.h)
set_psi!(c::Context, psi::Array{ComplexF32,3}) =
    GC.@preserve psi check(ccall((:wdm_set_psi, libwavedm), Int32, (Ptr{Cvoid}, Ptr{ComplexF32}, Int32),
                                 c.h, psi, WDM_HOST), c.h)
get_psi!(psi::CuArray{ComplexF32,3}, c::Context) =
    check(ccall((:wdm_get_psi, libwavedm), Int32, (Ptr{Cvoid}, CuPtr{ComplexF32}, Int32), c.h, psi, WDM_DEVICE), c.h)
get_phi!(phi::CuArray{Float32,3}, c::Context) =
    check(ccall((:wdm_get_phi, libwavedm), Int32, (Ptr{Cvoid}, CuPtr{Float32}, Int32), c.h, phi, WDM_DEVICE), c.h)

"Tidal tensors (Txx, Tyy, Tzz, Txy, Txz, Tyz) for the kicks of the next step call (one row per kick)."
function set_tidal!(c::Context, rows::Matrix{Float64})  # 6 x nrows
    GC.@preserve rows check(ccall((:wdm_set_tidal, libwavedm), Int32, (Ptr{Cvoid}, Ptr{Float64}, Int32, Int32),
                                  c.h, rows, size(rows, 2), 0), c.h)
end

set_particles!(c::Context, pos::Matrix{Float64}, mass::Vector{Float64}) =  # pos: 3 x n
    GC.@preserve pos mass check(ccall((:wdm_set_particles, libwavedm), Int32,
                                      (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64), c.h, pos, mass, length(mass)), c.h)

step!(c::Context, n, dt; t0=0.0, mode=WDM_STEP_STRANG) =
    check(ccall((:wdm_step, libwavedm), Int32, (Ptr{Cvoid}, Int32, Float64, Float64, Int32), c.h, n, dt, t0, mode), c.h)

const WDM_DIAG_FIELDS = 28
"""
The loop diagnostics of SPE3D_waveDM (simulation_main.jl:551-558,641-653) on the
device, one column per halo: mass, rho_max, argmax (0-based flat index), centre
of mass, virial sums, momentum, max|Phi|, max|psi|, the compute_timestep limits,
R, and the radii at p = 0.1:0.1:0.9 about the density maximum (rows 20:28).
"""
function diagnostics(c::Context; batch=1)
    out = zeros(Float64, WDM_DIAG_FIELDS, batch)
    GC.@preserve out check(ccall((:wdm_diagnostics, libwavedm), Int32, (Ptr{Cvoid}, Ptr{Float64}), c.h, out), c.h)
    out
end

# ---------------------------------------------------------------------------
# drop-in operators of src/solver/KDK.jl for the gpu path (state stays in `c`)
# ---------------------------------------------------------------------------
"apply_kick_step! of KDK.jl:37-77: psi <- exp(-i dt (Phi + V + tide)) psi, Phi from |psi|^2."
apply_kick_step!(c::Context, dt, t=0.0) =
    check(ccall((:wdm_kick, libwavedm), Int32, (Ptr{Cvoid}, Float64, Float64), c.h, dt, t), c.h)

"apply_drift_step! of KDK.jl:88-101: psi <- border .* ifft(exp(-i k^2 dt/2) fft(psi))."
apply_drift_step!(c::Context, dt) = check(ccall((:wdm_drift, libwavedm), Int32, (Ptr{Cvoid}, Float64), c.h, dt), c.h)

"parallel_poisson of parallel_poisson.jl:36-68 on device arrays: lap phi = rho - <rho>."
function parallel_poisson!(phi::CuArray{Float32,3}, c::Context, rho::CuArray{Float32,3})
    check(ccall((:wdm_poisson, libwavedm), Int32, (Ptr{Cvoid}, CuPtr{Float32}, CuPtr{Float32}, Int32),
                c.h, rho, phi, WDM_DEVICE), c.h)
    phi
end

# ---------------------------------------------------------------------------
# differentiation: L(psi0, a) = sum (|psi_N|^2 - rho_target)^2 dV for a tide a*D
# ---------------------------------------------------------------------------
function loss_and_gradient(c::Context, psi0::CuArray{ComplexF32,3}, nsteps, dt, rho_target::CuArray{Float32,3};
                           ckpt_every=20, tidal_dir::Union{Nothing,Vector{Float64}}=nothing)
    set_psi!(c, psi0)
    grad = similar(psi0)
    loss = Ref(0.0)
    damp = Ref(0.0)
    d6 = tidal_dir === nothing ? C_NULL : pointer(tidal_dir)
    GC.@preserve tidal_dir check(ccall((:wdm_adjoint, libwavedm), Int32,
        (Ptr{Cvoid}, Int32, Float64, Int32, CuPtr{Float32}, Int32, Ptr{Float64}, CuPtr{ComplexF32}, Int32,
         Ref{Float64}, Ref{Float64}),
        c.h, nsteps, dt, ckpt_every, rho_target, WDM_DEVICE, d6, grad, WDM_DEVICE, loss, damp), c.h)
    loss[], grad, damp[]
end

"Loss of the run from psi0 (the primal of the rrule below)."
function evolve_loss(c::Context, psi0, nsteps, dt, rho_target; kw...)
    loss, _, _ = loss_and_gradient(c, psi0, nsteps, dt, rho_target; kw...)
    loss
end

function ChainRulesCore.rrule(::typeof(evolve_loss), c::Context, psi0, nsteps, dt, rho_target; kw...)
    loss, grad, _ = loss_and_gradient(c, psi0, nsteps, dt, rho_target; kw...)
    # the library's gradient is dL/dRe psi0 + i dL/dIm psi0, ChainRules' convention for complex inputs
    pullback(dl) = (NoTangent(), NoTangent(), dl .* grad, NoTangent(), NoTangent(), NoTangent())
    loss, pullback
end

end # module
