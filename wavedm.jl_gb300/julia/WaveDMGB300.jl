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
using JLD2

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

"""
Tidal tensors (Txx, Tyy, Tzz, Txy, Txz, Tyz), one column per row of the
schedule.  Without `t_step` column s is used by kick s of every following
step! call; with `t_step` column s is the tensor at time t_first + s t_step and
each kick takes the column nearest to its own time (wdm_set_tidal_clock).
"""
function set_tidal!(c::Context, rows::Matrix{Float64}; t_first=0.0, t_step=nothing)  # 6 x nrows
    GC.@preserve rows check(ccall((:wdm_set_tidal, libwavedm), Int32, (Ptr{Cvoid}, Ptr{Float64}, Int32, Int32),
                                  c.h, rows, size(rows, 2), 0), c.h)
    t_step === nothing || check(ccall((:wdm_set_tidal_clock, libwavedm), Int32, (Ptr{Cvoid}, Float64, Float64),
                                      c.h, t_first, t_step), c.h)
    nothing
end

const WDM_TIDE_BOX_CENTRE, WDM_TIDE_REFERENCE, WDM_TIDE_DENSITY_MAX = Int32(0), Int32(1), Int32(2)
const TIDE_CENTERING = Dict(:box_centre => WDM_TIDE_BOX_CENTRE, :reference => WDM_TIDE_REFERENCE,
                            :density_max => WDM_TIDE_DENSITY_MAX)

"""
Where the tide is anchored (src/physics/tidal_fields.jl:114-146): :box_centre,
:reference (its value at the density maximum removed, as that code leaves the
potential) or :density_max (value and gradient removed there).
"""
set_tidal_centering!(c::Context, mode::Symbol) =
    check(ccall((:wdm_set_tidal_centering, libwavedm), Int32, (Ptr{Cvoid}, Int32), c.h, TIDE_CENTERING[mode]), c.h)

set_static_potential!(c::Context, V::Array{Float32,3}) =
    GC.@preserve V check(ccall((:wdm_set_static_potential, libwavedm), Int32, (Ptr{Cvoid}, Ptr{Float32}, Int32),
                               c.h, V, WDM_HOST), c.h)
get_psi!(psi::Array{ComplexF32,3}, c::Context) =
    GC.@preserve psi check(ccall((:wdm_get_psi, libwavedm), Int32, (Ptr{Cvoid}, Ptr{ComplexF32}, Int32),
                                 c.h, psi, WDM_HOST), c.h)
get_phi!(phi::Array{Float32,3}, c::Context) =
    GC.@preserve phi check(ccall((:wdm_get_phi, libwavedm), Int32, (Ptr{Cvoid}, Ptr{Float32}, Int32),
                                 c.h, phi, WDM_HOST), c.h)

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

"""
Loss of the run from psi0 under the tide a * tidal_dir (the primal of the rrule
below).  Gradients with respect to parameters of the initial condition (the
soliton core radius rc, for instance) follow from the psi0 cotangent by the
chain rule through the Julia code that builds psi0.
"""
function evolve_loss(c::Context, psi0, a::Real, nsteps, dt, rho_target; tidal_dir::Vector{Float64}, kw...)
    set_tidal!(c, reshape(a .* tidal_dir, 6, 1))
    loss, _, _ = loss_and_gradient(c, psi0, nsteps, dt, rho_target; tidal_dir=tidal_dir, kw...)
    loss
end

function ChainRulesCore.rrule(::typeof(evolve_loss), c::Context, psi0, a::Real, nsteps, dt, rho_target;
                              tidal_dir::Vector{Float64}, kw...)
    set_tidal!(c, reshape(a .* tidal_dir, 6, 1))
    loss, grad, damp = loss_and_gradient(c, psi0, nsteps, dt, rho_target; tidal_dir=tidal_dir, kw...)
    # the library's gradient is dL/dRe psi0 + i dL/dIm psi0, ChainRules' convention
    # for complex inputs; damp is dL/da for the amplitude of the tide
    pullback(dl) = (NoTangent(), NoTangent(), dl .* grad, dl * damp, NoTangent(), NoTangent(), NoTangent())
    loss, pullback
end

# ---------------------------------------------------------------------------
# the gpu=true solver entry of SPE3D_waveDM (src/simulation_main.jl:41-1064)
# ---------------------------------------------------------------------------
"""
    SPE3D_waveDM(; gpu=true, Nx, Ny, Nz, Xmax, Ymax, Zmax, Nt, Tmax, IC, kw...)

The gpu=true path of WaveDM.jl's solver entry with its keyword arguments for the
split-step loop.  The loop of src/simulation_main.jl:536-559 runs inside the
library: `StepsBetweenSnapshots` steps per wdm_step call (the literal
K(dt/2) D(dt) iteration when KDK_flag is true, as the reference's loop does;
`mode = WDM_STEP_STRANG` for the symmetric form), then the loop diagnostics of
:551-558 and :641-653 on the device (wdm_diagnostics), once per snapshot.

* `IC(x, y, z)` is broadcast over the reference grid x = LinRange(-Xmax, Xmax, Nx)
  (src/physics/poisson.jl:8-15) as setup_initial_conditions does; an array
  `IC[x, y, z]` is taken as is.
* `dt = Float32(Tmax / Nt)` (src/physics/poisson.jl:47); step i runs at time (i-1) dt.
* `V`: nothing or a static Float32 array; a closure V(x, y, z, psi) cannot run in
  the kernels (KDK.jl:64 evaluates it on the host every step) and throws.
* `kappa`: the local term kappa |psi|^2; `absorb_coeff`: the tanh absorbing mask.
* `tidal`: a function t -> (Txx, Tyy, Tzz, Txy, Txz, Tyz) of the tidal tensor,
  sampled once per step on a clocked schedule; `tidal_centering` as set_tidal_centering!.
* `particles`: (pos 3 x n, mass n) static baryons, CIC-deposited once and added to the
  density of every Poisson solve.
* `outputdir`: writes "<title>, <suffix> - Prop.jld2" with the keys of
  save_evolution_results (src/io/save.jl:25-34) through JLD2, and the property
  table "<title>, <suffix> - Prop.csv" (src/io/save.jl:41-72).

Returns a NamedTuple (ψ, Φ_all, t, dt, Prop) with ψ and Φ_all on the host in the
reference's [x, y, z] layout and Prop one NamedTuple of diagnostics per snapshot.
"""
function SPE3D_waveDM(; gpu::Bool=true, Nx::Integer=64, Ny::Integer=Nx, Nz::Integer=Nx, Xmax=10.0, Ymax=Xmax,
                      Zmax=Xmax, Nt::Integer=100, Tmax=1.0, IC, V=nothing, KDK_flag::Bool=true, absorb_coeff=0.0,
                      kappa=0.0, poisson_coeff=4π, StepsBetweenSnapshots::Integer=Nt - 1, tidal=nothing,
                      tidal_centering::Symbol=:box_centre, particles=nothing, phase_mode=WDM_PHASE_PRECISE,
                      mode=nothing, outputdir=nothing, title="WaveDM", suffix="GB300", uL=1.0)
    gpu || throw(ArgumentError("libwavedm is the gpu=true path; there is no CPU path"))
    V isa Function && throw(ArgumentError("a potential closure V(x, y, z, ψ) cannot run on the GPU path: pass " *
                                          "nothing, a static Float32 array, or kappa for kappa |ψ|^2"))
    x = LinRange(-Xmax, Xmax, Nx)
    y = LinRange(-Ymax, Ymax, Ny)
    z = LinRange(-Zmax, Zmax, Nz)
    ψ0 = IC isa AbstractArray ? ComplexF32.(IC) :
         ComplexF32.(IC.(reshape(x, Nx, 1, 1), reshape(y, 1, Ny, 1), reshape(z, 1, 1, Nz)))
    dt = Float32(Tmax / Nt)
    t = LinRange(0, Tmax, Nt)
    step_mode = mode === nothing ? (KDK_flag ? WDM_STEP_REFERENCE_LOOP : WDM_STEP_LIE) : Int32(mode)
    c = Context(Nx, Ny, Nz, 2Xmax, 2Ymax, 2Zmax; convention=WDM_GRID_REFERENCE, poisson_coeff=poisson_coeff,
                kerr=kappa, absorb_coeff=absorb_coeff, phase_mode=phase_mode)
    set_psi!(c, Array{ComplexF32,3}(ψ0))
    V === nothing || set_static_potential!(c, Array{Float32,3}(V))
    particles === nothing || set_particles!(c, Matrix{Float64}(particles[1]), Vector{Float64}(particles[2]))
    if tidal !== nothing
        rows = reduce(hcat, [collect(Float64, tidal(s * dt)) for s in 0:Nt-1])
        set_tidal!(c, rows; t_first=0.0, t_step=Float64(dt))
        set_tidal_centering!(c, tidal_centering)
    end
    names = (:mass, :rho_max, :argmax, :cm_x, :cm_y, :cm_z, :VirialPotential, :TotalKineticE, :TotalQuantumE,
             :Virial, :MomentumX, :MomentumY, :MomentumZ, :max_abs_Phi, :max_abs_psi, :dt_phase, :dt_grav, :dt_si,
             :R, :R1, :R2, :R3, :R4, :R5, :R6, :R7, :R8, :R9)
    prop = NamedTuple[]
    ψ_last_t = nothing
    done = 0
    while done < Nt - 1
        n = min(StepsBetweenSnapshots, Nt - 1 - done)
        if outputdir !== nothing && done + n == Nt - 1
            # the state one step before the end (ψ_last_t of the reference loop)
            n > 1 && step!(c, n - 1, Float64(dt); t0=done * dt, mode=step_mode)
            ψ_last_t = Array{ComplexF32,3}(undef, Nx, Ny, Nz)
            get_psi!(ψ_last_t, c)
            step!(c, 1, Float64(dt); t0=(done + n - 1) * dt, mode=step_mode)
        else
            step!(c, n, Float64(dt); t0=done * dt, mode=step_mode)
        end
        done += n
        d = diagnostics(c)[:, 1]
        push!(prop, merge((t=done * dt,), NamedTuple{names}(Tuple(d))))
    end
    ψ = Array{ComplexF32,3}(undef, Nx, Ny, Nz)
    get_psi!(ψ, c)
    Φ_all = Array{Float32,3}(undef, Nx, Ny, Nz)
    get_phi!(Φ_all, c)
    if outputdir !== nothing
        save_evolution_results(ψ, Φ_all, ψ_last_t, outputdir, title, suffix)
        save_property_table(prop, outputdir, title, suffix; uL=uL)
    end
    (ψ=ψ, Φ_all=Φ_all, t=t, dt=dt, Prop=prop)
end

"The final state with the keys of save_evolution_results (src/io/save.jl:25-34), through JLD2."
function save_evolution_results(ψ, Φ_all, ψ_last_t, outputdir, title, suffix)
    JLD2.jldsave(joinpath(outputdir, "$(title), $(suffix) - Prop.jld2");
                 ψ=ψ, Φ_all=Φ_all, ψ_last_t=ψ_last_t, ψ2_averaged=nothing)
end

"The property table of save_property_dataframe (src/io/save.jl:41-72), as plain CSV."
function save_property_table(prop, outputdir, title, suffix; uL=1.0)
    cols = (:t, :R, :R1, :R2, :R3, :R4, :R5, :R6, :R7, :R8, :R9, :TotalMass, :PE_abs, :KE, :QE, :Virial,
            :MomentumX, :MomentumY, :MomentumZ)
    open(joinpath(outputdir, "$(title), $(suffix) - Prop.csv"), "w") do io
        println(io, join(string.(cols), ","))
        for r in prop
            row = (r.t, r.R * uL, r.R1 * uL, r.R2 * uL, r.R3 * uL, r.R4 * uL, r.R5 * uL, r.R6 * uL, r.R7 * uL,
                   r.R8 * uL, r.R9 * uL, r.mass, r.VirialPotential, r.TotalKineticE, r.TotalQuantumE, r.Virial,
                   r.MomentumX, r.MomentumY, r.MomentumZ)
            println(io, join(string.(row), ","))
        end
    end
end

end # module
