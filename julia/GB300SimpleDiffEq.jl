"""
    GB300SimpleDiffEq

Ensemble solves of SimpleDiffEq.jl's GPU-crutch algorithms on one NVIDIA GB300
through the C ABI of `libgb300ode.so` (`include/gb300ode.h`).

SimpleDiffEq.jl defines `solve(prob::ODEProblem, alg::GPUSimple*)` for one
trajectory (`src/tsit5/gpuatsit5.jl:55-61,205-212`, `src/verner/gpuvern7.jl:55-61,300-307`,
`src/verner/gpuvern9.jl:55-61,411-418`, `src/rk4/gpurk4.jl:53-58`,
`src/euler/gpueuler.jl:53-58`) and no ensemble method; `GPUSimpleATsit5`,
`GPUSimpleAVern7` and `GPUSimpleAVern9` have no supertype.  This module adds
`SciMLBase.solve(::EnsembleProblem, alg::GPUSimple*; trajectories, ...)` for
every one of them (and `SimpleEM` for SDE ensembles): `prob_func` runs on the
host to build the structure-of-arrays inputs, one `ccall` solves the whole
ensemble, and the results come back as an `EnsembleSolution` of
`build_solution`s, as the per-trajectory calls would give.

The struct definitions below mirror `include/gb300ode.h` field for field
(names, order, widths); `tests/test_julia_binding.py` checks them against
the C compiler's `offsetof`/`sizeof`.
"""
module GB300SimpleDiffEq

using SimpleDiffEq, SciMLBase, StaticArrays

export compile_rhs, compile_output, compile_sde, learn_fit!, everystep_solve

const lib = get(ENV, "GB300ODE_LIB", "libgb300ode.so")
const ABI_VERSION = 6

# ----------------------------------------------------------------------------- C structs

# ode_solve_args
struct SolveArgs
    alg::Int32
    rhs::Int32
    precision::Int32
    schedule::Int32
    n::Int64
    dim::Int32
    nparams::Int32
    t0::Float64
    tf::Float64
    dt::Float64
    abstol::Float64
    reltol::Float64
    saveat::Ptr{Float64}
    nsave::Int64
    save_everystep::Int32
    memory::Int32
    maxiters::Int64
    u0::Ptr{Float64}
    p::Ptr{Float64}
    dt0::Ptr{Float64}
    stream::Ptr{Cvoid}
    output::Int32
    layout::Int32
    controller::Int32
end

# ode_solve_out
struct SolveOut
    us::Ptr{Float64}
    u_final::Ptr{Float64}
    t_final::Ptr{Float64}
    retcode::Ptr{Int8}
    naccept::Ptr{Int32}
    nreject::Ptr{Int32}
    dt_first::Ptr{Float64}
end

# ode_solve_stats
struct SolveStats
    kernel_ms::Float64
    total_ms::Float64
    attempts::Int64
    saves::Int64
    launches::Int32
    schedule_used::Int32
    graph_replayed::Int32
    jit::Int32
    kernel::Int32
end

# ode_everystep_out
struct EverystepOut
    offsets::Ptr{Int64}
    ts::Ptr{Float64}
    us::Ptr{Float64}
    capacity::Int64
    total::Int64
    u_final::Ptr{Float64}
    t_final::Ptr{Float64}
    retcode::Ptr{Int8}
    naccept::Ptr{Int32}
    nreject::Ptr{Int32}
end

# ode_sde_args
struct SdeArgs
    sde::Int32
    n::Int64
    dim::Int32
    nparams::Int32
    t0::Float64
    tf::Float64
    dt::Float64
    seed::UInt64
    save_everystep::Int32
    memory::Int32
    u0::Ptr{Float64}
    p::Ptr{Float64}
    stream::Ptr{Cvoid}
    noise_dim::Int32
end

# ode_sde_out
struct SdeOut
    us::Ptr{Float64}
    u_final::Ptr{Float64}
end

# ode_tune_variant
struct TuneVariant
    block::Int32
    max_registers::Int32
    stage_bytes::Int32
    ms::Float32
end

# ode_tune_report
struct TuneReport
    variants::Int32
    block::Int32
    max_registers::Int32
    stage_bytes::Int32
    default_ms::Float64
    best_ms::Float64
    sample::Int64
    tune_ms::Float64
    ntable::Int32
    table::NTuple{64, TuneVariant}
end

# ode_learn_opts
struct LearnOpts
    hidden::Int32
    epochs::Int32
    batch::Int32
    lr::Float32
    seed::UInt64
    seed_dt0::Int32
    dt0_safety::Float32
end

# ode_learn_report
struct LearnReport
    loss_first::Float32
    loss_last::Float32
    r2_attempts::Float32
    train_solve_ms::Float64
    train_fit_ms::Float64
    train_kernel_ms::Float64
    train_ctas::Int32
end

# ----------------------------------------------------------------------------- constants

const ALG_ID = Dict{DataType, Int32}(GPUSimpleRK4 => 0, GPUSimpleTsit5 => 1, GPUSimpleATsit5 => 2,
                                     GPUSimpleVern7 => 3, GPUSimpleAVern7 => 4, GPUSimpleVern9 => 5,
                                     GPUSimpleAVern9 => 6, GPUSimpleEuler => 7)
const GPUSimpleAlg = Union{GPUSimpleRK4, GPUSimpleEuler, GPUSimpleTsit5, GPUSimpleATsit5, GPUSimpleVern7,
                           GPUSimpleAVern7, GPUSimpleVern9, GPUSimpleAVern9}
const AdaptiveAlg = Union{GPUSimpleATsit5, GPUSimpleAVern7, GPUSimpleAVern9}

const RHS_BUILTIN = Dict(:lorenz => 0, :vanderpol => 1, :r3bp => 2, :kuramoto => 3, :linear => 4)
const PRECISION = Dict(:fp64 => 0, :fp32 => 1, :fp32_kahan => 2)
const SCHEDULE = Dict(:plain => 0, :persistent => 1, :learned => 2)
const CONTROLLER = Dict(:ds => 0, :fp64 => 1, :fp32 => 2, :ref => 3)
const SDE_BUILTIN = Dict(:gbm => 0, :ou => 1, :lorenz => 2, :mult => 3)
const ODE_OK, ODE_ETRAJ, ODE_ESMALL = 0, -6, -8
const RET_DTMIN, RET_MAXITERS = 1, 2

# ----------------------------------------------------------------------------- handle

mutable struct Handle
    ptr::Ptr{Cvoid}
    device::Int
end

const HANDLES = Dict{Int, Handle}()

function handle(device::Integer = 0)
    get!(HANDLES, device) do
        v = ccall((:ode_abi_version, lib), Cint, ())
        v == ABI_VERSION || error("libgb300ode ABI version $v, this binding expects $ABI_VERSION")
        p = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:ode_create, lib), Cint, (Ref{Ptr{Cvoid}}, Cint), p, device)
        rc == ODE_OK || error("ode_create failed ($rc)")
        h = Handle(p[], device)
        finalizer(h) do x
            x.ptr == C_NULL || ccall((:ode_destroy, lib), Cvoid, (Ptr{Cvoid},), x.ptr)
            x.ptr = C_NULL
        end
        h
    end
end

lasterr(h::Handle) = unsafe_string(ccall((:ode_last_error, lib), Cstring, (Ptr{Cvoid},), h.ptr))

function check(h::Handle, rc; allow = ())
    rc == ODE_OK || rc in allow || error("libgb300ode: " * lasterr(h) * " ($rc)")
    rc
end

# ----------------------------------------------------------------------------- run-time compiled functions

"""
    compile_rhs(body, dim, nparams; device = 0) -> Int32

The body of `template <class R> __device__ void rhs(R* du, const R* u, const R* p, R t)`
compiled with NVRTC (a Julia closure cannot run in a CUDA kernel); use the id as `rhs`.
"""
function compile_rhs(body::AbstractString, dim::Integer, nparams::Integer; device::Integer = 0)
    h = handle(device)
    id = Ref{Cint}(0)
    log = zeros(UInt8, 16384)
    check(h, ccall((:ode_rhs_compile, lib), Cint, (Ptr{Cvoid}, Cstring, Cint, Cint, Ref{Cint}, Ptr{UInt8}, Csize_t),
                   h.ptr, body, dim, nparams, id, log, length(log)))
    id[]
end

"""
    compile_output(body, dim, nparams, width; device = 0) -> Int32

An ensemble `output_func` compiled into the solver: the body of
`__device__ void output(double* out, const double* u, const double* p, double t)`
writing `width` values per saved point; use the id as `output`.
"""
function compile_output(body::AbstractString, dim::Integer, nparams::Integer, width::Integer; device::Integer = 0)
    h = handle(device)
    id = Ref{Cint}(0)
    log = zeros(UInt8, 16384)
    check(h, ccall((:ode_output_compile, lib), Cint,
                   (Ptr{Cvoid}, Cstring, Cint, Cint, Cint, Ref{Cint}, Ptr{UInt8}, Csize_t),
                   h.ptr, body, dim, nparams, width, id, log, length(log)))
    id[]
end

"""
    compile_sde(drift, diffusion, dim, nparams; noise_dim = 0, device = 0) -> Int32

A user SDE for `SimpleEM` ensembles: bodies of
`__device__ void drift(double* f, const double* u, const double* p, double t)` and
`__device__ void diffusion(double* g, const double* u, const double* p, double t)`
(`g` row-major `dim x noise_dim` for non-diagonal noise).
"""
function compile_sde(drift::AbstractString, diffusion::AbstractString, dim::Integer, nparams::Integer;
                     noise_dim::Integer = 0, device::Integer = 0)
    h = handle(device)
    id = Ref{Cint}(0)
    log = zeros(UInt8, 16384)
    check(h, ccall((:ode_sde_compile_noise, lib), Cint,
                   (Ptr{Cvoid}, Cstring, Cstring, Cint, Cint, Cint, Ref{Cint}, Ptr{UInt8}, Csize_t),
                   h.ptr, drift, diffusion, dim, noise_dim, nparams, id, log, length(log)))
    id[]
end

function rhs_id(h::Handle, rhs, dim, np)
    rhs isa Integer && return Int32(rhs)
    rhs isa AbstractString && return compile_rhs(rhs, dim, np; device = h.device)
    id = Ref{Cint}(0)
    check(h, ccall((:ode_rhs_builtin, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Ref{Cint}, Ptr{Cint}),
                   h.ptr, RHS_BUILTIN[rhs], dim, id, C_NULL))
    id[]
end

output_id(output::Symbol) = output === :state ? Int32(0) : output === :kuramoto_r ? Int32(1) :
                            error("unknown output $output")
output_id(output::Integer) = Int32(output)

# ----------------------------------------------------------------------------- inputs

# prob_func on the host; Julia's column-major n x D matrix is the C [D][n] layout
function soa_inputs(ep::EnsembleProblem, trajectories::Integer)
    probs = [ep.prob_func(deepcopy(ep.prob), i, 1) for i in 1:trajectories]
    D = length(ep.prob.u0)
    P = ep.prob.p === nothing || ep.prob.p isa SciMLBase.NullParameters ? 0 : length(ep.prob.p)
    u0 = Matrix{Float64}(undef, trajectories, D)
    p = Matrix{Float64}(undef, trajectories, max(P, 1))
    for (i, pr) in enumerate(probs)
        u0[i, :] .= pr.u0
        P > 0 && (p[i, :] .= pr.p)
    end
    probs, u0, p, D, P
end

# the saved series come back trajectory-major (ODE_LAYOUT_TRAJ): a Julia W x npts x n array, us[:, j, i]
# the j-th point of trajectory i, as the reference's per-trajectory sol.u
function solve_args(alg, h, rhs, u0, p, D, P, n, tspan, dt, abstol, reltol, sv, save_everystep, precision,
                    schedule, maxiters, output; controller::Symbol = :ds)
    SolveArgs(ALG_ID[typeof(alg)], rhs_id(h, rhs, D, P), PRECISION[precision], SCHEDULE[schedule], n, D, P,
              tspan[1], tspan[2], dt, abstol, reltol, isempty(sv) ? C_NULL : pointer(sv), length(sv),
              save_everystep, 0, maxiters, pointer(u0), pointer(p), C_NULL, C_NULL, output_id(output), 1,
              CONTROLLER[controller])
end

retcode_of(r) = r == RET_MAXITERS ? SciMLBase.ReturnCode.MaxIters : SciMLBase.ReturnCode.Default

# ----------------------------------------------------------------------------- ODE ensembles

"""
    solve(ep::EnsembleProblem, alg::GPUSimple*; trajectories, rhs, dt = 0.1, abstol = 1e-6,
          reltol = 1e-3, saveat = nothing, save_everystep = true, precision = :fp64,
          schedule = :persistent, maxiters = 0, output = :state, controller = :ds, device = 0)

The whole ensemble in one call of `ode_ensemble_solve` (`ode_ensemble_solve_everystep`
for the adaptive algorithms' default every-step output).  `rhs`: `:lorenz`,
`:vanderpol`, `:r3bp`, `:kuramoto`, `:linear`, an id from `compile_rhs`, or the
CUDA C++ body itself.  `controller` picks the error norm and step-size
controller arithmetic of adaptive FP64 solves: `:ds` (default, double-single,
ODE_CTRL_DS), `:fp64` (ODE_CTRL_FP64) or `:fp32` (ODE_CTRL_FP32); `:ref`
(ODE_CTRL_REF, FP64 only) runs the reference's own arithmetic throughout the
solve, fixed-step ones included.  Keyword defaults are the reference's;
`dt < dtmin` raises the reference's `error("dt<dtmin")`.
"""
function SciMLBase.solve(ep::EnsembleProblem, alg::GPUSimpleAlg; trajectories::Integer, rhs,
                         dt = 0.1, abstol = 1.0e-6, reltol = 1.0e-3, saveat = nothing,
                         save_everystep = true, precision::Symbol = :fp64, schedule::Symbol = :persistent,
                         maxiters::Integer = 0, output = :state, controller::Symbol = :ds, device::Integer = 0,
                         kwargs...)
    prob = ep.prob
    @assert !SciMLBase.isinplace(prob)   # as every GPUSimple solve
    h = handle(device)
    probs, u0, p, D, P = soa_inputs(ep, trajectories)
    n = trajectories
    sv = saveat === nothing ? Float64[] : collect(Float64, saveat)
    if isempty(sv) && save_everystep && alg isa AdaptiveAlg
        rows = everystep_solve(h, alg, rhs, u0, p, D, P, n, prob.tspan, dt, abstol, reltol, precision,
                               schedule, maxiters)
        sols = map(1:n) do i
            ts, us, ret = rows[i]
            SciMLBase.build_solution(probs[i], alg, ts, us; retcode = retcode_of(ret), calculate_error = false)
        end
        return SciMLBase.EnsembleSolution(sols, 0.0, true)
    end
    fixed_grid = collect(prob.tspan[1]:dt:prob.tspan[2])
    npts = !isempty(sv) ? length(sv) : (save_everystep && !(alg isa AdaptiveAlg) ? length(fixed_grid) : 0)
    W = output === :kuramoto_r ? 1 : D
    us = Array{Float64}(undef, W, max(npts, 1), n)    # C [n][npts][W] (ODE_LAYOUT_TRAJ)
    uf = Matrix{Float64}(undef, n, D)
    tf = Vector{Float64}(undef, n)
    ret = Vector{Int8}(undef, n)
    args = solve_args(alg, h, rhs, u0, p, D, P, n, prob.tspan, dt, abstol, reltol, sv,
                      save_everystep && !(alg isa AdaptiveAlg), precision, schedule, maxiters, output;
                      controller = controller)
    out = SolveOut(npts == 0 ? C_NULL : pointer(us), pointer(uf), pointer(tf), pointer(ret), C_NULL, C_NULL,
                   C_NULL)
    rc = GC.@preserve sv u0 p us uf tf ret ccall((:ode_ensemble_solve, lib), Cint,
                                                  (Ptr{Cvoid}, Ref{SolveArgs}, Ref{SolveOut}, Ptr{Cvoid}),
                                                  h.ptr, args, out, C_NULL)
    rc == ODE_ETRAJ && any(==(RET_DTMIN), ret) && error("dt<dtmin")   # the reference's exception
    check(h, rc; allow = (ODE_ETRAJ,))
    ts = npts == 0 ? [prob.tspan[1], prob.tspan[2]] : (isempty(sv) ? fixed_grid : sv)
    sols = map(1:n) do i
        u = npts == 0 ? [SVector{D}(u0[i, :]), SVector{D}(uf[i, :])] : [SVector{W}(view(us, :, j, i)) for j in 1:npts]
        SciMLBase.build_solution(probs[i], alg, ts, u; retcode = retcode_of(ret[i]), calculate_error = false)
    end
    SciMLBase.EnsembleSolution(sols, 0.0, true)
end

"""
    everystep_solve(h, alg, rhs, u0, p, D, P, n, tspan, dt, abstol, reltol, precision, schedule, maxiters)

Ragged every-step output of the adaptive solvers: one call counts each trajectory's
accepted steps (ODE_ESMALL reports the total), a second fills the rows.  Returns
`(ts, us, retcode)` per trajectory.
"""
function everystep_solve(h::Handle, alg, rhs, u0, p, D, P, n, tspan, dt, abstol, reltol, precision, schedule,
                         maxiters)
    sv = Float64[]
    args = solve_args(alg, h, rhs, u0, p, D, P, n, tspan, dt, abstol, reltol, sv, false, precision, schedule,
                      maxiters, :state)
    off = Vector{Int64}(undef, n + 1)
    ret = Vector{Int8}(undef, n)
    o = Ref(EverystepOut(pointer(off), C_NULL, C_NULL, 0, 0, C_NULL, C_NULL, pointer(ret), C_NULL, C_NULL))
    rc = GC.@preserve u0 p off ret ccall((:ode_ensemble_solve_everystep, lib), Cint,
                                         (Ptr{Cvoid}, Ref{SolveArgs}, Ref{EverystepOut}, Ptr{Cvoid}),
                                         h.ptr, args, o, C_NULL)
    check(h, rc; allow = (ODE_ESMALL, ODE_ETRAJ))
    total = o[].total
    ts = Vector{Float64}(undef, total)
    us = Matrix{Float64}(undef, D, total)     # C [rows][D]: row r is us[:, r]
    o = Ref(EverystepOut(pointer(off), pointer(ts), pointer(us), total, 0, C_NULL, C_NULL, pointer(ret), C_NULL,
                         C_NULL))
    rc = GC.@preserve u0 p off ts us ret ccall((:ode_ensemble_solve_everystep, lib), Cint,
                                               (Ptr{Cvoid}, Ref{SolveArgs}, Ref{EverystepOut}, Ptr{Cvoid}),
                                               h.ptr, args, o, C_NULL)
    rc == ODE_ETRAJ && any(==(RET_DTMIN), ret) && error("dt<dtmin")
    check(h, rc; allow = (ODE_ETRAJ,))
    [(ts[off[i]+1:off[i+1]], [SVector{D}(us[:, r]) for r in off[i]+1:off[i+1]], ret[i]) for i in 1:n]
end

# ----------------------------------------------------------------------------- learned schedule

"""
    learn_fit!(ep, alg; trajectories, rhs, dt, abstol, reltol, hidden = 64, epochs = 30,
               batch = 1024, lr = 5e-3, seed = 1, seed_dt0 = false, device = 0) -> LearnReport

Solve the training ensemble `ep` and fit the cost model that `schedule = :learned` uses.
"""
function learn_fit!(ep::EnsembleProblem, alg::AdaptiveAlg; trajectories::Integer, rhs, dt = 0.1,
                    abstol = 1.0e-6, reltol = 1.0e-3, precision::Symbol = :fp64, hidden::Integer = 64,
                    epochs::Integer = 30, batch::Integer = 1024, lr::Real = 5.0e-3, seed::Integer = 1,
                    seed_dt0::Bool = false, dt0_safety::Real = 1.0, device::Integer = 0)
    h = handle(device)
    _, u0, p, D, P = soa_inputs(ep, trajectories)
    args = solve_args(alg, h, rhs, u0, p, D, P, trajectories, ep.prob.tspan, dt, abstol, reltol, Float64[], false,
                      precision, :plain, 0, :state)
    opts = LearnOpts(hidden, epochs, batch, lr, seed, seed_dt0, dt0_safety)
    rep = Ref{LearnReport}()
    GC.@preserve u0 p check(h, ccall((:ode_learn_fit, lib), Cint,
                                     (Ptr{Cvoid}, Ref{SolveArgs}, Ref{LearnOpts}, Ref{LearnReport}),
                                     h.ptr, args, opts, rep))
    rep[]
end

# ----------------------------------------------------------------------------- SimpleEM ensembles

"""
    solve(ep::EnsembleProblem{<:SDEProblem}, alg::SimpleEM; trajectories, sde, dt, seed = 1,
          save_everystep = true, noise_dim = 0, device = 0)

`SimpleEM` (`src/euler_maruyama.jl:48-142`) for the whole ensemble.  `sde`: `:gbm`,
`:ou`, `:lorenz`, `:mult` or an id from `compile_sde`; `noise_dim` =
`size(noise_rate_prototype, 2)` for non-diagonal noise.  The noise is a
Philox4x32-10 stream keyed by `seed`: statistics agree with `randn`, single paths do not.
"""
function SciMLBase.solve(ep::EnsembleProblem{<:SDEProblem}, alg::SimpleEM; trajectories::Integer, sde, dt,
                         seed::Integer = 1, save_everystep::Bool = true, noise_dim::Integer = 0,
                         device::Integer = 0, kwargs...)
    h = handle(device)
    probs, u0, p, D, P = soa_inputs(ep, trajectories)
    n = trajectories
    t0, t1 = ep.prob.tspan
    npts = Int((t1 - t0) / dt) + 1
    us = Array{Float64}(undef, n, D, save_everystep ? npts : 1)
    uf = Matrix{Float64}(undef, n, D)
    id = sde isa Integer ? Int32(sde) : Int32(SDE_BUILTIN[sde])
    args = SdeArgs(id, n, D, P, t0, t1, dt, seed, save_everystep, 0, pointer(u0), pointer(p), C_NULL, noise_dim)
    out = SdeOut(save_everystep ? pointer(us) : C_NULL, pointer(uf))
    GC.@preserve u0 p us uf check(h, ccall((:ode_sde_solve, lib), Cint,
                                           (Ptr{Cvoid}, Ref{SdeArgs}, Ref{SdeOut}, Ptr{Cvoid}),
                                           h.ptr, args, out, C_NULL))
    ts = save_everystep ? [t0 + k * dt for k in 0:npts-1] : [t1]   # the grid of SimpleEM
    sols = map(1:n) do i
        u = save_everystep ? [SVector{D}(us[i, :, j]) for j in 1:npts] : [SVector{D}(uf[i, :])]
        SciMLBase.build_solution(probs[i], alg, ts, u; calculate_error = false)
    end
    SciMLBase.EnsembleSolution(sols, 0.0, true)
end

end # module
