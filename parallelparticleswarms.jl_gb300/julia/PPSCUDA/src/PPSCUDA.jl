"""
    PPSCUDA

ParallelParticleSwarms.jl's kernels on one GB300 through `libpps_cuda.so` (the C ABI of
`include/pps.h`).  The reference picks its device through the algorithm's `backend` field
(`src/algorithms.jl:78-85,115-121`); this package adds one backend value, `PPSBackend()`, and
routes the swarm's life cycle to the library:

  - `init(prob, alg)` with `alg.backend isa PPSBackend` builds a `PPSSwarm` (the device state)
    instead of `KernelAbstractions.allocate` (`src/init.jl:98-100`);
  - `solve!` runs `pps_sync_run` (`ParallelSyncPSOKernel`), `pps_queue_run`
    (`ParallelPSOKernel(global_update = true)`) or `pps_async_run` (`global_update = false`) and
    builds the reference's solution: `u`, `f(u, p)`, `original` = the positions (`src/solve.jl:11-59`);
  - HybridPSO's local stage, ode_pso fits, many solves (batches, the server) and sharded swarms
    have functions of their own below.

The objective crosses the ABI as an id of the engine's registry (`objective_id`) or as CUDA C
source registered once (`register_objective`).

Load with `PPSCUDA.set_library!(path)` when `libpps_cuda.so` is not next to this file.
"""
module PPSCUDA

using ParallelParticleSwarms, StaticArrays, SciMLBase

const LIB = Ref{String}(joinpath(@__DIR__, "..", "..", "..", "lib", "libpps_cuda.so"))
set_library!(path::AbstractString) = (LIB[] = String(path); nothing)
lib() = LIB[]

struct PPSBackend end

# pps_problem (include/pps.h)
struct PPSProblem
    objective::Int32
    dim::Int32
    lb::Ptr{Float32}
    ub::Ptr{Float32}
    u0::Ptr{Float32}
    params::Ptr{Float32}
    nparams::Int32
    data::Ptr{Float32}
    ndata::Int64
    ncons::Int32
    cons::Ptr{Float32}
end

# pps_local_opts
struct PPSLocalOpts
    history::Int32
    maxiters::Int32
    armijo_c1::Float32
    gtol::Float32
    max_backtracks::Int32
end

# pps_swarm_info
struct PPSSwarmInfo
    n::Int64
    dim::Int32
    objective::Int32
    iteration::UInt32
    async_lanes::Int32
    async_slice::Int32
    device::Int32
    seed::UInt64
    device_bytes::UInt64
end

# pps_serve_stats
struct PPSServeStats
    submitted::UInt64
    completed::UInt64
    launches::UInt64
    solves_per_s::Float64
    p50_ms::Float64
    p99_ms::Float64
    mean_ms::Float64
    max_ms::Float64
    mean_pack::Float64
    arena_bytes::UInt64
    arena_peak_bytes::UInt64
    queued::Int32
    running::Int32
end

# pps_device_swarm: a swarm in device buffers the caller owns (device pointers, e.g.
# reinterpret(Ptr{Float32}, pointer(a)) of a CUDA.jl CuArray a)
struct PPSDeviceSwarm
    n::Int64
    ld::Int64
    dim::Int32
    x::Ptr{Float32}
    v::Ptr{Float32}
    pbest::Ptr{Float32}
    pcost::Ptr{Float32}
    cost::Ptr{Float32}
    lb::Ptr{Float32}
    ub::Ptr{Float32}
    g::Ptr{Float32}
end

# pps_serve_config
struct PPSServeConfig
    memory_budget::UInt64
    max_launches::Int32
    max_pack::Int32
    threads::Int32
    ppt::Int32
    tick_us::Float64
    single_min_n::Int32
    ode_single_min_n::Int32
end

const SAMPLER_AUTO, SAMPLER_UNIFORM, SAMPLER_UNBOUNDED, SAMPLER_LHS = Int32(0), Int32(1), Int32(2), Int32(3)
const FIELD_POSITION, FIELD_VELOCITY, FIELD_PBEST, FIELD_PCOST, FIELD_COST = Int32.(0:4)
const LAYOUT_SOA, LAYOUT_AOS = Int32(0), Int32(1)

function check(rc::Integer)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:pps_last_error, lib()), Cstring, ()))
    rc == 1 ? throw(ArgumentError(msg)) : error("libpps_cuda.so status $rc: $msg")
end

# ---------------------------------------------------------------- library
"""The C ABI version the library implements (this package is written against 100)."""
version() = ccall((:pps_version, lib()), Int32, ())
function device_count()
    n = Ref{Int32}(0)
    check(ccall((:pps_device_count, lib()), Cint, (Ref{Int32},), n))
    return Int(n[])
end
"""Make `device` current for this thread: swarms are created on the current device (the
reference picks it through its backend object)."""
set_device!(device::Integer) = check(ccall((:pps_set_device, lib()), Cint, (Int32,), device))

# ---------------------------------------------------------------- objectives
# Registered objectives: Julia functions the user marks with their engine id.
const REGISTRY = IdDict{Any, Int32}()
register!(f, id::Integer) = (REGISTRY[f] = Int32(id); f)

"""Register `source` (CUDA C defining `pps_objective`, see include/pps.h) and return its id."""
function register_objective(source::AbstractString)
    id = Ref{Int32}(0)
    check(ccall((:pps_objective_register, lib()), Cint, (Cstring, Ref{Int32}), source, id))
    return id[]
end

objective_id(f) = haskey(REGISTRY, f) ? REGISTRY[f] :
                  error("objective $f is not registered with PPSCUDA (register! or register_objective)")

"""A PPSProblem and the Float32 arrays it points into (keep them alive while the library reads them)."""
function pps_problem(prob; data = nothing, cons = nothing)
    D = length(prob.u0)
    lb = Float32.(prob.lb === nothing ? fill(-Inf32, D) : collect(prob.lb))
    ub = Float32.(prob.ub === nothing ? fill(Inf32, D) : collect(prob.ub))
    u0 = Float32.(collect(prob.u0))
    p = prob.p === nothing || prob.p isa SciMLBase.NullParameters ? Float32[] : Float32.(collect(prob.p))
    d = data === nothing ? Float32[] : Float32.(vec(data))
    c = cons === nothing ? Float32[] : Float32.(vec(permutedims(cons)))   # rows (c_k, a_k, b_k)
    ncons = cons === nothing ? 0 : size(cons, 1)
    cp = PPSProblem(objective_id(prob.f.f), D, pointer(lb), pointer(ub), pointer(u0),
                    isempty(p) ? C_NULL : pointer(p), length(p),
                    isempty(d) ? C_NULL : pointer(d), length(d), ncons, isempty(c) ? C_NULL : pointer(c))
    return cp, (lb, ub, u0, p, d, c)
end

# ---------------------------------------------------------------- swarms
mutable struct PPSSwarm
    h::Ptr{Cvoid}
    n::Int
    dim::Int
end

function PPSSwarm(prob, n::Integer; seed::Integer = 0, cpu_backend_gbest::Bool = false,
                  sampler::Int32 = SAMPLER_AUTO, kw...)
    cp, bufs = pps_problem(prob; kw...)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve bufs begin
        check(ccall((:pps_swarm_create, lib()), Cint, (Ref{PPSProblem}, Int64, UInt64, UInt32, Ref{Ptr{Cvoid}}),
                    cp, n, seed, cpu_backend_gbest ? UInt32(1) : UInt32(0), out))
    end
    s = PPSSwarm(out[], Int(n), length(prob.u0))
    finalizer(x -> ccall((:pps_swarm_destroy, lib()), Cint, (Ptr{Cvoid},), x.h), s)
    reinit!(s; sampler)
    return s
end

"""reinit! (src/init.jl:117-141): resample the particles and select the global best."""
reinit!(s::PPSSwarm; sampler::Int32 = SAMPLER_AUTO) = check(ccall((:pps_swarm_init, lib()), Cint,
                                                                   (Ptr{Cvoid}, Int32), s.h, sampler))

function gbest(s::PPSSwarm)
    u = Vector{Float32}(undef, s.dim)
    cost = Ref{Float32}()
    idx = Ref{Int64}()
    check(ccall((:pps_get_gbest, lib()), Cint, (Ptr{Cvoid}, Ptr{Float32}, Ref{Float32}, Ref{Int64}),
                s.h, u, cost, idx))
    return ParallelParticleSwarms.SPSOGBest(SVector{s.dim}(u), cost[]), idx[]
end

"""Every particle's position as the reference's `Vector{SVector{D}}` (`get_pos.(particles)`)."""
function positions(s::PPSSwarm)
    x = Matrix{Float32}(undef, s.n, s.dim)                 # column d holds dim d of every particle (SoA)
    check(ccall((:pps_get_state, lib()), Cint, (Ptr{Cvoid}, Int32, Ptr{Float32}), s.h, FIELD_POSITION, x))
    return [SVector{s.dim}(view(x, i, :)) for i in 1:(s.n)]
end

"""One state field (FIELD_POSITION, _VELOCITY, _PBEST: n x dim; FIELD_PCOST, _COST: n) from the
device, or written to it with `set_state!` (e.g. reinit! from given velocities)."""
function state(s::PPSSwarm, field::Int32)
    out = field in (FIELD_PCOST, FIELD_COST) ? Vector{Float32}(undef, s.n) : Matrix{Float32}(undef, s.n, s.dim)
    check(ccall((:pps_get_state, lib()), Cint, (Ptr{Cvoid}, Int32, Ptr{Float32}), s.h, field, out))
    return out
end
function set_state!(s::PPSSwarm, field::Int32, values::AbstractArray{<:Real})
    v = Array{Float32}(values)
    length(v) == (field in (FIELD_PCOST, FIELD_COST) ? s.n : s.n * s.dim) ||
        throw(DimensionMismatch("field $field of this swarm has $(field in (FIELD_PCOST, FIELD_COST) ? s.n : s.n * s.dim) values"))
    check(ccall((:pps_set_state, lib()), Cint, (Ptr{Cvoid}, Int32, Ptr{Float32}), s.h, field, v))
    return s
end

"""The swarm as the reference's particle records, `Vector{SPSOParticle}` (3 D + 2 floats each)."""
function particles(s::PPSSwarm)
    D = s.dim
    T = ParallelParticleSwarms.SPSOParticle{SVector{D, Float32}, Float32}
    v = Vector{T}(undef, s.n)
    GC.@preserve v check(ccall((:pps_get_particles, lib()), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}),
                               s.h, LAYOUT_AOS, pointer(v)))
    return v
end

function set_particles!(s::PPSSwarm, v::Vector{<:ParallelParticleSwarms.SPSOParticle})
    length(v) == s.n || throw(DimensionMismatch("expected $(s.n) particles"))
    GC.@preserve v check(ccall((:pps_set_particles, lib()), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}),
                               s.h, LAYOUT_AOS, pointer(v)))
    return s
end

"""vectorized_solve! on the engine: maxiters iterations of the algorithm's kind."""
function run!(s::PPSSwarm, opt; maxiters = 100, w = 0.7298f0, wdamp = 1.0f0, c1 = 1.4962f0, c2 = 1.4962f0)
    fn = opt isa ParallelSyncPSOKernel ? :pps_sync_run :
         (opt isa ParallelPSOKernel && opt.global_update) ? :pps_queue_run : :pps_async_run
    ms = Ref{Float32}(0)
    if fn === :pps_sync_run
        check(ccall((:pps_sync_run, lib()), Cint, (Ptr{Cvoid}, Int32, Float32, Float32, Float32, Float32,
                                                   Ref{Float32}), s.h, maxiters, w, wdamp, c1, c2, ms))
    elseif fn === :pps_queue_run
        check(ccall((:pps_queue_run, lib()), Cint, (Ptr{Cvoid}, Int32, Float32, Float32, Float32, Float32,
                                                    Ref{Float32}), s.h, maxiters, w, wdamp, c1, c2, ms))
    else
        check(ccall((:pps_async_run, lib()), Cint, (Ptr{Cvoid}, Int32, Float32, Float32, Float32, Float32,
                                                    Ref{Float32}), s.h, maxiters, w, wdamp, c1, c2, ms))
    end
    return ms[]
end

"""Size, dimension, iterations run, seed and device bytes of a swarm (the cache's fields)."""
function info(s::PPSSwarm)
    r = Ref{PPSSwarmInfo}()
    check(ccall((:pps_swarm_info_get, lib()), Cint, (Ptr{Cvoid}, Ref{PPSSwarmInfo}), s.h, r))
    return r[]
end

"""The problem's objective at the rows of `X` (npoints x dim) on the device: prob.f(x, p) of a
registered objective (src/solve.jl:54-57)."""
function evaluate(prob, X::AbstractMatrix{<:Real})
    cp, bufs = pps_problem(prob)
    x = Matrix{Float32}(X)  # column-major npoints x dim = the dim-major layout of pps_eval_objective
    f = Vector{Float32}(undef, size(x, 1))
    GC.@preserve bufs x f check(ccall((:pps_eval_objective, lib()), Cint,
                                      (Ref{PPSProblem}, Int64, Ptr{Float32}, Ptr{Float32}),
                                      cp, size(x, 1), x, f))
    return f
end

"""The synchronous run on device buffers the caller owns, for callers that cannot let the
library allocate (CUDA.jl's pooled memory): `ds` describes them, `iteration` is the counter of
the first step (0 after an init; add maxiters per call).  Returns (gcost, gidx) after waiting
for `stream` (a CuStream's handle, or C_NULL for the default stream).  Calls share the
library's static scratch (at most 2^20 particles) and must not overlap on the GPU."""
function sync_run_noalloc!(objective::Integer, params::Vector{Float32}, ds::PPSDeviceSwarm; seed = 0,
                           iteration = 0, maxiters = 100, w = 0.7298f0, wdamp = 1.0f0, c1 = 1.4962f0,
                           c2 = 1.4962f0, gbest_from_position = false, stream::Ptr{Cvoid} = C_NULL)
    gcost, gidx = Ref{Float32}(), Ref{Int64}()
    check(ccall((:pps_sync_run_noalloc, lib()), Cint,
                (Int32, Ptr{Float32}, Int32, Ref{PPSDeviceSwarm}, UInt64, UInt32, Int32, Float32, Float32, Float32,
                 Float32, UInt32, Ptr{Cvoid}, Ref{Float32}, Ref{Int64}),
                objective, params, length(params), ds, seed, iteration, maxiters, w, wdamp, c1, c2,
                gbest_from_position ? UInt32(1) : UInt32(0), stream, gcost, gidx))
    return gcost[], gidx[]
end

"""solve(prob, alg) with alg.backend isa PPSBackend: the reference's solution fields (src/solve.jl:11-59)."""
function solve_pps(prob, opt; maxiters = 100, seed = 0, kwargs...)
    s = PPSSwarm(prob, opt.num_particles; seed)
    t0 = time()
    run!(s, opt; maxiters, kwargs...)
    t1 = time()
    g, _ = gbest(s)
    return SciMLBase.build_solution(SciMLBase.DefaultOptimizationCache(prob.f, prob.p), opt,
                                    g.position, prob.f(g.position, prob.p), original = positions(s),
                                    stats = SciMLBase.OptimizationStats(; time = t1 - t0))
end

# ---------------------------------------------------------------- HybridPSO local stage
"""HybridPSO's local stage on every particle (src/hybrid.jl:15-158): `:lbfgs` from the personal
bests or `:bfgs` (Broyden) from the positions.  Returns (u, f, index)."""
function local_stage!(s::PPSSwarm, kind::Symbol = :lbfgs; history = 10, maxiters = 50, armijo_c1 = 1f-4,
                      gtol = 1f-5, max_backtracks = 30)
    o = PPSLocalOpts(history, maxiters, armijo_c1, gtol, max_backtracks)
    u = Vector{Float32}(undef, s.dim)
    f = Ref{Float32}()
    idx = Ref{Int64}()
    ms = Ref{Float32}()
    if kind === :lbfgs
        check(ccall((:pps_hybrid_lbfgs, lib()), Cint, (Ptr{Cvoid}, Ref{PPSLocalOpts}, Ptr{Float32}, Ref{Float32},
                                                       Ref{Int64}, Ref{Float32}), s.h, o, u, f, idx, ms))
    else
        check(ccall((:pps_hybrid_bfgs, lib()), Cint, (Ptr{Cvoid}, Ref{PPSLocalOpts}, Ptr{Float32}, Ref{Float32},
                                                      Ref{Int64}, Ref{Float32}), s.h, o, u, f, idx, ms))
    end
    return SVector{s.dim}(u), f[], idx[]
end

# ---------------------------------------------------------------- ode_pso
"""The fit configuration p of an ODE fit (objective 4 = Lotka-Volterra, 5 = FitzHugh-Nagumo):
RK4 with a save every `save_every` steps, Tsit5 at a fixed step (`parameter_estim_ode!(...,
Val(false))`) or with adaptive steps from `dt` (`Val(true)`, reltol / abstol), saves at
multiples of `save_dt`."""
function ode_params(u0, dt; method::Symbol = :rk4, nsteps = 0, save_every = 1, l = 0.0f0, save_dt = 0.0f0,
                    reltol = 1f-3, abstol = 1f-6)
    method === :rk4 && return Float32[u0[1], u0[2], dt, nsteps, save_every, l]
    method === :tsit5 && return Float32[u0[1], u0[2], dt, nsteps, save_every, l, 1, save_dt]
    method === :tsit5_adaptive && return Float32[u0[1], u0[2], dt, reltol, abstol, l, 2, save_dt]
    throw(ArgumentError("method must be :rk4, :tsit5 or :tsit5_adaptive"))
end

# ---------------------------------------------------------------- many solves
"""Independent problems solved in one persistent launch (pps_batch_*): `add!` each, `run!`, then
`result` / `state` per slot.  Each result equals the problem solved alone."""
mutable struct PPSBatch
    h::Ptr{Cvoid}
    dims::Vector{Int}
    ns::Vector{Int}
end

function PPSBatch()
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pps_batch_create, lib()), Cint, (Ref{Ptr{Cvoid}},), out))
    b = PPSBatch(out[], Int[], Int[])
    finalizer(b) do x
        x.h != C_NULL && ccall((:pps_batch_destroy, lib()), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    return b
end

"""Queue one swarm; returns its slot."""
function add!(b::PPSBatch, prob, n::Integer; maxiters = 100, seed = 0, w = 0.7298f0, wdamp = 1.0f0,
              c1 = 1.4962f0, c2 = 1.4962f0)
    cp, bufs = pps_problem(prob)
    slot = Ref{Int32}()
    GC.@preserve bufs check(ccall((:pps_batch_add, lib()), Cint,
                                  (Ptr{Cvoid}, Ref{PPSProblem}, Int64, UInt64, Int32, Float32, Float32, Float32,
                                   Float32, Ref{Int32}),
                                  b.h, cp, n, seed, maxiters, w, wdamp, c1, c2, slot))
    push!(b.dims, length(prob.u0))
    push!(b.ns, Int(n))
    return slot[]
end

"""Fix the block shape (threads in {128, 256, 512}, particles per thread in {1, 2}); (0, 0)
returns to the autotuner."""
set_shape!(b::PPSBatch, threads::Integer, ppt::Integer) =
    check(ccall((:pps_batch_set_shape, lib()), Cint, (Ptr{Cvoid}, Int32, Int32), b.h, threads, ppt))

"""Solve every queued swarm in one launch; returns the device time in ms."""
function run!(b::PPSBatch)
    ms = Ref{Float32}(0)
    check(ccall((:pps_batch_run, lib()), Cint, (Ptr{Cvoid}, Ref{Float32}), b.h, ms))
    return ms[]
end

"""(u, cost, index) of a slot's swarm after `run!`."""
function result(b::PPSBatch, slot::Integer)
    u = Vector{Float32}(undef, b.dims[slot + 1])
    cost, idx = Ref{Float32}(), Ref{Int64}()
    check(ccall((:pps_batch_result, lib()), Cint, (Ptr{Cvoid}, Int32, Ptr{Float32}, Ref{Float32}, Ref{Int64}),
                b.h, slot, u, cost, idx))
    return u, cost[], idx[]
end

"""A state field of a slot's swarm after `run!` (n x dim, or n for FIELD_PCOST / FIELD_COST)."""
function state(b::PPSBatch, slot::Integer, field::Int32)
    n, D = b.ns[slot + 1], b.dims[slot + 1]
    out = field in (FIELD_PCOST, FIELD_COST) ? Vector{Float32}(undef, n) : Matrix{Float32}(undef, n, D)
    check(ccall((:pps_batch_get_state, lib()), Cint, (Ptr{Cvoid}, Int32, Int32, Ptr{Float32}), b.h, slot, field,
                out))
    return out
end

"""(swarms, threads, particles per thread, device bytes) of the last run."""
function batch_info(b::PPSBatch)
    ns, t, ppt, bytes = Ref{Int32}(), Ref{Int32}(), Ref{Int32}(), Ref{UInt64}()
    check(ccall((:pps_batch_info, lib()), Cint, (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}, Ref{Int32}, Ref{UInt64}),
                b.h, ns, t, ppt, bytes))
    return Int(ns[]), Int(t[]), Int(ppt[]), Int(bytes[])
end

"""Solve independent problems in one persistent launch; returns (u, cost) each."""
function solve_many(probs, n; maxiters = 100, w = 0.7298f0, wdamp = 1.0f0, c1 = 1.4962f0, c2 = 1.4962f0)
    b = PPSBatch()
    slots = [add!(b, prob, n; maxiters, seed = k, w, wdamp, c1, c2) for (k, prob) in enumerate(probs)]
    run!(b)
    return [result(b, slot)[1:2] for slot in slots]
end

# ---------------------------------------------------------------- device snapshots
"""A device snapshot of a swarm's state field: the reference's `sol.original`, a new device array
(src/solve.jl:51-56).  The swarm may run on or be destroyed while it lives; `read_copy` copies it
to the host."""
mutable struct PPSFieldCopy
    h::Ptr{Cvoid}
    n::Int
    dim::Int
    field::Int32
end

function snapshot(s::PPSSwarm, field::Int32 = FIELD_POSITION)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pps_field_copy_create, lib()), Cint, (Ptr{Cvoid}, Int32, Ref{Ptr{Cvoid}}), s.h, field, out))
    c = PPSFieldCopy(out[], s.n, s.dim, field)
    finalizer(c) do x
        x.h != C_NULL && ccall((:pps_field_copy_destroy, lib()), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    return c
end

function read_copy(c::PPSFieldCopy)
    out = c.field in (FIELD_PCOST, FIELD_COST) ? Vector{Float32}(undef, c.n) : Matrix{Float32}(undef, c.n, c.dim)
    check(ccall((:pps_field_copy_read, lib()), Cint, (Ptr{Cvoid}, Ptr{Float32}), c.h, out))
    return out
end

# ---------------------------------------------------------------- serving
"""A request server (pps_serve_*): problems submitted as they arrive are packed into batched
launches or run as swarms of their own, with their state in a device arena of `memory_budget`
bytes; every result equals the problem solved alone.  Zero settings take the library's
defaults; `single_min_n` / `ode_single_min_n` route requests by particle count."""
mutable struct PPSServer
    h::Ptr{Cvoid}
    dims::Dict{UInt64, Int}
end

function PPSServer(; memory_budget = 8 << 30, max_launches = 8, max_pack = 512, threads = 256, ppt = 1,
                   tick_us = 200.0, single_min_n = 0, ode_single_min_n = 0)
    cfg = Ref(PPSServeConfig(UInt64(memory_budget), Int32(max_launches), Int32(max_pack), Int32(threads),
                             Int32(ppt), Float64(tick_us), Int32(single_min_n), Int32(ode_single_min_n)))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pps_serve_start, lib()), Cint, (Ref{PPSServeConfig}, Ref{Ptr{Cvoid}}), cfg, out))
    srv = PPSServer(out[], Dict{UInt64, Int}())
    finalizer(serve_stop!, srv)
    return srv
end

"""Queue one problem (the library copies its buffers) and return its ticket."""
function submit!(srv::PPSServer, prob, n::Integer; maxiters = 100, seed = 0, w = 0.7298f0, wdamp = 1.0f0,
                 c1 = 1.4962f0, c2 = 1.4962f0)
    cp, bufs = pps_problem(prob)
    ticket = Ref{UInt64}(0)
    GC.@preserve bufs check(ccall((:pps_serve_submit, lib()), Cint,
                                  (Ptr{Cvoid}, Ref{PPSProblem}, Int64, UInt64, Int32, Float32, Float32, Float32,
                                   Float32, Ref{UInt64}),
                                  srv.h, cp, n, seed, maxiters, w, wdamp, c1, c2, ticket))
    srv.dims[ticket[]] = length(prob.u0)
    return ticket[]
end

"""(u, cost, index, latency in ms) of a finished request, or `nothing` while it runs."""
function poll(srv::PPSServer, ticket::UInt64)
    u = Vector{Float32}(undef, srv.dims[ticket])
    cost, idx, lat = Ref{Float32}(), Ref{Int64}(), Ref{Float64}()
    rc = ccall((:pps_serve_poll, lib()), Cint, (Ptr{Cvoid}, UInt64, Ptr{Float32}, Ref{Float32}, Ref{Int64}, Ref{Float64}),
               srv.h, ticket, u, cost, idx, lat)
    rc == 5 && return nothing  # PPS_EBUSY
    check(rc)
    delete!(srv.dims, ticket)
    return u, cost[], idx[], lat[]
end

"""Block until the request is done (an error after `timeout_s` seconds); returns (u, cost, index,
latency in ms)."""
function wait_result(srv::PPSServer, ticket::UInt64; timeout_s = 600.0)
    u = Vector{Float32}(undef, srv.dims[ticket])
    cost, idx, lat = Ref{Float32}(), Ref{Int64}(), Ref{Float64}()
    check(ccall((:pps_serve_wait, lib()), Cint,
                (Ptr{Cvoid}, UInt64, Ptr{Float32}, Ref{Float32}, Ref{Int64}, Ref{Float64}, Float64),
                srv.h, ticket, u, cost, idx, lat, Float64(timeout_s)))
    delete!(srv.dims, ticket)
    return u, cost[], idx[], lat[]
end

"""Requests submitted and completed, launches, solves/s and the p50 / p99 time to solution."""
function serve_stats(srv::PPSServer)
    r = Ref{PPSServeStats}()
    check(ccall((:pps_serve_stats_get, lib()), Cint, (Ptr{Cvoid}, Ref{PPSServeStats}), srv.h, r))
    return r[]
end

"""Finish the queued and running requests and release the server."""
function serve_stop!(srv::PPSServer)
    if srv.h != C_NULL
        ccall((:pps_serve_stop, lib()), Cint, (Ptr{Cvoid},), srv.h)
        srv.h = C_NULL
    end
    return nothing
end

# ---------------------------------------------------------------- sharded swarms
"""This process's shard (particles first .. first+count-1 of n_global) of a swarm split over
processes.  Per iteration: `shard_step!`, an all-gather of the `shard_record` bytes of every
shard into one buffer (e.g. NCCL.jl or MPI.jl), `shard_apply!`.  Bind the gather buffers with
`shard_bind!` (device pointers, e.g. from CUDA.jl)."""
function shard_create(prob, n_global, first, count; seed = 0)
    cp, bufs = pps_problem(prob)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve bufs check(ccall((:pps_shard_create, lib()), Cint,
                                  (Ref{PPSProblem}, Int64, Int64, Int64, UInt64, UInt32, Ref{Ptr{Cvoid}}),
                                  cp, n_global, first, count, seed, UInt32(0), out))
    s = PPSSwarm(out[], Int(count), length(prob.u0))
    finalizer(x -> ccall((:pps_swarm_destroy, lib()), Cint, (Ptr{Cvoid},), x.h), s)
    return s
end

function shard_record(s::PPSSwarm)
    rec = Ref{Ptr{Cvoid}}(C_NULL)
    nbytes = Ref{Int64}(0)
    stream = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pps_shard_record, lib()), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}, Ref{Int64}, Ref{Ptr{Cvoid}}),
                s.h, rec, nbytes, stream))
    return rec[], nbytes[], stream[]
end

shard_bind!(s::PPSSwarm, record::Ptr, records::Ptr, nrecords::Integer) =
    check(ccall((:pps_shard_bind, lib()), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int32), s.h, record, records,
                nrecords))
shard_step!(s::PPSSwarm, first_of_run::Bool; w = 0.7298f0, wdamp = 1.0f0, c1 = 1.4962f0, c2 = 1.4962f0) =
    check(ccall((:pps_shard_step, lib()), Cint, (Ptr{Cvoid}, Int32, Float32, Float32, Float32, Float32), s.h,
                first_of_run ? 1 : 0, w, wdamp, c1, c2))
"""ParallelPSOKernel(global_update = false) on the shard: maxiters iterations in one launch, the
record written after the last; exchange the records and `shard_apply!` once."""
shard_async!(s::PPSSwarm, maxiters::Integer; w = 0.7298f0, wdamp = 1.0f0, c1 = 1.4962f0, c2 = 1.4962f0) =
    check(ccall((:pps_shard_async, lib()), Cint, (Ptr{Cvoid}, Int32, Float32, Float32, Float32, Float32), s.h,
                maxiters, w, wdamp, c1, c2))
shard_apply!(s::PPSSwarm) = check(ccall((:pps_shard_apply, lib()), Cint, (Ptr{Cvoid},), s.h))
shard_finish!(s::PPSSwarm) = check(ccall((:pps_shard_finish, lib()), Cint, (Ptr{Cvoid},), s.h))

end # module
