"""
    GB300Backend

A GB300 (sm_103a) backend for the time-step hot path of GeothermalWells.jl:
the z-diffusion right-hand side `rhs_diffusion_z!` that ROCK2 evaluates, the
ADI x/y line solves and the semi-Lagrangian pipe advection of
`ADI_and_ADV_callback!`.  Every call goes through the plain C ABI of
`libgw_gb300.so` (`include/gw_gb300.h`) with `ccall`: no CUDA.jl, no
KernelAbstractions GPU code generation, no CPU fallback.

Two ways to run, both with the reference's own calls around them:

1. Fused (fast): the state stays on the GPU and every step is one replay of a
   captured CUDA graph (`gw_step`).

       backend = GB300(precision = :mixed)            # or :fp64
       T0 = initial_condition_thermal_gradient(backend, Float64, gridx, gridy, gridz;
                                               T_surface = 2.29, gradient = 0.035)
       cache = GB300Backend.create_cache(; backend, gridx, gridy, gridz, materials,
                                         boreholes, inlet_model)
       prob = ODEProblem(rhs_diffusion_z!, T0, tspan, cache)
       callback, saved_values = GB300Backend.get_simulation_callback(; saveat, print_every_n = 100)
       sol = solve(prob, ROCK2(max_stages = 100, eigen_est = eigen_estimator);
                   dt = Δt, adaptive = false, callback)
       cache.T_outlet[1]

   `solve` here is a method for problems whose parameter is a `GB300Cache`
   and whose state is a host `Array{Float64,3}`.

2. Integrator-driven (FP64): the state is a `GB300Field`, a device array
   handle.  OrdinaryDiffEq's own ROCK2 runs on it; its stage updates (linear
   combinations) become `gw_lincomb`, and the reference's own
   `ADI_and_ADV_callback!` and `get_simulation_callback` run unchanged:
   `diffusion_1D!(::GB300)`, `thomas_I_minus_A!(::GB300)` and
   `advection!(::GB300Field, ...)` dispatch to the library.

       u0 = GB300Field(cache, T0)
       prob = ODEProblem(rhs_diffusion_z!, u0, tspan, cache)
       callback, saved_values = get_simulation_callback(; saveat)   # the reference's
       solve(prob, ROCK2(max_stages = 100, eigen_est = eigen_estimator);
             dt = Δt, adaptive = false, callback)

`GB300Backend.create_cache` and `GB300Backend.get_simulation_callback` forward
any other backend to GeothermalWells' own functions, so a script can use them
for every backend.

Not run here: Julia is not installed where this package was written or on the
GPU machines it was tested on.  The library calls it makes are the ones the
Python binding (`geothermalwells_gb300`) makes and tests, and the struct
mirrors below are checked against the C header's layout by
`tests/test_layout.py`.
"""
module GB300Backend

using GeothermalWells
import GeothermalWells: rhs_diffusion_z!, diffusion_1D!, thomas_I_minus_A!, advection!,
                        initial_condition_thermal_gradient
using KernelAbstractions: CPU
import Adapt
import SciMLBase
using DiffEqCallbacks: SavedValues
import OrdinaryDiffEqStabilizedRK
import ChainRulesCore
import JLD2
using Libdl

export GB300, GB300Cache, GB300Field, ScheduleInlet, ExpressionInlet, AdjointDesign, outlet_series,
       extracted_heat, set_mixed_options!

# ---------------------------------------------------------------------------
# the library

const LIBPATH = Ref{String}("")
const HANDLE = Ref{Ptr{Cvoid}}(C_NULL)
const SYMS = Dict{Symbol,Ptr{Cvoid}}()

default_libpath() = get(ENV, "GW_GB300_LIB",
                        normpath(joinpath(@__DIR__, "..", "..", "..", "geothermalwells.jl_gb300",
                                          "lib", "libgw_gb300.so")))

function libgw()
    if HANDLE[] == C_NULL
        LIBPATH[] = default_libpath()
        isfile(LIBPATH[]) || error("libgw_gb300.so not found at $(LIBPATH[]); build it with " *
                                   "`python -c \"import __graft_entry__ as g; g.build()\"` " *
                                   "or set ENV[\"GW_GB300_LIB\"]")
        HANDLE[] = Libdl.dlopen(LIBPATH[])
    end
    return HANDLE[]
end

"Address of a library entry point (looked up once)."
fn(name::Symbol) = get!(() -> Libdl.dlsym(libgw(), name), SYMS, name)

function check(rc)
    rc == 0 && return nothing
    msg = unsafe_string(ccall(fn(:gw_last_error), Cstring, ()))
    error("gw_gb300 error $rc: $msg")
end

const GW_INLET_CONSTANT, GW_INLET_HEAT_EXCHANGER, GW_INLET_SCHEDULE = 0, 1, 2
const GW_INLET_EXPRESSION = 3
# postfix operations of an expression inlet (GW_OP_* of the header)
const GW_OP_CONST, GW_OP_TOUT, GW_OP_TIME, GW_OP_BH, GW_OP_SCHED, GW_OP_NEG = 0, 1, 2, 3, 4, 5
const GW_OP_ADD, GW_OP_SUB, GW_OP_MUL, GW_OP_DIV, GW_OP_MIN, GW_OP_MAX = 6, 7, 8, 9, 10, 11
const GW_MIXED_ROCK2_F64, GW_MIXED_REFINE = 1, 2
const GW_DIR = (x = Cint(0), y = Cint(1), z = Cint(2))

# ---------------------------------------------------------------------------
# mirrors of the C structs of include/gw_gb300.h (isbits: C layout)

struct BoreholeDesc
    xc::Cdouble; yc::Cdouble; h::Cdouble; r_inner::Cdouble; t_inner::Cdouble
    r_outer::Cdouble; t_outer::Cdouble; r_backfill::Cdouble; mdot::Cdouble
    insulation_depth::Cdouble
end

struct MaterialDesc
    n_layers::Cint
    k_rock_layers::Ptr{Cdouble}; rho_c_rock_layers::Ptr{Cdouble}; layer_depths::Ptr{Cdouble}
    k_water::Cdouble; rho_c_water::Cdouble; k_steel::Cdouble; rho_c_steel::Cdouble
    k_insulating::Cdouble; rho_c_insulating::Cdouble; k_backfill::Cdouble; rho_c_backfill::Cdouble
end

struct Desc
    nx::Cint; ny::Cint; nz::Cint
    gridx::Ptr{Cdouble}; gridy::Ptr{Cdouble}; gridz::Ptr{Cdouble}
    n_boreholes::Cint; boreholes::Ptr{BoreholeDesc}
    materials::MaterialDesc
    inlet_kind::Cint; inlet_param::Cdouble
    precision::Cint; device::Cint
end

struct GwInfo
    nx::Cint; ny::Cint; nz::Cint; n_boreholes::Cint
    countxy_inner::Cint; countxy_outer::Cint; countz::Cint
    n_zclass::Cint; n_profiles::Cint
    eigen_estimate::Cdouble
    device_bytes::Clonglong
    overlap::Cint; fused::Cint; modular_reason::Cint; tiling::Cint; mixed_options::Cint
    step_order::Cint
end

struct AdjointInfo
    objective::Cdouble
    n_params::Cint; stages::Cint; checkpoints::Cint
    forward_ms::Cdouble; reverse_ms::Cdouble
    peak_bytes::Clonglong
end

# ---------------------------------------------------------------------------
# backend, inlet schedule, cache

"""
    GB300(; device = 0, precision = :fp64)

The backend value passed to `create_cache` in place of `CPU()`.  `precision`
is `:fp64` (double everywhere, the reference's arithmetic) or `:mixed` (float
storage of T - T_ref(z) and float line solves; outlet, annulus means and the
energy balance in double; fused path only).
"""
struct GB300
    device::Int
    precision::Symbol
    function GB300(device::Integer, precision::Symbol)
        precision in (:fp64, :mixed) || throw(ArgumentError("precision is :fp64 or :mixed"))
        new(Int(device), precision)
    end
end
GB300(; device = 0, precision = :fp64) = GB300(device, precision)

"""
    ScheduleInlet(times, values)

A `CustomInlet` of the form `(bh, T_outlet, t) -> T_in(t)` with T_in linear
between the points and held constant outside them: the form of custom inlet
that crosses the C ABI (`GW_INLET_SCHEDULE`, `gw_set_inlet_schedule`).
"""
struct ScheduleInlet <: GeothermalWells.AbstractInletModel
    times::Vector{Float64}
    values::Vector{Float64}
    function ScheduleInlet(times, values)
        length(times) == length(values) >= 1 || throw(ArgumentError("one value per time"))
        all(diff(times) .> 0) || throw(ArgumentError("times must be strictly increasing"))
        new(Float64.(collect(times)), Float64.(collect(values)))
    end
end
function (m::ScheduleInlet)(bh_idx, T_outlet_values, t)
    ts, vs = m.times, m.values
    t <= ts[1] && return vs[1]
    t >= ts[end] && return vs[end]
    hi = searchsortedfirst(ts, t)
    ts[hi] == t && return vs[hi]
    lo = hi - 1
    a = (t - ts[lo]) / (ts[hi] - ts[lo])
    return fma(a, vs[hi] - vs[lo], vs[lo])
end

"""
    ExpressionInlet(ex; schedule = nothing)

A `CustomInlet` whose closure `(bh, T_outlet, t) -> T_in` is arithmetic: the
expression `ex` (a quoted Julia expression) over `T_out` (the borehole's
outlet temperature, `T_outlet[bh]`), `t`, `bh` (1-based, as in Julia),
numbers, `+ - * /`, unary `-`, `min`, `max` and `sched(x)` (the optional
piecewise-linear `schedule = (times, values)` at `x`).  A heat pump that takes
ΔT(t) out of the outlet but never cools the inlet below 5 °C:

    ExpressionInlet(:(max(5.0, T_out - sched(t))); schedule = ([0.0, 3600.0], [3.0, 6.0]))

It is compiled to the postfix program of `GW_INLET_EXPRESSION`
(`gw_set_inlet_program`), which the GPU evaluates in double where the
reference calls the inlet model (`src/solver.jl:349-350`); calling the object
evaluates the same program on the host, so it also runs on the reference's
`CPU()` backend.
"""
struct ExpressionInlet <: GeothermalWells.AbstractInletModel
    ex::Any
    ops::Vector{Cint}
    args::Vector{Float64}
    schedule::Union{Nothing,ScheduleInlet}
end

function ExpressionInlet(ex; schedule = nothing)
    sched = schedule === nothing ? nothing : ScheduleInlet(schedule[1], schedule[2])
    ops, args = Cint[], Float64[]
    emit(op, a = 0.0) = (push!(ops, op); push!(args, Float64(a)); nothing)
    binops = Dict(:+ => GW_OP_ADD, :- => GW_OP_SUB, :* => GW_OP_MUL, :/ => GW_OP_DIV)
    function walk(n)
        n isa Real && !(n isa Bool) && return emit(GW_OP_CONST, n)
        n === :T_out && return emit(GW_OP_TOUT)
        n === :t && return emit(GW_OP_TIME)
        if n === :bh   # 1-based in Julia: the library's index is 0-based
            emit(GW_OP_BH); emit(GW_OP_CONST, 1.0); return emit(GW_OP_ADD)
        end
        n isa Expr && n.head === :call || throw(ArgumentError("unsupported element in the inlet expression: $n"))
        f, a = n.args[1], n.args[2:end]
        if f === :- && length(a) == 1
            walk(a[1]); return emit(GW_OP_NEG)
        elseif f === :+ && length(a) == 1
            return walk(a[1])
        elseif haskey(binops, f) && length(a) >= 2
            walk(a[1])
            for x in a[2:end]   # Julia folds a + b + c into one call
                walk(x); emit(binops[f])
            end
            return nothing
        elseif f in (:min, :max) && length(a) >= 2
            walk(a[1])
            for x in a[2:end]
                walk(x); emit(f === :min ? GW_OP_MIN : GW_OP_MAX)
            end
            return nothing
        elseif f === :sched && length(a) == 1
            sched === nothing && throw(ArgumentError("sched(...) needs ExpressionInlet(ex; schedule = (times, values))"))
            walk(a[1]); return emit(GW_OP_SCHED)
        end
        throw(ArgumentError("unsupported call in the inlet expression: $n"))
    end
    walk(ex)
    depth, top = 0, 0
    for o in ops
        depth += o <= GW_OP_BH ? 1 : (o <= GW_OP_NEG ? 0 : -1)
        top = max(top, depth)
    end
    (length(ops) > 64 || top > 16) &&
        throw(ArgumentError("inlet expression too long (at most 64 operations, stack depth 16)"))
    return ExpressionInlet(ex, ops, args, sched)
end

function (m::ExpressionInlet)(bh_idx, T_outlet_values, t)
    st = Float64[]
    for (o, a) in zip(m.ops, m.args)
        if o == GW_OP_CONST
            push!(st, a)
        elseif o == GW_OP_TOUT
            push!(st, Float64(T_outlet_values[bh_idx]))
        elseif o == GW_OP_TIME
            push!(st, Float64(t))
        elseif o == GW_OP_BH
            push!(st, Float64(bh_idx - 1))
        elseif o == GW_OP_SCHED
            st[end] = m.schedule(bh_idx, T_outlet_values, st[end])
        elseif o == GW_OP_NEG
            st[end] = -st[end]
        else
            b = pop!(st)
            x = st[end]
            st[end] = o == GW_OP_ADD ? x + b : o == GW_OP_SUB ? x - b : o == GW_OP_MUL ? x * b :
                      o == GW_OP_DIV ? (b == 0 ? Inf : x / b) : o == GW_OP_MIN ? min(x, b) : max(x, b)
        end
    end
    return st[1]
end

"""
The cache `create_cache(; backend = GB300(), ...)` returns: the library
context plus the fields the reference's functions read from their cache
(`src/cache.jl:55-116`), so `ADI_and_ADV_callback!` and `eigen_estimator`
run on it unchanged.  `cache.T_outlet` reads the outlet temperatures back.
"""
mutable struct GB300Cache
    ctx::Ptr{Cvoid}
    backend::GB300
    gridx::Vector{Float64}
    gridy::Vector{Float64}
    gridz::Vector{Float64}
    Nx::Int
    Ny::Int
    Nz::Int
    N_bh::Int
    materials::Any
    boreholes::Any
    inlet_model::Any
    countxy_inner::Int
    countxy_outer::Int
    countz::Int
    eigen_estimate::Float64
    fused::Bool
    ValNx::Any
    ValNy::Any
    ValNz::Any
    ValTrue::Val{true}
    ValFalse::Val{false}
    Val_in_x::Val{:x}
    Val_in_y::Val{:y}
    Val_in_z::Val{:z}
end

function Base.getproperty(c::GB300Cache, s::Symbol)
    s === :T_outlet && return outlet(c)
    return getfield(c, s)
end

function outlet(c::GB300Cache)
    T = zeros(Float64, c.N_bh)
    check(ccall(fn(:gw_get_outlet), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), c.ctx, T))
    return T
end

function info(c::GB300Cache)
    r = Ref{GwInfo}()
    check(ccall(fn(:gw_get_info), Cint, (Ptr{Cvoid}, Ref{GwInfo}), c.ctx, r))
    return r[]
end

"""
    set_mixed_options!(cache; rock2_f64 = false, refine = false)

The mixed step's two optional double-precision parts (`gw_set_mixed_options`):
`rock2_f64` accumulates the ROCK2 stages in double over the float field,
`refine` follows every float line solve with its residual in double and one
correction solve.  FP64 contexts ignore them.
"""
function set_mixed_options!(c::GB300Cache; rock2_f64::Bool = false, refine::Bool = false)
    flags = (rock2_f64 ? GW_MIXED_ROCK2_F64 : 0) | (refine ? GW_MIXED_REFINE : 0)
    check(ccall(fn(:gw_set_mixed_options), Cint, (Ptr{Cvoid}, Cint), c.ctx, flags))
    return c
end

function destroy!(c::GB300Cache)
    if getfield(c, :ctx) != C_NULL
        ccall(fn(:gw_destroy), Cint, (Ptr{Cvoid},), getfield(c, :ctx))
        setfield!(c, :ctx, C_NULL)
    end
    return nothing
end

rock_layers(m::GeothermalWells.HomogenousMaterialProperties) = ([m.k_rock], [m.rho_c_rock], [Inf])
rock_layers(m::GeothermalWells.StratifiedMaterialProperties) =
    (collect(Float64, m.k_rock_layers), collect(Float64, m.rho_c_rock_layers),
     collect(Float64, m.layer_depths))

inlet_kind(m::GeothermalWells.ConstantInlet) = (GW_INLET_CONSTANT, Float64(m.T_const))
inlet_kind(m::GeothermalWells.HeatExchangerInlet) = (GW_INLET_HEAT_EXCHANGER, Float64(m.ΔT))
inlet_kind(m::ScheduleInlet) = (GW_INLET_SCHEDULE, 0.0)
inlet_kind(m::ExpressionInlet) = (GW_INLET_EXPRESSION, 0.0)
inlet_kind(::GeothermalWells.CustomInlet) =
    throw(ArgumentError("CustomInlet closures cannot cross the C ABI; write T_in as a ScheduleInlet " *
                        "(T_in(t)) or an ExpressionInlet (arithmetic in T_out, t, bh)"))

"""
    create_cache(; backend, gridx, gridy, gridz, materials, boreholes, inlet_model)

`create_cache` of `src/cache.jl:55` for `backend::GB300` (`gw_create`: material
tables, advection index lists and buffers on the GPU); any other backend goes
to `GeothermalWells.create_cache`.
"""
function create_cache(; backend, gridx, gridy, gridz, materials, boreholes, inlet_model)
    backend isa GB300 || return GeothermalWells.create_cache(; backend, gridx, gridy, gridz,
                                                             materials, boreholes, inlet_model)
    kind, param = inlet_kind(inlet_model)
    layers = rock_layers(materials)
    bhs = [BoreholeDesc(b.xc, b.yc, b.h, b.r_inner, b.t_inner, b.r_outer, b.t_outer, b.r_backfill,
                        b.ṁ, b.insulation_depth) for b in boreholes]
    gx, gy, gz = collect(Float64, gridx), collect(Float64, gridy), collect(Float64, gridz)
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve layers bhs gx gy gz begin
        m = MaterialDesc(length(layers[1]), pointer(layers[1]), pointer(layers[2]), pointer(layers[3]),
                         materials.k_water, materials.rho_c_water, materials.k_steel,
                         materials.rho_c_steel, materials.k_insulating, materials.rho_c_insulating,
                         materials.k_backfill, materials.rho_c_backfill)
        d = Ref(Desc(length(gx), length(gy), length(gz), pointer(gx), pointer(gy), pointer(gz),
                     length(bhs), pointer(bhs), m, kind, param,
                     backend.precision === :mixed ? 1 : 0, backend.device))
        check(ccall(fn(:gw_create), Cint, (Ref{Desc}, Ref{Ptr{Cvoid}}), d, ctx))
    end
    sched = inlet_model isa ScheduleInlet ? inlet_model :
            inlet_model isa ExpressionInlet ? inlet_model.schedule : nothing
    if sched !== nothing
        check(ccall(fn(:gw_set_inlet_schedule), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}),
                    ctx[], length(sched.times), sched.times, sched.values))
    end
    if inlet_model isa ExpressionInlet
        check(ccall(fn(:gw_set_inlet_program), Cint, (Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Cdouble}),
                    ctx[], length(inlet_model.ops), inlet_model.ops, inlet_model.args))
    end
    r = Ref{GwInfo}()
    check(ccall(fn(:gw_get_info), Cint, (Ptr{Cvoid}, Ref{GwInfo}), ctx[], r))
    i = r[]
    c = GB300Cache(ctx[], backend, gx, gy, gz, length(gx), length(gy), length(gz), length(bhs),
                   materials, boreholes, inlet_model, i.countxy_inner, i.countxy_outer, i.countz,
                   i.eigen_estimate, i.fused != 0, Val(length(gx)), Val(length(gy)), Val(length(gz)),
                   Val(true), Val(false), Val(:x), Val(:y), Val(:z))
    finalizer(destroy!, c)
    return c
end

"""
    initial_condition_thermal_gradient(::GB300, Float_used, gridx, gridy, gridz; T_surface, gradient)

`src/physics.jl:333-348` for the GB300 backend: the initial field as a host
array (the fused `solve` uploads it; `GB300Field(cache, T0)` puts it on the
GPU for the integrator-driven path).
"""
function initial_condition_thermal_gradient(::GB300, Float_used, gridx, gridy, gridz;
                                            T_surface, gradient)
    Nx, Ny, Nz = length(gridx), length(gridy), length(gridz)
    ϕ = zeros(Float_used, Nz, Ny, Nx)
    for i in 1:Nx, j in 1:Ny, k in 1:Nz
        ϕ[k, j, i] = T_surface + gradient * gridz[k]
    end
    return ϕ
end

# ---------------------------------------------------------------------------
# device fields (integrator-driven path)

"""
    GB300Field(cache)            # zeros
    GB300Field(cache, T::Array)  # a copy of the host field T

An `(Nz, Ny, Nx)` Float64 field on the cache's GPU (`gw_field_alloc`), the
state type of the integrator-driven path.  Scalar indexing is not
supported; copy it to the host with `Array(f)`.  Broadcasts that are linear
combinations of fields (what ROCK2's stage updates are) run as `gw_lincomb`.
"""
mutable struct GB300Field <: AbstractArray{Float64,3}
    ptr::Ptr{Cdouble}
    cache::GB300Cache
    function GB300Field(cache::GB300Cache)
        p = Ref{Ptr{Cdouble}}(C_NULL)
        check(ccall(fn(:gw_field_alloc), Cint, (Ptr{Cvoid}, Ref{Ptr{Cdouble}}), cache.ctx, p))
        f = new(p[], cache)
        finalizer(free!, f)
        return f
    end
end

function GB300Field(cache::GB300Cache, T::AbstractArray{<:Real,3})
    size(T) == (cache.Nz, cache.Ny, cache.Nx) || throw(DimensionMismatch("field is not Nz x Ny x Nx"))
    f = GB300Field(cache)
    copyto!(f, Array{Float64}(T))
    return f
end

function free!(f::GB300Field)
    if f.ptr != C_NULL && getfield(f.cache, :ctx) != C_NULL
        ccall(fn(:gw_field_free), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), f.cache.ctx, f.ptr)
    end
    f.ptr = C_NULL
    return nothing
end

Base.size(f::GB300Field) = (f.cache.Nz, f.cache.Ny, f.cache.Nx)
Base.IndexStyle(::Type{GB300Field}) = IndexLinear()
Base.getindex(::GB300Field, ::Int...) =
    error("scalar indexing of a GB300Field is not supported; copy it with Array(f)")
Base.setindex!(::GB300Field, v, ::Int...) =
    error("scalar indexing of a GB300Field is not supported")
Base.similar(f::GB300Field) = GB300Field(f.cache)
Base.similar(f::GB300Field, ::Type{Float64}) = GB300Field(f.cache)
Base.similar(f::GB300Field, ::Type{Float64}, dims::Dims{3}) =
    dims == size(f) ? GB300Field(f.cache) : throw(DimensionMismatch("GB300Fields have the grid's shape"))
Base.zero(f::GB300Field) = GB300Field(f.cache)

function fieldcopy!(cache::GB300Cache, dst::Ptr{Cdouble}, src::Ptr{Cdouble})
    check(ccall(fn(:gw_field_copy), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}), cache.ctx, dst, src))
end

function Base.copyto!(dst::GB300Field, src::GB300Field)
    fieldcopy!(dst.cache, dst.ptr, src.ptr)
    return dst
end
function Base.copyto!(dst::GB300Field, src::Array{Float64,3})
    size(src) == size(dst) || throw(DimensionMismatch("field is not Nz x Ny x Nx"))
    GC.@preserve src fieldcopy!(dst.cache, dst.ptr, pointer(src))
    return dst
end
function Base.copyto!(dst::Array{Float64,3}, src::GB300Field)
    size(src) == size(dst) || throw(DimensionMismatch("field is not Nz x Ny x Nx"))
    GC.@preserve dst fieldcopy!(src.cache, pointer(dst), src.ptr)
    return dst
end
Base.Array(f::GB300Field) = copyto!(Array{Float64,3}(undef, size(f)), f)
Base.copy(f::GB300Field) = copyto!(GB300Field(f.cache), f)
Adapt.adapt_storage(::CPU, f::GB300Field) = Array(f)

"dst = Σ coeffs[i] * srcs[i] on the device (gw_lincomb; dst may be a source)."
function lincomb!(dst::GB300Field, coeffs::Vector{Float64}, srcs::Vector{GB300Field})
    length(coeffs) == length(srcs) <= 8 || throw(ArgumentError("up to 8 terms, one coefficient each"))
    ptrs = Ptr{Cdouble}[s.ptr for s in srcs]
    GC.@preserve srcs ptrs coeffs check(ccall(fn(:gw_lincomb), Cint,
                                              (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Ptr{Ptr{Cdouble}}),
                                              dst.cache.ctx, dst.ptr, length(srcs), coeffs, ptrs))
    return dst
end

function Base.fill!(f::GB300Field, v)
    iszero(v) || error("GB300Field: fill! with a nonzero constant is not a linear combination of fields")
    return lincomb!(f, Float64[], GB300Field[])
end

# Broadcasting: a broadcast over GB300Fields must be a linear combination
# (scalars times fields, sums, differences, muladd), which is what the
# stage updates of ROCK2's perform_step! are.  It is flattened into terms and
# evaluated by one gw_lincomb (equal fields merged).
struct GB300Style <: Broadcast.AbstractArrayStyle{3} end
GB300Style(::Val{3}) = GB300Style()
Base.BroadcastStyle(::Type{GB300Field}) = GB300Style()
Base.BroadcastStyle(::GB300Style, ::Broadcast.DefaultArrayStyle{0}) = GB300Style()

firstfield(f::GB300Field) = f
firstfield(bc::Broadcast.Broadcasted) = (for a in bc.args
                                             r = firstfield(a); r === nothing || return r
                                         end; nothing)
firstfield(_) = nothing
Base.similar(bc::Broadcast.Broadcasted{GB300Style}, ::Type{Float64}) = GB300Field(firstfield(bc).cache)

scalar(x::Number) = Float64(x)
scalar(x::Base.RefValue) = Float64(x[])
scalar(x::AbstractArray{<:Number,0}) = Float64(x[])
isscalar(x) = x isa Number || x isa Base.RefValue || x isa AbstractArray{<:Number,0}

"Terms (coefficient, field) of a linear broadcast expression."
terms(f::GB300Field) = Tuple{Float64,GB300Field}[(1.0, f)]
function terms(bc::Broadcast.Broadcasted)
    f, a = bc.f, bc.args
    if f === identity && length(a) == 1
        return terms(a[1])
    elseif f === (+)
        return reduce(vcat, map(terms, a))
    elseif f === (-)
        length(a) == 1 && return [(-c, x) for (c, x) in terms(a[1])]
        return vcat(terms(a[1]), [(-c, x) for (c, x) in terms(a[2])])
    elseif f === (*)
        s, fieldarg = 1.0, nothing
        for x in a
            if isscalar(x)
                s *= scalar(x)
            elseif fieldarg === nothing
                fieldarg = x
            else
                error("GB300Field broadcast: a product of two fields is not linear")
            end
        end
        fieldarg === nothing && error("GB300Field broadcast: a constant term is not supported")
        return [(s * c, x) for (c, x) in terms(fieldarg)]
    elseif f === muladd && length(a) == 3
        return terms(Broadcast.Broadcasted(+, (Broadcast.Broadcasted(*, (a[1], a[2])), a[3])))
    end
    error("GB300Field broadcast supports linear combinations of fields only (got $(f))")
end
terms(x) = error("GB300Field broadcast: unsupported operand $(typeof(x))")

function Base.copyto!(dst::GB300Field, bc::Broadcast.Broadcasted{GB300Style})
    coeffs, srcs = Float64[], GB300Field[]
    for (c, x) in terms(bc)
        q = findfirst(s -> s === x, srcs)
        if q === nothing
            push!(coeffs, c); push!(srcs, x)
        else
            coeffs[q] += c
        end
    end
    return lincomb!(dst, coeffs, srcs)
end

# ---------------------------------------------------------------------------
# the reference's functions on GB300 fields

"""
    rhs_diffusion_z!(dϕ::GB300Field, ϕ::GB300Field, cache::GB300Cache, t)

`src/solver.jl:23-31` on the GPU: dϕ = A_z ϕ (`gw_rhs_diffusion_z`).
"""
function rhs_diffusion_z!(dϕ::GB300Field, ϕ::GB300Field, cache::GB300Cache, t)
    check(ccall(fn(:gw_rhs_diffusion_z), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}),
                cache.ctx, dϕ.ptr, ϕ.ptr))
    return nothing
end

# diffusion_1D!(backend)(dϕ, ϕ, gridx, gridy, gridz, boreholes, materials, dt,
# Val(dir), Val(plus_I); ndrange) and thomas_I_minus_A!(backend)(U, RHS, ...,
# dt, boreholes, materials, Val(N), Val(dir); ndrange), as
# ADI_and_ADV_callback! (src/solver.jl:432-464) launches them.
struct GB300Kernel{K} end
diffusion_1D!(::GB300) = GB300Kernel{:diffusion_1D}()
thomas_I_minus_A!(::GB300) = GB300Kernel{:thomas}()

function (::GB300Kernel{:diffusion_1D})(dϕ::GB300Field, ϕ::GB300Field, gridx, gridy, gridz, boreholes,
                                        materials, dt, ::Val{dir}, ::Val{plus_I}; ndrange = nothing) where {dir,plus_I}
    check(ccall(fn(:gw_diffusion_1d), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cint, Cint),
                dϕ.cache.ctx, dϕ.ptr, ϕ.ptr, dt, GW_DIR[dir], plus_I ? 1 : 0))
    return nothing
end

function (::GB300Kernel{:thomas})(U::GB300Field, RHS::GB300Field, gridx, gridy, gridz, dt, boreholes,
                                  materials, ::Val{N}, ::Val{dir}; ndrange = nothing) where {N,dir}
    check(ccall(fn(:gw_thomas), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cint),
                U.cache.ctx, U.ptr, RHS.ptr, dt, GW_DIR[dir]))
    return nothing
end

"""
    advection!(ϕ::GB300Field, dt, t, cache::GB300Cache, boreholes)

`src/solver.jl:250-264` on the GPU (`gw_advection`): outlet means, semi-Lagrangian
advection of the pipe columns, `cache.T_outlet` updated.
"""
function advection!(ϕ::GB300Field, dt, t, cache::GB300Cache, boreholes)
    check(ccall(fn(:gw_advection), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cdouble, Cdouble),
                cache.ctx, ϕ.ptr, dt, t))
    return nothing
end

# ---------------------------------------------------------------------------
# fused solve

"""
The callback set of the fused path: what `get_simulation_callback` asks for
(saving at `saveat` into `saved_values` as Float32 host arrays, optional JLD2
checkpoints, progress every `print_every_n` steps); the ADI/advection part is
inside every fused step.
"""
struct GB300Callback
    saveat::Vector{Float64}
    print_every_n::Int
    write_to_jld::Bool
    data_folder_dir::String
    saved_values::SavedValues{Float64,Array{Float32,3}}
    file_counter::Base.RefValue{Int}
end

"""
    get_simulation_callback(; saveat, print_every_n = 1000, write_to_jld = false, data_folder_dir = "")

`src/cache.jl:224-237` for the fused GB300 path; returns `(callback, saved_values)`.
Pass `backend = CPU()` (or any non-GB300 backend) to get GeothermalWells' own
callback set instead.
"""
function get_simulation_callback(; saveat, print_every_n = 1000, write_to_jld = false,
                                 data_folder_dir = "", backend = GB300())
    backend isa GB300 || return GeothermalWells.get_simulation_callback(; saveat, print_every_n,
                                                                        write_to_jld, data_folder_dir)
    if write_to_jld && isempty(data_folder_dir)
        error("When `write_to_jld` is true, `data_folder_dir` must be provided and cannot be an empty string")
    end
    sv = SavedValues(Float64, Array{Float32,3})
    cb = GB300Callback(collect(Float64, saveat), print_every_n, write_to_jld, data_folder_dir, sv, Ref(0))
    return cb, sv
end

function print_step(naccept, t)
    if t > 3600 * 24 * 365
        println("Step $(naccept), t = $(t) s, or $(round((t / 31536000), digits=4)) years")
    elseif t > 3600 * 24
        println("Step $(naccept), t = $(t) s, or $(round((t / 86400), digits=2)) days")
    else
        println("Step $(naccept), t = $(t) s, or $(round((t / 3600), digits=2)) hours")
    end
    flush(stdout)
end

function save!(cb::GB300Callback, cache::GB300Cache, t)
    T = zeros(Float64, cache.Nz, cache.Ny, cache.Nx)
    check(ccall(fn(:gw_get_field), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, T))
    save!(cb, t, Float32.(T))
end

function save!(cb::GB300Callback, t, u::Array{Float32,3})
    if cb.write_to_jld
        isdir(cb.data_folder_dir) || mkdir(cb.data_folder_dir)
        cb.file_counter[] += 1
        u_cpu = u
        JLD2.@save joinpath(cb.data_folder_dir, "checkpoint_$(cb.file_counter[]).jld2") u_cpu
    end
    push!(cb.saved_values.t, t)
    push!(cb.saved_values.saveval, u)
end

"Solution of the fused path: `u` at the start and the end, outlet series, energy."
struct GB300Solution
    t::Vector{Float64}
    u::Vector{Array{Float64,3}}
    outlet_t::Vector{Float64}
    T_outlet::Matrix{Float64}      # (nsteps, N_bh)
    energy::Vector{Float64}        # extracted heat per borehole [J]
    stages::Int
    retcode::Symbol
end

function steps_for(t, t0, dt, what)
    n = (t - t0) / dt
    r = round(Int, n)
    abs(n - r) <= 1e-9 * max(1.0, abs(n)) || error("$what time $t is not on the fixed-step grid (t0 = $t0, dt = $dt)")
    return r
end

"""
    solve(prob::ODEProblem{<:Array{Float64,3}, <:Any, true, GB300Cache}, alg::ROCK2;
          dt, adaptive = false, callback = nothing, kwargs...)

The fused path: `gw_step` runs ROCK2 on u' = A_z u (stage count from the
eigenvalue estimate, capped at `alg.max_stages`) and then the
ADI/advection split of `ADI_and_ADV_callback!`, one captured graph per step,
stopping only at save and print points.
"""
function SciMLBase.solve(prob::SciMLBase.ODEProblem{<:Array{Float64,3},<:Any,true,GB300Cache},
                         alg::OrdinaryDiffEqStabilizedRK.ROCK2; dt, adaptive = false,
                         save_everystep = false, callback = nothing, maxiters = typemax(Int), kwargs...)
    cache = prob.p
    adaptive && throw(ArgumentError("only fixed steps (adaptive = false) are supported, as in the reference"))
    callback === nothing || callback isa GB300Callback ||
        throw(ArgumentError("use GB300Backend.get_simulation_callback for the fused path"))
    max_stages = hasfield(typeof(alg), :max_stages) ? Int(getfield(alg, :max_stages)) : 100
    t0, t1 = Float64.(prob.tspan)
    nsteps = steps_for(t1, t0, dt, "final")
    nsteps <= maxiters || error("nsteps $nsteps exceeds maxiters")
    s, cov = Ref{Cint}(0), Ref{Cint}(0)
    check(ccall(fn(:gw_rock2_stages), Cint, (Ptr{Cvoid}, Cdouble, Cint, Ref{Cint}, Ref{Cint}),
                cache.ctx, dt, max_stages, s, cov))
    u0 = prob.u0
    check(ccall(fn(:gw_set_field), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, u0))
    check(ccall(fn(:gw_reset_energy), Cint, (Ptr{Cvoid},), cache.ctx))
    stops = Set([nsteps])
    save_steps = Dict{Int,Float64}()
    if callback !== nothing
        for ts in callback.saveat
            t0 <= ts <= t1 && get!(save_steps, steps_for(ts, t0, dt, "saveat"), ts)
        end
        union!(stops, keys(save_steps))
        callback.print_every_n > 0 && union!(stops, callback.print_every_n:callback.print_every_n:nsteps)
    end
    # saved fields: Float32 snapshots converted on the device and copied to
    # pinned host buffers on a second stream while the next steps run
    # (gw_snapshot); handed to the callback once every copy has landed
    snaps = Tuple{Float64,Ptr{Cfloat}}[]
    function snapshot(ts)
        ptr = Ref{Ptr{Cfloat}}(C_NULL)
        check(ccall(fn(:gw_snapshot_host_alloc), Cint, (Ptr{Cvoid}, Ref{Ptr{Cfloat}}), cache.ctx, ptr))
        push!(snaps, (ts, ptr[]))
        check(ccall(fn(:gw_snapshot), Cint, (Ptr{Cvoid}, Ptr{Cfloat}), cache.ctx, ptr[]))
    end
    haskey(save_steps, 0) && snapshot(save_steps[0])
    series = Matrix{Float64}[]
    done = 0
    for stop in sort!(collect(filter(>(0), stops)))
        n = stop - done
        check(ccall(fn(:gw_step), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Cint, Cint),
                    cache.ctx, t0 + done * dt, dt, n, max_stages))
        buf = zeros(Float64, cache.N_bh, n)
        check(ccall(fn(:gw_get_outlet_series), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint), cache.ctx, buf, n))
        push!(series, permutedims(buf))
        done = stop
        if callback !== nothing
            callback.print_every_n > 0 && done % callback.print_every_n == 0 && print_step(done, t0 + done * dt)
            haskey(save_steps, done) && snapshot(save_steps[done])
        end
    end
    if !isempty(snaps)
        check(ccall(fn(:gw_snapshot_wait), Cint, (Ptr{Cvoid},), cache.ctx))
        for (ts, ptr) in snaps
            u = copy(unsafe_wrap(Array, ptr, (cache.Nz, cache.Ny, cache.Nx)))
            check(ccall(fn(:gw_snapshot_host_free), Cint, (Ptr{Cvoid}, Ptr{Cfloat}), cache.ctx, ptr))
            save!(callback, ts, u)
        end
    end
    energy = zeros(Float64, cache.N_bh)
    check(ccall(fn(:gw_get_energy), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, energy))
    u_end = similar(u0)
    check(ccall(fn(:gw_get_field), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, u_end))
    outlet_series = isempty(series) ? zeros(0, cache.N_bh) : reduce(vcat, series)
    return GB300Solution([t0, t1], [u0, u_end], t0 .+ dt .* (1:nsteps), outlet_series, energy,
                         Int(s[]), :Success)
end

"Outlet temperature after each step of the last `solve` (rows) per borehole (columns)."
outlet_series(sol::GB300Solution) = sol.T_outlet

# ---------------------------------------------------------------------------
# gradients: the adjoint kernels behind a ChainRulesCore rrule

"""
    AdjointDesign(; backend, gridx, gridy, gridz, materials, boreholes, inlet_model, T0, dt,
                  nsteps, max_stages = 100, checkpoint_every = 64)

Everything but the differentiated parameters of an extracted-heat objective.
The parameters are `p = [k_rock_layers...; ṁ per borehole...; inlet parameter]`
(the inlet parameter is `T_const` of a `ConstantInlet` or `ΔT` of a
`HeatExchangerInlet`), the order of the library's gradient.
"""
Base.@kwdef struct AdjointDesign
    backend::GB300 = GB300()
    gridx::Vector{Float64}
    gridy::Vector{Float64}
    gridz::Vector{Float64}
    materials::Any
    boreholes::Any
    inlet_model::Any
    T0::Array{Float64,3}
    dt::Float64
    nsteps::Int
    max_stages::Int = 100
    checkpoint_every::Int = 64
end

n_layers(m::GeothermalWells.StratifiedMaterialProperties) = length(m.k_rock_layers)
n_layers(::GeothermalWells.HomogenousMaterialProperties) = 1

"The design's parameter vector p (layer conductivities, flow rates, inlet parameter)."
function parameters(d::AdjointDesign)
    m = d.materials
    k = m isa GeothermalWells.StratifiedMaterialProperties ? collect(Float64, m.k_rock_layers) : [m.k_rock]
    q = Float64[b.ṁ for b in d.boreholes]
    return vcat(k, q, inlet_kind(d.inlet_model)[2])
end

"The design's materials, boreholes and inlet with the parameters p applied."
function with_parameters(d::AdjointDesign, p::AbstractVector)
    m, nl, nb = d.materials, n_layers(d.materials), length(d.boreholes)
    length(p) == nl + nb + 1 || throw(DimensionMismatch("p has $(length(p)) entries, expected $(nl + nb + 1)"))
    mats = m isa GeothermalWells.StratifiedMaterialProperties ?
        GeothermalWells.StratifiedMaterialProperties(Tuple(Float64.(p[1:nl])), m.rho_c_rock_layers,
                                                     m.layer_depths, m.k_water, m.rho_c_water, m.k_steel,
                                                     m.rho_c_steel, m.k_insulating, m.rho_c_insulating,
                                                     m.k_backfill, m.rho_c_backfill) :
        GeothermalWells.HomogenousMaterialProperties(Float64(p[1]), m.rho_c_rock, m.k_water, m.rho_c_water,
                                                     m.k_steel, m.rho_c_steel, m.k_insulating,
                                                     m.rho_c_insulating, m.k_backfill, m.rho_c_backfill)
    bhs = [GeothermalWells.Borehole{Float64}(b.xc, b.yc, b.h, b.r_inner, b.t_inner, b.r_outer, b.t_outer,
                                             b.r_backfill, p[nl + q], b.insulation_depth)
           for (q, b) in enumerate(d.boreholes)]
    inlet = d.inlet_model isa GeothermalWells.ConstantInlet ? GeothermalWells.ConstantInlet(Float64(p[end])) :
            d.inlet_model isa GeothermalWells.HeatExchangerInlet ? GeothermalWells.HeatExchangerInlet(Float64(p[end])) :
            throw(ArgumentError("the adjoint takes a ConstantInlet or a HeatExchangerInlet"))
    return mats, bhs, inlet
end

function design_cache(d::AdjointDesign, p)
    mats, bhs, inlet = with_parameters(d, p)
    return create_cache(; backend = d.backend, gridx = d.gridx, gridy = d.gridy, gridz = d.gridz,
                        materials = mats, boreholes = bhs, inlet_model = inlet)
end

"""
    extracted_heat(d::AdjointDesign, p) -> J

Time-integrated extracted heat Σ_b E_b [J] over `d.nsteps` fused steps from
`d.T0`, E_b = Σ_n ṁ_b c_w (T_out - T_in) dt (`gw_get_energy`).  Its `rrule`
takes the gradient from the library's adjoint (`gw_adjoint`: transposed line
solves, scatter-add advection adjoint, reversed ROCK2 stages, checkpoints
every `d.checkpoint_every` steps with recomputation between them).
"""
function extracted_heat(d::AdjointDesign, p::AbstractVector)
    cache = design_cache(d, p)
    try
        check(ccall(fn(:gw_set_field), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, d.T0))
        check(ccall(fn(:gw_reset_energy), Cint, (Ptr{Cvoid},), cache.ctx))
        check(ccall(fn(:gw_step), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Cint, Cint),
                    cache.ctx, 0.0, d.dt, d.nsteps, d.max_stages))
        E = zeros(Float64, cache.N_bh)
        check(ccall(fn(:gw_get_energy), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, E))
        return sum(E)
    finally
        destroy!(cache)
    end
end

function ChainRulesCore.rrule(::typeof(extracted_heat), d::AdjointDesign, p::AbstractVector)
    cache = design_cache(d, p)
    g = zeros(Float64, length(p))
    r = Ref{AdjointInfo}()
    try
        check(ccall(fn(:gw_set_field), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), cache.ctx, d.T0))
        check(ccall(fn(:gw_adjoint), Cint,
                    (Ptr{Cvoid}, Cdouble, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Ptr{Cdouble},
                     Ref{AdjointInfo}),
                    cache.ctx, d.dt, d.nsteps, d.max_stages, d.checkpoint_every, 1.0, 0.0, g, C_NULL, r))
    finally
        destroy!(cache)
    end
    pullback(ΔJ) = (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), ΔJ .* g)
    return r[].objective, pullback
end

end # module
