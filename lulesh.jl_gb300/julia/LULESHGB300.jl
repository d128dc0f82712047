# Julia binding of liblulesh_gb300 for LULESH.jl (single rank, one GPU).
#
# `GPUDomain(prob)` replaces `Domain(prob)`; `timeIncrement!`,
# `lagrangeLeapFrog`, `commRecv`, `commSend`, `commSBN` and
# `verifyAndWriteFinalOutput` get methods for it and it answers the
# properties the script reads (`sizeX/Y/Z`, `nodalMass`, `time`, `stoptime`,
# `cycle`, `deltatime`, `e`, ...), so examples/benchmark.jl:22-110 runs with
# only `Domain(prob)` replaced by `GPUDomain(prob)` (and `enzyme` false).
# Its loop, for example:
#
#     using LULESH, LULESHGB300
#     prob = LuleshProblem(num_iters, true, nx, nr, balance, cost, Vector, Float64, nothing)
#     domain = GPUDomain(prob)
#     while domain.time < domain.stoptime
#         timeIncrement!(domain)
#         lagrangeLeapFrog(domain)
#         domain.cycle >= num_iters && break
#     end
#     verifyAndWriteFinalOutput(elapsed, domain, nx, 1)
#
# Scalars (`domain.time`, `domain.hgcoef`, ...) and fields (`domain.e`,
# `domain.x`, ...) read through to the device; a field read returns a host
# copy, `setproperty!` of a field uploads it.
module LULESHGB300

using LULESH

export GPUDomain, LuleshGPUError, GPUAdjoint, energy_gradient!, save_state, load_state!, set_overlap!

const libpath = get(ENV, "LULESH_GB300_LIB",
                    joinpath(@__DIR__, "..", "lib", "liblulesh_gb300.so"))

# lulesh_params / lulesh_scalars of include/lulesh_gb300.h
struct Params
    nx::Int32
    nr::Int32
    balance::Int32
    cost::Int32
    mode::Int32
    region_reps::Int32
    keep_aux::Int32
    device::Int32
    region_seed::UInt64
end

struct Scalars
    time::Float64
    deltatime::Float64
    dtcourant::Float64
    dthydro::Float64
    cycle::Int64
    status::Int32
    site::Int32
end

const FIELD_IDS = Dict{Symbol,Tuple{Int32,DataType}}()
let elem = (:e, :p, :q, :ql, :qq, :v, :volo, :delv, :vdov, :arealg, :ss, :elemMass, :vnew,
            :delv_xi, :delv_eta, :delv_zeta, :delx_xi, :delx_eta, :delx_zeta, :dxx, :dyy, :dzz),
    node = (:x, :y, :z, :xd, :yd, :zd, :xdd, :ydd, :zdd, :fx, :fy, :fz, :nodalMass),
    idx = (:nodelist, :lxim, :lxip, :letam, :letap, :lzetam, :lzetap, :symmX, :symmY, :symmZ,
           :nodeElemCount, :nodeElemStart, :nodeElemCornerList, :matElemlist, :regNumList,
           :regElemlist, :regCSR, :regReps, :regSorted, :regElemSize)
    for (i, s) in enumerate(elem); FIELD_IDS[s] = (Int32(i - 1), Float64); end
    for (i, s) in enumerate(node); FIELD_IDS[s] = (Int32(31 + i), Float64); end
    for (i, s) in enumerate(idx); FIELD_IDS[s] = (Int32(63 + i), Int64); end
    FIELD_IDS[:elemBC] = (Int32(96), UInt32)
end

const SCALAR_IDS = Dict(s => Int32(i - 1) for (i, s) in enumerate((
    :dtfixed, :deltatimemultlb, :deltatimemultub, :stoptime, :dtmax, :dthydro, :dtcourant, :time,
    :deltatime, :u_cut, :hgcoef, :qstop, :monoq_max_slope, :monoq_limiter_mult, :e_cut, :p_cut,
    :ss4o3, :q_cut, :v_cut, :qlc_monoq, :qqc_monoq, :qqc, :eosvmax, :eosvmin, :pmin, :emin,
    :dvovmax, :refdens, :cycle)))

# the reference's error(...) messages per (status, site)
const MESSAGES = Dict((1, 1) => "Early Volume Error", (1, 2) => "Volume Error: Volume is negative",
                      (1, 3) => "Mid Volume Error", (1, 4) => "Volume Error: calcKinematicsForElems",
                      (1, 5) => "Volume Error :2157", (1, 6) => "Volume Error :2887",
                      (1, 7) => "Volume Error :2908", (2, 0) => "QStopError", (3, 0) => "Error")

struct LuleshGPUError <: Exception
    msg::String
    status::Int32
end
Base.showerror(io::IO, e::LuleshGPUError) = print(io, e.msg)

mutable struct GPUDomain
    handle::Ptr{Cvoid}
    nx::Int
    # blocks_per_edge = tp > 1: the tp^3-rank decomposition of the (tp*nx)^3
    # mesh as blocks of one GPU handle (lulesh_create_blocks)
    function GPUDomain(prob::LuleshProblem; mode::Integer=0, device::Integer=0, keep_aux::Bool=false,
                       blocks_per_edge::Integer=1)
        prob.structured || error("Reading unstructured mesh is currently missing in the Julia version of LULESH.")
        p = Ref{Params}()
        ccall((:lulesh_default_params, libpath), Cvoid, (Ptr{Params}, Int32), p, prob.nx)
        p[] = Params(prob.nx, prob.nr, prob.balance, prob.cost, mode, 0, keep_aux, device, 0)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = blocks_per_edge > 1 ?
            ccall((:lulesh_create_blocks, libpath), Cint, (Ptr{Params}, Int32, Ptr{Ptr{Cvoid}}), p,
                  Int32(blocks_per_edge), h) :
            ccall((:lulesh_create, libpath), Cint, (Ptr{Params}, Ptr{Ptr{Cvoid}}), p, h)
        rc == 0 || throw(LuleshGPUError("Domain(prob) failed with status $rc", rc))
        d = new(h[], prob.nx)
        finalizer(d) do x
            x.handle == C_NULL || ccall((:lulesh_destroy, libpath), Cint, (Ptr{Cvoid},), x.handle)
            x.handle = C_NULL
        end
        return d
    end
end

function step_error(d::GPUDomain, rc)
    s = Ref{Scalars}()
    ccall((:lulesh_get_scalars, libpath), Cint, (Ptr{Cvoid}, Ptr{Scalars}), getfield(d, :handle), s)
    key = (Int(rc), rc == 1 ? Int(s[].site) : 0)
    throw(LuleshGPUError(get(MESSAGES, key, "status $rc"), rc))
end

function LULESH.timeIncrement!(d::GPUDomain)
    rc = ccall((:lulesh_time_increment, libpath), Cint, (Ptr{Cvoid},), getfield(d, :handle))
    rc == 0 || step_error(d, rc)
    return nothing
end

function LULESH.lagrangeLeapFrog(d::GPUDomain)
    rc = ccall((:lulesh_lagrange_leapfrog, libpath), Cint, (Ptr{Cvoid},), getfield(d, :handle))
    rc == 0 || step_error(d, rc)
    return nothing
end

# examples/benchmark.jl's whole loop on the device (no per-cycle host sync)
function run!(d::GPUDomain, num_iters::Integer)
    s = Ref{Scalars}()
    rc = ccall((:lulesh_run, libpath), Cint, (Ptr{Cvoid}, Int64, Ptr{Scalars}),
               getfield(d, :handle), num_iters, s)
    rc == 0 || step_error(d, rc)
    return s[]
end

function Base.getproperty(d::GPUDomain, s::Symbol)
    s in (:handle, :nx) && return getfield(d, s)
    h = getfield(d, :handle)
    if haskey(SCALAR_IDS, s)
        v = Ref{Float64}()
        ccall((:lulesh_get_scalar, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), h, SCALAR_IDS[s], v)
        return s === :cycle ? Int(v[]) : v[]
    elseif haskey(FIELD_IDS, s)
        id, T = FIELD_IDS[s]
        n = Ref{Int64}()
        ccall((:lulesh_field_length, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Int64}), h, id, n)
        out = Vector{T}(undef, n[])
        rc = ccall((:lulesh_download_field, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Int64),
                   h, id, out, n[])
        rc == 0 || throw(LuleshGPUError("download of $s failed", rc))
        return out
    elseif s === :numElem || s === :numNode
        ne, nn = Ref{Int64}(), Ref{Int64}()
        ccall((:lulesh_sizes, libpath), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}), h, ne, nn)
        return s === :numElem ? Int(ne[]) : Int(nn[])
    elseif s in (:sizeX, :sizeY, :sizeZ)
        # a cube of edge nx on one rank (src/domain.jl:536-543)
        return getfield(d, :nx)
    elseif s === :comm
        return nothing
    end
    error("GPUDomain has no field $s")
end

# ---- the one-rank communication calls of examples/benchmark.jl:57-64 ----
# At one rank (comm === nothing) the reference's commRecv, commSend and
# commSBN return at once (src/comm.jl:18-23, 296-302, 776-780); these methods
# do the same for a GPUDomain, so the script's initial boundary exchange runs
# unchanged. A GPUDomain is always one rank: its nodal masses are complete.
LULESH.commRecv(::GPUDomain, msgType, xferFields, dx, dy, dz, doRecv, planeOnly) = nothing
LULESH.commSend(::GPUDomain, msgType, fields, dx, dy, dz, doSend, planeOnly) = nothing
LULESH.commSBN(::GPUDomain, fields) = nothing

function Base.setproperty!(d::GPUDomain, s::Symbol, v)
    h = getfield(d, :handle)
    if haskey(SCALAR_IDS, s)
        ccall((:lulesh_set_scalar, libpath), Cint, (Ptr{Cvoid}, Int32, Float64), h, SCALAR_IDS[s], v)
    elseif haskey(FIELD_IDS, s)
        id, T = FIELD_IDS[s]
        a = convert(Vector{T}, v)
        rc = ccall((:lulesh_upload_field, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Int64),
                   h, id, a, length(a))
        rc == 0 || throw(LuleshGPUError("upload of $s failed", rc))
    else
        setfield!(d, s, v)
    end
    return v
end

# ---- full-state files (lulesh_save_state / lulesh_load_state) ----
"Write the domain's step state (state fields and scalars) to `path`."
function save_state(d::GPUDomain, path::AbstractString)
    rc = ccall((:lulesh_save_state, libpath), Cint, (Ptr{Cvoid}, Cstring), getfield(d, :handle), path)
    rc == 0 || throw(LuleshGPUError("save_state($path): status $rc", rc))
    return path
end

"Load a state file written for the same problem into `d`."
function load_state!(d::GPUDomain, path::AbstractString)
    rc = ccall((:lulesh_load_state, libpath), Cint, (Ptr{Cvoid}, Cstring), getfield(d, :handle), path)
    rc == 0 || throw(LuleshGPUError("load_state!($path): status $rc", rc))
    return d
end

# ---- reverse-mode adjoint of a run (lulesh_adj_* of include/lulesh_gb300.h) ----
#
# The reference differentiates one lagrangeLeapFrog call with Enzyme
# (examples/benchmark.jl:48-52, 85-86); this differentiates whole runs with
# the library's hand-written adjoint kernels. The objective after the run is
# the energy within `radius` of the origin (element internal energy times
# mass plus nodal kinetic energy, masked by the initial mesh); `set_seed!`
# replaces it with linear weights on state fields.

struct AdjResult
    loss::Float64
    grad_hgcoef::Float64
    forward_ms::Float64
    reverse_ms::Float64
    cycles::Int64
    checkpoints::Int32
    status::Int32
    sweep::Int32      # 0 sequential, 1 overlapped on two tapes, 2 on one
    reserved::Int32
end

mutable struct GPUAdjoint
    handle::Ptr{Cvoid}
    domain::GPUDomain
    function GPUAdjoint(d::GPUDomain; radius::Real = 0.3, checkpoint_every::Integer = 20)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:lulesh_adj_create, libpath), Cint, (Ptr{Cvoid}, Float64, Int32, Ptr{Ptr{Cvoid}}),
                   getfield(d, :handle), Float64(radius), Int32(checkpoint_every), h)
        rc == 0 || throw(LuleshGPUError("adjoint: status $rc", rc))
        a = new(h[], d)
        finalizer(x -> x.handle == C_NULL || ccall((:lulesh_adj_destroy, libpath), Cint, (Ptr{Cvoid},), x.handle), a)
        return a
    end
end

"Linear objective weights for one state field (x y z xd yd zd e p q v ss)."
function set_seed!(a::GPUAdjoint, field::Symbol, w::Vector{Float64})
    rc = ccall((:lulesh_adj_set_seed, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int64),
               a.handle, FIELD_IDS[field][1], w, length(w))
    rc == 0 || throw(LuleshGPUError("seed $field: status $rc", rc))
    return a
end

clear_seeds!(a::GPUAdjoint) = (ccall((:lulesh_adj_clear_seeds, libpath), Cint, (Ptr{Cvoid},), a.handle); a)

"""
    set_overlap!(a, mode)

How the reverse sweep runs: `false`/0 each checkpoint segment's recompute
and then its transpose; `true`/1 (the default) the recompute of one segment
overlapped with the transpose of the segment after it, on two tapes where
the second fits, else on one; 2 overlapped on one tape. The `sweep` field of
the result tells which plan a gradient took.
"""
function set_overlap!(a::GPUAdjoint, mode::Union{Bool,Integer})
    m = Int32(mode)
    0 <= m <= 2 || throw(ArgumentError("overlap mode is 0, 1 or 2"))
    rc = ccall((:lulesh_adj_set_overlap, libpath), Cint, (Ptr{Cvoid}, Int32), a.handle, m)
    rc == 0 || throw(LuleshGPUError("overlap: status $rc", rc))
    return a
end

"""
    gradient!(a, num_cycles) -> AdjResult

Advances the domain by up to `num_cycles` cycles (timeIncrement! +
lagrangeLeapFrog each, stopping at stoptime) and computes the gradient of
the objective w.r.t. the state before the run; `grad(a, :e)` returns it per
field, the result holds dL/dhgcoef.
"""
function gradient!(a::GPUAdjoint, num_cycles::Integer)
    r = Ref{AdjResult}()
    rc = ccall((:lulesh_adj_gradient, libpath), Cint, (Ptr{Cvoid}, Int64, Ptr{AdjResult}),
               a.handle, Int64(num_cycles), r)
    rc == 0 || step_error(a.domain, rc)
    return r[]
end

function grad(a::GPUAdjoint, field::Symbol)
    id = FIELD_IDS[field][1]
    n = id >= 32 ? (getfield(a.domain, :nx) + 1)^3 : getfield(a.domain, :nx)^3
    out = Vector{Float64}(undef, n)
    rc = ccall((:lulesh_adj_get_gradient, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int64),
               a.handle, id, out, n)
    rc == 0 || throw(LuleshGPUError("gradient of $field: status $rc", rc))
    return out
end

"""
    energy_gradient!(d, e0, hgcoef, num_cycles; radius = 0.3, checkpoint_every = 20)
        -> (L, dL/de0, dL/dhgcoef)

Sets the domain's energy field to `e0` and hgcoef, runs `num_cycles` cycles
and returns the energy within `radius` of the origin with its gradient. The
domain is left at the final state; the other state fields are the domain's
own at the call.
"""
function energy_gradient!(d::GPUDomain, e0::Vector{Float64}, hgcoef::Real, num_cycles::Integer;
                          radius::Real = 0.3, checkpoint_every::Integer = 20)
    d.e = e0
    d.hgcoef = Float64(hgcoef)
    a = GPUAdjoint(d; radius = radius, checkpoint_every = checkpoint_every)
    r = gradient!(a, num_cycles)
    return r.loss, grad(a, :e), r.grad_hgcoef
end

# verifyAndWriteFinalOutput reads domain.cycle and domain.e[...] only
LULESH.verifyAndWriteFinalOutput(t, d::GPUDomain, nx, ranks) = begin
    e = d.e
    LULESH.verifyAndWriteFinalOutput(t, (cycle = d.cycle, e = e), nx, ranks)
end

end # module
