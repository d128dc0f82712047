# ChainRulesCore rule for LULESHGB300's differentiable run (include after
# `using ChainRulesCore, LULESHGB300`): Zygote, Diffractor or any
# ChainRules-aware AD then differentiates through a GPU run with the
# library's adjoint instead of tracing the step.
#
#     ic = initial_condition(GPUDomain(prob))   # the state the runs start from
#     L = energy_after(ic, e0, hgcoef, 200)     # differentiable in e0 and hgcoef
#
# energy_after restores the captured state, puts e0 and hgcoef in, runs the
# cycles and returns the energy within `radius` of the origin; its rrule gets
# the value and both gradients from one lulesh_adj_gradient call.
module LULESHGB300ChainRules

using ChainRulesCore
using LULESHGB300
using LULESHGB300: GPUDomain, GPUAdjoint, gradient!, grad

export initial_condition, energy_after

const STATE = (:x, :y, :z, :xd, :yd, :zd, :e, :p, :q, :v, :ss)
const SCALARS = (:time, :deltatime, :dtcourant, :dthydro, :cycle)

struct InitialCondition
    domain::GPUDomain
    fields::Dict{Symbol,Vector{Float64}}
    scalars::Dict{Symbol,Float64}
end

initial_condition(d::GPUDomain) =
    InitialCondition(d, Dict(f => getproperty(d, f) for f in STATE),
                     Dict(s => Float64(getproperty(d, s)) for s in SCALARS))

function restore!(ic::InitialCondition, e0, hgcoef)
    d = ic.domain
    for (f, v) in ic.fields
        setproperty!(d, f, v)
    end
    for (s, v) in ic.scalars
        setproperty!(d, s, v)
    end
    d.e = e0
    d.hgcoef = Float64(hgcoef)
    return d
end

function _loss(a::GPUAdjoint)
    v = Ref(0.0)
    rc = ccall((:lulesh_adj_loss, LULESHGB300.libpath), Cint, (Ptr{Cvoid}, Ptr{Float64}), a.handle, v)
    rc == 0 || error("lulesh_adj_loss: status $rc")
    return v[]
end

function energy_after(ic::InitialCondition, e0::Vector{Float64}, hgcoef::Real, num_cycles::Integer;
                      radius::Real = 0.3, checkpoint_every::Integer = 20)
    d = restore!(ic, e0, hgcoef)
    LULESHGB300.run!(d, Int(ic.scalars[:cycle]) + num_cycles)
    return _loss(GPUAdjoint(d; radius = radius))
end

function ChainRulesCore.rrule(::typeof(energy_after), ic::InitialCondition, e0::Vector{Float64},
                              hgcoef::Real, num_cycles::Integer; radius::Real = 0.3,
                              checkpoint_every::Integer = 20)
    d = restore!(ic, e0, hgcoef)
    a = GPUAdjoint(d; radius = radius, checkpoint_every = checkpoint_every)
    r = gradient!(a, num_cycles)
    ge, ghg = grad(a, :e), r.grad_hgcoef
    energy_after_pullback(ȳ) = (NoTangent(), NoTangent(), ȳ .* ge, ȳ * ghg, NoTangent())
    return r.loss, energy_after_pullback
end

end # module
