# CLMGB300ADExt — reverse-mode rules of the GB300 column solve for CLM.jl: Enzyme rules
# for the batched band and tridiagonal solves on CuArrays, and a ChainRulesCore rrule
# plus an Enzyme rule for one whole column step.  A second package extension, loaded
# when CLM, CUDA, ChainRulesCore and Enzyme are all present; it calls the ccall layer
# of CLMGB300Ext.
#
# Not run in this build environment (no Julia); written to the C header's contracts,
# which the Python tests exercise on the GPU (tests/test_gpu_adjoint_solvers.py,
# tests/test_gpu_adjoint_step.py).
#
# The solve rules follow the reference's conventions (src/infrastructure/enzyme_rules.jl):
#   band_solve! (:72-107): the augmented primal keeps what the reverse needs, the
#     reverse solves A^T lambda = xbar, adds lambda to rbar and -lambda x^T to the band
#     entries, and consumes xbar;
#   tridiagonal_solve! (:142-201): the same with the transposed tridiagonal bands
#     (sub = c[j-1], super = a[j+1]), and an inactive-u variant.
# Here the primal keeps the factorisation itself (LAPACK gbtrf's product form, written by
# clmgb_batched_band_solve_factor), so the reverse refactorises nothing.
module CLMGB300ADExt

using CLM
using CUDA
using ChainRulesCore
import Enzyme
import Enzyme.EnzymeRules: augmented_primal, reverse, AugmentedReturn
using Enzyme: Const, Duplicated

const G = Base.get_extension(CLM, :CLMGB300Ext)

const _Ann = Union{Const{<:CuArray}, Duplicated{<:CuArray}}
_dval(::Const) = nothing
_dval(x::Duplicated) = x.dval

# ---------------------------------------------------------------------------
# batched_band_solve! (band_diagonal.jl:179) on CuArrays
# ---------------------------------------------------------------------------
function augmented_primal(config, func::Const{typeof(CLM.batched_band_solve!)}, ::Type{RT},
                          tvector::Duplicated{<:CuArray{Float64,2}}, bmatrix::_Ann, rvector::_Ann,
                          jtop::Const, jbot::Const, mask::Const, kl::Const, ku::Const,
                          nlevsno_off::Const) where {RT}
    nc, nlev = size(tvector.val)
    lu = CUDA.zeros(Float64, nc, 2 * kl.val + ku.val + 1, nlev)
    piv = CUDA.zeros(UInt8, nc, nlev)
    G.band_factor_solve!(tvector.val, bmatrix.val, rvector.val, jtop.val, jbot.val, mask.val,
                         kl.val, ku.val, nlevsno_off.val, lu, piv)
    # the solution (x in Abar -= lambda x^T) and the factorisation
    return AugmentedReturn(nothing, nothing, (copy(tvector.val), lu, piv))
end

function reverse(config, func::Const{typeof(CLM.batched_band_solve!)}, ::Type{RT}, tape,
                 tvector::Duplicated{<:CuArray{Float64,2}}, bmatrix::_Ann, rvector::_Ann,
                 jtop::Const, jbot::Const, mask::Const, kl::Const, ku::Const, nlevsno_off::Const) where {RT}
    x, lu, piv = tape
    # lambda = A^-T xbar; rbar += lambda; bbar -= lambda x^T in band; xbar consumed
    G.band_solve_adjoint!(x, tvector.dval, lu, piv, _dval(bmatrix), _dval(rvector), jtop.val, jbot.val,
                          mask.val, kl.val, ku.val, nlevsno_off.val)
    return (nothing, nothing, nothing, nothing, nothing, nothing, nothing, nothing, nothing)
end

# ---------------------------------------------------------------------------
# tridiagonal_multi! (tridiagonal.jl:129) on CuArrays
# ---------------------------------------------------------------------------
function augmented_primal(config, func::Const{typeof(CLM.tridiagonal_multi!)}, ::Type{RT},
                          u::Duplicated{<:CuArray{Float64,2}}, a::_Ann, b::_Ann, c::_Ann, r::_Ann,
                          jtop::Const, mask::Const, ncols::Const, nlevs::Const) where {RT}
    func.val(u.val, a.val, b.val, c.val, r.val, jtop.val, mask.val, ncols.val, nlevs.val)
    # the solution and the bands: the caller may overwrite a/b/c/r before the reverse
    return AugmentedReturn(nothing, nothing, (copy(u.val), copy(a.val), copy(b.val), copy(c.val)))
end

function reverse(config, func::Const{typeof(CLM.tridiagonal_multi!)}, ::Type{RT}, tape,
                 u::Duplicated{<:CuArray{Float64,2}}, a::_Ann, b::_Ann, c::_Ann, r::_Ann,
                 jtop::Const, mask::Const, ncols::Const, nlevs::Const) where {RT}
    x, a0, b0, c0 = tape
    G.tridiagonal_adjoint!(x, a0, b0, c0, u.dval, _dval(a), _dval(b), _dval(c), _dval(r), jtop.val, mask.val,
                           ncols.val, nlevs.val)
    return (nothing, nothing, nothing, nothing, nothing, nothing, nothing, nothing, nothing)
end

# u inactive: nothing downstream reads a derivative of the solution
function augmented_primal(config, func::Const{typeof(CLM.tridiagonal_multi!)}, ::Type{RT},
                          u::Const{<:CuArray{Float64,2}}, a::_Ann, b::_Ann, c::_Ann, r::_Ann,
                          jtop::Const, mask::Const, ncols::Const, nlevs::Const) where {RT}
    func.val(u.val, a.val, b.val, c.val, r.val, jtop.val, mask.val, ncols.val, nlevs.val)
    return AugmentedReturn(nothing, nothing, nothing)
end

reverse(config, func::Const{typeof(CLM.tridiagonal_multi!)}, ::Type{RT}, tape,
        u::Const{<:CuArray{Float64,2}}, a::_Ann, b::_Ann, c::_Ann, r::_Ann,
        jtop::Const, mask::Const, ncols::Const, nlevs::Const) where {RT} =
    (nothing, nothing, nothing, nothing, nothing, nothing, nothing, nothing, nothing)

# ---------------------------------------------------------------------------
# One whole column step: soil_temperature!, set_soil_water_fractions!, soil_water!
# (clmgb_column_step_logged / clmgb_column_step_vjp_logged), the counterpart of the
# reference's _reverse_step_into! (canopy_fluxes_reverse.jl:447-465).
#
# A StepContext holds the field buffers of the model's arrays (built once by
# CLMGB300Ext.soiltemp_fields / soilwater_fields), its bounds and configuration, and a
# substep log.  The differentiated state is
#   x = (t_soisno, h2osoi_liq, h2osoi_ice, t_grnd, t_h2osfc)        (CuArrays of the model)
# with the hydraulic parameters theta = (watsat, bsw, sucsat, hksat) ([nc, nlevsoi] each)
# and the step's qcharge as an extra output.
# ---------------------------------------------------------------------------
struct StepContext
    ft_buf::Vector{UInt8}
    fw_buf::Vector{UInt8}
    b::G.Bounds
    cfg::G.SwmConfig
    dtime::Float64
    snow_method::Int32
    t_ssbef::CuArray{Float64,2}
    t_h2osfc_bef::CuArray{Float64,1}
    log::NamedTuple
    state::NamedTuple        # the model's arrays the buffers point to: x fields, qcharge, theta fields
    nlevsoi::Int
end

const XFIELDS = (:t_soisno, :h2osoi_liq, :h2osoi_ice, :t_grnd, :t_h2osfc)
const PFIELDS = (:watsat, :bsw, :sucsat, :hksat)

# theta lives in the first nlevsoi rows of the [nc, nlevgrnd] soil-state matrices
set_params!(ctx, θ) = foreach(p -> copyto!(view(getfield(ctx.state, p), :, 1:ctx.nlevsoi), getfield(θ, p)), PFIELDS)
set_state!(ctx, x) = foreach(k -> copyto!(getfield(ctx.state, k), getfield(x, k)), XFIELDS)
snapshot(ctx) = NamedTuple{XFIELDS}(map(k -> copy(getfield(ctx.state, k)), XFIELDS))

function forward!(ctx::StepContext)
    G.column_step_logged!(ctx.ft_buf, ctx.fw_buf, ctx.b, ctx.cfg, ctx.dtime, ctx.snow_method, ctx.t_ssbef,
                          ctx.t_h2osfc_bef, ctx.log)
end

# the step's vector-Jacobian product from the input state x, parameters θ: lam holds
# the adjoints of the outputs on entry and those of the inputs on return; grad
# accumulates the parameters' adjoints
function pullback!(ctx::StepContext, x, θ, lam, grad)
    set_state!(ctx, x)
    set_params!(ctx, θ)
    G.column_step_vjp_logged!(ctx.ft_buf, ctx.fw_buf, ctx.b, ctx.cfg, ctx.dtime, ctx.snow_method, ctx.t_ssbef,
                              ctx.t_h2osfc_bef, lam, grad, ctx.log)
end

"""
    column_step(ctx, x, θ) -> (x_next, qcharge)

One column step from the state `x` with hydraulic parameters `θ`, on the model's arrays
(which it leaves holding the step's output).  Differentiable: ChainRulesCore.rrule and
an Enzyme rule of `column_step!` below.
"""
function column_step(ctx::StepContext, x, θ)
    set_state!(ctx, x)
    set_params!(ctx, θ)
    forward!(ctx)
    return snapshot(ctx), copy(ctx.state.qcharge)
end

function ChainRulesCore.rrule(::typeof(column_step), ctx::StepContext, x, θ)
    y = column_step(ctx, x, θ)
    function column_step_pullback(ȳ)
        x̄n, q̄ = unthunk(ȳ)
        nc = length(ctx.state.t_grnd)
        z(a) = fill!(similar(a), 0.0)
        g(k, a) = (x̄n isa AbstractZero || getfield(x̄n, k) isa AbstractZero) ? z(a) : copy(getfield(x̄n, k))
        lam = (t_soisno = g(:t_soisno, x.t_soisno), h2osoi_liq = g(:h2osoi_liq, x.h2osoi_liq),
               h2osoi_ice = g(:h2osoi_ice, x.h2osoi_ice), t_grnd = g(:t_grnd, x.t_grnd),
               t_h2osfc = g(:t_h2osfc, x.t_h2osfc),
               qcharge = q̄ isa AbstractZero ? CUDA.zeros(Float64, nc) : copy(q̄),
               forc_lwrad = CUDA.zeros(Float64, nc))
        grad = NamedTuple{PFIELDS}(map(p -> CUDA.zeros(Float64, nc, ctx.nlevsoi), PFIELDS))
        pullback!(ctx, x, θ, lam, grad)
        x̄ = Tangent{typeof(x)}(; t_soisno = lam.t_soisno, h2osoi_liq = lam.h2osoi_liq,
                                 h2osoi_ice = lam.h2osoi_ice, t_grnd = lam.t_grnd, t_h2osfc = lam.t_h2osfc)
        θ̄ = Tangent{typeof(θ)}(; grad...)
        return NoTangent(), NoTangent(), x̄, θ̄
    end
    return y, column_step_pullback
end

"""
    column_step!(ctx, x, θ)

The mutating form: advances the arrays of `x` (CuArrays of the model state) in place by
one step.  Its Enzyme rule tapes the input state; the reverse replays the step from it
with the shadows of `x` as the adjoints and accumulates the parameters' adjoints into
the shadows of `θ`.
"""
function column_step!(ctx::StepContext, x, θ)
    set_params!(ctx, θ)
    set_state!(ctx, x)
    forward!(ctx)
    foreach(k -> copyto!(getfield(x, k), getfield(ctx.state, k)), XFIELDS)
    nothing
end

function augmented_primal(config, func::Const{typeof(column_step!)}, ::Type{RT}, ctx::Const{StepContext},
                          x::Duplicated, θ::Duplicated) where {RT}
    x0 = NamedTuple{XFIELDS}(map(k -> copy(getfield(x.val, k)), XFIELDS))
    func.val(ctx.val, x.val, θ.val)
    return AugmentedReturn(nothing, nothing, x0)
end

function reverse(config, func::Const{typeof(column_step!)}, ::Type{RT}, x0, ctx::Const{StepContext},
                 x::Duplicated, θ::Duplicated) where {RT}
    c = ctx.val
    nc = length(c.state.t_grnd)
    # the shadows of x hold the adjoints of the step's output; the vjp turns them into
    # those of its input in place (the reference's _reverse_step_into! threads Enzyme's
    # shadow the same way), and adds the parameters' adjoints to θ's shadows
    lam = (t_soisno = x.dval.t_soisno, h2osoi_liq = x.dval.h2osoi_liq, h2osoi_ice = x.dval.h2osoi_ice,
           t_grnd = x.dval.t_grnd, t_h2osfc = x.dval.t_h2osfc, qcharge = CUDA.zeros(Float64, nc),
           forc_lwrad = CUDA.zeros(Float64, nc))
    grad = NamedTuple{PFIELDS}(map(p -> getfield(θ.dval, p), PFIELDS))
    pullback!(c, x0, θ.val, lam, grad)
    return (nothing, nothing, nothing)
end

end # module
