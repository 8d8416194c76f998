#
# rrule.jl -- ChainRulesCore.rrule of HyperelasticCUDA.evolve, so that Zygote (or
# any ChainRules-based AD) differentiates a run of the GPU step through the
# hand-written device adjoint: the forward pass records checkpoints every K steps
# (hyp_adjoint_record), the pullback steps the adjoint back (hyp_adjoint).
# Load after HyperelasticCUDA.jl when ChainRulesCore is available.
#
using ChainRulesCore
using .HyperelasticCUDA: ConfigC, Barton2009C, Solver, upload!, download, record!, adjoint, evolve

function ChainRulesCore.rrule(::typeof(evolve), cfg::ConfigC, Q0::Matrix{Float64}, n_steps::Integer; K::Integer=50)
  s = Solver(cfg)
  upload!(s, Q0)
  record!(s, n_steps; K=K)
  Q = download(s)
  function evolve_pullback(dQ)
    dQ0, (db0sq, dk0) = adjoint(s, Matrix{Float64}(unthunk(dQ)))
    # b0sq = b0^2 and k0 = c0^2 - 4/3 b0^2 (EquationsOfState.jl:111-112) in terms of (b0, c0)
    e = cfg.eos1
    db0 = db0sq * 2e.b0 + dk0 * (-8 / 3 * e.b0)
    dc0 = dk0 * 2e.c0
    deos = Tangent{Barton2009C}(; b0=db0, c0=dc0)
    (NoTangent(), Tangent{ConfigC}(; eos1=deos), dQ0, NoTangent())
  end
  Q, evolve_pullback
end
