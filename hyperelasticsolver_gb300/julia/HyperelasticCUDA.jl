#
# HyperelasticCUDA.jl -- Julia binding of libhyperelastic_cuda.so.
#
# Keeps the reference's module and function names (Strains, EquationsOfState,
# HyperelasticityMPh, NumFluxes) and forwards array-of-cells calls to the C ABI in
# include/hyperelastic.h. Arrays are Matrix{Float64}(n, k): one row per cell, which
# is exactly the ABI's structure-of-arrays layout. A driver replaces the per-cell
# loops of main.jl:202-241 by a Solver (hyp_create / hyp_upload / hyp_step).
#
module HyperelasticCUDA

const libhyp = get(ENV, "HYP_LIB", joinpath(@__DIR__, "..", "_build", "libhyperelastic_cuda.so"))

struct Barton2009C
  rho0::Float64; c0::Float64; cv::Float64; t0::Float64
  b0::Float64; alpha::Float64; beta::Float64; gamma::Float64
end
Barton2009C(; _rho0=8.93, _c0=4.6, _cv=3.9e-4, _t0=300, _b0=2.1, _alpha=1, _beta=3, _gamma=2) =
  Barton2009C(_rho0, _c0, _cv, _t0, _b0, _alpha, _beta, _gamma)

"Hank2016 parameters (EquationsOfState.jl:305-326); function-level evaluators only."
struct Hank2016C
  rho0::Float64; mu::Float64; gamma::Float64; pres_inf::Float64; a::Float64
end
Hank2016C() = Hank2016C(2.7, 26e9, 3.4, 21.5e9, 0.5)

struct ConfigC
  n_cells::Int64; model::Cint; flux::Cint; bc::Cint; precision::Cint
  x_length::Float64; cfl::Float64; eos1::Barton2009C; eos2::Barton2009C
end

const HYP_MODEL_SINGLE, HYP_MODEL_MULTI = Cint(1), Cint(2)
const HYP_FLUX_RUSANOV, HYP_FLUX_LXF, HYP_FLUX_HLL = Cint(0), Cint(1), Cint(2)
const HYP_BC_FROZEN, HYP_BC_TRANSMISSIVE = Cint(0), Cint(1)
const HYP_RELAX_NONE = Cint(0)
const HYP_RELAX_PRESSURE = Cint(1)
const HYP_RELAX_MECHANICAL = Cint(2)
const HYP_PREC_FP64, HYP_PREC_MIXED = Cint(0), Cint(1)

struct HypError <: Exception
  code::Cint
  msg::String
end
check(rc, what, ctx=C_NULL) = rc == 0 ? nothing :
  throw(HypError(rc, what * ": " * unsafe_string(ccall((:hyp_last_error, libhyp), Cstring, (Ptr{Cvoid},), ctx))))

config(eos, model; n=3, flux=HYP_FLUX_RUSANOV, bc=HYP_BC_FROZEN, prec=HYP_PREC_FP64, X=1.0, cfl=0.5) =
  ConfigC(n, model, flux, bc, prec, X, cfl, eos isa Tuple ? eos[1] : eos, eos isa Tuple ? eos[2] : eos)

module Strains
  import ..libhyp, ..check
  "finger(A::Matrix{Float64}(n, 9)) -> G (Strains.jl:26-32)"
  function finger(A::Matrix{Float64})
    G = similar(A)
    check(ccall((:hyp_eval_finger, libhyp), Cint, (Ptr{Float64}, Ptr{Float64}, Int64), A, G, size(A, 1)), "finger")
    G
  end
  function invariants(G::Matrix{Float64})
    out = Matrix{Float64}(undef, size(G, 1), 3)
    check(ccall((:hyp_eval_invariants, libhyp), Cint, (Ptr{Float64}, Ptr{Float64}, Int64), G, out, size(G, 1)), "invariants")
    out
  end
end

module EquationsOfState
  import ..libhyp, ..check, ..Barton2009C
  for (jl, c, k) in ((:energy, :hyp_eval_energy, 1), (:entropy, :hyp_eval_entropy, 1),
                     (:stress, :hyp_eval_stress, 9), (:acoustic, :hyp_eval_acoustic, 9))
    @eval function $jl(eos::Barton2009C, s::Vector{Float64}, M::Matrix{Float64})
      out = Matrix{Float64}(undef, size(M, 1), $k)
      e = Ref(eos)
      check(ccall(($(QuoteNode(c)), libhyp), Cint, (Ref{Barton2009C}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                  e, s, M, out, size(M, 1)), $(string(jl)))
      $k == 1 ? vec(out) : out
    end
  end
  """acoustic(eos, ent, F, n) for one direction per cell (dir: (m, 3)) (EquationsOfState.jl:223-246)"""
  function acoustic(eos::Barton2009C, s::Vector{Float64}, M::Matrix{Float64}, dir::Matrix{Float64})
    out = Matrix{Float64}(undef, size(M, 1), 9)
    check(ccall((:hyp_eval_acoustic_dir, libhyp), Cint,
                (Ref{Barton2009C}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                Ref(eos), s, M, dir, out, size(M, 1)), "acoustic")
    out
  end
  """stress(eos, den, e_int, F) (EquationsOfState.jl:162-176): the entropy from e_int, den as given"""
  function stress(eos::Barton2009C, den::Vector{Float64}, e_int::Vector{Float64}, M::Matrix{Float64})
    out = Matrix{Float64}(undef, size(M, 1), 9)
    check(ccall((:hyp_eval_stress_den, libhyp), Cint,
                (Ref{Barton2009C}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                Ref(eos), den, e_int, M, out, size(M, 1)), "stress")
    out
  end
  """acoustic(eos, P, n) (EquationsOfState.jl:192-221): P one phase's primitives (m, 15), dir (m, 3)"""
  function acoustic(eos::Barton2009C, P::Matrix{Float64}, dir::Matrix{Float64})
    out = Matrix{Float64}(undef, size(P, 1), 9)
    check(ccall((:hyp_eval_acoustic_prim, libhyp), Cint,
                (Ref{Barton2009C}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64), Ref(eos), P, dir, out, size(P, 1)),
          "acoustic")
    out
  end
end

module Hank
  import ..libhyp, ..check, ..Hank2016C
  # energy(eos, den, pres, G), pressure(eos, den, e_int, i), stress(eos, den, pres, F) over n cells
  for (jl, c, k_in, k_out) in ((:energy, :hyp_eval_hank2016_energy, 9, 1),
                               (:pressure, :hyp_eval_hank2016_pressure, 3, 1),
                               (:stress, :hyp_eval_hank2016_stress, 9, 9))
    @eval function $jl(eos::Hank2016C, x::Vector{Float64}, y::Vector{Float64}, M::Matrix{Float64})
      out = Matrix{Float64}(undef, size(M, 1), $k_out)
      check(ccall(($(QuoteNode(c)), libhyp), Cint,
                  (Ref{Hank2016C}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                  Ref(eos), x, y, M, out, size(M, 1)), $(string(jl)))
      $k_out == 1 ? vec(out) : out
    end
  end
end

module HyperelasticityMPh
  import ..libhyp, ..check, ..config, ..ConfigC, ..HYP_MODEL_MULTI
  for (jl, c, k) in ((:cons2prim_mph, :hyp_eval_cons2prim, 30), (:prim2cons_mph, :hyp_eval_prim2cons, 30),
                     (:flux_mph, :hyp_eval_flux, 30), (:get_eigvals, :hyp_eval_eigvals, 12))
    @eval function $jl(eos, Q::Matrix{Float64})
      out = Matrix{Float64}(undef, size(Q, 1), $k)
      cfg = Ref(config(eos, HYP_MODEL_MULTI))
      check(ccall(($(QuoteNode(c)), libhyp), Cint, (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Int64),
                  cfg, Q, out, size(Q, 1)), $(string(jl)))
      out
    end
  end
  """noncons_flux(eos, Q) (HyperelasticityMPh.jl:178-250): B per cell as an (n, 30, 30) array,
  whose only non-zero columns are 1 and 16 (the device computes just those two)."""
  function noncons_flux(eos, Q::Matrix{Float64})
    n = size(Q, 1)
    bcol = Matrix{Float64}(undef, n, 30)
    check(ccall((:hyp_eval_noncons, libhyp), Cint, (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Int64),
                Ref(config(eos, HYP_MODEL_MULTI)), Q, bcol, n), "noncons_flux")
    B = zeros(n, 30, 30)
    B[:, 1:15, 1] .= bcol[:, 1:15]
    B[:, 16:30, 16] .= bcol[:, 16:30]
    B
  end
  "get_eigvals(eos, Q, n) along one direction per cell (dir: (m, 3)), 12 speeds per cell"
  function get_eigvals(eos, Q::Matrix{Float64}, dir::Matrix{Float64})
    out = Matrix{Float64}(undef, size(Q, 1), 12)
    check(ccall((:hyp_eval_eigvals_dir, libhyp), Cint, (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                Ref(config(eos, HYP_MODEL_MULTI)), Q, dir, out, size(Q, 1)), "get_eigvals")
    out
  end
end

module Hyperelasticity
  import ..libhyp, ..check, ..config, ..ConfigC, ..Barton2009C, ..HYP_MODEL_SINGLE
  # single-phase cells (n, 14): the per-phase functions of HyperelasticityMPh.jl at alpha = 1
  for (jl, c, k) in ((:cons2prim, :hyp_eval_cons2prim, 14), (:prim2cons, :hyp_eval_prim2cons, 14),
                     (:flux, :hyp_eval_flux, 14), (:get_eigvals, :hyp_eval_eigvals, 6))
    @eval function $jl(eos::Barton2009C, Q::Matrix{Float64})
      out = Matrix{Float64}(undef, size(Q, 1), $k)
      cfg = Ref(config(eos, HYP_MODEL_SINGLE))
      check(ccall(($(QuoteNode(c)), libhyp), Cint, (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Int64),
                  cfg, Q, out, size(Q, 1)), $(string(jl)))
      out
    end
  end
  "get_eigvals(eos, Q, n) along one direction per cell (dir: (m, 3)), 6 speeds per cell"
  function get_eigvals(eos::Barton2009C, Q::Matrix{Float64}, dir::Matrix{Float64})
    out = Matrix{Float64}(undef, size(Q, 1), 6)
    check(ccall((:hyp_eval_eigvals_dir, libhyp), Cint, (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                Ref(config(eos, HYP_MODEL_SINGLE)), Q, dir, out, size(Q, 1)), "get_eigvals")
    out
  end
  "prim2cons_vjp(eos, P, Qbar) -> (Pbar, (dL/db0sq, dL/dk0)): the pullback of prim2cons over n cells"
  function prim2cons_vjp(eos::Barton2009C, P::Matrix{Float64}, Qbar::Matrix{Float64})
    Pbar, eb = similar(P), zeros(2)
    check(ccall((:hyp_eval_prim2cons_vjp, libhyp), Cint,
                (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                Ref(config(eos, HYP_MODEL_SINGLE)), P, Qbar, Pbar, eb, size(P, 1)), "prim2cons_vjp")
    Pbar, (eb[1], eb[2])
  end
end

module NumFluxes
  import ..libhyp, ..check, ..config, ..ConfigC, ..HYP_MODEL_SINGLE, ..HYP_MODEL_MULTI, ..HYP_FLUX_LXF, ..HYP_FLUX_HLL
  """lxf(eos, Q_l, Q_r, lambda) (NumFluxes.jl:25-60): (cons, D-, D+). `eos` one Barton2009C:
  single-phase cells (n, 14); a pair: two-phase cells (n, 30) with the Gauss-Lobatto D+-."""
  function lxf(eos, Ql::Matrix{Float64}, Qr::Matrix{Float64}, lam::Vector{Float64})
    n = size(Ql, 1)
    cons, dm, dp = similar(Ql), similar(Ql), similar(Ql)
    cfg = Ref(eos isa Tuple ? config(eos, HYP_MODEL_MULTI; flux=HYP_FLUX_LXF) : config(eos, HYP_MODEL_SINGLE))
    check(ccall((:hyp_eval_lxf, libhyp), Cint,
                (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
                cfg, Ql, Qr, lam, cons, dm, dp, n), "lxf")
    cons, dm, dp
  end
  """hll(eos, Q_l, Q_r, eigvals) for two-phase cells (n, 30) (NumFluxes.jl:70-132): (zeros, D-, D+).
  eigvals = (eig_l, eig_r), each (n, 12): s_l from minimum(eig_l), s_r from maximum(eig_r)
  (NumFluxes.jl:90-91); `nothing` takes the two cells' own speeds, as main.jl:225 passes them."""
  function hll(eos::Tuple, Ql::Matrix{Float64}, Qr::Matrix{Float64}, eigvals=nothing)
    n = size(Ql, 1)
    dm, dp = similar(Ql), similar(Ql)
    cfg = Ref(config(eos, HYP_MODEL_MULTI; flux=HYP_FLUX_HLL))
    if eigvals === nothing
      check(ccall((:hyp_eval_hll, libhyp), Cint,
                  (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64), cfg, Ql, Qr, dm, dp, n),
            "hll")
    else
      el, er = eigvals
      check(ccall((:hyp_eval_hll_eigvals, libhyp), Cint,
                  (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                   Int64), cfg, Ql, Qr, el, er, dm, dp, n), "hll")
    end
    zeros(size(Ql)), dm, dp
  end
end

"Device-resident solver for one 1D problem: the time loop of main.jl:202-241."
mutable struct Solver
  h::Ptr{Cvoid}
  n::Int64
  nvar::Int
  function Solver(cfg::ConfigC)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hyp_create, libhyp), Cint, (Ref{ConfigC}, Ref{Ptr{Cvoid}}), Ref(cfg), r), "hyp_create")
    s = new(r[], cfg.n_cells, cfg.model == HYP_MODEL_SINGLE ? 14 : 30)
    finalizer(x -> ccall((:hyp_destroy, libhyp), Cint, (Ptr{Cvoid},), x.h), s)
  end
end
upload!(s::Solver, Q::Matrix{Float64}, t0=0.0) =
  check(ccall((:hyp_upload, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64, Cint, Float64), s.h, Q, s.n, s.nvar, t0),
        "hyp_upload", s.h)
"set_eos!(s, phase, eos): replace the Barton2009 parameters of phase 0 (or 1, two phases); state and t are kept"
set_eos!(s::Solver, phase::Integer, eos::Barton2009C) =
  check(ccall((:hyp_set_eos, libhyp), Cint, (Ptr{Cvoid}, Cint, Ref{Barton2009C}), s.h, phase, eos), "hyp_set_eos", s.h)
function download(s::Solver)
  Q = Matrix{Float64}(undef, s.n, s.nvar)
  check(ccall((:hyp_download, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64, Cint), s.h, Q, s.n, s.nvar),
        "hyp_download", s.h)
  Q
end
"step!(s; max_steps, T): advance while t < T (main.jl:202); returns (steps, t)"
function step!(s::Solver; max_steps::Integer=0, T::Float64=Inf)
  n, t = Ref{Cint}(0), Ref{Float64}(0.0)
  check(ccall((:hyp_step, libhyp), Cint, (Ptr{Cvoid}, Cint, Float64, Ref{Cint}, Ref{Float64}), s.h, max_steps, T, n, t),
        "hyp_step", s.h)
  (n[], t[])
end

"""step_times!(s; max_steps, T): step! that also returns the time after every step
taken (the Step / t / dt log line of main.jl:229-237), read back once at the end:
(steps, t, t_hist); dt of step j is t_hist[j] - t_hist[j-1]."""
function step_times!(s::Solver; max_steps::Integer, T::Float64=Inf)
  max_steps >= 1 || throw(ArgumentError("max_steps >= 1"))
  n, t = Ref{Cint}(0), Ref{Float64}(0.0)
  hist = Vector{Float64}(undef, max_steps)
  check(ccall((:hyp_step_times, libhyp), Cint, (Ptr{Cvoid}, Cint, Float64, Ref{Cint}, Ref{Float64}, Ptr{Float64}),
              s.h, max_steps, T, n, t, hist), "hyp_step_times", s.h)
  (n[], t[], hist[1:n[]])
end

# ---- queries, kernel choices and timing of a context ----
"error_cell(s): the first cell that raised NEG_DET / NONFINITE in the last call (-1: none)"
error_cell(s::Solver) = ccall((:hyp_error_cell, libhyp), Int64, (Ptr{Cvoid},), s.h)
"max_wavespeed(s): max over cells of |u1| + c_max of the current state (main.jl:204-211)"
function max_wavespeed(s::Solver)
  v = Ref{Float64}(0.0)
  check(ccall((:hyp_max_wavespeed, libhyp), Cint, (Ptr{Cvoid}, Ref{Float64}), s.h, v), "hyp_max_wavespeed", s.h)
  v[]
end
"get_time(s) -> (t, steps taken since the upload)"
function get_time(s::Solver)
  t, n = Ref{Float64}(0.0), Ref{Int64}(0)
  check(ccall((:hyp_get_time, libhyp), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Int64}), s.h, t, n), "hyp_get_time", s.h)
  (t[], n[])
end
set_profiling!(s::Solver, on::Bool) =
  check(ccall((:hyp_set_profiling, libhyp), Cint, (Ptr{Cvoid}, Cint), s.h, on), "hyp_set_profiling", s.h)
"last_timing(s): device ms of the last step! call, per-kernel sums when profiling is on"
function last_timing(s::Solver)
  tot, mc, mu = Ref{Float64}(0.0), Ref{Float64}(0.0), Ref{Float64}(0.0)
  nc, nu = Ref{Cint}(0), Ref{Cint}(0)
  check(ccall((:hyp_last_timing, libhyp), Cint,
              (Ptr{Cvoid}, Ref{Float64}, Ref{Float64}, Ref{Cint}, Ref{Float64}, Ref{Cint}), s.h, tot, mc, nc, mu, nu),
        "hyp_last_timing", s.h)
  (ms_total=tot[], ms_cell=mc[], n_cell=nc[], ms_update=mu[], n_update=nu[])
end
"set_mixed_kernel!(s, kind): mixed-precision kernel family, :tile (0), :tma (1, single-phase) or :pair (2, packed FP32 pairs)"
function set_mixed_kernel!(s::Solver, kind::Symbol)
  k = Dict(:tile => 0, :tma => 1, :pair => 2)[kind]
  check(ccall((:hyp_set_mixed_kernel, libhyp), Cint, (Ptr{Cvoid}, Cint), s.h, k), "hyp_set_mixed_kernel", s.h)
end
"set_wait_limit!(s, tries): poll budget of the persistent kernel's device waits (0: every wait times out)"
set_wait_limit!(s::Solver, tries::Integer) =
  check(ccall((:hyp_set_wait_limit, libhyp), Cint, (Ptr{Cvoid}, Cint), s.h, tries), "hyp_set_wait_limit", s.h)
"snapshot(s): cons2prim of the current state, one row per cell ([alpha, rho, u, S, A] per phase)"
function snapshot(s::Solver)
  P = Matrix{Float64}(undef, s.n, s.nvar == 14 ? 15 : 30)
  check(ccall((:hyp_snapshot, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}), s.h, P), "hyp_snapshot", s.h)
  P
end

# ---- initial conditions on the device (main.jl:99-123, HyperelasticityMPh.jl:275-426) ----
"initial_states(eos::Tuple, testcase) -> (Ql, Qr): the conservative 30-vectors of a reference test case"
function initial_states(eos::Tuple, testcase::Integer)
  Ql, Qr = zeros(30), zeros(30)
  check(ccall((:hyp_initial_states, libhyp), Cint, (Ref{ConfigC}, Cint, Ptr{Float64}, Ptr{Float64}),
              Ref(config(eos, HYP_MODEL_MULTI)), testcase, Ql, Qr), "hyp_initial_states")
  Ql, Qr
end
"initial_condition!(s, Ql, Qr): the two-state fill of main.jl:99-106, made the current state at t = 0"
initial_condition!(s::Solver, Ql::Vector{Float64}, Qr::Vector{Float64}) =
  check(ccall((:hyp_init_riemann, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), s.h, Ql, Qr),
        "hyp_init_riemann", s.h)
"initial_condition_tanh!(s, Ql, Qr, eps): the tanh volume-fraction profile of main.jl:110-123"
initial_condition_tanh!(s::Solver, Ql::Vector{Float64}, Qr::Vector{Float64}, eps::Float64) =
  check(ccall((:hyp_init_tanh, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64), s.h, Ql, Qr, eps),
        "hyp_init_tanh", s.h)

# ---- two-phase pressure relaxation (an extension: the reference has none) ----
"set_relaxation!(s, mode): HYP_RELAX_NONE (default), HYP_RELAX_PRESSURE or HYP_RELAX_MECHANICAL after each two-phase step"
set_relaxation!(s::Solver, mode::Integer) =
  check(ccall((:hyp_set_relaxation, libhyp), Cint, (Ptr{Cvoid}, Cint), s.h, mode), "hyp_set_relaxation", s.h)
"relax_pressure(eos, Q; velocity=false): instantaneous (velocity and) pressure relaxation of two-phase cells (n, 30)"
function relax_pressure(eos::Tuple, Q::Matrix{Float64}; velocity::Bool=false)
  out = similar(Q)
  check(ccall((:hyp_eval_relax, libhyp), Cint, (Ref{ConfigC}, Cint, Ptr{Float64}, Ptr{Float64}, Int64),
              Ref(config(eos, HYP_MODEL_MULTI)), velocity ? HYP_RELAX_MECHANICAL : HYP_RELAX_PRESSURE, Q, out,
              size(Q, 1)), "relax_pressure")
  out
end

# ---- domain decomposition: one slab per rank (a ghost cell at each inner end) ----
"""set_slab!(s, dx, left_ghost, right_ghost): make s one slab of a decomposed domain with
the global dx; hyp_step then refuses it (a slab steps with the global max)"""
set_slab!(s::Solver, dx::Float64, left_ghost::Bool, right_ghost::Bool) =
  check(ccall((:hyp_set_slab, libhyp), Cint, (Ptr{Cvoid}, Float64, Cint, Cint), s.h, dx, left_ghost, right_ghost),
        "hyp_set_slab", s.h)
"slab_local_max(s): the max wave speed over the cells the slab owns"
function slab_local_max(s::Solver)
  v = Ref{Float64}(0.0)
  check(ccall((:hyp_slab_local_max, libhyp), Cint, (Ptr{Cvoid}, Ref{Float64}), s.h, v), "hyp_slab_local_max", s.h)
  v[]
end
"slab_step!(s, lam_max): one step with the global max (MPI.Allreduce of slab_local_max over the ranks); returns t"
function slab_step!(s::Solver, lam_max::Float64)
  t = Ref{Float64}(0.0)
  check(ccall((:hyp_slab_step, libhyp), Cint, (Ptr{Cvoid}, Float64, Ref{Float64}), s.h, lam_max, t), "hyp_slab_step", s.h)
  t[]
end
"cell_record_size(s): bytes per cell record (112 FP64, 128 mixed)"
function cell_record_size(s::Solver)
  b = Ref{Cint}(0)
  check(ccall((:hyp_cell_record_size, libhyp), Cint, (Ptr{Cvoid}, Ref{Cint}), s.h, b), "hyp_cell_record_size", s.h)
  Int(b[])
end
"get_cells!(s, first, rec): records of cells first .. first + size(rec, 1) - 1 (0-based) into rec (count, rows)"
get_cells!(s::Solver, first::Integer, rec::AbstractMatrix) =
  check(ccall((:hyp_get_cells, libhyp), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}), s.h, first, size(rec, 1), rec),
        "hyp_get_cells", s.h)
"set_cells!(s, first, rec): store records (a neighbour's boundary cells as this slab's ghosts)"
set_cells!(s::Solver, first::Integer, rec::AbstractMatrix) =
  check(ccall((:hyp_set_cells, libhyp), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}), s.h, first, size(rec, 1), rec),
        "hyp_set_cells", s.h)

# ---- caller-owned device memory and page-locked host memory ----
"""step_noalloc!(cfg, d_in, d_out, n_steps, t0; stream): single-phase FP64 steps on device
buffers the caller owns (e.g. pointer(::CuArray)), allocating nothing; returns t.

`stream` is required: pass the stream that wrote `d_in` (with CUDA.jl,
`CUDA.stream().handle`). CUDA.jl queues its work on a task-local stream that need
not order against the legacy default stream (C_NULL), so C_NULL is only safe after
`CUDA.synchronize()`."""
function step_noalloc!(cfg::ConfigC, d_in::Ptr{Float64}, d_out::Ptr{Float64}, n_steps::Integer, t0::Float64;
                       stream::Ptr{Cvoid})
  t, cell = Ref{Float64}(0.0), Ref{Int64}(-1)
  rc = ccall((:hyp_step_noalloc_f64, libhyp), Cint,
             (Ref{ConfigC}, Ptr{Float64}, Ptr{Float64}, Int64, Cint, Float64, Ptr{Cvoid}, Ref{Float64}, Ref{Int64}),
             Ref(cfg), d_in, d_out, cfg.n_cells, n_steps, t0, stream, t, cell)
  rc == 0 || throw(HypError(rc, "hyp_step_noalloc_f64 (cell $(cell[]))"))
  t[]
end
"measure_peaks(; reps=3, bytes=1<<30): (fp64_tflops, fp32_tflops, fp32x2_tflops, h2d_gbs, d2h_gbs, bidir_gbs)"
function measure_peaks(; reps::Integer=3, bytes::Integer=1 << 30)
  out = zeros(6)
  check(ccall((:hyp_measure_peaks, libhyp), Cint, (Cint, Int64, Ptr{Float64}), reps, bytes, out), "hyp_measure_peaks")
  Tuple(out)
end
"measure_layouts(; reps, cells): GB/s of the single-phase mixed step's memory traffic without the physics, (row-major, tile-major)"
function measure_layouts(; reps::Integer=3, cells::Integer=1 << 24)
  out = zeros(2)
  check(ccall((:hyp_measure_layouts, libhyp), Cint, (Cint, Int64, Ptr{Float64}), reps, cells, out), "hyp_measure_layouts")
  Tuple(out)
end
"pinned_matrix(n, k): a Matrix{Float64} in page-locked host memory (hyp_host_alloc) for fast copies"
function pinned_matrix(n::Integer, k::Integer)
  p = Ref{Ptr{Cvoid}}(C_NULL)
  check(ccall((:hyp_host_alloc, libhyp), Cint, (Int64, Ref{Ptr{Cvoid}}), Int64(n) * k * 8, p), "hyp_host_alloc")
  A = unsafe_wrap(Matrix{Float64}, Ptr{Float64}(p[]), (n, k); own=false)
  finalizer(_ -> ccall((:hyp_host_free, libhyp), Cint, (Ptr{Cvoid},), p[]), A)
  A
end

# ---- snapshots and restart (main.jl:62-95, 108, 174-198, 233-237) ----
"save_data(s, fname): the reference's save_data file of the current state (device cons2prim)"
save_data(s::Solver, fname::AbstractString) =
  check(ccall((:hyp_save_snapshot, libhyp), Cint, (Ptr{Cvoid}, Cstring), s.h, fname), "hyp_save_snapshot", s.h)
"read_data!(s, fname, t0): read_data + prim2cons; the file's state becomes current at t0 (main.jl:186-191)"
read_data!(s::Solver, fname::AbstractString, t0::Float64) =
  check(ccall((:hyp_load_snapshot, libhyp), Cint, (Ptr{Cvoid}, Cstring, Float64), s.h, fname, t0),
        "hyp_load_snapshot", s.h)
"run_logged!(s, dir; T, max_steps, log_freq, step_num): main.jl:196-241 with sol_%06i.csv every log_freq steps"
function run_logged!(s::Solver, dir::AbstractString; T::Float64=Inf, max_steps::Integer=0, log_freq::Integer=100,
                     step_num::Integer=0)
  n, t = Ref{Cint}(0), Ref{Float64}(0.0)
  check(ccall((:hyp_run_logged, libhyp), Cint,
              (Ptr{Cvoid}, Float64, Cint, Cint, Cstring, Int64, Ref{Cint}, Ref{Float64}),
              s.h, T, max_steps, log_freq, dir, step_num, n, t), "hyp_run_logged", s.h)
  (n[], t[])
end

# ---- batches of independent single-phase problems ----
"Many independent single-phase problems of uneven size stepped in lockstep (one CUDA graph per call)."
mutable struct Batch
  h::Ptr{Cvoid}
  total::Int64
  np::Int
  function Batch(cfg::ConfigC, offsets::Vector{Int64})
    r = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:hyp_batch_create, libhyp), Cint, (Ref{ConfigC}, Ptr{Int64}, Cint, Ref{Ptr{Cvoid}}),
               Ref(cfg), offsets, length(offsets) - 1, r)
    rc == 0 || throw(HypError(rc, "hyp_batch_create"))
    b = new(r[], offsets[end], length(offsets) - 1)
    finalizer(x -> ccall((:hyp_batch_destroy, libhyp), Cint, (Ptr{Cvoid},), x.h), b)
  end
end
bcheck(rc, b::Batch, what) = rc == 0 ? nothing :
  throw(HypError(rc, what * ": " * unsafe_string(ccall((:hyp_batch_last_error, libhyp), Cstring, (Ptr{Cvoid},), b.h))))
upload!(b::Batch, Q::Matrix{Float64}, t0=0.0) =
  bcheck(ccall((:hyp_batch_upload, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Float64), b.h, Q, t0), b, "hyp_batch_upload")
function download(b::Batch)
  Q = Matrix{Float64}(undef, b.total, 14)
  bcheck(ccall((:hyp_batch_download, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}), b.h, Q), b, "hyp_batch_download")
  Q
end
step!(b::Batch, n_steps::Integer; T::Float64=Inf) =
  bcheck(ccall((:hyp_batch_step, libhyp), Cint, (Ptr{Cvoid}, Cint, Float64), b.h, n_steps, T), b, "hyp_batch_step")
function autotune!(b::Batch; trial_steps::Integer=10)
  chosen, ms = Ref{Cint}(-1), zeros(3)  # HYP_BATCH_NUM_VARIANTS
  bcheck(ccall((:hyp_batch_autotune, libhyp), Cint, (Ptr{Cvoid}, Cint, Ref{Cint}, Ptr{Float64}), b.h, trial_steps,
               chosen, ms), b, "hyp_batch_autotune")
  (chosen[], ms)
end

"status(b) -> (t, steps) per problem"
function status(b::Batch)
  t, steps = zeros(b.np), zeros(Int64, b.np)
  bcheck(ccall((:hyp_batch_status, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Int64}), b.h, t, steps), b,
         "hyp_batch_status")
  t, steps
end
"last_ms(b): device ms of the last step! call"
function last_ms(b::Batch)
  ms = Ref{Float64}(0.0)
  bcheck(ccall((:hyp_batch_last_ms, libhyp), Cint, (Ptr{Cvoid}, Ref{Float64}), b.h, ms), b, "hyp_batch_last_ms")
  ms[]
end
"set_variant!(b, v): the tile kernel variant (0-2, as autotune! numbers them)"
set_variant!(b::Batch, v::Integer) =
  bcheck(ccall((:hyp_batch_set_variant, libhyp), Cint, (Ptr{Cvoid}, Cint), b.h, v), b, "hyp_batch_set_variant")

# ---- the adjoint of a single-phase FP64 Rusanov run ----
"density_misfit(s, rho_target) -> (L, dL/dQ): L = |rho - target|^2 / 2 of the current state"
function density_misfit(s::Solver, target::Vector{Float64})
  L, dQ = Ref{Float64}(0.0), Matrix{Float64}(undef, s.n, s.nvar)
  check(ccall((:hyp_density_misfit, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{Float64}, Ptr{Float64}), s.h,
              target, L, dQ), "hyp_density_misfit", s.h)
  L[], dQ
end
"adjoint_timing(s): device ms of the last record!, and of the recompute and adjoint steps of the last adjoint"
function adjoint_timing(s::Solver)
  r, c, a = Ref{Float64}(0.0), Ref{Float64}(0.0), Ref{Float64}(0.0)
  check(ccall((:hyp_adjoint_timing, libhyp), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Float64}, Ref{Float64}), s.h, r, c,
              a), "hyp_adjoint_timing", s.h)
  (ms_record=r[], ms_recompute=c[], ms_adjoint=a[])
end
"record!(s, n_steps; K): n_steps steps that keep a checkpoint every K steps (the rrule's forward pass)"
function record!(s::Solver, n_steps::Integer; K::Integer=50)
  t = Ref{Float64}(0.0)
  check(ccall((:hyp_adjoint_record, libhyp), Cint, (Ptr{Cvoid}, Cint, Cint, Ref{Float64}), s.h, n_steps, K, t),
        "hyp_adjoint_record", s.h)
  t[]
end
"adjoint(s, dQ): (dL/dQ0, (dL/db0sq, dL/dk0)) of the recorded run from dL/dQ of its final state"
function adjoint(s::Solver, dQ::Matrix{Float64})
  dQ0 = similar(dQ)
  de = zeros(2)
  check(ccall((:hyp_adjoint, libhyp), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), s.h, dQ, dQ0, de),
        "hyp_adjoint", s.h)
  dQ0, (de[1], de[2])
end
"evolve(cfg, Q0, n_steps; K): the final state of n_steps FP64 steps from Q0 (differentiable, see rrule.jl)"
function evolve(cfg::ConfigC, Q0::Matrix{Float64}, n_steps::Integer; K::Integer=50)
  s = Solver(cfg)
  upload!(s, Q0)
  step!(s; max_steps=n_steps)
  download(s)
end

end # module HyperelasticCUDA
