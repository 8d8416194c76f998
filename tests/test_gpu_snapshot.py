"""Snapshots and restart in the reference's file format (main.jl:62-95 save_data /
read_data, :108 sol_%06i.csv, :174-198 restart, :233-237 logging)."""
import os

import numpy as np
import pytest

from helpers import RTOL_FP64

pytestmark = pytest.mark.gpu

HEADER1 = ("a1\tr1\tu11\tu21\tu31\tS1\tF111\tF211\tF311\tF121\tF221\tF321\tF131\tF231\tF331")


def riemann_Q0(hyp, nx):
    from hyperelasticsolver_gb300._cases import riemann_1ph, initial_condition
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    eos = hyp.Barton2009()
    Pl, Pr = riemann_1ph(eos)
    return eos, initial_condition(H.prim2cons(eos, Pl), H.prim2cons(eos, Pr), nx)


def read_tsv(path):
    with open(path) as fh:
        head = fh.readline().rstrip("\n")
        rows = [list(map(float, l.split())) for l in fh if l.strip()]
    return head, np.array(rows).T


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_snapshot_file_matches_cons2prim(hyp, tmp_path, precision):
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    eos, Q0 = riemann_Q0(hyp, 300)
    with hyp.Solver(eos, 300, precision=precision) as s:
        s.upload(Q0)
        s.step(max_steps=40)
        Q = s.download()
        P = s.snapshot()
        path = str(tmp_path / "snap.csv")
        s.save_snapshot(path)
    head, Pf = read_tsv(path)
    assert head == HEADER1
    assert np.array_equal(Pf, P)  # shortest round-trip text reads back bitwise
    assert np.all(P[0] == 1.0)
    ref = H.cons2prim(eos, Q.T).T  # (rho, u, S, A)
    np.testing.assert_allclose(P[1:], ref, rtol=1e-12, atol=1e-14)
    with open(path) as fh:
        fh.readline()
        first = fh.readline().split("\t")
    assert first[0] == "1.0"  # Julia's layout of a Float64


def test_load_snapshot_round_trip(hyp, tmp_path):
    eos, Q0 = riemann_Q0(hyp, 257)
    path = str(tmp_path / "sol_000000.csv")
    with hyp.Solver(eos, 257) as s:
        s.upload(Q0)
        s.step(max_steps=25)
        Q = s.download()
        s.save_snapshot(path)
    with hyp.Solver(eos, 257) as s:
        s.load_snapshot(path, t0=1.5)
        Q1 = s.download()
        assert s.time()[0] == 1.5
    scale = np.maximum(np.max(np.abs(Q), axis=1, keepdims=True), 1e-30)
    assert np.max(np.abs(Q1 - Q) / scale) < 1e-13  # prim2cons(cons2prim(Q))


def test_run_logged_files_and_restart(hyp, tmp_path):
    from hyperelasticsolver_gb300.solver import last_snapshot
    eos, Q0 = riemann_Q0(hyp, 400)
    d = str(tmp_path / "run")
    os.makedirs(d)
    with hyp.Solver(eos, 400) as s:
        s.upload(Q0)
        n, t = s.run_logged(d, max_steps=250, log_freq=100)
        assert n == 250
        Qlog = s.download()
    assert sorted(os.listdir(d)) == ["sol_000000.csv", "sol_000100.csv", "sol_000200.csv"]  # T not reached
    with hyp.Solver(eos, 400) as s:
        s.upload(Q0)
        s.step(max_steps=250)
        assert np.array_equal(s.download(), Qlog)  # logging does not change the steps
        s.upload(Q0)
        s.step(max_steps=200)
        P200 = s.snapshot()
    _, Pf = read_tsv(os.path.join(d, "sol_000200.csv"))
    assert np.array_equal(Pf, P200)
    path, step, t0 = last_snapshot(d, dt=5e-6)
    assert step == 200 and path.endswith("sol_000200.csv") and t0 == 200 * 5e-6
    with hyp.Solver(eos, 400) as s:  # restart (main.jl:181-191) and continue the log numbering
        s.load_snapshot(path, t0)
        n, _ = s.run_logged(d, max_steps=100, log_freq=100, first_step=step)
        assert n == 100
    assert "sol_000300.csv" in os.listdir(d)


def test_twophase_snapshot_and_logged_t_end(hyp, orc, tmp_path):
    from hyperelasticsolver_gb300._cases import mph_case, initial_condition
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, nx=3, cfl=0.6,
                     eos=(orc.barton2009(), orc.barton2009(b0=2.1 * np.sqrt(0.1))))
    Pl, Pr = mph_case(6)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), 200)
    d = str(tmp_path)
    with hyp.Solver(eos, 200, model="multi", flux="hll", cfl=0.6) as s:
        s.upload(Q0)
        lam = s.max_wavespeed()
        t_end = 35.5 * 0.6 * (1.0 / 200) / lam  # stops between two logged steps
        n, t = s.run_logged(d, t_end=t_end, log_freq=10)
        assert t >= t_end
        P = s.snapshot()
    files = sorted(f for f in os.listdir(d) if f.startswith("sol_"))
    assert files[0] == "sol_000000.csv" and all(int(f[4:10]) % 10 == 0 for f in files)
    head, P0 = read_tsv(os.path.join(d, "sol_000000.csv"))
    assert head.split("\t")[15] == "a2" and P0.shape == (30, 200)
    np.testing.assert_allclose(P0, orc.cons2prim(pb, Q0.T).T, rtol=RTOL_FP64, atol=1e-15)
    assert P.shape == (30, 200) and np.all(np.isfinite(P))
    # the run reached T: result.csv holds the final state (main.jl:242-244), and the
    # reference's restart rule then starts afresh (main.jl:173-176)
    _, Pr = read_tsv(os.path.join(d, "result.csv"))
    assert np.array_equal(Pr, P)
    from hyperelasticsolver_gb300.solver import last_snapshot
    assert last_snapshot(d, dt=1e-6) is None and os.path.exists(os.path.join(d, "result.csv"))
    assert last_snapshot(d, dt=1e-6, clean=True) is None
    assert not any(f.startswith("sol_") or f == "result.csv" for f in os.listdir(d))


def test_load_snapshot_rejects_malformed_files(hyp, tmp_path):
    """A missing file, a short or long file, and rows with too few or too many
    columns are refused (HYP_ERR_INVALID) and leave the context usable."""
    eos, Q0 = riemann_Q0(hyp, 64)
    good = str(tmp_path / "good.csv")
    with hyp.Solver(eos, 64) as s:
        s.upload(Q0)
        s.save_snapshot(good)
        head, P = read_tsv(good)
        lines = open(good).read().splitlines()
        bad = {
            "missing": None,
            "short": lines[:-1],
            "long": lines + [lines[-1]],
            "few columns": lines[:5] + ["\t".join(lines[5].split("\t")[:-1])] + lines[6:],
            "many columns": lines[:5] + [lines[5] + "\t1.0"] + lines[6:],
        }
        for name, content in bad.items():
            path = str(tmp_path / f"bad_{name.replace(' ', '_')}.csv")
            if content is not None:
                with open(path, "w") as fh:
                    fh.write("\n".join(content) + "\n")
            with pytest.raises(hyp._lib.HypError) as err:
                s.load_snapshot(path)
            assert err.value.code == hyp._lib.HYP_ERR_INVALID, name
        s.load_snapshot(good)
        n, _ = s.step(max_steps=3)
        assert n == 3
