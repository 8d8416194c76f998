"""tests/c_abi_example.c: the library used from plain C through include/hyperelastic.h
(compiled and linked on CPU; run on the GPU against the same run through Python)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def example(hyp):
    from hyperelasticsolver_gb300.build import LIB
    d = tempfile.mkdtemp(prefix="hyp_c_")
    exe = os.path.join(d, "c_abi_example")
    r = subprocess.run(["gcc", "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "c_abi_example.c"), LIB, "-Wl,-rpath," + os.path.dirname(LIB), "-lm",
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_example_compiles_and_links(example):
    assert os.access(example, os.X_OK)


@pytest.mark.gpu
def test_c_example_matches_the_python_binding(hyp, example):
    r = subprocess.run([example, "1000", "60"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    _, steps, _, t, _, checksum = r.stdout.split()
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    Ql, Qr = HM.initial_states(eos, 6)
    with hyp.Solver(eos, 1000, model="multi", flux="hll", cfl=0.6) as s:
        s.init_riemann(Ql, Qr)
        n, tp = s.step(max_steps=60)
        Q = s.download()
    assert int(steps) == n == 60 and float(t) == tp
    assert float(checksum) == np.cumsum(np.abs(Q.reshape(-1)))[-1]  # the C loop's sequential sum
