"""Floating-point operations per cell-update of the step's formulation (the roofline's
compute side): tests/flop_count.cpp runs the product's FP64 physics on the host with
a scalar type that counts its operations. CPU only. The counts are the figures the
design documents; they move only when the formulation changes."""
import json
import os
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def counts():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "flop_count")
        r = subprocess.run(["g++", "-O1", "-std=c++17", "-o", exe, os.path.join(HERE, "flop_count.cpp")],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return json.loads(out)


def test_single_phase_rusanov(counts):
    c = counts["single_cell_update"]
    print("single-phase Rusanov per cell-update:", c)
    parts = sum(counts[k]["flops"] for k in ("single_cell_pass", "single_face", "single_update"))
    assert c["flops"] == parts
    assert 500 <= c["flops"] <= 900  # ~3 flops per algorithmic byte (224 B per cell-update)
    assert c["transcendental"] == 0  # default exponents: powers are products


def test_twophase_hll(counts):
    c = counts["twophase_cell_update"]
    print("two-phase HLL per cell-update:", c)
    assert 10_000 <= c["flops"] <= 20_000
    assert counts["twophase_hll_face"]["flops"] > 0.85 * c["flops"]  # the face's 18 evaluations of B dominate
