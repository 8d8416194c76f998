"""Shared tolerances and comparisons for the parity tests."""
import numpy as np

# FP64 GPU vs FP64 CPU oracle: the required parity tolerance. Bit equality is not
# expected (FMA contraction, closed-form derivatives vs dual numbers, cofactor
# vs LU determinant), 1e-12 relative is.
RTOL_FP64 = 1e-12


def rel_err(a, b, axis=None):
    """max |a - b| / max |b| along `axis` (per variable when axis=1 on SoA arrays)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    num = np.max(np.abs(a - b), axis=axis)
    den = np.max(np.abs(b), axis=axis)
    return num / np.where(den > 0, den, 1.0)


def assert_close(a, b, rtol, what=""):
    e = rel_err(a, b)
    assert np.all(np.isfinite(a)), f"{what}: non-finite values"
    assert e <= rtol, f"{what}: relative error {e:.3e} > {rtol:.1e}"


def assert_close_soa(a, b, rtol, what=""):
    """Per-variable check on SoA (nvar, n) arrays: max_i |a - b| <= rtol * max_i |b| for each variable,
    with variables that are identically zero in b compared against the state's overall scale."""
    a, b = np.asarray(a), np.asarray(b)
    scale = np.max(np.abs(b), axis=1)
    scale = np.where(scale > 0, scale, np.max(np.abs(b)))
    err = np.max(np.abs(a - b), axis=1) / scale
    assert np.all(np.isfinite(a)), f"{what}: non-finite values"
    worst = int(np.argmax(err))
    assert np.all(err <= rtol), f"{what}: variable {worst} relative error {err[worst]:.3e} > {rtol:.1e}"
    return float(np.max(err))
