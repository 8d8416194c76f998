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


def ulp_sensitivity(f, args, seed=0, trials=3):
    """Element-wise spread of f under a one-ulp perturbation of its array inputs.

    Each trial multiplies every float64 input element by (1 +- 2^-52) with random
    signs and records max |f(perturbed) - f(args)|. The result bounds how far two
    correct FP64 evaluations of f may differ when they round differently (FMA
    contraction, closed forms against dual numbers): the oracle's own conditioning,
    measured rather than assumed."""
    rng = np.random.default_rng(seed)
    base = np.asarray(f(*args), dtype=np.float64)
    spread = np.zeros_like(base)
    for _ in range(trials):
        pert = []
        for a in args:
            if isinstance(a, np.ndarray) and a.dtype == np.float64:
                s = rng.choice([-1.0, 1.0], size=a.shape)
                pert.append(a * (1.0 + s * 2.0 ** -52))
            else:
                pert.append(a)
        spread = np.maximum(spread, np.abs(np.asarray(f(*pert), dtype=np.float64) - base))
    return spread


def assert_within_sensitivity(got, ref, sens, rtol, what="", factor=4.0, axis=None):
    """|got - ref| <= max(rtol * scale, factor * sens) element-wise; scale = max |ref| over
    `axis` (None: the whole array). Returns the worst ratio of error to allowance."""
    got, ref, sens = (np.asarray(x, dtype=np.float64) for x in (got, ref, sens))
    assert np.all(np.isfinite(got)), f"{what}: non-finite values"
    scale = np.max(np.abs(ref), axis=axis, keepdims=axis is not None)
    allow = np.maximum(rtol * scale, factor * sens)
    err = np.abs(got - ref)
    ratio = err / np.where(allow > 0, allow, 1.0)
    worst = float(np.max(ratio))
    assert np.all(err <= allow), (f"{what}: error {float(np.max(err)):.3e} exceeds its allowance "
                                  f"(worst ratio {worst:.2f}; rtol {rtol:.1e}, {factor} x the 1-ulp sensitivity)")
    return worst
