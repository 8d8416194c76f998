"""The C ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares. No compute calls (CPU only)."""
import glob
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s+\*?(hyp_[A-Za-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    assert {"hyp_create", "hyp_step", "hyp_upload", "hyp_download", "hyp_eval_stress"} <= names


def test_library_exports_every_declared_symbol(hyp):
    lib = hyp._lib.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = declared_functions() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_python_binding_covers_header(hyp):
    assert declared_functions() <= set(hyp._lib.exported_symbols())


def test_julia_binding_covers_header():
    """Every entry point has a ccall in the Julia binding (which cannot run here)."""
    src = "".join(open(f).read() for f in glob.glob(os.path.join(ROOT, "hyperelasticsolver_gb300", "julia", "*.jl")))
    called = set(re.findall(r"ccall\(\(\$?\(?QuoteNode\(c\)\)?|ccall\(\(:(hyp_[A-Za-z0-9_]+)", src)) - {""}
    looped = set(re.findall(r"\(:[a-z_0-9]+, :(hyp_[A-Za-z0-9_]+)", src))  # symbols bound in @eval loops
    missing = declared_functions() - called - looped
    assert not missing, f"declared but not bound in Julia: {sorted(missing)}"


def test_library_loads_without_gpu(hyp):
    L = hyp._lib.load()
    assert L.hyp_last_error(None) == b"no context"


def test_invalid_arguments_rejected_before_any_device_work(hyp):
    import ctypes
    L = hyp._lib.load()
    h = ctypes.c_void_p()
    for model, eos in ((hyp._lib.HYP_MODEL_SINGLE, hyp.Barton2009()),
                       (hyp._lib.HYP_MODEL_MULTI, (hyp.Barton2009(), hyp.Barton2009()))):
        for n in (0, 1, 2):  # fewer than the reference's two frozen ends and one interior cell
            cfg = hyp._model.config(eos, model, n_cells=n)
            assert L.hyp_create(cfg, ctypes.byref(h)) == hyp._lib.HYP_ERR_INVALID
    cfg = hyp._model.config(hyp.Barton2009(), 5, n_cells=100)  # bad model
    assert L.hyp_create(cfg, ctypes.byref(h)) == hyp._lib.HYP_ERR_INVALID
    assert L.hyp_create(None, ctypes.byref(h)) == hyp._lib.HYP_ERR_INVALID
    # calls on a missing context are refused before any device work
    n, t = ctypes.c_int(0), ctypes.c_double(0.0)
    hist = (ctypes.c_double * 4)()
    b = hyp.Barton2009().c()
    assert L.hyp_set_eos(None, 0, ctypes.byref(b)) == hyp._lib.HYP_ERR_INVALID
    assert L.hyp_step_times(None, 4, float("inf"), ctypes.byref(n), ctypes.byref(t), hist) == hyp._lib.HYP_ERR_INVALID
    assert L.hyp_step(None, 4, float("inf"), ctypes.byref(n), ctypes.byref(t)) == hyp._lib.HYP_ERR_INVALID
