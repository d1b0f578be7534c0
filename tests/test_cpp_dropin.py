"""The header-only C++ drop-in (mesh-deform_gb300/deform/arap.h) used the way
the reference's tests and examples use inc/deform/arap.h: compiled against
include/arap_gpu.h and linked with libarap_gb300.so."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "mesh-deform_gb300"
SRC = ROOT / "tests" / "cpp" / "dropin_main.cpp"
OUT = ROOT / "tests" / "cpp" / "_build"


def build_dropin(reference_tests: Path | None = None) -> Path:
    """Compiles tests/cpp/dropin_main.cpp against the drop-in; with
    reference_tests, the reference's own tests/accessor.h is used unchanged."""
    import build_lib

    lib = build_lib.build()
    OUT.mkdir(exist_ok=True)
    exe = OUT / ("dropin_main_refaccessor" if reference_tests else "dropin_main")
    extra = ["-DDEFORM_REFERENCE_ACCESSOR", f"-I{reference_tests}"] if reference_tests else []
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{PKG}", f"-I{ROOT / 'include'}"] + extra + \
        [str(SRC), f"-L{PKG}", "-larap_gb300", f"-Wl,-rpath,{PKG}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert lib.exists()
    return exe


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def test_dropin_header_compiles_and_links(built):
    exe = build_dropin()
    assert exe.exists()


def test_dropin_with_the_reference_accessor(built):
    """The reference's tests/accessor.h (PrivateAccessor returning
    typename ARAP::SparseMatrix from a._edgeWeights) compiles unchanged
    against the drop-in. Needs a checkout of the reference: ARAP_REFERENCE_DIR,
    else a directory named `reference` beside this repository."""
    import os

    ref = Path(os.environ.get("ARAP_REFERENCE_DIR", str(ROOT.parent / "reference"))) / "tests"
    if not (ref / "accessor.h").exists():
        pytest.skip("no reference checkout")
    exe = build_dropin(ref)
    if not _has_gpu():
        r = subprocess.run([str(exe), "nodevice"], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr


def test_dropin_without_device_does_not_throw(built):
    if _has_gpu():
        pytest.skip("a GPU is present")
    exe = build_dropin()
    r = subprocess.run([str(exe), "nodevice"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "deform=0" in r.stdout and "arap_create" in r.stdout


@pytest.mark.gpu
def test_dropin_cotan_known_answer(built):
    exe = build_dropin()
    r = subprocess.run([str(exe), "kat"], capture_output=True, text=True)
    assert r.returncode == 0 and "kat ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("scalar,tol", [("double", 1e-10), ("float", 1e-6)])
def test_dropin_deform_matches_oracle(built, tmp_path, scalar, tol):
    exe = build_dropin()
    w = W.cfg_twisted_bar(h=0.1, iterations=10)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([w.V, w.F, len(w.cidx), w.iterations], np.int32).tofile(f)
        w.positions.astype(np.float64).tofile(f)
        w.faces.astype(np.int32).tofile(f)
        w.cidx.astype(np.int32).tofile(f)
        w.ctargets.astype(np.float64).tofile(f)
    r = subprocess.run([str(exe), "run", str(fin), str(fout), scalar], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(fout, np.float64).reshape(-1, 3)
    # PrecisionType=float casts the targets to float first (arap.h:83)
    tg = w.ctargets.astype(np.float32).astype(np.float64) if scalar == "float" else w.ctargets
    rest = w.positions.astype(np.float32).astype(np.float64) if scalar == "float" else w.positions
    ok, ref = O.run_deform(rest, w.faces, w.cidx, tg, w.iterations)
    assert ok
    assert W.bbox_rel_error(out, ref, w.positions) <= tol
