"""Task plan of the dense top's tensor-core products for many poses
(mesh-deform_gb300/csrc/arap_btop_plan.h, shared by the kernels and the host):
splits cover each row tile's part of the triangle exactly once and in order,
the kernel's task decoding agrees with the reduction's numbering, and the
partial products' layout is a bijection with aligned quads. No GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_btop_task_plan(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "btop_plan"
    subprocess.run([gxx, "-O2", "-std=c++17", "-Wall", "-Wextra", f"-I{ROOT / 'mesh-deform_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "cpp" / "btop_plan.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
