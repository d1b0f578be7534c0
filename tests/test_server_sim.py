"""Scheduler of the deform server (mesh-deform_gb300/csrc/arap_server.h) over
a host model of the device contexts (tests/cpp/server_sim.cpp): ordering,
factor reuse, multi-pose batching, admission by device footprint with LRU
eviction, error delivery, concurrent clients. No GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("callbacks", [0, 1])
def test_scheduler_on_host_model(tmp_path, callbacks):
    """callbacks=1: completions announced by callbacks from another thread, as
    the CUDA runtime does; 0: found by polling."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "server_sim"
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread", f"-DCALLBACKS={callbacks}",
                    f"-I{ROOT / 'mesh-deform_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "cpp" / "server_sim.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
