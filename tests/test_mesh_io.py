"""OBJ reading/writing (mesh_io.py, deform/obj_io.h) on the reference's
fixture meshes (tests/golden/meshes.npz holds them, read from etc/*.obj), in
every corner syntax the format allows."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import mesh_io

ROOT = Path(__file__).resolve().parent.parent
GOLD = np.load(ROOT / "tests" / "golden" / "meshes.npz")


def _write_styled(path, v, f, style):
    lines = ["# written by the test", "o mesh"] + [f"v {x!r} {y!r} {z!r}" for x, y, z in v.tolist()]
    lines += ["vn 0 0 1", "vt 0 0"]
    n = len(v)
    for a, b, c in (f + 1).tolist():
        if style == "plain":
            lines.append(f"f {a} {b} {c}")
        elif style == "normals":
            lines.append(f"f {a}//1 {b}//1 {c}//1")
        elif style == "full":
            lines.append(f"f {a}/1/1 {b}/1/1 {c}/1/1")
        elif style == "negative":
            lines.append(f"f {a - n - 1} {b - n - 1} {c - n - 1}")
    path.write_text("\n".join(lines) + "\n")


@pytest.mark.parametrize("name", ["sphere", "bar", "plane"])
@pytest.mark.parametrize("style", ["plain", "normals", "full", "negative"])
def test_read_write_round_trip(tmp_path, name, style):
    v, f = GOLD[f"{name}_v"], GOLD[f"{name}_f"]
    p = tmp_path / "m.obj"
    _write_styled(p, v, f, style)
    rv, rf = mesh_io.read_obj(p)
    np.testing.assert_array_equal(rv, v)
    np.testing.assert_array_equal(rf, f)
    q = tmp_path / "w.obj"
    mesh_io.write_obj(q, rv, rf)
    wv, wf = mesh_io.read_obj(q)
    np.testing.assert_array_equal(wv, v)
    np.testing.assert_array_equal(wf, f)


def test_polygons_are_fanned_and_errors_raised(tmp_path):
    p = tmp_path / "q.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n")
    v, f = mesh_io.read_obj(p)
    np.testing.assert_array_equal(f, [[0, 1, 2], [0, 2, 3]])
    p.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError):
        mesh_io.read_obj(p)


def test_cpp_reader_matches_python(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "obj_main"
    subprocess.run([gxx, "-O1", "-std=c++17", f"-I{ROOT / 'mesh-deform_gb300'}",
                    str(ROOT / "tests" / "cpp" / "obj_main.cpp"), "-o", str(exe)], check=True)
    for name in ("sphere", "bar", "plane"):
        v, f = GOLD[f"{name}_v"], GOLD[f"{name}_f"]
        src = tmp_path / f"{name}.obj"
        _write_styled(src, v, f, "full")
        dst = tmp_path / f"{name}_out.obj"
        r = subprocess.run([str(exe), str(src), str(dst)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
        assert r.stdout.split() == [str(len(v)), str(len(f))]
        cv, cf = mesh_io.read_obj(dst)
        np.testing.assert_array_equal(cv, v)
        np.testing.assert_array_equal(cf, f)
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    r = subprocess.run([str(exe), str(bad), str(tmp_path / "x.obj")], capture_output=True, text=True)
    assert r.returncode == 1 and "bad face index" in r.stdout
