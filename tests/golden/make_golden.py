"""Regenerates the golden fixtures in tests/golden/ from the reference tree.

Run with the path of a checkout of the reference (a required argument):

    python tests/golden/make_golden.py /path/to/mesh-deform

It reads, as text, without compiling or running anything of the reference:
  * tests/test_cotan.cpp:26-51   the cotan known-answer test (unit square in
                                  z=0, faces (0,1,2),(0,2,3), expected weights)
  * etc/sphere.obj, etc/bar.obj, etc/plane.obj   fixture meshes
  * etc/anchors.txt, etc/handles.txt              index lists of plane.obj
  * examples/deform_bar.cpp:30,33                 anchor/handle lists of bar.obj
  * examples/deform_sphere.cpp:60,65              anchor 37 / handle 32 of sphere.obj
and writes cotan_kat.json and meshes.npz. The GPU machine has no reference tree;
the tests read only these committed files.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def read_obj(path: Path):
    v, f = [], []
    for line in path.read_text().splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            v.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            idx = [int(x.split("/")[0]) - 1 for x in t[1:]]
            for k in range(1, len(idx) - 1):  # fan-triangulate polygons (all inputs are triangles)
                f.append([idx[0], idx[k], idx[k + 1]])
    return np.array(v, np.float64), np.array(f, np.int32)


def int_list(text: str, name: str):
    m = re.search(name + r"\s*=\s*\{([^}]*)\}", text)
    return [int(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]


def main(ref: Path):
    src = (ref / "tests" / "test_cotan.cpp").read_text()
    pts = [[float(a.rstrip("f")), float(b.rstrip("f")), float(c.rstrip("f"))]
           for a, b, c in re.findall(r"Mesh::Point\(([-\d.f]+),\s*([-\d.f]+),\s*([-\d.f]+)\)", src)]
    faces = [[int(a), int(b), int(c)] for a, b, c in
             re.findall(r"add_face\(Mesh::VertexHandle\((\d+)\),\s*Mesh::VertexHandle\((\d+)\),\s*"
                        r"Mesh::VertexHandle\((\d+)\)\)", src)]
    block = src[src.index("expected <<") + len("expected <<"): src.index(";", src.index("expected <<"))]
    expected = [float(x.strip().rstrip("f")) for x in block.replace("\n", " ").split(",")]
    tol = float(re.search(r"isApprox\(expected,\s*([\d.e-]+)f?\)", src).group(1))
    kat = {"source": "tests/test_cotan.cpp:26-53", "positions": pts, "faces": faces,
           "expected_weights": np.array(expected).reshape(4, 4).tolist(), "isApprox_tol": tol}
    (HERE / "cotan_kat.json").write_text(json.dumps(kat, indent=1) + "\n")

    etc = ref / "etc"
    sv, sf = read_obj(etc / "sphere.obj")
    bv, bf = read_obj(etc / "bar.obj")
    pv, pf = read_obj(etc / "plane.obj")
    bar_src = (ref / "examples" / "deform_bar.cpp").read_text()
    sph_src = (ref / "examples" / "deform_sphere.cpp").read_text()
    sph_idx = [int(x) for x in re.findall(r"mesh\.vertex_handle\((\d+)\)", sph_src)]
    np.savez_compressed(
        HERE / "meshes.npz",
        sphere_v=sv, sphere_f=sf,
        sphere_anchor=np.array(sph_idx[:1], np.int32), sphere_handle=np.array(sph_idx[1:2], np.int32),
        bar_v=bv, bar_f=bf,
        bar_anchors=np.array(int_list(bar_src, "anchors"), np.int32),
        bar_handles=np.array(int_list(bar_src, "handles"), np.int32),
        plane_v=pv, plane_f=pf,
        plane_anchors=np.array((etc / "anchors.txt").read_text().split(), np.int32),
        plane_handles=np.array((etc / "handles.txt").read_text().split(), np.int32),
    )
    write_oracle_deforms()
    print("wrote", HERE / "cotan_kat.json", HERE / "meshes.npz", HERE / "oracle_deforms.npz")


def example_cases(d):
    """Constraint sets in the style of the reference's examples."""
    out = {}
    v = d["sphere_v"]
    ph = -np.pi / 2 + 0.01  # first frame of examples/deform_sphere.cpp:75-86
    cidx = np.array([d["sphere_anchor"][0], d["sphere_handle"][0]], np.int32)
    tgt = np.stack([v[cidx[0]], v[cidx[1]] + np.array([0.0, 0.0, np.sin(ph)])])
    o = np.argsort(cidx)
    out["sphere"] = (v, d["sphere_f"], cidx[o], tgt[o], 5)
    v = d["bar_v"]  # examples/deform_bar.cpp:146-151,169-172,189-193: handles turned about x
    t = 0.05
    c, s = np.cos(np.pi * t), np.sin(np.pi * t)
    R = np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    a, h = d["bar_anchors"], d["bar_handles"]
    cidx = np.concatenate([a, h]).astype(np.int32)
    tgt = np.concatenate([v[a], v[h] @ R.T])
    o = np.argsort(cidx)
    out["bar"] = (v, d["bar_f"], cidx[o], tgt[o], 20)
    v = d["plane_v"]
    a, h = d["plane_anchors"], d["plane_handles"]
    cidx = np.concatenate([a, h]).astype(np.int32)
    tgt = np.concatenate([v[a], v[h] + np.array([0.0, 0.3, 0.1])])
    o = np.argsort(cidx)
    out["plane"] = (v, d["plane_f"], cidx[o], tgt[o], 10)
    return out


def write_oracle_deforms():
    """Oracle (FP64 C restatement) outputs for the example-style cases."""
    sys.path.insert(0, str(HERE.parent.parent))
    from oracle import oracle as O

    d = np.load(HERE / "meshes.npz")
    res = {}
    for name, (v, f, cidx, tgt, iters) in example_cases(d).items():
        ok, outp = O.run_deform(v, f, cidx, tgt, iters)
        assert ok
        res[f"{name}_cidx"] = cidx
        res[f"{name}_targets"] = tgt
        res[f"{name}_iterations"] = np.array(iters)
        res[f"{name}_out"] = outp
    np.savez_compressed(HERE / "oracle_deforms.npz", **res)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py /path/to/mesh-deform")
    main(Path(sys.argv[1]))
