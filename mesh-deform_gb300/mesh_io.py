"""Wavefront OBJ reading and writing (numpy), the Python counterpart of
deform/obj_io.h: `v x y z` lines and `f` lines whose corners may be `i`,
`i/t`, `i//n` or `i/t/n` (1-based, negative = relative to the end); polygons
are split into a triangle fan; other lines are ignored. The reference loads
its fixture meshes (etc/*.obj) through OpenMesh's reader."""
from __future__ import annotations

from pathlib import Path

import numpy as np


def read_obj(path) -> tuple[np.ndarray, np.ndarray]:
    v, f = [], []
    for lineno, line in enumerate(Path(path).read_text().splitlines(), 1):
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            if len(t) < 4:
                raise ValueError(f"{path}:{lineno}: bad vertex")
            v.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            nv = len(v)
            idx = []
            for tok in t[1:]:
                i = int(tok.split("/")[0])
                k = i - 1 if i > 0 else nv + i
                if i == 0 or not 0 <= k < nv:
                    raise ValueError(f"{path}:{lineno}: bad face index {tok}")
                idx.append(k)
            if len(idx) < 3:
                raise ValueError(f"{path}:{lineno}: face with <3 corners")
            for k in range(1, len(idx) - 1):
                f.append([idx[0], idx[k], idx[k + 1]])
    return np.array(v, np.float64).reshape(-1, 3), np.array(f, np.int32).reshape(-1, 3)


def write_obj(path, positions, faces) -> None:
    pos = np.asarray(positions, np.float64).reshape(-1, 3)
    fc = np.asarray(faces, np.int64).reshape(-1, 3) + 1
    lines = [f"v {x!r} {y!r} {z!r}" for x, y, z in pos.tolist()]
    lines += [f"f {a} {b} {c}" for a, b, c in fc.tolist()]
    Path(path).write_text("\n".join(lines) + "\n")
