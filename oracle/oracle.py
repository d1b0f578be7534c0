"""ctypes binding of the FP64 CPU oracle (arap_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by ``bench.py``'s CPU-baseline and reference legs, as the checker and the
timed CPU restatement of cheind/mesh-deform's ``inc/deform/arap.h``. The
product path never imports it.

The oracle is built from its single C file into ``oracle/_build/`` by
``build()`` (gcc, ``-ffp-contract=off`` so that x86-64 and aarch64 round the
same way). Parity status: cotan weights pinned by the reference's known-answer
test; end-to-end positions "parity unpinned" against the reference binary,
which needs Eigen and cannot be compiled here.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "arap_oracle.c"
BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "liboracle_arap.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile arap_oracle.c into oracle/_build/liboracle_arap.so."""
    BUILD_DIR.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, (HERE / "arap_oracle.h").stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           str(SRC), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    lib = C.CDLL(str(LIB))
    P = C.c_void_p
    ip = C.POINTER(C.c_int)
    dp = C.POINTER(C.c_double)
    sig = {
        "oa_create": (P, [C.c_int, C.c_int, ip, dp]),
        "oa_destroy": (None, [P]),
        "oa_set_mesh_positions": (None, [P, dp]),
        "oa_get_mesh_positions": (None, [P, dp]),
        "oa_set_constraint": (C.c_int, [P, C.c_int, C.c_double, C.c_double, C.c_double]),
        "oa_deform": (C.c_int, [P, C.c_int]),
        "oa_num_free": (C.c_int, [P]),
        "oa_weights_nnz": (C.c_int, [P]),
        "oa_get_weights": (None, [P, ip, ip, dp]),
        "oa_get_rotations": (None, [P, dp]),
        "oa_get_free_map": (None, [P, ip]),
        "oa_get_bfixed": (None, [P, dp]),
        "oa_get_ordering": (None, [P, ip]),
        "oa_get_etree": (None, [P, ip]),
        "oa_energy": (C.c_double, [P]),
        "oa_num_blocks": (C.c_int, [P]),
        "oa_get_blocks": (None, [P, ip]),
        "oa_factor_nnz": (C.c_longlong, [P]),
        "oa_rotation_from_covariance": (None, [dp, dp]),
        "oa_nd_order": (C.c_int, [C.c_int, ip, ip, ip, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleARAP:
    """AsRigidAsPossibleDeformation<Mesh, double> restated in C (arap.h:49-466).

    ``positions`` plays the mesh adapter: ``deform`` reads it when dirty and
    writes the result back into it (arap.h:133-135)."""

    def __init__(self, positions: np.ndarray, faces: np.ndarray):
        self.lib = load()
        self.V = int(positions.shape[0])
        self.F = int(faces.shape[0])
        self._faces = np.ascontiguousarray(faces, dtype=np.int32)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        self.h = self.lib.oa_create(self.V, self.F, _ip(self._faces), _dp(pos))

    def close(self):
        if self.h:
            self.lib.oa_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_mesh_positions(self, xyz):
        a = np.ascontiguousarray(xyz, dtype=np.float64)
        self.lib.oa_set_mesh_positions(self.h, _dp(a))

    def mesh_positions(self) -> np.ndarray:
        out = np.empty((self.V, 3), np.float64)
        self.lib.oa_get_mesh_positions(self.h, _dp(out))
        return out

    def set_constraint(self, vidx: int, xyz) -> None:
        if self.lib.oa_set_constraint(self.h, int(vidx), float(xyz[0]), float(xyz[1]), float(xyz[2])) != 0:
            raise IndexError(vidx)

    def set_constraints(self, idx, xyz) -> None:
        xyz = np.asarray(xyz, np.float64)
        for i, v in enumerate(np.asarray(idx)):
            self.set_constraint(int(v), xyz[i])

    def deform(self, iterations: int) -> bool:
        return bool(self.lib.oa_deform(self.h, int(iterations)))

    def num_free(self) -> int:
        return int(self.lib.oa_num_free(self.h))

    def weights_csr(self):
        nnz = self.lib.oa_weights_nnz(self.h)
        rp = np.zeros(self.V + 1, np.int32)
        col = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1), np.float64)
        self.lib.oa_get_weights(self.h, _ip(rp), _ip(col), _dp(val))
        return rp, col[:nnz], val[:nnz]

    def rotations(self) -> np.ndarray:
        out = np.empty((self.V, 3, 3), np.float64)
        self.lib.oa_get_rotations(self.h, _dp(out))
        return out

    def free_map(self) -> np.ndarray:
        out = np.empty(self.V, np.int32)
        self.lib.oa_get_free_map(self.h, _ip(out))
        return out

    def bfixed(self) -> np.ndarray:
        m = self.num_free()
        out = np.zeros((max(m, 1), 3), np.float64)
        self.lib.oa_get_bfixed(self.h, _dp(out))
        return out[:m]

    def ordering(self) -> np.ndarray:
        m = self.num_free()
        out = np.zeros(max(m, 1), np.int32)
        self.lib.oa_get_ordering(self.h, _ip(out))
        return out[:m]

    def energy(self) -> float:
        return float(self.lib.oa_energy(self.h))

    def etree(self) -> np.ndarray:
        m = self.num_free()
        out = np.zeros(max(m, 1), np.int32)
        self.lib.oa_get_etree(self.h, _ip(out))
        return out[:m]

    def blocks(self) -> np.ndarray:
        nb = self.lib.oa_num_blocks(self.h)
        out = np.zeros(nb + 1, np.int32)
        self.lib.oa_get_blocks(self.h, _ip(out))
        return out

    def factor_nnz(self) -> int:
        return int(self.lib.oa_factor_nnz(self.h))


def rotation_from_covariance(cov: np.ndarray) -> np.ndarray:
    """arap.h:376-382 for one 3x3 covariance."""
    lib = load()
    c = np.ascontiguousarray(cov, np.float64).reshape(9)
    r = np.empty(9, np.float64)
    lib.oa_rotation_from_covariance(_dp(c), _dp(r))
    return r.reshape(3, 3)


def nd_order(rowptr: np.ndarray, col: np.ndarray):
    """Nested-dissection ordering of a symmetric graph (the oracle's copy)."""
    lib = load()
    n = len(rowptr) - 1
    rp = np.ascontiguousarray(rowptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32) if len(col) else np.zeros(1, np.int32)
    perm = np.zeros(max(n, 1), np.int32)
    bp = np.zeros(n + 2, np.int32)
    nb = lib.oa_nd_order(n, _ip(rp), _ip(cl), _ip(perm), _ip(bp))
    return perm[:n], bp[: nb + 1]


def run_deform(positions, faces, cidx, ctargets, iterations: int):
    """One dirty deform on a fresh object: rest = positions, constraints set,
    ``deform(iterations)``. Returns (ok, positions after write-back)."""
    o = OracleARAP(positions, faces)
    o.set_constraints(cidx, ctargets)
    ok = o.deform(iterations)
    out = o.mesh_positions()
    o.close()
    return ok, out
