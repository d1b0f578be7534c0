"""Python binding of libarap_gb300.so (the C ABI in include/arap_gpu.h).

Two layers:

* ``ArapContext`` -- one-to-one wrapper of the C entry points (what a cgo/JNI
  binding would look like), numpy arrays in and out.
* ``AsRigidAsPossibleDeformation`` -- mirrors the reference's class template
  ``deform::AsRigidAsPossibleDeformation`` (inc/deform/arap.h:49-466) over a
  mesh adapter: ``set_constraint`` fills a map and marks the object dirty
  (arap.h:81-85); ``deform(n)`` re-captures the rest pose from the mesh when
  dirty (arap.h:102-120), iterates, and writes the positions back through the
  adapter (arap.h:133-135). Returns False where the reference returns false.

There is no CPU fallback: a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libarap_gb300.so"

ARAP_OK = 0
ARAP_ERR_INVALID_ARGUMENT = 1
ARAP_ERR_BAD_INDEX = 2
ARAP_ERR_NOT_SPD = 3
ARAP_ERR_OUT_OF_MEMORY = 4
ARAP_ERR_CUDA = 5
ARAP_ERR_TIMEOUT = 6
ARAP_ERR_ADMISSION_REFUSED = 7
ARAP_ERR_NO_DEVICE = 8
ARAP_ERR_UNSUPPORTED = 9
ARAP_PENDING = 10
ARAP_SOLVE_PERSISTENT = 0
ARAP_SOLVE_LEVELS = 1

PRECISION = {"fp64": 0, "mixed": 1}

# Every symbol include/arap_gpu.h declares: (restype, argtypes).
_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("refine_steps", C.c_int32),
                ("max_in_flight", C.c_int32), ("device_budget_bytes", C.c_int64), ("prep_threads", C.c_int32),
                ("max_batch", C.c_int32), ("max_queue", C.c_int32), ("poll_us", C.c_int32),
                ("solve_ctas", C.c_int32), ("per_set_ordering", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("n_constraints", C.c_int32), ("indices", _ip), ("targets", _dp),
                ("iterations", C.c_int32), ("pad", C.c_int32), ("out_xyz", _dp)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("factor_reused", C.c_int32), ("batch_size", C.c_int32),
                ("pad", C.c_int32), ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "refused", "factor_hits",
                                         "factor_misses", "evictions", "launches", "batched_launches",
                                         "batched_requests", "iterations_done", "resident_bytes",
                                         "peak_resident_bytes", "budget_bytes")] + \
        [(n, C.c_int32) for n in ("resident_factors", "queue_depth", "in_flight", "pad")] + \
        [(n, C.c_double) for n in ("scheduler_busy_ms", "worker_busy_ms", "analyze_ms", "staging_ms",
                                             "device_ms", "launch_ms")] + \
        [("launch_host_ms", C.c_double * 5)]


SIGNATURES = {
    "arap_status_string": (C.c_char_p, [C.c_int]),
    "arap_last_error": (C.c_char_p, [_P]),
    "arap_create": (C.c_int, [_I32, _I32, _ip, _I32, C.POINTER(_P)]),
    "arap_destroy": (None, [_P]),
    "arap_set_precision": (C.c_int, [_P, _I32, _I32]),
    "arap_set_factor_precision": (C.c_int, [_P, _I32]),
    "arap_set_rest_positions": (C.c_int, [_P, _dp]),
    "arap_set_constraints": (C.c_int, [_P, _I32, _ip, _dp]),
    "arap_deform": (C.c_int, [_P, _I32, _dp]),
    "arap_invalidate": (C.c_int, [_P]),
    "arap_get_positions": (C.c_int, [_P, _dp]),
    "arap_edge_weights_nnz": (C.c_int, [_P, _ip]),
    "arap_get_edge_weights": (C.c_int, [_P, _ip, _ip, _dp]),
    "arap_get_rotations": (C.c_int, [_P, _dp]),
    "arap_get_symbolic_sizes": (C.c_int, [_P, _ip, _ip, _lp]),
    "arap_get_symbolic": (C.c_int, [_P, _ip, _ip, _ip]),
    "arap_analyze_pattern": (C.c_int, [_I32, _I32, _ip, _I32, _ip, _ip, _ip, _lp, _ip, _ip, _ip]),
    "arap_get_timing": (C.c_int, [_P, _dp, _dp]),
    "arap_get_launch_count": (C.c_int, [_P, _lp]),
    "arap_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "arap_set_profiling": (C.c_int, [_P, _I32]),
    "arap_reset_kernel_stats": (C.c_int, [_P]),
    "arap_get_kernel_stats": (C.c_int, [_P, _I32, _dp, _lp]),
    "arap_get_kernel_model": (C.c_int, [_P, _I32, _dp, _dp]),
    "arap_cotan_weights_static": (C.c_int, [_I32, _I32, _P, _P, _P, _P, _I32, _P, _P]),
    "arap_cotan_weights_static_status": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "arap_deform_poses": (C.c_int, [_P, _I32, _dp, _I32, _dp]),
    "arap_deform_async": (C.c_int, [_P, _I32, _dp]),
    "arap_wait": (C.c_int, [_P]),
    "arap_set_graphs": (C.c_int, [_P, _I32]),
    "arap_set_symbolic_cache": (C.c_int, [_P, _I32]),
    "arap_set_wait_limit": (C.c_int, [_P, _I32]),
    "arap_set_solve_ctas": (C.c_int, [_P, _I32]),
    "arap_set_pose_tile": (C.c_int, [_P, _I32]),
    "arap_energy": (C.c_int, [_P, _dp]),
    "arap_set_cluster_threshold": (C.c_int, [_P, _I32]),
    "arap_set_dense_top": (C.c_int, [_P, _I32]),
    "arap_set_warp_rows": (C.c_int, [_P, _I32]),
    "arap_set_solve_schedule": (C.c_int, [_P, _I32]),
    "arap_set_solve_blocks": (C.c_int, [_P, _I32]),
    "arap_set_vertex_launch": (C.c_int, [_P, _I32, _I32, _I32]),
    "arap_set_ordering": (C.c_int, [_P, _I32]),
    "arap_set_done_callback": (C.c_int, [_P, _P, _P]),
    "arap_get_host_timing": (C.c_int, [_P, _dp]),
    "arap_vertex_normals": (C.c_int, [_P, _dp]),
    "arap_device_positions": (C.c_int, [_P, _I32, C.POINTER(_P), C.POINTER(_P)]),
    "arap_pose_targets": (C.c_int, [_P, _I32, _ip, _dp, _I32, _dp]),
    "arap_set_targets": (C.c_int, [_P, _I32, _dp]),
    "arap_deform_poses_async": (C.c_int, [_P, _I32, _dp, _I32, _dp]),
    "arap_query": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "arap_create_like": (C.c_int, [_P, C.POINTER(_P)]),
    "arap_plan_bytes": (C.c_int, [_P, _I32, C.POINTER(C.c_int64)]),
    "arap_device_bytes": (C.c_int64, [_P]),
    "arap_srv_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "arap_srv_destroy": (None, [_P]),
    "arap_srv_add_mesh": (C.c_int, [_P, _I32, _I32, _ip, _dp, _ip]),
    "arap_srv_submit": (C.c_int, [_P, C.POINTER(Request), _lp]),
    "arap_srv_poll": (C.c_int, [_P, _I64, C.POINTER(RequestInfo)]),
    "arap_srv_wait": (C.c_int, [_P, _I64, _I32, C.POINTER(RequestInfo)]),
    "arap_srv_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "arap_srv_last_error": (C.c_char_p, [_P]),
}

KERNEL_CLASSES = ["weights", "assemble", "factor", "local", "rhs", "residual", "solve_fwd", "solve_bwd", "gather"]
ARAP_K_LOCAL, ARAP_K_RHS, ARAP_K_RESIDUAL = 3, 4, 5

_lib = None


def load(path: Path | str | None = None):
    """Loads the library (and binds every declared symbol); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with build_lib.build() (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class ArapError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_status_name(code)}: {msg}")
        self.code = code


def _status_name(code: int) -> str:
    return load().arap_status_string(code).decode()


def _i32(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return a.ctypes.data_as(_dp)


class DeviceArray:
    """A V x 3 float64 array in device memory owned by a context, exposed
    through __cuda_array_interface__ (a view, no copy; the context rewrites it
    on its next call, so treat it as read-only)."""

    def __init__(self, ptr: int, shape):
        self.ptr = int(ptr)
        self.shape = tuple(shape)
        self.__cuda_array_interface__ = {"shape": self.shape, "typestr": "<f8", "data": (self.ptr, False),
                                         "version": 3, "strides": None}


class ArapContext:
    """Thin object wrapper over one ``arap_ctx``."""

    def __init__(self, n_vertices: int, faces: np.ndarray, device: int = 0):
        self.lib = load()
        self.V = int(n_vertices)
        self.faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        h = _P()
        rc = self.lib.arap_create(self.V, len(self.faces), _i32(self.faces), int(device), C.byref(h))
        if rc != ARAP_OK:
            raise ArapError(rc, self.lib.arap_last_error(None).decode())
        self.h = h

    def _check(self, rc: int):
        if rc != ARAP_OK:
            raise ArapError(rc, self.lib.arap_last_error(self.h).decode())

    def status(self, rc: int) -> int:
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.arap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_precision(self, precision: str = "fp64", refine_steps: int = 1):
        self._check(self.lib.arap_set_precision(self.h, PRECISION[precision], int(refine_steps)))

    def set_wait_limit(self, polls: int = 0):
        """Poll limit of the solves' waits for another task (0: the default)."""
        self._check(self.lib.arap_set_wait_limit(self.h, int(polls)))

    def set_symbolic_cache(self, enable: bool = True):
        """False: every dirty deform redoes the symbolic analysis, as the
        reference's SimplicialLDLT::compute does."""
        self._check(self.lib.arap_set_symbolic_cache(self.h, 1 if enable else 0))

    def set_factor_precision(self, bits: int = 64):
        """Mixed form: 64 = FP64 numeric factor rounded to FP32 for the solves
        (default), 32 = FP32 factor."""
        self._check(self.lib.arap_set_factor_precision(self.h, int(bits)))

    def set_rest_positions(self, xyz: np.ndarray):
        a = np.ascontiguousarray(xyz, dtype=np.float64).reshape(self.V, 3)
        self._check(self.lib.arap_set_rest_positions(self.h, _f64(a)))

    def set_constraints(self, idx, xyz):
        i = np.ascontiguousarray(idx, dtype=np.int32).reshape(-1)
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self._check(self.lib.arap_set_constraints(self.h, len(i), _i32(i), _f64(x)))

    def deform_rc(self, iterations: int, out: np.ndarray | None = None) -> int:
        ptr = _f64(out) if out is not None else None
        return self.lib.arap_deform(self.h, int(iterations), ptr)

    def deform(self, iterations: int, want_output: bool = True) -> np.ndarray | None:
        out = np.empty((self.V, 3), np.float64) if want_output else None
        self._check(self.deform_rc(iterations, out))
        return out

    def deform_poses_rc(self, targets, iterations: int, out=None) -> int:
        """arap_deform_poses: targets P x n_constrained x 3 (constrained vertices
        in ascending order) or None to reuse the device copy."""
        if targets is None:
            return self.lib.arap_deform_poses(self.h, int(self._nposes), None, int(iterations),
                                             _f64(out) if out is not None else None)
        t = np.ascontiguousarray(targets, dtype=np.float64)
        self._nposes = t.shape[0]
        return self.lib.arap_deform_poses(self.h, int(t.shape[0]), _f64(t), int(iterations),
                                         _f64(out) if out is not None else None)

    def deform_poses(self, targets, iterations: int) -> np.ndarray:
        """targets None: the ones already on the device (the previous call's,
        or arap_pose_targets')."""
        t = None if targets is None else np.ascontiguousarray(targets, dtype=np.float64)
        out = np.empty((self._nposes if t is None else t.shape[0], self.V, 3), np.float64)
        self._check(self.deform_poses_rc(t, iterations, out))
        return out

    def deform_async(self, iterations: int, out: np.ndarray | None = None) -> None:
        self._check(self.lib.arap_deform_async(self.h, int(iterations), _f64(out) if out is not None else None))

    def wait(self) -> None:
        self._check(self.lib.arap_wait(self.h))

    def set_graphs(self, enable: bool) -> None:
        self._check(self.lib.arap_set_graphs(self.h, 1 if enable else 0))

    def pose_targets(self, handles, transforms, origin=None):
        """Targets of len(transforms) rigid poses computed on the device
        (arap_pose_targets); the next deform_poses(None, ...) uses them."""
        h = np.ascontiguousarray(handles, dtype=np.int32).reshape(-1)
        t = np.ascontiguousarray(transforms, dtype=np.float64).reshape(-1, 12)
        o = None if origin is None else np.ascontiguousarray(origin, dtype=np.float64).reshape(12)
        self._check(self.lib.arap_pose_targets(self.h, len(h), _i32(h), _f64(o) if o is not None else None,
                                               len(t), _f64(t)))
        self._nposes = len(t)

    def vertex_normals(self) -> np.ndarray:
        out = np.empty((self.V, 3), np.float64)
        self._check(self.lib.arap_vertex_normals(self.h, _f64(out)))
        return out

    def device_positions(self, with_normals: bool = False):
        """(positions, normals) as DeviceArray views of the context's device
        buffers (no host copy; normals None unless asked); valid until the next
        call on the context. torch.as_tensor(view, device="cuda") wraps them."""
        p, n = _P(), _P()
        self._check(self.lib.arap_device_positions(self.h, int(bool(with_normals)), C.byref(p), C.byref(n)))
        pos = DeviceArray(p.value, (self.V, 3))
        return pos, (DeviceArray(n.value, (self.V, 3)) if with_normals else None)

    def host_timing(self) -> dict:
        v = np.zeros(5)
        self._check(self.lib.arap_get_host_timing(self.h, _f64(v)))
        return dict(zip(("analysis_upload", "alloc", "setup_enqueue", "iter_enqueue", "rest"), v.tolist()))

    def energy(self) -> float:
        e = C.c_double()
        self._check(self.lib.arap_energy(self.h, C.byref(e)))
        return e.value

    def set_ordering(self, mode: str):
        """"per_set" (default) or "mesh" (arap_set_ordering)."""
        self._check(self.lib.arap_set_ordering(self.h, {"per_set": 0, "mesh": 1}[mode]))

    def set_cluster_threshold(self, nbytes: int):
        self._check(self.lib.arap_set_cluster_threshold(self.h, int(nbytes)))

    def set_warp_rows(self, rows: int):
        """Largest front (rows) of the warp-per-supernode solves of the bottom levels (0: none)."""
        self._check(self.lib.arap_set_warp_rows(self.h, int(rows)))

    def set_vertex_launch(self, kernel, threads_per_vertex: int, block_threads: int = 256):
        """Launch shape of 'local', 'rhs' or 'residual' (or an ARAP_K_* code)."""
        code = {"local": ARAP_K_LOCAL, "rhs": ARAP_K_RHS, "residual": ARAP_K_RESIDUAL}.get(kernel, kernel)
        self._check(self.lib.arap_set_vertex_launch(self.h, int(code), int(threads_per_vertex), int(block_threads)))

    def set_solve_blocks(self, max_columns: int):
        """Largest level-1 subtree (columns) solved as one block by the
        single-request sweeps (0: none)."""
        self._check(self.lib.arap_set_solve_blocks(self.h, int(max_columns)))

    def set_solve_schedule(self, schedule):
        """'persistent' (one launch of persistent CTAs per sweep) or 'levels'
        (one launch per tree level, no waits) for the single-CTA solve levels."""
        code = {"persistent": ARAP_SOLVE_PERSISTENT, "levels": ARAP_SOLVE_LEVELS}.get(schedule, schedule)
        self._check(self.lib.arap_set_solve_schedule(self.h, int(code)))

    def set_dense_top(self, max_columns: int):
        """Columns of the tree's top solved through an explicit inverse (0: default, <0: none)."""
        self._check(self.lib.arap_set_dense_top(self.h, int(max_columns)))

    def set_solve_ctas(self, n: int):
        self._check(self.lib.arap_set_solve_ctas(self.h, int(n)))

    def set_pose_tile(self, poses: int):
        """Poses per batched-solve task of deform_poses (0: automatic)."""
        self._check(self.lib.arap_set_pose_tile(self.h, int(poses)))

    def set_targets(self, xyz):
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self._check(self.lib.arap_set_targets(self.h, len(x), _f64(x)))

    def device_bytes(self) -> int:
        return int(self.lib.arap_device_bytes(self.h))

    def invalidate(self):
        self._check(self.lib.arap_invalidate(self.h))

    def positions(self) -> np.ndarray:
        out = np.empty((self.V, 3), np.float64)
        self._check(self.lib.arap_get_positions(self.h, _f64(out)))
        return out

    def edge_weights(self):
        nnz = C.c_int32()
        self._check(self.lib.arap_edge_weights_nnz(self.h, C.byref(nnz)))
        rp = np.zeros(self.V + 1, np.int32)
        col = np.zeros(max(nnz.value, 1), np.int32)
        val = np.zeros(max(nnz.value, 1), np.float64)
        self._check(self.lib.arap_get_edge_weights(self.h, _i32(rp), _i32(col), _f64(val)))
        return rp, col[: nnz.value], val[: nnz.value]

    def rotations(self) -> np.ndarray:
        out = np.empty((self.V, 3, 3), np.float64)
        self._check(self.lib.arap_get_rotations(self.h, _f64(out)))
        return out

    def symbolic(self):
        m, s, nz = C.c_int32(), C.c_int32(), C.c_int64()
        self._check(self.lib.arap_get_symbolic_sizes(self.h, C.byref(m), C.byref(s), C.byref(nz)))
        perm = np.zeros(max(m.value, 1), np.int32)
        et = np.zeros(max(m.value, 1), np.int32)
        bp = np.zeros(s.value + 1, np.int32)
        self._check(self.lib.arap_get_symbolic(self.h, _i32(perm), _i32(et), _i32(bp)))
        return {"m": m.value, "perm": perm[: m.value], "etree": et[: m.value], "block_ptr": bp,
                "factor_nnz": nz.value}

    def timing(self):
        a, b = C.c_double(), C.c_double()
        self._check(self.lib.arap_get_timing(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check(self.lib.arap_get_launch_count(self.h, C.byref(n)))
        return n.value

    def stream(self) -> int:
        p = _P()
        self._check(self.lib.arap_get_stream(self.h, C.byref(p)))
        return int(p.value or 0)

    def set_profiling(self, enable: bool):
        self._check(self.lib.arap_set_profiling(self.h, 1 if enable else 0))

    def reset_kernel_stats(self):
        self._check(self.lib.arap_reset_kernel_stats(self.h))

    def kernel_model(self) -> dict:
        out = {}
        for k, name in enumerate(KERNEL_CLASSES):
            b, f = C.c_double(), C.c_double()
            self._check(self.lib.arap_get_kernel_model(self.h, k, C.byref(b), C.byref(f)))
            out[name] = (b.value, f.value)
        return out

    def kernel_stats(self) -> dict:
        out = {}
        for k, name in enumerate(KERNEL_CLASSES):
            ms, n = C.c_double(), C.c_int64()
            self._check(self.lib.arap_get_kernel_stats(self.h, k, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out


class MeshBatch:
    """Several meshes of uneven sizes deformed together in one set of launches.

    The meshes are packed into one block-diagonal problem over their disjoint
    union (mesh k's vertices at offset[k], its faces and constrained indices
    shifted by it): one context, so every kernel launch covers all meshes.
    The nested dissection orders each mesh (a connected component of the
    union) on its own, in parallel threads, so the elimination forest is the
    meshes' trees side by side; the persistent triangular solves take
    (mesh, supernode) tasks from one ticket queue, and the factorisation's
    launches of one tree level cover that level of every mesh. Each mesh is
    the reference's per-object problem (inc/deform/arap.h:101-138) and gets
    the result a context of its own would give up to the order of sums (the
    dense top of the union may differ from a lone mesh's). Every mesh needs
    a constrained vertex in each of its components, as a lone deform does.
    """

    def __init__(self, meshes, device: int = 0):
        """meshes: sequence of (n_vertices, faces)."""
        self.sizes = [int(v) for v, _ in meshes]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        faces = [np.ascontiguousarray(f, dtype=np.int64).reshape(-1, 3) + self.offsets[k]
                 for k, (_, f) in enumerate(meshes)]
        self.ctx = ArapContext(int(self.offsets[-1]), np.concatenate(faces).astype(np.int32), device=device)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def close(self):
        self.ctx.close()

    def set_rest_positions(self, positions):
        """positions: one (n_k, 3) array per mesh."""
        self.ctx.set_rest_positions(np.concatenate([np.asarray(p, dtype=np.float64).reshape(-1, 3)
                                                    for p in positions]))

    def _union_indices(self, idx):
        return np.concatenate([np.asarray(i, dtype=np.int64).reshape(-1) + self.offsets[k]
                               for k, i in enumerate(idx)]).astype(np.int32)

    def set_constraints(self, idx, targets):
        """idx, targets: one index array and one (c_k, 3) target array per mesh."""
        self._order = [np.argsort(np.asarray(i).reshape(-1), kind="stable") for i in idx]
        self.ctx.set_constraints(self._union_indices(idx),
                                 np.concatenate([np.asarray(t, dtype=np.float64).reshape(-1, 3) for t in targets]))

    def set_targets(self, targets):
        """New targets for the same constrained sets (no refactorisation), one
        (c_k, 3) array per mesh in the order of its set_constraints indices."""
        self.ctx.set_targets(np.concatenate([np.asarray(t, dtype=np.float64).reshape(-1, 3)[o]
                                             for t, o in zip(targets, self._order)]))

    def split(self, union_xyz: np.ndarray):
        return [union_xyz[self.offsets[k]:self.offsets[k + 1]] for k in range(len(self.sizes))]

    def deform(self, iterations: int):
        """One deform of every mesh; returns one (n_k, 3) array per mesh."""
        return self.split(self.ctx.deform(iterations))


def analyze_pattern(n_vertices: int, faces: np.ndarray, constrained) -> dict:
    """Host-only symbolic analysis (no GPU needed), see arap_analyze_pattern."""
    lib = load()
    f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
    c = np.ascontiguousarray(constrained, dtype=np.int32).reshape(-1)
    V = int(n_vertices)
    perm = np.zeros(max(V, 1), np.int32)
    et = np.zeros(max(V, 1), np.int32)
    bp = np.zeros(V + 1, np.int32)
    m, s, nz = C.c_int32(), C.c_int32(), C.c_int64()
    rc = lib.arap_analyze_pattern(V, len(f), _i32(f), len(c), _i32(c) if len(c) else None, C.byref(m),
                                  C.byref(s), C.byref(nz), _i32(perm), _i32(et), _i32(bp))
    if rc != ARAP_OK:
        raise ArapError(rc, lib.arap_last_error(None).decode())
    return {"m": m.value, "perm": perm[: m.value], "etree": et[: m.value], "block_ptr": bp[: s.value + 1],
            "factor_nnz": nz.value}


class ArapServer:
    """The request loop of ``arap_srv_*``: submit deform requests (mesh,
    constraint set, targets, iterations) from any thread; results arrive in
    per-request numpy arrays kept alive here until the ticket is collected."""

    def __init__(self, device: int = 0, precision: str = "mixed", refine_steps: int = 1, max_in_flight: int = 0,
                 budget_bytes: int = 0, prep_threads: int = 0, max_batch: int = 0, max_queue: int = 0,
                 poll_us: int = 0, solve_ctas: int = 0, per_set_ordering: bool = False):
        self.lib = load()
        cfg = ServerConfig(int(device), PRECISION[precision], int(refine_steps), int(max_in_flight),
                           int(budget_bytes), int(prep_threads), int(max_batch), int(max_queue), int(poll_us),
                           int(solve_ctas), int(bool(per_set_ordering)))
        h = _P()
        rc = self.lib.arap_srv_create(C.byref(cfg), C.byref(h))
        if rc != ARAP_OK:
            raise ArapError(rc, self.lib.arap_srv_last_error(None).decode())
        self.h = h
        self.V = {}
        self._live = {}

    def _check(self, rc: int):
        if rc != ARAP_OK:
            raise ArapError(rc, self.lib.arap_srv_last_error(self.h).decode())

    def add_mesh(self, positions, faces) -> int:
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        mid = C.c_int32()
        self._check(self.lib.arap_srv_add_mesh(self.h, len(pos), len(f), _i32(f), _f64(pos), C.byref(mid)))
        self.V[mid.value] = len(pos)
        return mid.value

    def submit(self, mesh: int, cidx, ctargets, iterations: int) -> int:
        idx = np.ascontiguousarray(cidx, dtype=np.int32).reshape(-1)
        tgt = np.ascontiguousarray(ctargets, dtype=np.float64).reshape(-1, 3)
        out = np.empty((self.V[mesh], 3), np.float64)
        req = Request(int(mesh), len(idx), _i32(idx), _f64(tgt), int(iterations), 0, _f64(out))
        t = C.c_int64()
        self._check(self.lib.arap_srv_submit(self.h, C.byref(req), C.byref(t)))
        self._live[t.value] = out
        return t.value

    @staticmethod
    def _info(i: RequestInfo) -> dict:
        return {"status": i.status, "factor_reused": bool(i.factor_reused), "batch_size": i.batch_size,
                "queue_ms": i.queue_ms, "latency_ms": i.latency_ms}

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(positions, info) once the request finished; None on timeout.
        Raises ArapError when the request failed."""
        info = RequestInfo()
        rc = self.lib.arap_srv_wait(self.h, int(ticket), int(timeout_ms), C.byref(info))
        if rc == ARAP_PENDING:
            return None
        out = self._live.pop(ticket, None)
        if rc != ARAP_OK:
            raise ArapError(rc, self.lib.arap_srv_last_error(self.h).decode())
        return out, self._info(info)

    def poll(self, ticket: int):
        return self.wait(ticket, 0)

    def stats(self) -> dict:
        st = ServerStats()
        self._check(self.lib.arap_srv_stats(self.h, C.byref(st)))
        out = {n: getattr(st, n) for n, _ in ServerStats._fields_ if n != "pad"}
        out["launch_host_ms"] = list(st.launch_host_ms)
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.arap_srv_destroy(self.h)
            self.h = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ArrayMesh:
    """Array-backed mesh adapter: the five accessors of the adapter concept
    (inc/deform/openmesh_adapter.h:74-113) over numpy arrays."""

    def __init__(self, positions: np.ndarray, faces: np.ndarray, scalar=np.float64):
        self.scalar = scalar
        self.positions = np.array(positions, dtype=scalar).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)

    def number_of_vertices(self) -> int:
        return len(self.positions)

    def number_of_faces(self) -> int:
        return len(self.faces)

    def vertex_location(self, i, value=None):
        if value is None:
            return self.positions[i].copy()
        self.positions[i] = value

    def face(self, i):
        return self.faces[i]


class AsRigidAsPossibleDeformation:
    """deform::AsRigidAsPossibleDeformation<Mesh, PrecisionType> on the GPU.

    ``precision`` "fp64" is PrecisionType=double; "mixed" is the FP32 GPU form
    with FP64-residual refinement (the reference's PrecisionType=float maps here)."""

    def __init__(self, mesh: ArrayMesh, precision: str = "fp64", refine_steps: int = 2, device: int = 0):
        self.mesh = mesh
        self.precision = precision
        self.ctx = ArapContext(mesh.number_of_vertices(), mesh.faces, device)
        self.ctx.set_precision(precision, refine_steps)
        self.scalar = np.float64 if precision == "fp64" else np.float32
        self._constraints: dict[int, np.ndarray] = {}
        self._dirty = True

    def set_constraint(self, vidx: int, loc) -> None:
        """arap.h:81-85: store loc cast to the compute scalar, mark dirty."""
        self._constraints[int(vidx)] = np.asarray(loc, dtype=self.scalar).astype(np.float64)
        self._dirty = True

    def deform(self, iterations: int) -> bool:
        """arap.h:101-138."""
        ctx = self.ctx
        if self._dirty:
            rest = self.mesh.positions.astype(self.scalar).astype(np.float64)
            ctx.set_rest_positions(rest)
            if self._constraints:
                idx = np.fromiter(self._constraints.keys(), np.int32, len(self._constraints))
                xyz = np.stack([self._constraints[int(i)] for i in idx])
            else:
                idx = np.zeros(0, np.int32)
                xyz = np.zeros((0, 3))
            rc = ctx.lib.arap_set_constraints(ctx.h, len(idx), _i32(idx), _f64(np.ascontiguousarray(xyz)))
            if rc != ARAP_OK:
                return False
        out = np.empty((ctx.V, 3), np.float64)
        rc = ctx.deform_rc(iterations, out)
        if rc == ARAP_ERR_NOT_SPD or rc == ARAP_ERR_BAD_INDEX:
            return False
        if rc != ARAP_OK:
            raise ArapError(rc, ctx.lib.arap_last_error(ctx.h).decode())
        if not self._constraints:
            return True  # arap.h:113-114: stays dirty, no write-back
        self._dirty = False
        self.mesh.positions[:] = out.astype(self.mesh.scalar)
        return True

    def cotan_weights(self):
        """PrivateAccessor<ARAP>::cotanWeights (tests/accessor.h:19-21) as a dense matrix."""
        rp, col, val = self.ctx.edge_weights()
        W = np.zeros((self.ctx.V, self.ctx.V))
        for i in range(self.ctx.V):
            W[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
        return W
