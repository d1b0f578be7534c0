"""Launch-shape autotuner: picks the number of CTAs per triangular-solve
launch (arap_set_solve_ctas) for a workload and a number of requests in
flight, the pose tile of the batched solves (arap_set_pose_tile), the
column cap of the elimination tree's dense top (arap_set_dense_top) and the
threads per vertex and block size of the per-vertex kernels
(arap_set_vertex_launch), by timing short trial runs through the C ABI.

One request alone is fastest with as many CTAs as fit on the device (the
default, 0); several requests in flight share the SMs, and a smaller count
per launch lets their solves run side by side instead of queueing behind
each other's CTAs. The best count depends on the mesh, the precision and the
concurrency, so it is measured rather than modelled. Results are cached per
(device, mesh size, constrained count, precision, concurrency, iterations) in
memory and, when a path is given, in a JSON file.
"""
from __future__ import annotations

import json
import time
from pathlib import Path

import numpy as np

import arap_gpu as G

CANDIDATES = (0, 64, 96, 128, 192, 256)
_cache: dict = {}


def _key(device: int, V: int, n_constrained: int, precision: str, concurrency: int, iterations: int,
         schedule: str = "persistent") -> str:
    return f"dev{device}:V{V}:c{n_constrained}:{precision}:x{concurrency}:it{iterations}:{schedule}"


def tune_solve_ctas(positions, faces, cidx, ctargets, iterations: int, precision: str = "mixed",
                    refine: int = 1, concurrency: int = 1, device: int = 0, candidates=CANDIDATES,
                    trials: int = 2, cache_file: str | Path | None = None, schedule: str = "persistent",
                    warp_rows: int = 0, solve_blocks: int = 0):
    """Returns (best_count, {count: iterations/s}) for `concurrency` concurrent
    dirty deforms of the given problem under the given solve schedule
    ('persistent' or 'levels', arap_set_solve_schedule)."""
    key = _key(device, len(positions), len(cidx), precision, concurrency, iterations,
               f"{schedule}:w{warp_rows}:b{solve_blocks}")
    if cache_file and Path(cache_file).exists():
        try:
            _cache.update(json.loads(Path(cache_file).read_text()))
        except Exception:
            pass
    if key in _cache:
        hit = _cache[key]
        return int(hit["best"]), {int(k): v for k, v in hit["rates"].items()}
    faces = np.ascontiguousarray(faces, dtype=np.int32)
    ctxs = []
    for _ in range(max(1, concurrency)):
        c = G.ArapContext(len(positions), faces, device=device)
        c.set_precision(precision, refine)
        c.set_solve_schedule(schedule)
        c.set_warp_rows(warp_rows)
        c.set_solve_blocks(solve_blocks)
        c.set_rest_positions(positions)
        c.set_constraints(cidx, ctargets)
        ctxs.append(c)
    rates = {}
    try:
        for n in candidates:
            for c in ctxs:
                c.set_solve_ctas(int(n))
                c.deform(iterations, want_output=False)  # set-up and graph capture, untimed
            best_dt = float("inf")
            for _ in range(max(1, trials)):
                t0 = time.perf_counter()
                for c in ctxs:
                    c.invalidate()
                    rc = c.lib.arap_deform_async(c.h, iterations, None)
                    if rc != G.ARAP_OK:
                        raise G.ArapError(rc, c.lib.arap_last_error(c.h).decode())
                for c in ctxs:
                    c.wait()
                best_dt = min(best_dt, time.perf_counter() - t0)
            rates[int(n)] = len(ctxs) * iterations / best_dt
    finally:
        for c in ctxs:
            c.close()
    best = max(rates, key=rates.get)
    _cache[key] = {"best": best, "rates": rates}
    if cache_file:
        try:
            Path(cache_file).write_text(json.dumps(_cache, indent=1))
        except Exception:
            pass
    return best, rates


POSE_TILES = (1, 2, 4, 8, 16)


def tune_pose_tile(ctx, iterations: int, candidates=POSE_TILES, trials: int = 2, dirty: bool = True):
    """Returns (best_tile, {tile: ms per call}) for arap_deform_poses on a
    context whose pose targets are already on the device (a previous
    deform_poses or pose_targets). Tiles the mesh's fronts do not allow are
    skipped. dirty=True times a full dirty call (weights and factor included),
    as DeformationUtil's loop of dirty deforms does. Leaves the best tile set."""
    times = {}
    for pt in candidates:
        try:
            ctx.set_pose_tile(int(pt))
            ctx.deform_poses(None, iterations)  # schedule reset and first launch, untimed
            ctx.deform_poses(None, iterations)  # graph capture, untimed
        except G.ArapError as e:
            if e.code == G.ARAP_ERR_UNSUPPORTED:
                continue
            raise
        best = float("inf")
        for _ in range(max(1, trials)):
            if dirty:
                ctx.invalidate()
            t0 = time.perf_counter()
            rc = ctx.deform_poses_rc(None, iterations, None)
            if rc != G.ARAP_OK:
                raise G.ArapError(rc, ctx.lib.arap_last_error(ctx.h).decode())
            best = min(best, time.perf_counter() - t0)
        times[int(pt)] = 1e3 * best
    if not times:
        raise G.ArapError(G.ARAP_ERR_UNSUPPORTED, "no pose tile fits this mesh")
    best_pt = min(times, key=times.get)
    ctx.set_pose_tile(best_pt)
    return best_pt, times


DENSE_TOPS = (-1, 1024, 2048, 3072, 4096)


def tune_dense_top(ctx, iterations: int, batched: bool, candidates=DENSE_TOPS, trials: int = 2):
    """Returns (best_cap, {cap: ms per call}): the column cap of the tree's top
    solved through its explicit inverse (arap_set_dense_top; -1: none), timed
    on full dirty calls (weights, factor, inverse of the top, iterations) of
    arap_deform_poses when batched (pose targets already on the device) or of
    arap_deform. A wider top trades the supernodal tasks of the upper levels
    for wider products with T, formed once per factorisation. Leaves the best
    cap set."""
    times = {}
    for cap in candidates:
        ctx.set_dense_top(int(cap))

        def call():
            if batched:
                return ctx.deform_poses_rc(None, iterations, None)
            return ctx.deform_rc(iterations)

        for _ in range(2):  # set-up and schedule reset, then graph capture: untimed
            ctx.invalidate()
            rc = call()
            if rc != G.ARAP_OK:
                raise G.ArapError(rc, ctx.lib.arap_last_error(ctx.h).decode())
        best = float("inf")
        for _ in range(max(1, trials)):
            ctx.invalidate()
            t0 = time.perf_counter()
            rc = call()
            if rc != G.ARAP_OK:
                raise G.ArapError(rc, ctx.lib.arap_last_error(ctx.h).decode())
            best = min(best, time.perf_counter() - t0)
        times[int(cap)] = 1e3 * best
    best_cap = min(times, key=times.get)
    ctx.set_dense_top(best_cap)
    return best_cap, times


# (threads per vertex, block threads) candidates of the per-vertex kernels
VERTEX_SHAPES = {
    "local": ((1, 64), (1, 128), (1, 256), (2, 128), (2, 256), (4, 256)),
    "rhs": ((1, 128), (1, 256), (1, 512), (2, 256), (4, 256), (8, 256), (32, 256)),
    "residual": ((1, 128), (1, 256), (1, 512), (2, 256), (4, 256), (8, 256), (32, 256)),
}


def tune_vertex_launch(ctx, iterations: int, shapes=None, trials: int = 2):
    """Per-vertex kernels of the single-request iterations (local step, RHS,
    FP64 residual): threads per vertex (lanes of a warp splitting a vertex's
    adjacency entries, up to a warp per vertex) and block size, each timed by
    the per-launch profiler over `iterations` iterations of the context's
    current problem (set up and deformed once before). Returns
    {kernel: ((tpv, block), {"tpv x block": us per launch})} and leaves the
    best shapes set."""
    shapes = shapes or VERTEX_SHAPES
    out = {}
    ctx.set_profiling(True)
    try:
        for name, cands in shapes.items():
            times = {}
            for tpv, blk in cands:
                ctx.set_vertex_launch(name, tpv, blk)
                best = float("inf")
                for _ in range(max(1, trials)):
                    ctx.reset_kernel_stats()
                    ctx.deform(iterations, want_output=False)
                    ms, n = ctx.kernel_stats()[name]
                    if n:
                        best = min(best, ms / n)
                if best < float("inf"):
                    times[(tpv, blk)] = best
            if not times:  # the kernel does not run in this precision
                ctx.set_vertex_launch(name, 1, 256)
                continue
            pick = min(times, key=times.get)
            ctx.set_vertex_launch(name, *pick)
            out[name] = (pick, {f"{t}x{b}": round(v * 1e3, 2) for (t, b), v in times.items()})
    finally:
        ctx.set_profiling(False)
    return out
