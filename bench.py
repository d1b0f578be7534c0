#!/usr/bin/env python
"""ARAP deformation benchmark: ARAP iterations/s on one GB300.

Workload (one "step"): 16 concurrent dirty deforms (one per host thread, as
the reference arm runs one request per host thread) of the twisted bar -- the
10x1x1 box surface at 0.025 spacing (67,202 vertices, 134,400 triangles),
anchors x<0.2 (2,801), handles x>9.8 (2,801) turned 90 deg about the bar axis
and shifted (0,0.5,0) -- in the mixed-precision form (FP64 numeric factor,
FP32 local steps and solves, two FP64-residual refinement solves per
iteration), 30 local/global iterations each. A dirty deform is what the
reference does after setConstraint (inc/deform/arap.h:102-129): the symbolic
analysis of the constrained Laplacian (redone on every request, as
SimplicialLDLT::compute does), cotan weights, numeric factorisation, then the
iterations. Inputs are seeded synthetic meshes (the reference publishes no
data set).

value: iterations/s with the rest pose and targets already in device memory,
       timed with CUDA events from a start event on the idle device to the
       last request's end event; L2 (129 MB) is flushed before each step by
       writing a 256 MB buffer, outside the timed events.
e2e:   the same steps through the C ABI with host buffers: pinned rest
       positions and targets copied in, deformed positions copied out, wall
       clock; one end-to-end step precedes each timed device step.
repose_refactor: the same steps with the symbolic analysis kept (the
       constrained set does not change), reported beside the headline.
cpu_baseline: the FP64 C restatement of arap.h (the oracle) on one host core,
       full requests of the same workload; its output also gives the error of
       the GPU result (bbox-diagonal-relative, stated on every line).

--impl reference times the reference's CPU path (the oracle restatement,
since the reference needs Eigen and cannot be built) with one independent
request per host thread.
Multi-GPU: replicas only (one independent replica per rank, no collective);
--gpus N without torchrun starts N replicas through torch.distributed.run.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "mesh-deform_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "ARAP iterations/s and p50/p99 deform latency at <=1e-6 bbox-rel error vs FP64"
UNIT = "iterations/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload(args):
    import arap_workloads as W

    if args.workload == "twisted_bar":
        return W.cfg_twisted_bar(h=args.h, iterations=args.iterations, precision=args.precision)
    if args.workload == "icosphere_l4":
        w = W.cfg_icosphere_l4(iterations=args.iterations)
        w.precision = args.precision
        return w
    if args.workload == "noisy_sphere":
        return W.cfg_noisy_sphere(iterations=args.iterations, precision=args.precision)
    if args.workload == "pose_batch":
        return W.cfg_pose_batch(level=5, n_poses=args.poses, iterations=args.iterations, precision="mixed")
    raise SystemExit(f"unknown workload {args.workload}")


def config_of(w, args, extra=None):
    c = {
        "workload": w.name,
        "vertices": w.V,
        "faces": w.F,
        "constrained": int(len(w.cidx)),
        "free": int(w.V - len(w.cidx)),
        "iterations_per_step": w.iterations,
        "precision": args.precision,
        "step": "dirty deform (weights + factor + iterations)",
        "l2": "flushed before every step (256 MB write)",
        "parallelism": f"replicas{int(os.environ.get('WORLD_SIZE', '1'))}",
    }
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_requests(w, n_requests: int, threads: int):
    """n_requests full dirty deforms of w by the FP64 oracle, on `threads` threads.
    Returns (seconds, last output)."""
    from oracle import oracle as O

    O.build()
    O.load()

    def one(_):
        ok, out = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
        assert ok
        return out

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        outs = list(ex.map(one, range(n_requests)))
    return time.perf_counter() - t0, outs[-1]


def run_reference(args):
    """The reference's CPU path (oracle restatement), one request per host thread."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    w = workload(args)
    threads = os.cpu_count() or 1
    per_step = []
    for s in range(args.warmup + args.steps):
        dt, _ = cpu_oracle_requests(w, threads, threads)
        if s >= args.warmup:
            per_step.append(dt)
    total = sum(per_step)
    its = threads * w.iterations * len(per_step)
    value = its / total
    sample = f"{threads} concurrent dirty deform({w.iterations}) requests per step on {w.name}"
    line = {
        "impl": "reference",
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / len(per_step), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(w, args, {"precision": "fp64", "threads": threads}),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "latency_ms": {"p50": 1e3 * statistics.median(per_step), "p99": 1e3 * float(np.percentile(per_step, 99))},
    }
    print(json.dumps(line), flush=True)
    return 0


FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64, nominal (the measured peaks hold no FP64 figure)


def roofline_of(kstats, kmodel, steps, peaks, wname, factorisations):
    """Roofline of the dominant kernel class and of the factorisation.

    The dominant class is the one with the most device time among the
    classes that run one kernel kind per launch (local step, RHS, residual,
    the two sweeps, ...): HBM-bound, algorithmic bytes of one launch over its
    average CUDA-event duration against the measured copy bandwidth. The
    factorisation is a sequence of seven kernel kinds over the tree's levels
    (none of them alone as long as a sweep class) and is bound by the FP64
    units: its algorithmic flops (the dense Cholesky's, sum over supernodes of
    c^3/3 + c^2 b + c b^2) over its time per factorisation, against the
    nominal FP64 rate."""
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    cands = {k: v for k, v in kstats.items() if k != "factor" and v[1] > 0}
    dom = max(cands, key=lambda k: cands[k][0])
    dom_ms, dom_n = kstats[dom]
    per_launch_ms = dom_ms / max(dom_n, 1)
    dom_bytes = kmodel[dom][0]
    achieved = dom_bytes / (per_launch_ms * 1e-3) / 1e9
    traffic = None
    tfile = ROOT / "profiles" / "ncu_traffic.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get(wname, {}).get(dom)
        except Exception:
            traffic = None
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "traffic": traffic,
            "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
            "bytes_per_launch": dom_bytes, "ms_per_launch": per_launch_ms,
            "dominant_by": "device time among the single-kernel classes; the factorisation is in factor_roofline"}
    fms = kstats.get("factor", (0.0, 0))[0] / max(factorisations, 1)
    ffl = kmodel.get("factor", (0.0, 0.0))[1]
    froof = None
    if fms > 0:
        tf = ffl / (fms * 1e-3) / 1e12
        froof = {"bound": "fp64", "achieved": tf, "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                 "frac": tf / FP64_NOMINAL_TFLOPS, "peak_source": "nominal",
                 "flops_per_factorisation": ffl, "ms_per_factorisation": fms,
                 "share_of_request_kernel_time": kstats["factor"][0] / max(sum(v[0] for v in kstats.values()), 1e-9)}
    return roof, froof



def run_batch(args):
    """Many poses of one mesh per step (arap_deform_poses): one factorisation
    shared by all poses, P x 3 right-hand sides per triangular solve."""
    import torch
    import arap_gpu as G
    import arap_workloads as W

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = workload(args)
    P = w.poses.shape[0]
    ctx = G.ArapContext(w.V, w.faces, device=local)
    ctx.set_precision("mixed", args.refine)
    ctx.set_factor_precision(args.factor_bits)
    ctx.set_rest_positions(w.positions)
    ctx.set_constraints(w.cidx, w.poses[0])
    dense_tuned = None
    if args.dense_top == "auto":
        import arap_tune

        ctx.deform_poses(w.poses, w.iterations)  # targets on the device
        best_cap, times = arap_tune.tune_dense_top(ctx, w.iterations, batched=True)
        dense_tuned = {"dense_top": best_cap, "ms_per_call": {str(k): round(v, 3) for k, v in times.items()}}
        log(f"autotuned dense top: {best_cap} {dense_tuned['ms_per_call']}")
    else:
        ctx.set_dense_top(int(args.dense_top))
    first = ctx.deform_poses(w.poses, w.iterations)
    tuned = None
    if args.pose_tile < 0:
        import arap_tune

        best, times = arap_tune.tune_pose_tile(ctx, w.iterations)
        tuned = {"pose_tile": best, "ms_per_call": {str(k): round(v, 3) for k, v in times.items()}}
        log(f"autotuned pose tile: {best} {tuned['ms_per_call']}")
        args.pose_tile = best
    else:
        ctx.set_pose_tile(args.pose_tile)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        ctx.invalidate()  # refactor each step: the step is a full dirty deform of every pose
        rc = ctx.deform_poses_rc(None, w.iterations, None)
        if rc != G.ARAP_OK:
            raise G.ArapError(rc, ctx.lib.arap_last_error(ctx.h).decode())

    ctx.set_symbolic_cache(args.cached_analysis)
    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        step()
    clocks = ClockSampler(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches = 0
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks.start()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
        launches += ctx.launch_count()
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    repose = None
    if not args.cached_analysis:  # the same step with the symbolic analysis kept
        ctx.set_symbolic_cache(True)
        for _ in range(args.warmup):
            flush.zero_()
            torch.cuda.synchronize()
            step()
        rms = []
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            rms.append(a.elapsed_time(b))
        repose = {"value": P * w.iterations * args.steps / (sum(rms) / 1e3), "unit": UNIT,
                  "ms_per_step": sum(rms) / len(rms),
                  "step": "the same step with the symbolic analysis of the unchanged constraint set kept"}
        ctx.set_symbolic_cache(args.cached_analysis)
    ctx.set_profiling(True)
    ctx.reset_kernel_stats()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        step()
    kstats = ctx.kernel_stats()
    kmodel = ctx.kernel_model()
    ctx.set_profiling(False)
    total_ms = sum(step_ms)
    if dist is not None:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    its_total = P * w.iterations * args.steps * world
    value = its_total / (total_ms / 1e3)
    tg_h = torch.from_numpy(np.ascontiguousarray(w.poses)).pin_memory().numpy()
    tf_h = torch.from_numpy(np.ascontiguousarray(w.info["transforms"].reshape(P, 12))).pin_memory().numpy()
    handles = w.info["handle_ids"]
    out_h = torch.empty((P, w.V, 3), dtype=torch.float64).pin_memory().numpy()
    # e2e: each step maps the P rigid poses to handle targets on the device
    # (arap_pose_targets, DeformationUtil::updateConstraints) and deforms them;
    # e2e_explicit_targets uploads the P x n_constrained x 3 targets instead
    e2e_s, e2e_x = [], []
    for k in range(0 if args.skip_e2e else args.warmup + args.steps):
        for mode in ("rigid", "explicit"):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.invalidate()
            if mode == "rigid":
                ctx.pose_targets(handles, tf_h, w.info["origin"])
                rc = ctx.deform_poses_rc(None, w.iterations, out_h)
            else:
                rc = ctx.deform_poses_rc(tg_h, w.iterations, out_h)
            t1 = time.perf_counter()
            if rc != G.ARAP_OK:
                raise G.ArapError(rc, ctx.lib.arap_last_error(ctx.h).decode())
            if k >= args.warmup:
                (e2e_s if mode == "rigid" else e2e_x).append(t1 - t0)
    e2e_total = sum(e2e_s) if e2e_s else float("nan")
    if dist is not None and e2e_s:
        t = torch.tensor([e2e_total], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    roof, froof = roofline_of(kstats, kmodel, args.steps, peaks, w.name, args.steps)
    cpu = None
    err = None
    if rank == 0 and not args.no_cpu_baseline and e2e_s:
        from oracle import oracle as O

        O.build()
        n = min(args.cpu_requests * 4, P)
        t0 = time.perf_counter()
        errs = []
        for p in range(n):
            ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.poses[p], w.iterations)
            errs.append(W.bbox_rel_error(out_h[p], ref, w.positions))
        dt = time.perf_counter() - t0
        err = max(errs)
        cpu = {"value": n * w.iterations / dt, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{n} poses of {w.name}, one dirty deform({w.iterations}) each on one thread ({dt:.1f} s)"}
        log(f"max error vs FP64 oracle over {n} poses: {err:.3e}")
    lat = sorted(step_ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": config_of(w, args, {"poses": P,
                                      "step": f"dirty deform of {P} poses (symbolic analysis "
                                              f"{'kept' if args.cached_analysis else 'redone'}, one shared "
                                              f"factorisation, {w.iterations} iterations)",
                                      "factor": f"fp{args.factor_bits}",
                                      "fp64_residual_solves_per_iteration": 1 + args.refine,
                                      "precision": "mixed", "pose_tile": args.pose_tile,
                                      "pose_tile_autotune": tuned,
                                      "dense_top": dense_tuned["dense_top"] if dense_tuned else int(args.dense_top),
                                      "dense_top_autotune": dense_tuned}),
        "e2e": {"value": its_total / e2e_total if e2e_s else None, "unit": UNIT,
                "h2d_bytes_per_step": int(tf_h.nbytes + handles.nbytes + 96), "d2h_bytes_per_step": int(out_h.nbytes),
                "inputs": "P rigid transforms, targets mapped on the device"},
        "repose_refactor": repose,
        "e2e_explicit_targets": {"value": its_total / sum(e2e_x) if e2e_x else None, "unit": UNIT,
                                 "h2d_bytes_per_step": int(tg_h.nbytes), "d2h_bytes_per_step": int(out_h.nbytes)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "factor_roofline": froof,
        "cpu_baseline": cpu,
        "error_vs_fp64_oracle": err,
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": float(np.percentile(lat, 99))},
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in kstats.items()},
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0

def mesh_batch_workloads(iterations: int):
    """Sixteen meshes of uneven sizes (642 to 67,202 vertices, 238,882 in
    all), each with its own constraint set: bars of different lengths and
    spacings, icospheres and noisy spheres of levels 3 to 6."""
    import arap_workloads as W

    ws = [W.cfg_twisted_bar(h=0.025, iterations=iterations), W.cfg_twisted_bar(h=0.05, iterations=iterations),
          W.cfg_twisted_bar(h=0.04, iterations=iterations, length=6.0),
          W.cfg_twisted_bar(h=0.1, iterations=iterations)]
    ws += [W.cfg_icosphere_l4(level=lv, iterations=iterations) for lv in (6, 5, 5, 4, 4, 3)]
    ws += [W.cfg_noisy_sphere(level=lv, seed=100 + k, iterations=iterations) for k, lv in enumerate((6, 5, 5, 4, 4, 3))]
    return ws


def run_mesh_batch(args):
    """Meshes of uneven sizes per step in one set of launches (MeshBatch: the
    disjoint union as one block-diagonal problem), against the same meshes as
    separate contexts, one host thread each, all in flight at once."""
    import torch
    import arap_gpu as G

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ws = mesh_batch_workloads(args.iterations)
    its = args.iterations
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    mb = G.MeshBatch([(w.V, w.faces) for w in ws], device=local)
    mb.ctx.set_precision(args.precision, args.refine)
    if args.precision == "mixed":
        mb.ctx.set_factor_precision(args.factor_bits)
    mb.set_rest_positions([w.positions for w in ws])
    mb.set_constraints([w.cidx for w in ws], [w.ctargets for w in ws])
    outs = mb.deform(its)
    stream = torch.cuda.ExternalStream(mb.ctx.stream(), device=dev)

    def batch_step():
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mb.ctx.invalidate()
        mb.ctx.deform(its, want_output=False)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), mb.ctx.launch_count()

    for _ in range(args.warmup):
        batch_step()
    clocks = ClockSampler(local)
    clocks.start()
    ms, launches = [], 0
    for _ in range(args.steps):
        t, n = batch_step()
        ms.append(t)
        launches += n
    clk = clocks.stop()
    # end to end: host buffers in (rest poses, constraint sets and targets),
    # deformed positions out, through the same API
    rest_h = [torch.from_numpy(np.ascontiguousarray(w.positions)).pin_memory().numpy() for w in ws]
    idx_h = [np.ascontiguousarray(w.cidx, dtype=np.int32) for w in ws]
    tgt_h = [np.ascontiguousarray(w.ctargets) for w in ws]
    e2e = []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mb.set_rest_positions(rest_h)
        mb.set_constraints(idx_h, tgt_h)
        mb.deform(its)
        if k >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    # the same meshes as separate contexts, one host thread each
    ctxs = []
    for w in ws:
        c = G.ArapContext(w.V, w.faces, device=local)
        c.set_precision(args.precision, args.refine)
        if args.precision == "mixed":
            c.set_factor_precision(args.factor_bits)
        c.set_rest_positions(w.positions)
        c.set_constraints(w.cidx, w.ctargets)
        c.deform(its, want_output=False)
        ctxs.append(c)
    streams = [torch.cuda.ExternalStream(c.stream(), device=dev) for c in ctxs]
    pool = ThreadPoolExecutor(max_workers=len(ctxs))

    def separate_step():
        flush.zero_()
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        start.record(streams[0])
        ends = [torch.cuda.Event(enable_timing=True) for _ in ctxs]

        def one(i):
            c = ctxs[i]
            c.invalidate()
            rc = c.lib.arap_deform_async(c.h, its, None)
            ends[i].record(streams[i])
            if rc != G.ARAP_OK:
                raise G.ArapError(rc, c.lib.arap_last_error(c.h).decode())
            c.wait()

        list(pool.map(one, range(len(ctxs))))
        torch.cuda.synchronize()
        return max(start.elapsed_time(e) for e in ends)

    for _ in range(args.warmup):
        separate_step()
    sep = [separate_step() for _ in range(args.steps)]
    pool.shutdown()
    for c in ctxs:
        c.close()
    # errors against the oracle on the smaller meshes of the batch
    from oracle import oracle as O

    err = 0.0
    checked = 0
    for w, got in zip(ws, outs):
        if w.V > 12000:
            continue
        ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, its)
        if ok:
            err = max(err, W_bbox(got, ref, w.positions))
            checked += 1
    mb.close()
    total_its = len(ws) * its
    value = total_its * args.steps / (sum(ms) / 1e3)
    h2d = sum(r.nbytes for r in rest_h) + sum(i.nbytes for i in idx_h) + sum(t.nbytes for t in tgt_h)
    d2h = sum(w.V * 24 for w in ws)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(ms) / len(ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": "mesh_batch_16", "meshes": len(ws), "vertices": [w.V for w in ws],
                   "vertices_total": sum(w.V for w in ws), "iterations_per_step": its,
                   "precision": args.precision,
                   "step": "one dirty deform of every mesh of the batch in one set of launches (the constraint "
                           "sets are unchanged, so the symbolic analysis is kept): weights, numeric "
                           "factorisation, iterations",
                   "l2": "flushed before every step (256 MB write)", "parallelism": "replicas1",
                   "factor": f"fp{args.factor_bits}" if args.precision == "mixed" else "fp64"},
        "e2e": {"value": total_its * len(e2e) / sum(e2e), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "timing": "host wall clock: rest poses, constraint sets and targets uploaded, deform, "
                          "positions copied out"},
        "separate_contexts": {"value": total_its * len(sep) / (sum(sep) / 1e3), "unit": UNIT,
                              "ms_per_step": sum(sep) / len(sep),
                              "step": "the same meshes as 16 contexts, one host thread each, all in flight"},
        "gpu_launches": launches,
        "error_vs_fp64_oracle": {"max": err, "meshes_checked": checked},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    return 0


def W_bbox(a, b, rest):
    import arap_workloads as W

    return W.bbox_rel_error(a, b, rest)


def _pct(xs, q):
    return float(np.percentile(xs, q)) if xs else None


def _serve_stream(G, W, pool, reqs, args, local, clocks=None):
    """Submits reqs at their arrival times to a fresh server, collects every
    result; returns per-request (latency_ms, queue_ms, reused, batch, mesh V,
    iterations) and the stream's wall time and server stats."""
    srv = G.ArapServer(device=local, precision="mixed", refine_steps=args.refine,
                       max_in_flight=args.serve_in_flight, prep_threads=args.serve_prep_threads,
                       max_batch=args.serve_max_batch, solve_ctas=args.serve_solve_ctas)
    ids = [srv.add_mesh(m.positions, m.faces) for m in pool]
    tickets = [None] * len(reqs)
    t0 = time.perf_counter()

    def submitter():
        for k, r in enumerate(reqs):
            dt = r.arrival - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets[k] = srv.submit(ids[r.mesh], r.cidx, r.ctargets, r.iterations)

    th = threading.Thread(target=submitter)
    if clocks:
        clocks.start()
    th.start()
    rows, outs = [], {}
    for k, r in enumerate(reqs):
        while tickets[k] is None:
            time.sleep(50e-6)
        out, info = srv.wait(tickets[k])
        rows.append((info["latency_ms"], info["queue_ms"], info["factor_reused"], info["batch_size"],
                     pool[r.mesh].V, r.iterations))
        if k < args.serve_check:
            outs[k] = out
    wall = time.perf_counter() - t0
    th.join()
    clk = clocks.stop() if clocks else None
    st = srv.stats()
    srv.close()
    return rows, wall, st, outs, clk


def run_serving(args):
    """Serving stream: Poisson arrivals of deform requests over a pool of 64
    meshes (noisy icospheres L3-L6, bars of 1k-200k vertices), each with 1-8
    handle caps plus an anchor cap, half reusing a constraint set seen before,
    5-50 iterations; through arap_srv_* (resident factors keyed by mesh and
    constraint set, admission by device footprint, multi-pose batching,
    concurrent launches). Reported per arrival rate: iterations/s and p50/p99
    latency (submit -> result in host memory), beside the plain per-request
    FP64 GPU form (a dirty arap_deform per request, one at a time)."""
    import torch
    import arap_gpu as G
    import arap_workloads as W

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    pool = W.serving_pool(n_meshes=64, seed=20261203)
    rates = [float(x) for x in args.serve_rates.split(",")]
    runs = []
    peak_clk = None
    # warm-up: a short stream (graph capture, kernel attribute set-up, pool memory)
    warm = W.serving_requests(pool, max(8, args.warmup * 4), seed=1, rate_hz=None)
    _serve_stream(G, W, pool, warm, args, local)
    for i, rate in enumerate(rates):
        reqs = W.serving_requests(pool, args.serve_requests, seed=20261204 + i, rate_hz=None if rate <= 0 else rate)
        clocks = ClockSampler(local)
        rows, wall, st, outs, clk = _serve_stream(G, W, pool, reqs, args, local, clocks)
        lat = [r[0] for r in rows]
        hit = [r[0] for r in rows if r[2]]
        miss = [r[0] for r in rows if not r[2]]
        its = sum(r[5] for r in rows)
        small = [r[0] for r in rows if 8000 <= r[4] <= 12000]
        run = {"rate_hz": rate if rate > 0 else "all at t=0", "requests": len(rows), "wall_s": wall,
               "iterations_per_s": its / wall, "requests_per_s": len(rows) / wall,
               "latency_ms": {"p50": _pct(lat, 50), "p99": _pct(lat, 99)},
               "latency_ms_factor_reused": {"n": len(hit), "p50": _pct(hit, 50), "p99": _pct(hit, 99)},
               "latency_ms_new_factor": {"n": len(miss), "p50": _pct(miss, 50), "p99": _pct(miss, 99)},
               "latency_ms_10k_meshes": {"n": len(small), "p50": _pct(small, 50), "p99": _pct(small, 99)},
               "queue_ms": {"p50": _pct([r[1] for r in rows], 50), "p99": _pct([r[1] for r in rows], 99)},
               "stats": {k: st[k] for k in ("factor_hits", "factor_misses", "evictions", "launches",
                                             "batched_launches", "batched_requests", "peak_resident_bytes",
                                             "budget_bytes", "scheduler_busy_ms", "worker_busy_ms", "analyze_ms",
                                             "staging_ms", "device_ms", "launch_ms", "launch_host_ms")},
               "device_spans_in_flight_avg": st["device_ms"] / (1e3 * wall),
               "scheduler_busy_frac": st["scheduler_busy_ms"] / (1e3 * wall),
               "clocks": clk}
        # error against the FP64 oracle on a sample of small requests
        if rank == 0 and not args.no_cpu_baseline:
            from oracle import oracle as O

            O.build()
            errs = []
            for k, out in outs.items():
                r = reqs[k]
                m = pool[r.mesh]
                if m.V > 20000:
                    continue
                ok, ref = O.run_deform(m.positions, m.faces, r.cidx, r.ctargets, r.iterations)
                errs.append(W.bbox_rel_error(out, ref, m.positions))
            run["error_vs_fp64_oracle"] = {"max": max(errs) if errs else None, "checked": len(errs)}
        runs.append(run)
        log(json.dumps(run))
        if clk:
            peak_clk = clk
    # the plain per-request FP64 GPU form on the first requests of the same stream
    reqs = W.serving_requests(pool, args.serve_fp64_requests, seed=20261204)
    ctxs = {}
    lat64 = []
    its64 = 0
    t0 = time.perf_counter()
    for r in reqs:
        m = pool[r.mesh]
        if r.mesh not in ctxs:
            c = G.ArapContext(m.V, m.faces, device=local)
            c.set_precision("fp64", 0)
            c.set_rest_positions(m.positions)
            ctxs[r.mesh] = c
        c = ctxs[r.mesh]
        a = time.perf_counter()
        c.set_constraints(r.cidx, r.ctargets)
        c.deform(r.iterations)
        lat64.append(1e3 * (time.perf_counter() - a))
        its64 += r.iterations
    wall64 = time.perf_counter() - t0
    for c in ctxs.values():
        c.close()
    fp64 = {"requests": len(reqs), "iterations_per_s": its64 / wall64,
            "latency_ms": {"p50": _pct(lat64, 50), "p99": _pct(lat64, 99)},
            "form": "one dirty arap_deform per request, FP64, one request at a time"}
    best = max(runs, key=lambda x: x["iterations_per_s"])
    line = {
        "metric": METRIC, "value": best["iterations_per_s"], "unit": UNIT, "n_gpus": 1,
        "steps": len(runs), "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "serving_stream", "meshes": len(pool),
                   "pool_vertices": int(sum(m.V for m in pool)),
                   "requests_per_rate": args.serve_requests, "rates_hz": rates,
                   "max_in_flight": args.serve_in_flight, "prep_threads": args.serve_prep_threads,
                   "max_batch": args.serve_max_batch, "precision": "mixed", "refine_steps": args.refine},
        "latency_ms": best["latency_ms"],
        "runs": runs,
        "fp64_per_request": fp64,
        "served_vs_fp64_iterations_ratio": best["iterations_per_s"] / fp64["iterations_per_s"],
        "clocks": peak_clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def reduce_max(x: float, dist, device=None) -> float:
    """Largest x over the ranks of the process group (x itself without one):
    the step time of a replica run is the slowest rank's."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def spawn_replicas(args) -> int:
    """bench.py --gpus N (N > 1) started without torchrun: one replica process
    per GPU through torch.distributed.run on this node, rank 0 prints."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve())] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="twisted_bar")
    ap.add_argument("--h", type=float, default=0.025)
    ap.add_argument("--iterations", type=int, default=None,
                    help="local/global iterations per deform (default: the configuration's own: twisted bar 30, "
                         "icosphere L4 10, noisy sphere 50, pose batch 20, mesh batch 30)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--refine", type=int, default=1,
                    help="mixed form: refinement solves per iteration beyond the first (every solve corrects the "
                         "positions from an FP64 residual; 1 gives two per iteration)")
    ap.add_argument("--factor-bits", type=int, default=64, choices=[32, 64],
                    help="mixed form: numeric factorisation in FP64 (default) or FP32")
    ap.add_argument("--cached-analysis", action="store_true",
                    help="headline step keeps the symbolic analysis of the unchanged constraint set")
    ap.add_argument("--cpu-requests", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true", help="profiling runs: skip the end-to-end pass")
    ap.add_argument("--poses", type=int, default=256, help="pose_batch: handle poses per step")
    ap.add_argument("--dense-top", default="auto",
                    help="pose_batch: column cap of the tree's dense top (-1: none; 0: the library default; "
                         "'auto': autotuned)")
    ap.add_argument("--pose-tile", type=int, default=-1,
                    help="pose_batch: poses per batched-solve task (0: largest that fits; -1: autotuned)")
    ap.add_argument("--solve-schedule", default="auto", choices=["auto", "persistent", "levels"],
                    help="single-request solves: persistent CTAs per sweep or one launch per tree level "
                         "(auto: autotuned with the CTA count when requests run concurrently)")
    ap.add_argument("--vertex-launch", default="auto", choices=["auto", "default"],
                    help="threads per vertex and block size of the local step, RHS and residual "
                         "(auto: autotuned per kernel before the timed region)")
    ap.add_argument("--solve-blocks", type=int, default=512,
                    help="single-request solves: level-1 subtrees of at most this many columns as one block (0: none)")
    ap.add_argument("--warp-rows", type=int, default=-1,
                    help="single-request solves: fronts of at most this many rows solved one warp per supernode "
                         "(-1: autotuned with the CTA count when requests run concurrently, else 0)")
    ap.add_argument("--solve-ctas", type=int, default=-1,
                    help="CTAs per triangular-solve launch (0: as many as fit; -1: autotuned for the concurrency)")
    ap.add_argument("--concurrent", type=int, default=os.cpu_count() or 1,
                    help="independent requests in flight per step (default: host threads, as the reference arm)")
    ap.add_argument("--serve-rates", default="50,100,200,0",
                    help="serving: Poisson arrival rates in requests/s (0: all requests at once)")
    ap.add_argument("--serve-requests", type=int, default=400)
    ap.add_argument("--serve-in-flight", type=int, default=8)
    ap.add_argument("--serve-prep-threads", type=int, default=4,
                    help="serving: preparation threads (measured best at saturation: 4 of 2/4/6/8)")
    ap.add_argument("--serve-max-batch", type=int, default=64)
    ap.add_argument("--serve-check", type=int, default=40, help="serving: results checked against the oracle")
    ap.add_argument("--serve-fp64-requests", type=int, default=100)
    ap.add_argument("--serve-solve-ctas", type=int, default=0, help="serving: CTAs per solve launch (0: auto)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.iterations is None:
        args.iterations = {"icosphere_l4": 10, "noisy_sphere": 50, "pose_batch": 20}.get(args.workload, 30)

    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_replicas(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "pose_batch":
        return run_batch(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "mesh_batch":
        return run_mesh_batch(args)
    # concurrent requests, one stream each: every stream gets its own hardware
    # queue (with CUDA's default of 8, 16 streams share queues and wait on each
    # other); read when the process's CUDA context is created, which happens
    # after this point. The serving stream keeps the default (slower with 32).
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    return run_requests(args)


def run_requests(args):
    """N concurrent single-request dirty deforms per step (the default
    workload): one host thread per request, as the reference arm runs one
    request per host thread."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    import arap_gpu as G
    import arap_workloads as W

    w = workload(args)
    N = max(1, args.concurrent)
    mixed = args.precision == "mixed"
    tuned = None
    # the persistent schedule is the faster one on every measured mesh, alone
    # and concurrent; the level schedule is tried only when asked for
    schedules = ("persistent",) if args.solve_schedule == "auto" else (args.solve_schedule,)
    warps = (0, 128, 256) if args.warp_rows < 0 else (args.warp_rows,)
    if args.solve_ctas < 0 and N > 1:
        import arap_tune

        tuned = {}
        pick = None
        for sch in schedules:
            for wr in warps:
                best, rates = arap_tune.tune_solve_ctas(w.positions, w.faces, w.cidx, w.ctargets, w.iterations,
                                                        args.precision, args.refine, N, device=local, schedule=sch,
                                                        warp_rows=wr, solve_blocks=args.solve_blocks)
                key = f"{sch}/warp_rows={wr}"
                tuned[key] = {"solve_ctas": best, "iterations_per_s": {str(k): round(v, 1) for k, v in rates.items()}}
                log(f"autotuned solve CTAs for {N} requests in flight, {key}: {best} {tuned[key]}")
                if pick is None or rates[best] > pick[3]:
                    pick = (sch, wr, best, rates[best])
        args.solve_schedule, args.warp_rows, args.solve_ctas = pick[0], pick[1], pick[2]
    else:
        if args.solve_ctas < 0:
            args.solve_ctas = 0
        if args.solve_schedule == "auto":
            args.solve_schedule = "persistent"
        if args.warp_rows < 0:
            args.warp_rows = 0
    ctxs = []
    for _ in range(N):
        c = G.ArapContext(w.V, w.faces, device=local)
        c.set_precision(args.precision, args.refine)
        if mixed:
            c.set_factor_precision(args.factor_bits)
        c.set_solve_ctas(args.solve_ctas)
        c.set_solve_schedule(args.solve_schedule)
        c.set_warp_rows(args.warp_rows)
        c.set_solve_blocks(args.solve_blocks)
        c.set_rest_positions(w.positions)
        c.set_constraints(w.cidx, w.ctargets)
        ctxs.append(c)
    first = ctxs[0].deform(w.iterations)  # allocation and graph capture, untimed
    vtuned = None
    if args.vertex_launch == "auto" and mixed:
        import arap_tune

        res = arap_tune.tune_vertex_launch(ctxs[0], w.iterations)
        vtuned = {k: {"threads_per_vertex": sh[0], "block": sh[1], "us_per_launch": t} for k, (sh, t) in res.items()}
        log(f"autotuned vertex kernels: {vtuned}")
        for c in ctxs[1:]:
            for k, (sh, _) in res.items():
                c.set_vertex_launch(k, *sh)
    for c in ctxs[1:]:
        c.deform(w.iterations, want_output=False)
    streams = [torch.cuda.ExternalStream(c.stream(), device=dev) for c in ctxs]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    pool = ThreadPoolExecutor(max_workers=N)

    def set_analysis(cached: bool):
        for c in ctxs:
            c.set_symbolic_cache(cached)

    def device_step():
        """One step with inputs resident on the device: every request is a
        dirty deform started by its own host thread. Device time = from a
        start event recorded on the first request's stream before the threads
        are dispatched (the device is idle then) to the last request's end
        event, recorded on its stream after its enqueue: the union of the
        requests' spans, host analysis and enqueue gaps included."""
        flush.zero_()
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        start.record(streams[0])
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(N)]

        def one(i):
            c = ctxs[i]
            c.invalidate()
            rc = c.lib.arap_deform_async(c.h, w.iterations, None)
            ends[i].record(streams[i])
            if rc != G.ARAP_OK:
                raise G.ArapError(rc, c.lib.arap_last_error(c.h).decode())
            c.wait()
            return c.launch_count()

        launches = sum(pool.map(one, range(N)))
        torch.cuda.synchronize()
        return max(start.elapsed_time(e) for e in ends), launches

    # ---- end to end through the C ABI with pinned host buffers: rest pose,
    # constraint indices and targets in, deformed positions out, per request
    # on its own host thread; wall clock around the whole step ----
    rest_h = torch.from_numpy(np.ascontiguousarray(w.positions)).pin_memory().numpy()
    idx_h = torch.from_numpy(np.ascontiguousarray(w.cidx, dtype=np.int32)).pin_memory().numpy()
    tgt_h = torch.from_numpy(np.ascontiguousarray(w.ctargets)).pin_memory().numpy()
    outs_h = [torch.empty((w.V, 3), dtype=torch.float64).pin_memory().numpy() for _ in ctxs]

    def e2e_one(i):
        c = ctxs[i]
        c.set_rest_positions(rest_h)
        c.set_constraints(idx_h, tgt_h)
        c.deform_async(w.iterations, outs_h[i])
        c.wait()

    def e2e_step():
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        list(pool.map(e2e_one, range(N)))
        return time.perf_counter() - t0

    # ---- timed region: dirty deforms with inputs resident on the device.
    # Each one is preceded by one end-to-end step (not counted in `value`), so
    # both measures see the same conditions over the run ----
    set_analysis(args.cached_analysis)
    for _ in range(args.warmup):
        device_step()
        if not args.skip_e2e:
            e2e_step()
    clocks = ClockSampler(local)
    launches = 0
    step_ms = []
    e2e_s = []
    barrier()
    clocks.start()
    for k in range(args.steps):
        if not args.skip_e2e:
            e2e_s.append(e2e_step())
        ms, nl = device_step()
        step_ms.append(ms)
        launches += nl
    barrier()
    clk = clocks.stop()
    total_ms = reduce_max(sum(step_ms), dist, dev)
    its_total = N * w.iterations * args.steps * world
    value = its_total / (total_ms / 1e3)
    # ---- the same step with the symbolic analysis kept (re-pose + refactor) ----
    repose = None
    if not args.cached_analysis:
        set_analysis(True)
        for _ in range(args.warmup):
            device_step()
        rms = [device_step()[0] for _ in range(args.steps)]
        repose = {"value": N * w.iterations * args.steps / (sum(rms) / 1e3), "unit": UNIT,
                  "ms_per_step": sum(rms) / len(rms),
                  "step": "the same dirty deforms with the symbolic analysis of the unchanged constraint set kept: "
                          "weights, numeric factorisation and iterations only"}
        set_analysis(args.cached_analysis)
    # per-request latency of a single request alone (p50/p99 over the steps),
    # with the launch shape a lone request prefers, with and without the
    # symbolic analysis
    c0 = ctxs[0]
    if args.solve_ctas != 0 or args.warp_rows != 0:
        c0.set_solve_ctas(0)
        c0.set_warp_rows(0)
        c0.deform(w.iterations, want_output=False)
    lat_alone = {}
    for cached in ((True,) if args.cached_analysis else (False, True)):
        c0.set_symbolic_cache(cached)
        c0.deform(w.iterations, want_output=False)
        lat = []
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(streams[0])
            c0.invalidate()
            c0.deform(w.iterations, want_output=False)
            e1.record(streams[0])
            torch.cuda.synchronize()
            lat.append(e0.elapsed_time(e1))
        lat.sort()
        key = "cached_analysis" if cached else "with_analysis"
        lat_alone[key] = {"p50": lat[len(lat) // 2], "p99": float(np.percentile(lat, 99)),
                          "host_ms_last": c0.host_timing()}
    # ---- per-kernel device time of one request, every launch bracketed by
    # CUDA events on its stream (a separate pass: the events do not inflate
    # the timed region above) ----
    c0.set_symbolic_cache(True)
    c0.set_profiling(True)
    c0.reset_kernel_stats()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        c0.invalidate()
        c0.deform(w.iterations, want_output=False)
    kstats = c0.kernel_stats()
    kmodel = c0.kernel_model()
    c0.set_profiling(False)
    setup_ms, iter_ms = c0.timing()
    if args.solve_ctas != 0 or args.warp_rows != 0:
        c0.set_solve_ctas(args.solve_ctas)
        c0.set_warp_rows(args.warp_rows)
    c0.set_symbolic_cache(args.cached_analysis)

    pool.shutdown()
    e2e_total = reduce_max(sum(e2e_s), dist, dev) if e2e_s else float("nan")
    e2e_value = its_total / e2e_total if e2e_s else None
    h2d = N * (w.positions.nbytes + idx_h.nbytes + tgt_h.nbytes)
    d2h = N * outs_h[0].nbytes

    # ---- roofline of the dominant kernel class ----
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    roof, froof = roofline_of(kstats, kmodel, args.steps, peaks, w.name, args.steps)

    # ---- CPU baseline (oracle, one core) + error of the GPU result ----
    cpu = None
    err = None
    if rank == 0 and not args.no_cpu_baseline:
        dt, ref = cpu_oracle_requests(w, args.cpu_requests, 1)
        from oracle import oracle as O

        t0 = time.perf_counter()
        O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, 0)  # set-up alone: weights + factor
        setup_s = time.perf_counter() - t0
        per_req = dt / args.cpu_requests
        cpu = {"value": args.cpu_requests * w.iterations / dt, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{args.cpu_requests} dirty deform({w.iterations}) requests of {w.name} on one thread "
                         f"({dt:.1f} s)",
               "setup_ms": 1e3 * setup_s, "ms_per_iteration": 1e3 * max(per_req - setup_s, 0.0) / w.iterations}
        err_first = W.bbox_rel_error(first, ref, w.positions)
        err = max([W.bbox_rel_error(o, ref, w.positions) for o in outs_h] if e2e_s else [err_first])
        log(f"error vs FP64 oracle: {err:.3e} (first deform {err_first:.3e})")

    analysis = "kept for the unchanged constraint set" if args.cached_analysis else \
        "redone on every request (ordering, elimination tree, supernodes, plan), as SimplicialLDLT::compute"
    extra = {"requests_per_step": N, "solve_blocks": args.solve_blocks,
             "vertex_launch": vtuned or "1 thread per vertex, 256-thread blocks",
             "solve_schedule": args.solve_schedule, "warp_rows": args.warp_rows,
             "solve_ctas": args.solve_ctas,
             "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
             "solve_ctas_autotune": tuned,
             "symbolic_analysis": analysis,
             "step": f"{N} concurrent dirty deform requests, one host thread each (symbolic analysis "
                     f"{'kept' if args.cached_analysis else 'redone'}, weights, numeric factorisation, "
                     f"{w.iterations} iterations)",
             "timing": "CUDA events: a start event on the idle device before the requests' threads are "
                       "dispatched, an end event on each request's stream after its enqueue; the step is the "
                       "latest end"}
    if mixed:
        extra.update({"factor": f"fp{args.factor_bits}",
                      "fp64_residual_solves_per_iteration": 1 + args.refine})
    else:
        extra.update({"factor": "fp64"})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if mixed else "f64", "data": "synthetic",
        "config": config_of(w, args, extra),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "timing": "host wall clock around each step (uploads, enqueues, waits, result copies); one "
                          "end-to-end step before each timed device step"},
        "repose_refactor": repose,
        "gpu_launches": int(launches),
        "roofline": roof,
        "factor_roofline": froof,
        "cpu_baseline": cpu,
        "error_vs_fp64_oracle": err,
        "latency_ms": {"request_alone": lat_alone, "step_p50": sorted(step_ms)[len(step_ms) // 2],
                       "steps": [round(x, 3) for x in step_ms],
                       "e2e_steps": [round(1e3 * x, 3) for x in e2e_s]},
        "kernel_ms_per_request": {k: v[0] / args.steps for k, v in kstats.items()},
        "last_request_ms": {"setup": setup_ms, "iterations": iter_ms},
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    for c in ctxs:
        c.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
