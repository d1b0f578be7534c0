"""The benchmark configurations at full size against the FP64 oracle.

Each workload that bench.py times is checked here with the settings bench.py
uses, so the timed numbers rest on a tested result:

* twisted bar, 0.025 spacing (67,202 vertices), 30 iterations, mixed form:
  FP64 numeric factor with two FP64-residual solves per iteration (the bench
  default), and the FP32-factor option, each <= 1e-6 of the bbox diagonal;
* noisy icosphere L7 (163,842 vertices), 16 handle caps and an anchor cap,
  50 iterations, mixed form with the FP64 factor: <= 1e-6;
* icosphere L5 x 256 poses, 20 iterations, one factor for all poses, the
  dense top's column cap and the pose tile autotuned as bench.py does: every
  pose against the oracle, <= 1e-6, except at most two ill-conditioned poses
  whose own FP64 result moves by more than 1e-6 under a 1e-7 relative change
  of the input, which must stay within that sensitivity (the hardest poses
  also stretch one-rings close to rank one in the first iterations, which
  the FP32 rotation fit handles without squaring the covariance and refits
  in FP64 where it is close to rank one); 99% of the poses <= 1e-7;
* icosphere L4, FP64 form, 10 iterations: <= 1e-10.

A dirty deform that redoes the symbolic analysis on every call (the
reference's SimplicialLDLT::compute, inc/deform/arap.h:337) must give the same
positions, bit for bit, as one that keeps it.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def oracle_many(w, targets_list, iterations):
    """The oracle's dirty deforms for several target sets, on host threads."""
    def one(t):
        ok, ref = O.run_deform(w.positions, w.faces, w.cidx, t, iterations)
        assert ok
        return ref

    with ThreadPoolExecutor(max_workers=16) as ex:
        return list(ex.map(one, targets_list))


def mixed_deform(gpu, w, factor_bits=64, refine=1, cached=True):
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", refine)
        ctx.set_factor_precision(factor_bits)
        ctx.set_symbolic_cache(cached)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        out = ctx.deform(w.iterations)
        # a second dirty deform (analysis redone when not cached) repeats the first
        ctx.invalidate()
        again = ctx.deform(w.iterations)
    np.testing.assert_array_equal(out, again)
    return out


@pytest.fixture(scope="module")
def bar():
    w = W.cfg_twisted_bar(h=0.025, iterations=30)
    assert w.V == 67202
    ref = oracle_many(w, [w.ctargets], w.iterations)[0]
    return w, ref


def test_twisted_bar_fp64_factor_matches_oracle(gpu, bar):
    w, ref = bar
    out = mixed_deform(gpu, w, factor_bits=64, refine=1, cached=False)
    err = W.bbox_rel_error(out, ref, w.positions)
    assert err <= 1e-6, err
    np.testing.assert_array_equal(out[w.cidx], w.ctargets)
    cached = mixed_deform(gpu, w, factor_bits=64, refine=1, cached=True)
    np.testing.assert_array_equal(out, cached)


def test_twisted_bar_fp32_factor_matches_oracle(gpu, bar):
    w, ref = bar
    out = mixed_deform(gpu, w, factor_bits=32, refine=1)
    assert W.bbox_rel_error(out, ref, w.positions) <= 1e-6


def test_noisy_sphere_l7_matches_oracle(gpu):
    w = W.cfg_noisy_sphere(level=7, iterations=50)
    assert w.V == 163842
    ref = oracle_many(w, [w.ctargets], w.iterations)[0]
    out = mixed_deform(gpu, w, factor_bits=64, refine=1)
    err = W.bbox_rel_error(out, ref, w.positions)
    assert err <= 1e-6, err


def test_pose_batch_l5x256_autotuned_matches_oracle(gpu):
    import arap_tune

    w = W.cfg_pose_batch(level=5, n_poses=256, iterations=20)
    P = w.poses.shape[0]
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        ctx.deform_poses(w.poses, w.iterations)
        arap_tune.tune_dense_top(ctx, w.iterations, batched=True, trials=1)
        arap_tune.tune_pose_tile(ctx, w.iterations, trials=1)
        ctx.invalidate()
        out = ctx.deform_poses(None, w.iterations)
    refs = oracle_many(w, list(w.poses), w.iterations)
    errs = np.array([W.bbox_rel_error(out[p], refs[p], w.positions) for p in range(P)])
    # The FP32 local step perturbs every iteration at the FP32 rounding level.
    # A pose whose FP64 trajectory itself moves by more than 1e-6 when its
    # input moves by 1e-7 (relative; FP32's rounding is 6e-8) cannot be held to
    # 1e-6 by an FP32 computation: there the bound is that sensitivity.
    hard = [p for p in range(P) if errs[p] > 1e-6]
    assert len(hard) <= 2, hard
    if hard:
        scaled = oracle_many(W.Workload(w.name, w.positions * (1 + 1e-7), w.faces, w.cidx, w.ctargets,
                                        w.iterations, w.precision), [w.poses[p] for p in hard], w.iterations)
        for p, r in zip(hard, scaled):
            sensitivity = W.bbox_rel_error(r, refs[p], w.positions)
            assert sensitivity > 1e-6 and errs[p] <= sensitivity, (p, errs[p], sensitivity)
    assert np.percentile(errs, 99) <= 1e-7, np.percentile(errs, 99)
    for p in range(P):
        np.testing.assert_array_equal(out[p][w.cidx], w.poses[p])


def test_icosphere_l4_fp64_matches_oracle(gpu):
    w = W.cfg_icosphere_l4(level=4, iterations=10)
    ref = oracle_many(w, [w.ctargets], w.iterations)[0]
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("fp64", 0)
        ctx.set_symbolic_cache(False)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        out = ctx.deform(w.iterations)
    assert W.bbox_rel_error(out, ref, w.positions) <= 1e-10
