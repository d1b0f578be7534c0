"""Failure detection on the GPU without a fault: a bounded wait that runs out.

The triangular solves schedule supernode tasks over persistent CTAs; a task
waits (bounded) for its children's completion flags. arap_set_wait_limit
shrinks that bound to a few polls, so waits for children still running expire.
The kernel then records the timeout and every CTA leaves at its next task (no
trap, no fault, no copy left in flight), arap_deform returns
ARAP_ERR_TIMEOUT within milliseconds, and the next deform on the same context,
with the default limit back, is correct: bit-identical to a deform that never
timed out. The reference reports failures through deform's bool
(inc/deform/arap.h:116-117); its solves are sequential and never wait.
"""
import time

import numpy as np
import pytest

import arap_workloads as W

pytestmark = pytest.mark.gpu


def _expire(deform_rc, gpu, tries=4):
    """Runs dirty deforms until one reports the timeout; returns its seconds."""
    for _ in range(tries):
        t0 = time.perf_counter()
        rc = deform_rc()
        dt = time.perf_counter() - t0
        if rc == gpu.ARAP_ERR_TIMEOUT:
            return dt
        assert rc == gpu.ARAP_OK, rc
    pytest.fail("no wait expired with a one-poll limit")


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_wait_limit_expires_and_context_recovers(gpu, precision):
    w = W.cfg_twisted_bar(h=0.05, iterations=10)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision(precision, 1)
        ctx.set_dense_top(-1)  # every level as supernode tasks that wait for their children
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        good = ctx.deform(w.iterations)
        ctx.set_wait_limit(1)

        def dirty():
            ctx.invalidate()
            return ctx.deform_rc(w.iterations, np.empty((w.V, 3)))

        dt = _expire(dirty, gpu)
        assert dt < 2.0, dt
        assert b"wait expired" in ctx.lib.arap_last_error(ctx.h)
        ctx.set_wait_limit(0)
        again = ctx.deform(w.iterations)
        np.testing.assert_array_equal(again, good)


def test_wait_limit_expires_in_the_pose_batch(gpu):
    w = W.cfg_pose_batch(level=4, n_poses=16, iterations=6)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_dense_top(-1)  # every level as supernode tasks that wait for their children
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        good = ctx.deform_poses(w.poses, w.iterations)
        ctx.set_wait_limit(1)

        def dirty():
            ctx.invalidate()
            return ctx.deform_poses_rc(None, w.iterations, None)

        _expire(dirty, gpu)
        ctx.set_wait_limit(0)
        again = ctx.deform_poses(None, w.iterations)
        np.testing.assert_array_equal(again, good)


def test_wait_limit_rejects_negative(gpu):
    w = W.cfg_icosphere_l4(level=2, iterations=1)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        with pytest.raises(gpu.ArapError) as e:
            ctx.set_wait_limit(-1)
        assert e.value.code == gpu.ARAP_ERR_INVALID_ARGUMENT
