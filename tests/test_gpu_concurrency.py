"""Several requests in flight at once (arap_deform_async on several contexts,
then arap_wait) give the same positions as the same requests one after the
other, and CUDA-graph replay gives the same positions as direct launches."""
import numpy as np
import pytest

import arap_workloads as W

pytestmark = pytest.mark.gpu


def make(gpu, w, precision):
    ctx = gpu.ArapContext(w.V, w.faces)
    ctx.set_precision(precision, 1)
    ctx.set_rest_positions(w.positions)
    ctx.set_constraints(w.cidx, w.ctargets)
    return ctx


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_requests_in_flight_match_sequential(gpu, precision):
    works = [W.cfg_icosphere_l4(level=3, iterations=6), W.cfg_twisted_bar(h=0.1, iterations=6),
             W.cfg_noisy_sphere(level=3, iterations=6), W.cfg_icosphere_l4(level=4, iterations=6)]
    seq = []
    for w in works:
        with make(gpu, w, precision) as ctx:
            seq.append(ctx.deform(w.iterations))
    ctxs = [make(gpu, w, precision) for w in works]
    outs = [np.empty((w.V, 3)) for w in works]
    for c, w, o in zip(ctxs, works, outs):
        c.deform_async(w.iterations, o)
    for c in ctxs:
        c.wait()
    for a, b in zip(seq, outs):
        np.testing.assert_array_equal(a, b)
    for c in ctxs:
        c.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_direct_launches(gpu, precision):
    w = W.cfg_twisted_bar(h=0.1, iterations=5)
    with make(gpu, w, precision) as ctx:
        ctx.set_graphs(False)
        direct = ctx.deform(5)
    with make(gpu, w, precision) as ctx:
        first = ctx.deform(5)          # captures the graphs
        ctx.invalidate()
        replay = ctx.deform(5)         # replays them
    np.testing.assert_array_equal(direct, first)
    np.testing.assert_array_equal(direct, replay)
