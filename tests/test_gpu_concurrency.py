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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_cta_count_does_not_change_results(gpu, precision):
    """The triangular solves give every supernode to whichever CTA takes its
    ticket; one CTA, a few, or as many as fit compute the same numbers. (The
    default dense top is wider for an uncapped grid, so it is pinned here.)"""
    w = W.cfg_twisted_bar(h=0.1, iterations=4)
    outs = []
    for n in (0, 1, 3, 64):
        with make(gpu, w, precision) as ctx:
            ctx.set_dense_top(2048)
            ctx.set_solve_ctas(n)
            a = ctx.deform(4)
            ctx.set_targets(w.ctargets + 0.05)   # re-pose: same launch shape, counters carry on
            b = ctx.deform(4)
            outs.append((a, b))
    for a, b in outs[1:]:
        np.testing.assert_array_equal(a, outs[0][0])
        np.testing.assert_array_equal(b, outs[0][1])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
@pytest.mark.parametrize("threshold", [1, 4096, 16384])
def test_cluster_levels_match_single_cta_levels(gpu, precision, tol, threshold):
    """Solving the top levels of the tree with CTA clusters (a low threshold
    puts most levels there) gives the positions of the single-CTA solves up to
    the order of the sums, and stays within the oracle tolerance."""
    from oracle import oracle as O

    w = W.cfg_twisted_bar(h=0.1, iterations=6)
    with make(gpu, w, precision) as ctx:
        ctx.set_cluster_threshold(-1)
        ref = ctx.deform(6)
    with make(gpu, w, precision) as ctx:
        ctx.set_cluster_threshold(threshold)
        got = ctx.deform(6)
        ctx.set_targets(w.ctargets + 0.02)   # a second deform on the same launch shape
        got2 = ctx.deform(6)
        ctx.set_cluster_threshold(-1)
        ref2 = ctx.deform(6)
    assert W.bbox_rel_error(got, ref, w.positions) <= tol
    assert W.bbox_rel_error(got2, ref2, w.positions) <= tol
    ok, o = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, 6)
    assert ok and W.bbox_rel_error(got, o, w.positions) <= (1e-10 if precision == "fp64" else 1e-6)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-6)])
@pytest.mark.parametrize("cols", [-1, 256, 0, 4096])
def test_dense_top_matches_supernodal_top(gpu, precision, tol, cols):
    """The top levels solved through T = inv(L_top) (any column cap, none with
    -1) give the positions of the supernodal sweeps up to the order of sums,
    and stay within the oracle tolerance; repeated deforms (graph replay) are
    bit-identical."""
    from oracle import oracle as O

    w = W.cfg_twisted_bar(h=0.1, iterations=6)
    with make(gpu, w, precision) as ctx:
        ctx.set_dense_top(-1)
        ref = ctx.deform(6)
    with make(gpu, w, precision) as ctx:
        ctx.set_dense_top(cols)
        got = ctx.deform(6)
        ctx.invalidate()
        again = ctx.deform(6)
        ctx.invalidate()
        third = ctx.deform(6)
    np.testing.assert_array_equal(got, again)
    np.testing.assert_array_equal(got, third)
    assert W.bbox_rel_error(got, ref, w.positions) <= tol
    ok, o = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, 6)
    assert ok and W.bbox_rel_error(got, o, w.positions) <= (1e-10 if precision == "fp64" else 1e-6)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-6)])
def test_warp_solves_match_cta_solves(gpu, precision, tol):
    """The bottom levels solved one warp per supernode (arap_set_warp_rows)
    against the CTA-per-supernode sweep of every level and against the
    oracle: any front limit gives the same positions up to the order of sums,
    and repeated calls repeat bit for bit."""
    from oracle import oracle as O

    w = W.cfg_twisted_bar(h=0.05, iterations=8)
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok
    outs = {}
    for rows in (0, 64, 128, 256):
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision(precision, 1)
            ctx.set_warp_rows(rows)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.ctargets)
            out = ctx.deform(w.iterations)
            ctx.invalidate()
            np.testing.assert_array_equal(ctx.deform(w.iterations), out)
        outs[rows] = out
        assert W.bbox_rel_error(out, ref, w.positions) <= (1e-10 if precision == "fp64" else 1e-6)
    for rows in (64, 128, 256):
        assert W.bbox_rel_error(outs[rows], outs[0], w.positions) <= tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("workload", ["bar", "sphere"])
def test_level_schedule_matches_persistent(gpu, precision, workload):
    """One solve launch per tree level (arap_set_solve_schedule) runs the same
    tasks with the same sums as the persistent sweep: positions bit for bit
    equal, with and without the dense top (its cap pinned: the default is
    wider for an uncapped grid), and with a capped grid."""
    from oracle import oracle as O

    w = (W.cfg_twisted_bar(h=0.05, iterations=8) if workload == "bar"
         else W.cfg_noisy_sphere(level=4, iterations=8))
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok
    for dense in (2048, -1):
        outs = []
        for schedule, cap in (("persistent", 0), ("levels", 0), ("levels", 7)):
            with gpu.ArapContext(w.V, w.faces) as ctx:
                ctx.set_precision(precision, 1)
                ctx.set_dense_top(dense)
                ctx.set_solve_schedule(schedule)
                ctx.set_solve_ctas(cap)
                ctx.set_rest_positions(w.positions)
                ctx.set_constraints(w.cidx, w.ctargets)
                out = ctx.deform(w.iterations)
                ctx.invalidate()
                np.testing.assert_array_equal(ctx.deform(w.iterations), out)
            outs.append(out)
        np.testing.assert_array_equal(outs[1], outs[0])
        np.testing.assert_array_equal(outs[2], outs[0])
        assert W.bbox_rel_error(outs[1], ref, w.positions) <= (1e-10 if precision == "fp64" else 1e-6)


def test_level_schedule_rejects_unknown(gpu):
    w = W.cfg_icosphere_l4(level=2, iterations=1)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        with pytest.raises(gpu.ArapError) as e:
            ctx.set_solve_schedule(7)
        assert e.value.code == gpu.ARAP_ERR_INVALID_ARGUMENT


def test_vertex_launch_shapes_match(gpu):
    """Every launch shape of the local step, RHS and residual (threads per
    vertex up to a warp per vertex, block sizes) gives the default's result up
    to the order of sums, and the oracle's within the mixed tolerance; the
    autotuner leaves a valid shape set."""
    import arap_tune
    from oracle import oracle as O

    w = W.cfg_twisted_bar(h=0.05, iterations=6)
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        base = ctx.deform(w.iterations)
        for name, shapes in arap_tune.VERTEX_SHAPES.items():
            for tpv, blk in shapes:
                ctx.set_vertex_launch(name, tpv, blk)
                ctx.invalidate()
                got = ctx.deform(w.iterations)
                assert W.bbox_rel_error(got, base, w.positions) <= 1e-6, (name, tpv, blk)
                assert W.bbox_rel_error(got, ref, w.positions) <= 1e-6, (name, tpv, blk)
            ctx.set_vertex_launch(name, 1, 256)
        res = arap_tune.tune_vertex_launch(ctx, w.iterations)
        assert set(res) == {"local", "rhs", "residual"}
        ctx.invalidate()
        assert W.bbox_rel_error(ctx.deform(w.iterations), ref, w.positions) <= 1e-6
        with pytest.raises(gpu.ArapError):
            ctx.set_vertex_launch("local", 3, 256)
        with pytest.raises(gpu.ArapError):
            ctx.set_vertex_launch("local", 1, 512)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-6)])
@pytest.mark.parametrize("workload", ["bar", "sphere", "l4"])
def test_solve_blocks_match_supernodal_sweeps(gpu, precision, tol, workload):
    """Level-1 subtrees solved as blocks (arap_set_solve_blocks) through the
    dense inverse of their diagonal block give the supernodal sweeps' positions
    up to the order of sums, and the oracle's within the form's tolerance; with
    and without the dense top and warp solves, repeated calls bit for bit."""
    from oracle import oracle as O

    w = {"bar": lambda: W.cfg_twisted_bar(h=0.05, iterations=8),
         "sphere": lambda: W.cfg_noisy_sphere(level=5, iterations=8),
         "l4": lambda: W.cfg_icosphere_l4(level=4, iterations=8)}[workload]()
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok
    for dense, warp in ((0, 0), (-1, 0), (0, 256)):
        outs = []
        for blocks in (0, 512):
            with gpu.ArapContext(w.V, w.faces) as ctx:
                ctx.set_precision(precision, 1)
                ctx.set_dense_top(dense)
                ctx.set_warp_rows(warp)
                ctx.set_solve_blocks(blocks)
                ctx.set_rest_positions(w.positions)
                ctx.set_constraints(w.cidx, w.ctargets)
                out = ctx.deform(w.iterations)
                ctx.invalidate()
                np.testing.assert_array_equal(ctx.deform(w.iterations), out)
            outs.append(out)
            assert W.bbox_rel_error(out, ref, w.positions) <= (1e-10 if precision == "fp64" else 1e-6)
        assert W.bbox_rel_error(outs[1], outs[0], w.positions) <= tol


def test_solve_blocks_reject_negative(gpu):
    w = W.cfg_icosphere_l4(level=2, iterations=1)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        with pytest.raises(gpu.ArapError) as e:
            ctx.set_solve_blocks(-1)
        assert e.value.code == gpu.ARAP_ERR_INVALID_ARGUMENT
