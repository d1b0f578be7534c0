"""Many poses of one mesh in one pass (arap_deform_poses) against the FP64
oracle run pose by pose: each pose is a dirty deform from the rest pose with
the handles at that pose's targets (inc/deform/deformation_util.h:48-57
followed by deform, inc/deform/arap.h:101-138)."""
import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("level,n_poses,iters", [(3, 5, 6), (4, 19, 10)])
def test_pose_batch_matches_oracle(gpu, level, n_poses, iters):
    w = W.cfg_pose_batch(level=level, n_poses=n_poses, iterations=iters)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        out = ctx.deform_poses(w.poses, iters)
    assert out.shape == (n_poses, w.V, 3)
    for p in range(n_poses):
        ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.poses[p], iters)
        assert ok
        err = W.bbox_rel_error(out[p], ref, w.positions)
        assert err <= 1e-6, (p, err)
        np.testing.assert_array_equal(out[p][w.cidx], w.poses[p])


def test_pose_batch_equals_single_requests(gpu):
    """The same poses one at a time through arap_deform agree with the batch
    to the mixed tolerance, and a second batch call with the targets left on
    the device repeats the first."""
    w = W.cfg_pose_batch(level=3, n_poses=4, iterations=5)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        batch = ctx.deform_poses(w.poses, 5)
        again = np.empty_like(batch)
        assert ctx.deform_poses_rc(None, 5, again) == gpu.ARAP_OK
        np.testing.assert_array_equal(batch, again)
        for p in range(4):
            ctx.set_constraints(w.cidx, w.poses[p])
            single = ctx.deform(5)
            assert W.bbox_rel_error(single, batch[p], w.positions) <= 1e-6


def test_pose_batch_rejects_fp64(gpu):
    w = W.cfg_pose_batch(level=2, n_poses=2, iterations=2)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("fp64")
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        with pytest.raises(gpu.ArapError) as e:
            ctx.deform_poses(w.poses, 2)
        assert e.value.code == gpu.ARAP_ERR_UNSUPPORTED


def test_pose_targets_on_device_match_host_targets(gpu):
    """arap_pose_targets (DeformationUtil::updateConstraints for many rigid
    poses, inc/deform/deformation_util.h:48-57) gives the targets the host
    computes, and the poses deformed from them."""
    w = W.cfg_pose_batch(level=3, n_poses=12, iterations=5)
    ctx = gpu.ArapContext(w.V, w.faces)
    ctx.set_precision("mixed", 1)
    ctx.set_rest_positions(w.positions)
    ctx.set_constraints(w.cidx, w.poses[0] * 0 + w.positions[w.cidx])
    host = ctx.deform_poses(w.poses, w.iterations)
    ctx.pose_targets(w.info["handle_ids"], w.info["transforms"], w.info["origin"])
    dev = ctx.deform_poses(None, w.iterations)
    ctx.close()
    for p in range(len(w.poses)):
        assert W.bbox_rel_error(dev[p], host[p], w.positions) <= 1e-12


def test_pose_targets_rejects_unconstrained_handle(gpu):
    w = W.cfg_pose_batch(level=2, n_poses=2, iterations=2)
    free = np.setdiff1d(np.arange(w.V), w.cidx)[0]
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        with pytest.raises(gpu.ArapError) as e:
            ctx.pose_targets([int(free)], w.info["transforms"], w.info["origin"])
        assert e.value.code == gpu.ARAP_ERR_BAD_INDEX


def test_pose_tile_and_launch_shape_give_identical_results(gpu):
    """Each (supernode, pose tile) task sums its columns in the same order
    whatever the tile or the number of persistent CTAs, so every launch shape
    gives bit-identical poses; repeated calls (graph capture on the second
    call, replay on the third) and graphs switched off repeat them too. 19
    poses leave a ragged last tile for every tile size; 7 iterations run
    through the 4-, 2- and 1-iteration graphs."""
    w = W.cfg_pose_batch(level=4, n_poses=19, iterations=7)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_dense_top(2048)  # the default is wider for an uncapped grid
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        ref = ctx.deform_poses(w.poses, 7)
        for _ in range(2):
            np.testing.assert_array_equal(ctx.deform_poses(None, 7), ref)
        for pt in (1, 2, 4, 8, 16):
            ctx.set_pose_tile(pt)
            for _ in range(3):
                np.testing.assert_array_equal(ctx.deform_poses(None, 7), ref, err_msg=f"pose tile {pt}")
        ctx.set_pose_tile(0)
        for ctas in (1, 5, 0):
            ctx.set_solve_ctas(ctas)
            for _ in range(3):
                np.testing.assert_array_equal(ctx.deform_poses(w.poses, 7), ref, err_msg=f"{ctas} CTAs")
        ctx.set_graphs(False)
        np.testing.assert_array_equal(ctx.deform_poses(None, 7), ref)
        with pytest.raises(gpu.ArapError) as e:
            ctx.set_pose_tile(3)
        assert e.value.code == gpu.ARAP_ERR_INVALID_ARGUMENT


def test_pose_batch_pose_count_change_resets_schedule(gpu):
    """Changing the pose count between calls (new tiles, new grid, new
    scheduling counters) keeps every call exact against the per-pose batch."""
    w = W.cfg_pose_batch(level=3, n_poses=9, iterations=4)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        full = ctx.deform_poses(w.poses, 4)
        for n in (1, 5, 9, 3, 9):
            for _ in range(2):
                np.testing.assert_array_equal(ctx.deform_poses(w.poses[:n], 4), full[:n])
        # the device holds targets for 9 poses, not for 5
        assert ctx.lib.arap_deform_poses(ctx.h, 5, None, 4, None) == gpu.ARAP_ERR_INVALID_ARGUMENT


def test_pose_tile_that_does_not_fit_is_refused(gpu):
    """The twisted bar's largest front has 544 rows: 136 quads x 16 poses is
    more than the 1,024 items a batched-solve CTA holds, so tile 16 is refused
    (ARAP_ERR_UNSUPPORTED) and the automatic choice still runs."""
    w = W.cfg_twisted_bar(iterations=2)
    poses = np.stack([w.ctargets, w.ctargets + 0.01])
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        ctx.set_pose_tile(16)
        with pytest.raises(gpu.ArapError) as e:
            ctx.deform_poses(poses, 2)
        assert e.value.code == gpu.ARAP_ERR_UNSUPPORTED
        ctx.set_pose_tile(0)
        out = ctx.deform_poses(poses, 2)
        assert np.isfinite(out).all()


@pytest.mark.parametrize("cols", [256, 0, 4096])
def test_pose_batch_dense_top_matches_supernodal_top(gpu, cols):
    """The batched sweeps with the tree's top levels through T = inv(L_top)
    (a matrix product over all poses) agree with the sweeps over the whole
    tree to the mixed tolerance and with the oracle pose by pose, for caps
    from a few levels up to most of this mesh's tree."""
    w = W.cfg_pose_batch(level=4, n_poses=7, iterations=6)

    def run(c):
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision("mixed", 1)
            ctx.set_dense_top(c)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.poses[0])
            out = ctx.deform_poses(w.poses, 6)
            again = ctx.deform_poses(None, 6)
            np.testing.assert_array_equal(out, again)
            return out

    ref, got = run(-1), run(cols)
    for p in range(len(w.poses)):
        assert W.bbox_rel_error(got[p], ref[p], w.positions) <= 1e-6, p
        ok, o = O.run_deform(w.positions, w.faces, w.cidx, w.poses[p], 6)
        assert ok and W.bbox_rel_error(got[p], o, w.positions) <= 1e-6, p
        np.testing.assert_array_equal(got[p][w.cidx], w.poses[p])


def test_pose_batch_dense_top_several_column_tiles(gpu):
    """90 poses pack into 270 right-hand-side columns: two 256-column tiles of
    the tensor-core products, the second ragged. Every pose agrees with the
    sweeps over the whole tree; every ninth with the oracle."""
    w = W.cfg_pose_batch(level=4, n_poses=90, iterations=4)

    def run(c):
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision("mixed", 1)
            ctx.set_dense_top(c)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.poses[0])
            return ctx.deform_poses(w.poses, 4)

    ref, got = run(-1), run(0)
    for p in range(len(w.poses)):
        assert W.bbox_rel_error(got[p], ref[p], w.positions) <= 1e-6, p
        np.testing.assert_array_equal(got[p][w.cidx], w.poses[p])
    for p in range(0, len(w.poses), 9):
        ok, o = O.run_deform(w.positions, w.faces, w.cidx, w.poses[p], 4)
        assert ok and W.bbox_rel_error(got[p], o, w.positions) <= 1e-6, p


def test_dense_top_autotune(gpu):
    """arap_tune.tune_dense_top times every candidate cap on full dirty calls,
    leaves the fastest set, and the results stay within the mixed tolerance
    of the default cap (batched) and of the oracle (one request)."""
    import arap_tune

    w = W.cfg_pose_batch(level=4, n_poses=6, iterations=3)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[0])
        ref = ctx.deform_poses(w.poses, 3)
        best, times = arap_tune.tune_dense_top(ctx, 3, batched=True, candidates=(-1, 256, 2048), trials=1)
        assert set(times) == {-1, 256, 2048} and best in times
        assert all(t > 0 for t in times.values())
        got = ctx.deform_poses(None, 3)
        for p in range(len(w.poses)):
            assert W.bbox_rel_error(got[p], ref[p], w.positions) <= 1e-6, p
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.poses[1])
        best, times = arap_tune.tune_dense_top(ctx, 3, batched=False, candidates=(-1, 512), trials=1)
        assert set(times) == {-1, 512} and best in times
        ctx.invalidate()  # a dirty deform from the rest pose, as the oracle runs
        out = ctx.deform(3)
    ok, o = O.run_deform(w.positions, w.faces, w.cidx, w.poses[1], 3)
    assert ok and W.bbox_rel_error(out, o, w.positions) <= 1e-6


def test_batched_sweeps_with_solve_blocks(gpu):
    """The batched sweeps over the solve blocks (the default) and over the
    supernodes alone give the same poses up to the order of sums."""
    w = W.cfg_pose_batch(level=4, n_poses=24, iterations=6)
    outs = []
    for blocks in (512, 0):
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision("mixed", 1)
            ctx.set_solve_blocks(blocks)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.poses[0])
            outs.append(ctx.deform_poses(w.poses, w.iterations))
    for p in range(len(w.poses)):
        assert W.bbox_rel_error(outs[0][p], outs[1][p], w.positions) <= 1e-6
