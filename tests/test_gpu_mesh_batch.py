"""Meshes of uneven sizes deformed in one set of launches (MeshBatch): the
disjoint union as one block-diagonal problem, every kernel launch covering
all meshes. Each mesh must get what it gets alone (the reference's
per-object loop, inc/deform/arap.h:101-138): against the oracle per mesh, and
against a context of its own."""
import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _meshes():
    return [W.cfg_twisted_bar(h=0.05, iterations=8), W.cfg_icosphere_l4(level=4, iterations=8),
            W.cfg_noisy_sphere(level=5, iterations=8), W.cfg_twisted_bar(h=0.1, iterations=8),
            W.cfg_icosphere_l4(level=3, iterations=8)]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_mesh_batch_matches_each_mesh_alone(gpu, precision, tol):
    ws = _meshes()
    with gpu.MeshBatch([(w.V, w.faces) for w in ws]) as mb:
        mb.ctx.set_precision(precision, 1)
        mb.set_rest_positions([w.positions for w in ws])
        mb.set_constraints([w.cidx for w in ws], [w.ctargets for w in ws])
        outs = mb.deform(8)
        mb.ctx.invalidate()
        np.testing.assert_array_equal(np.concatenate(mb.deform(8)), np.concatenate(outs))
    for w, got in zip(ws, outs):
        ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, 8)
        assert ok
        assert W.bbox_rel_error(got, ref, w.positions) <= tol
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision(precision, 1)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.ctargets)
            alone = ctx.deform(8)
        assert W.bbox_rel_error(got, alone, w.positions) <= (1e-11 if precision == "fp64" else 1e-6)


def test_mesh_batch_repose(gpu):
    """New targets for the same constrained sets (no refactorisation) in the
    batch give what each mesh gets from a fresh deform with those targets."""
    ws = _meshes()
    rng = np.random.default_rng(7)
    with gpu.MeshBatch([(w.V, w.faces) for w in ws]) as mb:
        mb.ctx.set_precision("mixed", 1)
        mb.set_rest_positions([w.positions for w in ws])
        mb.set_constraints([w.cidx for w in ws], [w.ctargets for w in ws])
        mb.deform(8)
        moved = [w.ctargets + rng.uniform(-0.05, 0.05, size=(1, 3)) for w in ws]
        mb.set_targets(moved)
        outs = mb.deform(8)
    for w, t, got in zip(ws, moved, outs):
        # a re-pose starts from the rest pose with the constrained vertices at
        # the new targets, as a dirty deform after setConstraint does
        ok, ref = O.run_deform(w.positions, w.faces, w.cidx, t, 8)
        assert ok
        assert W.bbox_rel_error(got, ref, w.positions) <= 1e-6
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision("mixed", 1)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.ctargets)
            ctx.deform(8)
            ctx.set_targets(t)
            alone = ctx.deform(8)
        assert W.bbox_rel_error(got, alone, w.positions) <= 1e-6
