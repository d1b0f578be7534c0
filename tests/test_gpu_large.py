"""Meshes whose supernode fronts exceed one solve pass (1,024 rows): the
single-CTA sweeps take such fronts in several passes, X = inv(L11) is built
without holding a column block in shared memory, and the result matches the
FP64 oracle as any other mesh does."""
import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_bar_with_fronts_beyond_one_pass_matches_oracle(gpu):
    w = W.cfg_twisted_bar(h=0.01, iterations=4)  # 420,002 vertices; fronts of more than 1,024 rows
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("mixed", 1)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        got = ctx.deform(w.iterations)
        assert max(int(np.diff(ctx.symbolic()["block_ptr"]).max()), 0) > 0
        # the plain FP64 form runs on the same fronts, within its tolerance
        ctx.set_precision("fp64", 0)
        got64 = ctx.deform(w.iterations)
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok
    assert W.bbox_rel_error(got, ref, w.positions) <= 1e-6
    assert W.bbox_rel_error(got64, ref, w.positions) <= 1e-10


def test_fp64_fronts_beyond_the_chunk_size_icosphere_l9(gpu):
    """Icosphere L9 (2,621,442 vertices) with its caps constrained: fronts of up
    to 2,822 rows below the dense top (levels 14-17 of its tree), more than a
    16 KB chunk holds as FP64 columns. Fronts of several passes stream row
    segments of each pass, so the FP64 form runs on them: a deform with every
    target at its rest position returns the rest pose (rotations are the
    identity, the solves return L^-1 L p = p), and the real deformation in FP64
    agrees with the mixed form."""
    w = W.cfg_icosphere_l4(level=9, iterations=4)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision("fp64", 0)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.positions[w.cidx])
        still = ctx.deform(2)
        assert W.bbox_rel_error(still, w.positions, w.positions) <= 1e-10  # measured 1.8e-12
        ctx.set_constraints(w.cidx, w.ctargets)
        got64 = ctx.deform(w.iterations)
        ctx.set_precision("mixed", 1)
        ctx.invalidate()
        got = ctx.deform(w.iterations)
    assert W.bbox_rel_error(got, got64, w.positions) <= 1e-6
