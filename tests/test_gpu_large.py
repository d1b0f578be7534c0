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
