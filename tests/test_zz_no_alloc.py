"""arap_cotan_weights_static: cotan weights for callers that cannot allocate
device memory (a viewer's per-frame callback that must not stall on
cudaMalloc, or a host that owns all device memory through its own pool).

The entry point keeps its scratch in a static device array and writes into
buffers the caller owns. The test owns those buffers (allocated with torch
here, as such a caller would have them from its pool), calls the entry point
through the C ABI twice in a row, and compares each result with the weights
the context path (arap_deform + arap_get_edge_weights) computes: bit for bit,
the tolerance the other weight tests use. It runs alone or after the rest of
the suite; this file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import arap_workloads as W

pytestmark = pytest.mark.gpu

STATIC_MAX_FACES = 1 << 19


def context_weights(gpu, w):
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        ctx.deform(0)
        return ctx.edge_weights()


def dev(t):
    return C.c_void_p(t.data_ptr())


def test_static_scratch_weights_match_context_path(gpu):
    import torch

    lib = gpu.load()
    cuda = torch.device("cuda", 0)
    torch.cuda.set_device(cuda)
    stream = torch.cuda.current_stream(cuda)
    cases = [W.cfg_noisy_sphere(level=5), W.cfg_twisted_bar(h=0.05)]
    expected = [context_weights(gpu, w) for w in cases]
    # two calls in a row per mesh, meshes alternating, so a call never sees a
    # clean scratch array
    for w, (rp, col, val) in [(cases[0], expected[0]), (cases[1], expected[1]),
                              (cases[0], expected[0]), (cases[0], expected[0])]:
        faces = torch.from_numpy(np.ascontiguousarray(w.faces, np.int32).ravel()).to(cuda)
        xyz = torch.from_numpy(np.ascontiguousarray(w.positions, np.float64).ravel()).to(cuda)
        rowptr = torch.from_numpy(rp).to(cuda)
        colv = torch.from_numpy(col).to(cuda)
        out = torch.full((len(val),), float("nan"), dtype=torch.float64, device=cuda)
        rc = lib.arap_cotan_weights_static(w.V, w.F, dev(faces), dev(xyz), dev(rowptr), dev(colv), len(val),
                                           dev(out), C.c_void_p(stream.cuda_stream))
        assert rc == gpu.ARAP_OK, lib.arap_last_error(None)
        stream.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), val)


def test_static_scratch_rejects_oversize(gpu):
    lib = gpu.load()
    rc = lib.arap_cotan_weights_static(3 * STATIC_MAX_FACES, STATIC_MAX_FACES + 1, C.c_void_p(16),
                                       C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), 1, C.c_void_p(16), None)
    assert rc == gpu.ARAP_ERR_UNSUPPORTED
    assert b"static scratch limit" in lib.arap_last_error(None)
