"""arap_cotan_weights_static: cotan weights for callers that cannot allocate
device memory (a viewer's per-frame callback that must not stall on
cudaMalloc, or a host that owns all device memory through its own pool).

The entry point keeps its scratch in a static device array and writes into
buffers the caller owns. The tests own those buffers (allocated with torch
here, as such a caller would have them from its pool) and call the entry point
through the C ABI twice in a row. Each result is compared with the weights the
context path (arap_deform + arap_get_edge_weights) computes and with the FP64
oracle's weights: bit for bit, the tolerance the other weight tests use. The
second call must leave the device's free memory unchanged. A face with an
out-of-range index is skipped by the kernels' own bounds checks, counted, and
reported by arap_cotan_weights_static_status. The file runs alone or after the
rest of the suite; it is named to be collected last.
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


def oracle_weights(w):
    from oracle import oracle

    o = oracle.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    o.deform(0)
    rp, col, val = o.weights_csr()
    o.close()
    return rp, col, val


def dev(t):
    return C.c_void_p(t.data_ptr())


def status(gpu, lib, stream):
    n = C.c_int32(-1)
    rc = lib.arap_cotan_weights_static_status(C.c_void_p(stream.cuda_stream), C.byref(n))
    return rc, n.value


def device_inputs(w, rp, col, cuda, faces=None):
    import torch

    f = np.ascontiguousarray(w.faces if faces is None else faces, np.int32).ravel()
    return (torch.from_numpy(f).to(cuda),
            torch.from_numpy(np.ascontiguousarray(w.positions, np.float64).ravel()).to(cuda),
            torch.from_numpy(rp).to(cuda), torch.from_numpy(col).to(cuda))


def test_static_scratch_weights_match_context_path(gpu):
    import torch

    lib = gpu.load()
    cuda = torch.device("cuda", 0)
    torch.cuda.set_device(cuda)
    stream = torch.cuda.current_stream(cuda)
    cases = [W.cfg_noisy_sphere(level=5), W.cfg_twisted_bar(h=0.05)]
    expected = [context_weights(gpu, w) for w in cases]
    for w, (rp, col, val) in zip(cases, expected):
        orp, ocol, oval = oracle_weights(w)
        np.testing.assert_array_equal(rp, orp)
        np.testing.assert_array_equal(col, ocol)
        np.testing.assert_array_equal(val, oval)
    # two calls in a row per mesh, meshes alternating, so a call never sees a
    # clean scratch array
    order = [0, 1, 0, 0]
    inputs = [device_inputs(w, rp, col, cuda) for w, (rp, col, _) in zip(cases, expected)]
    outs = [torch.full((len(expected[i][2]),), float("nan"), dtype=torch.float64, device=cuda) for i in order]
    torch.cuda.synchronize()
    for call, i in enumerate(order):
        w, (rp, col, val) = cases[i], expected[i]
        faces, xyz, rowptr, colv = inputs[i]
        out = outs[call]
        free_before = torch.cuda.mem_get_info(cuda)[0]
        rc = lib.arap_cotan_weights_static(w.V, w.F, dev(faces), dev(xyz), dev(rowptr), dev(colv), len(val),
                                           dev(out), C.c_void_p(stream.cuda_stream))
        assert rc == gpu.ARAP_OK, lib.arap_last_error(None)
        assert status(gpu, lib, stream) == (gpu.ARAP_OK, 0)
        stream.synchronize()
        free_after = torch.cuda.mem_get_info(cuda)[0]
        if call > 0:  # the first call may load the library's device code (a one-time driver allocation)
            assert free_after == free_before, (call, free_before, free_after)
        np.testing.assert_array_equal(out.cpu().numpy(), val)


@pytest.mark.parametrize("bad", ["past_end", "negative"])
def test_static_scratch_skips_out_of_range_faces(gpu, bad):
    import torch

    lib = gpu.load()
    cuda = torch.device("cuda", 0)
    torch.cuda.set_device(cuda)
    stream = torch.cuda.current_stream(cuda)
    w = W.cfg_icosphere_l4(level=3)
    rp, col, val = context_weights(gpu, w)
    f_bad = w.F // 2
    corners = [int(v) for v in w.faces[f_bad]]
    faces_bad = np.array(w.faces, np.int32, copy=True)
    faces_bad[f_bad, 1] = w.V + 5 if bad == "past_end" else -1
    faces, xyz, rowptr, colv = device_inputs(w, rp, col, cuda, faces_bad)
    out = torch.full((len(val),), float("nan"), dtype=torch.float64, device=cuda)
    rc = lib.arap_cotan_weights_static(w.V, w.F, dev(faces), dev(xyz), dev(rowptr), dev(colv), len(val), dev(out),
                                       C.c_void_p(stream.cuda_stream))
    assert rc == gpu.ARAP_OK, lib.arap_last_error(None)
    assert status(gpu, lib, stream) == (gpu.ARAP_ERR_BAD_INDEX, 1)
    assert b"outside [0, n_vertices)" in lib.arap_last_error(None)
    got = out.cpu().numpy()
    # the skipped face's six directed edge entries lose its half; every other
    # entry is the full weight
    touched = np.zeros(len(val), bool)
    for k in range(3):
        a, b = corners[k], corners[(k + 1) % 3]
        for r, c in ((a, b), (b, a)):
            e = rp[r] + int(np.searchsorted(col[rp[r]:rp[r + 1]], c))
            assert col[e] == c
            touched[e] = True
    assert touched.sum() == 6
    np.testing.assert_array_equal(got[~touched], val[~touched])
    assert np.all(got[touched] < val[touched])
    # the next call on good input clears the count
    faces_ok = torch.from_numpy(np.ascontiguousarray(w.faces, np.int32).ravel()).to(cuda)
    rc = lib.arap_cotan_weights_static(w.V, w.F, dev(faces_ok), dev(xyz), dev(rowptr), dev(colv), len(val),
                                       dev(out), C.c_void_p(stream.cuda_stream))
    assert rc == gpu.ARAP_OK
    assert status(gpu, lib, stream) == (gpu.ARAP_OK, 0)
    np.testing.assert_array_equal(out.cpu().numpy(), val)


def test_static_scratch_rejects_oversize(gpu):
    lib = gpu.load()
    rc = lib.arap_cotan_weights_static(3 * STATIC_MAX_FACES, STATIC_MAX_FACES + 1, C.c_void_p(16),
                                       C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), 1, C.c_void_p(16), None)
    assert rc == gpu.ARAP_ERR_UNSUPPORTED
    assert b"static scratch limit" in lib.arap_last_error(None)
