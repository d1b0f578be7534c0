"""The deform server (arap_srv_*): each request's result is the same alone
and in the mix; resident factors are reused; admission by device footprint
evicts cold factors; errors reach the request that caused them. Also the
re-pose entry point the server is built on (arap_set_targets)."""
import threading

import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6   # bbox-relative, mixed form vs FP64
FP64_TOL = 1e-10   # bbox-relative, FP64 form vs FP64


def small_pool():
    pool = W.serving_pool(n_meshes=6, seed=7, levels=(3, 4), v_min=600, v_max=3000)
    return pool


def lone(gpu, mesh, req, precision, ordering="mesh"):
    """The request on a fresh context, as a plain arap_deform (with the
    server's default ordering: the mesh's dissection restricted to the free
    vertices)."""
    with gpu.ArapContext(mesh.V, mesh.faces) as ctx:
        ctx.set_precision(precision, 1)
        ctx.set_ordering(ordering)
        ctx.set_rest_positions(mesh.positions)
        ctx.set_constraints(req.cidx, req.ctargets)
        return ctx.deform(req.iterations)


def err(a, b, rest):
    return W.bbox_rel_error(a, b, rest)


def test_set_targets_matches_fresh_setup(gpu):
    """Re-posing a constraint set (factor kept) equals setting it up anew."""
    w = W.cfg_pose_batch(level=3, n_poses=3, iterations=8)
    for precision, tol in (("fp64", 1e-12), ("mixed", 1e-7)):
        with gpu.ArapContext(w.V, w.faces) as ctx:
            ctx.set_precision(precision, 1)
            ctx.set_rest_positions(w.positions)
            ctx.set_constraints(w.cidx, w.poses[0])
            ctx.deform(w.iterations)
            outs = []
            for p in (1, 2):
                ctx.set_targets(w.poses[p])
                outs.append(ctx.deform(w.iterations))
        for p, got in zip((1, 2), outs):
            with gpu.ArapContext(w.V, w.faces) as fresh:
                fresh.set_precision(precision, 1)
                fresh.set_rest_positions(w.positions)
                fresh.set_constraints(w.cidx, w.poses[p])
                ref = fresh.deform(w.iterations)
            assert err(got, ref, w.positions) <= tol
            ok, o = O.run_deform(w.positions, w.faces, w.cidx, w.poses[p], w.iterations)
            assert ok
            assert err(got, o, w.positions) <= (FP64_TOL if precision == "fp64" else MIXED_TOL)


def test_set_targets_rejects_other_sizes(gpu):
    w = W.cfg_icosphere_l4(level=2, iterations=2)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        with pytest.raises(gpu.ArapError) as e:
            ctx.set_targets(w.ctargets[:-1])
        assert e.value.code == gpu.ARAP_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_results_same_alone_and_in_the_mix(gpu, precision):
    pool = small_pool()
    reqs = W.serving_requests(pool, 40, seed=11, reuse=0.5, it_range=(3, 12), max_handles=4)
    # a few identical (constraint set, iteration count) pairs so batches form
    for k in range(30, 40):
        src = reqs[k - 10]
        reqs[k] = W.ServeRequest(src.mesh, src.cidx, src.ctargets + 0.01 * (k - 29), src.iterations, True)
    alone = [lone(gpu, pool[r.mesh], r, precision) for r in reqs]
    srv = gpu.ArapServer(precision=precision, max_in_flight=6, prep_threads=3)
    ids = [srv.add_mesh(m.positions, m.faces) for m in pool]
    tickets = [srv.submit(ids[r.mesh], r.cidx, r.ctargets, r.iterations) for r in reqs]
    infos = []
    for k, (t, r) in enumerate(zip(tickets, reqs)):
        out, info = srv.wait(t)
        infos.append(info)
        rest = pool[r.mesh].positions
        if precision == "fp64":
            assert err(out, alone[k], rest) <= FP64_TOL, k
        else:
            assert err(out, alone[k], rest) <= MIXED_TOL, k
            if info["batch_size"] == 1:
                # a lone launch on a resident factor runs the same kernels as a fresh context
                assert err(out, alone[k], rest) <= 1e-9, k
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["factor_hits"] > 0
    # host time of the launch calls, and its phases (the struct layout matches the C ABI)
    assert st["launch_ms"] > 0 and len(st["launch_host_ms"]) == 5
    assert 0 < sum(st["launch_host_ms"]) <= st["launch_ms"] * 1.01
    if precision == "mixed":
        assert st["batched_launches"] > 0
    # the oracle pins a sample of them
    for k in (0, 7, 33):
        r = reqs[k]
        m = pool[r.mesh]
        ok, o = O.run_deform(m.positions, m.faces, r.cidx, r.ctargets, r.iterations)
        assert ok
        assert err(alone[k], o, m.positions) <= (FP64_TOL if precision == "fp64" else MIXED_TOL)


def test_factor_reuse_and_concurrent_clients(gpu):
    pool = small_pool()
    srv = gpu.ArapServer(max_in_flight=4, prep_threads=2)
    ids = [srv.add_mesh(m.positions, m.faces) for m in pool]
    reqs = W.serving_requests(pool, 48, seed=3, reuse=0.7, it_range=(2, 6), max_handles=3)
    results = [None] * len(reqs)
    lock = threading.Lock()

    def client(part):
        for k in part:
            r = reqs[k]
            t = srv.submit(ids[r.mesh], r.cidx, r.ctargets, r.iterations)
            out, info = srv.wait(t)
            with lock:
                results[k] = (out, info)

    th = [threading.Thread(target=client, args=(range(i, len(reqs), 4),)) for i in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert sum(1 for _, i in results if i["factor_reused"]) == st["factor_hits"] > 0
    for k in (0, 5, 21, 47):
        r = reqs[k]
        ref = lone(gpu, pool[r.mesh], r, "mixed")
        assert err(results[k][0], ref, pool[r.mesh].positions) <= MIXED_TOL


def test_budget_evicts_cold_factors(gpu):
    pool = small_pool()
    big = max(range(len(pool)), key=lambda i: pool[i].V)
    m = pool[big]
    reqs = W.serving_requests([m], 6, seed=5, reuse=0.0, it_range=(3, 3), max_handles=2)
    # the footprint of the mesh plus one resident factor, then a budget of 1.5 times that
    probe = gpu.ArapServer()
    pid = probe.add_mesh(m.positions, m.faces)
    probe.wait(probe.submit(pid, reqs[0].cidx, reqs[0].ctargets, 3))
    one = probe.stats()["resident_bytes"]
    probe.close()
    budget = int(one * 1.5)
    srv = gpu.ArapServer(budget_bytes=budget, max_batch=1)
    mid = srv.add_mesh(m.positions, m.faces)
    for r in reqs:
        out, info = srv.wait(srv.submit(mid, r.cidx, r.ctargets, r.iterations))
        ref = lone(gpu, m, r, "mixed")
        assert err(out, ref, m.positions) <= 1e-9
    st = srv.stats()
    srv.close()
    assert st["evictions"] >= 3
    assert st["peak_resident_bytes"] <= budget


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_mesh_ordering_matches_oracle(gpu, precision, tol):
    """ARAP_ORDER_MESH (one dissection per mesh, restricted to each constraint
    set's free vertices) changes only the factor's ordering: the positions
    stay within the form's tolerance of the oracle, for several constraint
    sets on one mesh."""
    pool = small_pool()
    m = max(pool, key=lambda x: x.V)
    reqs = W.serving_requests([m], 3, seed=9, reuse=0.0, it_range=(5, 5), max_handles=3)
    for r in reqs:
        got = lone(gpu, m, r, precision, "mesh")
        per_set = lone(gpu, m, r, precision, "per_set")
        ok, o = O.run_deform(m.positions, m.faces, r.cidx, r.ctargets, r.iterations)
        assert ok
        assert err(got, o, m.positions) <= tol
        assert err(per_set, o, m.positions) <= tol


def test_errors_reach_their_request(gpu):
    v, f = W.icosphere(2)
    pos = np.concatenate([v, v + 3.0])
    faces = np.concatenate([f, f + len(v)])
    srv = gpu.ArapServer(max_in_flight=2)
    mid = srv.add_mesh(pos, faces)
    # the second sphere has no constrained vertex: singular Laplacian
    with pytest.raises(gpu.ArapError) as e:
        srv.wait(srv.submit(mid, [0, 5], pos[[0, 5]], 3))
    assert e.value.code == gpu.ARAP_ERR_NOT_SPD
    with pytest.raises(gpu.ArapError) as e:
        srv.submit(mid, [0, len(pos)], pos[[0, 0]], 3)
    assert e.value.code == gpu.ARAP_ERR_BAD_INDEX
    # both spheres constrained: fine afterwards
    idx = [0, 5, len(v) + 1, len(v) + 9]
    out, info = srv.wait(srv.submit(mid, idx, pos[idx] + 0.1, 4))
    ok, o = O.run_deform(pos, faces, np.array(idx, np.int32), pos[idx] + 0.1, 4)
    assert ok and err(out, o, pos) <= MIXED_TOL
    # no constraints: the rest pose comes back (deform() returns early, arap.h:113-114)
    out, _ = srv.wait(srv.submit(mid, [], np.zeros((0, 3)), 4))
    np.testing.assert_array_equal(out, pos)
    # a budget smaller than one factor refuses the request
    tiny = gpu.ArapServer(budget_bytes=srv.stats()["peak_resident_bytes"] // 50 + 1)
    srv.close()
    try:
        tid = tiny.add_mesh(pos, faces)
        with pytest.raises(gpu.ArapError) as e:
            tiny.wait(tiny.submit(tid, idx, pos[idx], 3))
        assert e.value.code == gpu.ARAP_ERR_ADMISSION_REFUSED
    finally:
        tiny.close()
