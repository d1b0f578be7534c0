"""CPU tests of the library's host side: the shared object loads and exports
every entry point include/arap_gpu.h declares, and the host symbolic analysis
(adjacency, nested-dissection ordering, elimination tree, supernode partition)
is bit-exact against the oracle's own restatement."""
import re
from pathlib import Path

import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(arap_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_every_declared_symbol(gpu):
    lib = gpu.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert names == set(gpu.SIGNATURES), names ^ set(gpu.SIGNATURES)


def test_status_strings(gpu):
    lib = gpu.load()
    assert lib.arap_status_string(0) == b"ARAP_OK"
    assert lib.arap_status_string(3) == b"ARAP_ERR_NOT_SPD"


def test_create_without_device_fails_loudly(gpu):
    """On a machine without a GPU the library refuses instead of falling back."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu.ArapError) as e:
        gpu.ArapContext(3, np.array([[0, 1, 2]]))
    assert e.value.code == gpu.ARAP_ERR_NO_DEVICE


def test_server_without_device_fails_loudly(gpu):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu.ArapError) as e:
        gpu.ArapServer()
    assert e.value.code == gpu.ARAP_ERR_NO_DEVICE


CASES = [
    lambda: W.cfg_icosphere_l4(level=4),
    lambda: W.cfg_twisted_bar(h=0.05),
    lambda: W.cfg_noisy_sphere(level=5),
    lambda: W.cfg_pose_batch(level=4, n_poses=1),
    # large enough that the dissection runs its two sides on threads
    lambda: W.cfg_twisted_bar(h=0.025),
    lambda: W.cfg_noisy_sphere(level=7),
]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_symbolic_bitexact_against_oracle(gpu, k):
    w = CASES[k]()
    a = gpu.analyze_pattern(w.V, w.faces, w.cidx)
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    o.deform(0)
    assert a["m"] == o.num_free()
    np.testing.assert_array_equal(a["perm"], o.ordering())
    np.testing.assert_array_equal(a["etree"], o.etree())
    np.testing.assert_array_equal(a["block_ptr"], o.blocks())
    # the oracle's LDL^T stores the strictly lower part, the library counts the diagonal too
    assert a["factor_nnz"] == o.factor_nnz() + o.num_free()


def test_symbolic_disconnected_components(gpu):
    """Two separate spheres, each with constraints: the dissection orders the
    components one after the other (in order of their smallest vertex)."""
    v, f = W.icosphere(3)
    pos = np.concatenate([v, v + 3.0])
    faces = np.concatenate([f, f + len(v)])
    cidx = np.array([0, 5, len(v) + 7], np.int32)
    a = gpu.analyze_pattern(len(pos), faces, cidx)
    o = O.OracleARAP(pos, faces)
    o.set_constraints(cidx, pos[cidx])
    o.deform(0)
    np.testing.assert_array_equal(a["perm"], o.ordering())
    np.testing.assert_array_equal(a["etree"], o.etree())
    np.testing.assert_array_equal(a["block_ptr"], o.blocks())


def test_symbolic_matches_standalone_nd(gpu):
    """The oracle's nd_order on the free graph equals the library's ordering."""
    w = W.cfg_twisted_bar(h=0.1)
    a = gpu.analyze_pattern(w.V, w.faces, w.cidx)
    free = np.setdiff1d(np.arange(w.V), w.cidx)
    fidx = -np.ones(w.V, np.int64)
    fidx[free] = np.arange(len(free))
    nbr = [set() for _ in range(len(free))]
    for tri in w.faces:
        for x, y in ((tri[0], tri[1]), (tri[1], tri[2]), (tri[2], tri[0])):
            if fidx[x] >= 0 and fidx[y] >= 0 and x != y:
                nbr[fidx[x]].add(fidx[y])
                nbr[fidx[y]].add(fidx[x])
    rp = np.zeros(len(free) + 1, np.int32)
    rp[1:] = np.cumsum([len(s) for s in nbr])
    col = np.concatenate([sorted(s) for s in nbr]).astype(np.int32)
    perm, bp = O.nd_order(rp, col)
    np.testing.assert_array_equal(a["perm"], perm)
    np.testing.assert_array_equal(a["block_ptr"], bp)


def test_floating_component_is_rejected(gpu):
    """A mesh component without any constrained vertex makes L singular."""
    v, f = W.icosphere(2)
    pos = np.concatenate([v, v + 3.0])
    faces = np.concatenate([f, f + len(v)])
    with pytest.raises(gpu.ArapError) as e:
        gpu.analyze_pattern(len(pos), faces, np.array([0], np.int32))
    assert e.value.code == gpu.ARAP_ERR_NOT_SPD


def test_bad_face_index_is_rejected(gpu):
    with pytest.raises(gpu.ArapError) as e:
        gpu.analyze_pattern(3, np.array([[0, 1, 5]]), np.array([0], np.int32))
    assert e.value.code == gpu.ARAP_ERR_BAD_INDEX


def test_workload_sizes():
    """The benchmark configurations have the stated sizes."""
    assert W.cfg_icosphere_l4().V == 2562 and W.cfg_icosphere_l4().F == 5120
    b = W.cfg_twisted_bar()
    assert (b.V, b.F, b.info["anchors"], b.info["handles"]) == (67202, 134400, 2801, 2801)
    p = W.cfg_pose_batch(level=5, n_poses=4)
    assert p.V == 10242 and p.poses.shape == (4, 2058, 3)
    assert W.icosphere(7)[0].shape == (163842, 3)


def test_threaded_dissection_is_deterministic(gpu):
    """The dissection of a large free graph splits over threads; repeated
    analyses give the same ordering, tree and blocks every time."""
    w = W.cfg_twisted_bar(h=0.025)
    first = gpu.analyze_pattern(w.V, w.faces, w.cidx)
    for _ in range(3):
        again = gpu.analyze_pattern(w.V, w.faces, w.cidx)
        for key in ("perm", "etree", "block_ptr"):
            np.testing.assert_array_equal(first[key], again[key])


def test_dissection_of_a_mesh_batch_orders_each_mesh_as_alone(gpu):
    """A batch of meshes (their disjoint union) is dissected one mesh per
    component, the components on a pool of threads: each mesh gets the
    ordering, elimination tree and blocks it gets alone, shifted by the free
    vertices of the meshes before it, and repeated analyses agree."""
    parts = [W.cfg_twisted_bar(h=0.05, iterations=1), W.cfg_icosphere_l4(level=5, iterations=1),
             W.cfg_twisted_bar(h=0.04, iterations=1, length=6.0)]
    offs = np.cumsum([0] + [p.V for p in parts])
    faces = np.concatenate([p.faces + offs[k] for k, p in enumerate(parts)])
    cidx = np.concatenate([np.asarray(p.cidx) + offs[k] for k, p in enumerate(parts)])
    union = gpu.analyze_pattern(int(offs[-1]), faces, cidx)
    assert len(union["perm"]) >= 16384  # large enough for the threaded path
    M = 0
    perm, etree, bptr = [], [], [0]
    for p in parts:
        a = gpu.analyze_pattern(p.V, p.faces, p.cidx)
        perm.append(np.asarray(a["perm"]) + M)
        e = np.asarray(a["etree"]).copy()
        e[e >= 0] += M
        etree.append(e)
        bptr.extend((np.asarray(a["block_ptr"])[1:] + M).tolist())
        M += len(a["perm"])
    np.testing.assert_array_equal(union["perm"], np.concatenate(perm))
    np.testing.assert_array_equal(union["etree"], np.concatenate(etree))
    np.testing.assert_array_equal(union["block_ptr"], np.asarray(bptr))
    again = gpu.analyze_pattern(int(offs[-1]), faces, cidx)
    for key in ("perm", "etree", "block_ptr"):
        np.testing.assert_array_equal(union[key], again[key])


def test_concurrent_analyses_match_a_lone_analysis(gpu):
    """Several analyses at once (the library splits its row loops over threads
    only when an analysis runs alone) give the ordering, elimination tree and
    blocks of a lone analysis."""
    import threading

    w = W.cfg_twisted_bar(h=0.025)
    alone = gpu.analyze_pattern(w.V, w.faces, w.cidx)
    outs = [None] * 4

    def run(i):
        outs[i] = gpu.analyze_pattern(w.V, w.faces, w.cidx)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(outs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for o in outs:
        for key in ("perm", "etree", "block_ptr"):
            np.testing.assert_array_equal(o[key], alone[key])
