"""CPU tests of the FP64 oracle: pinned against the reference's known-answer
test and golden fixtures, cross-checked against an independent numpy/scipy
restatement, and checked on exact properties of ARAP."""
import json
from pathlib import Path

import numpy as np
import pytest

import arap_workloads as W
import np_arap
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def dense(rp, col, val, n):
    M = np.zeros((n, n))
    for i in range(n):
        M[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    return M


def test_cotan_known_answer():
    """tests/test_cotan.cpp:20-54: unit square, deform(0), isApprox(expected, 1e-4)."""
    kat = json.loads((GOLDEN / "cotan_kat.json").read_text())
    pos = np.array(kat["positions"])
    faces = np.array(kat["faces"], np.int32)
    o = O.OracleARAP(pos, faces)
    assert o.deform(0)
    Wd = dense(*o.weights_csr(), 4)
    E = np.array(kat["expected_weights"])
    assert Wd.shape == (4, 4)
    assert np.linalg.norm(Wd - E) <= kat["isApprox_tol"] * min(np.linalg.norm(Wd), np.linalg.norm(E))
    # the diagonal's cotangent of a right angle is clamped to 1e-10 per face (arap.h:216-218)
    assert Wd[0, 2] == pytest.approx(1e-10, rel=1e-6)
    np.testing.assert_array_equal(Wd, Wd.T)
    assert np.all(np.diag(Wd) == 0)


def test_no_constraints_returns_true_without_writeback():
    """arap.h:113-114."""
    v, f = W.icosphere(2)
    o = O.OracleARAP(v, f)
    o.set_mesh_positions(v + 1.0)
    assert o.deform(5)
    np.testing.assert_array_equal(o.mesh_positions(), v + 1.0)


@pytest.mark.parametrize("name", ["sphere", "bar", "plane"])
def test_oracle_reproduces_golden_deforms(name):
    """Fixture meshes from the reference's etc/ with example-style constraints;
    the committed outputs were produced by the oracle on x86-64 (make_golden.py),
    so this also pins x86-64 against aarch64 rounding."""
    m = np.load(GOLDEN / "meshes.npz")
    g = np.load(GOLDEN / "oracle_deforms.npz")
    v, f = m[f"{name}_v"], m[f"{name}_f"]
    ok, out = O.run_deform(v, f, g[f"{name}_cidx"], g[f"{name}_targets"], int(g[f"{name}_iterations"]))
    assert ok
    assert W.bbox_rel_error(out, g[f"{name}_out"], v) <= 1e-12


CASES = [
    lambda: W.cfg_icosphere_l4(level=3, iterations=5),
    lambda: W.cfg_twisted_bar(h=0.1, iterations=8),
    lambda: W.cfg_noisy_sphere(level=3, iterations=6),
]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_oracle_matches_numpy_restatement(k):
    w = CASES[k]()
    ok, a = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    ok2, b = np_arap.deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok and ok2
    assert W.bbox_rel_error(a, b, w.positions) <= 1e-11


@pytest.mark.parametrize("name", ["sphere", "bar", "plane"])
def test_golden_fixtures_match_numpy_restatement(name):
    m = np.load(GOLDEN / "meshes.npz")
    g = np.load(GOLDEN / "oracle_deforms.npz")
    v, f = m[f"{name}_v"], m[f"{name}_f"]
    ok, b = np_arap.deform(v, f, g[f"{name}_cidx"], g[f"{name}_targets"], int(g[f"{name}_iterations"]))
    assert W.bbox_rel_error(g[f"{name}_out"], b, v) <= 1e-11


def test_weights_match_numpy():
    w = W.cfg_noisy_sphere(level=3)
    o = O.OracleARAP(w.positions, w.faces)
    o.deform(0)
    Wo = dense(*o.weights_csr(), w.V)
    Wn = np_arap.cotan_weights(w.positions, w.faces).toarray()
    np.testing.assert_allclose(Wo, Wn, rtol=1e-13, atol=1e-15)


def test_rotation_fit_matches_lapack_svd():
    rng = np.random.default_rng(7)
    covs = rng.normal(size=(200, 3, 3))
    # planar one-rings (rank 2) and nearly symmetric near-identity cases
    e = rng.normal(size=(200, 6, 3))
    e[:, :, 2] = 0.0
    f = e + 0.05 * rng.normal(size=e.shape)
    covs = np.concatenate([covs, np.einsum("nki,nkj->nij", e, f)])
    for c in covs:
        R = O.rotation_from_covariance(c)
        U, S, Vt = np.linalg.svd(c)
        Vm, Ut = Vt.T, U.T
        D = np.diag([1.0, 1.0, np.linalg.det(Vm @ Ut)])
        np.testing.assert_allclose(R, Vm @ D @ Ut, atol=1e-10)
        np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
        assert np.linalg.det(R) == pytest.approx(1.0, abs=1e-12)


def test_rigid_motion_known_answer():
    """With every constraint moved by one rigid motion the optimum is that motion."""
    w = W.cfg_icosphere_l4(level=3)
    R = W.rotation_matrix([0.3, -0.5, 0.8], 0.7)
    t = np.array([0.2, -0.4, 0.1])
    ok, out = O.run_deform(w.positions, w.faces, w.cidx, w.positions[w.cidx] @ R.T + t, 200)
    assert ok
    assert W.bbox_rel_error(out, w.positions @ R.T + t, w.positions) <= 1e-12


def test_deform_zero_snaps_targets():
    w = W.cfg_icosphere_l4(level=2)
    ok, out = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, 0)
    exp = w.positions.copy()
    exp[w.cidx] = w.ctargets
    np.testing.assert_array_equal(out, exp)


def test_constraint_map_overwrite():
    """setConstraint on the same vertex twice keeps the last target (arap.h:83)."""
    w = W.cfg_icosphere_l4(level=2)
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets + 5.0)
    o.set_constraints(w.cidx, w.ctargets)
    assert o.deform(3)
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, 3)
    np.testing.assert_array_equal(o.mesh_positions(), ref)


def test_isolated_free_vertex_fails():
    """A zero pivot makes SimplicialLDLT fail; deform returns false (arap.h:116-117)."""
    v, f = W.icosphere(2)
    pos = np.concatenate([v, [[3.0, 0.0, 0.0]]])
    o = O.OracleARAP(pos, f)
    o.set_constraint(0, pos[0])
    assert o.deform(2) is False


def test_nd_ordering_is_a_permutation_and_blocks_cover():
    w = W.cfg_twisted_bar(h=0.1)
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    o.deform(0)
    perm = o.ordering()
    assert sorted(perm.tolist()) == list(range(o.num_free()))
    bp = o.blocks()
    assert bp[0] == 0 and bp[-1] == o.num_free() and np.all(np.diff(bp) > 0)
    et = o.etree()
    # elimination tree: parent index is larger than the child's
    assert np.all((et == -1) | (et > np.arange(len(et))))
