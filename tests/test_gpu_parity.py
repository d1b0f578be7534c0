"""GPU parity: the CUDA library (through the C ABI) against the FP64 oracle.

Tolerances (bounding-box-diagonal-relative max vertex error):
  FP64 form   <= 1e-10
  mixed form  <= 1e-6
Cotan weights are compared bit-exactly (both sides round every operation of
arap.h:189-238 in the same order); adjacency, ordering, elimination tree and
supernode partition are compared exactly.
"""
import numpy as np
import pytest

import arap_workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-6}


def small_cases():
    return [
        W.cfg_icosphere_l4(level=3, iterations=5),
        W.cfg_icosphere_l4(level=4, iterations=10),          # the reference-runnable config
        W.cfg_twisted_bar(h=0.1, iterations=10),
        W.cfg_noisy_sphere(level=4, iterations=8),
    ]


def gpu_deform(gpu, w, precision, iterations=None, refine=2):
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision(precision, refine)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        out = ctx.deform(w.iterations if iterations is None else iterations)
        return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", range(4))
def test_deform_matches_oracle(gpu, precision, case):
    w = small_cases()[case]
    ok, ref = O.run_deform(w.positions, w.faces, w.cidx, w.ctargets, w.iterations)
    assert ok
    out = gpu_deform(gpu, w, precision)
    err = W.bbox_rel_error(out, ref, w.positions)
    assert err <= TOL[precision], f"{w.name} {precision}: {err:.3e}"
    # constrained vertices sit exactly on their targets
    np.testing.assert_array_equal(out[w.cidx], w.ctargets)


def test_cotan_kat_and_bitexact_weights(gpu):
    """tests/test_cotan.cpp:26-53 through the GPU: unit square, deform(0)."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], float)
    faces = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    mesh = gpu.ArrayMesh(pos, faces)
    arap = gpu.AsRigidAsPossibleDeformation(mesh)
    assert arap.deform(0)
    Wd = arap.cotan_weights()
    expected = np.array([[0, .5, 0, .5], [.5, 0, .5, 0], [0, .5, 0, .5], [.5, 0, .5, 0]])
    # Eigen isApprox(expected, 1e-4): ||a-b|| <= 1e-4 * min(||a||, ||b||)
    assert np.linalg.norm(Wd - expected) <= 1e-4 * min(np.linalg.norm(Wd), np.linalg.norm(expected))
    o = O.OracleARAP(pos, faces)
    o.deform(0)
    rp, col, val = o.weights_csr()
    grp, gcol, gval = arap.ctx.edge_weights()
    np.testing.assert_array_equal(rp, grp)
    np.testing.assert_array_equal(col, gcol)
    np.testing.assert_array_equal(val, gval)


def test_weights_bitexact_large(gpu):
    w = W.cfg_noisy_sphere(level=5, iterations=1)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        ctx.deform(0)
        grp, gcol, gval = ctx.edge_weights()
        sym = ctx.symbolic()
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    o.deform(0)
    rp, col, val = o.weights_csr()
    np.testing.assert_array_equal(rp, grp)
    np.testing.assert_array_equal(col, gcol)
    np.testing.assert_array_equal(val, gval)
    np.testing.assert_array_equal(sym["perm"], o.ordering())
    np.testing.assert_array_equal(sym["etree"], o.etree())
    np.testing.assert_array_equal(sym["block_ptr"], o.blocks())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rotations_match_oracle(gpu, precision):
    w = W.cfg_icosphere_l4(level=3, iterations=3)
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    o.deform(3)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision(precision, 2)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        ctx.deform(3)
        R = ctx.rotations()
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.abs(R - o.rotations()).max() <= tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_continued_deform_without_new_constraints(gpu, precision):
    """Two deform(4) calls without setConstraint in between continue from
    _pprime and reuse the factor (arap.h:102,119,122-129)."""
    w = W.cfg_twisted_bar(h=0.1, iterations=4)
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    o.deform(4)
    o.deform(4)
    ref = o.mesh_positions()
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision(precision, 2)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, w.ctargets)
        ctx.deform(4, want_output=False)
        out = ctx.deform(4)
    assert W.bbox_rel_error(out, ref, w.positions) <= TOL[precision]


def test_dirty_deform_recaptures_rest_pose(gpu):
    """After setConstraint the next deform rebuilds the problem from the mesh's
    current positions (arap.h:102-120,162-168), as the bar example relies on."""
    w = W.cfg_icosphere_l4(level=3, iterations=4)
    mesh_o = w.positions.copy()
    o = O.OracleARAP(mesh_o, w.faces)
    mesh = gpu.ArrayMesh(w.positions, w.faces)
    g = gpu.AsRigidAsPossibleDeformation(mesh)
    for c, t in zip(w.cidx, w.ctargets):
        o.set_constraint(c, t)
        g.set_constraint(c, t)
    assert o.deform(4) and g.deform(4)
    shift = np.array([0.0, 0.2, -0.1])
    for c, t in zip(w.cidx[:10], w.ctargets[:10]):
        o.set_constraint(c, t + shift)
        g.set_constraint(c, t + shift)
    assert o.deform(4) and g.deform(4)
    assert W.bbox_rel_error(mesh.positions, o.mesh_positions(), w.positions) <= 1e-10


def test_zero_iterations_snaps_targets(gpu):
    w = W.cfg_icosphere_l4(level=3, iterations=0)
    out = gpu_deform(gpu, w, "fp64", iterations=0)
    exp = w.positions.copy()
    exp[w.cidx] = w.ctargets
    np.testing.assert_array_equal(out, exp)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rigid_motion_is_reproduced(gpu, precision):
    """All constrained vertices moved by one rigid motion: the ARAP optimum is
    that motion of the whole mesh (energy 0); 200 iterations from the rest pose
    reach it to rounding (the FP64 CPU path gets 4e-15)."""
    w = W.cfg_icosphere_l4(level=3, iterations=200)
    R = W.rotation_matrix([0.3, -0.5, 0.8], 0.7)
    t = np.array([0.2, -0.4, 0.1])
    tgt = w.positions[w.cidx] @ R.T + t
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_precision(precision, 2)
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(w.cidx, tgt)
        out = ctx.deform(200)
    exp = w.positions @ R.T + t
    assert W.bbox_rel_error(out, exp, w.positions) <= (1e-9 if precision == "fp64" else 2e-6)


def test_singular_system_reports_not_spd(gpu):
    """A free vertex without faces makes L singular; the reference's deform
    returns false (arap.h:116-117,339)."""
    v, f = W.icosphere(2)
    pos = np.concatenate([v, [[5.0, 5.0, 5.0]]])
    mesh = gpu.ArrayMesh(pos, f)
    g = gpu.AsRigidAsPossibleDeformation(mesh)
    g.set_constraint(0, pos[0] + 0.1)
    assert g.deform(3) is False
    o = O.OracleARAP(pos, f)
    o.set_constraint(0, pos[0] + 0.1)
    assert o.deform(3) is False


def test_bad_constraint_index(gpu):
    w = W.cfg_icosphere_l4(level=2, iterations=1)
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_rest_positions(w.positions)
        with pytest.raises(gpu.ArapError) as e:
            ctx.set_constraints([w.V + 3], [[0, 0, 0]])
        assert e.value.code == gpu.ARAP_ERR_BAD_INDEX


def test_all_vertices_constrained(gpu):
    w = W.cfg_icosphere_l4(level=2, iterations=2)
    tgt = w.positions + 0.25
    with gpu.ArapContext(w.V, w.faces) as ctx:
        ctx.set_rest_positions(w.positions)
        ctx.set_constraints(np.arange(w.V), tgt)
        out = ctx.deform(2)
    np.testing.assert_array_equal(out, tgt)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["sphere", "bar", "plane"])
def test_golden_fixture_deforms(gpu, name, precision):
    """The reference's etc/ meshes with example-style constraint sets, against
    the committed oracle outputs (tests/golden/oracle_deforms.npz)."""
    from pathlib import Path

    g = Path(__file__).resolve().parent / "golden"
    m = np.load(g / "meshes.npz")
    d = np.load(g / "oracle_deforms.npz")
    v, f = m[f"{name}_v"], m[f"{name}_f"]
    with gpu.ArapContext(len(v), f) as ctx:
        ctx.set_precision(precision, 2)
        ctx.set_rest_positions(v)
        ctx.set_constraints(d[f"{name}_cidx"], d[f"{name}_targets"])
        out = ctx.deform(int(d[f"{name}_iterations"]))
    assert W.bbox_rel_error(out, d[f"{name}_out"], v) <= TOL[precision]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_energy_matches_oracle_and_decreases(gpu, precision, tol):
    """K9: the FP64 ARAP energy of the GPU state equals the oracle's energy of
    its own state (relative tolerance of the precision form) after every
    iteration, and the iteration does not increase it."""
    from oracle import oracle as O

    w = W.cfg_icosphere_l4(level=3, iterations=1)
    o = O.OracleARAP(w.positions, w.faces)
    o.set_constraints(w.cidx, w.ctargets)
    ctx = gpu.ArapContext(w.V, w.faces)
    ctx.set_precision(precision, 1)
    ctx.set_rest_positions(w.positions)
    ctx.set_constraints(w.cidx, w.ctargets)
    prev = None
    for k in range(6):
        ctx.deform(1)
        o.deform(1)
        eg, eo = ctx.energy(), o.energy()
        assert abs(eg - eo) <= tol * eo, (k, eg, eo)
        if prev is not None and precision == "fp64":
            assert eg <= prev * (1 + 1e-12)
        prev = eg
    ctx.close()


def test_vertex_normals_and_device_positions(gpu):
    """Vertex normals of the deformed mesh (OpenMesh's update_normals rule,
    examples/osg_viewer.cpp:53,60-62) against numpy, and the device-resident
    positions against the host copy of the same deform."""
    import torch

    w = W.cfg_icosphere_l4(level=3, iterations=5)
    ctx = gpu.ArapContext(w.V, w.faces)
    ctx.set_rest_positions(w.positions)
    ctx.set_constraints(w.cidx, w.ctargets)
    out = ctx.deform(w.iterations)
    n = ctx.vertex_normals()
    a, b, c = out[w.faces[:, 0]], out[w.faces[:, 1]], out[w.faces[:, 2]]
    fn = np.cross(b - a, c - a)
    fn /= np.linalg.norm(fn, axis=1, keepdims=True)
    vn = np.zeros_like(out)
    for k in range(3):
        np.add.at(vn, w.faces[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    np.testing.assert_allclose(n, vn, atol=1e-12)
    pos, nrm = ctx.device_positions(with_normals=True)
    np.testing.assert_array_equal(torch.as_tensor(pos, device="cuda").cpu().numpy(), out)
    np.testing.assert_allclose(torch.as_tensor(nrm, device="cuda").cpu().numpy(), vn, atol=1e-12)
    ctx.close()
