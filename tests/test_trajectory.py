"""TrajectorySE3 (deform/trajectory.h, the reference's inc/deform/trajectory.h:
33-83 without Eigen/Sophus): the reference's own test (tests/test_trajectory.cpp:
17-39: the path passes through its first and last key poses) and samples in
between against an independent restatement (scipy's B-spline with the same
chord-length parameters and averaged knots, scipy's rotation log/exp)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def rot_x(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def affine(R=np.eye(3), t=(0, 0, 0)):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def reference_test_poses():
    """The key poses of tests/test_trajectory.cpp:23-34."""
    p0 = np.eye(4)
    p1 = affine(t=(0, 0, 1)) @ p0
    p2 = affine(t=(0, 0, 1)) @ affine(R=rot_x(np.pi / 4)) @ p1
    p3 = affine(t=(0, 0, 1)) @ p2
    return [p0, p1, p2, p3]


def np_log(T):
    from scipy.spatial.transform import Rotation

    om = Rotation.from_matrix(T[:3, :3]).as_rotvec()
    th = np.linalg.norm(om)
    W = np.array([[0, -om[2], om[1]], [om[2], 0, -om[0]], [-om[1], om[0], 0]])
    b = 1 / 12 if th < 1e-8 else (1 - th * np.sin(th) / (2 * (1 - np.cos(th)))) / th**2
    Vinv = np.eye(3) - 0.5 * W + b * W @ W
    return np.concatenate([Vinv @ T[:3, 3], om])


def np_exp(x):
    from scipy.spatial.transform import Rotation

    om = x[3:]
    th = np.linalg.norm(om)
    W = np.array([[0, -om[2], om[1]], [om[2], 0, -om[0]], [-om[1], om[0], 0]])
    if th < 1e-8:
        V = np.eye(3) + 0.5 * W
    else:
        V = np.eye(3) + (1 - np.cos(th)) / th**2 * W + (th - np.sin(th)) / th**3 * W @ W
    return affine(Rotation.from_rotvec(om).as_matrix(), V @ x[:3])


def np_path(poses, times):
    from scipy.interpolate import make_interp_spline

    pts = np.array([np_log(T) for T in poses])
    n, p = len(pts), 3
    u = np.concatenate([[0], np.cumsum(np.linalg.norm(np.diff(pts, axis=0), axis=1))])
    u /= u[-1]
    knots = np.concatenate([np.zeros(p + 1), [u[j:j + p].mean() for j in range(1, n - p)], np.ones(p + 1)])
    spl = make_interp_spline(u, pts, k=p, t=knots)
    return [np_exp(spl(t)) for t in times]


def cpp_path(tmp_path, poses, times):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "traj"
    subprocess.run([gxx, "-O1", "-std=c++17", f"-I{ROOT / 'mesh-deform_gb300'}",
                    str(ROOT / "tests" / "cpp" / "trajectory_main.cpp"), "-o", str(exe)], check=True)
    inp = [str(len(poses))] + [" ".join(repr(float(x)) for x in T[:3].ravel()) for T in poses]
    inp += [str(len(times)), " ".join(repr(float(t)) for t in times)]
    r = subprocess.run([str(exe)], input="\n".join(inp) + "\n", capture_output=True, text=True, check=True)
    out = []
    for line in r.stdout.strip().splitlines():
        T = np.eye(4)
        T[:3] = np.array([float(x) for x in line.split()]).reshape(3, 4)
        out.append(T)
    return out


def test_reference_trajectory_test(tmp_path):
    poses = reference_test_poses()
    got = cpp_path(tmp_path, poses, [0.0, 1.0])
    # Eigen's isApprox(b, 1e-3): |a - b| <= 1e-3 * min(|a|, |b|) (Frobenius)
    for a, b in ((got[0], poses[0]), (got[1], poses[3])):
        assert np.linalg.norm(a - b) <= 1e-3 * min(np.linalg.norm(a), np.linalg.norm(b))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_samples_match_independent_restatement(tmp_path, seed):
    rng = np.random.default_rng(seed)
    poses = reference_test_poses() if seed == 0 else []
    if seed:
        from scipy.spatial.transform import Rotation

        for _ in range(4 + 2 * seed):
            poses.append(affine(Rotation.from_rotvec(rng.uniform(-1.2, 1.2, 3)).as_matrix(), rng.uniform(-1, 1, 3)))
    times = np.linspace(0, 1, 11)
    got = cpp_path(tmp_path, poses, times)
    ref = np_path(poses, times)
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a, b, atol=1e-9)
    # rotations stay rotations
    for a in got:
        np.testing.assert_allclose(a[:3, :3] @ a[:3, :3].T, np.eye(3), atol=1e-12)
