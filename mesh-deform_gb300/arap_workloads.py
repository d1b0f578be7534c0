"""Seeded synthetic ARAP workloads (meshes, constraint sets, handle poses).

The reference publishes no benchmark data; its examples deform an icosphere
(examples/deform_sphere.cpp) and a box bar (examples/deform_bar.cpp) with
anchor/handle index sets. These generators produce the same kinds of inputs at
the benchmark sizes:

* ``icosphere(level)``     unit icosphere, 10*4^level + 2 vertices
* ``bar_grid(...)``        surface of an axis-aligned box on a regular grid,
                           two triangles per quad
* ``cfg_icosphere_l4``     2,562 vertices, anchors z<-0.8, handles z>0.8 moved by (0.3,0,0.5)
* ``cfg_twisted_bar``      10x1x1 box at 0.025 spacing (67,202 vertices), anchors x<0.2,
                           handles x>9.8 turned 90 deg about the bar axis (y=z=0.5) and
                           shifted (0,0.5,0)
* ``cfg_noisy_sphere``     icosphere level 7 with radial noise, 16 handle caps, 1 anchor cap
* ``cfg_pose_batch``       icosphere level 5, bottom cap anchored, top cap handle, many poses
* ``serving_pool`` / ``serving_requests``
                           a pool of noisy icospheres (levels 3-6) and bars (1k-200k
                           vertices, log-uniform) and a stream of requests with 1-8
                           handle caps plus one anchor cap, half of them reusing a
                           constraint set seen before, 5-50 iterations

Every function is deterministic for a given seed. Faces are counter-clockwise
seen from outside, as the adapter concept asks (inc/deform/openmesh_adapter.h:88).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    positions: np.ndarray          # V x 3 float64, rest pose
    faces: np.ndarray              # F x 3 int32
    cidx: np.ndarray               # constrained vertex indices, ascending
    ctargets: np.ndarray           # len(cidx) x 3 float64
    iterations: int
    precision: str = "fp64"        # "fp64" | "mixed"
    poses: np.ndarray | None = None   # P x len(cidx) x 3 targets for pose batches
    info: dict = field(default_factory=dict)

    @property
    def V(self) -> int:
        return int(self.positions.shape[0])

    @property
    def F(self) -> int:
        return int(self.faces.shape[0])

    def bbox_diag(self) -> float:
        return float(np.linalg.norm(self.positions.max(0) - self.positions.min(0)))


def _orient_outward(pos: np.ndarray, faces: np.ndarray, centre: np.ndarray) -> np.ndarray:
    a, b, c = pos[faces[:, 0]], pos[faces[:, 1]], pos[faces[:, 2]]
    n = np.cross(b - a, c - a)
    out = (a + b + c) / 3.0 - centre
    flip = (n * out).sum(1) < 0
    faces = faces.copy()
    faces[flip] = faces[flip][:, [0, 2, 1]]
    return faces


def icosahedron():
    phi = (1.0 + np.sqrt(5.0)) / 2.0
    v = []
    for s1, s2 in itertools.product((-1.0, 1.0), repeat=2):
        v.append((0.0, s1, s2 * phi))
        v.append((s1, s2 * phi, 0.0))
        v.append((s2 * phi, 0.0, s1))
    v = np.array(v, np.float64)
    n = len(v)
    faces = []
    d2 = ((v[:, None, :] - v[None, :, :]) ** 2).sum(-1)
    edge = np.isclose(d2, 4.0)
    for i, j, k in itertools.combinations(range(n), 3):
        if edge[i, j] and edge[j, k] and edge[i, k]:
            faces.append((i, j, k))
    faces = np.array(faces, np.int32)
    v = v / np.linalg.norm(v, axis=1, keepdims=True)
    faces = _orient_outward(v, faces, np.zeros(3))
    assert v.shape == (12, 3) and faces.shape == (20, 3)
    return v, faces


def icosphere(level: int):
    """Unit icosphere: each subdivision splits every triangle into four and
    pushes the new edge midpoints onto the sphere."""
    v, f = icosahedron()
    for _ in range(level):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
        lo, hi = np.minimum(e[:, 0], e[:, 1]).astype(np.int64), np.maximum(e[:, 0], e[:, 1]).astype(np.int64)
        key = lo * nv + hi
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // nv, uk % nv
        mid = (v[a] + v[b]) * 0.5
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid], 0)
        nf = len(f)
        m01 = nv + inv[:nf]
        m12 = nv + inv[nf:2 * nf]
        m20 = nv + inv[2 * nf:]
        f0, f1, f2 = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([
            np.stack([f0, m01, m20], 1),
            np.stack([f1, m12, m01], 1),
            np.stack([f2, m20, m12], 1),
            np.stack([m01, m12, m20], 1),
        ], 0).astype(np.int32)
    return v.astype(np.float64), f.astype(np.int32)


def bar_grid(length: float = 10.0, width: float = 1.0, height: float = 1.0, h: float = 0.025):
    """Surface of the box [0,length]x[0,width]x[0,height] on a grid of spacing
    h, two triangles per quad. Returns (positions, faces, grid index (V,3))."""
    nx, ny, nz = int(round(length / h)), int(round(width / h)), int(round(height / h))
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    boundary = (I == 0) | (I == nx) | (J == 0) | (J == ny) | (K == 0) | (K == nz)
    ids = -np.ones(boundary.shape, np.int64)
    ids[boundary] = np.arange(int(boundary.sum()))
    grid = np.stack([I[boundary], J[boundary], K[boundary]], 1)
    pos = grid.astype(np.float64) * h
    quads = []

    def add(a, b, c, d):
        quads.append(np.stack([a.ravel(), b.ravel(), c.ravel(), d.ravel()], 1))

    # x = const sides
    for i in (0, nx):
        jj, kk = np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")
        add(ids[i, jj, kk], ids[i, jj + 1, kk], ids[i, jj + 1, kk + 1], ids[i, jj, kk + 1])
    for j in (0, ny):
        ii, kk = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
        add(ids[ii, j, kk], ids[ii + 1, j, kk], ids[ii + 1, j, kk + 1], ids[ii, j, kk + 1])
    for k in (0, nz):
        ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        add(ids[ii, jj, k], ids[ii + 1, jj, k], ids[ii + 1, jj + 1, k], ids[ii, jj + 1, k])
    q = np.concatenate(quads, 0)
    assert (q >= 0).all()
    tris = np.concatenate([q[:, [0, 1, 2]], q[:, [0, 2, 3]]], 0).astype(np.int32)
    centre = np.array([length, width, height]) * 0.5
    tris = _orient_outward(pos, tris, centre)
    return pos, tris, grid


def rotation_matrix(axis, angle: float) -> np.ndarray:
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = np.cos(angle), np.sin(angle)
    C = 1.0 - c
    return np.array([
        [c + x * x * C, x * y * C - z * s, x * z * C + y * s],
        [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
        [z * x * C - y * s, z * y * C + x * s, c + z * z * C],
    ])


def cfg_icosphere_l4(level: int = 4, iterations: int = 10) -> Workload:
    """Unit icosphere L4, anchors z<-0.8 held, handles z>0.8 moved by (0.3,0,0.5)."""
    v, f = icosphere(level)
    anchors = np.nonzero(v[:, 2] < -0.8)[0]
    handles = np.nonzero(v[:, 2] > 0.8)[0]
    cidx = np.sort(np.concatenate([anchors, handles])).astype(np.int32)
    tgt = v[cidx].copy()
    tgt[np.isin(cidx, handles)] += np.array([0.3, 0.0, 0.5])
    return Workload(f"icosphere_l{level}", v, f, cidx, tgt, iterations, "fp64",
                    info={"anchors": int(len(anchors)), "handles": int(len(handles))})


def cfg_twisted_bar(h: float = 0.025, iterations: int = 30, precision: str = "mixed",
                    length: float = 10.0) -> Workload:
    """Box 10x1x1 at spacing h; anchors x<0.2; handles x>length-0.2 turned 90 deg
    about the x axis through (y,z)=(0.5,0.5) and shifted (0,0.5,0)."""
    pos, faces, grid = bar_grid(length, 1.0, 1.0, h)
    nx = int(round(length / h))
    ring = int(round(0.2 / h))
    anchors = np.nonzero(grid[:, 0] < ring)[0]
    handles = np.nonzero(grid[:, 0] > nx - ring)[0]
    # the integer selection equals the stated coordinate thresholds
    assert np.array_equal(anchors, np.nonzero(pos[:, 0] < 0.2)[0])
    assert np.array_equal(handles, np.nonzero(pos[:, 0] > length - 0.2)[0])
    cidx = np.sort(np.concatenate([anchors, handles])).astype(np.int32)
    tgt = pos[cidx].copy()
    hm = np.isin(cidx, handles)
    R = rotation_matrix([1.0, 0.0, 0.0], np.pi / 2)
    c = np.array([0.0, 0.5, 0.5])
    tgt[hm] = (tgt[hm] - c) @ R.T + c + np.array([0.0, 0.5, 0.0])
    return Workload(f"twisted_bar_h{h}", pos, faces, cidx, tgt, iterations, precision,
                    info={"anchors": int(len(anchors)), "handles": int(len(handles))})


def _caps(v, centres, radius):
    d = v / np.linalg.norm(v, axis=1, keepdims=True)
    return [np.nonzero(np.arccos(np.clip(d @ c, -1.0, 1.0)) <= radius)[0] for c in centres]


def cfg_noisy_sphere(level: int = 7, seed: int = 20261203, iterations: int = 50,
                     n_handles: int = 16, cap: float = 0.15, precision: str = "mixed") -> Workload:
    """Icosphere with radius 1+N(0,0.01) per vertex; 16 handle caps (geodesic
    radius 0.15, centres uniform on the sphere, translations U[-0.3,0.3]^3) and
    one anchor cap at the south pole. A vertex in the anchor cap is an anchor;
    a vertex in several handle caps follows the first of them."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(level)
    v = v * (1.0 + rng.normal(0.0, 0.01, size=(len(v), 1)))
    c = rng.normal(size=(n_handles, 3))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    trans = rng.uniform(-0.3, 0.3, size=(n_handles, 3))
    owner = -np.ones(len(v), np.int64)
    for k, idx in enumerate(_caps(v, c, cap)):
        sel = idx[owner[idx] == -1]
        owner[sel] = k
    (south,) = _caps(v, [np.array([0.0, 0.0, -1.0])], cap)
    owner[south] = n_handles  # anchor wins
    cidx = np.nonzero(owner >= 0)[0].astype(np.int32)
    tgt = v[cidx].copy()
    o = owner[cidx]
    hm = o < n_handles
    tgt[hm] += trans[o[hm]]
    return Workload(f"noisy_sphere_l{level}", v, f, cidx, tgt, iterations, precision,
                    info={"seed": seed, "anchors": int((o == n_handles).sum()), "handle_vertices": int(hm.sum())})


def cfg_pose_batch(level: int = 5, n_poses: int = 256, seed: int = 20261203,
                   iterations: int = 20, precision: str = "mixed") -> Workload:
    """Icosphere L5, anchors z<-0.8, handles z>0.8; each pose turns the handle
    cap by an angle U[0,60deg] about a random axis through the cap centroid and
    shifts it by U[-0.5,0.5]^3 (the origin*t*origin^-1 convention of
    inc/deform/deformation_util.h:48-57)."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(level)
    anchors = np.nonzero(v[:, 2] < -0.8)[0]
    handles = np.nonzero(v[:, 2] > 0.8)[0]
    cidx = np.sort(np.concatenate([anchors, handles])).astype(np.int32)
    hm = np.isin(cidx, handles)
    origin = v[handles].mean(0)
    poses = np.empty((n_poses, len(cidx), 3))
    transforms = np.zeros((n_poses, 3, 4))
    for p in range(n_poses):
        axis = rng.normal(size=3)
        ang = rng.uniform(0.0, np.pi / 3)
        t = rng.uniform(-0.5, 0.5, size=3)
        R = rotation_matrix(axis, ang)
        tg = v[cidx].copy()
        tg[hm] = (tg[hm] - origin) @ R.T + origin + t
        poses[p] = tg
        transforms[p, :, :3] = R
        transforms[p, :, 3] = t
    # the same poses as DeformationUtil inputs: tabs = O * [R|t] * O^-1 with O = [I|origin]
    O = np.zeros((3, 4))
    O[:, :3] = np.eye(3)
    O[:, 3] = origin
    return Workload(f"pose_batch_l{level}x{n_poses}", v, f, cidx, poses[0].copy(), iterations,
                    precision, poses=poses,
                    info={"seed": seed, "anchors": int(len(anchors)), "handles": int(len(handles)),
                          "handle_ids": handles.astype(np.int32), "transforms": transforms, "origin": O})


@dataclass
class PoolMesh:
    name: str
    positions: np.ndarray
    faces: np.ndarray
    kind: str                      # "sphere" | "bar"

    @property
    def V(self) -> int:
        return int(self.positions.shape[0])


@dataclass
class ServeRequest:
    mesh: int
    cidx: np.ndarray
    ctargets: np.ndarray
    iterations: int
    reused: bool                   # constraint set drawn from the ones used before
    arrival: float = 0.0           # seconds from the stream's start


def serving_pool(n_meshes: int = 64, seed: int = 20261203, levels=(3, 4, 5, 6), v_min: int = 1000,
                 v_max: int = 200_000) -> list:
    """Half noisy icospheres (radius 1+N(0,0.01), level uniform in `levels`),
    half bars 10x1x1 whose vertex count is log-uniform in [v_min, v_max]
    (the grid spacing that gives it: V ~ 42/h^2)."""
    rng = np.random.default_rng(seed)
    pool, spheres = [], {}
    for i in range(n_meshes):
        if rng.uniform() < 0.5:
            lv = int(rng.choice(levels))
            if lv not in spheres:
                spheres[lv] = icosphere(lv)
            v, f = spheres[lv]
            v = v * (1.0 + rng.normal(0.0, 0.01, size=(len(v), 1)))
            pool.append(PoolMesh(f"sphere{i}_l{lv}", v, f, "sphere"))
        else:
            target = float(np.exp(rng.uniform(np.log(v_min), np.log(v_max))))
            h = 10.0 / max(2, round(10.0 / np.sqrt(42.0 / target)))
            v, f, _ = bar_grid(10.0, 1.0, 1.0, h)
            pool.append(PoolMesh(f"bar{i}_h{h:.4f}", v, f, "bar"))
    return pool


def _cap_sets(mesh: PoolMesh, rng, n_handles: int, radius: float = 0.15):
    """Index sets of n_handles handle caps and one anchor cap: geodesic disks
    on a sphere (the anchor at the south pole), Euclidean balls around random
    surface vertices on a bar (the anchor at the x=0 end)."""
    v = mesh.positions
    if mesh.kind == "sphere":
        c = rng.normal(size=(n_handles, 3))
        c /= np.linalg.norm(c, axis=1, keepdims=True)
        handles = _caps(v, c, radius)
        (anchor,) = _caps(v, [np.array([0.0, 0.0, -1.0])], radius)
    else:
        centres = v[rng.integers(0, len(v), size=n_handles)]
        handles = [np.nonzero(np.linalg.norm(v - c, axis=1) <= radius)[0] for c in centres]
        anchor = np.nonzero(v[:, 0] < 0.2)[0]
    return handles, anchor


def serving_requests(pool: list, n_requests: int, seed: int = 20261204, reuse: float = 0.5,
                     rate_hz: float | None = None, it_range=(5, 50), max_handles: int = 8) -> list:
    """Requests over `pool`: mesh uniform; with probability `reuse` the
    constraint set of an earlier request on the same mesh (new handle
    translations), otherwise 1..max_handles new handle caps plus the anchor cap
    (anchor wins overlaps, a vertex in several handle caps follows the first);
    handle translations U[-0.3,0.3]^3; iterations uniform in it_range; Poisson
    arrivals at rate_hz (all at t=0 when None)."""
    rng = np.random.default_rng(seed)
    seen = {i: [] for i in range(len(pool))}
    out, t = [], 0.0
    for _ in range(n_requests):
        mi = int(rng.integers(0, len(pool)))
        mesh = pool[mi]
        reused = bool(seen[mi]) and rng.uniform() < reuse
        if reused:
            cidx, owner, nh = seen[mi][int(rng.integers(0, len(seen[mi])))]
        else:
            nh = int(rng.integers(1, max_handles + 1))
            handles, anchor = _cap_sets(mesh, rng, nh)
            own = -np.ones(mesh.V, np.int64)
            for k, idx in enumerate(handles):
                sel = idx[own[idx] == -1]
                own[sel] = k
            own[anchor] = nh
            cidx = np.nonzero(own >= 0)[0].astype(np.int32)
            owner = own[cidx]
            seen[mi].append((cidx, owner, nh))
        trans = rng.uniform(-0.3, 0.3, size=(nh + 1, 3))
        trans[nh] = 0.0
        tgt = mesh.positions[cidx] + trans[owner]
        iters = int(rng.integers(it_range[0], it_range[1] + 1))
        if rate_hz:
            t += float(rng.exponential(1.0 / rate_hz))
        out.append(ServeRequest(mi, cidx, tgt, iters, reused, t))
    return out


def bbox_rel_error(x: np.ndarray, ref: np.ndarray, rest: np.ndarray) -> float:
    """max_v |x_v - ref_v| / |bbox_max - bbox_min| of the rest mesh."""
    diag = float(np.linalg.norm(rest.max(0) - rest.min(0)))
    return float(np.linalg.norm(x - ref, axis=1).max() / diag)
