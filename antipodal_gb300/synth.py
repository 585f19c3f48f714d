"""Seeded synthetic meshes, boundaries and query sets for the GWN benchmarks and parity tests.

Everything here is plain numpy and deterministic for a given seed (numpy's PCG64 ``default_rng``), so the
same inputs are rebuilt on any machine.  The workloads:

* ``unit_cube`` -- the reference test suite's +-0.5 cube, closed or with the +Y face removed, and its
  hand-oriented open boundary (test/test_gwn_mesh.cc:27-85 of the antipodal project).
* ``rotated_open_cube`` -- the same open cube under a seeded uniform random rotation, 1e5 uniform queries in
  [-1.5, 1.5]^3 and a seeded unit x0 (the small CPU-runnable configuration).
* ``open_icosphere`` -- an icosphere at subdivision level 6 (81,920 triangles) with a 30 degree spherical cap
  removed, seeded Gaussian vertex noise, and a 256^3 query grid over its bounding box scaled by 1.2 (the
  single-large-open-mesh configuration).
* ``noisy_torus`` / ``two_tori`` / ``bezier_patches`` -- inputs of the batched, robust and parametric
  configurations.
"""

from __future__ import annotations

import math

import numpy as np

# --------------------------------------------------------------------------------------------------------------
# reference fixtures
# --------------------------------------------------------------------------------------------------------------

CUBE_VERTS = np.array(
    [[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [-0.5, 0.5, -0.5], [0.5, 0.5, -0.5],
     [-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [-0.5, 0.5, 0.5], [0.5, 0.5, 0.5]], dtype=np.float64)

CUBE_IDX_CLOSED = np.array(
    [0, 2, 1, 1, 2, 3,  # -Z
     4, 5, 6, 6, 5, 7,  # +Z
     0, 4, 2, 2, 4, 6,  # -X
     1, 3, 5, 5, 3, 7,  # +X
     0, 1, 4, 4, 1, 5,  # -Y
     2, 6, 3, 3, 6, 7],  # +Y
    dtype=np.int32)

CUBE_IDX_OPEN_Y = CUBE_IDX_CLOSED[:30].copy()


def cube_open_y_boundary(dtype=np.float64) -> np.ndarray:
    """Open boundary of the +Y-removed cube in the reference fixtures' orientation: v6->v2, v7->v6, v3->v7, v2->v3."""
    v = CUBE_VERTS
    segs = [(v[6], v[2]), (v[7], v[6]), (v[3], v[7]), (v[2], v[3])]
    return np.array([np.concatenate([a, b, [1.0]]) for a, b in segs], dtype=dtype)


def unit_x0(dtype=np.float64) -> np.ndarray:
    """normalize(0.31, 0.57, 0.76), the reference tests' antipodal direction, rounded in ``dtype``."""
    v = np.array([0.31, 0.57, 0.76], dtype=dtype)
    return (v / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])).astype(dtype)


SAMPLE_POINTS = np.array(
    [[0, 0, 0], [0.1, -0.2, 0.3], [-0.4, 0.4, -0.4], [0.49, 0, 0],
     [2, 0, 0], [-2, -2, -2], [0, 1.5, 0], [1, 1, 1]], dtype=np.float64)


# --------------------------------------------------------------------------------------------------------------
# helpers
# --------------------------------------------------------------------------------------------------------------

def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform (Haar) random rotation from a normalised Gaussian quaternion."""
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def random_unit(rng: np.random.Generator) -> np.ndarray:
    v = rng.standard_normal(3)
    return v / np.linalg.norm(v)


def boundary_segments(verts: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """Open boundary as (n, 7) [pos0, pos1, weight] rows: net +-1 per undirected edge, positive weight,
    sorted by (lo, hi) vertex index.  Same rule as build_boundary_segments (src/antipodal/math/common.hh:123-174
    of the antipodal project), vectorised."""
    tri = np.asarray(idx, np.int64).reshape(-1, 3)
    u = tri.reshape(-1)
    v = np.roll(tri, -1, axis=1).reshape(-1)
    lo, hi = np.minimum(u, v), np.maximum(u, v)
    sign = np.where(u < v, 1, -1)
    key = lo * (1 << 32) + hi
    uniq, inv = np.unique(key, return_inverse=True)
    net = np.zeros(len(uniq), np.int64)
    np.add.at(net, inv, sign)
    keep = net != 0
    k, n = uniq[keep], net[keep]
    a, b = k >> 32, k & 0xFFFFFFFF
    p0 = np.where((n > 0)[:, None], verts[a], verts[b])
    p1 = np.where((n > 0)[:, None], verts[b], verts[a])
    return np.concatenate([p0, p1, np.abs(n)[:, None].astype(verts.dtype)], axis=1)


def grid_queries(lo: np.ndarray, hi: np.ndarray, n: int, scale: float = 1.2, dtype=np.float64) -> np.ndarray:
    """n^3 grid (x fastest) spanning the box [lo, hi] scaled by ``scale`` about its centre."""
    c, h = (lo + hi) / 2, (hi - lo) / 2 * scale
    ax = [np.linspace(c[k] - h[k], c[k] + h[k], n) for k in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(dtype)


# --------------------------------------------------------------------------------------------------------------
# configuration builders
# --------------------------------------------------------------------------------------------------------------

def rotated_open_cube(seed: int = 0, n_queries: int = 100_000, dtype=np.float64):
    """Unit cube (2 triangles per face) with the +Y face removed, under a seeded uniform rotation.
    Returns (verts, idx, boundary, queries, x0)."""
    rng = np.random.default_rng(seed)
    R = random_rotation(rng)
    verts = CUBE_VERTS @ R.T
    bnd = cube_open_y_boundary()
    bnd[:, 0:3] = bnd[:, 0:3] @ R.T
    bnd[:, 3:6] = bnd[:, 3:6] @ R.T
    q = rng.uniform(-1.5, 1.5, size=(n_queries, 3))
    x0 = random_unit(rng)
    return verts.astype(dtype), CUBE_IDX_OPEN_Y.copy(), bnd.astype(dtype), q.astype(dtype), x0.astype(dtype)


def icosphere(level: int):
    """Unit icosphere: the 20-face icosahedron, each level splitting every face into 4 at the normalised edge
    midpoints.  Faces are oriented outward.  Returns (verts float64 (V,3), faces int64 (F,3))."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * (1 << 32) + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq >> 32, uniq & 0xFFFFFFFF
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = len(v) + inv.reshape(3, -1).T  # (F, 3): midpoints of edges 01, 12, 20
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m[:, 0], m[:, 2]], 1),
            np.stack([f[:, 1], m[:, 1], m[:, 0]], 1),
            np.stack([f[:, 2], m[:, 2], m[:, 1]], 1),
            m])
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = np.einsum("ij,ij->i", n, v[f].mean(1)) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def _compact(verts: np.ndarray, faces: np.ndarray):
    used = np.unique(faces)
    remap = np.full(len(verts), -1, np.int64)
    remap[used] = np.arange(len(used))
    return verts[used], remap[faces]


def open_icosphere(seed: int = 0, level: int = 6, cap_deg: float = 30.0, sigma: float = 1e-3, grid: int = 256,
                   dtype=np.float64):
    """Icosphere at ``level`` with the triangles whose centroid lies within ``cap_deg`` of +z removed, seeded
    Gaussian vertex noise of std ``sigma``, and a grid^3 query grid over the bounding box scaled by 1.2.
    Returns (verts, idx int32 (3F,), boundary (S,7), queries (grid^3,3), x0)."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(level)
    c = v[f].mean(1)
    keep = c[:, 2] / np.linalg.norm(c, axis=1) <= math.cos(math.radians(cap_deg))
    v, f = _compact(v, f[keep])
    v = v + rng.normal(0.0, sigma, size=v.shape)
    idx = f.reshape(-1).astype(np.int32)
    bnd = boundary_segments(v, idx)
    q = grid_queries(v.min(0), v.max(0), grid, 1.2, dtype) if grid > 0 else np.zeros((0, 3), dtype)
    x0 = random_unit(rng)
    return v.astype(dtype), idx, bnd.astype(dtype), q, x0.astype(dtype)


def torus(n_major: int, n_minor: int, R: float = 1.0, r: float = 0.3):
    """Closed torus around +z, n_major x n_minor quads split into outward-facing triangles."""
    i, j = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    u = 2 * np.pi * i / n_major
    w = 2 * np.pi * j / n_minor
    verts = np.stack([(R + r * np.cos(w)) * np.cos(u), (R + r * np.cos(w)) * np.sin(u), r * np.sin(w)], -1)
    verts = verts.reshape(-1, 3)
    a = i * n_minor + j
    b = ((i + 1) % n_major) * n_minor + j
    c = ((i + 1) % n_major) * n_minor + (j + 1) % n_minor
    d = i * n_minor + (j + 1) % n_minor
    faces = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    n = np.cross(verts[faces[:, 1]] - verts[faces[:, 0]], verts[faces[:, 2]] - verts[faces[:, 0]])
    cen = verts[faces].mean(1)
    ring = np.stack([np.cos(np.arctan2(cen[:, 1], cen[:, 0])), np.sin(np.arctan2(cen[:, 1], cen[:, 0])),
                     np.zeros(len(cen))], -1) * R
    flip = np.einsum("ij,ij->i", n, cen - ring) < 0
    faces[flip] = faces[flip][:, [0, 2, 1]]
    return verts, faces


def punch_holes(verts: np.ndarray, faces: np.ndarray, n_holes: int, rng: np.random.Generator,
                radius_frac: float = 0.08):
    """Remove the triangles whose centroid lies within a random radius of ``n_holes`` random surface points."""
    cen = verts[faces].mean(1)
    ext = np.linalg.norm(verts.max(0) - verts.min(0))
    keep = np.ones(len(faces), bool)
    for _ in range(n_holes):
        c = cen[rng.integers(len(cen))]
        rad = radius_frac * ext * rng.uniform(0.3, 1.0) / max(1.0, math.sqrt(n_holes) / 2)
        keep &= np.linalg.norm(cen - c, axis=1) > rad
    return _compact(verts, faces[keep])


def noisy_mesh(kind: str, n_tris: int, n_holes: int, rng: np.random.Generator, sigma_rel: float = 1e-3):
    """A noisy icosphere or torus with about ``n_tris`` triangles and ``n_holes`` holes."""
    if kind == "icosphere":
        level = max(1, int(round(math.log(max(n_tris, 80) / 20.0, 4))))
        v, f = icosphere(level)
    else:
        m = max(8, int(math.sqrt(n_tris / 2.0 * 3.33)))
        v, f = torus(m, max(3, int(m / 3.33)))
    v, f = punch_holes(v, f, n_holes, rng)
    v = v + rng.normal(0.0, sigma_rel, size=v.shape)
    return v, f.reshape(-1).astype(np.int32)


def two_tori(seed: int = 0, n_tris: int = 1_000_000, n_holes: int = 20, n_queries: int = 10_000_000,
             dtype=np.float64):
    """Two interpenetrating perturbed tori (self-intersecting union, ``n_tris`` triangles in total) with
    ``n_holes`` holes.  Half the queries are uniform in the bounding box, half are offset from seeded surface
    points along the face normal by a log-uniform distance in [1e-9, 1e-3].
    Returns (verts, idx, boundary, queries)."""
    rng = np.random.default_rng(seed)
    per = n_tris // 2
    m = max(8, int(math.sqrt(per / 2.0 * 3.33)))
    n = max(3, int(m / 3.33))
    va, fa = torus(m, n)
    vb, fb = torus(m, n)
    R = random_rotation(rng)
    vb = vb @ R.T + np.array([0.6, 0.2, 0.1])
    v = np.concatenate([va, vb])
    f = np.concatenate([fa, fb + len(va)])
    v = v + rng.normal(0.0, 1e-4, size=v.shape)
    v, f = punch_holes(v, f, n_holes, rng, radius_frac=0.03)
    idx = f.reshape(-1).astype(np.int32)
    bnd = boundary_segments(v, idx)
    half = n_queries // 2
    lo, hi = v.min(0), v.max(0)
    q_uni = rng.uniform(lo, hi, size=(half, 3))
    t = rng.integers(len(f), size=n_queries - half)
    bary = rng.dirichlet([1, 1, 1], size=len(t))
    tri = v[f[t]]
    p = np.einsum("ij,ijk->ik", bary, tri)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = 10 ** rng.uniform(-9, -3, size=len(t)) * rng.choice([-1.0, 1.0], size=len(t))
    q = np.concatenate([q_uni, p + d[:, None] * nrm])
    return v.astype(dtype), idx, bnd.astype(dtype), q.astype(dtype)


def bezier_patches(seed: int = 0, n_patches: int = 256, n_queries: int = 1_000_000, near_frac: float = 0.3,
                   near_dist: float = 1e-3, return_patches: bool = False):
    """``n_patches`` bicubic Bezier patches with control points ~N(0,1); each patch contributes its 4 boundary
    cubics, oriented counter-clockwise in (u, v) so the patch lies on their left.  ``near_frac`` of the queries
    lie within ``near_dist`` of a boundary curve, the rest are uniform in the control points' bounding box.
    Returns (curves (4*n_patches, 12), queries (n,3), x0), and with ``return_patches`` also the patches
    (n_patches, 4, 4, 3) = P[patch][v][u]."""
    rng = np.random.default_rng(seed)
    P = rng.standard_normal((n_patches, 4, 4, 3))
    curves = []
    for k in range(n_patches):
        g = P[k]
        curves.append(g[0, :, :])          # v = 0, u: 0 -> 1
        curves.append(g[:, 3, :])          # u = 1, v: 0 -> 1
        curves.append(g[3, ::-1, :])       # v = 1, u: 1 -> 0
        curves.append(g[::-1, 0, :])       # u = 0, v: 1 -> 0
    curves = np.stack(curves).reshape(-1, 12)
    n_near = int(round(near_frac * n_queries))
    lo, hi = P.reshape(-1, 3).min(0), P.reshape(-1, 3).max(0)
    q_far = rng.uniform(lo, hi, size=(n_queries - n_near, 3))
    ci = rng.integers(len(curves), size=n_near)
    t = rng.uniform(0, 1, size=n_near)
    c = curves[ci].reshape(-1, 4, 3)
    u = 1 - t
    pts = (u ** 3)[:, None] * c[:, 0] + (3 * u * u * t)[:, None] * c[:, 1] + (3 * u * t * t)[:, None] * c[:, 2] \
        + (t ** 3)[:, None] * c[:, 3]
    off = rng.standard_normal((n_near, 3))
    off *= (near_dist * rng.uniform(0, 1, size=n_near) / np.linalg.norm(off, axis=1))[:, None]
    q = np.concatenate([q_far, pts + off])
    q = q[rng.permutation(len(q))]
    x0 = random_unit(rng)
    if return_patches:
        return curves, q, x0, P
    return curves, q, x0


def bezier_patch_boundary(patches: np.ndarray) -> np.ndarray:
    """The 4 boundary cubics of each bicubic patch (n, 4, 4, 3) = P[v][u], counter-clockwise in (u, v) so the patch
    lies on their left, as (4 n, 12) rows of control points."""
    out = []
    for g in np.asarray(patches, np.float64).reshape(-1, 4, 4, 3):
        out += [g[0, :, :], g[:, 3, :], g[3, ::-1, :], g[::-1, 0, :]]
    return np.stack(out).reshape(-1, 12)


def bezier_cube(inflate: float = 0.3) -> np.ndarray:
    """A closed surface of 6 bicubic patches: the faces of the cube [-1, 1]^3, each a 4 x 4 control grid oriented
    outward (S_u x S_v along the outward normal), every control point p then scaled by 1 + inflate (sqrt(3)/|p| - 1),
    which keeps the corners and bulges the faces.  The scaling is a function of the point alone, so neighbouring
    faces keep sharing their edge curves and the surface stays closed.  Returns (6, 4, 4, 3) = P[face][v][u]."""
    axes = np.eye(3)
    faces = [(0, 1, 2), (0, 2, 1), (1, 2, 0), (1, 0, 2), (2, 0, 1), (2, 1, 0)]  # (normal axis, u axis, v axis)
    s = np.linspace(-1.0, 1.0, 4)
    out = []
    for sign in (1.0, -1.0):
        for n_ax, a_ax, b_ax in faces[::2] if sign > 0 else faces[1::2]:
            n, a, b = sign * axes[n_ax], axes[a_ax], axes[b_ax]
            if np.dot(np.cross(a, b), n) < 0:
                a, b = b, a
            g = n[None, None, :] + s[None, :, None] * a[None, None, :] + s[:, None, None] * b[None, None, :]
            out.append(g)
    P = np.stack(out)
    r = np.linalg.norm(P, axis=-1, keepdims=True)
    return P * ((1.0 + inflate * (np.sqrt(3.0) / r - 1.0)))
