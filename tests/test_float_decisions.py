"""Soundness of the float pre-decision of a candidate leaf (certain_leaf in antipodal_gb300/csrc/hier.cuh, with the
margins margin_rotated and margin_permuted), on the CPU.

The integer terms decide most candidate triangles in float and give only the undecided ones to the exact test
(NaiveIntersector's FP64 Moller-Trumbore, or the robust evaluator's exact predicates), so the counts stay the exact
ones only if every decided leaf gets the exact answer.  Here the device's float arithmetic is restated in numpy
float32 -- the query rounded to float and rotated by the float frame, the corners projected in FP64 and rounded,
the edge functions, depths and bounds of certain_leaf -- over adversarial cases: queries within 1e-9..1e-2 of an
edge, of a vertex and of the triangle's plane, at scene scales 1e-3..1e3 and offsets up to 30 scene scales from the
origin.  Every decided case is compared with the crossing computed in exact rational arithmetic.  The margins are
worst-case bounds: on these cases they still decide correctly at 1/100 of their value, and at 0.3% of it (below
the rounding itself) the same cases give wrong decisions, which shows that the cases reach the rounding.
"""

import os
import re
from fractions import Fraction

import numpy as np

F32 = np.float32
HIER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "antipodal_gb300", "csrc",
                    "hier.cuh")


def device_margin_constants():
    """The constants of margin_rotated and margin_permuted as hier.cuh writes them, so this test checks the margins
    the kernels use: (q, s) with delta = q qmax + s scene_scale (rotated) and d with delta = d (qmax + scene_scale)
    (permuted), each multiplied by 8 into m8."""
    src = open(HIER).read()
    rot = re.search(r"margin_rotated\(float qmax, float scene_scale\)\s*\{\s*return 8\.0f \* fmaf\(([0-9.e+-]+)f, qmax, "
                    r"([0-9.e+-]+)f \* scene_scale\);", src)
    per = re.search(r"margin_permuted\(float qmax, float scene_scale\)\s*\{\s*return 8\.0f \* ([0-9.e+-]+)f \* "
                    r"\(qmax \+ scene_scale\);", src)
    assert rot and per, "margin functions not found in hier.cuh"
    return (float(rot.group(1)), float(rot.group(2))), float(per.group(1))


(ROT_Q, ROT_S), PERM_D = device_margin_constants()


def ray_frame(d):
    """The frame of hier.cuh's ray_frame (lbvh.cu): rows e1, e2, e3 = d / |d|, in the same float64 operations."""
    nn = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    z = d / nn
    m = 0
    for k in (1, 2):
        if abs(z[k]) < abs(z[m]):
            m = k
    a = np.zeros(3)
    a[m] = 1.0
    x = np.array([a[1] * z[2] - a[2] * z[1], a[2] * z[0] - a[0] * z[2], a[0] * z[1] - a[1] * z[0]])
    x = x / np.sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2])
    y = np.array([z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]])
    return np.stack([x, y, z])


def project_query(rf, p):
    """float(p) rotated by the float frame rf, each product and sum rounded to float32 (vectorised over queries)."""
    o = p.astype(F32)
    uvw = [((rf[r, 0] * o[:, 0]) + (rf[r, 1] * o[:, 1])) + (rf[r, 2] * o[:, 2]) for r in range(3)]
    return uvw, np.max(np.abs(o), axis=1)


def project_corners(rd, tri):
    """Corners projected with the FP64 frame and rounded once (k_leaves in lbvh.cu); tri: (n, 3 vertices, 3)."""
    out = []
    for r in range(3):
        c = (rd[r, 0] * tri[:, :, 0] + rd[r, 1] * tri[:, :, 1]) + rd[r, 2] * tri[:, :, 2]
        out.append(c.astype(F32))
    return out  # u, v, w: (n, 3) each


def margin_rotated(qmax, scene):
    return F32(8.0) * (F32(ROT_Q) * qmax + F32(ROT_S) * scene)


def margin_permuted(qmax, scene):
    return F32(8.0) * F32(PERM_D) * (qmax + scene)


def may_hit(pu, pv, u, v, m8):
    """may_hit of hier.cuh in float32, vectorised: False only if the point is certainly outside the projected
    triangle (one edge function beyond +margin and another beyond -margin); such a leaf is skipped."""
    pu, pv = pu.astype(F32), pv.astype(F32)
    pos = np.zeros(len(u), bool)
    neg = np.zeros(len(u), bool)
    for k in range(3):
        k1 = (k + 1) % 3
        du, dv = pu[:, k1] - pu[:, k], pv[:, k1] - pv[:, k]
        ru, rv = u - pu[:, k], v - pv[:, k]
        ek = du * rv - dv * ru
        m = m8 * (((np.abs(du) + np.abs(dv)) + np.abs(ru)) + np.abs(rv))
        pos |= ek > m
        neg |= ek < -m
    return ~(pos & neg)


def certain_leaf(pu, pv, pw, u, v, w, m8):
    """certain_leaf of hier.cuh in float32, vectorised: 1 / -1 (crosses, with that orientation), 0 (does not),
    2 (undecided)."""
    pu, pv, pw = pu.astype(F32), pv.astype(F32), pw.astype(F32)
    dw = [pw[:, k] - w for k in range(3)]
    e, err = [], []
    pos = np.ones(len(u), bool)
    neg = np.ones(len(u), bool)
    for k in range(3):
        k1 = (k + 1) % 3
        du, dv = pu[:, k1] - pu[:, k], pv[:, k1] - pv[:, k]
        ru, rv = u - pu[:, k], v - pv[:, k]
        sabs = ((np.abs(du) + np.abs(dv)) + np.abs(ru)) + np.abs(rv)
        ek = du * rv - dv * ru
        e.append(ek)
        err.append(F32(0.375) * m8 * sabs)
        pos &= ek > m8 * sabs
        neg &= ek < -m8 * sabs
    out = np.full(len(u), 2, np.int8)
    inside = pos | neg
    E = (e[0] + e[1]) + e[2]
    errE = (err[0] + err[1]) + err[2]
    N = (e[1] * dw[0] + e[2] * dw[1]) + e[0] * dw[2]
    two_delta = F32(0.25) * m8
    errN = ((err[1] * np.abs(dw[0]) + err[2] * np.abs(dw[1])) + err[0] * np.abs(dw[2])) + two_delta * (
        (np.abs(e[0]) + np.abs(e[1])) + np.abs(e[2]))
    aE = np.abs(E)
    ok = inside & (aE > F32(2.0) * errE)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        depth = N / E
        bound = F32(2.0) * (errN + np.abs(depth) * errE) / (aE - errE)
    front = ok & (depth > bound)
    behind = ok & (depth < -bound)
    out[front] = np.where(pos[front], 1, -1)
    out[behind] = 0
    return out


def float_decision(pu, pv, pw, u, v, w, m8):
    """What the integer kernels take from float arithmetic for a candidate leaf: 0 when may_hit rejects it, else
    certain_leaf's answer (2: the exact test decides)."""
    out = certain_leaf(pu, pv, pw, u, v, w, m8)
    out[~may_hit(pu, pv, u, v, m8)] = 0
    return out


def exact_crossing(p, d, a, b, c):
    """The signed crossing of the ray p + t d (t > 0) with triangle abc in exact rational arithmetic: sign of the
    normal along the ray when the ray meets the open triangle, else 0 (no case here lies on an edge or the plane)."""
    P = [Fraction(float(x)) for x in p]
    D = [Fraction(float(x)) for x in d]
    A, B, C = ([Fraction(float(x)) for x in v] for v in (a, b, c))
    e1 = [B[i] - A[i] for i in range(3)]
    e2 = [C[i] - A[i] for i in range(3)]
    s = [P[i] - A[i] for i in range(3)]

    def cross(x, y):
        return [x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]]

    def dot(x, y):
        return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]

    h = cross(D, e2)
    det = dot(e1, h)
    if det == 0:
        return 0
    beta = dot(s, h) / det
    qv = cross(s, e1)
    gamma = dot(D, qv) / det
    t = dot(e2, qv) / det
    if beta > 0 and gamma > 0 and beta + gamma < 1 and t > 0:
        ng_d = dot(cross(e1, e2), D)
        return 1 if ng_d > 0 else -1
    return 0


def make_cases(rng, n, permuted):
    """Triangles and queries near their edges, vertices and planes (and uniform ones), with ray directions."""
    scale = 10.0 ** rng.uniform(-3, 3, n)
    centre = rng.normal(size=(n, 3)) * scale[:, None] * rng.choice([0.0, 1.0, 30.0], n)[:, None]
    tri = centre[:, None, :] + rng.normal(size=(n, 3, 3)) * scale[:, None, None]
    if permuted:
        d = np.tile(np.array([-1.0, 0.0, 0.0]), (n, 1))
    else:
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
    kind = rng.integers(0, 4, n)
    bary = rng.dirichlet([1, 1, 1], n)
    inner = np.einsum("nk,nkj->nj", bary, tri)
    off = 10.0 ** rng.uniform(-9, -2, n) * scale * rng.choice([-1.0, 1.0], n)
    k0 = rng.integers(0, 3, n)
    a = tri[np.arange(n), k0]
    b = tri[np.arange(n), (k0 + 1) % 3]
    t = rng.uniform(0.05, 0.95, n)
    on_edge = a + t[:, None] * (b - a)
    normal = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    edge_dir = np.cross(normal, b - a)
    edge_dir /= np.linalg.norm(edge_dir, axis=1)[:, None]
    near_vertex = a + rng.normal(size=(n, 3)) * off[:, None]
    depth = rng.uniform(0.1, 3.0, n) * scale
    p = np.where((kind == 0)[:, None], inner - depth[:, None] * d,                      # in front of the interior
        np.where((kind == 1)[:, None], on_edge + off[:, None] * edge_dir - depth[:, None] * d,  # near an edge
        np.where((kind == 2)[:, None], near_vertex - depth[:, None] * d,                 # near a vertex
                 inner + off[:, None] * d)))                                             # near the plane
    return tri, p, d


def run(permuted, margin_scale=1.0, n=6000, seed=0):
    rng = np.random.default_rng(seed + (7 if permuted else 0))
    tri, p, d = make_cases(rng, n, permuted)
    decided, wrong = 0, 0
    for i0 in range(0, n, 500):
        sl = slice(i0, min(n, i0 + 500))
        dec = np.empty(sl.stop - sl.start, np.int8)
        for j, i in enumerate(range(sl.start, sl.stop)):
            rd = ray_frame(d[i])
            rf = rd.astype(F32)
            (u, v, w), qmax = project_query(rf, p[i:i + 1])
            cu, cv, cw = project_corners(rd, tri[i:i + 1])
            scene = np.max(np.abs(tri[i].astype(F32)))
            m = margin_permuted(qmax, scene) if permuted else margin_rotated(qmax, scene)
            dec[j] = float_decision(cu, cv, cw, u, v, w, F32(margin_scale) * m)[0]
        for j, i in enumerate(range(sl.start, sl.stop)):
            if dec[j] == 2:
                continue
            decided += 1
            if int(dec[j]) != exact_crossing(p[i], d[i], tri[i, 0], tri[i, 1], tri[i, 2]):
                wrong += 1
    return decided, wrong


def test_margins_cover_their_derivation():
    # the lower bounds the margins are derived from (hier.cuh): rotated frame 7 sqrt(3) eps of qmax for the query
    # and 4 eps sqrt(3) of (qmax + scene_scale) for the edge functions' rounding; permuted frame 4 eps of (qmax +
    # scene_scale)
    eps = 2.0 ** -24
    assert ROT_Q >= 7 * np.sqrt(3) * eps and ROT_Q >= 4 * np.sqrt(3) * eps
    assert ROT_S >= 4 * np.sqrt(3) * eps and ROT_S >= np.sqrt(3) * eps
    assert PERM_D >= 4 * eps


def test_permuted_frame_matches_the_exact_order():
    # the robust evaluator's frame for the -x ray is (z, y, -x): its float coordinates are the roundings alone
    rd = ray_frame(np.array([-1.0, 0.0, 0.0]))
    assert np.array_equal(rd, np.array([[0.0, 0.0, 1.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0]]))


def test_rotated_frame_projection_error_bound():
    # a query rotated in float errs by at most 7 sqrt(3) eps qmax (eps = 2^-24), the query part of margin_rotated
    rng = np.random.default_rng(3)
    eps = 2.0 ** -24
    worst = 0.0
    for _ in range(200):
        d = rng.normal(size=3)
        rd = ray_frame(d)
        rf = rd.astype(F32)
        p = rng.normal(size=(2000, 3)) * 10.0 ** rng.uniform(-3, 3)
        (u, v, w), qmax = project_query(rf, p)
        exact = p @ rd.T
        err = np.max(np.abs(np.stack([u, v, w], 1).astype(np.float64) - exact), axis=1) / qmax.astype(np.float64)
        worst = max(worst, float(err.max()))
    assert worst <= 7 * np.sqrt(3) * eps
    assert worst > 0.5 * eps  # the errors are real, not all zero


def test_rotated_frame_decisions_are_exact():
    decided, wrong = run(permuted=False)
    assert wrong == 0
    assert decided > 2000


def test_permuted_frame_decisions_are_exact():
    decided, wrong = run(permuted=True)
    assert wrong == 0
    assert decided > 2000


def test_margin_below_the_rounding_decides_wrongly():
    # the cases reach the rounding: at 0.3% of the margins (below the float errors themselves) the emulation
    # decides some of them wrongly, in both frames
    _, wrong_rot = run(permuted=False, margin_scale=0.003)
    _, wrong_perm = run(permuted=True, margin_scale=0.003)
    assert wrong_rot > 0 and wrong_perm > 0
