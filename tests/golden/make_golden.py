"""Generates the golden fixtures in this directory from the antipodal reference itself.

Run in a checkout where the reference sources exist (the reference is compiled from its own headers into
oracle/_ref/libref_gwn.so by ``make -C oracle ref``):

    python tests/golden/make_golden.py

Every array is an output of the reference's own functions (eval_gwnr_mesh_batch*, NaiveIntersector,
build_boundary_segments, RobustMeshGwn through the fake Embree backend, the robust predicates, IntegratorGK15,
eval_gwnr_parametric_batch_fractional with the project's cubic Bezier curve) on seeded synthetic inputs.  The
tests compare the CPU restatement (oracle/liboracle.so) and the GPU path against these files on machines where
the reference is absent.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from antipodal_gb300 import synth  # noqa: E402
from oracle.oracle import Oracle, build, reference_src  # noqa: E402

POLICIES = ["int64_grid", "int128_grid", "exact_float"]


def robust_cases():
    """Meshes and queries of the reference's robust tests (test/test_gwn_mesh_robust.cc:109-430)."""
    cases = {}
    tri = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64)
    tri_i = np.array([0, 1, 2], np.int32)
    sweep = np.array([[100.0, 0.7 - 5e-7 + 1e-6 * i / 1000.0, 0.3] for i in range(1001)])
    near = np.array([[x, 0.3, 0.7 + dz] for x in (1e-8, -1e-8, 1e-10, -1e-10) for dz in (1e-9, -1e-9)])
    far = np.array([p for d in (10.0, 100.0, 300.0, 1e3, 5e3, 1e5, 1e9)
                    for p in ([0.5, d, 0.2], [d, 0.2, 0.2], [-d, 0.2, 0.2], [d, -d, d])])
    cases["triangle"] = (tri, tri_i, np.concatenate([sweep, near, far]))
    seen = np.array([[1, 0, 0], [0, 0, 0], [0, 1, 1]], np.float64)
    along = np.array([[x, off * sy, off * sz] for x in (1.5, 3.0, 10.0) for off in (1e-4, 1e-6, 1e-8, 1e-10, 1e-12)
                      for sy, sz in ((1.0, 0.0), (0.0, 1.0), (1.0, -1.0), (-1.0, 0.3))])
    cases["edge_along_ray"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 1]], np.float64), tri_i, along)
    v4 = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 1], [0.5, 1, 1]], np.float64)
    thru = np.array([[v[0] + d, v[1], v[2]] for v in v4 for d in (0.25, 1.0, 3.0, 17.0)])
    cases["vertex_on_ray"] = (v4, np.array([0, 1, 2, 1, 3, 2], np.int32), thru)
    a = [0, 0.4303914952519497, 0.64558724287792457]
    b = [1, 0.68425246596985911, 1.0263786989547887]
    c = [0.29999999999999999, 0.19952205828266512, 0.29928308742399767]
    d = [0.5, 0.83805533983482472, 0.25708300975223697]
    ys = [c[1] + (b[1] - c[1]) * (i / 200.0) for i in range(201)]
    wall = np.array([[5, y + off, 1.5 * y - off] for y in ys for off in (0.0, 3e-7, -3e-7)]
                    + [[5, 0.20194571032110109, 0.30291856548165164]])
    cases["tet_parallel_face"] = (np.array([a, b, c, d]), np.array([0, 1, 2, 0, 3, 1, 1, 3, 2, 2, 3, 0], np.int32),
                                  wall)
    rng = np.random.default_rng(11)
    cases["cube_closed"] = (synth.CUBE_VERTS, synth.CUBE_IDX_CLOSED,
                            np.concatenate([synth.SAMPLE_POINTS, rng.uniform(-1.5, 1.5, (200, 3))]))
    cases["cube_open"] = (synth.CUBE_VERTS, synth.CUBE_IDX_OPEN_Y,
                          np.concatenate([synth.SAMPLE_POINTS, rng.uniform(-1.5, 1.5, (200, 3))]))
    v, i, _, _, _ = synth.open_icosphere(seed=4, level=3, grid=0)
    cases["icosphere3_open"] = (v, i, rng.uniform(-1.3, 1.3, (300, 3)))
    return cases


def main():
    src = reference_src()
    if src is None:
        raise SystemExit("the reference sources are needed: set ANTIPODAL_REFERENCE_SRC to the reference's src/")
    build(reference_src=src)
    ref = Oracle(reference=True)
    out = {}

    # mesh path: reference fixtures, the rotated open cube, an icosphere sample
    for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
        for closed in (True, False):
            verts = synth.CUBE_VERTS.astype(dt)
            idx = synth.CUBE_IDX_CLOSED if closed else synth.CUBE_IDX_OPEN_Y
            bnd = np.zeros((0, 7), dt) if closed else synth.cube_open_y_boundary(dt)
            x0 = synth.unit_x0(dt)
            q = synth.SAMPLE_POINTS.astype(dt)
            key = f"cube_{'closed' if closed else 'open'}_{tag}"
            out[key + "_full"] = ref.full_naive(q, x0, verts, idx, bnd)
            out[key + "_int"] = ref.int_naive(q, x0, verts, idx)
        verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=0, n_queries=2000, dtype=dt)
        out[f"rcube_{tag}_full"] = ref.full_naive(q, x0, verts, idx, bnd)
        out[f"rcube_{tag}_frac"] = ref.frac_batch(q, x0, bnd)
        out[f"rcube_{tag}_int"] = ref.int_naive(q, x0, verts, idx)
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=0, grid=0)
    q = synth.grid_queries(verts.min(0), verts.max(0), 8, 1.2)
    out["ico_full"] = ref.full_naive(q, x0, verts, idx, bnd)
    out["ico_frac"] = ref.frac_batch(q, x0, bnd)
    out["ico_int"] = ref.int_naive(q, x0, verts, idx)
    bref = ref.boundary(verts, idx)
    out["ico_boundary_sorted"] = bref[np.lexsort(bref.T[::-1])]

    # VOS known answers of test/test_common.cc:26-121
    vos_in = np.array([[[0, 0, 1], [1, 0, 0], [1, 0, 0]], [[0, 0, 1], [0, 0, 1], [1, 0, 0]],
                       [[0, 0, 1], [1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 1, 0], [1, 0, 0]],
                       [[0, 0, -1], [1, 0, 0], [0, 1, 0]], [[0, 0, 1], [1.3, -0.4, 0.2], [-0.7, 1.1, 0.5]],
                       [[0, 0, 1], [9.1, -2.8, 1.4], [-0.007, 0.011, 0.005]]], np.float64)
    out["vos_in"] = vos_in
    out["vos_f64"] = np.array([ref.vos_half(*v) for v in vos_in])
    out["vos_f32"] = np.array([ref.vos_half(*v.astype(np.float32)) for v in vos_in], np.float32)

    # robust evaluator under every (scalar, policy)
    for name, (v, i, q) in robust_cases().items():
        bnd = synth.boundary_segments(v, i)
        for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
            for pol in POLICIES:
                g, c, f = ref.robust_eval(pol, v.astype(dt), i, bnd.astype(dt), q.astype(dt))
                out[f"robust_{name}_{tag}_{pol}_gwn"] = g
                out[f"robust_{name}_{tag}_{pol}_count"] = c
                out[f"robust_{name}_{tag}_{pol}_frac"] = f
        out[f"robust_{name}_verts"] = v
        out[f"robust_{name}_idx"] = i
        out[f"robust_{name}_queries"] = q

    # predicates on seeded vectors (the distributions of test/math/test_robust_predicates.cc)
    rng = np.random.default_rng(1234)
    q32 = rng.integers(-(1 << 20), 1 << 20, size=(4, 2000, 3)).astype(np.int32)
    out["pred_i32_in"] = q32
    rng = np.random.default_rng(42)
    q64 = rng.integers(-(1 << 50), 1 << 50, size=(4, 2000, 3)).astype(np.int64)
    es, num, ins = ref.predicates(1, *q64)
    out["pred_i64_in"], out["pred_i64_sign"], out["pred_i64_num"], out["pred_i64_inside"] = q64, es, num, ins
    rng = np.random.default_rng(99)
    base = rng.integers(-(1 << 50), 1 << 50, size=(2000, 3)).astype(np.int64)
    dirv = rng.integers(-1024, 1025, size=(2000, 3)).astype(np.int64)
    k = rng.integers(-1024, 1025, size=(2000, 1)).astype(np.int64)
    nudge = rng.integers(-1, 2, size=(2000, 1)).astype(np.int64)
    qq = base + k * dirv
    qq[:, 1:2] += nudge
    pts = np.stack([qq, base, base + dirv, base + 3 * dirv + 1]).astype(np.float64) * 2.0 ** -20
    pts[..., 0] = 0.0
    es, num, ins = ref.predicates(2, *pts)
    out["pred_f64_in"], out["pred_f64_sign"], out["pred_f64_num"], out["pred_f64_inside"] = pts, es, num, ins
    es, num, ins = ref.predicates(0, *q32)
    out["pred_i32_sign"], out["pred_i32_num"], out["pred_i32_inside"] = es, num, ins
    # the 50-bit integer vectors as exact doubles (times 2^-20) under exact_float: random triangles, about 8% of
    # the queries inside, so the weights are exercised as well
    pts = q64.astype(np.float64) * 2.0 ** -20
    es, num, ins = ref.predicates(2, *pts)
    out["pred_f64tri_in"], out["pred_f64tri_sign"], out["pred_f64tri_num"], out["pred_f64tri_inside"] = pts, es, num, ins
    # project_into_tri's weights on the same vectors
    for pol, tag in ((0, "i32"), (1, "i64"), (2, "f64"), (2, "f64tri")):
        out[f"pred_{tag}_weights"] = ref.predicate_weights(pol, *out[f"pred_{tag}_in"])

    # GK15 closed forms (test/math/test_integrate_gk15.cc:18-72)
    gk = [(0, 0.0, np.pi, 0, 10, 1e-10), (1, 0.0, 1.0, 0, 10, 1e-10), (2, 0.0, 1.0, 0, 10, 1e-12),
          (3, 0.0, 1.0, 3, 10, 1.0), (4, 0.0, 1.0, 0, 3, 0.0), (4, 0.0, 1.0, 0, 10, 1e-9), (0, 0.5, 0.5, 0, 10, 1e-6)]
    out["gk15_cases"] = np.array(gk, np.float64)
    out["gk15_out"] = np.array([ref.gk15_known(int(c[0]), c[1], c[2], int(c[3]), int(c[4]), c[5]) for c in gk])

    # parametric: 4 bicubic patches (16 boundary cubics), 64 queries, tol 1e-10
    curves, q, x0 = synth.bezier_patches(seed=3, n_patches=4, n_queries=64)
    out["param_curves"], out["param_queries"], out["param_x0"] = curves, q, x0
    out["param_out"] = ref.param_frac_bezier3(q, x0, curves, 0, 10, 1e-10)
    # and the line-curve cube of test/test_gwn_parametric.cc:184-204 as straight "cubics"
    b = synth.cube_open_y_boundary()
    lines = np.stack([np.concatenate([s[0:3], (2 * s[0:3] + s[3:6]) / 3, (s[0:3] + 2 * s[3:6]) / 3, s[3:6]]) for s in b])
    qc = np.random.default_rng(0xC0FFEE).uniform(-1.5, 1.5, (100, 3))
    out["param_lines_curves"], out["param_lines_queries"] = lines, qc
    out["param_lines_out"] = ref.param_frac_bezier3(qc, synth.unit_x0(), lines, 0, 10, 1e-6)
    out["param_lines_mesh_frac"] = ref.frac_batch(qc, synth.unit_x0(), b)

    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
