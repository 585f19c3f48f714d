"""Pins the CPU oracle (oracle/gwn_oracle.cc) before it is trusted as the checker.

1. Against the golden fixtures in tests/golden/reference_golden.npz, which are outputs of the antipodal
   reference compiled from its own sources (tests/golden/make_golden.py).
2. Against the known answers of the reference's own test suite, restated here on the oracle
   (test/test_common.cc, test/test_gwn_mesh.cc, test/test_intersector.cc, test/test_gwn_mesh_robust.cc,
   test/math/test_robust_predicates.cc, test/math/test_integrate_gk15.cc, test/test_gwn_parametric.cc).
3. Against the reference itself (oracle/_ref) on fresh seeded inputs, where it was built.
"""

import os

import numpy as np
import pytest

from antipodal_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz")
POLICIES = ["int64_grid", "int128_grid", "exact_float"]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


# ---- 1. golden fixtures -----------------------------------------------------------------------------------------
@pytest.mark.parametrize("dt,tag", [(np.float64, "f64"), (np.float32, "f32")])
def test_mesh_golden(oracle, golden, dt, tag):
    tol = 1e-15 if dt == np.float64 else 1e-6
    for closed in (True, False):
        verts = synth.CUBE_VERTS.astype(dt)
        idx = synth.CUBE_IDX_CLOSED if closed else synth.CUBE_IDX_OPEN_Y
        bnd = np.zeros((0, 7), dt) if closed else synth.cube_open_y_boundary(dt)
        q = synth.SAMPLE_POINTS.astype(dt)
        key = f"cube_{'closed' if closed else 'open'}_{tag}"
        np.testing.assert_allclose(oracle.full_naive(q, synth.unit_x0(dt), verts, idx, bnd), golden[key + "_full"],
                                   rtol=0, atol=tol)
        assert np.array_equal(oracle.int_naive(q, synth.unit_x0(dt), verts, idx), golden[key + "_int"])
    verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=0, n_queries=2000, dtype=dt)
    np.testing.assert_allclose(oracle.full_naive(q, x0, verts, idx, bnd), golden[f"rcube_{tag}_full"], rtol=0, atol=tol)
    np.testing.assert_allclose(oracle.frac_batch(q, x0, bnd), golden[f"rcube_{tag}_frac"], rtol=0, atol=tol)
    assert np.array_equal(oracle.int_naive(q, x0, verts, idx), golden[f"rcube_{tag}_int"])


def test_icosphere_golden(oracle, golden):
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=0, grid=0)
    assert len(idx) // 3 == 76496 and len(bnd) == 212
    q = synth.grid_queries(verts.min(0), verts.max(0), 8, 1.2)
    np.testing.assert_allclose(oracle.full_naive(q, x0, verts, idx, bnd), golden["ico_full"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(oracle.frac_batch(q, x0, bnd), golden["ico_frac"], rtol=0, atol=1e-14)
    assert np.array_equal(oracle.int_naive(q, x0, verts, idx), golden["ico_int"])
    b = oracle.boundary(verts, idx)
    assert np.array_equal(b[np.lexsort(b.T[::-1])], golden["ico_boundary_sorted"])
    s = synth.boundary_segments(verts, idx)
    assert np.array_equal(s[np.lexsort(s.T[::-1])], golden["ico_boundary_sorted"])


def test_vos_golden(oracle, golden):
    for v, r64, r32 in zip(golden["vos_in"], golden["vos_f64"], golden["vos_f32"]):
        assert abs(oracle.vos_half(*v) - r64) <= 1e-15
        assert abs(oracle.vos_half(*v.astype(np.float32)) - r32) <= 1e-6


def test_robust_golden(oracle, golden):
    names = sorted({k.split("_f64_")[0][len("robust_"):] for k in golden.files if k.startswith("robust_") and "_f64_" in k})
    assert len(names) >= 7
    for name in names:
        v, i, q = golden[f"robust_{name}_verts"], golden[f"robust_{name}_idx"], golden[f"robust_{name}_queries"]
        bnd = synth.boundary_segments(v, i)
        for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
            tol = 1e-15 if dt == np.float64 else 1e-6
            for pol in POLICIES:
                g, c, f = oracle.robust_eval(pol, v.astype(dt), i, bnd.astype(dt), q.astype(dt))
                assert np.array_equal(c, golden[f"robust_{name}_{tag}_{pol}_count"]), (name, tag, pol)
                np.testing.assert_allclose(f, golden[f"robust_{name}_{tag}_{pol}_frac"], rtol=0, atol=tol)
                np.testing.assert_allclose(g, golden[f"robust_{name}_{tag}_{pol}_gwn"], rtol=0, atol=tol)


@pytest.mark.parametrize("policy,tag", [(0, "i32"), (1, "i64"), (2, "f64"), (2, "f64tri")])
def test_predicates_golden(oracle, golden, policy, tag):
    es, num, ins = oracle.predicates(policy, *golden[f"pred_{tag}_in"])
    assert np.array_equal(es, golden[f"pred_{tag}_sign"])
    assert np.array_equal(num, golden[f"pred_{tag}_num"])
    assert np.array_equal(ins, golden[f"pred_{tag}_inside"])
    assert np.array_equal(oracle.predicate_weights(policy, *golden[f"pred_{tag}_in"]), golden[f"pred_{tag}_weights"])


def test_gk15_golden(oracle, golden):
    for c, r in zip(golden["gk15_cases"], golden["gk15_out"]):
        got = oracle.gk15_known(int(c[0]), c[1], c[2], int(c[3]), int(c[4]), c[5])
        assert got[0] == pytest.approx(r[0], abs=1e-15)
        assert got[2] == r[2]


def test_parametric_golden(oracle, golden):
    got = oracle.param_frac_bezier3(golden["param_queries"], golden["param_x0"], golden["param_curves"], 0, 10, 1e-10)
    np.testing.assert_allclose(got, golden["param_out"], rtol=0, atol=1e-13)
    got = oracle.param_frac_bezier3(golden["param_lines_queries"], synth.unit_x0(), golden["param_lines_curves"], 0, 10,
                                    1e-6)
    np.testing.assert_allclose(got, golden["param_lines_out"], rtol=0, atol=1e-13)


# ---- 2. the reference's known answers ----------------------------------------------------------------------------
@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
def test_vos_known_answers(oracle, dt, tol):
    # test/test_common.cc:26-121
    x1, a, x, y = (np.array(v, dt) for v in ([0, 0, 1], [1, 0, 0], [1, 0, 0], [0, 1, 0]))
    assert abs(oracle.vos_half(x1, a, a)) <= tol
    assert abs(oracle.vos_half(x1, x1, a)) <= tol
    assert abs(oracle.vos_half(x1, a, x1)) <= tol
    assert abs(abs(oracle.vos_half(x1, x, y)) - np.pi / 4) <= tol
    assert abs(oracle.vos_half(x1, x, y) + oracle.vos_half(x1, y, x)) <= tol
    assert abs(oracle.vos_half(x1, x, y) + oracle.vos_half(-x1, x, y)) <= tol
    corners = np.array([[1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0]], dt)
    s = sum(oracle.vos_half(x1, corners[i], corners[(i + 1) % 4]) for i in range(4))
    assert abs(abs(s) - np.pi) <= 4 * tol
    v0, v1 = np.array([1.3, -0.4, 0.2], dt), np.array([-0.7, 1.1, 0.5], dt)
    base = oracle.vos_half(x1, v0, v1)
    assert abs(oracle.vos_half(x1, dt(7) * v0, dt(0.01) * v1) - base) <= tol * 10
    assert abs(oracle.vos_half(x1, dt(0.001) * v0, dt(1000) * v1) - base) <= tol * 10


@pytest.mark.parametrize("dt,rel", [(np.float64, 1e-9), (np.float32, 1e-4)])
def test_cube_matches_baseline(oracle, dt, rel):
    # test/test_gwn_mesh.cc:101-162
    for closed in (True, False):
        verts = synth.CUBE_VERTS.astype(dt)
        idx = synth.CUBE_IDX_CLOSED if closed else synth.CUBE_IDX_OPEN_Y
        bnd = np.zeros((0, 7), dt) if closed else synth.cube_open_y_boundary(dt)
        q = synth.SAMPLE_POINTS.astype(dt)
        got = oracle.full_naive(q, synth.unit_x0(dt), verts, idx, bnd)
        ref = oracle.gwn_baseline(q, verts, idx)
        assert np.all(np.abs(got - ref) <= rel * np.maximum(1, np.abs(ref)))


def test_intersector_known_counts(oracle):
    # test/test_intersector.cc:78-106
    q = np.array([[0, 0, 0], [0.1, -0.2, 0.3], [2, 0, 0], [-2, -2, -2]], np.float64)
    for d in ([0.31, 0.57, 0.76], [-0.6, 0.4, -0.69], [0.83, -0.21, 0.51]):
        for dt in (np.float64, np.float32):
            c = oracle.int_naive(q.astype(dt), np.array(d, dt), synth.CUBE_VERTS.astype(dt), synth.CUBE_IDX_CLOSED)
            assert c.tolist() == [1, 1, 0, 0]


def _robust(oracle, pol, v, i, q, dt=np.float64):
    return oracle.robust_eval(pol, np.asarray(v, dt), np.asarray(i, np.int32), synth.boundary_segments(
        np.asarray(v, np.float64), np.asarray(i, np.int32)).astype(dt), np.asarray(q, dt))


def test_robust_grazing_sweep_is_smooth(oracle):
    # test/test_gwn_mesh_robust.cc:224-287 (robust part): max jump between neighbours < 0.1
    v, i = [[0, 0, 0], [0, 1, 0], [0, 0, 1]], [0, 1, 2]
    q = np.array([[100.0, 0.7 - 5e-7 + 1e-6 * k / 1000.0, 0.3] for k in range(1001)])
    for pol in POLICIES:
        g, _, _ = _robust(oracle, pol, v, i, q)
        assert np.max(np.abs(np.diff(g))) < 0.1


def test_robust_accuracy_near_open_edge(oracle):
    # test/test_gwn_mesh_robust.cc:291-322
    v, i = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64), np.array([0, 1, 2], np.int32)
    q = np.array([[x, 0.3, 0.7 + dz] for x in (1e-8, -1e-8, 1e-10, -1e-10) for dz in (1e-9, -1e-9)])
    ref = oracle.gwn_baseline(q, v, i)
    err = {p: np.max(np.abs(_robust(oracle, p, v, i, q)[0] - ref)) for p in POLICIES}
    assert err["int128_grid"] < 1e-6 and err["exact_float"] < 1e-6 and err["int64_grid"] > 1e-2


def test_robust_edge_along_ray_and_vertex_on_ray(oracle):
    # test/test_gwn_mesh_robust.cc:326-369
    v, i = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 1]], np.float64), np.array([0, 1, 2], np.int32)
    q = np.array([[x, off * sy, off * sz] for x in (1.5, 3.0, 10.0) for off in (1e-4, 1e-6, 1e-8, 1e-10, 1e-12)
                  for sy, sz in ((1.0, 0.0), (0.0, 1.0), (1.0, -1.0), (-1.0, 0.3))])
    ref = oracle.gwn_baseline(q, v, i)
    for pol, tol in (("int64_grid", 1e-6), ("int128_grid", 1e-10), ("exact_float", 1e-10)):
        assert np.max(np.abs(_robust(oracle, pol, v, i, q)[0] - ref)) < tol
    v4 = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 1], [0.5, 1, 1]], np.float64)
    i4 = np.array([0, 1, 2, 1, 3, 2], np.int32)
    q = np.array([[p[0] + d, p[1], p[2]] for p in v4 for d in (0.25, 1.0, 3.0, 17.0)])
    ref = oracle.gwn_baseline(q, v4, i4)
    for pol in POLICIES:
        assert np.max(np.abs(_robust(oracle, pol, v4, i4, q)[0] - ref)) < 1e-6


def test_robust_far_queries(oracle):
    # test/test_gwn_mesh_robust.cc:374-395
    v, i = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64), np.array([0, 1, 2], np.int32)
    for pol in POLICIES:
        for d in (10.0, 100.0, 300.0, 1e3, 5e3, 1e5, 1e9):
            q = np.array([[0.5, d, 0.2], [d, 0.2, 0.2], [-d, 0.2, 0.2], [d, -d, d]])
            ref = oracle.gwn_baseline(q, v, i)
            near = 1e-6 if pol == "int64_grid" else 1e-12
            clamped = 1e-6 if pol != "exact_float" else 1e-12
            assert np.max(np.abs(_robust(oracle, pol, v, i, q)[0] - ref)) < (near if d <= 300 else clamped)


def test_robust_face_parallel_to_ray(oracle):
    # test/test_gwn_mesh_robust.cc:401-430: every count is 0
    a = [0, 0.4303914952519497, 0.64558724287792457]
    b = [1, 0.68425246596985911, 1.0263786989547887]
    c = [0.29999999999999999, 0.19952205828266512, 0.29928308742399767]
    d = [0.5, 0.83805533983482472, 0.25708300975223697]
    v = np.array([a, b, c, d])
    i = np.array([0, 1, 2, 0, 3, 1, 1, 3, 2, 2, 3, 0], np.int32)
    ys = [c[1] + (b[1] - c[1]) * (k / 200.0) for k in range(201)]
    q = np.array([[5, y + off, 1.5 * y - off] for y in ys for off in (0.0, 3e-7, -3e-7)]
                 + [[5, 0.20194571032110109, 0.30291856548165164]])
    for pol in POLICIES:
        _, cnt, _ = oracle.robust_eval(pol, v, i, np.zeros((0, 7)), q)
        assert np.all(cnt == 0)


def test_predicates_known_answers(oracle):
    # test/math/test_robust_predicates.cc:18-58
    A = 1 << 50
    q0, q1 = [0, 0, 0], [0, A, A - 2]
    es, num, _ = oracle.predicates(1, [[0, A // 2, A // 2 - 1]], [q0], [q1], [q0])
    assert num[0] == 0 and es[0] == -1
    es, num, _ = oracle.predicates(1, [[0, A // 2, A // 2], [0, A // 2, A // 2 - 2]], [q0, q0], [q1, q1], [q0, q0])
    assert num.tolist() == [-float(A), float(A)] and es.tolist() == [1, -1]
    _, _, ins = oracle.predicates(1, [[0, 1, 1], [0, -1, 1]], [q0, q0], [q1, q1], [[0, 0, A], [0, 0, A]])
    assert ins[0] != 0 and ins[1] == 0
    rng = np.random.default_rng(1234)
    pts = rng.integers(-(1 << 20), 1 << 20, size=(4, 10000, 3))
    e32 = oracle.predicates(0, *pts.astype(np.int32))
    e64 = oracle.predicates(1, *pts.astype(np.int64))
    for a, b in zip(e32, e64):
        assert np.array_equal(a, b)


def test_gk15_known_answers(oracle):
    # test/math/test_integrate_gk15.cc:18-72
    r, err, n = oracle.gk15_known(0, 0.0, np.pi, 0, 10, 1e-10)
    assert r == pytest.approx(2.0, rel=1e-12) and err >= 0 and n >= 1
    assert oracle.gk15_known(1, 0.0, 1.0, 0, 10, 1e-10)[0] == pytest.approx(1 / 3, rel=1e-14)
    assert oracle.gk15_known(2, 0.0, 1.0, 0, 10, 1e-12)[0] == pytest.approx(np.e - 1, rel=1e-12)
    assert oracle.gk15_known(3, 0.5, 0.5, 0, 10, 1e-6) == (0.0, 0.0, 0)
    r, _, n = oracle.gk15_known(3, 0.0, 1.0, 3, 10, 1.0)
    assert r == pytest.approx(0.5, rel=1e-14) and n >= 8


def test_parametric_lines_match_mesh(oracle):
    # test/test_gwn_parametric.cc:184-204: straight boundary curves reproduce the mesh fractional term
    b = synth.cube_open_y_boundary()
    lines = np.stack([np.concatenate([s[0:3], (2 * s[0:3] + s[3:6]) / 3, (s[0:3] + 2 * s[3:6]) / 3, s[3:6]]) for s in b])
    q = np.random.default_rng(0xC0FFEE).uniform(-1.5, 1.5, (100, 3))
    got = oracle.param_frac_bezier3(q, synth.unit_x0(), lines, 0, 10, 1e-6)
    ref = oracle.frac_batch(q, synth.unit_x0(), b)
    assert np.all(np.abs(got - ref) <= 1e-6 * np.maximum(1, np.abs(ref)))
    assert np.all(oracle.param_frac_bezier3(q[:16], synth.unit_x0(), np.zeros((0, 12))) == 0)


# ---- 3. the reference itself, fresh inputs ----------------------------------------------------------------------
def test_port_equals_reference_mesh(oracle, ref_oracle):
    for seed in range(3):
        for dt in (np.float64, np.float32):
            verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=100 + seed, n_queries=3000, dtype=dt)
            assert np.array_equal(oracle.full_naive(q, x0, verts, idx, bnd), ref_oracle.full_naive(q, x0, verts, idx, bnd))
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=7, level=4, grid=0)
    q = np.random.default_rng(7).uniform(-1.3, 1.3, (2000, 3))
    assert np.array_equal(oracle.full_naive(q, x0, verts, idx, bnd), ref_oracle.full_naive(q, x0, verts, idx, bnd))
    b1, b2 = oracle.boundary(verts, idx), ref_oracle.boundary(verts, idx)
    assert np.array_equal(b1[np.lexsort(b1.T[::-1])], b2[np.lexsort(b2.T[::-1])])


def test_port_equals_reference_robust(oracle, ref_oracle):
    verts, idx, _, _, _ = synth.open_icosphere(seed=8, level=3, grid=0)
    bnd = synth.boundary_segments(verts, idx)
    q = np.random.default_rng(8).uniform(-1.3, 1.3, (800, 3))
    for dt in (np.float64, np.float32):
        for pol in POLICIES:
            a = oracle.robust_eval(pol, verts.astype(dt), idx, bnd.astype(dt), q.astype(dt))
            b = ref_oracle.robust_eval(pol, verts.astype(dt), idx, bnd.astype(dt), q.astype(dt))
            for x, y in zip(a, b):
                assert np.array_equal(x, y), (dt, pol)


def test_port_equals_reference_parametric(oracle, ref_oracle):
    curves, q, x0 = synth.bezier_patches(seed=21, n_patches=3, n_queries=48)
    assert np.array_equal(oracle.param_frac_bezier3(q, x0, curves, 0, 10, 1e-10),
                          ref_oracle.param_frac_bezier3(q, x0, curves, 0, 10, 1e-10))
