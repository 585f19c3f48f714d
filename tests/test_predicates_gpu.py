"""The robust evaluator's exact predicates on the device, against the reference's own predicate vectors.

The reference pins edge_sign / atan2_num / project_into_tri and its 128-bit products in
test/math/test_robust_predicates.cc:18-191.  Here the same checks run on the device functions the robust kernels
call (csrc/robust.cuh), through agwn_robust_predicates and agwn_probe_i128_mul_sub:
  * the golden outputs of the reference itself on seeded vectors (pred_* in reference_golden.npz), bit for bit,
    weights included;
  * the known answers at 50-bit coordinates, where 64-bit determinants would overflow (:18-41), and the sliver
    whose weights must carry the triangle's exact sign (:171-191);
  * int32 and int64 coordinates agreeing on the 20-bit grid (:43-58);
  * 100,000 seeded exact_float cases on and one unit off collinear lines, whose signs must equal the exact integer
    ones, with more than 1,000 exactly collinear fallbacks (:136-169);
  * 128-bit products a*b - c*d on the int64 edge values and 100,000 seeded pairs, against Python's exact integers,
    with the conversion to double correctly rounded (:60-133).
"""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz")
DT = {0: np.int32, 1: np.int64, 2: np.float64}
I64_MIN, I64_MAX = -(1 << 63), (1 << 63) - 1


def device_predicates(gwn, disp, policy, q, q0, q1, q2):
    """edge_sign(q, q0, q1), atan2_num(q, q0, q1) as double, project_into_tri(q, q0, q1, q2) sign and weights."""
    lib = gwn.library()
    arrs = [np.ascontiguousarray(a, DT[policy]).reshape(-1, 3) for a in (q, q0, q1, q2)]
    n = len(arrs[0])
    es, num, ins = np.empty(n, np.int32), np.empty(n, np.float64), np.empty(n, np.int32)
    w = np.empty((n, 3), np.float64)
    rc = lib.agwn_robust_predicates(disp.handle, policy, *[a.ctypes.data for a in arrs], n, es.ctypes.data,
                                    num.ctypes.data, ins.ctypes.data, w.ctypes.data)
    assert rc == 0, lib.agwn_last_error_message()
    return es, num, ins, w


@pytest.mark.parametrize("policy,tag", [(0, "i32"), (1, "i64"), (2, "f64"), (2, "f64tri")])
def test_device_predicates_match_reference_golden(gwn, disp, policy, tag):
    g = np.load(GOLDEN)
    es, num, ins, w = device_predicates(gwn, disp, policy, *g[f"pred_{tag}_in"])
    assert np.array_equal(es, g[f"pred_{tag}_sign"])
    assert np.array_equal(num, g[f"pred_{tag}_num"])
    assert np.array_equal(ins, g[f"pred_{tag}_inside"])
    assert np.array_equal(w, g[f"pred_{tag}_weights"])


def test_device_predicates_known_answers_at_50_bits(gwn, disp):
    a = 1 << 50
    q0, q1, q2 = (0, 0, 0), (0, a, a - 2), (0, 0, a)
    rows = [((0, a // 2, a // 2 - 1), "on"), ((0, a // 2, a // 2), "above"), ((0, a // 2, a // 2 - 2), "below"),
            ((0, 1, 1), "inside"), ((0, -1, 1), "outside")]
    q = np.array([r for r, _ in rows])
    n = len(rows)
    es, num, ins, _ = device_predicates(gwn, disp, 1, q, [q0] * n, [q1] * n, [q2] * n)
    assert num[0] == 0 and es[0] == -1 and -es[0] == 1  # on the edge: the perturbation decides
    assert num[1] == -float(a) and es[1] == 1
    assert num[2] == float(a) and es[2] == -1
    assert ins[3] != 0 and ins[4] == 0


def test_device_exact_float_sliver_weights_carry_the_sign(gwn, disp):
    b, t = 2.0 ** 28, 2.0 ** -21
    q0, q1, q2 = (0, b, b), (0, b + 2, b + 1), (0, b + 4, b + 2 + 2 * t)
    q = [(0, b + 3, b + 1.5 + 1.25 * t), (0, b + 3, b + 1.5 + 0.75 * t)]  # strictly inside; just outside q1q2
    _, _, ins, w = device_predicates(gwn, disp, 2, q, [q0] * 2, [q1] * 2, [q2] * 2)
    assert ins[0] != 0
    assert np.all(w[0] * ins[0] > 0)
    assert ins[1] == 0


def test_device_int32_and_int64_agree_on_the_20_bit_grid(gwn, disp):
    rng = np.random.default_rng(1234)
    pts = rng.integers(-(1 << 20), (1 << 20) + 1, size=(4, 10_000, 3))
    r32 = device_predicates(gwn, disp, 0, *pts.astype(np.int32))
    r64 = device_predicates(gwn, disp, 1, *pts.astype(np.int64))
    for x, y in zip(r32, r64):
        assert np.array_equal(x, y)


def exact_edge_det(q, q0, q1):
    """(q - q0) x (q1 - q0) in (y, z) with the reference's orientation, in Python's exact integers."""
    o = lambda a, k: a[:, k].astype(object)  # noqa: E731
    return (o(q, 1) - o(q0, 1)) * (o(q0, 2) - o(q1, 2)) + (o(q, 2) - o(q0, 2)) * (o(q1, 1) - o(q0, 1))


def test_device_exact_float_signs_match_exact_integers(gwn, disp, oracle):
    rng = np.random.default_rng(99)
    n = 100_000
    big = lambda *s: rng.integers(-(1 << 50), (1 << 50) + 1, size=s)  # noqa: E731
    small = lambda *s: rng.integers(-1024, 1025, size=s)  # noqa: E731
    zero = np.zeros((n, 1), np.int64)
    q0 = np.hstack([zero, big(n, 2)])
    d = np.hstack([zero, small(n, 2)])
    q1 = q0 + d
    q = q0 + small(n, 1) * d
    q[:, 1] += rng.integers(-1, 2, size=n)  # on the line through q0, q1, or one unit off it
    far = np.arange(n) % 4 == 0
    q[far] = np.hstack([zero[far], small(int(far.sum()), 2)])  # a small query far from a big edge
    q2 = q0 + np.hstack([zero, small(n, 2)])
    ref_es, ref_num, _, _ = device_predicates(gwn, disp, 1, q, q0, q1, q2)
    scale = 2.0 ** -20
    got_es, got_num, _, _ = device_predicates(gwn, disp, 2, *(a.astype(np.float64) * scale for a in (q, q0, q1, q2)))
    assert np.array_equal(got_es, ref_es)
    assert np.array_equal(got_num > 0, ref_num > 0)
    assert np.array_equal(got_num == 0, ref_num == 0)
    det = exact_edge_det(q, q0, q1)
    sign = np.array([(x > 0) - (x < 0) for x in det])
    fallbacks = int(np.sum(sign == 0))
    assert fallbacks > 1000  # the exactly collinear case really was exercised
    nz = sign != 0
    assert np.array_equal(ref_es[nz], sign[nz])  # the exact determinant decides where it is not zero
    # and the CPU restatement (pinned to the reference's golden vectors) agrees on every case
    o_es, o_num, _ = oracle.predicates(2, *(a.astype(np.float64) * scale for a in (q, q0, q1, q2)))
    assert np.array_equal(o_es, got_es) and np.array_equal(o_num, got_num)


def test_device_int128_products_are_exact(gwn, disp):
    lib = gwn.library()
    edge = [0, 1, -1, 2, -2, I64_MIN, I64_MIN + 1, I64_MAX, I64_MAX - 1, 1 << 32, -(1 << 32)]
    ab = [(x, y) for x in edge for y in edge]
    rng = np.random.default_rng(42)
    m = 100_000
    first = np.array([x for x, _ in ab], np.int64)
    second = np.array([y for _, y in ab], np.int64)
    ones, zeros = np.ones(len(ab), np.int64), np.zeros(len(ab), np.int64)
    rand = lambda: rng.integers(I64_MIN // 2, I64_MAX // 2, m, dtype=np.int64)  # noqa: E731
    a = np.concatenate([first, zeros, rand()])
    b = np.concatenate([second, zeros, rand()])
    c = np.concatenate([ones, first, rand()])
    d = np.concatenate([ones, second, rand()])
    a, b, c, d = (np.ascontiguousarray(x, np.int64) for x in (a, b, c, d))
    n = len(a)
    lo, hi, dbl = np.empty(n, np.uint64), np.empty(n, np.int64), np.empty(n, np.float64)
    rc = lib.agwn_probe_i128_mul_sub(disp.handle, a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n,
                                     lo.ctypes.data, hi.ctypes.data, dbl.ctypes.data)
    assert rc == 0, lib.agwn_last_error_message()
    exact = a.astype(object) * b.astype(object) - c.astype(object) * d.astype(object)
    got = hi.astype(object) * (1 << 64) + lo.astype(object)
    assert all(x == y for x, y in zip(got, exact))
    # the conversion is correctly rounded: Python's int -> float rounds to nearest, ties to even
    assert np.array_equal(dbl, np.array([float(x) for x in exact]))
