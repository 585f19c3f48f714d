"""Parity of the device parametric fractional GWN (adaptive GK15 over cubic Bezier curves) with the reference.

The golden fixtures are outputs of the reference's own eval_gwnr_parametric_batch_fractional with IntegratorGK15
(test/test_gwn_parametric.cc's setting: straight-line cube at tol 1e-6, and bicubic patches at tol 1e-10).  The
device integrator does the reference's IEEE operations in the reference's order, so values must agree bit for bit;
the tree it builds (leaves, deepest level) must equal the oracle's for every (query, curve) pair.
"""

import os

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def run(gwn, disp, q, x0, curves, cfg, **kw):
    out = np.empty(len(q), np.float64)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, out, x0, curves, cfg, **kw)
    return out


def patches(seed, n_patches, n_queries):
    curves, q, x0 = synth.bezier_patches(seed=seed, n_patches=n_patches, n_queries=n_queries)
    return curves, q, x0


def test_param_bezier_golden_bit_exact(gwn, disp, golden):
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    got = run(gwn, disp, golden["param_queries"], golden["param_x0"], golden["param_curves"], cfg)
    ref = golden["param_out"]
    assert np.array_equal(got, ref), f"max |diff| {np.abs(got - ref).max():.3e}"


def test_param_lines_golden(gwn, disp, golden):
    cfg = gwn.IntegrateConfig(0, 10, 1e-6)
    got = run(gwn, disp, golden["param_lines_queries"], synth.unit_x0(), golden["param_lines_curves"], cfg)
    assert np.array_equal(got, golden["param_lines_out"]), np.abs(got - golden["param_lines_out"]).max()
    # straight "cubics" integrate the same fractional term as the polygon boundary of the mesh path
    np.testing.assert_allclose(got, golden["param_lines_mesh_frac"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("tol,min_depth,max_depth", [(1e-10, 0, 10), (1e-6, 2, 8), (1e-12, 0, 12)])
def test_param_matches_oracle_with_tree_stats(gwn, disp, oracle, tol, min_depth, max_depth):
    curves, q, x0 = patches(3, 6, 300)
    cfg = gwn.IntegrateConfig(min_depth, max_depth, tol)
    st = np.empty((len(q), len(curves)), np.uint32)
    nodes = np.empty(len(q), np.int32)
    got = run(gwn, disp, q, x0, curves, cfg, pair_stats=st, nodes_per_query=nodes)
    ref, leaves, depth = oracle.param_frac_bezier3(q, x0, curves, min_depth, max_depth, tol, stats=True)
    assert np.array_equal(got, ref), f"max |diff| {np.abs(got - ref).max():.3e}"
    lv, dmin, dmax = gwn.unpack_pair_stats(st)
    assert np.array_equal(lv, leaves)
    assert np.array_equal(dmax, depth)
    assert (dmin <= dmax).all() and (dmin >= min_depth).all()
    # a binary tree with L leaves has L - 1 internal panels, all evaluated by the plain method
    assert np.array_equal(nodes, (2 * leaves - 1).sum(axis=1))


def test_param_start_depth_below_shallowest_leaf_is_bit_identical(gwn, disp):
    curves, q, x0 = patches(5, 4, 256)
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    st = np.empty((len(q), len(curves)), np.uint32)
    nodes = np.empty(len(q), np.int32)
    plain = run(gwn, disp, q, x0, curves, cfg, pair_stats=st, nodes_per_query=nodes)
    lv, dmin, _ = gwn.unpack_pair_stats(st)
    rng = np.random.default_rng(0)
    start = (dmin - rng.integers(0, 2, size=dmin.shape)).clip(0).astype(np.uint8)
    nodes2 = np.empty(len(q), np.int32)
    st2 = np.empty_like(st)
    got = run(gwn, disp, q, x0, curves, cfg, start_depth=start, pair_stats=st2, nodes_per_query=nodes2)
    assert np.array_equal(got, plain)
    assert np.array_equal(st2, st)
    # the panels above the start depth are skipped: 2^s - 1 per pair, exactly
    saved = ((1 << start.astype(np.int64)) - 1).sum(axis=1)
    assert np.array_equal(nodes, nodes2 + saved)


def test_param_start_depth_above_shallowest_leaf_refines_within_tolerance(gwn, disp):
    curves, q, x0 = patches(6, 4, 256)
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    st = np.empty((len(q), len(curves)), np.uint32)
    plain = run(gwn, disp, q, x0, curves, cfg, pair_stats=st)
    _, dmin, _ = gwn.unpack_pair_stats(st)
    start = np.minimum(dmin + 1, 10).astype(np.uint8)
    st2 = np.empty_like(st)
    got = run(gwn, disp, q, x0, curves, cfg, start_depth=start, pair_stats=st2)
    _, dmin2, _ = gwn.unpack_pair_stats(st2)
    assert (dmin2 >= start).all()
    # every leaf still passed the error test; the finer tree agrees with the plain one to the tolerance's order
    assert np.abs(got - plain).max() < 1e-9


def test_param_edge_cases(gwn, disp):
    curves, q, x0 = patches(7, 2, 40)
    cfg = gwn.IntegrateConfig(0, 10, 1e-8)
    # no curves -> zero; no queries -> nothing written
    out = run(gwn, disp, q, x0, np.zeros((0, 12)), cfg)
    assert (out == 0).all()
    run(gwn, disp, np.zeros((0, 3)), x0, curves, cfg)
    # max_depth 0 accepts the root everywhere: one panel per pair
    nodes = np.empty(len(q), np.int32)
    run(gwn, disp, q, x0, curves, gwn.IntegrateConfig(0, 0, 1e-30), nodes_per_query=nodes)
    assert (nodes == len(curves)).all()
    # ragged query counts across block boundaries agree with the full run
    full = run(gwn, disp, q, x0, curves, cfg)
    for m in (1, 7, 33):
        np.testing.assert_array_equal(run(gwn, disp, q[:m], x0, curves, cfg), full[:m])
    with pytest.raises(gwn.GwnError):
        run(gwn, disp, q, x0, curves, gwn.IntegrateConfig(0, 25, 1e-8))
    with pytest.raises(gwn.GwnError):
        run(gwn, disp, q, x0, curves, gwn.IntegrateConfig(0, 10, float("nan")))
    with pytest.raises(ValueError):
        run(gwn, disp, q, x0, curves, cfg, start_depth=np.zeros(3, np.uint8))


def test_param_more_curves_than_a_tile(gwn, disp, oracle):
    curves, q, x0 = patches(8, 300, 64)  # 1200 curves: two shared-memory tiles
    cfg = gwn.IntegrateConfig(0, 10, 1e-8)
    got = run(gwn, disp, q, x0, curves, cfg)
    ref = oracle.param_frac_bezier3(q, x0, curves, 0, 10, 1e-8)
    assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_param_device_tensors(gwn, disp):
    torch = pytest.importorskip("torch")
    curves, q, x0 = patches(9, 3, 100)
    cfg = gwn.IntegrateConfig(0, 10, 1e-9)
    host = run(gwn, disp, q, x0, curves, cfg)
    qd = torch.from_numpy(q).cuda()
    cd = torch.from_numpy(curves).cuda()
    out = torch.empty(len(q), dtype=torch.float64, device="cuda")
    gwn.eval_gwnr_parametric_batch_fractional(disp, qd, out, x0, cd, cfg)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)


@pytest.mark.parametrize("tol", [1e-10, 1e-6])
def test_param_double_float_form_agrees_with_plain(gwn, disp, tol):
    """The double-float (FP32-pipe) integrator: the same tree rule in ~44-bit arithmetic.  Its values stay within
    the integrator's own error scale of the plain FP64 ones, and nearly every pair builds the same tree."""
    curves, q, x0 = patches(41, 6, 400)
    cfg = gwn.IntegrateConfig(0, 10, tol)
    st_e = np.empty((len(q), len(curves)), np.uint32)
    exact = run(gwn, disp, q, x0, curves, cfg, pair_stats=st_e)
    disp.set_param_precision("mixed")
    try:
        st_m = np.empty_like(st_e)
        mixed = run(gwn, disp, q, x0, curves, cfg, pair_stats=st_m)
    finally:
        disp.set_param_precision("exact")
    # leaves forced at max_depth carry error estimates above tol, so no partition bound holds there: the bar is
    # the product's 1e-7 against FP64, with margin; typical pairs agree to ~1e-13
    d = np.abs(mixed - exact)
    assert d.max() <= 1e-8, d.max()
    assert np.median(d) <= 1e-12
    assert np.mean(st_m == st_e) > 0.99
    # on straight-line curves too (the golden line-curve cube)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz"))
    disp.set_param_precision("mixed")
    try:
        got = run(gwn, disp, g["param_lines_queries"], synth.unit_x0(), g["param_lines_curves"],
                  gwn.IntegrateConfig(0, 10, 1e-6))
    finally:
        disp.set_param_precision("exact")
    assert np.abs(got - g["param_lines_out"]).max() <= 1e-9


@pytest.mark.parametrize("scale", [0.5, 2.0])
def test_param_non_unit_x0(gwn, disp, oracle, scale):
    """x0 is used as given, unnormalised, as in the reference.  The plain form stays bit-exact with the oracle; the
    double-float form takes its general closed form (the short one holds for |x0| = 1 only) and stays within the
    same bounds as for a unit x0."""
    curves, q, x0 = patches(43, 4, 300)
    x0 = x0 * scale
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    exact = run(gwn, disp, q, x0, curves, cfg)
    assert np.array_equal(exact, oracle.param_frac_bezier3(q, x0, curves, 0, 10, 1e-10))
    disp.set_param_precision("mixed")
    try:
        mixed = run(gwn, disp, q, x0, curves, cfg)
    finally:
        disp.set_param_precision("exact")
    d = np.abs(mixed - exact)
    assert d.max() <= 1e-8, d.max()
    assert np.median(d) <= 1e-12
