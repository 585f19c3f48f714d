"""RobustMeshGwn over an axis-aligned grid with the rasterized integer term: every cell must equal the per-point
evaluator at the same point, bit for bit (counts, fractional term and GWN), under every policy and both scalar
types -- including a grid whose points lie exactly on the mesh's faces, edges and vertices -- and the CPU oracle
(the reference's RobustMeshGwn rule) at the grid points: counts bit for bit, values within the golden tests'
tolerance."""

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu
POLICIES = ["int64_grid", "int128_grid", "exact_float"]


def cases():
    # the open unit cube on a grid through its faces, edges and vertices (x = -0.5, 0, 0.5 are grid lines)
    yield "cube ties", synth.CUBE_VERTS, synth.CUBE_IDX_OPEN_Y, (-1.0, -1.0, -1.0), (0.25, 0.25, 0.25), (9, 9, 9)
    rng = np.random.default_rng(5)
    v, i = synth.noisy_mesh("torus", 6000, 6, rng)
    lo, hi = v.min(0) - 0.1, v.max(0) + 0.1
    yield "torus", v, i, tuple(lo), tuple((hi - lo) / np.array([37, 23, 19])), (38, 24, 20)
    v, i = synth.noisy_mesh("icosphere", 3000, 3, rng)
    yield "icosphere, slab", v, i, (-1.3, -0.2, -1.25), (0.07, 0.11, 0.05), (40, 1, 51)


@pytest.mark.parametrize("pol", POLICIES)
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_grid_equals_pointwise(gwn, disp, pol, dt):
    for name, v, i, start, spacing, shape in cases():
        b = synth.boundary_segments(v, i)
        r = gwn.CudaRobustMeshGwn(disp, v.astype(dt), i, b.astype(dt), precision=pol)
        cells = int(np.prod(shape))
        og, cg, fg = np.empty(cells, dt), np.empty(cells, np.int32), np.empty(cells, dt)
        r.evaluate_grid(start, spacing, shape, og, cg, fg)
        pts = r.grid_points(start, spacing, shape, dt)
        op, cp, fp = np.empty(cells, dt), np.empty(cells, np.int32), np.empty(cells, dt)
        r.evaluate(pts, op, cp, fp)
        assert np.array_equal(cg, cp), (name, pol, int(np.sum(cg != cp)))
        assert np.array_equal(fg, fp), (name, pol)
        assert np.array_equal(og, op), (name, pol)
        r.close()


@pytest.mark.parametrize("pol", POLICIES)
@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-12), (np.float32, 1e-6)])
def test_grid_matches_oracle(gwn, disp, oracle, pol, dt, tol):
    rng = np.random.default_rng(19)
    for name, v, i, start, spacing, shape in cases():
        b = synth.boundary_segments(v, i)
        r = gwn.CudaRobustMeshGwn(disp, v.astype(dt), i, b.astype(dt), precision=pol)
        cells = int(np.prod(shape))
        og, cg, fg = np.empty(cells, dt), np.empty(cells, np.int32), np.empty(cells, dt)
        r.evaluate_grid(start, spacing, shape, og, cg, fg)
        pts = r.grid_points(start, spacing, shape, dt)
        pick = np.arange(cells) if cells <= 1000 else np.sort(rng.choice(cells, size=1000, replace=False))
        gw, rc, rf = oracle.robust_eval(pol, v.astype(dt), i, b.astype(dt), pts[pick])
        assert np.array_equal(cg[pick], rc), (name, pol, int(np.sum(cg[pick] != rc)))
        assert np.max(np.abs(fg[pick].astype(np.float64) - rf.astype(np.float64))) <= tol, (name, pol)
        assert np.max(np.abs(og[pick].astype(np.float64) - gw.astype(np.float64))) <= tol, (name, pol)
        r.close()


def test_grid_mixed_mode_and_errors(gwn, disp, oracle):
    v, i = synth.noisy_mesh("torus", 4000, 5, np.random.default_rng(9))
    b = synth.boundary_segments(v, i)
    r = gwn.CudaRobustMeshGwn(disp, v.astype(np.float32), i, b.astype(np.float32), precision="int64_grid")
    start, spacing, shape = (-1.5, -1.5, -0.6), (0.05, 0.06, 0.07), (61, 51, 18)
    disp.set_robust_precision("mixed")
    try:
        og = r.evaluate_grid(start, spacing, shape)
        op = np.empty_like(og)
        pts = r.grid_points(start, spacing, shape, np.float32)
        r.evaluate(pts, op)
        assert np.array_equal(og, op)
        # against the oracle's FP64 rule: within the 1e-7 term bound plus two float ulps of the value
        pick = np.sort(np.random.default_rng(3).choice(len(og), size=1500, replace=False))
        gw, _, _ = oracle.robust_eval("int64_grid", v.astype(np.float32), i, b.astype(np.float32), pts[pick])
        ref = gw.astype(np.float64)
        assert np.all(np.abs(og[pick].astype(np.float64) - ref) <= 1e-7 + 2 * 2.0 ** -23 * np.maximum(1, np.abs(ref)))
    finally:
        disp.set_robust_precision("exact")
    with pytest.raises(gwn.GwnError):
        r.evaluate_grid(start, (0.1, -0.1, 0.1), (4, 4, 4))
    with pytest.raises(ValueError):
        r.evaluate_grid(start, spacing, (4, 4, 4), out=np.empty(10, np.float32))
    assert r.evaluate_grid(start, spacing, (0, 4, 4)).shape == (0,)
    r.close()
