"""The parametric integer term on the GPU: the Bezier-patch intersector (csrc/patch.cu) behind
eval_gwnr_parametric_batch_integer and eval_gwnr_parametric_batch (src/antipodal/gwn_parametric.hh:204-284).

The reference has no parametric intersector, so parity is with the CPU restatement of the same rule and method
(oracle/gwn_oracle.cc), which tests/test_patch.py pins against NaiveIntersector on a fine tessellation, a closed
surface and the x0-independence of the full GWN.  Here: device counts equal the oracle's, far from and near the
surface; the full GWN of a closed surface of patches is the winding number; the full GWN of open patches does not
depend on x0 and equals the oracle's fractional + integer terms.
"""

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu


def random_patches(seed, n):
    return np.random.default_rng(seed).standard_normal((n, 4, 4, 3))


def surface_points(patches, rng, n):
    """n points on random patches at random (u, v)."""
    k = rng.integers(0, len(patches), n)
    u, v = rng.uniform(0, 1, n), rng.uniform(0, 1, n)
    bern = lambda t: np.stack([(1 - t) ** 3, 3 * t * (1 - t) ** 2, 3 * t * t * (1 - t), t ** 3], -1)  # noqa: E731
    return np.einsum("nv,nu,nvuc->nc", bern(v), bern(u), patches[k])


def test_device_patch_counts_equal_the_oracle(gwn, disp, oracle):
    patches = random_patches(5, 64)
    rng = np.random.default_rng(6)
    lo, hi = patches.reshape(-1, 3).min(0), patches.reshape(-1, 3).max(0)
    q = rng.uniform(lo, hi, size=(3000, 3))
    isect = gwn.CudaBezierPatchIntersector(disp, patches)
    nonzero = 0
    for x0 in (synth.random_unit(rng), synth.random_unit(rng), synth.unit_x0(), np.array([0.0, 0.0, 1.0])):
        got, deg = np.empty(len(q), np.int32), np.empty(len(q), np.int32)
        gwn.eval_gwnr_parametric_batch_integer(disp, isect, q, got, x0, out_degenerate=deg)
        ref, ref_deg = oracle.patch_count_bezier3x3(q, x0, patches, degenerate=True)
        assert not deg.any() and not ref_deg.any()
        assert np.array_equal(got, ref), np.flatnonzero(got != ref)[:10]
        nonzero += int(np.count_nonzero(got))
    assert nonzero > 1000
    isect.close()


@pytest.mark.parametrize("offset", [1e-2, 1e-4, 1e-6, 1e-9])
def test_device_patch_counts_near_the_surface(gwn, disp, oracle, offset):
    """Queries at a small distance off the patches (float cannot decide their depth below ~1e-4: those pairs run in
    FP64) and rays at every angle to the surface, grazing ones included, where crossings pair up near folds."""
    patches = random_patches(9, 32)
    rng = np.random.default_rng(int(round(-np.log10(offset))))
    on = surface_points(patches, rng, 2000)
    d = rng.standard_normal((len(on), 3))
    q = on + offset * d / np.linalg.norm(d, axis=1, keepdims=True)
    isect = gwn.CudaBezierPatchIntersector(disp, patches)
    for x0 in (synth.random_unit(rng), synth.random_unit(rng)):
        got, deg = np.empty(len(q), np.int32), np.empty(len(q), np.int32)
        gwn.eval_gwnr_parametric_batch_integer(disp, isect, q, got, x0, out_degenerate=deg)
        ref, ref_deg = oracle.patch_count_bezier3x3(q, x0, patches, degenerate=True)
        # a query within about 2^-40 of the coordinates' scale of the surface (~5e-12 here, more along a grazing
        # ray) is degenerate: only the smallest offset reaches that, for about 1.5% of its queries
        clear = (deg == 0) & (ref_deg == 0)
        assert clear.all() if offset >= 1e-6 else clear.mean() > 0.95
        assert np.array_equal(got[clear], ref[clear]), np.flatnonzero((got != ref) & clear)[:10]
    isect.close()


def test_device_patch_reports_degenerate_rays(gwn, disp, oracle):
    """The flat square of tests/test_patch.py: interior hits count, a ray through a corner or along an edge and a
    query on the patch are reported as degenerate, as the oracle reports them."""
    s = np.arange(4) / 3.0
    flat = np.zeros((1, 4, 4, 3))
    flat[0, :, :, 0] = s[None, :]
    flat[0, :, :, 1] = s[:, None]
    x0 = np.array([0.0, 0.0, 1.0])
    q = np.array([[0.3, 0.6, -1.0], [0.3, 0.6, 1.0], [2.0, 0.5, -1.0], [0.0, 0.0, -1.0], [1.0, 0.4, -1.0],
                  [0.5, 0.5, 0.0]])
    isect = gwn.CudaBezierPatchIntersector(disp, flat)
    got, deg = np.empty(len(q), np.int32), np.empty(len(q), np.int32)
    gwn.eval_gwnr_parametric_batch_integer(disp, isect, q, got, x0, out_degenerate=deg)
    ref, ref_deg = oracle.patch_count_bezier3x3(q, x0, flat, degenerate=True)
    assert list(got[:3]) == [1, 0, 0] and not deg[:3].any()
    assert np.all(deg[3:] > 0) and np.array_equal(deg > 0, ref_deg > 0)
    isect.close()


@pytest.mark.parametrize("inflate", [0.0, 0.3])
def test_device_closed_patch_surface_is_the_winding_number(gwn, disp, inflate):
    patches = synth.bezier_cube(inflate)
    curves = synth.bezier_patch_boundary(patches)
    rng = np.random.default_rng(8)
    q = rng.uniform(-2.0, 2.0, size=(4000, 3))
    inside, outside = np.all(np.abs(q) < 0.99, axis=1), np.linalg.norm(q, axis=1) > 1.8
    isect = gwn.CudaBezierPatchIntersector(disp, patches)
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    first = None
    for x0 in (synth.random_unit(rng), synth.random_unit(rng)):
        out = np.empty(len(q))
        gwn.eval_gwnr_parametric_batch(disp, isect, q, out, x0, curves, cfg)
        assert np.max(np.abs(out - np.rint(out))) < 1e-9
        w = np.rint(out).astype(int)
        assert set(np.unique(w)) <= {0, 1}
        assert np.all(w[inside] == 1) and np.all(w[outside] == 0)
        if first is None:
            first = w
        assert np.array_equal(w, first)
    isect.close()


def test_device_full_parametric_gwn_is_independent_of_x0_and_equals_the_oracle(gwn, disp, oracle):
    patches = random_patches(11, 8)
    curves = synth.bezier_patch_boundary(patches)
    rng = np.random.default_rng(12)
    lo, hi = patches.reshape(-1, 3).min(0), patches.reshape(-1, 3).max(0)
    q = rng.uniform(lo, hi, size=(600, 3))
    isect = gwn.CudaBezierPatchIntersector(disp, patches)
    cfg = gwn.IntegrateConfig(0, 12, 1e-11)
    outs = []
    for x0 in (synth.random_unit(rng), synth.random_unit(rng), synth.random_unit(rng)):
        out = np.empty(len(q))
        gwn.eval_gwnr_parametric_batch(disp, isect, q, out, x0, curves, cfg)
        ref = oracle.param_frac_bezier3(q, x0, curves, 0, 12, 1e-11) + oracle.patch_count_bezier3x3(q, x0, patches)
        assert np.max(np.abs(out - ref)) <= 1e-12
        outs.append(out)
    for o in outs[1:]:
        d = np.abs(o - outs[0])
        assert np.median(d) < 1e-10
        assert np.mean(d < 1e-6) > 0.99, np.sort(d)[-10:]
    isect.close()


def test_patch_intersector_inputs_and_errors(gwn, disp, oracle):
    torch = pytest.importorskip("torch")
    patches = random_patches(2, 16)
    rng = np.random.default_rng(3)
    q = rng.uniform(-2, 2, size=(777, 3))
    x0 = synth.unit_x0()
    dev = torch.device("cuda:0")
    isect = gwn.CudaBezierPatchIntersector(disp, torch.from_numpy(patches).to(dev))
    ref = oracle.patch_count_bezier3x3(q, x0, patches)
    got = torch.full((len(q),), -99, dtype=torch.int32, device=dev)
    gwn.eval_gwnr_parametric_batch_integer(disp, isect, torch.from_numpy(q).to(dev), got, x0)
    disp.synchronize()
    assert np.array_equal(got.cpu().numpy(), ref)
    # the full GWN into a device tensor equals the host-array result
    curves = synth.bezier_patch_boundary(patches)
    cfg = gwn.IntegrateConfig(0, 10, 1e-8)
    out_d = torch.empty(len(q), dtype=torch.float64, device=dev)
    gwn.eval_gwnr_parametric_batch(disp, isect, torch.from_numpy(q).to(dev), out_d, x0, torch.from_numpy(curves).to(dev),
                                   cfg)
    out_h = np.empty(len(q))
    gwn.eval_gwnr_parametric_batch(disp, isect, q, out_h, x0, curves, cfg)
    disp.synchronize()
    assert np.array_equal(out_d.cpu().numpy(), out_h)
    # the work counters (with timing on): every pair past the box test blossoms at least its root cell
    disp.set_option(gwn._lib.OPT_TIMING, 1)
    disp.stats(reset=True)
    gwn.eval_gwnr_parametric_batch_integer(disp, isect, q, np.empty(len(q), np.int32), x0)
    st = disp.stats(reset=True)["patches"]
    disp.set_option(gwn._lib.OPT_TIMING, 0)
    assert 0 < st["pairs"] <= len(q) * len(patches)
    assert st["cells"] >= st["pairs"] and st["pieces"] > 0 and 0 <= st["fp64_pairs"] <= st["pairs"]
    # empty queries, no patches, a bad direction
    gwn.eval_gwnr_parametric_batch_integer(disp, isect, np.zeros((0, 3)), np.zeros(0, np.int32), x0)
    none = gwn.CudaBezierPatchIntersector(disp, np.zeros((0, 4, 4, 3)))
    c = np.full(len(q), 5, np.int32)
    gwn.eval_gwnr_parametric_batch_integer(disp, none, q, c, x0)
    assert not c.any()
    with pytest.raises(gwn.GwnError):
        gwn.eval_gwnr_parametric_batch_integer(disp, isect, q, c, np.zeros(3))
    none.close()
    isect.close()
