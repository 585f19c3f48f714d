"""The CPU restatement of the Bezier-patch intersector (oracle/gwn_oracle.cc, orc_patch_count_bezier3x3_f64), checked
without a GPU against what pins it down, since the reference has no parametric intersector of its own:

* a fine tessellation of the same patches counted by NaiveIntersector's rule (the oracle's restatement of
  src/antipodal/intersector/intersector.hh:55-100, itself pinned to the reference's golden outputs), on queries
  whose rays pass well clear of the patches' edges;
* a closed surface of patches: the integer term alone is the winding number (1 inside, 0 outside) for any ray, and
  the fractional term of its boundary curves, which cancel in pairs, is 0;
* open patches: fractional (the reference integrator's rule, pinned to golden outputs) + integer does not depend
  on x0, which holds only if the crossings are found and signed as the boundary's orientation requires;
* the degenerate cases are reported: a ray through a patch's corner, a query on a patch.
"""

import numpy as np

from antipodal_gb300 import synth


def tessellate(patches, t):
    """Every patch sampled on a (t + 1)^2 grid and split into 2 t^2 triangles with the orientation of S_u x S_v."""
    s = np.linspace(0.0, 1.0, t + 1)
    b = np.stack([(1 - s) ** 3, 3 * s * (1 - s) ** 2, 3 * s * s * (1 - s), s ** 3], 1)  # (t+1, 4)
    verts, idx = [], []
    for k, g in enumerate(np.asarray(patches).reshape(-1, 4, 4, 3)):
        pts = np.einsum("vi,uj,ijc->vuc", b, b, g).reshape(-1, 3)  # row v, column u
        base = k * (t + 1) ** 2
        iv, iu = np.meshgrid(np.arange(t), np.arange(t), indexing="ij")
        a = base + iv * (t + 1) + iu
        quad_b, quad_c, quad_d = a + 1, a + t + 2, a + t + 1  # (u+1, v), (u+1, v+1), (u, v+1)
        idx.append(np.stack([a, quad_b, quad_c, a, quad_c, quad_d], -1).reshape(-1))
        verts.append(pts)
    return np.concatenate(verts), np.concatenate(idx).astype(np.int32)


def ray_clear_of_edges(q, x0, patches, t, clearance):
    """Queries whose ray, seen along x0, passes farther than `clearance` from every patch edge."""
    z = x0 / np.linalg.norm(x0)
    e1 = np.cross(z, [1.0, 0.0, 0.0] if abs(z[0]) < 0.9 else [0.0, 1.0, 0.0])
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(z, e1)
    s = np.linspace(0.0, 1.0, t + 1)
    bez = np.stack([(1 - s) ** 3, 3 * s * (1 - s) ** 2, 3 * s * s * (1 - s), s ** 3], 1)
    curves = synth.bezier_patch_boundary(patches).reshape(-1, 4, 3)
    pts = np.einsum("si,cik->csk", bez, curves)  # polylines of the edges
    a, b = pts[:, :-1].reshape(-1, 3), pts[:, 1:].reshape(-1, 3)
    P = lambda x: np.stack([x @ e1, x @ e2], -1)  # noqa: E731
    qa, qb, qq = P(a), P(b), P(q)
    d = qb - qa
    ok = np.ones(len(q), bool)
    for i in range(len(q)):
        w = qq[i] - qa
        t_ = np.clip(np.einsum("ij,ij->i", w, d) / np.maximum(np.einsum("ij,ij->i", d, d), 1e-300), 0, 1)
        dist = np.linalg.norm(w - t_[:, None] * d, axis=1).min()
        ok[i] = dist > clearance
    return ok


def test_patch_oracle_matches_tessellated_naive_count(oracle):
    rng = np.random.default_rng(7)
    patches = rng.standard_normal((4, 4, 4, 3))
    verts, idx = tessellate(patches, 128)
    lo, hi = patches.reshape(-1, 3).min(0), patches.reshape(-1, 3).max(0)
    q = rng.uniform(lo, hi, size=(1000, 3))
    checked = 0
    for x0 in (synth.random_unit(rng), synth.random_unit(rng)):
        ok = ray_clear_of_edges(q, x0, patches, 64, 2e-3)
        exact, deg = oracle.patch_count_bezier3x3(q, x0, patches, degenerate=True)
        assert not deg.any()
        naive = oracle.int_naive(q, x0, verts, idx)
        assert np.array_equal(exact[ok], naive[ok]), np.flatnonzero((exact != naive) & ok)[:10]
        assert np.count_nonzero(exact[ok]) > 50  # the rays do cross the patches
        checked += int(ok.sum())
    assert checked > 1800


def test_patch_oracle_on_a_closed_surface(oracle):
    patches = synth.bezier_cube(0.3)
    rng = np.random.default_rng(3)
    q = rng.uniform(-2.0, 2.0, size=(3000, 3))
    inside, outside = np.all(np.abs(q) < 0.99, axis=1), np.linalg.norm(q, axis=1) > 1.8
    counts = [oracle.patch_count_bezier3x3(q, synth.random_unit(rng), patches) for _ in range(3)]
    for c in counts:
        assert set(np.unique(c)) <= {0, 1}
        assert np.all(c[inside] == 1) and np.all(c[outside] == 0)
        assert np.array_equal(c, counts[0])  # the winding number, whatever the ray
    curves = synth.bezier_patch_boundary(patches)
    frac = oracle.param_frac_bezier3(q[:200], synth.unit_x0(), curves, 0, 10, 1e-10)
    assert np.max(np.abs(frac)) < 1e-12


def test_patch_oracle_full_gwn_does_not_depend_on_x0(oracle):
    rng = np.random.default_rng(11)
    patches = rng.standard_normal((8, 4, 4, 3))
    curves = synth.bezier_patch_boundary(patches)
    lo, hi = patches.reshape(-1, 3).min(0), patches.reshape(-1, 3).max(0)
    q = rng.uniform(lo, hi, size=(400, 3))
    gwn = []
    for x0 in (synth.random_unit(rng), synth.random_unit(rng), synth.random_unit(rng)):
        frac = oracle.param_frac_bezier3(q, x0, curves, 0, 12, 1e-11)
        gwn.append(frac + oracle.patch_count_bezier3x3(q, x0, patches))
    for g in gwn[1:]:
        d = np.abs(g - gwn[0])
        assert np.median(d) < 1e-10
        assert np.mean(d < 1e-6) > 0.99, np.sort(d)[-10:]  # away from the surface and its edges


def test_patch_oracle_reports_degenerate_rays(oracle):
    """A flat unit square patch in z = 0, normal +z.  Rays along +z from below: through the interior they count +1,
    from above they miss; a ray through the patch's corner or along its edge, and a query on the patch, are
    degenerate and reported."""
    s = np.arange(4) / 3.0
    flat = np.zeros((1, 4, 4, 3))
    flat[0, :, :, 0] = s[None, :]  # u along x
    flat[0, :, :, 1] = s[:, None]  # v along y
    x0 = np.array([0.0, 0.0, 1.0])
    q = np.array([[0.3, 0.6, -1.0], [0.3, 0.6, 1.0], [2.0, 0.5, -1.0], [0.0, 0.0, -1.0], [1.0, 0.4, -1.0],
                  [0.5, 0.5, 0.0]])
    c, deg = oracle.patch_count_bezier3x3(q, x0, flat, degenerate=True)
    assert list(c[:3]) == [1, 0, 0]
    assert list(deg[:3] > 0) == [False, False, False]
    assert np.all(deg[3:] > 0)
    # the opposite direction flips the sign of the crossing seen from above
    c2 = oracle.patch_count_bezier3x3(q[:3], -x0, flat)
    assert list(c2) == [0, -1, 0]
