"""Parity of the device robust evaluator (RobustMeshGwn) with the reference and the oracle.

Golden fixtures are outputs of the reference's own RobustMeshGwn (compiled here with the project's fake Embree
backend) on the meshes and queries of test/test_gwn_mesh_robust.cc; counts must match bit for bit under every
(scalar, policy), the fractional term and the full GWN up to atan2's last bits (1e-12 double, 1e-6 float).
"""

import os

import numpy as np
import pytest

from antipodal_gb300 import _lib, synth

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz")
POLICIES = ["int64_grid", "int128_grid", "exact_float"]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def run(gwn, disp, pol, v, i, b, q):
    r = gwn.CudaRobustMeshGwn(disp, v, i, b, precision=pol)
    out = np.empty(len(q), q.dtype)
    cnt = np.empty(len(q), np.int32)
    fr = np.empty(len(q), q.dtype)
    r.evaluate(q, out, cnt, fr)
    r.close()
    return out, cnt, fr


@pytest.mark.parametrize("pol", POLICIES)
@pytest.mark.parametrize("dt,tag,tol", [(np.float64, "f64", 1e-12), (np.float32, "f32", 1e-6)])
def test_robust_matches_reference_golden(gwn, disp, golden, pol, dt, tag, tol):
    names = sorted({k.split("_f64_")[0][len("robust_"):] for k in golden.files if k.startswith("robust_") and "_f64_" in k})
    for name in names:
        v, i, q = golden[f"robust_{name}_verts"], golden[f"robust_{name}_idx"], golden[f"robust_{name}_queries"]
        b = synth.boundary_segments(v, i)
        g, c, f = run(gwn, disp, pol, v.astype(dt), i, b.astype(dt), q.astype(dt))
        assert np.array_equal(c, golden[f"robust_{name}_{tag}_{pol}_count"]), name
        np.testing.assert_allclose(f, golden[f"robust_{name}_{tag}_{pol}_frac"], rtol=0, atol=tol, err_msg=name)
        np.testing.assert_allclose(g, golden[f"robust_{name}_{tag}_{pol}_gwn"], rtol=0, atol=tol, err_msg=name)


@pytest.mark.parametrize("pol", POLICIES)
def test_robust_matches_oracle_on_noisy_open_mesh(gwn, disp, oracle, pol):
    # an open icosphere (level 4) with queries everywhere, including 1e-9 .. 1e-3 from the surface
    v, idx, b, _, _ = synth.open_icosphere(seed=11, level=4, grid=0)
    rng = np.random.default_rng(11)
    q_far = rng.uniform(-1.4, 1.4, size=(3000, 3))
    t = rng.integers(len(idx) // 3, size=2000)
    tri = v[idx.reshape(-1, 3)[t]]
    bary = rng.dirichlet([1, 1, 1], size=len(t))
    p = np.einsum("ij,ijk->ik", bary, tri)
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    d = 10 ** rng.uniform(-9, -3, size=len(t)) * rng.choice([-1.0, 1.0], size=len(t))
    q = np.concatenate([q_far, p + d[:, None] * n])
    g, c, f = run(gwn, disp, pol, v, idx, b, q)
    rg, rc, rf = oracle.robust_eval(pol, v, idx, b, q)
    assert np.array_equal(c, rc)
    assert np.max(np.abs(f - rf)) <= 1e-12
    assert np.max(np.abs(g - rg)) <= 1e-12


def test_robust_grazing_sweep_is_smooth(gwn, disp):
    # test/test_gwn_mesh_robust.cc:224-287: across a grazed edge the robust GWN does not jump
    v = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64)
    i = np.array([0, 1, 2], np.int32)
    q = np.array([[100.0, 0.7 - 5e-7 + 1e-6 * k / 1000.0, 0.3] for k in range(1001)])
    for pol in POLICIES:
        g, _, _ = run(gwn, disp, pol, v, i, synth.boundary_segments(v, i), q)
        assert np.max(np.abs(np.diff(g))) < 0.1


def test_robust_two_tori_small(gwn, disp, oracle):
    # a small version of the robust stress input: two interpenetrating perturbed tori with holes
    v, idx, b, q = synth.two_tori(seed=4, n_tris=20_000, n_holes=6, n_queries=6000)
    for pol in ("int128_grid", "exact_float"):
        g, c, f = run(gwn, disp, pol, v, idx, b, q)
        rg, rc, rf = oracle.robust_eval(pol, v, idx, b, q)
        assert np.array_equal(c, rc), pol
        assert np.max(np.abs(g - rg)) <= 1e-11, pol


def test_robust_empty_and_device_inputs(gwn, disp):
    torch = pytest.importorskip("torch")
    v, i = synth.CUBE_VERTS, synth.CUBE_IDX_CLOSED
    q = synth.SAMPLE_POINTS
    g, c, _ = run(gwn, disp, "exact_float", v, i, np.zeros((0, 7)), q)
    assert np.array_equal(c, np.rint(g).astype(np.int32))
    dev = torch.device("cuda:0")
    with gwn.CudaDispatcher(stream=torch.cuda.current_stream(dev), mixed_min_pairs=0) as d:
        r = gwn.CudaRobustMeshGwn(d, torch.from_numpy(v).to(dev), torch.from_numpy(i).to(dev),
                                  torch.zeros((0, 7), dtype=torch.float64, device=dev))
        out = torch.empty(len(q), dtype=torch.float64, device=dev)
        gwn.eval_gwnr_mesh_batch_robust(d, r, torch.from_numpy(q).to(dev), out)
        d.synchronize()
        assert np.array_equal(out.cpu().numpy(), g)


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-7), (np.float32, 2e-7)])
def test_robust_mixed_int64_grid_matches_exact(gwn, disp, dt, tol):
    """The FP32-pair form of the int64_grid fractional term: counts identical, fractional term within the bar."""
    rng = np.random.default_rng(17)
    for kind, ntri, holes in [("icosphere", 2000, 4), ("torus", 5000, 9)]:
        v, i = synth.noisy_mesh(kind, ntri, holes, rng)
        b = synth.boundary_segments(v, i)
        q = np.concatenate([synth.grid_queries(v.min(0), v.max(0), 24),
                            v[rng.integers(len(v), size=3000)] + rng.normal(0, 1e-4, (3000, 3))]).astype(dt)
        r = gwn.CudaRobustMeshGwn(disp, v.astype(dt), i, b.astype(dt), precision="int64_grid")
        outs = {}
        for mode in ("exact", "mixed"):
            disp.set_robust_precision(mode)
            o, c, f = np.empty(len(q), dt), np.empty(len(q), np.int32), np.empty(len(q), dt)
            r.evaluate(q, o, c, f)
            outs[mode] = (o, c, f)
        disp.set_robust_precision("exact")
        assert np.array_equal(outs["exact"][1], outs["mixed"][1])
        d = np.abs(outs["exact"][2].astype(np.float64) - outs["mixed"][2].astype(np.float64))
        assert d.max() <= tol, (kind, d.max())
        r.close()


def test_robust_mixed_batch_equals_per_mesh(gwn, disp):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(23)
    meshes, pos, outs, refs = [], [], [], []
    disp.set_robust_precision("mixed")
    for kind, ntri, holes, side in [("icosphere", 1500, 3, 20), ("torus", 2500, 6, 14), ("torus", 700, 2, 9)]:
        v, i = synth.noisy_mesh(kind, ntri, holes, rng)
        b = synth.boundary_segments(v, i)
        q = synth.grid_queries(v.min(0), v.max(0), side).astype(np.float32)
        r = gwn.CudaRobustMeshGwn(disp, v.astype(np.float32), i, b.astype(np.float32))
        ref = np.empty(len(q), np.float32)
        r.evaluate(q, ref)
        meshes.append(r)
        refs.append(ref)
        pos.append(torch.from_numpy(q).cuda())
        outs.append(torch.empty(len(q), dtype=torch.float32, device="cuda"))
    batch = gwn.CudaRobustBatch(disp, meshes, pos, outs)
    for cfg in [(128, 1, 256, 64), (256, 2, 512, 64)]:
        batch.set_config(*cfg)
        batch.run(graph=True)
        torch.cuda.synchronize()
        for o, ref in zip(outs, refs):
            assert np.array_equal(o.cpu().numpy(), ref)
    disp.set_robust_precision("exact")
    batch.close()
    for r in meshes:
        r.close()


def test_robust_mixed_exact_float_matches_exact(gwn, disp):
    """exact_float with double queries in mixed mode: the mesh functions' mixed kernel along -x, with the robust
    evaluator's FP64 rule (its exact branches) for the pairs it turns down.  Counts identical; fractional term and
    GWN within 1e-7 of the exact (FP64) form -- on grid points, on points 1e-9..1e-3 off the surface, and on points
    whose -x ray runs exactly through a boundary vertex (the reference's special branches)."""
    rng = np.random.default_rng(29)
    for kind, ntri, holes in [("torus", 6000, 7), ("icosphere", 3000, 3)]:
        v, i = synth.noisy_mesh(kind, ntri, holes, rng)
        b = synth.boundary_segments(v, i)
        tri = v[i.reshape(-1, 3)]
        pick = tri[rng.integers(len(tri), size=3000)]
        bary = rng.dirichlet([1, 1, 1], size=3000)
        n = np.cross(pick[:, 1] - pick[:, 0], pick[:, 2] - pick[:, 0])
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        off = (bary[:, :, None] * pick).sum(1) + n * (10.0 ** rng.uniform(-9, -3, 3000) * rng.choice([-1, 1], 3000))[:, None]
        on_ray = b[rng.integers(len(b), size=500), :3] + np.stack([rng.uniform(0.01, 2, 500), np.zeros(500),
                                                                   np.zeros(500)], axis=1)
        q = np.concatenate([synth.grid_queries(v.min(0), v.max(0), 20), off, on_ray]).astype(np.float64)
        r = gwn.CudaRobustMeshGwn(disp, v, i, b, precision="exact_float")
        outs = {}
        try:
            for mode in ("exact", "mixed"):
                disp.set_robust_precision(mode)
                o, c, f = np.empty(len(q)), np.empty(len(q), np.int32), np.empty(len(q))
                r.evaluate(q, o, c, f)
                o2 = np.empty(len(q))
                r.evaluate(q, o2)  # without the separate outputs: the other launch path
                assert np.array_equal(o, o2)
                outs[mode] = (o, c, f)
            # the mixed kernel's certified boundary groups (on by default) change no value
            disp.set_option(_lib.OPT_MIXED_CERTIFY, 0)
            o3 = np.empty(len(q))
            r.evaluate(q, o3)
            assert np.array_equal(o3, outs["mixed"][0])
        finally:
            disp.set_option(_lib.OPT_MIXED_CERTIFY, 1)
            disp.set_robust_precision("exact")
            r.close()
        assert np.array_equal(outs["exact"][1], outs["mixed"][1])
        for k in (0, 2):
            d = np.abs(outs["exact"][k] - outs["mixed"][k])
            assert d.max() <= 1e-7, (kind, k, d.max())


def test_robust_mixed_exact_float_chunked_equals_single_chunks(gwn, disp):
    """exact_float mixed over 2^21 or more queries runs counts and fractional term in chunks on two compute streams;
    the values must equal those of calls on single chunks (below 2^21, one stream) bit for bit, and the counts those
    of the separate-output path."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(41)
    v, i = synth.noisy_mesh("torus", 8000, 9, rng)
    b = synth.boundary_segments(v, i)
    q = synth.grid_queries(v.min(0), v.max(0), 129, 1.2)
    assert len(q) >= 1 << 21
    r = gwn.CudaRobustMeshGwn(disp, v, i, b, precision="exact_float")
    try:
        disp.set_robust_precision("mixed")
        qd = torch.from_numpy(q).cuda()
        out = torch.empty(len(q), dtype=torch.float64, device="cuda")
        r.evaluate(qd, out)
        disp.synchronize()
        for a, e in ((0, 1 << 20), (1 << 20, 1 << 21)):
            part = torch.empty(e - a, dtype=torch.float64, device="cuda")
            r.evaluate(qd[a:e].contiguous(), part)
            disp.synchronize()
            assert torch.equal(part, out[a:e]), a
        # the separate outputs (counts and fractional term) take the unchunked path: same values
        o, c, f = np.empty(len(q)), np.empty(len(q), np.int32), np.empty(len(q))
        r.evaluate(q, o, c, f)
        assert np.array_equal(o, out.cpu().numpy())
    finally:
        disp.set_robust_precision("exact")
        r.close()


def test_robust_mixed_exact_float_incoherent_order(gwn, disp):
    """exact_float mixed over 2^20 or more queries in random order runs on a spatially sorted copy (the mixed
    kernel then certifies far more boundary groups) and scatters the results back: values and counts equal those of
    the per-pair path on the given order bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(43)
    v, i = synth.noisy_mesh("torus", 6000, 7, rng)
    b = synth.boundary_segments(v, i)
    lo, hi = v.min(0), v.max(0)
    q = rng.uniform(lo - 0.1 * (hi - lo), hi + 0.1 * (hi - lo), size=((1 << 20) + 333, 3))
    r = gwn.CudaRobustMeshGwn(disp, v, i, b, precision="exact_float")
    try:
        disp.set_robust_precision("mixed")
        qd = torch.from_numpy(q).cuda()
        outs = {}
        for cert in (1, 0):
            disp.set_option(_lib.OPT_MIXED_CERTIFY, cert)
            o = torch.empty(len(q), dtype=torch.float64, device="cuda")
            c = torch.empty(len(q), dtype=torch.int32, device="cuda")
            r.evaluate(qd, o, c)
            f = np.empty(len(q))
            o2 = np.empty(len(q))
            r.evaluate(qd.cpu().numpy(), o2, None, f)  # host arrays with the separate fractional output
            outs[cert] = (o.cpu().numpy(), c.cpu().numpy(), o2, f)
        for k in range(4):
            assert np.array_equal(outs[1][k], outs[0][k]), k
        assert np.array_equal(outs[1][0], outs[1][2])
    finally:
        disp.set_option(_lib.OPT_MIXED_CERTIFY, 1)
        disp.set_robust_precision("exact")
        r.close()


@pytest.mark.parametrize("pol", ["int64_grid", "int128_grid", "exact_float"])
def test_robust_counts_cells_equal_the_walk(gwn, pol):
    """The robust counts with candidate leaves from the cell grid (default) and from the hierarchy walk (option 0):
    identical, on grid points, points on vertices and edges, points near the surface and far away."""
    from antipodal_gb300 import _lib
    rng = np.random.default_rng(31)
    v, i = synth.noisy_mesh("torus", 4000, 5, rng)
    b = synth.boundary_segments(v, i)
    tri = i.reshape(-1, 3)[rng.integers(len(i) // 3, size=400)]
    q = np.concatenate([synth.grid_queries(v.min(0), v.max(0), 22), v[rng.integers(len(v), size=400)],
                        0.5 * (v[tri[:, 0]] + v[tri[:, 1]]), v[rng.integers(len(v), size=400)] + rng.normal(0, 1e-7, (400, 3)),
                        rng.uniform(-30, 30, size=(400, 3))])
    with gwn.CudaDispatcher() as d:
        r = gwn.CudaRobustMeshGwn(d, v, i, b, precision=pol)
        got = {}
        for cells in (1, 0):
            d.set_option(_lib.OPT_INTEGER_CELLS, cells)
            o, c = np.empty(len(q)), np.empty(len(q), np.int32)
            r.evaluate(q, o, c)
            got[cells] = (o, c)
        r.close()
    assert np.array_equal(got[1][1], got[0][1])
    assert np.array_equal(got[1][0], got[0][0])
