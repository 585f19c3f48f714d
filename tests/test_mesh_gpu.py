"""Parity of the CUDA mesh path (fractional term, LBVH integer term, fused batch) with the CPU oracle.

Mirrors the reference's tests (test/test_gwn_mesh.cc, test/test_intersector.cc, test/test_common.cc of the
antipodal project) on the GPU, then extends them to the benchmark inputs and the edge cases of the kernels.
Tolerances: exact form (double) 1e-12 absolute against the oracle -- the reference arithmetic up to atan2's last
bit; float 2e-5; mixed form 1e-7 absolute (its accuracy target); integer counts bit-exact.
"""

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu

TOL_EXACT64 = 1e-12
TOL_EXACT32 = 2e-5
TOL_MIXED = 1e-7


def run_full(gwn, disp, verts, idx, q, x0, bnd, precision="exact"):
    disp.set_precision(precision)
    isect = gwn.CudaIntersector(disp, verts, idx)
    out = np.empty(len(q), dtype=q.dtype)
    gwn.eval_gwnr_mesh_batch(disp, isect, q, out, x0, bnd)
    isect.close()
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("closed", [True, False])
def test_cube_matches_baseline_and_oracle(gwn, disp, oracle, dtype, closed):
    # test/test_gwn_mesh.cc:101-138: closed and +Y-open cube, eight probe points, x0 = normalize(.31,.57,.76)
    verts = synth.CUBE_VERTS.astype(dtype)
    idx = synth.CUBE_IDX_CLOSED if closed else synth.CUBE_IDX_OPEN_Y
    bnd = np.zeros((0, 7), dtype) if closed else synth.cube_open_y_boundary(dtype)
    x0 = synth.unit_x0(dtype)
    q = synth.SAMPLE_POINTS.astype(dtype)
    got = run_full(gwn, disp, verts, idx, q, x0, bnd)
    base = oracle.gwn_baseline(q, verts, idx)
    ref = oracle.full_naive(q, x0, verts, idx, bnd)
    rel = 1e-4 if dtype == np.float32 else 1e-9
    assert np.all(np.abs(got - base) <= rel * np.maximum(1.0, np.abs(base)))
    tol = TOL_EXACT32 if dtype == np.float32 else TOL_EXACT64
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_intersector_cube_counts(gwn, disp, dtype):
    # test/test_intersector.cc:78-106: inside 1, outside 0, three generic directions
    verts = synth.CUBE_VERTS.astype(dtype)
    isect = gwn.CudaIntersector(disp, verts, synth.CUBE_IDX_CLOSED)
    q = np.array([[0, 0, 0], [0.1, -0.2, 0.3], [2, 0, 0], [-2, -2, -2]], dtype)
    for d in ([0.31, 0.57, 0.76], [-0.6, 0.4, -0.69], [0.83, -0.21, 0.51]):
        c = np.empty(4, np.int32)
        gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, c, np.array(d, dtype))
        assert c.tolist() == [1, 1, 0, 0]


def test_ties_on_axis_aligned_cube_rays(gwn, disp, oracle):
    """test/test_intersector.cc:85-89: NaiveIntersector is plain Moller-Trumbore and counts a ray through an edge or
    vertex once per triangle that shares it.  Axis-aligned rays from the closed cube's centre cross each face on the
    diagonal shared by its two triangles, so they count 2 where a generic direction counts 1.  The device counts
    (cell grid and hierarchy walk) reproduce the oracle's counts, double counts included, and the tie-reporting
    scan flags exactly the rays whose hits lie on an edge or vertex."""
    from antipodal_gb300 import _lib
    verts, idx = synth.CUBE_VERTS, synth.CUBE_IDX_CLOSED
    q = np.array([[0, 0, 0], [0.1, -0.2, 0.3], [0.0, 0.25, 0.0], [2, 0, 0], [-2, 0, 0]], np.float64)
    isect = gwn.CudaIntersector(disp, verts, idx)
    try:
        for d in ([1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, 0, -1], [0.31, 0.57, 0.76]):
            d = np.array(d, np.float64)
            ref = oracle.int_naive(q, d, verts, idx)
            for cells in (1, 0):
                disp.set_option(_lib.OPT_INTEGER_CELLS, cells)
                c = np.empty(len(q), np.int32)
                gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, c, d)
                assert np.array_equal(c, ref), (d, cells, c, ref)
            bf, ties = np.empty(len(q), np.int32), np.empty(len(q), np.int32)
            gwn.eval_gwnr_mesh_batch_integer_bruteforce(disp, verts, idx, q, bf, d, out_ties=ties)
            assert np.array_equal(bf, ref)
            axis = np.count_nonzero(d) == 1
            if axis:
                assert ref[0] == 2 and ties[0] == 2  # both triangles of the exit face, on their shared diagonal
            else:
                assert ref[0] == 1 and not ties.any()
    finally:
        disp.set_option(_lib.OPT_INTEGER_CELLS, 1)
        isect.close()


def test_rotated_open_cube_full_size(gwn, disp, oracle):
    verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=0, n_queries=100_000)
    ref = oracle.full_naive(q, x0, verts, idx, bnd)
    got = run_full(gwn, disp, verts, idx, q, x0, bnd, "exact")
    assert np.max(np.abs(got - ref)) <= TOL_EXACT64
    got = run_full(gwn, disp, verts, idx, q, x0, bnd, "mixed")
    assert np.max(np.abs(got - ref)) <= TOL_MIXED
    # integer term alone, bit exact
    isect = gwn.CudaIntersector(disp, verts, idx)
    c = np.empty(len(q), np.int32)
    gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, c, x0)
    assert np.array_equal(c, oracle.int_naive(q, x0, verts, idx))


def test_rotated_open_cube_float(gwn, disp, oracle):
    verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=1, n_queries=20_000, dtype=np.float32)
    isect = gwn.CudaIntersector(disp, verts, idx)
    c = np.empty(len(q), np.int32)
    gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, c, x0)
    assert np.array_equal(c, oracle.int_naive(q, x0, verts, idx))
    out = np.empty(len(q), np.float32)
    gwn.eval_gwnr_mesh_batch_fractional(disp, q, out, x0, bnd)
    np.testing.assert_allclose(out, oracle.frac_batch(q, x0, bnd), rtol=0, atol=TOL_EXACT32)


@pytest.mark.parametrize("n", [0, 1, 31, 33, 1000, 4097])
@pytest.mark.parametrize("n_seg", [0, 1, 3])
def test_ragged_sizes(gwn, disp, oracle, n, n_seg):
    rng = np.random.default_rng(n * 7 + n_seg)
    q = rng.uniform(-1.5, 1.5, size=(n, 3))
    segs = np.concatenate([rng.uniform(-1, 1, size=(n_seg, 6)), rng.integers(1, 3, size=(n_seg, 1))], axis=1)
    x0 = synth.unit_x0()
    out = np.empty(n)
    gwn.eval_gwnr_mesh_batch_fractional(disp, q, out, x0, segs)
    np.testing.assert_allclose(out, oracle.frac_batch(q, x0, segs), rtol=0, atol=TOL_EXACT64)
    disp.set_precision("mixed")
    gwn.eval_gwnr_mesh_batch_fractional(disp, q, out, x0, segs)
    np.testing.assert_allclose(out, oracle.frac_batch(q, x0, segs), rtol=0, atol=TOL_MIXED)


@pytest.mark.parametrize("n_seg", [511, 512, 513, 1100])
@pytest.mark.parametrize("qpt", [1, 2, 4, 8])
def test_segment_tiles_and_queries_per_thread(gwn, oracle, n_seg, qpt):
    # tile edges of the double-buffered shared-memory pipeline (tile 512) and every queries-per-thread variant
    rng = np.random.default_rng(n_seg + qpt)
    q = rng.uniform(-2, 2, size=(3001, 3))
    a = rng.uniform(-1, 1, size=(n_seg, 3))
    segs = np.concatenate([a, a + rng.normal(0, 0.05, size=(n_seg, 3)), np.ones((n_seg, 1))], axis=1)
    x0 = synth.unit_x0()
    ref = oracle.frac_batch(q, x0, segs)
    with gwn.CudaDispatcher(queries_per_thread=qpt, seg_tile=512, mixed_min_pairs=0) as d:
        out = np.empty(len(q))
        gwn.eval_gwnr_mesh_batch_fractional(d, q, out, x0, segs)
        np.testing.assert_allclose(out, ref, rtol=0, atol=TOL_EXACT64)
        d.set_precision("mixed")
        gwn.eval_gwnr_mesh_batch_fractional(d, q, out, x0, segs)
        np.testing.assert_allclose(out, ref, rtol=0, atol=TOL_MIXED)


def test_icosphere_subset_against_oracle(gwn, disp, oracle):
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=0, grid=0)
    q = synth.grid_queries(verts.min(0), verts.max(0), 14, 1.2)  # 2744 queries
    ref_int = oracle.int_naive(q, x0, verts, idx)
    isect = gwn.CudaIntersector(disp, verts, idx)
    c = np.empty(len(q), np.int32)
    gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, c, x0)
    assert 0 < isect.info()["depth"] < 64
    assert np.array_equal(c, ref_int)
    out = np.empty(len(q))
    gwn.eval_gwnr_mesh_batch(disp, isect, q, out, x0, bnd)
    ref = oracle.full_naive(q, x0, verts, idx, bnd)
    assert np.max(np.abs(out - ref)) <= TOL_EXACT64
    disp.set_precision("mixed")
    gwn.eval_gwnr_mesh_batch(disp, isect, q, out, x0, bnd)
    assert np.max(np.abs(out - ref)) <= TOL_MIXED


def test_lbvh_counts_equal_bruteforce_on_grid(gwn, disp):
    # the hierarchy only culls: on a 48^3 grid its counts equal the every-triangle scan's
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=3, level=4, grid=0)
    q = synth.grid_queries(verts.min(0), verts.max(0), 48, 1.3)
    isect = gwn.CudaIntersector(disp, verts, idx)
    a = np.empty(len(q), np.int32)
    b = np.empty(len(q), np.int32)
    gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, a, x0)
    gwn.eval_gwnr_mesh_batch_integer_bruteforce(disp, verts, idx, q, b, x0)
    assert np.array_equal(a, b)


def test_device_resident_tensors(gwn, oracle):
    torch = pytest.importorskip("torch")
    verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=2, n_queries=50_000)
    ref = oracle.full_naive(q, x0, verts, idx, bnd)
    dev = torch.device("cuda:0")
    with gwn.CudaDispatcher(stream=torch.cuda.current_stream(), mixed_min_pairs=0) as d:
        tq = torch.from_numpy(q).to(dev)
        tb = torch.from_numpy(bnd).to(dev)
        tv = torch.from_numpy(verts).to(dev)
        ti = torch.from_numpy(idx).to(dev)
        out = torch.empty(len(q), dtype=torch.float64, device=dev)
        isect = gwn.CudaIntersector(d, tv, ti)
        gwn.eval_gwnr_mesh_batch(d, isect, tq, out, x0, tb)
        d.synchronize()
        assert np.max(np.abs(out.cpu().numpy() - ref)) <= TOL_EXACT64


def test_errors_are_reported(gwn, disp):
    verts = synth.CUBE_VERTS
    with pytest.raises(gwn.GwnError) as e:
        gwn.CudaIntersector(disp, verts, np.array([0, 1, 99], np.int32))
    assert e.value.status == 1
    with pytest.raises(ValueError):
        gwn.eval_gwnr_mesh_batch_fractional(disp, np.zeros((4, 3)), np.zeros(3), synth.unit_x0(), np.zeros((1, 7)))
    with pytest.raises(gwn.GwnError):
        disp.set_option(2, 3)  # queries per thread must be 1, 2, 4 or 8
    isect32 = gwn.CudaIntersector(disp, verts.astype(np.float32), synth.CUBE_IDX_CLOSED)
    with pytest.raises(gwn.GwnError):
        gwn.eval_gwnr_mesh_batch_integer(disp, isect32, np.zeros((2, 3)), np.zeros(2, np.int32), synth.unit_x0())
    with pytest.raises(TypeError):
        disp.parallel_for(0, 4, lambda i: None)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_integer_term_along_many_directions(gwn, disp, oracle, dtype):
    # the hierarchy is built per ray direction and cached per context: switch directions back and forth,
    # including axis-aligned and unnormalised ones, and compare with the scan of every triangle
    verts, idx, _, _, _ = synth.open_icosphere(seed=6, level=4, grid=0)
    verts = verts.astype(dtype)
    rng = np.random.default_rng(6)
    q = rng.uniform(-1.4, 1.4, size=(4000, 3)).astype(dtype)
    isect = gwn.CudaIntersector(disp, verts, idx)
    dirs = [synth.unit_x0(), [1, 0, 0], [0, -1, 0], [0, 0, 5.0], [-3e-3, 2e-3, 1e-3], synth.unit_x0(), [1, 0, 0]]
    for d in dirs:
        d = np.asarray(d, dtype)
        c = np.empty(len(q), np.int32)
        gwn.eval_gwnr_mesh_batch_integer(disp, isect, q, c, d)
        assert np.array_equal(c, oracle.int_naive(q, d, verts, idx)), d


def test_own_atan2_against_cuda_and_fp64(gwn, disp):
    # the mixed kernel's float atan2 (octant reduction + minimax polynomial): max error within 6 ulp of the
    # result, measured against FP64 atan2; CUDA's atan2f is shown alongside
    rng = np.random.default_rng(17)
    y = np.concatenate([rng.standard_normal(200_000), rng.uniform(-1, 1, 50_000) * 1e-6,
                        [0.0, -0.0, 1.0, -1.0, 1e-30, 3.0]]).astype(np.float32)
    x = np.concatenate([rng.standard_normal(200_000), rng.uniform(-1, 1, 50_000),
                        [1.0, -1.0, 0.0, 0.0, -1.0, -1e-30]]).astype(np.float32)
    ours = np.empty_like(y)
    ref = np.empty_like(y)
    assert gwn.library().agwn_probe_atan2(disp.handle, y.ctypes.data, x.ctypes.data, len(y), ours.ctypes.data,
                                          ref.ctypes.data) == 0
    exact = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    err_ours = np.abs(ours - exact) / ulp
    err_cuda = np.abs(ref - exact) / ulp
    assert np.max(err_ours) <= 6.0, np.max(err_ours)
    assert np.max(err_cuda) <= 6.0


def test_host_arrays_pipelined_equal_device_arrays(gwn):
    """Host queries and results of 2^21 or more run through the chunked upload/compute/download pipeline, and device
    arrays of that size in chunks on two compute streams; the values must equal each other and those of calls on
    single chunks (below 2^21, one stream) bit for bit, in both precisions of the fractional term."""
    torch = pytest.importorskip("torch")
    verts, idx, bnd, q, x0 = synth.open_icosphere(seed=2, level=4, grid=128)
    assert len(q) >= 1 << 21
    s = torch.cuda.Stream()
    disp = gwn.CudaDispatcher(stream=s)
    isect = gwn.CudaIntersector(disp, verts, idx)
    for prec in ("exact", "mixed"):
        disp.set_precision(prec)
        qd = torch.from_numpy(q).cuda()
        od = torch.empty(len(q), dtype=torch.float64, device="cuda")
        gwn.eval_gwnr_mesh_batch(disp, isect, qd, od, x0, torch.from_numpy(bnd).cuda())
        disp.synchronize()
        # the first two chunks (2^20 queries each here) as calls of their own
        for a, b in ((0, 1 << 20), (1 << 20, 1 << 21)):
            part = torch.empty(b - a, dtype=torch.float64, device="cuda")
            gwn.eval_gwnr_mesh_batch(disp, isect, qd[a:b].contiguous(), part, x0, torch.from_numpy(bnd).cuda())
            disp.synchronize()
            assert torch.equal(part, od[a:b]), (prec, a)
        qh = torch.from_numpy(q).pin_memory().numpy()
        oh = torch.empty(len(q), dtype=torch.float64).pin_memory().numpy()
        gwn.eval_gwnr_mesh_batch(disp, isect, qh, oh, x0, bnd)
        assert np.array_equal(oh, od.cpu().numpy()), prec
        # pageable host memory takes the same path
        op = np.empty(len(q))
        gwn.eval_gwnr_mesh_batch(disp, isect, q, op, x0, bnd)
        assert np.array_equal(op, oh)
    isect.close()
    disp.close()


def _polyline(rng, n, closed, centre=(0.0, 0.0, 0.0), radius=1.0):
    t = np.sort(rng.uniform(0, 2 * np.pi, size=n))
    v = np.stack([np.cos(t), np.sin(t), 0.3 * np.sin(3 * t)], axis=1) * radius + np.asarray(centre)
    v = v + rng.normal(0, 0.01, size=v.shape)
    nxt = np.roll(v, -1, axis=0)
    segs = np.concatenate([v, nxt, np.ones((n, 1))], axis=1)
    return segs if closed else segs[:-1]


def _check_mixed(gwn, oracle, q, x0, segs, seg_tile=512, qpt=2):
    ref = oracle.frac_batch(q, x0, segs)
    with gwn.CudaDispatcher(precision="mixed", queries_per_thread=qpt, seg_tile=seg_tile, mixed_min_pairs=0) as d:
        out = np.empty(len(q))
        gwn.eval_gwnr_mesh_batch_fractional(d, q, out, x0, segs)
    assert np.abs(out - ref).max() <= TOL_MIXED, np.abs(out - ref).max()
    return out


def test_mixed_boundary_chains_any_order(gwn, oracle):
    """The mixed kernel walks the boundary as chains of segments that share endpoints (found by exact equality,
    whatever the input order).  On loops and open chains where at most two segments meet at a vertex every pair is
    evaluated and routed (FP32 or FP64) the same way in any order, so any order agrees with itself up to summation
    order.  Where more segments meet at a vertex (or duplicates and zero-length segments sit there), the linking
    decides which neighbour sets a vertex's near threshold, so a few pairs may be routed differently: still within
    the mixed tolerance of the oracle."""
    rng = np.random.default_rng(11)
    x0 = synth.unit_x0()
    q = rng.uniform(-1.6, 1.6, size=(2001, 3))
    loop_a = _polyline(rng, 97, True)
    loop_b = _polyline(rng, 40, True, centre=(0.3, -0.2, 0.4), radius=0.5)
    open_c = _polyline(rng, 31, False, centre=(-0.2, 0.5, -0.3), radius=0.7)
    manifold = np.concatenate([loop_a, loop_b, open_c])
    base = _check_mixed(gwn, oracle, q, x0, manifold)
    for seed in range(3):
        perm = np.random.default_rng(seed).permutation(len(manifold))
        got = _check_mixed(gwn, oracle, q, x0, manifold[perm])
        assert np.abs(got - base).max() <= 1e-12
    # two more segments leave and re-enter a vertex of loop_a: four segments meet there
    p = loop_a[10, :3]
    extra = np.array([np.r_[p, p + [0.2, 0.1, 0.0], 1.0], np.r_[p + [0.2, 0.1, 0.0], p, 1.0]])
    dup = loop_b[:3].copy()  # the same segments twice
    zero = np.array([np.r_[p, p, 2.0], np.r_[p, p, 1.0]])  # zero-length segments at a shared vertex
    rev = open_c[5:9][:, [3, 4, 5, 0, 1, 2, 6]]  # reversed copies: they chain among themselves only
    segs = np.concatenate([manifold, extra, dup, zero, rev])
    base = _check_mixed(gwn, oracle, q, x0, segs)
    for seed in range(3):
        perm = np.random.default_rng(seed).permutation(len(segs))
        got = _check_mixed(gwn, oracle, q, x0, segs[perm])
        assert np.abs(got - base).max() <= TOL_MIXED


@pytest.mark.parametrize("n_seg,seg_tile,qpt", [(101, 32, 2), (101, 64, 1), (255, 32, 4), (63, 32, 8)])
def test_mixed_chains_across_tiles(gwn, oracle, n_seg, seg_tile, qpt):
    # chains longer than a tile, odd entry counts, several chains per tile, every queries-per-thread variant
    rng = np.random.default_rng(n_seg + seg_tile)
    x0 = synth.unit_x0()
    q = rng.uniform(-1.6, 1.6, size=(1500, 3))
    segs = np.concatenate([_polyline(rng, n_seg, True), _polyline(rng, 17, False, centre=(0.1, 0.1, 0.1), radius=0.3),
                           _polyline(rng, 8, True, centre=(-0.3, 0.0, 0.2), radius=0.2)])
    _check_mixed(gwn, oracle, q, x0, segs, seg_tile=seg_tile, qpt=qpt)


def _clustered_queries(rng, n_clusters, lo=-1.6, hi=1.6, spread=0.03):
    # 32 consecutive queries (one warp slot of the fractional kernels) around each of n_clusters random centres
    c = rng.uniform(lo, hi, size=(n_clusters, 1, 3))
    return (c + rng.uniform(-spread, spread, size=(n_clusters, 32, 3))).reshape(-1, 3)


@pytest.mark.parametrize("n_seg,seg_tile,qpt", [(212, 512, 2), (600, 512, 2), (600, 128, 4), (300, 64, 8)])
def test_mixed_certified_groups_equal_the_per_pair_path(gwn, oracle, n_seg, seg_tile, qpt):
    """Boundary groups of 8 entries that lie far enough across the ray from all of a warp's queries (every pair's
    error bound below the FP64 threshold, every angle in the first octant) are evaluated without the per-pair bound
    and octant unfolding.  The operations left are the per-pair path's own, so certification on and off give the
    same results bit for bit: one tile or several, chain starts inside groups, every queries-per-thread variant."""
    from antipodal_gb300 import _lib
    rng = np.random.default_rng(n_seg + seg_tile)
    x0 = synth.unit_x0()
    q = _clustered_queries(rng, 1024)
    segs = np.concatenate([_polyline(rng, n_seg, True), _polyline(rng, 40, False, centre=(0.2, -0.1, 0.3),
                                                                   radius=0.4)])
    ref = oracle.frac_batch(q, x0, segs)
    outs, stats = {}, {}
    for cert in (1, 0):
        with gwn.CudaDispatcher(precision="mixed", queries_per_thread=qpt, seg_tile=seg_tile, mixed_min_pairs=0,
                                timing=True) as d:
            assert d.get_option(_lib.OPT_MIXED_CERTIFY) == 1.0
            d.set_option(_lib.OPT_MIXED_CERTIFY, cert)
            out = np.empty(len(q))
            gwn.eval_gwnr_mesh_batch_fractional(d, q, out, x0, segs)
            outs[cert], stats[cert] = out, d.stats()
    assert np.array_equal(outs[1], outs[0])
    assert np.abs(outs[1] - ref).max() <= TOL_MIXED, np.abs(outs[1] - ref).max()
    assert stats[0]["certified_pairs"] == 0
    # (eight query slots per warp and 64-entry tiles certify the fewest: 8% of the pairs)
    assert stats[1]["certified_pairs"] >= 0.05 * stats[1]["pairs"], (stats[1]["certified_pairs"], stats[1]["pairs"])
    assert stats[1]["fp64_pairs"] == stats[0]["fp64_pairs"]


def test_mixed_certified_groups_range_guard(gwn, oracle):
    # far-off queries (2^25 across) and a boundary scaled to 1e-12: no group is certified there (float products of
    # the certified path would overflow or underflow), and the results still equal the per-pair path's
    from antipodal_gb300 import _lib
    rng = np.random.default_rng(5)
    x0 = synth.unit_x0()
    segs = _polyline(rng, 200, True)
    for scale, qscale in ((1.0, 3.4e7), (1e-12, 1e-12)):
        s = segs.copy()
        s[:, :6] *= scale
        q = _clustered_queries(rng, 64) * qscale
        outs = {}
        for cert in (1, 0):
            with gwn.CudaDispatcher(precision="mixed", mixed_min_pairs=0, timing=True) as d:
                d.set_option(_lib.OPT_MIXED_CERTIFY, cert)
                out = np.empty(len(q))
                gwn.eval_gwnr_mesh_batch_fractional(d, q, out, x0, s)
                outs[cert] = out
                if cert:
                    assert d.stats()["certified_pairs"] == 0
        assert np.array_equal(outs[1], outs[0])
        assert np.all(np.isfinite(outs[1]))
        assert np.abs(outs[1] - oracle.frac_batch(q, x0, s)).max() <= TOL_MIXED


def test_mixed_incoherent_queries_run_in_spatial_order(gwn, oracle):
    """Queries in random order (warps of scattered queries certify almost no boundary group) run on a copy sorted
    along a 2D Morton curve across the ray and are scattered back: the same values bit for bit as the per-pair path
    on the given order, and most pairs certified.  Full GWN and fractional term on device arrays of 2^20 queries
    and more."""
    torch = pytest.importorskip("torch")
    from antipodal_gb300 import _lib
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=2, level=6, grid=0)
    rng = np.random.default_rng(9)
    q = rng.uniform(-1.3, 1.3, size=((1 << 20) + 4099, 3))
    qd = torch.from_numpy(q).cuda()
    res = {}
    for cert in (1, 0):
        with gwn.CudaDispatcher(precision="mixed", timing=True) as d:
            d.set_option(_lib.OPT_MIXED_CERTIFY, cert)
            isect = gwn.CudaIntersector(d, verts, idx)
            full = torch.empty(len(q), dtype=torch.float64, device="cuda")
            gwn.eval_gwnr_mesh_batch(d, isect, qd, full, x0, bnd)
            d.stats(reset=True)
            frac = torch.empty_like(full)
            gwn.eval_gwnr_mesh_batch_fractional(d, qd, frac, x0, bnd)
            st = d.stats(reset=True)
            isect.close()
            res[cert] = (full.cpu().numpy(), frac.cpu().numpy(), st["certified_pairs"] / max(1, st["pairs"]))
    assert np.array_equal(res[1][0], res[0][0])
    assert np.array_equal(res[1][1], res[0][1])
    assert res[0][2] == 0.0
    assert res[1][2] > 0.5, res[1][2]
    sample = rng.choice(len(q), 2000, replace=False)
    ref = oracle.full_naive(q[sample], x0, verts, idx, bnd)
    assert np.abs(res[1][0][sample] - ref).max() <= TOL_MIXED


def test_mixed_query_order_decision_is_only_a_speed_matter(gwn):
    """The order decision is kept per (array, size, direction).  Overwriting the same device array with queries in
    another order keeps the old decision; either way the values equal those of a fresh context bit for bit."""
    torch = pytest.importorskip("torch")
    verts, idx, bnd, _, x0 = synth.open_icosphere(seed=5, level=5, grid=0)
    n = (1 << 20) + 77
    rng = np.random.default_rng(13)
    q_rand = rng.uniform(-1.3, 1.3, size=(n, 3))
    side = int(np.ceil(n ** (1 / 3)))
    q_grid = synth.grid_queries(verts.min(0), verts.max(0), side, 1.2)[:n]
    qd = torch.from_numpy(q_rand).cuda()
    out = torch.empty(n, dtype=torch.float64, device="cuda")

    def fresh(q):
        with gwn.CudaDispatcher(precision="mixed") as d:
            o = torch.empty(n, dtype=torch.float64, device="cuda")
            gwn.eval_gwnr_mesh_batch_fractional(d, torch.from_numpy(q).cuda(), o, x0, bnd)
            return o.cpu().numpy()

    with gwn.CudaDispatcher(precision="mixed") as d:
        gwn.eval_gwnr_mesh_batch_fractional(d, qd, out, x0, bnd)  # decided incoherent: sorted
        first = out.cpu().numpy()
        qd.copy_(torch.from_numpy(q_grid))  # the same array, now in grid order; the kept decision still sorts
        gwn.eval_gwnr_mesh_batch_fractional(d, qd, out, x0, bnd)
        second = out.cpu().numpy()
    assert np.array_equal(first, fresh(q_rand))
    assert np.array_equal(second, fresh(q_grid))


@pytest.mark.parametrize("n_seg", [4096, 4097])
def test_mixed_chain_limit(gwn, oracle, n_seg):
    # up to 4096 segments the boundary is chained; above, every segment is a chain of its own
    rng = np.random.default_rng(n_seg)
    x0 = synth.unit_x0()
    q = rng.uniform(-1.6, 1.6, size=(1200, 3))
    segs = _polyline(rng, n_seg, True)
    _check_mixed(gwn, oracle, q, x0, segs)



@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_integer_cells_equal_the_walk_and_the_oracle(gwn, oracle, dtype):
    """The integer term looks up each ray's candidate triangles in a uniform grid over the plane across the ray
    (default) or walks the hierarchy (option 0): the same counts, equal to the scan of every triangle.  Queries on
    a grid through the mesh, far outside it (a tolerance above the grid's widening: those take the walk inside the
    grid kernel), beyond the grid's extent, on vertices and edges; two directions, switched back and forth so the
    grid is rebuilt with the hierarchy."""
    from antipodal_gb300 import _lib
    verts, idx, _, _, _ = synth.open_icosphere(seed=4, level=4, grid=0)
    verts = verts.astype(dtype)
    rng = np.random.default_rng(4)
    g = synth.grid_queries(verts.min(0), verts.max(0), 24, 1.2)
    far = rng.uniform(-40, 40, size=(2000, 3))
    outside = rng.uniform(-1, 1, size=(500, 3)) + np.array([3.0, -3.0, 0.5])
    on_vertex = verts[rng.integers(0, len(verts), size=500)].astype(np.float64)
    tri = idx.reshape(-1, 3)[rng.integers(0, len(idx) // 3, size=500)]
    on_edge = 0.5 * (verts[tri[:, 0]].astype(np.float64) + verts[tri[:, 1]])
    q = np.concatenate([g, far, outside, on_vertex, on_edge]).astype(dtype)
    with gwn.CudaDispatcher() as d:
        isect = gwn.CudaIntersector(d, verts, idx)
        for x0 in [synth.unit_x0(), [0.0, 0.0, 1.0], synth.unit_x0()]:
            x0 = np.asarray(x0, dtype)
            ref = oracle.int_naive(q, x0, verts, idx)
            got = {}
            for cells in (1, 0):
                d.set_option(_lib.OPT_INTEGER_CELLS, cells)
                c = np.empty(len(q), np.int32)
                gwn.eval_gwnr_mesh_batch_integer(d, isect, q, c, x0)
                got[cells] = c
            assert np.array_equal(got[1], got[0]), np.flatnonzero(got[1] != got[0])[:10]
            assert np.array_equal(got[1], ref), np.flatnonzero(got[1] != ref)[:10]
            if dtype == np.float64:
                # the every-triangle scan (its box cull included) gives the oracle's counts as well
                scan = np.empty(len(q), np.int32)
                gwn.eval_gwnr_mesh_batch_integer_bruteforce(d, verts, idx, q, scan, x0)
                assert np.array_equal(scan, ref), np.flatnonzero(scan != ref)[:10]
        isect.close()


def test_mixed_mode_runs_exact_kernels_below_its_minimum(gwn, oracle):
    # on a boundary of fewer than 32 segments (and below the minimum pair count, default 2^14 per call) the mixed
    # mode runs the exact kernels: bit-identical to the exact mode; with the minimum at 0 it runs the mixed kernel
    # (within the mixed tolerance)
    from antipodal_gb300 import _lib
    verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=3, n_queries=20_000)
    with gwn.CudaDispatcher() as d:
        assert d.get_option(_lib.OPT_MIXED_MIN_PAIRS) == float(1 << 14)
        isect = gwn.CudaIntersector(d, verts, idx)
        outs = {}
        for prec, minp in (("exact", 1 << 14), ("mixed", 1 << 14), ("mixed", 0)):
            d.set_precision(prec)
            d.set_option(_lib.OPT_MIXED_MIN_PAIRS, minp)
            o = np.empty(len(q))
            gwn.eval_gwnr_mesh_batch(d, isect, q, o, x0, bnd)
            outs[(prec, minp)] = o
        isect.close()
    assert np.array_equal(outs[("mixed", 1 << 14)], outs[("exact", 1 << 14)])
    assert np.abs(outs[("mixed", 0)] - outs[("exact", 1 << 14)]).max() <= TOL_MIXED
    assert np.abs(outs[("exact", 1 << 14)] - oracle.full_naive(q, x0, verts, idx, bnd)).max() <= TOL_EXACT64
