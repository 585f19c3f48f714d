"""Device boundary extraction (build_boundary_segments, src/antipodal/math/common.hh:123-174) against the oracle's
restatement, which the CPU tests pin to the reference: identical rows in ascending (lo, hi) order, for manifold and
non-manifold meshes, degenerate edges, both precisions, host and device arrays."""

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu


def meshes():
    rng = np.random.default_rng(3)
    yield "open cube", synth.CUBE_VERTS, synth.CUBE_IDX_OPEN_Y
    v, i = synth.noisy_mesh("icosphere", 20000, 7, rng)
    yield "icosphere with holes", v, i
    v, i = synth.noisy_mesh("torus", 50000, 15, rng)
    yield "torus with holes", v, i
    # non-manifold: three triangles on one edge, and a triangle with a repeated vertex (degenerate edges)
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [2, 2, 2]], np.float64)
    i = np.array([0, 1, 2, 1, 0, 3, 0, 1, 4, 5, 5, 2], np.int32)
    yield "non-manifold", v, i


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_boundary_matches_oracle(gwn, disp, oracle, dt):
    for name, v, i in meshes():
        got = gwn.build_boundary_segments(disp, v.astype(dt), i)
        ref = oracle.boundary(v.astype(dt), i)
        assert got.dtype == dt and got.shape == ref.shape, name
        assert np.array_equal(got, ref), name


def test_boundary_large_mesh(gwn, disp, oracle):
    v, i, b, _ = synth.two_tori(seed=1, n_tris=400_000, n_holes=20, n_queries=2)
    got = gwn.build_boundary_segments(disp, v, i)
    assert np.array_equal(got, oracle.boundary(v, i))
    assert np.array_equal(got, b)  # the generator's own (numpy) boundary follows the same rule and order


def test_boundary_device_arrays_and_capacity(gwn, disp):
    torch = pytest.importorskip("torch")
    v, i = synth.noisy_mesh("icosphere", 5000, 4, np.random.default_rng(1))
    host = gwn.build_boundary_segments(disp, v, i)
    dev = gwn.build_boundary_segments(disp, torch.from_numpy(v).cuda(), torch.from_numpy(i).cuda())
    torch.cuda.synchronize()
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), host)
    # the count alone, and a truncated copy
    import ctypes as C
    lib = gwn.library()
    cnt = C.c_int64()
    vv, ii = np.ascontiguousarray(v), np.ascontiguousarray(i)
    assert lib.agwn_build_boundary_segments_f64(disp.handle, vv.ctypes.data, len(vv), ii.ctypes.data, len(ii), None, 0,
                                                C.byref(cnt)) == 0
    assert cnt.value == len(host)
    part = np.full((5, 7), -1.0)
    assert lib.agwn_build_boundary_segments_f64(disp.handle, vv.ctypes.data, len(vv), ii.ctypes.data, len(ii),
                                                part.ctypes.data, 3, C.byref(cnt)) == 0
    assert np.array_equal(part[:3], host[:3]) and (part[3:] == -1).all()


def test_boundary_errors_and_empty(gwn, disp):
    v = synth.CUBE_VERTS
    assert gwn.build_boundary_segments(disp, v, np.zeros(0, np.int32)).shape == (0, 7)
    closed = gwn.build_boundary_segments(disp, v, synth.CUBE_IDX_CLOSED)
    assert closed.shape == (0, 7)  # a closed manifold has no boundary
    with pytest.raises(gwn.GwnError):
        gwn.build_boundary_segments(disp, v, np.array([0, 1, 8], np.int32))
    # the context stays usable after the rejected call
    assert gwn.build_boundary_segments(disp, v, synth.CUBE_IDX_OPEN_Y).shape == (4, 7)
