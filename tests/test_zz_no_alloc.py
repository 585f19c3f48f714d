"""The fractional entry point that allocates nothing, checked against the regular one.

Callers that own all of the GPU's memory themselves (their own pool allocator with a fixed budget, or a plugin
inside a framework whose caching allocator must not be bypassed) cannot let a library call cudaMalloc.
agwn_mesh_batch_fractional_mixed_noalloc_f64 serves them from one fixed static device array instead of a context.
This test calls it through the C ABI several times in a row on different inputs (no call may see the previous
call's leftovers in the shared array), and compares each result with agwn_mesh_batch_fractional_f64 in the mixed
mode on the same device inputs.  The boundaries cover both of its tile paths: one 512-entry tile (the icosphere's
and the cube's boundaries), several double-buffered tiles over chained loops (1,100 segments), and the unchained
stream of one start entry per segment above 4,096 segments (6,000, and the 8,192-segment maximum).  The file is
named so pytest collects it last.
"""

import ctypes as C

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the exact-arithmetic tolerance of the mesh tests: both calls run the same kernels
MAX_SEGMENTS = 8192


def _entry(lib):
    f = lib.agwn_mesh_batch_fractional_mixed_noalloc_f64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
    return f


def _loops(seed, n_loops, per_loop):
    """Closed noisy loops of ``per_loop`` segments each, as (n, 7) [pos0, pos1, weight] rows."""
    rng = np.random.default_rng(seed)
    rows = []
    t = np.linspace(0.0, 2.0 * np.pi, per_loop, endpoint=False)
    for _ in range(n_loops):
        r = rng.uniform(0.2, 0.6)
        pts = np.stack([r * np.cos(t), r * np.sin(t), 0.05 * np.sin(3.0 * t)], 1) @ synth.random_rotation(rng).T
        pts = pts + rng.normal(scale=0.4, size=3) + rng.normal(scale=1e-3, size=pts.shape)
        w = np.full((per_loop, 1), float(rng.integers(1, 3)))
        rows.append(np.hstack([pts, np.roll(pts, -1, axis=0), w]))
    return np.ascontiguousarray(np.vstack(rows))


def _inputs():
    v, idx, bnd, _, x0 = synth.open_icosphere(seed=5, level=5, grid=0)
    q1 = synth.grid_queries(v.min(0), v.max(0), 40, 1.2)
    _, _, bnd2, q2, x02 = synth.rotated_open_cube(seed=9, n_queries=30_000)
    cases = [(q1, bnd, x0), (q2, bnd2, x02)]
    for seed, n_loops, per_loop in ((11, 5, 220), (12, 20, 300), (13, 32, 256)):
        b = _loops(seed, n_loops, per_loop)
        ends = b[:, :6].reshape(-1, 3)
        q = synth.grid_queries(ends.min(0), ends.max(0), 24, 1.3)
        cases.append((q, b, synth.random_unit(np.random.default_rng(seed))))
    assert [len(c[1]) for c in cases[2:]] == [1100, 6000, MAX_SEGMENTS]
    return cases


def test_noalloc_matches_regular_entry_point_on_calls_in_a_row(gwn):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    f = _entry(gwn.library())
    with gwn.CudaDispatcher(stream=torch.cuda.current_stream(dev), precision="mixed", mixed_min_pairs=0) as disp:
        for q, bnd, x0 in _inputs():
            qd = torch.from_numpy(q).to(dev)
            bd = torch.from_numpy(bnd).to(dev)
            ref = torch.empty(len(q), dtype=torch.float64, device=dev)
            out = torch.full((len(q),), float("nan"), dtype=torch.float64, device=dev)
            gwn.eval_gwnr_mesh_batch_fractional(disp, qd, ref, x0, bd)
            disp.synchronize()
            x = np.ascontiguousarray(x0, np.float64)
            rc = f(None, qd.data_ptr(), len(q), out.data_ptr(), x.ctypes.data, bd.data_ptr(), len(bnd))
            assert rc == 0, gwn.library().agwn_last_error_message()
            torch.cuda.synchronize(dev)
            err = float((out - ref).abs().max().item())
            assert err <= TOL, err


def test_noalloc_rejects_boundaries_beyond_its_scratch(gwn):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    f = _entry(gwn.library())
    q = torch.zeros((16, 3), dtype=torch.float64, device=dev)
    out = torch.empty(16, dtype=torch.float64, device=dev)
    b = torch.zeros((MAX_SEGMENTS + 1, 7), dtype=torch.float64, device=dev)
    x = np.array(synth.unit_x0())
    rc = f(None, q.data_ptr(), 16, out.data_ptr(), x.ctypes.data, b.data_ptr(), MAX_SEGMENTS + 1)
    assert rc == 1
    assert b"8192" in gwn.library().agwn_last_error_message()
