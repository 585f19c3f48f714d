"""The fractional entry point that allocates nothing, checked against the regular one.

Callers that own all of the GPU's memory themselves (their own pool allocator with a fixed budget, or a plugin
inside a framework whose caching allocator must not be bypassed) cannot let a library call cudaMalloc.
agwn_mesh_batch_fractional_mixed_noalloc_f64 serves them from one fixed static device array instead of a context.
This test calls it through the C ABI, twice in a row on different inputs (the second call must not see the first
call's leftovers in the shared array), and compares each result with agwn_mesh_batch_fractional_f64 in the mixed
mode on the same device inputs.  The file is named so pytest collects it last.
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


def _inputs():
    v, idx, bnd, _, x0 = synth.open_icosphere(seed=5, level=5, grid=0)
    q1 = synth.grid_queries(v.min(0), v.max(0), 40, 1.2)
    _, _, bnd2, q2, x02 = synth.rotated_open_cube(seed=9, n_queries=30_000)
    return [(q1, bnd, x0), (q2, bnd2, x02)]


def test_noalloc_matches_regular_entry_point_on_two_calls(gwn):
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
