"""The C ABI and the C++ front end, without a GPU: the library loads and exports every function the header
declares; calls fail loudly (no CPU fallback) when no device is present; the front end compiles against the
reference's own headers, its overloads win overload resolution, and a generic call with CudaDispatcher does not
compile.  The GPU run of the front end is in test_frontend_gpu.py."""

import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from oracle.oracle import reference_src

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "antipodal_gb300.h")
REF_SRC = reference_src() or ""


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int|void)\s+(agwn_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from antipodal_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def test_every_declared_function_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    from antipodal_gb300 import _lib
    # and every binding the Python package declares exists in the header
    for n in _lib.declared_symbols():
        assert n in names, n


def test_status_strings_and_version(lib):
    assert lib.agwn_abi_version() == 2
    assert lib.agwn_status_string(0) == b"ok"
    assert lib.agwn_status_string(7) == b"no CUDA device"


def test_no_cpu_fallback_without_gpu(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import antipodal_gb300 as ag
    with pytest.raises(ag.GwnError) as e:
        ag.CudaDispatcher()
    assert e.value.status == 7


def test_invalid_arguments_rejected_before_any_device_work(lib):
    import ctypes as C
    # null context and negative sizes are argument errors, reported without touching a device
    assert lib.agwn_mesh_batch_fractional_f64(None, None, 0, None, None, None, 0) == 1
    assert lib.agwn_context_set_option(None, 0, 0.0) == 1
    out = C.c_void_p()
    assert lib.agwn_context_create(0, None, None) == 1
    assert lib.agwn_bvh_info(None, None, None) == 1
    assert lib.agwn_mesh_batch_fractional_mixed_noalloc_f64(None, None, 5, None, None, None, 10000) == 1
    assert b"8192" in lib.agwn_last_error_message()
    del out


def _gxx():
    return shutil.which("g++")


def _compile(src: str, extra: list[str], out: str | None = None, libs: list[str] | None = None):
    cmd = [_gxx(), "-std=c++20", "-I", os.path.join(ROOT, "include")] + extra
    cmd += ["-fsyntax-only", src] if out is None else [src, "-o", out] + (libs or [])
    return subprocess.run(cmd, capture_output=True, text=True)


needs_ref = pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference headers absent")


@needs_ref
def test_frontend_compiles_against_reference_headers(tmp_path):
    # the reference's headers come first; our overloads must be chosen (the reference template would instantiate
    # CudaDispatcher::parallel_for, whose static_assert fails)
    src = tmp_path / "use.cc"
    src.write_text("""
#include <antipodal/gwn_mesh.hh>
#include <antipodal/gwn_parametric.hh>
#include <antipodal/math/robust_predicates.hh>
#include <antipodal/dispatcher/dispatcher_threadpool.hh>
#include <antipodal/cuda/gwn_cuda.hh>
#include <array>
#include <vector>
using namespace antipodal;
void run(cuda::CudaDispatcher& d, cuda::CudaIntersector<double> const& i, std::vector<dvec3> const& p,
         std::vector<double>& o, std::vector<int>& c, std::vector<weighted_dsegment3> const& b, dvec3 x0) {
    eval_gwnr_mesh_batch(d, i, std::span<dvec3 const>{p}, std::span<double>{o}, x0, std::span<weighted_dsegment3 const>{b});
    eval_gwnr_mesh_batch_fractional(d, std::span<dvec3 const>{p}, std::span<double>{o}, x0, std::span<weighted_dsegment3 const>{b});
    eval_gwnr_mesh_batch_integer(d, i, std::span<dvec3 const>{p}, std::span<int>{c}, x0);
    // robust (the reference's precision tags are accepted) and parametric overloads
    cuda::CudaRobustMeshGwn<double, robust::int128_grid> rob{d, std::span<dvec3 const>{p}, std::span<int const>{},
                                                             std::span<weighted_dsegment3 const>{b}};
    eval_gwnr_mesh_batch_robust(d, rob, std::span<dvec3 const>{p}, std::span<double>{o});
    std::vector<std::array<dvec3, 4>> curves;
    cuda::CubicBezierBoundary const cb{std::span<std::array<dvec3, 4> const>{curves}};
    eval_gwnr_parametric_batch_fractional(d, std::span<dvec3 const>{p}, std::span<double>{o}, x0, cb);
    eval_gwnr_parametric_batch_fractional(d, std::span<dvec3 const>{p}, std::span<double>{o}, x0, cb,
                                          integrate_config{0, 10, 1e-10});
    cuda::LearnedGK15Proposal net{d};
    eval_gwnr_parametric_batch_fractional(d, std::span<dvec3 const>{p}, std::span<double>{o}, x0, cb,
                                          integrate_config{}, net);
    std::vector<std::array<dvec3, 16>> pats;
    cuda::CudaBezierPatchIntersector const pint{d, std::span<std::array<dvec3, 16> const>{pats}};
    eval_gwnr_parametric_batch_integer(d, pint, std::span<dvec3 const>{p}, std::span<int>{c}, x0);
    eval_gwnr_parametric_batch(d, pint, std::span<dvec3 const>{p}, std::span<double>{o}, x0, cb);
    eval_gwnr_parametric_batch(d, pint, std::span<dvec3 const>{p}, std::span<double>{o}, x0, cb, integrate_config{}, net);
    (void)pint.signed_intersection_count(x0, x0);
    std::vector<cuda::CudaRobustBatch<double, robust::int128_grid>::Job> jobs{{&rob, p.data(), 0, o.data()}};
    cuda::CudaRobustBatch<double, robust::int128_grid> batch{d, jobs};
    batch.tune();
    batch.run();
    auto const segs = build_boundary_segments(d, std::span<dvec3 const>{p}, std::span<int const>{});
    (void)segs;
    // the reference's CPU path still works alongside
    PoolDispatcher pool{2};
    NaiveIntersector<double> naive{std::span<dvec3 const>{p}, std::span<int const>{}};
    eval_gwnr_mesh_batch(pool, naive, std::span<dvec3 const>{p}, std::span<double>{o}, x0, std::span<weighted_dsegment3 const>{b});
}
""")
    r = _compile(str(src), ["-I", REF_SRC])
    assert r.returncode == 0, r.stderr


@needs_ref
def test_generic_call_with_cuda_dispatcher_does_not_compile(tmp_path):
    src = tmp_path / "bad.cc"
    src.write_text("""
#include <antipodal/gwn_mesh.hh>
#include <antipodal/cuda/gwn_cuda.hh>
using namespace antipodal;
void run(cuda::CudaDispatcher& d, NaiveIntersector<double> const& n, std::span<dvec3 const> p, std::span<double> o,
         std::span<weighted_dsegment3 const> b, dvec3 x0) {
    eval_gwnr_mesh_batch(d, n, p, o, x0, b);   // NaiveIntersector has no device form: must not compile
}
""")
    r = _compile(str(src), ["-I", REF_SRC])
    assert r.returncode != 0
    assert "no CPU fallback" in r.stderr or "GWN kernels only" in r.stderr


def test_frontend_program_reports_missing_gpu(lib, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the GPU run is in test_frontend_gpu.py)")
    inc = REF_SRC if os.path.isdir(REF_SRC) else os.path.join(ROOT, "tests", "cpp", "shim")
    exe = str(tmp_path / "frontend_run")
    libdir = os.path.join(ROOT, "antipodal_gb300")
    r = _compile(os.path.join(ROOT, "tests", "cpp", "frontend_run.cc"), ["-I", inc], out=exe,
                 libs=["-L", libdir, "-lantipodal_gb300", f"-Wl,-rpath,{libdir}"])
    assert r.returncode == 0, r.stderr
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 3 and p.stdout.startswith("error 7")


def test_synthetic_workloads_are_deterministic():
    from antipodal_gb300 import synth
    a = synth.open_icosphere(seed=0, grid=0)
    b = synth.open_icosphere(seed=0, grid=0)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert len(a[1]) // 3 == 76496 and len(a[2]) == 212
    v, f = synth.icosphere(6)
    assert len(f) == 81920 and len(v) == 40962
    q = synth.grid_queries(np.zeros(3), np.ones(3), 4)
    assert q.shape == (64, 3) and np.allclose(q[1] - q[0], [1.2 / 3, 0, 0])
    c, qq, x0 = synth.bezier_patches(seed=1, n_patches=2, n_queries=100)
    assert c.shape == (8, 12) and qq.shape == (100, 3)
    # consecutive boundary curves of a patch share end points (closed loop)
    cc = c.reshape(-1, 4, 4, 3)
    for k in range(4):
        assert np.array_equal(cc[0, k, 3], cc[0, (k + 1) % 4, 0])
