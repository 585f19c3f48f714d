"""GB300-native batch generalized winding numbers, with the antipodal library's batch API.

This Python module mirrors the reference's C++ entry points (same names, argument order and meaning) over the
C ABI of libantipodal_gb300.so, so tests and benchmarks read like the reference's own:

    disp = CudaDispatcher()                                   # a Dispatcher that runs on one GPU
    isect = CudaIntersector(disp, vertices, indices)          # an Intersector backed by a device LBVH
    eval_gwnr_mesh_batch(disp, isect, positions, out, x0, boundary)

Arrays may be numpy arrays (host memory) or torch tensors (host or CUDA); shapes follow the reference value
types: positions (n, 3), boundary (s, 7) = [pos0, pos1, weight], vertices (v, 3), indices (3 f,) int32.
Every call runs the CUDA kernels; if the extension is not built, or no GPU is present, calls raise -- there is
no CPU fallback.  (The CPU oracle used by the tests lives in oracle/, outside this package.)
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FRAC_EXACT, FRAC_MIXED, Stats

__all__ = [
    "GwnError", "CudaDispatcher", "CudaIntersector", "CudaRobustMeshGwn", "eval_gwnr_mesh_batch_fractional",
    "eval_gwnr_mesh_batch_integer", "eval_gwnr_mesh_batch", "eval_gwnr_mesh_batch_robust", "build_boundary_segments",
    "IntegrateConfig", "IntegratorGK15", "eval_gwnr_parametric_batch_fractional", "unpack_pair_stats",
    "CudaBezierPatchIntersector", "eval_gwnr_parametric_batch_integer", "eval_gwnr_parametric_batch",
    "LearnedGK15Proposal", "CudaRobustBatch", "library",
]


class GwnError(RuntimeError):
    """A non-zero status from the C ABI; ``status`` holds the code, the message the library's detail."""

    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: {_lib.STATUS.get(status, 'error')} ({status}): {detail}")
        self.status = status


def library():
    return _lib.load()


def _check(status: int, where: str):
    if status != _lib.AGWN_OK:
        detail = library().agwn_last_error_message()
        raise GwnError(status, where, detail.decode() if detail else "")


# --------------------------------------------------------------------------------------------------------------
# array plumbing
# --------------------------------------------------------------------------------------------------------------
def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _dtype_of(a):
    if _is_torch(a):
        import torch
        table = {torch.float64: np.float64, torch.float32: np.float32, torch.int32: np.int32, torch.uint8: np.uint8}
        if hasattr(torch, "uint32"):
            table[torch.uint32] = np.uint32
        return table.get(a.dtype)
    return np.asarray(a).dtype.type


class _View:
    """Pointer + element count of a contiguous array; keeps any temporary copy alive."""

    def __init__(self, a, dtype, cols: int | None, name: str, writable: bool = False):
        if _is_torch(a):
            if not a.is_contiguous():
                raise ValueError(f"{name}: tensor must be contiguous")
            if _dtype_of(a) is not dtype:
                raise TypeError(f"{name}: expected {np.dtype(dtype).name}, got {a.dtype}")
            self.keep = a
            self.ptr = a.data_ptr()
            numel = a.numel()
        else:
            if writable:
                if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
                    raise TypeError(f"{name}: output must be a C-contiguous {np.dtype(dtype).name} numpy array")
                arr = a
            else:
                arr = np.ascontiguousarray(a, dtype=dtype)
            self.keep = arr
            self.ptr = arr.ctypes.data if arr.size else None
            numel = arr.size
        if cols and numel % cols:
            raise ValueError(f"{name}: size {numel} is not a multiple of {cols}")
        self.n = numel // cols if cols else numel


def _vec3(x0, dtype):
    v = np.ascontiguousarray(np.asarray(x0.cpu() if _is_torch(x0) else x0, dtype=dtype).reshape(3))
    return v, v.ctypes.data


def _float_kind(positions):
    dt = _dtype_of(positions)
    if dt not in (np.float64, np.float32):
        raise TypeError("positions must be float64 or float32")
    return dt, ("f64" if dt is np.float64 else "f32")


# --------------------------------------------------------------------------------------------------------------
# Dispatcher / Intersector
# --------------------------------------------------------------------------------------------------------------
class CudaDispatcher:
    """The reference's Dispatcher role (src/antipodal/dispatcher/dispatcher.hh:3-36) on one GPU.

    Holds a device, a stream and scratch memory, plus the fractional-term options:
    ``precision`` "exact" (the reference's arithmetic, the default) or "mixed" (FP32 pairs with TwoSum
    accumulation and FP64 near / ill-conditioned / branch-cut pairs; double inputs), ``tau`` (mixed mode
    near-pair ratio), ``term_err`` (mixed mode per-pair FP32 error bound, radians),
    ``queries_per_thread``, ``block`` (0: automatic) and ``seg_tile`` (kernel shape), ``timing`` (CUDA-event
    kernel timing), ``mixed_min_pairs`` (below this many (query, segment) pairs per call, or on a boundary of
    fewer than 32 segments, the mixed modes run the exact kernels; 0 always runs the mixed ones; None keeps the
    library default, 2^14).
    Like PoolDispatcher it runs one job at a time.  ``parallel_for`` is not provided: arbitrary host callables
    have no device form here, and the library has no CPU fallback.
    """

    def __init__(self, device: int = 0, stream=None, precision: str = "exact", tau: float = 4.0,
                 term_err: float = 6e-8, queries_per_thread: int = 2, block: int = 0, seg_tile: int = 512,
                 timing: bool = False, mixed_min_pairs: float | None = None):
        lib = library()
        handle = None
        if stream is not None:
            handle = stream if isinstance(stream, int) else stream.cuda_stream  # torch.cuda.Stream
            if handle == 0:
                handle = 1  # cudaStreamLegacy: the legacy default stream (NULL would mean "create one")
        h = C.c_void_p()
        _check(lib.agwn_context_create(device, handle, C.byref(h)), "agwn_context_create")
        self._h = h
        self.device = device
        self.set_precision(precision)
        self.set_option(_lib.OPT_MIXED_TAU, tau)
        self.set_option(_lib.OPT_MIXED_TERM_ERR, term_err)
        self.set_option(_lib.OPT_QUERIES_PER_THREAD, queries_per_thread)
        self.set_option(_lib.OPT_FRAC_BLOCK, block)
        self.set_option(_lib.OPT_SEG_TILE, seg_tile)
        self.set_option(_lib.OPT_TIMING, 1 if timing else 0)
        if mixed_min_pairs is not None:
            self.set_option(_lib.OPT_MIXED_MIN_PAIRS, mixed_min_pairs)

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("dispatcher is closed")
        return self._h

    def set_option(self, option: int, value: float):
        _check(library().agwn_context_set_option(self.handle, option, float(value)), "agwn_context_set_option")

    def get_option(self, option: int) -> float:
        v = C.c_double()
        _check(library().agwn_context_get_option(self.handle, option, C.byref(v)), "agwn_context_get_option")
        return v.value

    def set_precision(self, precision: str):
        mode = {"exact": FRAC_EXACT, "mixed": FRAC_MIXED}[precision]
        self.set_option(_lib.OPT_FRAC_MODE, mode)
        self.precision = precision

    def synchronize(self):
        _check(library().agwn_context_synchronize(self.handle), "agwn_context_synchronize")

    def stats(self, reset: bool = False) -> dict:
        s = Stats()
        _check(library().agwn_context_get_stats(self.handle, C.byref(s), int(reset)), "agwn_context_get_stats")
        names = ["fractional", "integer", "robust", "parametric", "other"]
        return {"kernel_ms": dict(zip(names, list(s.kernel_ms))), "launches": dict(zip(names, list(s.launches))),
                "fp64_pairs": s.fp64_pairs, "pairs": s.pairs, "certified_pairs": s.certified_pairs,
                "integer": {"queries": s.int_queries, "cell_entries": s.int_cell_entries, "leaves": s.int_leaves,
                            "exact_tests": s.int_exact_tests},
                "patches": {"pairs": s.patch_pairs, "cells": s.patch_cells, "pieces": s.patch_pieces,
                            "fp64_pairs": s.patch_fp64_pairs}}

    def probe_fp32_peak(self) -> float:
        """Measured FP32 FMA throughput of this GPU, TFLOP/s."""
        v = C.c_double()
        _check(library().agwn_probe_fp32_peak(self.handle, C.byref(v)), "agwn_probe_fp32_peak")
        return v.value

    def set_robust_precision(self, precision: str):
        """Robust evaluator's fractional term: "exact" (default; the reference's FP64 arithmetic) or "mixed".  Under
        int64_grid, mixed evaluates FP32 pairs on the exact integer differences under a first-order error estimate
        (term bound: the robust term error option); under exact_float with double queries it runs the mesh
        functions' mixed kernel along -x (term bound: the mixed term error option).  The pairs turned down take the
        evaluator's own FP64 rule.  Counts are unchanged; int128_grid stays exact."""
        modes = {"exact": _lib.ROBUST_EXACT, "mixed": _lib.ROBUST_MIXED}
        if precision not in modes:
            raise ValueError("robust precision must be 'exact' or 'mixed'")
        self.set_option(_lib.OPT_ROBUST_MODE, modes[precision])

    def set_param_precision(self, precision: str):
        """Parametric integrator: "exact" (default; FP64 in the reference's operation order, bit for bit) or
        "mixed" (double-float arithmetic on the FP32 pipe, about 44 significant bits, same tree rule)."""
        modes = {"exact": _lib.PARAM_EXACT, "mixed": _lib.PARAM_MIXED}
        if precision not in modes:
            raise ValueError("parametric precision must be 'exact' or 'mixed'")
        self.set_option(_lib.OPT_PARAM_MODE, modes[precision])

    def set_robust_term_err(self, radians: float):
        """Robust mixed mode: per-pair error estimate above which a pair is evaluated in FP64 (default 1e-7)."""
        self.set_option(_lib.OPT_ROBUST_TERM_ERR, float(radians))

    def probe_fp64_peak(self) -> float:
        """Measured FP64 FMA throughput of this GPU, TFLOP/s."""
        v = C.c_double()
        _check(library().agwn_probe_fp64_peak(self.handle, C.byref(v)), "agwn_probe_fp64_peak")
        return v.value

    def parallel_for(self, begin, end, f):  # noqa: D401 - concept member, deliberately unavailable
        raise TypeError("CudaDispatcher runs the library's GWN kernels only; generic host callables are not "
                        "executed (no CPU fallback)")

    def close(self):
        if getattr(self, "_h", None) is not None:
            library().agwn_context_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CudaIntersector:
    """The reference's Intersector role (src/antipodal/intersector/intersector.hh:3-40) over a device LBVH.

    Counts equal NaiveIntersector<T>'s (intersector.hh:55-100) bit for bit.  Unlike NaiveIntersector it copies
    the mesh to the device, so the caller's arrays need not outlive it.
    """

    def __init__(self, dispatcher: CudaDispatcher, vertices, indices):
        dt = _dtype_of(vertices)
        if dt not in (np.float64, np.float32):
            raise TypeError("vertices must be float64 or float32")
        self.dtype = dt
        self.kind = "f64" if dt is np.float64 else "f32"
        v = _View(vertices, dt, 3, "vertices")
        i = _View(indices, np.int32, None, "indices")
        if i.n % 3:
            raise ValueError("indices: length must be a multiple of 3")
        h = C.c_void_p()
        fn = getattr(library(), f"agwn_bvh_create_{self.kind}")
        _check(fn(dispatcher.handle, v.ptr, v.n, i.ptr, i.n, C.byref(h)), "agwn_bvh_create")
        self._h = h
        self.n_triangles = i.n // 3

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("intersector is closed")
        return self._h

    def info(self) -> dict:
        n = C.c_int64()
        d = C.c_int32()
        _check(library().agwn_bvh_info(self.handle, C.byref(n), C.byref(d)), "agwn_bvh_info")
        return {"triangles": n.value, "depth": d.value}

    def close(self):
        if getattr(self, "_h", None) is not None:
            library().agwn_bvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CudaRobustMeshGwn:
    """RobustMeshGwn<T, Precision> (src/antipodal/gwn_mesh_robust.hh:170-424) on the device.

    ``precision`` is "int64_grid", "int128_grid" or "exact_float"; None picks the reference's default
    (int64_grid for float32 geometry, exact_float for float64).  Counts equal the reference's bit for bit.
    """

    POLICIES = {"int64_grid": 0, "int128_grid": 1, "exact_float": 2}

    def __init__(self, dispatcher: CudaDispatcher, vertices, indices, boundary, precision: str | None = None):
        dt = _dtype_of(vertices)
        if dt not in (np.float64, np.float32):
            raise TypeError("vertices must be float64 or float32")
        self.dtype = dt
        self.kind = "f64" if dt is np.float64 else "f32"
        self.precision = precision or ("exact_float" if dt is np.float64 else "int64_grid")
        v = _View(vertices, dt, 3, "vertices")
        i = _View(indices, np.int32, None, "indices")
        b = _View(boundary, dt, 7, "boundary")
        h = C.c_void_p()
        fn = getattr(library(), f"agwn_robust_create_{self.kind}")
        _check(fn(dispatcher.handle, self.POLICIES[self.precision], v.ptr, v.n, i.ptr, i.n, b.ptr, b.n, C.byref(h)),
               "agwn_robust_create")
        self._h = h
        self.dispatcher = dispatcher

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("evaluator is closed")
        return self._h

    @staticmethod
    def axis():
        """The fixed ray direction of the integer term (gwn_mesh_robust.hh:226)."""
        return np.array([-1.0, 0.0, 0.0])

    def info(self) -> dict:
        c = (C.c_double * 3)()
        sc = C.c_double()
        d = C.c_int32()
        _check(library().agwn_robust_info(self.handle, C.cast(c, C.c_void_p), C.byref(sc), C.byref(d)),
               "agwn_robust_info")
        return {"center": list(c), "scale": sc.value, "depth": d.value}

    @staticmethod
    def grid_points(start, spacing, shape, dtype=np.float64) -> np.ndarray:
        """The points evaluate_grid uses: (start + i * spacing) per axis in double, rounded to dtype, x fastest."""
        nx, ny, nz = shape
        ax = [(np.float64(start[k]) + np.arange(n, dtype=np.float64) * np.float64(spacing[k])).astype(dtype)
              for k, n in enumerate((nx, ny, nz))]
        zz, yy, xx = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        return np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)

    def evaluate_grid(self, start, spacing, shape, out=None, counts=None, fractional=None,
                      dispatcher: CudaDispatcher | None = None):
        """eval at every point of the axis-aligned grid ``start + (ix, iy, iz) * spacing`` (see grid_points), stored
        x fastest; the integer term is rasterized per column with the exact crossing rule (no traversal)."""
        nx, ny, nz = (int(v) for v in shape)
        cells = nx * ny * nz
        if out is None:
            out = np.empty(cells, self.dtype)
        o = _View(out, self.dtype, None, "out", writable=True)
        c = _View(counts, np.int32, None, "counts", writable=True) if counts is not None else None
        f = _View(fractional, self.dtype, None, "fractional", writable=True) if fractional is not None else None
        if o.n != cells or (c and c.n != cells) or (f and f.n != cells):
            raise ValueError("outputs must hold one value per grid cell")
        s = np.ascontiguousarray(start, np.float64).reshape(3)
        h = np.ascontiguousarray(spacing, np.float64).reshape(3)
        d = dispatcher or self.dispatcher
        fn = getattr(library(), f"agwn_robust_eval_grid_{self.kind}")
        _check(fn(d.handle, self.handle, s.ctypes.data, h.ctypes.data, nx, ny, nz, o.ptr, c.ptr if c else None,
                  f.ptr if f else None), "agwn_robust_eval_grid")
        return out

    def evaluate(self, positions, out=None, counts=None, fractional=None, dispatcher: CudaDispatcher | None = None):
        """Full GWN per query (and optionally the integer count and the fractional term)."""
        p = _View(positions, self.dtype, 3, "positions")
        if out is None:
            out = np.empty(p.n, self.dtype)
        o = _View(out, self.dtype, None, "out", writable=True)
        c = _View(counts, np.int32, None, "counts", writable=True) if counts is not None else None
        f = _View(fractional, self.dtype, None, "fractional", writable=True) if fractional is not None else None
        if o.n != p.n or (c and c.n != p.n) or (f and f.n != p.n):
            raise ValueError("positions and outputs must have the same size")
        fn = getattr(library(), f"agwn_robust_eval_{self.kind}")
        d = dispatcher or self.dispatcher
        _check(fn(d.handle, self.handle, p.ptr, p.n, o.ptr, c.ptr if c else None, f.ptr if f else None),
               "agwn_robust_eval")
        return out

    def close(self):
        if getattr(self, "_h", None) is not None:
            library().agwn_robust_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------------------------------------------
# batch functions (src/antipodal/gwn_mesh.hh)
# --------------------------------------------------------------------------------------------------------------
def eval_gwnr_mesh_batch_fractional(dispatcher: CudaDispatcher, positions, out_wnrs, x0, boundary):
    """gwn_mesh.hh:67-83: out_wnrs[i] = fractional GWN at positions[i]."""
    dt, kind = _float_kind(positions)
    p = _View(positions, dt, 3, "positions")
    o = _View(out_wnrs, dt, None, "out_wnrs", writable=True)
    if p.n != o.n:
        raise ValueError("positions and out_wnrs must have the same size")
    b = _View(boundary, dt, 7, "boundary")
    _, xp = x = _vec3(x0, dt)
    fn = getattr(library(), f"agwn_mesh_batch_fractional_{kind}")
    _check(fn(dispatcher.handle, p.ptr, p.n, o.ptr, xp, b.ptr, b.n), "eval_gwnr_mesh_batch_fractional")
    del x


def eval_gwnr_mesh_batch_integer(dispatcher: CudaDispatcher, intersector: CudaIntersector, positions, out_counts,
                                 x0):
    """gwn_mesh.hh:127-143: out_counts[i] = signed ray crossings along (positions[i], x0)."""
    dt, kind = _float_kind(positions)
    p = _View(positions, dt, 3, "positions")
    o = _View(out_counts, np.int32, None, "out_counts", writable=True)
    if p.n != o.n:
        raise ValueError("positions and out_counts must have the same size")
    _, xp = x = _vec3(x0, dt)
    fn = getattr(library(), f"agwn_mesh_batch_integer_{kind}")
    _check(fn(dispatcher.handle, intersector.handle, p.ptr, p.n, o.ptr, xp), "eval_gwnr_mesh_batch_integer")
    del x


def eval_gwnr_mesh_batch(dispatcher: CudaDispatcher, intersector: CudaIntersector | None, positions, out_wnrs, x0,
                         boundary):
    """gwn_mesh.hh:201-219: out_wnrs[i] = fractional + integer GWN, fused per query.  ``intersector`` None
    means no integer term (an all-boundary evaluation)."""
    dt, kind = _float_kind(positions)
    p = _View(positions, dt, 3, "positions")
    o = _View(out_wnrs, dt, None, "out_wnrs", writable=True)
    if p.n != o.n:
        raise ValueError("positions and out_wnrs must have the same size")
    b = _View(boundary, dt, 7, "boundary")
    _, xp = x = _vec3(x0, dt)
    fn = getattr(library(), f"agwn_mesh_batch_{kind}")
    ih = intersector.handle if intersector is not None else None
    _check(fn(dispatcher.handle, ih, p.ptr, p.n, o.ptr, xp, b.ptr, b.n), "eval_gwnr_mesh_batch")
    del x


def eval_gwnr_mesh_batch_integer_bruteforce(dispatcher: CudaDispatcher, vertices, indices, positions, out_counts,
                                            x0, out_ties=None):
    """Every query against every triangle (no hierarchy); double precision only.  With ``out_ties`` (int32, one per
    query) also the number of counted hits that lie exactly on a triangle's edge or vertex, or at the query: the
    queries whose NaiveIntersector counts include its double count at shared edges."""
    p = _View(positions, np.float64, 3, "positions")
    o = _View(out_counts, np.int32, None, "out_counts", writable=True)
    v = _View(vertices, np.float64, 3, "vertices")
    i = _View(indices, np.int32, None, "indices")
    _, xp = x = _vec3(x0, np.float64)
    if out_ties is None:
        _check(library().agwn_mesh_batch_integer_bruteforce_f64(dispatcher.handle, v.ptr, v.n, i.ptr, i.n, p.ptr,
                                                                p.n, o.ptr, xp), "bruteforce")
    else:
        t = _View(out_ties, np.int32, None, "out_ties", writable=True)
        if t.n != p.n:
            raise ValueError("out_ties needs one entry per query")
        _check(library().agwn_mesh_batch_integer_ties_f64(dispatcher.handle, v.ptr, v.n, i.ptr, i.n, p.ptr, p.n,
                                                          o.ptr, t.ptr, xp), "bruteforce with ties")
    del x


def build_boundary_segments(dispatcher: CudaDispatcher, vertices, indices):
    """build_boundary_segments (src/antipodal/math/common.hh:123-174) on the device: the open boundary as (s, 7)
    [pos0, pos1, weight] rows in ascending (lo, hi) vertex order.  Returns a numpy array for host vertices and a
    CUDA tensor for CUDA vertices."""
    dt, kind = _float_kind(vertices)
    v = _View(vertices, dt, 3, "vertices")
    i = _View(indices, np.int32, None, "indices")
    fn = getattr(library(), f"agwn_build_boundary_segments_{kind}")
    cnt = C.c_int64()
    _check(fn(dispatcher.handle, v.ptr, v.n, i.ptr, i.n, None, 0, C.byref(cnt)), "build_boundary_segments")
    out = _empty_like_input(vertices, (cnt.value, 7), dt)
    o = _View(out, dt, None, "out", writable=True)
    _check(fn(dispatcher.handle, v.ptr, v.n, i.ptr, i.n, o.ptr, cnt.value, C.byref(cnt)), "build_boundary_segments")
    return out


class CudaRobustBatch:
    """Many CudaRobustMeshGwn meshes with their own query arrays, evaluated in one persistent launch.

    Equivalent to ``eval_gwnr_mesh_batch_robust(disp, meshes[i], positions[i], outs[i])`` for every i, bit for
    bit (no reference counterpart for the batching itself).  positions / outs / counts are CUDA tensors, kept
    alive by this object; the meshes must stay open while it is used.  ``tune()`` picks the launch configuration
    by timing every candidate; ``run(graph=True)`` replays a captured CUDA graph after the first call.
    """

    def __init__(self, dispatcher: CudaDispatcher, meshes, positions, outs, counts=None):
        if not (len(meshes) == len(positions) == len(outs)) or not meshes:
            raise ValueError("one positions and one out array per mesh")
        if counts is not None and len(counts) != len(meshes):
            raise ValueError("one counts array per mesh")
        self.dispatcher = dispatcher
        self._keep = []
        pp, nq, oo, cc = [], [], [], []
        for i, (m, p, o) in enumerate(zip(meshes, positions, outs)):
            if not (_is_torch(p) and p.is_cuda and _is_torch(o) and o.is_cuda):
                raise TypeError(f"mesh {i}: positions and out must be CUDA tensors")
            pv = _View(p, m.dtype, 3, f"positions[{i}]")
            ov = _View(o, m.dtype, None, f"out[{i}]", writable=True)
            if pv.n != ov.n:
                raise ValueError(f"mesh {i}: positions and out sizes differ")
            cv = None
            if counts is not None and counts[i] is not None:
                cv = _View(counts[i], np.int32, None, f"counts[{i}]", writable=True)
                if cv.n != pv.n:
                    raise ValueError(f"mesh {i}: counts size differs")
            self._keep += [pv, ov, cv]
            pp.append(pv.ptr or 0)
            nq.append(pv.n)
            oo.append(ov.ptr or 0)
            cc.append(cv.ptr if cv else 0)
        n = len(meshes)
        self._meshes = list(meshes)
        arr_m = (C.c_void_p * n)(*[m.handle.value for m in meshes])
        arr_p = (C.c_void_p * n)(*pp)
        arr_n = (C.c_int64 * n)(*nq)
        arr_o = (C.c_void_p * n)(*oo)
        arr_c = (C.c_void_p * n)(*cc) if counts is not None else None
        h = C.c_void_p()
        _check(library().agwn_batch_create(dispatcher.handle, C.cast(arr_m, C.c_void_p), n, C.cast(arr_p, C.c_void_p),
                                           C.cast(arr_n, C.c_void_p), C.cast(arr_o, C.c_void_p),
                                           C.cast(arr_c, C.c_void_p) if arr_c is not None else None, C.byref(h)),
               "agwn_batch_create")
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("batch is closed")
        return self._h

    def tune(self, repeats: int = 2) -> dict:
        _check(library().agwn_batch_tune(self.dispatcher.handle, self.handle, int(repeats)), "agwn_batch_tune")
        return self.info()

    def set_config(self, block: int, k: int, seg_tile: int, stack: int):
        cfg = (C.c_int32 * 4)(block, k, seg_tile, stack)
        _check(library().agwn_batch_set_config(self.handle, C.cast(cfg, C.c_void_p)), "agwn_batch_set_config")

    def info(self) -> dict:
        cfg = (C.c_int32 * 4)()
        ncap = C.c_int32(64)
        ms = (C.c_double * 64)()
        items, tq, tp = C.c_int64(), C.c_int64(), C.c_double()
        _check(library().agwn_batch_info(self.handle, C.cast(cfg, C.c_void_p), C.byref(ncap), C.cast(ms, C.c_void_p),
                                         C.byref(items), C.byref(tq), C.byref(tp)), "agwn_batch_info")
        return {"config": {"block": cfg[0], "k": cfg[1], "seg_tile": cfg[2], "stack": cfg[3]},
                "candidates": ncap.value, "tune_ms": list(ms[:min(ncap.value, 64)]), "items": items.value,
                "queries": tq.value, "pairs": tp.value}

    def run(self, graph: bool = True):
        _check(library().agwn_batch_run(self.dispatcher.handle, self.handle, 1 if graph else 0), "agwn_batch_run")

    def close(self):
        if getattr(self, "_h", None) is not None:
            library().agwn_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eval_gwnr_mesh_batch_robust(dispatcher: CudaDispatcher, robust: CudaRobustMeshGwn, positions, out_wnrs):
    """gwn_mesh_robust.hh:441-456: out_wnrs[i] = robust.eval(positions[i])."""
    robust.evaluate(positions, out_wnrs, dispatcher=dispatcher)


# --------------------------------------------------------------------------------------------------------------
# parametric surfaces (src/antipodal/gwn_parametric.hh)
# --------------------------------------------------------------------------------------------------------------
class IntegrateConfig:
    """integrate_config (src/antipodal/math/integrate.hh:11-22): min_depth, max_depth, tol (halved per level)."""

    def __init__(self, min_depth: int = 0, max_depth: int = 10, tol: float = 1e-6):
        self.min_depth, self.max_depth, self.tol = int(min_depth), int(max_depth), float(tol)

    def __repr__(self):
        return f"IntegrateConfig(min_depth={self.min_depth}, max_depth={self.max_depth}, tol={self.tol:g})"


class IntegratorGK15:
    """The plain adaptive G7-K15 integrator (src/antipodal/math/integrate_gk15.hh:63-290), run on the device."""

    def start_depths(self, dispatcher, positions, x0, curves, cfg):
        return None


def unpack_pair_stats(stats):
    """Split agwn_param_batch_fractional_bezier3_f64's packed per-pair stats into (leaves, shallowest leaf depth,
    deepest leaf depth)."""
    s = np.asarray(stats.cpu() if _is_torch(stats) else stats).astype(np.uint32)
    return (s & 0xFFFF).astype(np.int32), ((s >> 16) & 0xFF).astype(np.int32), (s >> 24).astype(np.int32)


def eval_gwnr_parametric_batch_fractional(dispatcher: CudaDispatcher, positions, out_wnrs, x0, curves,
                                          cfg: IntegrateConfig | None = None, integrator=None, *, start_depth=None,
                                          pair_stats=None, nodes_per_query=None):
    """gwn_parametric.hh:168-186 for boundaries of cubic Bezier curves: out_wnrs[i] = (sum over curves of the
    adaptive GK15 integral of w - d_eta over [0, 1]) / (4 pi).

    curves: (c, 12) or (c, 4, 3) float64 control points, in the order for_each_boundary visits them.
    integrator: IntegratorGK15 (default, the plain method) or an object with a start_depths(...) method returning
    per-(query, curve) start depths (the learned proposal); start_depth may also be given directly as an
    (n, c) uint8 array.  pair_stats (n, c) uint32 and nodes_per_query (n,) int32 are optional outputs."""
    cfg = cfg or IntegrateConfig()
    p = _View(positions, np.float64, 3, "positions")
    o = _View(out_wnrs, np.float64, None, "out_wnrs", writable=True)
    if p.n != o.n:
        raise ValueError("positions and out_wnrs must have the same size")
    c = _View(curves, np.float64, 12, "curves")
    learned = start_depth is None and isinstance(integrator, LearnedGK15Proposal)
    if start_depth is None and integrator is not None and not learned:
        start_depth = integrator.start_depths(dispatcher, positions, x0, curves, cfg)
    sd = _View(start_depth, np.uint8, None, "start_depth") if start_depth is not None else None
    if sd is not None and sd.n != p.n * c.n:
        raise ValueError("start_depth must hold one byte per (query, curve) pair")
    st_dt = np.int32 if pair_stats is not None and _dtype_of(pair_stats) is np.int32 else np.uint32  # same bits
    st = _View(pair_stats, st_dt, None, "pair_stats", writable=True) if pair_stats is not None else None
    if st is not None and st.n != p.n * c.n:
        raise ValueError("pair_stats must hold one entry per (query, curve) pair")
    nd = _View(nodes_per_query, np.int32, None, "nodes_per_query", writable=True) \
        if nodes_per_query is not None else None
    if nd is not None and nd.n != p.n:
        raise ValueError("nodes_per_query must hold one entry per query")
    _, xp = x = _vec3(x0, np.float64)
    if learned:  # propose and integrate in one call; the start depths stay in device scratch
        fn = library().agwn_param_batch_fractional_learned_bezier3_f64
        panel = integrator.panel
        if panel is not None:
            _check(library().agwn_param_set_panel_network(dispatcher.handle, panel.handle, panel.alpha),
                   "agwn_param_set_panel_network")
        try:
            _check(fn(dispatcher.handle, integrator.handle, p.ptr, p.n, o.ptr, xp, c.ptr, c.n, integrator.n_classes,
                      cfg.min_depth, cfg.max_depth, cfg.tol, integrator.alpha, st.ptr if st else None,
                      nd.ptr if nd else None), "eval_gwnr_parametric_batch_fractional")
        finally:
            if panel is not None:
                library().agwn_param_set_panel_network(dispatcher.handle, None, C.c_float(0.5))
    else:
        fn = library().agwn_param_batch_fractional_bezier3_f64
        _check(fn(dispatcher.handle, p.ptr, p.n, o.ptr, xp, c.ptr, c.n, cfg.min_depth, cfg.max_depth, cfg.tol,
                  sd.ptr if sd else None, st.ptr if st else None, nd.ptr if nd else None),
               "eval_gwnr_parametric_batch_fractional")
    del x


class CudaBezierPatchIntersector:
    """The Intersector role for parametric surfaces made of bicubic Bezier patches: the integer term that
    eval_gwnr_parametric_batch_integer / eval_gwnr_parametric_batch forward to (gwn_parametric.hh:204-284; the
    reference ships no parametric intersector).  Each crossing of the ray p + lambda x0 (lambda > 0) counts
    sign(N . x0) with N = S_u x S_v, the orientation under which boundary curves running counter-clockwise in (u, v)
    (synth.bezier_patch_boundary) make fractional + integer the winding number.

    patches: (n, 4, 4, 3) or (n, 48) float64 control points P[patch][v index][u index][xyz]; copied to the
    device."""

    def __init__(self, dispatcher: CudaDispatcher, patches):
        self._disp = dispatcher
        c = _View(patches, np.float64, 48, "patches")
        h = C.c_void_p()
        _check(library().agwn_patches_create_f64(dispatcher.handle, c.ptr, c.n, C.byref(h)), "agwn_patches_create_f64")
        self._h = h
        self.n = c.n

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("intersector is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            library().agwn_patches_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eval_gwnr_parametric_batch_integer(dispatcher: CudaDispatcher, intersector: CudaBezierPatchIntersector,
                                       positions, out_counts, x0, out_degenerate=None):
    """gwn_parametric.hh:210-226: out_counts[i] = intersector.signed_intersection_count(positions[i], x0).  With
    ``out_degenerate`` (int32, one per query): how many of the query's decisions were degenerate (the ray on a
    patch cell's boundary image, or the query on the surface, within 2^-42 of the coordinates' scale)."""
    p = _View(positions, np.float64, 3, "positions")
    o = _View(out_counts, np.int32, None, "out_counts", writable=True)
    if p.n != o.n:
        raise ValueError("positions and out_counts must have the same size")
    _, xp = x = _vec3(x0, np.float64)
    if out_degenerate is None:
        _check(library().agwn_param_batch_integer_bezier3x3_f64(dispatcher.handle, intersector.handle, p.ptr, p.n,
                                                                o.ptr, xp), "eval_gwnr_parametric_batch_integer")
    else:
        d = _View(out_degenerate, np.int32, None, "out_degenerate", writable=True)
        if d.n != p.n:
            raise ValueError("out_degenerate needs one entry per query")
        _check(library().agwn_param_batch_integer_degenerate_bezier3x3_f64(dispatcher.handle, intersector.handle,
                                                                           p.ptr, p.n, o.ptr, d.ptr, xp),
               "eval_gwnr_parametric_batch_integer")
    del x


def eval_gwnr_parametric_batch(dispatcher: CudaDispatcher, intersector: CudaBezierPatchIntersector, positions,
                               out_wnrs, x0, curves, cfg: IntegrateConfig | None = None, integrator=None):
    """gwn_parametric.hh:259-284: out_wnrs[i] = the fractional term over the boundary curves (as
    eval_gwnr_parametric_batch_fractional, any integrator) + the patches' signed crossing count along x0."""
    eval_gwnr_parametric_batch_fractional(dispatcher, positions, out_wnrs, x0, curves, cfg, integrator)
    p = _View(positions, np.float64, 3, "positions")
    o = _View(out_wnrs, np.float64, None, "out_wnrs", writable=True)
    _, xp = x = _vec3(x0, np.float64)
    _check(library().agwn_param_add_integer_bezier3x3_f64(dispatcher.handle, intersector.handle, p.ptr, p.n, o.ptr,
                                                          xp), "eval_gwnr_parametric_batch")
    del x


class LearnedGK15Proposal:
    """Learned start depths for IntegratorGK15 on the parametric path (no counterpart in the reference).

    A 12 -> 64 -> 64 -> 16 MLP, run and trained on the GPU's tensor cores (BF16 weights and activations, FP32
    accumulation), predicts for each (query, curve) pair the shallowest depth at which the plain integrator
    accepts a panel.  Used as ``integrator=`` of eval_gwnr_parametric_batch_fractional, it only chooses where the
    plain integrator starts evaluating; every evaluated panel is still accepted or refined by the plain error
    test, so the plain method is both the fallback and the arbiter.  ``alpha`` bounds the predicted probability
    that a proposed depth overshoots the true one (an overshoot refines beyond the plain tree; it never skips the
    error test).  The label is the shallowest accepted depth, a lower bound on the cheapest start depth, so a large
    alpha is the faster one: on 256-patch workloads, 0.9 evaluates 26% fewer panels than no proposal against 15%
    at the default 0.02.
    """

    FORMAT = 2

    def __init__(self, dispatcher: CudaDispatcher, seed: int = 0, n_classes: int = 11, alpha: float = 0.02,
                 params=None):
        self.dispatcher = dispatcher
        self.n_classes = int(n_classes)
        self.alpha = float(alpha)
        self.panel = None  # optional per-panel network (2 classes; its alpha is the skip threshold beta)
        h = C.c_void_p()
        _check(library().agwn_mlp_create(dispatcher.handle, int(seed) & 0xFFFFFFFFFFFFFFFF, C.byref(h)),
               "agwn_mlp_create")
        self._h = h
        if params is not None:
            self.params = params

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("network is closed")
        return self._h

    @property
    def params(self) -> np.ndarray:
        out = np.empty(library().agwn_mlp_param_count(), np.float32)
        _check(library().agwn_mlp_get_params(self.dispatcher.handle, self.handle, out.ctypes.data),
               "agwn_mlp_get_params")
        return out

    @params.setter
    def params(self, value):
        v = np.ascontiguousarray(value, np.float32).ravel()
        if v.size != library().agwn_mlp_param_count():
            raise ValueError(f"expected {library().agwn_mlp_param_count()} parameters, got {v.size}")
        _check(library().agwn_mlp_set_params(self.dispatcher.handle, self.handle, v.ctypes.data),
               "agwn_mlp_set_params")

    def save(self, path):
        """Write the FP32 weights and the decision settings (the only state the proposal has) to an .npz file."""
        extra = {}
        if self.panel is not None:
            extra = {"panel_params": self.panel.params, "panel_beta": self.panel.alpha}
        np.savez(path, params=self.params, n_classes=self.n_classes, alpha=self.alpha, format=self.FORMAT, **extra)

    @classmethod
    def load(cls, dispatcher: CudaDispatcher, path):
        z = np.load(path)
        if int(z["format"]) not in (1, cls.FORMAT):
            raise ValueError(f"{path}: unsupported format {int(z['format'])}")
        net = cls(dispatcher, n_classes=int(z["n_classes"]), alpha=float(z["alpha"]), params=z["params"])
        if "panel_params" in z.files:
            net.panel = cls(dispatcher, n_classes=2, alpha=float(z["panel_beta"]), params=z["panel_params"])
        return net

    # -- the per-panel network ----------------------------------------------------------------------------------
    def panel_data(self, positions, x0, curves, cfg: IntegrateConfig, capacity: int = 4_000_000):
        """Features and labels (accepted or split) of the panels the integrator evaluates (in the dispatcher's
        parametric arithmetic), up to ``capacity`` of them."""
        p = _View(positions, np.float64, 3, "positions")
        c = _View(curves, np.float64, 12, "curves")
        log = _empty_like_input(positions, (int(capacity), 2), np.int32)  # uint32 words, same bits
        lv = _View(log, np.int32, None, "log", writable=True)
        _, xp = x = _vec3(x0, np.float64)
        cnt = C.c_int64()
        _check(library().agwn_param_panel_log_bezier3_f64(self.dispatcher.handle, p.ptr, p.n, xp, c.ptr, c.n,
                                                          cfg.min_depth, cfg.max_depth, cfg.tol, lv.ptr,
                                                          int(capacity), C.byref(cnt)), "agwn_param_panel_log")
        m = min(cnt.value, int(capacity))
        feats = _empty_like_input(positions, (m, 12), np.float32)
        labels = _empty_like_input(positions, (m,), np.uint8)
        fv = _View(feats, np.float32, None, "features", writable=True)
        lb = _View(labels, np.uint8, None, "labels", writable=True)
        if m:
            _check(library().agwn_param_panel_features_bezier3_f64(self.dispatcher.handle, p.ptr, p.n, xp, c.ptr, c.n,
                                                                   cfg.tol, lv.ptr, m, fv.ptr, lb.ptr),
                   "agwn_param_panel_features")
        del x
        return feats, labels

    def fit_panels(self, positions, x0, curves, cfg: IntegrateConfig, beta: float = 0.02, capacity: int = 4_000_000,
                   seed: int = 7, **train_kw):
        """Train the per-panel network (split or accept) on the integrator's own panels; returns the loss history."""
        feats, labels = self.panel_data(positions, x0, curves, cfg, capacity)
        if self.panel is None:
            self.panel = LearnedGK15Proposal(self.dispatcher, seed=seed, n_classes=2, alpha=beta)
        self.panel.alpha = float(beta)
        return self.panel.train(feats, labels, **train_kw)

    # -- data ---------------------------------------------------------------------------------------------------
    def features(self, positions, x0, curves, tol: float):
        """The 12 features of every (query, curve) pair, (n * c, 12) float32 (a device tensor for device input)."""
        p = _View(positions, np.float64, 3, "positions")
        c = _View(curves, np.float64, 12, "curves")
        out = _empty_like_input(positions, (p.n * c.n, 12), np.float32)
        o = _View(out, np.float32, None, "features", writable=True)
        _, xp = x = _vec3(x0, np.float64)
        _check(library().agwn_param_features_bezier3_f64(self.dispatcher.handle, p.ptr, p.n, xp, c.ptr, c.n,
                                                         float(tol), o.ptr), "agwn_param_features_bezier3_f64")
        del x
        return out

    def labels(self, positions, x0, curves, cfg: IntegrateConfig):
        """Training labels: the plain integrator's shallowest accepted depth for every pair, (n * c,) uint8."""
        p = _View(positions, np.float64, 3, "positions")
        c = _View(curves, np.float64, 12, "curves")
        stats = _empty_like_input(positions, (p.n, c.n), np.uint32)
        out = _empty_like_input(positions, (p.n,), np.float64)
        eval_gwnr_parametric_batch_fractional(self.dispatcher, positions, out, x0, curves, cfg, pair_stats=stats)
        if _is_torch(stats):
            return ((stats.view(-1).to(__import__("torch").int64) >> 16) & 0xFF).to(__import__("torch").uint8)
        return ((stats.ravel() >> 16) & 0xFF).astype(np.uint8)

    # -- training -----------------------------------------------------------------------------------------------
    def loss_grad(self, features, labels):
        """Mean cross-entropy and its gradient on the given rows, from the device training kernels."""
        f = _View(features, np.float32, 12, "features")
        lb = _View(labels, np.uint8, None, "labels")
        if lb.n != f.n:
            raise ValueError("one label per feature row")
        g = np.empty(library().agwn_mlp_param_count(), np.float32)
        loss = C.c_double()
        _check(library().agwn_mlp_loss_grad(self.dispatcher.handle, self.handle, f.ptr, lb.ptr, f.n, self.n_classes,
                                            g.ctypes.data, C.byref(loss)), "agwn_mlp_loss_grad")
        return loss.value, g

    def train(self, features, labels, steps: int = 3000, batch: int = 8192, lr: float = 2e-3, seed: int = 1):
        """Adam on mini-batches drawn from (features, labels); returns each step's mean loss."""
        f = _View(features, np.float32, 12, "features")
        lb = _View(labels, np.uint8, None, "labels")
        if lb.n != f.n:
            raise ValueError("one label per feature row")
        hist = np.empty(max(int(steps), 0), np.float32)
        _check(library().agwn_mlp_train(self.dispatcher.handle, self.handle, f.ptr, lb.ptr, f.n, self.n_classes,
                                        int(steps), int(batch), float(lr), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                        hist.ctypes.data if hist.size else None), "agwn_mlp_train")
        return hist

    def fit(self, positions, x0, curves, cfg: IntegrateConfig, **train_kw):
        """Label (query, curve) pairs with the plain integrator, compute their features and train on them."""
        lab = self.labels(positions, x0, curves, cfg)
        feat = self.features(positions, x0, curves, cfg.tol)
        return self.train(feat, lab, **train_kw)

    # -- inference ----------------------------------------------------------------------------------------------
    def start_depths(self, dispatcher, positions, x0, curves, cfg: IntegrateConfig, logits=None):
        """Proposed start depth of every pair, (n, c) uint8 (a device tensor for device input)."""
        p = _View(positions, np.float64, 3, "positions")
        c = _View(curves, np.float64, 12, "curves")
        out = _empty_like_input(positions, (p.n, c.n), np.uint8)
        o = _View(out, np.uint8, None, "start_depth", writable=True)
        lg = _View(logits, np.float32, 16, "logits", writable=True) if logits is not None else None
        _, xp = x = _vec3(x0, np.float64)
        _check(library().agwn_param_propose_depth_bezier3_f64(
            dispatcher.handle, self.handle, p.ptr, p.n, xp, c.ptr, c.n, self.n_classes, cfg.min_depth, cfg.max_depth,
            cfg.tol, self.alpha, o.ptr, lg.ptr if lg else None), "agwn_param_propose_depth_bezier3_f64")
        del x
        return out

    def close(self):
        if getattr(self, "panel", None) is not None:
            self.panel.close()
            self.panel = None
        if getattr(self, "_h", None) is not None:
            library().agwn_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _empty_like_input(like, shape, dtype):
    """An output array on the same side (host numpy / device torch) as the input ``like``."""
    if _is_torch(like) and like.is_cuda:
        import torch
        tdt = {np.float32: torch.float32, np.float64: torch.float64, np.uint8: torch.uint8, np.int32: torch.int32}
        if dtype is np.uint32:
            return torch.empty(shape, dtype=torch.int32, device=like.device)  # same bits, viewed as uint32
        return torch.empty(shape, dtype=tdt[dtype], device=like.device)
    return np.empty(shape, dtype)
