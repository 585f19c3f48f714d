"""ctypes wrapper over the CPU oracle (test infrastructure only).

``Oracle()`` loads ``oracle/liboracle.so`` -- the restatement in ``gwn_oracle.cc`` -- and
``Oracle(reference=True)`` loads ``oracle/_ref/libref_gwn.so`` -- the antipodal reference compiled from its
own headers (only present where the reference sources were available at build time).  Both expose the same
entry points, so a test can run the same call on either and compare.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this module, as the checker or
as the timed CPU baseline.  The product package never imports it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_gwn.so")
# Where the reference's src/ directory is read from: $ANTIPODAL_REFERENCE_SRC, else the development container's
# mount of the reference.  The GPU machines have neither; every user of it falls back when it is absent.
DEFAULT_REFERENCE_SRC = "/root/reference/src"


def reference_src() -> str | None:
    """The reference's src/ directory if it exists here, else None."""
    p = os.environ.get("ANTIPODAL_REFERENCE_SRC", DEFAULT_REFERENCE_SRC)
    return p if p and os.path.isdir(p) else None

_P = C.c_void_p
_I64 = C.c_int64
_I = C.c_int
_D = C.c_double


def build(reference_src: str | None = None, quiet: bool = True) -> None:
    """Compile liboracle.so, and _ref/libref_gwn.so when ``reference_src`` (the reference's src/) exists."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-C", HERE, "all"], stdout=out)
    if reference_src and os.path.isdir(reference_src):
        subprocess.check_call(["make", "-C", HERE, "ref", f"REF_SRC={reference_src}"], stdout=out)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Oracle:
    """CPU batch GWN functions with the reference's semantics (see gwn_oracle.cc for the citations)."""

    def __init__(self, reference: bool = False, path: str | None = None):
        self.reference = reference
        self.path = path or (REF_LIB if reference else LIB)
        if not os.path.exists(self.path):
            raise FileNotFoundError(self.path)
        self.lib = C.CDLL(self.path)
        self.pre = "ref_" if reference else "orc_"
        self._declare()

    def _fn(self, name, restype, *argtypes):
        f = getattr(self.lib, self.pre + name)
        f.restype = restype
        f.argtypes = list(argtypes)
        return f

    def _declare(self):
        for suf in ("f64", "f32"):
            setattr(self, f"_frac_{suf}", self._fn(f"frac_batch_{suf}", None, _P, _I64, _P, _P, _P, _I64, _I))
            setattr(self, f"_int_{suf}", self._fn(f"int_naive_{suf}", None, _P, _I64, _P, _P, _P, _I64, _P, _I64, _I))
            setattr(self, f"_full_{suf}",
                    self._fn(f"full_naive_{suf}", None, _P, _I64, _P, _P, _P, _I64, _P, _I64, _P, _I64, _I))
            setattr(self, f"_bnd_{suf}", self._fn(f"boundary_{suf}", _I64, _P, _I64, _P, _I64, _P, _I64))
            setattr(self, f"_vos_{suf}", self._fn(f"vos_half_{suf}", _D if suf == "f64" else C.c_float, _P, _P, _P))
            if not self.reference:
                setattr(self, f"_base_{suf}", self._fn(f"gwn_baseline_{suf}", None, _P, _I64, _P, _P, _I64, _P, _I64, _I))
        self._robust = self._fn("robust_eval", _I, _I, _I, _P, _I64, _P, _I64, _P, _I64, _P, _I64, _P, _P, _P, _I)
        self._pred = self._fn("predicates", _I, _I, _P, _P, _P, _P, _I64, _P, _P, _P)
        self._pred_w = self._fn("predicate_weights", _I, _I, _P, _P, _P, _P, _I64, _P)
        self._param = self._fn("param_frac_bezier3_f64", None, _P, _I64, _P, _P, _P, _I64, _I, _I, _D, _P, _P, _I)
        self._gk15 = self._fn("gk15_known", _D, _I, _D, _D, _I, _I, _D, C.POINTER(_D), C.POINTER(_I))
        if not self.reference:
            self._patch = self._fn("patch_count_bezier3x3_f64", None, _P, _I64, _P, _P, _I64, _P, _P, _I)
        if not self.reference:
            self._feat = self._fn("param_features_bezier3", None, _P, _I64, _P, _P, _I64, _D, _P)
            self._mlp_logits = self._fn("mlp_logits", None, _P, _P, _I64, _P)
            self._mlp_grad = self._fn("mlp_loss_grad", None, _P, _P, _P, _I64, _I, _P, _P)
            self.mlp_param_count = self._fn("mlp_param_count", _I)()

    @staticmethod
    def _dt(a):
        return np.float64 if np.asarray(a).dtype == np.float64 else np.float32

    # -- mesh path ---------------------------------------------------------------------------------------------
    def vos_half(self, x1, v0, v1):
        dt = self._dt(x1)
        f = self._vos_f64 if dt == np.float64 else self._vos_f32
        return float(f(_ptr(_c(x1, dt)), _ptr(_c(v0, dt)), _ptr(_c(v1, dt))))

    def frac_batch(self, pos, x0, segs, threads=0):
        dt = self._dt(pos)
        pos, segs, x0 = _c(pos, dt), _c(segs, dt).reshape(-1, 7), _c(x0, dt)
        out = np.empty(len(pos), dt)
        f = self._frac_f64 if dt == np.float64 else self._frac_f32
        f(_ptr(pos), len(pos), _ptr(out), _ptr(x0), _ptr(segs), len(segs), threads)
        return out

    def int_naive(self, pos, dirv, verts, idx, threads=0):
        dt = self._dt(pos)
        pos, verts, dirv, idx = _c(pos, dt), _c(verts, dt), _c(dirv, dt), _c(idx, np.int32).ravel()
        out = np.empty(len(pos), np.int32)
        f = self._int_f64 if dt == np.float64 else self._int_f32
        f(_ptr(pos), len(pos), _ptr(out), _ptr(dirv), _ptr(verts), len(verts), _ptr(idx), len(idx), threads)
        return out

    def full_naive(self, pos, x0, verts, idx, segs, threads=0):
        dt = self._dt(pos)
        pos, verts, x0 = _c(pos, dt), _c(verts, dt), _c(x0, dt)
        idx, segs = _c(idx, np.int32).ravel(), _c(segs, dt).reshape(-1, 7)
        out = np.empty(len(pos), dt)
        f = self._full_f64 if dt == np.float64 else self._full_f32
        f(_ptr(pos), len(pos), _ptr(out), _ptr(x0), _ptr(verts), len(verts), _ptr(idx), len(idx), _ptr(segs),
          len(segs), threads)
        return out

    def gwn_baseline(self, pos, verts, idx, threads=0):
        dt = self._dt(pos)
        pos, verts, idx = _c(pos, dt), _c(verts, dt), _c(idx, np.int32).ravel()
        out = np.empty(len(pos), dt)
        f = self._base_f64 if dt == np.float64 else self._base_f32
        f(_ptr(pos), len(pos), _ptr(out), _ptr(verts), len(verts), _ptr(idx), len(idx), threads)
        return out

    def boundary(self, verts, idx):
        dt = self._dt(verts)
        verts, idx = _c(verts, dt), _c(idx, np.int32).ravel()
        f = self._bnd_f64 if dt == np.float64 else self._bnd_f32
        n = f(_ptr(verts), len(verts), _ptr(idx), len(idx), None, 0)
        out = np.empty((n, 7), dt)
        f(_ptr(verts), len(verts), _ptr(idx), len(idx), _ptr(out), n)
        return out

    # -- robust path -------------------------------------------------------------------------------------------
    POLICY = {"int64_grid": 0, "int128_grid": 1, "exact_float": 2}

    def robust_eval(self, policy, verts, idx, segs, pos, threads=0, want_count=True, want_frac=True):
        dt = self._dt(verts)
        verts, idx, pos = _c(verts, dt), _c(idx, np.int32).ravel(), _c(pos, dt)
        segs = _c(segs, dt).reshape(-1, 7)
        out = np.empty(len(pos), dt)
        cnt = np.empty(len(pos), np.int32) if want_count else None
        fr = np.empty(len(pos), dt) if want_frac else None
        rc = self._robust(8 if dt == np.float64 else 4, self.POLICY[policy], _ptr(verts), len(verts), _ptr(idx),
                          len(idx), _ptr(segs), len(segs), _ptr(pos), len(pos), _ptr(out), _ptr(cnt), _ptr(fr),
                          threads)
        if rc != 0:
            raise ValueError("robust_eval failed")
        return out, cnt, fr

    def predicates(self, policy, q, q0, q1, q2):
        dt = {0: np.int32, 1: np.int64, 2: np.float64}[policy]
        q, q0, q1, q2 = (_c(a, dt).reshape(-1, 3) for a in (q, q0, q1, q2))
        n = len(q)
        es, num, ins = np.empty(n, np.int32), np.empty(n, np.float64), np.empty(n, np.int32)
        if self._pred(policy, _ptr(q), _ptr(q0), _ptr(q1), _ptr(q2), n, _ptr(es), _ptr(num), _ptr(ins)) != 0:
            raise ValueError("bad policy")
        return es, num, ins

    def predicate_weights(self, policy, q, q0, q1, q2):
        """project_into_tri's weights (n, 3): (w0, w1, w2), zero where the query is outside."""
        dt = {0: np.int32, 1: np.int64, 2: np.float64}[policy]
        q, q0, q1, q2 = (_c(a, dt).reshape(-1, 3) for a in (q, q0, q1, q2))
        w = np.empty((len(q), 3), np.float64)
        if self._pred_w(policy, _ptr(q), _ptr(q0), _ptr(q1), _ptr(q2), len(q), _ptr(w)) != 0:
            raise ValueError("bad policy")
        return w

    # -- parametric path ---------------------------------------------------------------------------------------
    def patch_count_bezier3x3(self, pos, x0, patches, threads=0, degenerate=False):
        """Signed crossing counts of the rays pos + lambda x0 with bicubic Bezier patches (n, 4, 4, 3); with
        ``degenerate`` also, per query, how many decisions fell within the margin (ray on a cell edge's image,
        query on the surface)."""
        pos, x0 = _c(pos, np.float64).reshape(-1, 3), _c(x0, np.float64)
        ctrl = _c(patches, np.float64).reshape(-1, 48)
        out = np.empty(len(pos), np.int32)
        deg = np.empty(len(pos), np.int32)
        self._patch(_ptr(pos), len(pos), _ptr(x0), _ptr(ctrl), len(ctrl), _ptr(out), _ptr(deg), threads)
        return (out, deg) if degenerate else out

    def param_frac_bezier3(self, pos, x0, ctrl, min_depth=0, max_depth=10, tol=1e-6, threads=0, stats=False):
        pos, x0, ctrl = _c(pos, np.float64), _c(x0, np.float64), _c(ctrl, np.float64).reshape(-1, 12)
        out = np.empty(len(pos), np.float64)
        leaves = np.empty((len(pos), len(ctrl)), np.int32) if stats else None
        depth = np.empty((len(pos), len(ctrl)), np.int32) if stats else None
        self._param(_ptr(pos), len(pos), _ptr(out), _ptr(x0), _ptr(ctrl), len(ctrl), min_depth, max_depth, tol,
                    _ptr(leaves), _ptr(depth), threads)
        return (out, leaves, depth) if stats else out

    def gk15_known(self, fn, a, b, min_depth, max_depth, tol):
        err, leaves = _D(0.0), _I(0)
        r = self._gk15(fn, a, b, min_depth, max_depth, tol, C.byref(err), C.byref(leaves))
        return r, err.value, leaves.value

    # -- learned proposal (the network's checker; no reference counterpart) -------------------------------------
    def param_features(self, pos, x0, ctrl, tol):
        pos, x0, ctrl = _c(pos, np.float64), _c(x0, np.float64), _c(ctrl, np.float64).reshape(-1, 12)
        out = np.empty((len(pos) * len(ctrl), 12), np.float32)
        self._feat(_ptr(pos), len(pos), _ptr(x0), _ptr(ctrl), len(ctrl), tol, _ptr(out))
        return out

    def mlp_logits(self, params, feats):
        params, feats = _c(params, np.float32), _c(feats, np.float32).reshape(-1, 12)
        out = np.empty((len(feats), 16), np.float64)
        self._mlp_logits(_ptr(params), _ptr(feats), len(feats), _ptr(out))
        return out

    def mlp_loss_grad(self, params, feats, labels, n_classes):
        params, feats = _c(params, np.float32), _c(feats, np.float32).reshape(-1, 12)
        labels = _c(labels, np.uint8)
        grads = np.empty(self.mlp_param_count, np.float64)
        loss = _D(0.0)
        self._mlp_grad(_ptr(params), _ptr(feats), _ptr(labels), len(feats), n_classes, _ptr(grads), C.byref(loss))
        return loss.value, grads
