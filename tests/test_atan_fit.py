"""Provenance of the mixed kernels' float atan: re-derives the polynomial of atan_unit (csrc/frac_kernels.cuh) on
the CPU and checks that the kernel's coefficients are that fit.

The kernels evaluate atan(t) = t * P(t^2) on [0, 1] with P of degree 8 in s = t^2.  P is the minimax polynomial of
f(s) = atan(sqrt(s)) / sqrt(s) on s in [0, 1] under relative error, which is the relative error of atan(t) itself.
This test finds it with the Remez exchange algorithm in 40-digit arithmetic: solve for P and the levelled error E
on n + 2 alternation points, move the points to the extrema of the weighted error, repeat until the largest error
equals |E|.  The GPU error test of the whole atan2 (against FP64 and CUDA's atan2f) is in test_mesh_gpu.py.
"""

import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KERNELS = os.path.join(ROOT, "antipodal_gb300", "csrc", "frac_kernels.cuh")
DEGREE = 8


def kernel_coefficients():
    """The coefficients of both copies of the polynomial (scalar and lane vector), highest degree first."""
    text = open(KERNELS).read()
    out = []
    for name in ("float atan_unit(float t)", "V atan_unit_lv(V t)"):
        body = text[text.index(name):]
        body = body[:body.index("return")]
        out.append([float(x) for x in re.findall(r"(-?\d+\.\d+(?:e-?\d+)?)f", body)])
    return out


def remez_relative(degree: int):
    """Minimax P (coefficients, lowest degree first) of atan(sqrt(s))/sqrt(s) on [0, 1] under relative error, and
    the levelled error E."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40

    def f(s):
        if s == 0:
            return mp.mpf(1)
        r = mp.sqrt(s)
        return mp.atan(r) / r

    m = degree + 2
    xs = [(1 - mp.cos(mp.pi * i / (m - 1))) / 2 for i in range(m)]  # Chebyshev extrema on [0, 1]
    grid_n = 2000
    grid = [mp.mpf(k) / grid_n for k in range(grid_n + 1)]
    for _ in range(30):
        a = mp.matrix(m, m)
        b = mp.matrix(m, 1)
        for i, x in enumerate(xs):
            for j in range(degree + 1):
                a[i, j] = x ** j
            a[i, degree + 1] = (-1) ** i * f(x)  # (P(x) - f(x)) / f(x) = (-1)^i E
            b[i] = f(x)
        sol = mp.lu_solve(a, b)
        c = [sol[j] for j in range(degree + 1)]
        e_lev = sol[degree + 1]

        def err(s):
            return (sum(c[j] * s ** j for j in range(degree + 1)) - f(s)) / f(s)

        ev = [err(g) for g in grid]
        cand = [0] + [k for k in range(1, grid_n) if (ev[k] - ev[k - 1]) * (ev[k + 1] - ev[k]) <= 0] + [grid_n]
        pts = []
        for k in cand:
            if k in (0, grid_n):
                pts.append(grid[k])
                continue
            lo, hi = grid[k - 1], grid[k + 1]
            sgn = 1 if ev[k] > 0 else -1
            for _ in range(60):  # golden-section search for the extremum in the bracket
                m1, m2 = lo + (hi - lo) * 0.382, lo + (hi - lo) * 0.618
                if -sgn * err(m1) < -sgn * err(m2):
                    hi = m2
                else:
                    lo = m1
            pts.append((lo + hi) / 2)
        alt = []
        for p in pts:  # one point per sign run, the largest
            v = err(p)
            if alt and mp.sign(alt[-1][1]) == mp.sign(v):
                if abs(v) > abs(alt[-1][1]):
                    alt[-1] = (p, v)
            else:
                alt.append((p, v))
        while len(alt) > m:
            alt.pop(0 if abs(alt[0][1]) < abs(alt[-1][1]) else -1)
        largest = max(abs(v) for _, v in alt)
        if len(alt) == m:
            xs = [p for p, _ in alt]
        if abs(largest - abs(e_lev)) < 1e-12 * largest:
            break
    return [float(x) for x in c], float(abs(e_lev)), float(largest)


def test_both_copies_of_the_polynomial_agree():
    scalar, lanes = kernel_coefficients()
    assert len(scalar) == DEGREE + 1
    assert scalar == lanes


def test_kernel_coefficients_are_the_relative_minimax_fit():
    scalar, _ = kernel_coefficients()
    c, e_lev, largest = remez_relative(DEGREE)
    # converged: the error levels out, at the 1.5e-8 the kernel's comment states
    assert abs(largest - e_lev) <= 1e-9 * e_lev
    assert 1.5e-8 <= e_lev <= 1.55e-8
    derived = np.array(c[::-1])
    kernel = np.array(scalar)
    # the kernels hold float32 constants: each derived coefficient rounds to the kernel's float, or its neighbour
    d32, k32 = derived.astype(np.float32), kernel.astype(np.float32)
    ulps = np.abs(d32.view(np.int32).astype(np.int64) - k32.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1, (derived, kernel)
    assert np.max(np.abs(derived - kernel)) < 2e-11


def test_fit_in_float_meets_the_stated_bound():
    """The kernel's polynomial, evaluated with float32 Horner FMAs like the device, against FP64 atan on a dense
    sample of [0, 1]: the float evaluation adds a few ulps to the fit's 1.5e-8."""
    scalar, _ = kernel_coefficients()
    t = np.linspace(0.0, 1.0, 200_001).astype(np.float32)
    s = (t * t).astype(np.float32)
    p = np.float32(scalar[0])
    for a in scalar[1:]:
        p = (p.astype(np.float64) * s + np.float32(a)).astype(np.float32)  # one rounding per FMA
    r = (t * p).astype(np.float32).astype(np.float64)
    exact = np.arctan(t.astype(np.float64))
    nz = t > 0
    rel = np.abs(r[nz] - exact[nz]) / exact[nz]
    assert rel.max() < 3.0e-7  # a few float ulps


def small_series_coefficients():
    """The coefficients of atan_small_lv (the short series of the certified groups), highest degree first."""
    text = open(KERNELS).read()
    body = text[text.index("V atan_small_lv(V t)"):]
    body = body[:body.index("return")]
    return [float(x) for x in re.findall(r"(-?\d+\.\d*(?:e-?\d+)?)f", body)]


def test_small_series_is_the_taylor_series_and_meets_its_bound():
    """atan_small_lv evaluates atan(t) = t (1 - s/3 + s^2/5 - s^3/7) for t <= 0.125 (every pair of a certified group
    has t <= 0.101).  Its coefficients are the Taylor series' own, and evaluated in float32 Horner FMAs like the
    device it stays within a few float ulps of FP64 atan there (the truncation itself is below 6.6e-9)."""
    c = small_series_coefficients()
    assert np.allclose(c, [-1 / 7, 1 / 5, -1 / 3, 1.0], rtol=1e-7, atol=0)
    t = np.linspace(0.0, 0.125, 200_001).astype(np.float32)
    s = (t * t).astype(np.float32)
    p = np.float32(c[0])
    for a in c[1:]:
        p = (p.astype(np.float64) * s + np.float32(a)).astype(np.float32)
    r = (t * p).astype(np.float32).astype(np.float64)
    exact = np.arctan(t.astype(np.float64))
    nz = t > 0
    rel = np.abs(r[nz] - exact[nz]) / exact[nz]
    assert rel.max() < 2.0e-7
    # the truncation alone, in FP64
    t64 = np.linspace(1e-6, 0.125, 10_001)
    s64 = t64 * t64
    trunc = np.abs(t64 * (1 - s64 / 3 + s64 ** 2 / 5 - s64 ** 3 / 7) - np.arctan(t64)) / np.arctan(t64)
    assert trunc.max() < 6.6e-9
