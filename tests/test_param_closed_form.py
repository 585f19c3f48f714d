"""The closed form of the parametric integrand that the double-float GK15 kernel evaluates (csrc/param.cu,
integrand_df), checked in numpy against the reference's expression (src/antipodal/gwn_parametric.hh:73-103, with
normalize_fd from src/antipodal/math/fwd_diff.hh:497-532) on the CPU.

With s = |r|, m = x0.r, T = r'.(x0 x r) and n = |x0|^2 the expression equals
-T / (s^2 + (n - 2) m^2) - m T / (s |x0 x r|^2), which is -T / (s (s - m)) for a unit x0; for m >= 0 the kernel
forms s - m as |x0 x r|^2 / (s + m).  Extended precision (np.longdouble) stands in for the exact value near the
poles, where the form of s - m decides the accuracy."""

import numpy as np
import pytest


def dot(a, b):
    return np.sum(a * b, axis=-1)


def reference_expression(r, dr, x0):
    """w - d_eta as the reference writes it, in the dtype of its arguments."""
    s = np.sqrt(dot(r, r))
    inv_s = 1 / s
    s1 = dot(r, dr) * inv_s
    G = r * inv_s[..., None]
    Gp = (dr - G * s1[..., None]) * inv_s[..., None]
    a, ap = dot(x0, G), dot(x0, Gp)
    X = x0 - G * a[..., None]
    Xp = -(G * ap[..., None] + Gp * a[..., None])
    d_eta = dot(G, np.cross(X, Xp)) / dot(X, X)
    x1 = -x0
    b, bp = dot(x1, G), dot(x1, Gp)
    v = G - x1 * b[..., None]
    vp = Gp - x1 * bp[..., None]
    w = dot(x1, np.cross(v, vp)) / dot(v, v)
    return w - d_eta


def closed_form(r, dr, x0, unit, lagrange=True):
    """The kernel's form; lagrange=False forms s - m by subtraction for every m (the form it avoids)."""
    q = dot(r, r)
    s = np.sqrt(q)
    xr = np.cross(x0, r)
    T, m = dot(dr, xr), dot(x0, r)
    if not unit:
        n = dot(x0, x0)
        return -T / (q + (n - 2) * m * m) - m * T / (s * dot(xr, xr))
    if not lagrange:
        return -T / (s * (s - m))
    return np.where(m < 0, -T / (s * (s - m)), -T * (s + m) / (s * dot(xr, xr)))


def unit_x0(rng):
    x0 = rng.standard_normal(3)
    return x0 / np.linalg.norm(x0)


def test_closed_form_equals_the_expression_at_generic_points():
    rng = np.random.default_rng(5)
    x0 = unit_x0(rng)
    r, dr = rng.standard_normal((20000, 3)), rng.standard_normal((20000, 3))
    ref = reference_expression(r, dr, x0)
    got = closed_form(r, dr, x0, unit=True)
    # away from the poles both are within a few ulps of the value, relative to its scale |r'| / |r|
    scale = np.linalg.norm(dr, axis=-1) / np.linalg.norm(r, axis=-1)
    keep = np.abs(dot(r, x0)) < 0.99 * np.linalg.norm(r, axis=-1)
    assert np.max(np.abs(got - ref)[keep] / scale[keep]) < 1e-12


@pytest.mark.parametrize("norm", [0.5, 2.0, 1.0 + 1e-6])
def test_general_form_for_non_unit_x0(norm):
    rng = np.random.default_rng(6)
    x0 = unit_x0(rng) * norm
    r, dr = rng.standard_normal((20000, 3)), rng.standard_normal((20000, 3))
    ref = reference_expression(r, dr, x0)
    got = closed_form(r, dr, x0, unit=False)
    scale = np.linalg.norm(dr, axis=-1) / np.linalg.norm(r, axis=-1)
    keep = np.abs(dot(r, x0)) < 0.9 * np.linalg.norm(r, axis=-1) * np.linalg.norm(x0)
    assert np.max(np.abs(got - ref)[keep] / scale[keep]) < 1e-10


def near_axis(rng, x0, sign, angle, count):
    """r at the given angle from sign * x0 (random azimuth and length), r' random."""
    e1 = np.cross(x0, [1.0, 0.0, 0.0] if abs(x0[0]) < 0.9 else [0.0, 1.0, 0.0])
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(x0, e1)
    phi = rng.uniform(0, 2 * np.pi, count)
    length = rng.uniform(0.5, 2.0, count)
    perp = np.cos(phi)[:, None] * e1 + np.sin(phi)[:, None] * e2
    r = length[:, None] * (sign * np.cos(angle) * x0 + np.sin(angle) * perp)
    return r, rng.standard_normal((count, 3))


def relative_error(got, exact):
    return np.abs(got - exact.astype(np.float64)) / np.abs(exact.astype(np.float64))


@pytest.mark.parametrize("angle", [1e-3, 1e-5])
def test_near_the_ray_of_x0_the_lagrange_form_keeps_the_angle_precision(angle):
    """m -> s: the curve crosses the ray of x0 from the query, where the integrand has its pole."""
    if np.finfo(np.longdouble).eps >= np.finfo(np.float64).eps:
        pytest.skip("np.longdouble is no wider than float64 here")
    rng = np.random.default_rng(7)
    x0 = unit_x0(rng)
    r, dr = near_axis(rng, x0, 1.0, angle, 2000)
    exact = reference_expression(r.astype(np.longdouble), dr.astype(np.longdouble), x0.astype(np.longdouble))
    # both float64 forms of the value lose about eps / angle; s - m by subtraction loses eps / angle^2
    ulp_angle = np.finfo(np.float64).eps / angle
    err_ref = relative_error(reference_expression(r, dr, x0), exact)
    err_kernel = relative_error(closed_form(r, dr, x0, unit=True), exact)
    err_sub = relative_error(closed_form(r, dr, x0, unit=True, lagrange=False), exact)
    assert np.median(err_kernel) < 4 * ulp_angle
    assert np.median(err_kernel) <= 4 * np.median(err_ref) + 1e-15
    assert np.median(err_sub) > 20 * np.median(err_kernel)


def test_opposite_the_ray_of_x0_the_closed_form_has_no_cancellation():
    """m -> -s at angle t from -x0: the expression's w and d_eta both grow like 1 / t while their difference is of
    order t, so it loses about eps / t^3 relative (1e-7 in float64 at t = 1e-3, 1e-10 in the 64-bit-mantissa
    long double that stands in for the exact value); the closed form loses about eps / t."""
    if np.finfo(np.longdouble).eps >= np.finfo(np.float64).eps:
        pytest.skip("np.longdouble is no wider than float64 here")
    rng = np.random.default_rng(8)
    x0 = unit_x0(rng)
    r, dr = near_axis(rng, x0, -1.0, 1e-3, 2000)
    exact = reference_expression(r.astype(np.longdouble), dr.astype(np.longdouble), x0.astype(np.longdouble))
    err_kernel = relative_error(closed_form(r, dr, x0, unit=True), exact)
    err_ref = relative_error(reference_expression(r, dr, x0), exact)
    assert np.median(err_kernel) < 1e-9
    assert np.median(err_ref) > 10 * np.median(err_kernel)
