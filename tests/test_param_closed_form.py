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


def power_about_half(cp):
    """The double-float kernel's conversion (csrc/param.cu, power_about_half): control points c0..c3 (..., 4, 3) to
    r(1/2), r'(1/2), r''(1/2) / 2 and r''' / 6, in the dtype of cp."""
    c0, c1, c2, c3 = cp[..., 0, :], cp[..., 1, :], cp[..., 2, :], cp[..., 3, :]
    dt = cp.dtype.type
    s03, s12, d30, d21 = c0 + c3, c1 + c2, c3 - c0, c2 - c1
    return (s03 + dt(3) * s12) * dt(0.125), (d30 + d21) * dt(0.75), (s03 - s12) * dt(1.5), d30 - dt(3) * d21


def curve_power(cp, t):
    """r and r' (..., T, 3) at parameters t (..., T) by Horner's rule at t - 1/2, as the kernel's integrand
    evaluates them."""
    a0, a1, a2, a3 = (a[..., None, :] for a in power_about_half(cp))
    dt = cp.dtype.type
    d = (t - 0.5).astype(cp.dtype)[..., None]
    a3d = a3 * d
    return a0 + d * (a1 + d * (a2 + a3d)), a1 + d * (dt(2) * a2 + dt(3) * a3d)


def curve_bernstein(cp, t):
    """r and r' (..., T, 3) at parameters t (..., T) from the Bernstein basis, summed c0 b0 + c1 b1 + c2 b2 + c3 b3
    as the reference does."""
    u = 1 - t
    b = [u**3, 3 * u * u * t, 3 * u * t * t, t**3]
    d = [-3 * u * u, 3 * u * u - 6 * u * t, 6 * u * t - 3 * t * t, 3 * t * t]
    r, dr = 0, 0
    for k in range(4):
        ck = cp[..., None, k, :]
        r = r + b[k].astype(cp.dtype)[..., None] * ck
        dr = dr + d[k].astype(cp.dtype)[..., None] * ck
    return r, dr


def random_pairs():
    """Boundary cubics of seeded bicubic patches minus queries (16 random curves per query), 64 parameters each."""
    from antipodal_gb300 import synth

    curves, q, _ = synth.bezier_patches(seed=0, n_patches=256, n_queries=2000)
    rng = np.random.default_rng(1)
    P = curves.reshape(-1, 4, 3)
    cp = P[rng.integers(0, len(P), (len(q), 16))] - q[:, None, None, :]
    return cp, np.broadcast_to(rng.uniform(0, 1, 64), cp.shape[:-2] + (64,))


def near_pairs(rho):
    """20,000 random boundary cubics, each with a query at distance rho from its point at a random t*, evaluated at
    t* - 0.02 ... t* + 0.02: the evaluations that a near query's deep panels make."""
    from antipodal_gb300 import synth

    curves, _, _ = synth.bezier_patches(seed=0, n_patches=256, n_queries=10)
    rng = np.random.default_rng(2)
    P = curves.reshape(-1, 4, 3)[rng.integers(0, 1024, 20000)]
    ts = rng.uniform(0.05, 0.95, len(P))
    point, _ = curve_bernstein(P, ts[:, None])
    dirs = rng.standard_normal((len(P), 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    cp = P - (point[:, 0] + rho * dirs)[:, None, :]
    return cp, ts[:, None] + np.linspace(-0.02, 0.02, 9)[None, :]


def fp32_error(f, cp, t):
    """Relative error of r in FP32 (control points rounded to FP32) against the same form in FP64."""
    r64, _ = f(cp, t)
    r32, _ = f(cp.astype(np.float32), t)
    return np.linalg.norm(r32.astype(np.float64) - r64, axis=-1) / np.linalg.norm(r64, axis=-1)


def test_power_form_about_half_is_the_curve():
    cp, t = random_pairs()
    r_b, dr_b = curve_bernstein(cp, t)
    r_p, dr_p = curve_power(cp, t)
    scale = np.abs(cp).max(axis=(-2, -1))[..., None]
    assert np.max(np.linalg.norm(r_p - r_b, axis=-1) / scale) < 1e-14
    assert np.max(np.linalg.norm(dr_p - dr_b, axis=-1) / scale) < 1e-13


def test_power_form_rounds_about_as_the_bernstein_form():
    """In FP32 against FP64.  At random pairs the power form's median relative error in r is about 1.2x the Bernstein
    form's, with a lower maximum; near a query (1e-4 to 1e-2 from the curve) about 1.7x, p99 about 2.1x."""
    cp, t = random_pairs()
    e_b, e_p = fp32_error(curve_bernstein, cp, t), fp32_error(curve_power, cp, t)
    assert np.median(e_p) < 1.5 * np.median(e_b)
    assert e_p.max() <= e_b.max()
    for rho in (1e-2, 1e-3, 1e-4):
        cp, t = near_pairs(rho)
        e_b, e_p = fp32_error(curve_bernstein, cp, t), fp32_error(curve_power, cp, t)
        assert np.median(e_p) < 2.0 * np.median(e_b), rho
        assert np.quantile(e_p, 0.99) < 2.5 * np.quantile(e_b, 0.99), rho
