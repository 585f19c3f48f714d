"""The slice example (examples/slice.cc) on the GPU: the reference's examples/main.cc pipeline (OBJ in, boundary,
full GWN on a plane, PNG out) through the C++ front end.  Its dumped values are checked against the CPU oracle's
eval_gwnr_mesh_batch (NaiveIntersector + FP64 fractional term) on the same points: 1e-12 in the exact mode, 1e-7
in the mixed one; its image against the reference's colour map of those values."""

import os
import subprocess

import numpy as np
import pytest

from antipodal_gb300 import synth
from test_examples import compile_slice, read_png

pytestmark = pytest.mark.gpu


def write_obj(path, verts, idx):
    with open(path, "w") as f:
        f.write("# generated mesh\n")
        for v in verts:
            f.write("v %.17g %.17g %.17g\n" % tuple(v))
        for t in np.asarray(idx).reshape(-1, 3):
            f.write("f %d/1/1 %d/1/1 %d/1/1\n" % tuple(t + 1))


def colour(w):
    """The reference's diverging map (examples/main.cc:99-117), rounding half away from zero as lround does."""
    w = np.clip(w, -1.0, 1.0)
    out_c = np.array([47.0, 89.0, 148.0])
    to = np.where((w >= 0)[:, None], np.array([243.0, 230.0, 118.0]), np.array([210.0, 85.0, 46.0]))
    v = np.clip(out_c + (to - out_c) * np.abs(w)[:, None], 0, 255)
    return np.floor(v + 0.5).astype(np.uint8)


@pytest.fixture(scope="module")
def slice_exe(tmp_path_factory):
    return compile_slice(str(tmp_path_factory.mktemp("slice") / "slice"))


@pytest.mark.parametrize("case", ["cube", "icosphere", "icosphere_mixed"])
def test_slice_example_matches_oracle(slice_exe, oracle, tmp_path, case):
    if case == "cube":
        verts, idx, _, _, _ = synth.rotated_open_cube(seed=11, n_queries=1)
        res, extra = 48, []
    else:
        verts, idx, _, _, _ = synth.open_icosphere(seed=6, level=3, grid=0)
        res = 96 if case == "icosphere" else 320
        extra = ["0.4", "0.2", "1", "0.5", "1.3", "mixed" if case == "icosphere_mixed" else "exact"]
    obj, png, vals = str(tmp_path / "m.obj"), str(tmp_path / "s.png"), str(tmp_path / "v.bin")
    write_obj(obj, verts, idx)
    if not extra:
        extra = ["0.5", "0", "1", "0", "1.2", "exact"]
    p = subprocess.run([slice_exe, obj, png, str(res)] + extra + [vals], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "open boundary:" in p.stdout
    rows = np.fromfile(vals, dtype=np.float64).reshape(res * res, 4)
    q, w = rows[:, :3], rows[:, 3]
    # the same plane and window, computed here
    n = np.array([float(v) for v in extra[1:4]])
    n = n / np.sqrt(n @ n)
    helper = np.array([1.0, 0, 0]) if abs(n[0]) < 0.9 else np.array([0, 1.0, 0])
    u = np.cross(helper, n)
    u = u / np.sqrt(u @ u)
    v = np.cross(n, u)
    d, a, b = verts @ n, verts @ u, verts @ v
    side = float(extra[4]) * max(a.max() - a.min(), b.max() - b.min())
    t = ((np.arange(res) + 0.5) / res - 0.5) * side
    au, bv = np.meshgrid((a.min() + a.max()) / 2 + t, (b.min() + b.max()) / 2 + t)
    expect_q = (d.min() + float(extra[0]) * (d.max() - d.min())) * n + au.reshape(-1, 1) * u + bv.reshape(-1, 1) * v
    assert np.abs(q - expect_q).max() <= 1e-14
    # values against the oracle at the example's own points, with the reference's fixed direction
    x0 = np.array([0.31, 0.57, 0.76])
    x0 = x0 / np.sqrt(x0 @ x0)
    ref = oracle.full_naive(q, x0, verts, idx, oracle.boundary(verts, idx))
    tol = 1e-7 if case == "icosphere_mixed" else 1e-12
    assert np.abs(w - ref).max() <= tol
    assert np.any(np.abs(w - np.round(w)) > 1e-3)  # the slice crosses the fractional region
    # the image: rows top to bottom (+v up), the reference's colour map
    img = read_png(png)
    assert img.shape == (res, res, 3)
    assert np.array_equal(img, colour(w).reshape(res, res, 3)[::-1])
