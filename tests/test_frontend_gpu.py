"""The C++ front end on the GPU: tests/cpp/frontend_run.cc is compiled against include/antipodal/cuda/gwn_cuda.hh
(with the reference's value types, or the test stand-in where the reference is not installed), linked to
libantipodal_gb300.so and run; its outputs are checked against the CPU oracle on the same queries."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from antipodal_gb300 import synth
from oracle.oracle import reference_src

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = reference_src() or ""


def test_frontend_program_matches_oracle(gwn, oracle, tmp_path):
    inc = REF_SRC if os.path.isdir(REF_SRC) else os.path.join(ROOT, "tests", "cpp", "shim")
    exe = str(tmp_path / "frontend_run")
    libdir = os.path.join(ROOT, "antipodal_gb300")
    cmd = [shutil.which("g++"), "-std=c++20", "-I", os.path.join(ROOT, "include"), "-I", inc,
           os.path.join(ROOT, "tests", "cpp", "frontend_run.cc"), "-o", exe, "-L", libdir, "-lantipodal_gb300",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    p = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    rows = np.array([[float(v) for v in line.split()] for line in p.stdout.strip().splitlines()])
    q = rows[:, 0:3]
    verts, idx, bnd, x0 = synth.CUBE_VERTS, synth.CUBE_IDX_OPEN_Y, synth.cube_open_y_boundary(), synth.unit_x0()
    full = oracle.full_naive(q, x0, verts, idx, bnd)
    assert np.max(np.abs(rows[:, 3] - full)) <= 1e-12
    assert np.max(np.abs(rows[:, 4] - full)) <= 1e-7
    assert np.max(np.abs(rows[:, 5] - oracle.frac_batch(q, x0, bnd))) <= 1e-12
    assert np.array_equal(rows[:, 6].astype(np.int32), oracle.int_naive(q, x0, verts, idx))
    # robust (exact_float) and parametric overloads
    rob, _, _ = oracle.robust_eval("exact_float", verts, idx, bnd, q)
    assert np.max(np.abs(rows[:, 7] - rob)) <= 1e-12
    lines = np.stack([np.concatenate([s[0:3], (2 * s[0:3] + s[3:6]) / 3, (s[0:3] + 2 * s[3:6]) / 3, s[3:6]])
                      for s in bnd])
    par = oracle.param_frac_bezier3(q, x0, lines, 0, 10, 1e-6)
    assert np.max(np.abs(rows[:, 8] - par)) <= 1e-15
    # the faces as flat patches: the same surface, so the mesh's crossing counts; the full parametric GWN adds them
    pcount = rows[:, 9].astype(np.int32)
    assert np.array_equal(pcount, oracle.int_naive(q, x0, verts, idx))
    assert np.max(np.abs(rows[:, 10] - (par + pcount))) <= 1e-15
