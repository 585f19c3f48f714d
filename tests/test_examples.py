"""The slice example (examples/slice.cc, the reference's examples/main.cc on the GPU) without a GPU: its OBJ reader
and PNG writer (examples/obj_png.hh) through a small driver, and the example itself building against the front end
and failing loudly when no device is present.  The GPU run is in test_examples_gpu.py."""

import os
import shutil
import struct
import subprocess
import zlib

import numpy as np
import pytest

from oracle.oracle import reference_src

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = reference_src() or ""
LIBDIR = os.path.join(ROOT, "antipodal_gb300")


def value_type_headers():
    return REF_SRC if os.path.isdir(REF_SRC) else os.path.join(ROOT, "tests", "cpp", "shim")


def compile_slice(out):
    from antipodal_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    cmd = [shutil.which("g++"), "-std=c++20", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
           value_type_headers(), os.path.join(ROOT, "examples", "slice.cc"), "-o", out, "-L", LIBDIR,
           "-lantipodal_gb300", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def read_png(path):
    """Decodes an 8-bit RGB PNG with filter type 0 rows (what the writer emits), checking every chunk's CRC."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body), kind
        chunks.append((kind, body))
        pos += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 2, 0, 0, 0)
    raw = zlib.decompress(b"".join(b for k, b in chunks if k == b"IDAT"))
    rows = np.frombuffer(raw, np.uint8).reshape(h, 3 * w + 1)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("objpng") / "obj_png_run")
    r = subprocess.run([shutil.which("g++"), "-std=c++20", "-O2", "-Wall", "-Werror",
                        os.path.join(ROOT, "tests", "cpp", "obj_png_run.cc"), "-o", exe], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_obj_reader_faces_and_corner_forms(driver, tmp_path):
    # v/vt/vn corner forms, a quad and a pentagon (fan-triangulated from the first corner), negative (relative)
    # indices, and lines that are not vertices or faces
    obj = tmp_path / "m.obj"
    obj.write_text("# comment\nmtllib x.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nvt 0.5 0.5\n"
                   "o thing\nf 1 2 3\nf 1/1 2/1 3/1 4/1\nv 0.5 2 0\nf -5//1 -4//1 -3//1 -2//1 -1//1\n"
                   "  f\t2/1/1 3/1/1 4/1/1\r\ns off\n")
    png = str(tmp_path / "p.png")
    p = subprocess.run([driver, str(obj), png, "3", "2"], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.split("\n")
    assert lines[0] == "5"
    tris = [tuple(int(v) for v in line.split()) for line in lines[1:] if line]
    assert tris == [(0, 1, 2), (0, 1, 2), (0, 2, 3), (0, 1, 2), (0, 2, 3), (0, 3, 4), (1, 2, 3)]


@pytest.mark.parametrize("text", ["v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n", "v 0 0 0\nf 0 1 1\n",
                                  "v 0 0 0\nv 1 0 0\nf -3 1 2\n", "v 0 0\n", "v 0 0 0\nf 1 x 2\n"])
def test_obj_reader_rejects_bad_files(driver, tmp_path, text):
    obj = tmp_path / "bad.obj"
    obj.write_text(text)
    p = subprocess.run([driver, str(obj), str(tmp_path / "p.png"), "1", "1"], capture_output=True, text=True)
    assert p.returncode == 2 and p.stderr.startswith("line "), (p.returncode, p.stderr)
    p = subprocess.run([driver, str(tmp_path / "missing.obj"), str(tmp_path / "p.png"), "1", "1"],
                       capture_output=True, text=True)
    assert p.returncode == 2 and "could not open" in p.stderr


@pytest.mark.parametrize("w,h", [(1, 1), (7, 5), (300, 400)])
def test_png_writer_round_trip(driver, tmp_path, w, h):
    # 300 x 400 spans several stored deflate blocks (more than 65,535 bytes of scanlines)
    obj = tmp_path / "t.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    png = str(tmp_path / "p.png")
    p = subprocess.run([driver, str(obj), png, str(w), str(h)], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    img = read_png(png)
    x, y = np.meshgrid(np.arange(w), np.arange(h))
    assert img.shape == (h, w, 3)
    assert np.array_equal(img[..., 0], (x % 256).astype(np.uint8))
    assert np.array_equal(img[..., 1], (y % 256).astype(np.uint8))
    assert np.array_equal(img[..., 2], ((x ^ y) % 256).astype(np.uint8))


def test_slice_example_builds_and_reports_errors(tmp_path):
    exe = compile_slice(str(tmp_path / "slice"))
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 1 and "usage" in p.stderr
    p = subprocess.run([exe, str(tmp_path / "missing.obj"), str(tmp_path / "o.png"), "8"], capture_output=True,
                       text=True)
    assert p.returncode == 1 and "could not open" in p.stderr
    obj = tmp_path / "tri.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    p = subprocess.run([exe, str(obj), str(tmp_path / "o.png"), "8", "0.5", "0", "1", "0", "1.2", "fast"],
                       capture_output=True, text=True)
    assert p.returncode == 1 and "precision" in p.stderr
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        return
    # no device: the library's error, not a CPU result
    p = subprocess.run([exe, str(obj), str(tmp_path / "o.png"), "8"], capture_output=True, text=True)
    assert p.returncode == 1 and "no CUDA device" in p.stderr, p.stderr
    assert not os.path.exists(tmp_path / "o.png")
