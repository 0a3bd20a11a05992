"""OBJ frame export on the CPU (no GPU):

* the device text formatter (eol-cloth_gb300/csrc/objfmt.cuh), built into a
  host program (objfmt_check.cu), prints every number exactly as the C
  library's printf "%f" / "%i" — ties, signed zeros, subnormals, NaN/Inf and
  random values over 106 binades, and refuses |v| >= 2^63;
* the oracle's files (oracle/export.cpp) have the reference's layout
  (Cloth.cpp:535-590, BrenderManager.cpp:34-84), checked line by line
  against Python's own correctly rounded "%f" on a perturbed sheet and a
  Delaunay mesh;
* the oracle's node normals (ArcSim normal<WS>) agree with a vectorised
  numpy evaluation of the same formula.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
import scenes

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fmt_prog(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("objfmt") / "objfmt_check")
    # PTX only: the program runs no device code
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-gencode",
                           "arch=compute_103a,code=compute_103a",
                           os.path.join(HERE, "objfmt_check.cu"), "-o", exe])
    return exe


def test_formatter_matches_printf(fmt_prog):
    out = subprocess.run([fmt_prog, "300000"], capture_output=True, text=True)
    print(out.stdout.strip())
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout


def numpy_normals(x, tri):
    """sum over incident faces of cross(e1, e2) / (2 |e1|^2 |e2|^2), normalised."""
    P = x.reshape(-1, 3)
    n = np.zeros_like(P)
    for j in range(3):
        v, a, b = tri[:, j], tri[:, (j + 1) % 3], tri[:, (j + 2) % 3]
        e1, e2 = P[a] - P[v], P[b] - P[v]
        w = np.cross(e1, e2) / (2 * (e1 * e1).sum(1) * (e2 * e2).sum(1))[:, None]
        np.add.at(n, v, w)
    m = np.linalg.norm(n, axis=1)
    out = np.zeros_like(n)
    ok = m > 0
    out[ok] = n[ok] / m[ok, None]
    return out.ravel()


def python_text(x, X, tri, nrm, frame, time):
    """The two files with Python's "%f" (correctly rounded, like glibc)."""
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    Xr, xr, nr = X.reshape(-1, 2), f32(x).reshape(-1, 3), f32(nrm).reshape(-1, 3)
    tr = f32(X).reshape(-1, 2)
    faces = ["f %d/%d/%d %d/%d/%d %d/%d/%d\n" % tuple(np.repeat(t + 1, 3)) for t in tri]
    files = []
    for which, name in enumerate(("Cloth2D", "Cloth3D")):
        s = ["# frame %06d \n" % frame, "# time %f \n" % time, "# name %s \n" % name]
        if which == 0:
            s += ["v %f %f %f\n" % (u[0], u[1], 0.0) for u in Xr]
        else:
            s += ["v %f %f %f\n" % tuple(p) for p in xr]
        s += ["vt %f %f\n" % tuple(u) for u in tr]
        if which == 0:
            s += ["vn %f %f %f\n" % (0.0, 0.0, 1.0)] * len(Xr)
        else:
            s += ["vn %f %f %f\n" % tuple(q) for q in nr]
        s += faces
        files.append("".join(s).encode())
    return files


def perturbed_sheet(quads, seed):
    s = scenes.sheet(quads)
    rng = np.random.default_rng(seed)
    x = s["x"] + rng.normal(0, 0.05, s["x"].size)
    x[2::3] += rng.normal(0, 0.3, s["n"])  # folds: normals in every direction
    return x, s["X"], s["tri"]


@pytest.mark.parametrize("case", ["sheet", "delaunay"])
def test_oracle_layout_and_numbers(case):
    if case == "sheet":
        x, X, tri = perturbed_sheet(12, 1)
    else:
        d = scenes.delaunay_sheet(600, np.random.default_rng(2))
        x = d["x"] + np.random.default_rng(3).normal(0, 0.02, d["x"].size)
        X, tri = d["X"], d["tri"]
    a, b = O.obj_text(x, X, tri, frame=12, time=0.06)
    nrm = O.node_normals(x, tri)
    pa, pb = python_text(x, X, np.asarray(tri), nrm, 12, 0.06)
    assert a == pa
    assert b == pb
    n = len(x) // 3
    lines = b.decode().splitlines()
    assert lines[:3] == ["# frame 000012 ", "# time 0.060000 ", "# name Cloth3D "]
    assert len(lines) == 3 + 3 * n + len(tri)


def test_oracle_normals_match_numpy():
    x, X, tri = perturbed_sheet(10, 4)
    got = O.node_normals(x, tri)
    want = numpy_normals(x, np.asarray(tri))
    assert np.abs(got - want).max() <= 1e-12
    assert np.allclose(np.linalg.norm(got.reshape(-1, 3), axis=1), 1.0)
