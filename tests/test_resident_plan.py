"""Resident solvers' plan on the CPU: build_patch_plan (csrc/patch.cu) run on
real meshes by a host program (resident_plan_check.cu) that replays the
device's warp-compacted record / slot arithmetic and checks the image and
coarse-space invariants, and that the plan built on several host threads
equals the single-threaded one.  No GPU: the program only runs host code."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

import scenes

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def plan_prog(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("plan") / "resident_plan_check")
    # PTX only: the program runs no device code
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-gencode",
                           "arch=compute_103a,code=compute_103a",
                           os.path.join(HERE, "resident_plan_check.cu"), "-o", exe])
    return exe


def bsr_pattern(n, tri, hinge):
    """Node pairs coupled by a triangle or a hinge (the BSR pattern of MDK)."""
    tri = np.asarray(tri, np.int64).reshape(-1, 3)
    hinge = np.asarray(hinge, np.int64).reshape(-1, 4)
    rows = [np.repeat(tri, 3, axis=1).ravel(), np.repeat(hinge, 4, axis=1).ravel()]
    cols = [np.tile(tri, (1, 3)).ravel(), np.tile(hinge, (1, 4)).ravel()]
    r, c = np.concatenate(rows), np.concatenate(cols)
    m = sp.csr_matrix((np.ones(len(r)), (r, c)), shape=(n, n))
    m.sum_duplicates()
    m.sort_indices()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32)


def run(plan_prog, tmp_path, s):
    rp, ci = bsr_pattern(s["n"], s["tri"], s["hinge"])
    path = tmp_path / "pattern.bin"
    with open(path, "wb") as f:
        np.array([s["n"], len(ci)], np.int32).tofile(f)
        rp.tofile(f)
        ci.tofile(f)
        np.asarray(s["X"], np.float64).reshape(-1).tofile(f)
    out = subprocess.run([plan_prog, str(path)], capture_output=True, text=True)
    print(out.stdout.strip())
    assert out.returncode == 0, out.stdout + out.stderr
    assert "problems 0" in out.stdout


@pytest.mark.parametrize("quads", [8, 20, 64, 256])
def test_sheet_plans(plan_prog, tmp_path, quads):
    run(plan_prog, tmp_path, scenes.sheet(quads))


@pytest.mark.parametrize("n_tri", [5000, 50000])
def test_irregular_plans(plan_prog, tmp_path, n_tri):
    run(plan_prog, tmp_path, scenes.delaunay_sheet(n_tri, np.random.default_rng(n_tri)))
