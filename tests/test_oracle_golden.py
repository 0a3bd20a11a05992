"""Pins the oracle's element math to the reference's own routines.

tests/golden/elements.npz holds inputs and outputs of ComputeMembrane,
ComputeBending, ComputeInertial and intersect_triangle3_inc compiled from the
reference sources (tests/golden/make_golden.py).  The oracle restates those
energies in closed form, so agreement is to rounding: 1e-10 relative to the
largest entry for W, f, K; the ray-triangle test is restated operation by
operation and must agree bit for bit.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "elements.npz")
TOL = 1e-10


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_membrane_matches_reference(oracle, gold):
    for k in range(len(gold["mem_x"])):
        W, f, K = oracle.membrane(gold["mem_x"][k], gold["mem_X"][k], gold["mem_e"][k],
                                  gold["mem_nu"][k], gold["mem_P"][k], gold["mem_Q"][k])
        assert abs(W - gold["mem_W"][k]) <= TOL * max(abs(gold["mem_W"][k]), 1e-300), k
        assert rel(f, gold["mem_f"][k]) <= TOL, k
        assert rel(K.ravel(), gold["mem_K"][k]) <= TOL, k


def test_bending_matches_reference(oracle, gold):
    for k in range(len(gold["bend_x"])):
        X = gold["bend_X"][k]
        W, f, K = oracle.bending(gold["bend_x"][k], X, gold["bend_beta"][k])
        # W = c (1 - cos theta) and f ~ c sin theta cancel for nearly flat
        # hinges, in the reference as much as here: judge W on the scale of
        # c and f on the scale of |K| * edge length.
        dX = X[2:4] - X[0:2]
        c = 3 * gold["bend_beta"][k] * dX @ dX / (dX[0] * (X[5] - X[7]) - dX[1] * (X[4] - X[6]))
        L = np.sqrt(dX @ dX)
        assert abs(W - gold["bend_W"][k]) <= max(TOL * abs(gold["bend_W"][k]), 1e-13 * abs(c)), k
        fscale = max(np.abs(gold["bend_f"][k]).max(), np.abs(gold["bend_K"][k]).max() * L)
        assert np.abs(f - gold["bend_f"][k]).max() <= TOL * fscale, k
        assert rel(K.ravel(), gold["bend_K"][k]) <= TOL, k


def test_inertial_matches_reference(oracle, gold):
    for k in range(len(gold["iner_x"])):
        W, f, M = oracle.inertial(gold["iner_x"][k], gold["iner_X"][k], gold["iner_g"][k],
                                  gold["iner_rho"][k])
        assert abs(W - gold["iner_W"][k]) <= TOL * abs(gold["iner_W"][k]) + 1e-300, k
        assert rel(f, gold["iner_f"][k]) <= TOL, k
        assert rel(M.ravel(), gold["iner_M"][k]) <= TOL, k


def test_raytri_bit_exact(oracle, gold):
    n_hit = 0
    for k in range(len(gold["ray_o"])):
        v = gold["ray_v"][k]
        hit, tuv = oracle.raytri(gold["ray_o"][k], gold["ray_d"][k], v[0:3], v[3:6], v[6:9])
        assert hit == gold["ray_hit"][k], k
        if hit:
            n_hit += 1
            assert np.array_equal(tuv, gold["ray_tuv"][k]), k
    assert 50 < n_hit < len(gold["ray_o"]) - 50


def test_element_derivatives_consistent(oracle):
    """f = -dW/dx and K = d(-f)/dx by central differences (FP64)."""
    rng = np.random.default_rng(3)
    X = np.array([0, 0, 0.02, 0, 0.01, 0.017, 0.008, -0.015])
    x = np.concatenate([np.append(X[2 * i:2 * i + 2], 0) for i in range(4)]) + rng.normal(0, 2e-3, 12)
    W, f, K = oracle.bending(x, X, 1e-3)
    eps = 1e-7
    for i in range(12):
        d = np.zeros(12); d[i] = eps
        Wp, fp, _ = oracle.bending(x + d, X, 1e-3)
        Wm, fm, _ = oracle.bending(x - d, X, 1e-3)
        assert abs(-(Wp - Wm) / (2 * eps) - f[i]) <= 1e-5 * np.abs(f).max()
        assert np.abs(-(fp - fm) / (2 * eps) - K[:, i]).max() <= 1e-5 * np.abs(K).max()


# ---- collision detection: the reference's own boxTriCollision.cpp -----------
CD_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cd_ref.npz")
CD_SCENES = ("drape24", "points16", "drape128")


def cd_cases(g, name):
    """(positions, tri, boxes, points, normals, threshold, contact bytes) of
    every snapshot of one fixture scene (tests/golden/make_cd_golden.py)."""
    import oracle as O
    tri = g[name + "_tri"]
    boxes = [O.axis_box([0, 0, 0], d) for d in g[name + "_dim"]]
    for b, E1 in zip(boxes, g[name + "_E1"]):
        for k in range(16):
            b.E1[k] = E1[k]
    pts = g[name + "_pts"] if name + "_pts" in g.files else None
    nrm = g[name + "_nrm"] if name + "_nrm" in g.files else None
    size = 264  # sizeof(eolc_contact)
    counts = g[name + "_n"]
    offs = np.concatenate([[0], np.cumsum(counts)]) * size
    raw = g[name + "_contacts"]
    for k, x in enumerate(g[name + "_x"]):
        yield x, tri, boxes, pts, nrm, float(g[name + "_thr"]), raw[offs[k]:offs[k + 1]].tobytes()


@pytest.mark.parametrize("name", CD_SCENES)
def test_cd2_matches_reference_fixtures(oracle, name):
    """The restated CD2 returns the reference's own contact records, bit for
    bit and in order (fixtures from src/boxTriCollision.cpp compiled
    unmodified)."""
    g = np.load(CD_GOLD)
    n = 0
    for x, tri, boxes, pts, nrm, thr, want in cd_cases(g, name):
        got = oracle.cd2(x, tri, boxes=boxes, points=pts, normals=nrm, threshold=thr, raw=True)
        assert got == want
        n += len(want) // 264
    assert n > 0


def test_reference_cd_library_matches_oracle(oracle):
    """Where the reference sources were present at build time, the compiled
    reference CD2 itself (oracle/_ref/libeolc_ref_cd.so) against the oracle
    on fresh seeded snapshots."""
    import ctypes
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "oracle", "_ref", "libeolc_ref_cd.so")
    if not os.path.exists(path):
        pytest.skip("reference collision library not built (reference sources absent)")
    import scenes
    L = ctypes.CDLL(path)
    x0, X, tri, center, snaps = scenes.drape_positions(20, 16, seed=11)
    box = oracle.axis_box(center, (0.4, 0.4, 0.2))
    barr = (oracle.Box * 1)(box)
    tri32 = np.ascontiguousarray(tri, np.int32)
    total = 0
    for x in snaps:
        cap = 4 * (len(x) // 3) + 64
        out = (oracle.Contact * cap)()
        z = np.zeros(3)
        k = L.ref_cd2(len(x) // 3, oracle.dp(x), oracle.ip(tri32), len(tri32), barr, 1,
                      oracle.dp(z), oracle.dp(z), 0, ctypes.c_double(1e-3), out, cap)
        got = ctypes.string_at(out, ctypes.sizeof(oracle.Contact) * k)
        assert got == oracle.cd2(x, tri, boxes=[box], threshold=1e-3, raw=True)
        total += k
    assert total > 0
