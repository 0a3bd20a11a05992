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
