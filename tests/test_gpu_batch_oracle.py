"""Batched stepping at the benchmark sizes, against the oracle.

Configuration 3: 256 sheets whose side is drawn from 16..96 quads and whose
Young's modulus is drawn from U(20, 100) (seeded), corners 3 and 4 pinned.
Configuration 5: 64 Delaunay sheets of 5k-50k triangles (seeded), top
corners pinned, learned batched solve with the Jacobi fallback.  Every
instance steps in one batched launch; a seeded sample of 16 instances that
spans the size range is compared with the oracle: its Forces::fill (the
reference's element math and triplet assembly, Forces.cpp:331-930) and an
FP64 sparse direct solve of the pinned system (the QP's equality-only
optimum, GeneralizedSolver.cpp:107-173) from the same state.  Tolerances:
FP64 batched solve to rel-res 1e-13, velocities within 1e-10 of the direct
solve; mixed precision (FP32 matrix, FP64 refinement to 1e-8), within 1e-5.
"""
import os

import numpy as np
import pytest

import oracle as O
import scenes

pytestmark = pytest.mark.gpu
WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "eol-cloth_gb300", "weights", "lpc.npy")


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _sample(sizes, n=16):
    """n instances spanning the size range: evenly spaced ranks of the
    instances ordered by node count."""
    order = np.argsort(sizes, kind="stable")
    return sorted(int(order[k]) for k in np.linspace(0, len(order) - 1, n).round().astype(int))


def _oracle_velocity(s, mat, x, v):
    import scipy.sparse.linalg as sla
    F = O.Forces(x, s["X"], s["tri"], s["hinge"], O.material(**mat), scenes.GRAV, scenes.H)
    b = F.rhs(v, scenes.H)
    fixed = s["fixed"]
    beq = 0.99 * v[fixed] + s["fixed_vel"]
    A = F.csr(1).tocsr()
    free = np.setdiff1d(np.arange(len(x)), fixed)
    out = np.zeros(len(x))
    out[fixed] = beq
    out[free] = sla.spsolve(A[free][:, free].tocsc(), (-b - A[:, fixed] @ beq)[free])
    return out


def _batched_step(eolc, B, x, v, lpc=None):
    ctx = eolc.Context(0)
    ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in B["sheets"]])
    ctx.set_instance_materials([eolc.Material(**m) for m in B["mats"]])
    if lpc is not None:
        lpc.attach(ctx)
    ctx.state_upload(x, B["X"], v)
    return ctx


def _check(B, picks, x, v, vb, tol):
    off = B["node_off"]
    worst = 0.0
    for k in picks:
        s, m = B["sheets"][k], B["mats"][k]
        sl = slice(3 * off[k], 3 * off[k + 1])
        want = _oracle_velocity(s, m, x[sl], v[sl])
        err = np.abs(vb[sl] - want).max() / np.abs(want).max()
        worst = max(worst, err)
        assert err <= tol, (k, s["n"], err)
    return worst


def _moving_state(B, seed, jitter=2e-4):
    """Positions jittered by `jitter` (0.2 mm: at most 3% of the smallest
    element of the regular sheets, so every MDK stays positive definite) and
    a random velocity field, so the step's solve is not the pure gravity load
    of a sheet at rest."""
    rng = np.random.default_rng(seed)
    x = B["x"] + rng.normal(0, jitter, B["x"].size)
    v = rng.normal(0, 0.05, B["x"].size)
    return x, v


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_config3_batch_matches_oracle(eolc, precision):
    B = scenes.batch(256)  # sides U{16..96}, E ~ U(20, 100), seed 3
    assert len(B["sheets"]) == 256
    x, v = _moving_state(B, 31)
    prec = eolc.PREC_MIXED if precision == "mixed" else eolc.PREC_FP64
    rel_tol = 1e-8 if precision == "mixed" else 1e-13
    opts = eolc.SolveOpts(rel_tol=rel_tol, max_iter=20000, precision=prec)
    ctx = _batched_step(eolc, B, x, v)
    tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.status == eolc.OK and tot.n_failed == 0
    assert all(i.rel_res <= rel_tol for i in infos)
    _, vb = ctx.state_download()
    picks = _sample([s["n"] for s in B["sheets"]])
    worst = _check(B, picks, x, v, vb, 1e-5 if precision == "mixed" else 1e-10)
    print("config 3 %s: worst velocity error %.2e over %d sampled instances"
          % (precision, worst, len(picks)))


def test_config5_learned_batch_matches_oracle(eolc):
    B = scenes.delaunay_batch(64)  # U(5k, 50k) triangles, seed 5
    assert len(B["sheets"]) == 64
    # positions at rest: the Delaunay sheets have sliver triangles that a
    # jitter can invert; the random velocities still load the solve
    x, v = _moving_state(B, 53, jitter=0.0)
    lpc = eolc.LearnedPC(0)
    lpc.set_params(np.load(WEIGHTS))
    ctx = _batched_step(eolc, B, x, v, lpc)
    # a Jacobi step sets every instance's reference iteration count (the
    # fallback cap), then the learned step runs from the same state
    ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], eolc.SolveOpts())
    ctx.state_upload(x, B["X"], v)
    opts = eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=2)
    tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.status == eolc.OK and tot.n_failed == 0 and tot.max_rel_res <= 1e-8
    _, vb = ctx.state_download()
    picks = _sample([s["n"] for s in B["sheets"]])
    worst = _check(B, picks, x, v, vb, 1e-5)
    print("config 5 learned: worst velocity error %.2e, %d fallbacks" % (worst, tot.n_fallback))
