"""The library on the GPU against the committed 100-step trace of the 20 x 20
sheet (tests/golden/trace_c1.npz, made by tests/golden/make_trace.py from the
oracle), read as a fixture: no oracle call.

* FP64 fills at the checkpoint states: the weighted checksums of f, M and
  MDK match the trace's within 1e-10 of the sums of |entries|.
* One step from the first state of each consecutive checkpoint pair
  reproduces the second.  The trace's CG stopped at a relative residual of
  1e-8, which leaves its velocities up to 2.2e-8 (relative) from the exact
  solve (measured on the CPU against the oracle's direct solve), so: FP64
  path v within 1e-7 relative and x within 5e-9; mixed path v within 1e-5.
"""
import os
import sys

import numpy as np
import pytest

import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_trace  # noqa: E402  (checksum definition and scene constants)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


@pytest.fixture(scope="module")
def trace():
    return np.load(os.path.join(HERE, "golden", "trace_c1.npz"))


@pytest.fixture(scope="module")
def sheet_ctx(eolc):
    s = scenes.sheet(make_trace.QUADS)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    return s, ctx


def test_fills_match_trace_checksums(eolc, trace, sheet_ctx):
    s, ctx = sheet_ctx
    mat = eolc.Material(**scenes.material_c1())
    for c, x in zip(trace["checkpoints"], trace["x"]):
        if c >= make_trace.STEPS:
            continue  # the trace holds fills of steps 1..100 (states 0..99)
        f, M, MDK = ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_FP64)
        got = make_trace.checksums(f, eolc.bsr_to_csr(ctx, M), eolc.bsr_to_csr(ctx, MDK))
        want = trace["fill_sums"][c]
        for k in range(3):
            err = abs(got[2 * k] - want[2 * k])
            assert err <= 1e-10 * want[2 * k + 1], (c, k, err, want[2 * k + 1])
            assert abs(got[2 * k + 1] - want[2 * k + 1]) <= 1e-10 * want[2 * k + 1]


@pytest.mark.parametrize("precision", [0, 1])
def test_single_steps_reproduce_trace(eolc, trace, sheet_ctx, precision):
    s, ctx = sheet_ctx
    mat = eolc.Material(**scenes.material_c1())
    tol = 1e-12 if precision == eolc.PREC_FP64 else 1e-8
    opts = eolc.SolveOpts(rel_tol=tol, precision=precision)
    cp = list(trace["checkpoints"])
    for a in (1, 5, 50):
        i, j = cp.index(a), cp.index(a + 1)
        x, v = trace["x"][i].copy(), trace["v"][i].copy()
        info = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                        opts)
        assert info.status == eolc.OK and info.rel_res <= tol
        ev = np.abs(v - trace["v"][j]).max() / np.abs(trace["v"][j]).max()
        ex = np.abs(x - trace["x"][j]).max()
        print("step %d -> %d, precision %d: v %.2e, x %.2e" % (a, a + 1, precision, ev, ex))
        if precision == eolc.PREC_FP64:
            assert ev <= 1e-7 and ex <= 5e-9, (a, ev, ex)
        else:
            assert ev <= 1e-5, (a, ev)
