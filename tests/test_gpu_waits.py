"""Bounded device waits: with a wait limit of one poll, the persistent
solvers' grid barriers and the resident patch kernel's neighbour exchange
give up, the call reports TIMEOUT without hanging or faulting, and the
same context then solves normally (the limit back at its default) to the
same answer as a fresh context.  Nothing here faults, traps or hangs the GPU:
the waits run out because their limit is tiny, not because a CTA stalls."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


ARMS = {
    # streamed cg_kernel: one grid barrier per iteration, 15 CTAs at 40^2
    "streamed": dict(precond=0, streamed=1),
    # resident Jacobi kernel: grid barrier inside every reduction, 4 CTAs
    "resident": dict(precond=0),
    # resident patch kernel: tagged neighbour exchange + grid barrier
    "patch": dict(precond=3),
}


def _step(eolc, ctx, s, x, v, opts):
    mat = eolc.Material(**scenes.material_c1())
    return ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"], opts)


@pytest.mark.parametrize("arm", sorted(ARMS))
def test_tiny_wait_limit_times_out_and_context_recovers(eolc, arm):
    s = scenes.sheet(40)
    opts = eolc.SolveOpts(precision=eolc.PREC_MIXED, **ARMS[arm])
    rng = np.random.default_rng(2)
    x0 = s["x"] + rng.normal(0, 1e-3, s["x"].size)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    _step(eolc, ctx, s, x0.copy(), np.zeros_like(x0), opts)  # plans built, a normal solve
    ctx.set_wait_limit(1)
    for _ in range(2):  # twice: a timed-out launch leaves nothing behind
        with pytest.raises(eolc.EolcError) as e:
            _step(eolc, ctx, s, x0.copy(), np.zeros_like(x0), opts)
        assert e.value.status == eolc.TIMEOUT, e.value
    ctx.set_wait_limit(0)  # the default
    x1, v1 = x0.copy(), np.zeros_like(x0)
    info = _step(eolc, ctx, s, x1, v1, opts)
    assert info.status == eolc.OK and info.rel_res <= 1e-8
    fresh = eolc.Context(0)
    fresh.set_topology(s["n"], s["tri"], s["hinge"])
    x2, v2 = x0.copy(), np.zeros_like(x0)
    _step(eolc, fresh, s, x2, v2, opts)
    # solves are bit-reproducible: the recovered context gives the fresh
    # context's answer exactly
    assert np.array_equal(v1, v2) and np.array_equal(x1, x2)


def test_wait_limit_argument_checks(eolc):
    ctx = eolc.Context(0)
    with pytest.raises(eolc.EolcError) as e:
        ctx.set_wait_limit(-1)
    assert e.value.status == eolc.BAD_ARG
