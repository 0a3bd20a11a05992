"""The learned preconditioner on the GPU.

* its hand-written backward kernels against the CPU reference
  (oracle/learned_ref.py: the same network in FP64 with torch.autograd);
* the preconditioned solve reaches the same FP64 relative residual as Jacobi
  and gives the same velocities (the preconditioner is SPD by construction);
* the Jacobi fallback engages when the learned solve runs past its cap;
* training lowers the probe loss, and the committed trained network
  (eol-cloth_gb300/weights/lpc.npy) needs fewer PCG iterations than Jacobi on
  a sheet it was not trained on.
"""
import os

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WEIGHTS = os.path.join(ROOT, "eol-cloth_gb300", "weights", "lpc.npy")


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _system(eolc, quads, density, seed):
    s = scenes.sheet(quads)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    m = scenes.material_c1()
    m["density"] = density
    mat = eolc.Material(**m)
    rng = np.random.default_rng(seed)
    x = s["x"] + rng.normal(0, 0.01, s["x"].size)
    _, _, MDK = ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_MIXED)
    return s, ctx, mat, MDK, rng


def test_backward_kernels_match_cpu_reference(eolc):
    import learned_ref
    # a mass-dominated system keeps the FP32 products A w, G y free of
    # cancellation, so the comparison measures the network's derivatives
    s, ctx, mat, MDK, rng = _system(eolc, 6, 50.0, 0)
    lpc = eolc.LearnedPC(0, seed=3)
    p = lpc.get_params() + rng.normal(0, 0.05, lpc.num_params()).astype(np.float32)
    lpc.set_params(p)
    probes = rng.normal(0, 1, (3, 3 * s["n"])).astype(np.float32)
    loss, grad = lpc.loss_grad(ctx, s["fixed"], probes)
    rowptr, colidx = ctx.bsr_pattern()
    pinned = np.zeros(3 * s["n"], bool)
    pinned[s["fixed"]] = True
    lref, gref = learned_ref.loss_and_grad(p, MDK.astype(np.float32).reshape(-1, 9), rowptr,
                                           colidx, pinned, probes)
    rel_loss = abs(loss - lref) / abs(lref)
    rel_grad = np.linalg.norm(grad - gref) / np.linalg.norm(gref)
    print("loss %.8g vs %.8g (%.1e), gradient %.1e" % (loss, lref, rel_loss, rel_grad))
    assert rel_loss <= 1e-5, (loss, lref)
    assert rel_grad <= 1e-4, rel_grad


def test_learned_solve_reaches_fp64_residual(eolc):
    s = scenes.sheet(24)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    lpc = eolc.LearnedPC(0, seed=5)
    rng = np.random.default_rng(5)
    lpc.set_params(lpc.get_params() + rng.normal(0, 0.02, lpc.num_params()).astype(np.float32))
    lpc.attach(ctx)
    x0 = s["x"] + rng.normal(0, 0.003, s["x"].size)
    xa, va = x0.copy(), np.zeros(3 * s["n"])
    xb, vb = x0.copy(), np.zeros(3 * s["n"])
    for k in range(5):
        ia = ctx.step(xa, s["X"], va, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_JACOBI))
        ib = ctx.step(xb, s["X"], vb, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=0))
        assert ia.status == ib.status == eolc.OK
        assert ib.rel_res <= 1e-8 and ib.used_fallback == 0
        assert np.abs(vb - va).max() <= 1e-5 * np.abs(va).max()
        xb, vb = xa.copy(), va.copy()  # same state for the next comparison


def test_fallback_to_jacobi(eolc):
    s = scenes.sheet(16)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    lpc = eolc.LearnedPC(0, seed=7)
    lpc.attach(ctx)
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    # a reference count of 1 iteration caps the learned solve at 2
    import ctypes
    assert eolc.lib.eolc_set_jacobi_reference(ctx.handle, 1) == eolc.OK
    info = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                    eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=2))
    assert info.status == eolc.OK and info.used_fallback == 1 and info.rel_res <= 1e-8


def test_training_lowers_the_loss(eolc):
    import train_lpc
    lpc = eolc.LearnedPC(0, seed=2)
    train_lpc.generate(lpc, 60, quads=16, steps_per_run=20, seed=2)
    assert lpc.num_systems() == 60
    losses = lpc.train(6, lr=2e-3, seed=2)
    assert losses[-1] < 0.97 * losses[0], losses
    # training is deterministic
    lpc2 = eolc.LearnedPC(0, seed=2)
    train_lpc.generate(lpc2, 60, quads=16, steps_per_run=20, seed=2)
    losses2 = lpc2.train(6, lr=2e-3, seed=2)
    assert np.array_equal(losses, losses2)


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights committed")
def test_trained_network_needs_fewer_iterations_than_jacobi(eolc):
    """Gain of the trained network over the method without it (Jacobi), on
    the first steps of a 128x128-quad sheet, a size it was not trained on
    (train_lpc.py's recipe: 2,000 systems of a batch holding a 48x48 grid,
    the 256x256 sheet and six Delaunay sheets)."""
    s = scenes.sheet(128)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    lpc = eolc.LearnedPC(0)
    lpc.set_params(np.load(WEIGHTS))
    lpc.attach(ctx)
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    it_j, it_l, it_2 = [], [], []
    for k in range(6):
        xl, vl = x.copy(), v.copy()
        x2, v2 = x.copy(), v.copy()
        ij = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_JACOBI))
        il = ctx.step(xl, s["X"], vl, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=0, no_coarse=1))
        i2 = ctx.step(x2, s["X"], v2, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=0))
        assert il.status == eolc.OK and il.rel_res <= 1e-8
        assert i2.status == eolc.OK and i2.rel_res <= 1e-8
        assert np.abs(v2 - v).max() <= 1e-5 * np.abs(v).max()
        it_j.append(ij.iterations)
        it_l.append(il.iterations)
        it_2.append(i2.iterations)
    gain = 1.0 - np.mean(it_l) / np.mean(it_j)
    print("mean PCG iterations: Jacobi %.1f, learned %.1f (%.1f%% fewer), learned + coarse %.1f"
          % (np.mean(it_j), np.mean(it_l), 100 * gain, np.mean(it_2)))
    # the committed network alone (white-noise probes) needs ~45% fewer here
    assert gain >= 0.30
    # and the coarse-grid correction removes more
    assert np.mean(it_2) <= np.mean(it_l)


def test_learned_refresh_reuses_the_network_output(eolc):
    """With a refresh interval of 3 the network runs on solves 1 and 4 only;
    every solve still reaches the FP64 residual and Jacobi's velocities."""
    s = scenes.sheet(32)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    lpc = eolc.LearnedPC(0, seed=4)
    if os.path.exists(WEIGHTS):
        lpc.set_params(np.load(WEIGHTS))
    lpc.attach(ctx)
    ctx.set_learned_refresh(3)
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    counts = []
    for k in range(5):
        xl, vl = x.copy(), v.copy()
        ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                 eolc.SolveOpts(precond=eolc.PC_JACOBI))
        c0 = ctx.launch_count()
        info = ctx.step(xl, s["X"], vl, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                        eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=0))
        counts.append(ctx.launch_count() - c0)
        assert info.status == eolc.OK and info.rel_res <= 1e-8
        assert np.abs(vl - v).max() <= 1e-5 * np.abs(v).max()
    # the network (and the re-layout of its output) runs on solves 1 and 4
    assert counts[0] == counts[3] > counts[1] == counts[2] == counts[4], counts


def test_inference_blocks_match_cpu_reference(eolc):
    """The fused inference forward (the blocks EOLC_PC_LEARNED applies)
    against the same network in FP64 on the CPU (oracle/learned_ref.py)."""
    import learned_ref
    s, ctx, mat, MDK, rng = _system(eolc, 8, 0.5, 11)
    lpc = eolc.LearnedPC(0, seed=6)
    if os.path.exists(WEIGHTS):
        lpc.set_params(np.load(WEIGHTS))
    p = lpc.get_params() + rng.normal(0, 0.02, lpc.num_params()).astype(np.float32)
    lpc.set_params(p)
    G = lpc.blocks(ctx, s["fixed"]).astype(np.float64)
    rowptr, colidx = ctx.bsr_pattern()
    pinned = np.zeros(3 * s["n"], bool)
    pinned[s["fixed"]] = True
    Gref = learned_ref.g_blocks(p, MDK.astype(np.float32).reshape(-1, 9), rowptr, colidx, pinned)
    err = np.abs(G - Gref).max() / np.abs(Gref).max()
    print("inference G vs CPU reference: %.2e" % err)
    assert err <= 1e-5, err


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights committed")
def test_learned_step_is_faster_than_jacobi_step(eolc):
    """At 128x128 quads the learned step (network re-run every 4 solves, the
    coarse correction on) takes less time than the resident Jacobi step,
    both to the same FP64 relative residual (host time around one call of
    the resident stepper, which returns after the step's status has been
    read back; 6 steps after 2 untimed ones, the same start state)."""
    import time
    s = scenes.sheet(128)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    lpc = eolc.LearnedPC(0)
    lpc.set_params(np.load(WEIGHTS))
    lpc.attach(ctx)
    x0, v0 = s["x"].copy(), np.zeros(3 * s["n"])
    ms = {}
    for name, opts, refresh in (
            ("jacobi", eolc.SolveOpts(precond=eolc.PC_JACOBI), 1),
            ("learned", eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=0), 4)):
        ctx.set_learned_refresh(refresh)
        ctx.set_coarse_refresh(refresh)
        ctx.state_upload(x0, s["X"], v0)
        ctx.step_resident(2, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"], opts)
        t = []
        for k in range(6):
            t0 = time.perf_counter()
            info = ctx.step_resident(1, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                                     opts)
            t.append(1e3 * (time.perf_counter() - t0))
            assert info.status == eolc.OK and info.rel_res <= 1e-8
        ms[name] = float(np.mean(t))
    ctx.set_learned_refresh(1)
    ctx.set_coarse_refresh(1)
    print("step ms at 128^2: Jacobi %.3f, learned %.3f (%.2fx)"
          % (ms["jacobi"], ms["learned"], ms["jacobi"] / ms["learned"]))
    assert ms["learned"] < ms["jacobi"]
