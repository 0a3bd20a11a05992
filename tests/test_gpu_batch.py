"""Batched stepping: many sheets of uneven size in one persistent launch.

Every batched result is compared with the one-sheet path (itself checked
against the oracle in test_gpu_parity.py): from the same state, a batched
step of every instance must give the velocities and positions of a one-sheet
step of that instance with its own material, to the tolerance the two
solves' relative residual allows.  Every solver configuration the autotuner
may pick is run, and each must reach the FP64 relative residual.
"""
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


def _batch_ctx(eolc, B):
    ctx = eolc.Context(0)
    ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in B["sheets"]])
    ctx.set_instance_materials([eolc.Material(**m) for m in B["mats"]])
    return ctx


def _single_steps(eolc, B, x, v, opts):
    """One one-sheet step of every instance from the batched state (x, v)."""
    off = B["node_off"]
    xs, vs, infos = [], [], []
    for k, (s, m) in enumerate(zip(B["sheets"], B["mats"])):
        ctx = eolc.Context(0)
        ctx.set_topology(s["n"], s["tri"], s["hinge"])
        xk = x[3 * off[k]:3 * off[k + 1]].copy()
        vk = v[3 * off[k]:3 * off[k + 1]].copy()
        info = ctx.step(xk, s["X"], vk, eolc.Material(**m), scenes.GRAV, scenes.H, s["fixed"],
                        s["fixed_vel"], opts)
        xs.append(xk)
        vs.append(vk)
        infos.append(info)
    return np.concatenate(xs), np.concatenate(vs), infos


def _perturbed(B, seed, amp=0.003):
    rng = np.random.default_rng(seed)
    return B["x"] + rng.normal(0, amp, B["x"].size)


def _compare(B, got, want, tol):
    off = B["node_off"]
    for k in range(len(B["sheets"])):
        g = got[3 * off[k]:3 * off[k + 1]]
        w = want[3 * off[k]:3 * off[k + 1]]
        err = np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)
        assert err <= tol, (k, err)


@pytest.mark.parametrize("precision,tol,rel_tol", [("mixed", 1e-5, 1e-8), ("fp64", 1e-9, 1e-12)])
def test_batched_steps_match_one_sheet_steps(eolc, precision, tol, rel_tol):
    B = scenes.batch(7, lo=4, hi=20, seed=11)
    prec = eolc.PREC_MIXED if precision == "mixed" else eolc.PREC_FP64
    opts = eolc.SolveOpts(rel_tol=rel_tol, precision=prec)
    ctx = _batch_ctx(eolc, B)
    x, v = _perturbed(B, 1), B["v"].copy()
    for step in range(3):
        ctx.state_upload(x, B["X"], v)
        tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
        assert tot.status == eolc.OK and tot.n_failed == 0 and tot.steps == 1
        assert all(i.status == eolc.OK and i.rel_res <= rel_tol for i in infos)
        xb, vb = ctx.state_download()
        xs, vs, sinfo = _single_steps(eolc, B, x, v, opts)
        _compare(B, vb, vs, tol)
        _compare(B, xb, xs, tol)
        # the instance iteration counts are those of a one-sheet solve
        for ib, isg in zip(infos, sinfo):
            assert abs(ib.iterations - isg.iterations) <= max(3, isg.iterations // 10)
        x, v = xs, vs  # teacher forcing: the next step starts from the same state


def test_every_configuration_converges(eolc):
    B = scenes.batch(6, lo=4, hi=24, seed=5)
    opts = eolc.SolveOpts(rel_tol=1e-8)
    ctx = _batch_ctx(eolc, B)
    x = _perturbed(B, 2)
    xs, vs, _ = _single_steps(eolc, B, x, B["v"], opts)
    ran = 0
    for c in range(eolc.batch_num_configs()):
        ctx.batch_set_config(c)
        ctx.state_upload(x, B["X"], B["v"])
        tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
        assert tot.config == c, eolc.batch_config_name(c)
        assert tot.status == eolc.OK and tot.max_rel_res <= 1e-8, eolc.batch_config_name(c)
        _, vb = ctx.state_download()
        _compare(B, vb, vs, 1e-5)
        ran += 1
    assert ran == eolc.batch_num_configs()


def test_autotuner_keeps_the_fastest_configuration(eolc):
    B = scenes.batch(12, lo=8, hi=40, seed=9)
    opts = eolc.SolveOpts()
    ctx = _batch_ctx(eolc, B)
    ctx.state_upload(_perturbed(B, 3), B["X"], B["v"])
    x0, v0 = ctx.state_download()
    chosen, ms = ctx.batch_autotune(scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    valid = ms >= 0
    assert valid.any() and valid[chosen] and ms[chosen] == ms[valid].min()
    print("autotune: " + ", ".join("%d: %.3f ms" % (c, t) for c, t in enumerate(ms)))
    print("chosen %d (%s)" % (chosen, eolc.batch_config_name(chosen)))
    # the autotuner leaves the state alone
    x1, v1 = ctx.state_download()
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    tot, _ = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.config == chosen and tot.status == eolc.OK


def test_graph_replays_are_deterministic(eolc):
    """n steps in one call (n graph replays) equal n calls of one step, bit for
    bit, and equal a fresh context's run."""
    B = scenes.batch(5, lo=6, hi=18, seed=4)
    opts = eolc.SolveOpts()
    x = _perturbed(B, 4)
    ctx = _batch_ctx(eolc, B)
    ctx.batch_set_config(0)
    ctx.state_upload(x, B["X"], B["v"])
    tot, _ = ctx.step_batched(3, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.steps == 3 and tot.status == eolc.OK
    xa, va = ctx.state_download()
    ctx2 = _batch_ctx(eolc, B)
    ctx2.batch_set_config(0)
    ctx2.state_upload(x, B["X"], B["v"])
    for _ in range(3):
        ctx2.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    xb, vb = ctx2.state_download()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_block_jacobi_batched(eolc):
    B = scenes.batch(4, lo=6, hi=16, seed=8)
    opts = eolc.SolveOpts(precond=eolc.PC_BLOCK_JACOBI)
    ctx = _batch_ctx(eolc, B)
    x = _perturbed(B, 5)
    ctx.state_upload(x, B["X"], B["v"])
    tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.status == eolc.OK
    _, vb = ctx.state_download()
    _, vs, _ = _single_steps(eolc, B, x, B["v"], eolc.SolveOpts())
    _compare(B, vb, vs, 1e-5)


def test_batch_argument_errors(eolc):
    B = scenes.batch(3, lo=4, hi=6, seed=1)
    ctx = eolc.Context(0)
    ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in B["sheets"]])
    with pytest.raises(eolc.EolcError) as e:  # no materials yet
        ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"])
    assert e.value.status == eolc.BAD_ARG
    with pytest.raises(eolc.EolcError) as e:  # wrong material count
        ctx.set_instance_materials([eolc.Material(**B["mats"][0])])
    assert e.value.status == eolc.BAD_ARG
    ctx.set_instance_materials([eolc.Material(**m) for m in B["mats"]])
    with pytest.raises(eolc.EolcError) as e:
        ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"],
                         eolc.SolveOpts(precond=eolc.PC_LEARNED))
    assert e.value.status == eolc.BAD_ARG
    # a triangle that joins two instances is rejected
    s0, s1 = B["sheets"][0], B["sheets"][1]
    bad = s1["tri"].copy()
    bad[0, 0] = -s0["n"]  # becomes node 0 of instance 0 after the offset
    with pytest.raises(eolc.EolcError) as e:
        ctx.set_topology_batched([(s0["n"], s0["tri"], s0["hinge"]), (s1["n"], bad, s1["hinge"])])
    assert e.value.status == eolc.BAD_ARG


WEIGHTS = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.dirname(
    __import__("os").path.abspath(__file__))), "eol-cloth_gb300", "weights", "lpc.npy")


def _learned_batch(eolc, B, seed=0, trained=True):
    ctx = _batch_ctx(eolc, B)
    lpc = eolc.LearnedPC(0, seed=seed)
    if trained:
        lpc.set_params(np.load(WEIGHTS))
    lpc.attach(ctx)
    return ctx, lpc


def test_batched_learned_steps_on_delaunay_meshes(eolc):
    """Irregular meshes, learned batched solve: every instance reaches the
    FP64 residual and the velocities of a one-sheet Jacobi step."""
    B = scenes.delaunay_batch(5, tri_lo=600, tri_hi=3000, seed=2)
    ctx, lpc = _learned_batch(eolc, B)
    x = B["x"].copy()
    ctx.state_upload(x, B["X"], B["v"])
    # Jacobi steps set every instance's reference count; the last one from a
    # moving state (the first solve from rest, a pure gravity load, is short)
    tot, _ = ctx.step_batched(2, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"],
                              eolc.SolveOpts())
    assert tot.status == eolc.OK
    x1, v1 = ctx.state_download()
    opts = eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=2)
    tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.status == eolc.OK and tot.max_rel_res <= 1e-8
    assert tot.n_fallback == 0, [i.iterations for i in infos]
    _, vb = ctx.state_download()
    _, vs, sinfo = _single_steps(eolc, B, x1, v1, eolc.SolveOpts())
    _compare(B, vb, vs, 1e-5)
    print("learned iterations %s, Jacobi %s" % ([i.iterations for i in infos],
                                                 [i.iterations for i in sinfo]))
    assert sum(i.iterations for i in infos) < sum(i.iterations for i in sinfo)


def test_batched_learned_falls_back_per_instance(eolc):
    """References of 1 iteration cap every learned solve at 2: each instance
    falls back to Jacobi inside the same step and still converges."""
    B = scenes.delaunay_batch(4, tri_lo=600, tri_hi=2000, seed=3)
    ctx, lpc = _learned_batch(eolc, B, trained=False)
    ctx.state_upload(B["x"], B["X"], B["v"])
    ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], eolc.SolveOpts())
    x1, v1 = ctx.state_download()
    refs = np.ones(len(B["sheets"]), np.int32)
    refs[0] = 100000  # instance 0 is not capped
    ctx.batch_set_jacobi_reference(refs)
    opts = eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=2)
    tot, infos = ctx.step_batched(1, scenes.GRAV, scenes.H, B["fixed"], B["fixed_vel"], opts)
    assert tot.status == eolc.OK and tot.max_rel_res <= 1e-8
    assert [i.used_fallback for i in infos] == [0] + [1] * (len(infos) - 1)
    _, vb = ctx.state_download()
    _, vs, _ = _single_steps(eolc, B, x1, v1, eolc.SolveOpts())
    _compare(B, vb, vs, 1e-5)
