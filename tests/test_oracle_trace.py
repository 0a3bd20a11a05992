"""The oracle's whole step against its committed 100-step trace of the 20 x 20
sheet (tests/golden/trace_c1.npz, made by tests/golden/make_trace.py): per
step the CG iteration count, the relative residual and weighted checksums of
f, M and MDK; at the checkpoints x and v.  A regression pin of the oracle's
Cloth::step (its element math is pinned to the reference's own routines by
test_oracle_golden.py)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_trace  # noqa: E402


def _rel(a, b):
    return np.abs(a - b).max() / max(1e-300, np.abs(b).max())


def test_oracle_reproduces_trace(oracle):
    want = np.load(os.path.join(HERE, "golden", "trace_c1.npz"))
    got = make_trace.run()
    assert np.array_equal(got["checkpoints"], want["checkpoints"])
    # the same arithmetic on the same inputs: counts equal up to one
    # iteration where a residual sits on the 1e-8 threshold
    assert np.abs(got["iters"] - want["iters"]).max() <= 1
    assert got["rel_res"].max() <= 1e-8
    # weighted sums against the sums of |entries| (columns 1, 3, 5)
    scale = want["fill_sums"][:, 1::2].repeat(2, axis=1)
    assert np.abs(got["fill_sums"] - want["fill_sums"]).max() <= 1e-9 * scale.min()
    assert _rel(got["x"], want["x"]) <= 1e-9
    assert _rel(got["v"], want["v"]) <= 1e-7


def test_trace_is_a_falling_pinned_sheet():
    """Physical sanity of the stored run: the pinned corners stay put, the
    sheet falls (mean z decreases), the first fill's mass checksum is the
    same at every step (M depends on X only), and every consecutive
    checkpoint pair is one step x' = x + h v'."""
    d = np.load(os.path.join(HERE, "golden", "trace_c1.npz"))
    import scenes
    s = scenes.sheet(make_trace.QUADS)
    for x in d["x"]:
        assert np.array_equal(x[s["fixed"]], s["x"][s["fixed"]])
    z = d["x"][:, 2::3].mean(axis=1)
    assert np.all(np.diff(z) < 0)
    cp = list(d["checkpoints"])
    for a in (1, 5, 50):
        i, j = cp.index(a), cp.index(a + 1)
        assert np.abs(d["x"][j] - (d["x"][i] + 5e-3 * d["v"][j])).max() <= 1e-15
    m = d["fill_sums"][:, 2:4]
    assert np.abs(m - m[0]).max() <= 1e-12 * m[0, 1]
