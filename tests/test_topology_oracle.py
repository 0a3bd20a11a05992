"""The topology oracle (oracle/topology_ref.py) on the CPU: its BSR pattern
is the block sparsity of the oracle's assembled MDK, every block's
contribution list holds exactly the elements that contain both nodes, and
each node's face list is its faces in order."""
import numpy as np

import oracle as O
import scenes
import topology_ref


def _check(s):
    tri, hinge, n = np.asarray(s["tri"]).reshape(-1, 3), np.asarray(s["hinge"]).reshape(-1, 4), s["n"]
    t = topology_ref.build(n, tri, hinge)
    F = O.Forces(s["x"], s["X"], tri, hinge, O.material(), scenes.GRAV, scenes.H)
    A = F.csr(1).tocoo()
    blocks = set(zip((A.row // 3).tolist(), (A.col // 3).tolist()))
    got = {(i, int(c)) for i in range(n) for c in t["colidx"][t["rowptr"][i]:t["rowptr"][i + 1]]}
    assert got == blocks
    for i in range(n):
        cols = t["colidx"][t["rowptr"][i]:t["rowptr"][i + 1]]
        assert (np.diff(cols) > 0).all()
    for b in range(0, len(t["colidx"]), max(1, len(t["colidx"]) // 500)):
        row = int(np.searchsorted(t["rowptr"], b, side="right") - 1)
        col = int(t["colidx"][b])
        codes = t["contrib"][t["cptr"][b]:t["cptr"][b + 1]]
        want = [(f << 7) | (a << 3) | c for f in range(len(tri)) for a in range(3)
                for c in range(3) if tri[f, a] == row and tri[f, c] == col]
        want += [(e << 7) | 64 | (a << 3) | c for e in range(len(hinge)) for a in range(4)
                 for c in range(4) if hinge[e, a] == row and hinge[e, c] == col]
        assert codes.tolist() == want
    for i in range(0, n, max(1, n // 100)):
        lst = t["nf_list"][t["nf_ptr"][i]:t["nf_ptr"][i + 1]].tolist()
        assert lst == [(f << 2) | a for f in range(len(tri)) for a in range(3) if tri[f, a] == i]


def test_sheet():
    _check(scenes.sheet(8))


def test_delaunay():
    _check(scenes.delaunay_sheet(300, np.random.default_rng(1)))
