"""Configuration 2 at its size: the contact set of CD2 on a 128 x 128-quad
sheet (16,641 nodes, 32,768 triangles) over a 0.4 x 0.4 x 0.2 m box whose top
face starts 0.05 m below the sheet, threshold 1e-3 m, node positions
jittered N(0, 1e-4 m) from a recorded seed, 200 steps.  At every step the
library's eolc_cd2 and the oracle's restatement of Collisions::CD2 /
btc::boxTriCollision (Collisions.cpp:55-78, boxTriCollision.cpp:602-1063)
get the same positions and must return the same contacts bit for bit, in
the same order.  The 200 positions follow the seeded drape of
tests/scenes.py: the sheet approaches the box, sinks through its top face
within a few thresholds and folds down over its edges, so vertex-face,
corner-face and edge-edge contacts all occur."""
import ctypes

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

C2_QUADS = 128
C2_STEPS = 200
C2_SEED = 2024        # seed of the N(0, 1e-4) jitter
C2_BOX = (0.4, 0.4, 0.2)
C2_GAP = 0.05
C2_THRESHOLD = 1e-3


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _first_difference(eolc, got, want):
    """Index and field of the first contact that differs (for the message)."""
    size = ctypes.sizeof(eolc.Contact)
    n = min(len(got), len(want)) // size
    for k in range(n):
        a, b = got[k * size:(k + 1) * size], want[k * size:(k + 1) * size]
        if a != b:
            ca, cb = eolc.Contact.from_buffer_copy(a), eolc.Contact.from_buffer_copy(b)
            for name, _ in eolc.Contact._fields_:
                va, vb = getattr(ca, name), getattr(cb, name)
                va = list(va) if hasattr(va, "__len__") else va
                vb = list(vb) if hasattr(vb, "__len__") else vb
                if va != vb:
                    return "contact %d field %s: %r vs %r" % (k, name, va, vb)
    return "counts %d vs %d" % (len(got) // size, len(want) // size)


def test_c2_contact_set_bit_exact_200_steps(eolc, oracle):
    x0, X, tri, center, snaps = scenes.drape_positions(
        C2_QUADS, C2_STEPS, seed=C2_SEED, jitter=1e-4, box_dim=C2_BOX, gap=C2_GAP,
        threshold=C2_THRESHOLD)
    n = len(x0) // 3
    assert n == 16641 and len(tri) == 32768
    ctx = eolc.Context(0)
    ctx.set_topology(n, tri, eolc.mesh_hinges(tri))
    ob = oracle.axis_box(center, C2_BOX)
    gb = eolc.Box(list(ob.dim), list(ob.E1))
    size = ctypes.sizeof(eolc.Contact)
    kinds, total, steps_with_contacts = set(), 0, 0
    for k, x in enumerate(snaps):
        want = oracle.cd2(x, tri, boxes=[ob], threshold=C2_THRESHOLD, raw=True)
        got = ctx.cd2(x, boxes=[gb], threshold=C2_THRESHOLD, raw=True)
        assert got == want, "step %d: %s" % (k, _first_difference(eolc, got, want))
        m = len(want) // size
        total += m
        steps_with_contacts += m > 0
        for j in range(m):
            c = eolc.Contact.from_buffer_copy(want[j * size:(j + 1) * size])
            kinds.add((c.count1, c.count2))
    # vertex / box face, box corner / cloth face and edge / edge contacts
    assert {(3, 1), (1, 3), (2, 2)} <= kinds, kinds
    assert steps_with_contacts > C2_STEPS // 2 and total > 100000, (steps_with_contacts, total)


def test_cd2_matches_reference_fixtures(eolc):
    """eolc_cd2 returns the reference's own contact records (fixtures from
    src/boxTriCollision.cpp compiled unmodified), bit for bit and in order,
    on the drape, point-obstacle and configuration-2 snapshots."""
    import test_oracle_golden as TG
    g = np.load(TG.CD_GOLD)
    n = 0
    for name in TG.CD_SCENES:
        ctx = eolc.Context(0)
        tri = g[name + "_tri"]
        nn = len(g[name + "_x"][0]) // 3
        ctx.set_topology(nn, tri, eolc.mesh_hinges(tri))
        for x, tri, boxes, pts, nrm, thr, want in TG.cd_cases(g, name):
            gb = [eolc.Box(list(b.dim), list(b.E1)) for b in boxes]
            got = ctx.cd2(x, boxes=gb, points=pts, normals=nrm, threshold=thr, raw=True)
            assert got == want, "%s: %s" % (name, _first_difference(eolc, got, want))
            n += len(want) // ctypes.sizeof(eolc.Contact)
    assert n > 2500
