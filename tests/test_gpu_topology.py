"""Device topology build (csrc/topology_gpu.cu) against the oracle
(oracle/topology_ref.py), array for array: BSR pattern, per-block
contribution lists in the reference's insertion order, node -> face lists;
on a regular sheet, irregular Delaunay meshes and a batched topology; from
host arrays and from device arrays; invalid topologies rejected; and a
refresh followed by a step gives the same result as a fresh context."""
import time

import numpy as np
import pytest

import oracle as O
import scenes
import topology_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _same(got, want):
    for k in ("rowptr", "colidx", "cptr", "contrib", "nf_ptr", "nf_list"):
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("case", ["sheet8", "sheet256", "delaunay", "delaunay_big"])
def test_device_build_matches_oracle(eolc, case):
    if case.startswith("sheet"):
        s = scenes.sheet(int(case[5:]))
    else:
        s = scenes.delaunay_sheet(2000 if case == "delaunay" else 60000,
                                  np.random.default_rng(7))
    ctx = eolc.Context(0)
    t0 = time.perf_counter()
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    ms = 1e3 * (time.perf_counter() - t0)
    print("%s: %d nodes, set_topology %.2f ms" % (case, s["n"], ms))
    _same(ctx.topology_arrays(), topology_ref.build(s["n"], s["tri"], s["hinge"]))


def test_batched_topology_matches_oracle(eolc):
    B = scenes.batch(6, lo=8, hi=20, seed=2)
    ctx = eolc.Context(0)
    ctx.set_topology_batched([(sh["n"], sh["tri"], sh["hinge"]) for sh in B["sheets"]])
    off, tris, hinges = 0, [], []
    for sh in B["sheets"]:
        tris.append(np.asarray(sh["tri"]).reshape(-1, 3) + off)
        hinges.append(np.asarray(sh["hinge"]).reshape(-1, 4) + off)
        off += sh["n"]
    _same(ctx.topology_arrays(), topology_ref.build(off, np.concatenate(tris),
                                                    np.concatenate(hinges)))


def test_device_arrays_and_refresh(eolc):
    """eolc_set_topology_device from CUDA tensors equals the host-array
    build; a context refreshed from one mesh to another steps like a fresh
    context on the second mesh."""
    import torch
    a = scenes.sheet(12)
    b = scenes.delaunay_sheet(800, np.random.default_rng(3))
    ctx = eolc.Context(0)
    ctx.set_topology(a["n"], a["tri"], a["hinge"])
    tri = torch.tensor(np.asarray(b["tri"], np.int32).ravel(), device="cuda")
    hin = torch.tensor(np.asarray(b["hinge"], np.int32).ravel(), device="cuda")
    torch.cuda.synchronize()
    ctx.set_topology_device(b["n"], tri.data_ptr(), len(b["tri"]), hin.data_ptr(),
                            len(np.asarray(b["hinge"]).reshape(-1, 4)))
    _same(ctx.topology_arrays(), topology_ref.build(b["n"], b["tri"], b["hinge"]))
    fresh = eolc.Context(0)
    fresh.set_topology(b["n"], b["tri"], b["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    out = []
    for c in (ctx, fresh):
        x, v = b["x"].copy(), np.zeros(3 * b["n"])
        for k in range(2):
            c.step(x, b["X"], v, mat, scenes.GRAV, scenes.H, b["fixed"], b["fixed_vel"])
        out.append((x, v))
        rp, ci = c.bsr_pattern()
        assert rp[-1] == len(ci)
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("bad", ["range", "degenerate", "isolated"])
def test_invalid_topologies_are_rejected(eolc, bad):
    s = scenes.sheet(4)
    tri = np.asarray(s["tri"]).reshape(-1, 3).copy()
    n = s["n"]
    if bad == "range":
        tri[3, 1] = n
    elif bad == "degenerate":
        tri[2, 2] = tri[2, 0]
    else:
        n = n + 1  # a node no element uses
    ctx = eolc.Context(0)
    with pytest.raises(eolc.EolcError) as e:
        ctx.set_topology(n, tri, s["hinge"] if bad != "isolated" else s["hinge"])
    assert e.value.status == eolc.BAD_ARG
    # the context is still usable
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    _same(ctx.topology_arrays(), topology_ref.build(s["n"], s["tri"], s["hinge"]))


@pytest.mark.parametrize("case", ["sheet16", "sheet160", "delaunay"])
def test_edge_list_matches_oracle(eolc, case):
    """CD2's edge list built on the device against the oracle's createEdges
    (oracle/collide.cpp), row for row; the 160x160 sheet (51,200 faces) is
    past the size where the reference's 32-bit hash wraps."""
    if case.startswith("sheet"):
        s = scenes.sheet(int(case[5:]))
    else:
        s = scenes.delaunay_sheet(5000, np.random.default_rng(4))
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    got = ctx.edge_list()
    want = O.create_edges(s["x"], s["tri"])
    assert got.shape[0] == want.shape[0]
    assert np.array_equal(got[:, 0], want[:, 0]) and np.array_equal(got[:, 1], want[:, 1])
    assert np.array_equal(got[:, 2], want[:, 4]) and np.array_equal(got[:, 3], want[:, 5])
