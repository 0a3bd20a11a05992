"""The library's mesh input builders (eolc.sheet_mesh, eolc.mesh_hinges)
against the oracle's C restatement of Cloth::build's blend (Cloth.cpp:63-76)
and ArcSim's edge creation (mesh.cpp:356-378): bit-identical positions,
triangles and hinges."""
import numpy as np
import pytest

import eolc
import scenes


@pytest.mark.parametrize("r0,r1", [(2, 2), (3, 5), (21, 21), (65, 33), (129, 129), (257, 257)])
def test_sheet_mesh_matches_oracle(oracle, r0, r1):
    x, X, tri = oracle.grid2(r0, r1)
    x2, X2, tri2 = eolc.sheet_mesh(r0, r1)
    assert np.array_equal(x.view(np.int64), x2.view(np.int64))
    assert np.array_equal(X.view(np.int64), X2.view(np.int64))
    assert np.array_equal(tri, tri2)
    assert np.array_equal(oracle.hinges(r0 * r1, tri), eolc.mesh_hinges(tri2))
    assert eolc.corner_ids(r0, r1) == oracle.corner_ids(r0, r1)


def test_hinges_of_irregular_meshes_match_oracle(oracle):
    rng = np.random.default_rng(11)
    for n_tri in (60, 900, 7000, 24000):
        s = scenes.delaunay_sheet(n_tri, rng)
        assert np.array_equal(oracle.hinges(s["n"], s["tri"]), eolc.mesh_hinges(s["tri"]))
    # the reference's centre-node grid (four triangles per quad)
    x, X, tri = oracle.gridc(9, 7)
    assert np.array_equal(oracle.hinges(len(x) // 3, tri), eolc.mesh_hinges(tri))


def test_hinges_edge_cases():
    assert eolc.mesh_hinges(np.zeros((0, 3), np.int32)).shape == (0, 4)
    # one triangle: no interior edge
    assert eolc.mesh_hinges(np.array([[0, 1, 2]], np.int32)).shape == (0, 4)
    # two triangles sharing edge (0, 2): one hinge, x2 / x3 on the right sides
    h = eolc.mesh_hinges(np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    assert h.tolist() == [[2, 0, 1, 3]]
