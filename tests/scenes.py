"""Seeded synthetic scenes with the shapes of the benchmark configurations.

The reference ships no scenes with the benchmark sizes and no datasets; these
generators build the same meshes (two-triangle grids of the stated node and
triangle counts, the reference's corner pins and material) so tests, smoke()
and bench.py all run the same workloads.
"""
import numpy as np

import eolc  # the library's own mesh input builders (numpy; no GPU needed)

GRAV = [0.0, 0.0, -9.8]
H = 5e-3


def material_c1():
    """Configuration 1 material: rho 0.1, E 50, nu 0.3, beta 1e-5, damping (0, 1)."""
    return dict(density=0.1, e=50.0, nu=0.3, beta=1e-5, damping=(0.0, 1.0))


def sheet(quads, pins=(3, 4)):
    """Unit square sheet of quads x quads two-triangle quads, pinned at the
    named corners (ids of parseParams.cpp:298-305, all three axes, zero
    scripted velocity)."""
    r = quads + 1
    x, X, tri = eolc.sheet_mesh(r, r)
    hinge = eolc.mesh_hinges(tri)
    ids = eolc.corner_ids(r, r)
    fixed = np.array([3 * ids[k] + c for k in pins for c in range(3)], np.int32)
    return dict(x=x, X=X, tri=tri, hinge=hinge, fixed=fixed,
                fixed_vel=np.zeros(len(fixed)), n=r * r)


def drape_positions(quads, steps, seed=7, jitter=1e-4, box_dim=(0.4, 0.4, 0.2),
                    gap=0.05, threshold=1e-3):
    """Kinematic drape of a quads x quads sheet over an axis-aligned box whose
    top face starts `gap` below the sheet: the sheet sinks through the top face
    while its outer part bends down over the box edges, so the three contact
    kinds (cloth vertex / box face, box corner / cloth face, edge / edge)
    all occur.  Each snapshot is jittered N(0, jitter) from a seeded
    generator.  Returns (x0, X, tri, box_center, snapshots)."""
    r = quads + 1
    x0, X, tri = eolc.sheet_mesh(r, r)
    rng = np.random.default_rng(seed)
    xy = x0.reshape(-1, 3)[:, :2]
    half = np.array(box_dim[:2]) / 2
    c = np.array([0.5, 0.5])
    d_out = np.linalg.norm(np.maximum(np.abs(xy - c) - half, 0.0), axis=1)
    top = -gap
    center = [0.5, 0.5, top - box_dim[2] / 2]
    snaps = []
    for k in range(steps):
        t = k / max(1, steps - 1)
        # approach during the first quarter, then hover within +-4 thresholds
        # of the top face while the outer part folds down over the edges
        if t < 0.25:
            lift = gap * (1 - 4 * t) ** 2 + 4 * threshold
        else:
            lift = 4 * threshold * np.cos(9 * np.pi * (t - 0.25))
        z = top + lift - 1.5 * d_out * min(1.0, 2 * t)
        x = x0.copy().reshape(-1, 3)
        x[:, 2] = z
        x = x.ravel() + rng.normal(0.0, jitter, x.size)
        snaps.append(x)
    return x0, X, tri, center, snaps


def batch(n_sheets, lo=16, hi=96, seed=3, e_range=(20.0, 100.0), pins=(3, 4)):
    """Batched workload: n_sheets independent unit sheets whose side (in
    quads) is drawn uniformly from lo..hi and whose Young's modulus is drawn
    uniformly from e_range (seeded), the configuration-1 material otherwise,
    each pinned at the named corners.  Returns the per-sheet scenes, their
    materials and the concatenated state and fixed-DOF list (global DOFs)."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(lo, hi + 1, n_sheets)
    es = rng.uniform(e_range[0], e_range[1], n_sheets)
    sheets, mats, off = [], [], [0]
    for q, e in zip(sides, es):
        s = sheet(int(q), pins)
        sheets.append(s)
        m = material_c1()
        m["e"] = float(e)
        mats.append(m)
        off.append(off[-1] + s["n"])
    x = np.concatenate([s["x"] for s in sheets])
    X = np.concatenate([s["X"] for s in sheets])
    fixed = np.concatenate([s["fixed"] + 3 * o for s, o in zip(sheets, off[:-1])]).astype(np.int32)
    return dict(sheets=sheets, mats=mats, sides=sides, node_off=np.array(off), x=x, X=X,
                v=np.zeros_like(x), fixed=fixed, fixed_vel=np.zeros(len(fixed)))


def delaunay_sheet(n_tri, rng, gradient=3.0):
    """Irregular unit sheet of about n_tri triangles, mimicking a remeshed
    sheet refined toward one side: the seeded Delaunay triangulation of a
    jittered lattice (each point moved by up to 0.35 of a cell) whose x
    coordinate is warped so that the point density grows linearly along x
    (density 1 + gradient x), boundary points on the square's edges.
    Triangles counter-clockwise in material space, hinges in ArcSim edge
    order, the two top corners (0, 1), (1, 1) pinned."""
    from scipy.spatial import Delaunay
    m = max(2, int(round(np.sqrt(max(8, n_tri // 2)))))
    g = gradient

    def warp(u):  # inverse CDF of the density (1 + g x) / (1 + g / 2) on [0, 1]
        return (-1 + np.sqrt(1 + 2 * g * u * (1 + g / 2))) / g if g > 0 else u

    t = np.arange(m + 1) / m
    bnd = np.concatenate([np.stack([warp(t), np.zeros(m + 1)], 1),
                          np.stack([warp(t), np.ones(m + 1)], 1),
                          np.stack([np.zeros(m - 1), t[1:-1]], 1),
                          np.stack([np.ones(m - 1), t[1:-1]], 1)])
    ii, jj = np.meshgrid(np.arange(1, m), np.arange(1, m), indexing="ij")
    u = (ii + rng.uniform(-0.35, 0.35, ii.shape)) / m
    v = (jj + rng.uniform(-0.35, 0.35, jj.shape)) / m
    inner = np.stack([warp(u.ravel()), v.ravel()], 1)
    pts = np.concatenate([bnd, inner])
    tri = Delaunay(pts).simplices.astype(np.int64)
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    area = 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
    flip = area < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    tri = tri[np.abs(area) > 1e-12]
    used = np.unique(tri)
    remap = -np.ones(len(pts), np.int64)
    remap[used] = np.arange(len(used))
    tri = remap[tri].astype(np.int32)
    X = pts[used]
    n = len(X)
    x = np.concatenate([X, np.zeros((n, 1))], 1).ravel()
    hinge = eolc.mesh_hinges(tri)
    corners = [int(np.argmin((X[:, 0] - cx) ** 2 + (X[:, 1] - 1.0) ** 2)) for cx in (0.0, 1.0)]
    fixed = np.array([3 * k + c for k in corners for c in range(3)], np.int32)
    return dict(x=x, X=X.ravel(), tri=tri, hinge=hinge, fixed=fixed, fixed_vel=np.zeros(len(fixed)),
                n=n)


def delaunay_batch(n_meshes, tri_lo=5000, tri_hi=50000, seed=5):
    """Batched irregular workload: n_meshes Delaunay sheets of U(tri_lo,
    tri_hi) triangles (seeded), configuration-1 material, top corners pinned;
    the same layout as batch()."""
    rng = np.random.default_rng(seed)
    sheets, mats, off = [], [], [0]
    for k in range(n_meshes):
        s = delaunay_sheet(int(rng.integers(tri_lo, tri_hi + 1)), rng)
        sheets.append(s)
        mats.append(material_c1())
        off.append(off[-1] + s["n"])
    x = np.concatenate([s["x"] for s in sheets])
    X = np.concatenate([s["X"] for s in sheets])
    fixed = np.concatenate([s["fixed"] + 3 * o for s, o in zip(sheets, off[:-1])]).astype(np.int32)
    return dict(sheets=sheets, mats=mats, node_off=np.array(off), x=x, X=X,
                v=np.zeros_like(x), fixed=fixed, fixed_vel=np.zeros(len(fixed)))


def eol_edge_sheet(quads, pins=True):
    """A unit sheet lying on a box whose +x/+z edge runs along y at x = 0.5,
    z = 0 (box 1 x 2 x 0.2 centred at (0, 0.5, -0.1)): the half x < 0.5 rests
    on the top face, the half x > 0.5 hangs free, and the column of nodes on
    the edge line are the EOL nodes (EoL_index in node order), each on box
    edge 10 (faces +x and +z, constraint-table column 18 with no point
    obstacles), the edges between them preserved.  quads must be even.
    pins=True pins the two corners on the far side of the top face (x = 0).
    Returns the mesh, the EOL tables, the obstacle (as an axis-aligned box
    centre and dimensions) and the pins."""
    assert quads % 2 == 0
    r = quads + 1
    x, X, tri = eolc.sheet_mesh(r, r)
    xy = x.reshape(-1, 3)
    eol = np.flatnonzero(np.abs(xy[:, 0] - 0.5) < 1e-12).astype(np.int32)
    edges = eolc.mesh_edges(tri)
    is_eol = np.zeros(len(xy), bool)
    is_eol[eol] = True
    preserve = (is_eol[edges[:, 0]] & is_eol[edges[:, 1]]).astype(np.int32)
    fixed = np.zeros(0, np.int32)
    if pins:
        far = np.flatnonzero((np.abs(xy[:, 0]) < 1e-12) &
                             ((np.abs(xy[:, 1]) < 1e-12) | (np.abs(xy[:, 1] - 1) < 1e-12)))
        fixed = np.array([3 * a + c for a in far for c in range(3)], np.int32)
    return dict(x=x, X=X, tri=tri, hinge=eolc.mesh_hinges(tri), edges=edges, eol=eol,
                preserve=preserve, corner=-np.ones(len(eol), np.int32),
                cd=np.full(len(eol), 8 + 10, np.int32), box_center=[0.0, 0.5, -0.1],
                box_dim=[1.0, 2.0, 0.2], fixed=fixed, fixed_vel=np.zeros(len(fixed)),
                n=len(xy))
