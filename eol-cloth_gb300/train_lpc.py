"""Train the learned preconditioner on systems the simulator generates.

Systems: runs of the implicit-Euler stepper on a quads x quads sheet with
seeded random pinning (a random non-empty subset of the four corners, plus a
few random boundary nodes), random wind (a constant horizontal body force
added to gravity), Young's modulus ~ U(20, 100) and a density scaled so that
the ratio of h^2 K to M spans the range of 64^2..256^2 sheets.  After every
step the context's FP32 MDK becomes one training system, with three probe
vectors.  probes="white" (default): seeded standard-normal vectors, for which
the expected probe loss is the Frobenius objective |F (G A - I)|_F^2 / n of
a sparse approximate inverse (all modes weighted alike, which is what the
conjugate-gradient iteration count depends on); probes="smooth": the step's
velocity and two seeded smooth random fields.

meshes="mixed" (generate_mixed): the systems come from one batched context
holding a 48x48 grid, a 256x256 grid (the benchmark sheet; --big) and six
irregular Delaunay sheets, so the network sees the benchmark's stencil and
remeshed-like ones.

Training: eolc_lpc_train (Adam on the GPU, the library's own forward and
backward kernels).  The committed weights come from the defaults, i.e.:

    python eol-cloth_gb300/train_lpc.py --systems 2000 --epochs 40 --lr 3e-3 --lr-final 1e-4 \
        --probes white --meshes mixed --big 256 --seed 1 --out eol-cloth_gb300/weights/lpc.npy
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)

import eolc  # noqa: E402

GRAV = np.array([0.0, 0.0, -9.8])
H = 5e-3


def grid_sheet(quads):
    """Two-triangle grid, node k = i*r + j at material (j, i)/(r-1), the
    reference's corner convention; hinges in ArcSim edge order."""
    r = quads + 1
    jj, ii = np.meshgrid(np.arange(r), np.arange(r))
    X = np.stack([jj.ravel() / (r - 1.0), ii.ravel() / (r - 1.0)], 1)
    x = np.concatenate([X, np.zeros((r * r, 1))], 1)
    tri = []
    for i in range(r - 1):
        for j in range(r - 1):
            k0 = i * r + j
            tri.append((k0, k0 + 1, k0 + r + 1))
            tri.append((k0, k0 + r + 1, k0 + r))
    tri = np.array(tri, np.int32)
    hinge = hinges_arcsim(r * r, tri)
    corners = {1: 0, 2: r * (r - 1), 3: r * r - 1, 4: r - 1}
    return x.ravel(), X.ravel(), tri, hinge, corners


def hinges_arcsim(n_nodes, tri):
    """Interior edges in the order ArcSim's Mesh::add(Face) creates them
    (mesh.cpp:356-378) with the stencil of Forces.cpp:687-697."""
    edges, lookup = [], {}
    for f, v in enumerate(tri):
        for i in range(3):
            a, b = int(v[i]), int(v[(i + 1) % 3])
            key = (min(a, b), max(a, b))
            if key not in lookup:
                lookup[key] = len(edges)
                edges.append([a, b, -1, -1])
        for i in range(3):
            a, b = int(v[(i + 1) % 3]), int(v[(i + 2) % 3])
            e = edges[lookup[(min(a, b), max(a, b))]]
            if e[0] == a:
                e[2] = f
            else:
                e[3] = f
    out = []
    for a, b, f0, f1 in edges:
        if f0 < 0 or f1 < 0:
            continue
        other = lambda f: [int(t) for t in tri[f] if t != a and t != b][0]
        out.append((a, b, other(f0), other(f1)))
    return np.array(out, np.int32)


def smooth_field(rng, X, n_modes=4):
    w = np.zeros((len(X) // 2, 3))
    Xr = X.reshape(-1, 2)
    for c in range(3):
        for _ in range(n_modes):
            kx, ky = rng.integers(1, 4, 2)
            ph = rng.uniform(0, 2 * np.pi, 2)
            w[:, c] += rng.normal() * np.sin(np.pi * kx * Xr[:, 0] + ph[0]) * \
                np.sin(np.pi * ky * Xr[:, 1] + ph[1])
    return w.ravel()


def make_probes(rng, X, v, kind, n=3):
    if kind == "white":
        return rng.standard_normal((n, v.size)).astype(np.float32)
    return np.stack([v / max(np.abs(v).max(), 1e-30)] +
                    [smooth_field(rng, X) for _ in range(n - 1)]).astype(np.float32)


def generate(lpc, n_systems, quads=64, steps_per_run=50, seed=1, device=0, ctx=None,
             probes="white"):
    """Adds n_systems simulator systems to lpc; returns the context."""
    rng = np.random.default_rng(seed)
    x0, X, tri, hinge, corners = grid_sheet(quads)
    n = len(x0) // 3
    if ctx is None:
        ctx = eolc.Context(device)
    ctx.set_topology(n, tri, hinge)
    r = quads + 1
    boundary = np.unique(np.concatenate([np.arange(r), np.arange(r) * r, np.arange(r) * r + r - 1,
                                         r * (r - 1) + np.arange(r)]))
    made = 0
    runs = 0
    while made < n_systems:
        runs += 1
        if runs > 50 * max(1, n_systems // steps_per_run + 1):
            raise RuntimeError("the simulator keeps failing; no training systems")
        k = rng.integers(1, 5)
        pins = [corners[c] for c in rng.choice([1, 2, 3, 4], size=k, replace=False)]
        pins += list(rng.choice(boundary, size=rng.integers(0, 4), replace=False))
        fixed = np.array(sorted({3 * p + c for p in pins for c in range(3)}), np.int32)
        wind = np.array([rng.normal(0, 3.0), rng.normal(0, 3.0), 0.0])
        n_eff = rng.uniform(64, 256)
        mat = eolc.Material(density=0.1 * (quads / n_eff) ** 2, e=rng.uniform(20, 100), nu=0.3,
                            beta=1e-5, damping=(0.0, 1.0))
        x, v = x0.copy(), np.zeros(3 * n)
        opts = eolc.SolveOpts(precision=eolc.PREC_MIXED, precond=eolc.PC_JACOBI)
        for s in range(steps_per_run):
            try:
                ctx.step(x, X, v, mat, GRAV + wind, H, fixed, np.zeros(len(fixed)), opts)
            except eolc.EolcError:
                # an indefinite MDK (the bending Hessian is not convex) ends
                # this run; its systems so far are kept
                break
            lpc.add_system(ctx, fixed, make_probes(rng, X, v, probes))
            made += 1
            if made >= n_systems:
                break
    return ctx


def generate_mixed(lpc, n_systems, seed=1, steps_per_run=40, device=0, n_delaunay=6,
                   quads=48, big=0, probes="white"):
    """Training systems on one batched topology that holds a quads x quads
    grid sheet, a big x big grid sheet (big > 0: the benchmark's own size)
    and n_delaunay irregular Delaunay sheets of 1,500-6,000 triangles
    (density gradient along x), so the network sees regular and
    remeshed-like stencils.  Per run: random pins per instance (a non-empty
    subset of the corners plus a few boundary nodes), random wind, E ~ U(20,
    100) and a density giving h^2 K / M of 64^2..256^2 sheets; every batched
    Jacobi step adds the whole batch's MDK as one system."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes  # mesh generators shared with the tests
    rng = np.random.default_rng(seed)
    sheets = []
    for q in ([quads] + ([big] if big > 0 else [])):
        x0, X, tri, hinge, corners = grid_sheet(q)
        sheets.append(dict(x=x0, X=X, tri=tri, hinge=hinge, n=len(x0) // 3,
                           corners=[corners[c] for c in (1, 2, 3, 4)]))
    for k in range(n_delaunay):
        d = scenes.delaunay_sheet(int(rng.integers(1500, 6001)), rng)
        Xd = d["X"].reshape(-1, 2)
        cs = [int(np.argmin((Xd[:, 0] - cx) ** 2 + (Xd[:, 1] - cy) ** 2))
              for cx, cy in ((0, 0), (0, 1), (1, 1), (1, 0))]
        sheets.append(dict(x=d["x"], X=d["X"], tri=d["tri"], hinge=d["hinge"], n=d["n"],
                           corners=cs))
    ctx = eolc.Context(device)
    off = ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in sheets])
    xall = np.concatenate([s["x"] for s in sheets])
    Xall = np.concatenate([s["X"] for s in sheets])
    made, runs = 0, 0
    while made < n_systems:
        runs += 1
        if runs > 50 * max(1, n_systems // steps_per_run + 1):
            raise RuntimeError("the simulator keeps failing; no training systems")
        mats, fixed = [], []
        for k, s in enumerate(sheets):
            n_eff = rng.uniform(64, 256)
            side = np.sqrt(s["n"])
            mats.append(eolc.Material(density=0.1 * (side / n_eff) ** 2, e=rng.uniform(20, 100),
                                      nu=0.3, beta=1e-5, damping=(0.0, 1.0)))
            pins = list(rng.choice(s["corners"], size=rng.integers(1, 5), replace=False))
            fixed += [3 * (off[k] + p) + c for p in pins for c in range(3)]
        ctx.set_instance_materials(mats)
        fixed = np.array(sorted(set(fixed)), np.int32)
        wind = np.array([rng.normal(0, 3.0), rng.normal(0, 3.0), 0.0])
        ctx.state_upload(xall, Xall, np.zeros_like(xall))
        opts = eolc.SolveOpts(precision=eolc.PREC_MIXED, precond=eolc.PC_JACOBI)
        for step in range(steps_per_run):
            try:
                ctx.step_batched(1, GRAV + wind, H, fixed, np.zeros(len(fixed)), opts)
            except eolc.EolcError:
                break  # an indefinite MDK ends this run; its systems so far are kept
            _, v = ctx.state_download()
            lpc.add_system(ctx, fixed, make_probes(rng, Xall, v, probes))
            made += 1
            if made >= n_systems:
                break
    return ctx


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4,
                    help="cosine decay of the learning rate from --lr to this over the epochs "
                         "(one eolc_lpc_train call per epoch, Adam state carried); 0: "
                         "constant --lr in one call")
    ap.add_argument("--quads", type=int, default=64)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--probes", default="white", choices=["white", "smooth"])
    ap.add_argument("--meshes", default="mixed", choices=["grid", "mixed"],
                    help="grid: one quads x quads sheet; mixed: a batch of a grid and "
                         "irregular Delaunay sheets")
    ap.add_argument("--big", type=int, default=256,
                    help="mixed: also a big x big grid sheet in the batch (0: none)")
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "lpc.npy"))
    args = ap.parse_args()
    lpc = eolc.LearnedPC(0, seed=args.seed)
    t0 = time.time()
    if args.meshes == "mixed":
        generate_mixed(lpc, args.systems, seed=args.seed, big=args.big, probes=args.probes)
    else:
        generate(lpc, args.systems, quads=args.quads, seed=args.seed, probes=args.probes)
    t1 = time.time()
    if not args.lr_final:
        losses = lpc.train(args.epochs, lr=args.lr, seed=args.seed)
    else:
        losses = []
        for e in range(args.epochs):
            w = 0.5 * (1 + np.cos(np.pi * e / max(1, args.epochs - 1)))
            lr = args.lr_final + (args.lr - args.lr_final) * w
            losses.append(lpc.train(1, lr=lr, seed=args.seed * 1000 + e)[0])
            print("epoch %d lr %.2e loss %.4f" % (e, lr, losses[-1]), flush=True)
    t2 = time.time()
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    np.save(args.out, lpc.get_params())
    print("generated %d systems in %.1fs, trained %d epochs in %.1fs, loss %s"
          % (args.systems, t1 - t0, args.epochs, t2 - t1,
             " ".join("%.4f" % l for l in losses)), flush=True)


if __name__ == "__main__":
    main()
