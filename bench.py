"""Steps/s of the EOL-Cloth hot path on a 256x256-quad sheet (GB300).

Workload (the headline configuration): a 1 m square sheet of 256 x 256
two-triangle quads (66,049 nodes, 131,072 triangles, 196,096 bending hinges,
198,147 DOF, 852,481 3x3 blocks), corners 3 and 4 pinned, gravity -9.8,
h = 5e-3, density 0.1, E = 50, nu = 0.3, bending 1e-5.  One step = the
reference's Cloth::step for this scene: BSR assembly of M/MDK and f,
pinned-corner rows, b = -(M v + h f), the velocity solve to an FP64 relative
residual of 1e-8, and x += h v.  Steps continue one trajectory from rest.

Arms:
  (default)          this library, one GPU per rank (the sheet does not
                     shard: N > 1 runs independent replicas, scaling "weak").
                     Every solver arm (resident Jacobi, streamed Jacobi, the
                     patch preconditioner, the learned preconditioner) is
                     timed on the same steps; `value` is the fastest arm and
                     config.arms has each.
  --impl reference   the reference's algorithm on the host cores: the CPU
                     oracle (reference element math restated, triplet
                     assembly, Eigen-style Jacobi CG in FP64), single thread
                     as the reference is; each step is one full step.

Timing: W warm-up steps, then K steps each bracketed by CUDA events on the
library's stream, with L2 flushed (a 256 MiB write) before every step and
outside the timed interval; max over ranks.  Every arm starts from the same
post-warm-up state after one untimed step of its own from that state, and
its first timed step re-evaluates the learned network and updates the
coarse inverse (the refresh counts restart), so no arm inherits another's
solver state.  `e2e` runs the same steps
through the host-buffer call eolc_step (H2D of x, X, v and D2H of x, v inside
the timed region).  The roofline entry is for the fastest arm's solver
kernel, which dominates the step: its algorithmic HBM bytes per launch (the
matrix read once, FP64 right-hand side in and solution out) over the
launch's CUDA-event time, its ncu DRAM traffic, its microseconds per
iteration beside the resident Jacobi iteration (the one-reduction floor), and
the bytes an HBM-streamed implementation of the same method would move.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in ("eol-cloth_gb300", "tests"):
    sys.path.insert(0, os.path.join(ROOT, sub))

METRIC = "steps/s @256^2 sheet: learned-PCG vs Jacobi-PCG on same GPU, rel-res 1e-8"
QUADS = 256


def scene(quads):
    import numpy as np
    import eolc
    r = quads + 1
    x, X, tri = eolc.sheet_mesh(r, r)
    hinge = eolc.mesh_hinges(tri)
    ids = eolc.corner_ids(r, r)
    fixed = np.array([3 * ids[k] + c for k in (3, 4) for c in range(3)], np.int32)
    return dict(x=x, X=X, tri=tri, hinge=hinge, fixed=fixed, fixed_vel=np.zeros(len(fixed)),
                n=r * r)


MAT = dict(density=0.1, e=50.0, nu=0.3, beta=1e-5, damping=(0.0, 1.0))
GRAV = [0.0, 0.0, -9.8]
H = 5e-3


def algorithmic_bytes_per_iter(n_nodes, n_blocks):
    """One Jacobi-PCG iteration: SpMV (FP32 block values + int32 column
    index per block + row pointers + input and output 3-vectors) plus 14
    passes over FP32 3-vectors."""
    spmv = n_blocks * (36 + 4) + (n_nodes + 1) * 4 + 2 * n_nodes * 12
    return spmv + 14 * n_nodes * 12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index),
                                      "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout
                vals = [v.strip() for v in out.strip().split(",")]
                if len(vals) == 7:
                    self.samples.append(vals)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons}


def cpu_step_seconds(sc, x, v, max_seconds=40.0):
    """One oracle step (assembly + Jacobi CG to 1e-8 + update) on this state."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # the CPU baseline leg: the oracle is the thing timed here
    mat = O.material(**MAT)
    t0 = time.perf_counter()
    F = O.Forces(x, sc["X"], sc["tri"], sc["hinge"], mat, GRAV, H)
    b = F.rhs(v, H)
    beq = (1 - 0.01) * v[sc["fixed"]] + sc["fixed_vel"]
    vn, it, rr = F.solve(b, sc["fixed"], beq, tol=1e-8)
    _ = x + H * vn
    return time.perf_counter() - t0, it


def batch_cpu_baseline(B, x, v, n_sample=16):
    """The oracle's step (triplet assembly + FP64 Jacobi CG to 1e-8) on
    n_sample instances spanning the batch's size range (evenly spaced ranks
    by node count), from the batch's state, one thread; the whole batch's
    time is estimated as the sample's time x (all nodes / sampled nodes)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # the CPU baseline leg: the oracle is the thing timed here
    sizes = np.array([s["n"] for s in B["sheets"]])
    order = np.argsort(sizes, kind="stable")
    picks = sorted(set(int(order[k]) for k in
                       np.linspace(0, len(order) - 1, n_sample).round().astype(int)))
    off = B["node_off"]
    secs, nodes = 0.0, 0
    for k in picks:
        s, m = B["sheets"][k], B["mats"][k]
        xk = x[3 * off[k]:3 * off[k + 1]].copy()
        vk = v[3 * off[k]:3 * off[k + 1]].copy()
        t0 = time.perf_counter()
        O.step(xk, s["X"], vk, s["tri"], s["hinge"], O.material(**m), GRAV, H, s["fixed"],
               s["fixed_vel"], tol=1e-8)
        secs += time.perf_counter() - t0
        nodes += s["n"]
    est = secs * float(sizes.sum()) / nodes
    return {"value": len(B["sheets"]) / est, "unit": "sheet-steps/s", "cores": 1, "kind": "port",
            "sample": "oracle steps of %d of the %d instances (evenly spaced by size) from the "
                      "post-warm-up state, %.1f s; the batch's time scaled by node count"
                      % (len(picks), len(B["sheets"]), secs)}


def run_batched(args, local_rank, stream, flush):
    """Batched workload: 256 independent sheets, side ~ U{16..96} quads, E ~
    U(20, 100) (seeded), corners 3 and 4 pinned, all stepped by one graph
    launch per step (one persistent batched-PCG launch inside), FP32 Jacobi
    PCG with FP64 dots and refinement to rel-res 1e-8."""
    import numpy as np
    import torch
    import eolc
    import scenes
    t0 = time.perf_counter()
    B = scenes.batch(args.batch_sheets, lo=16, hi=96, seed=3)
    ctx = eolc.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in B["sheets"]])
    ctx.set_instance_materials([eolc.Material(**m) for m in B["mats"]])
    ctx.state_upload(B["x"], B["X"], B["v"])
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=eolc.PC_JACOBI)
    setup_s = time.perf_counter() - t0
    chosen, ms = ctx.batch_autotune(GRAV, H, B["fixed"], B["fixed_vel"], opts)
    ctx.step_batched(args.warmup, GRAV, H, B["fixed"], B["fixed_vel"], opts)
    step_ms, iters, worst = [], 0, 0.0
    launches0 = ctx.launch_count()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        tot, _ = ctx.step_batched(1, GRAV, H, B["fixed"], B["fixed_vel"], opts)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        iters += tot.iterations
        worst = max(worst, tot.max_rel_res)
    launches = ctx.launch_count() - launches0
    total = sum(step_ms)
    n_nodes = int(B["node_off"][-1])
    x_w, v_w = ctx.state_download()
    cpu = optional_line(lambda: batch_cpu_baseline(B, x_w, v_w))
    return {
        "workload": "%d sheets, side U{16..96} quads (seed 3), E U(20,100), %d nodes total,"
                    " 2 corners pinned each" % (args.batch_sheets, n_nodes),
        "sheet_steps_per_s": args.batch_sheets * args.steps / (total / 1e3),
        "batch_steps_per_s": args.steps / (total / 1e3),
        "ms_per_batch_step": total / args.steps,
        "mean_pcg_iters_per_sheet": iters / (args.steps * args.batch_sheets),
        "max_rel_res": worst,
        "autotuned_config": eolc.batch_config_name(chosen),
        "autotune_ms": {eolc.batch_config_name(c): (None if t < 0 else round(float(t), 3))
                        for c, t in enumerate(ms)},
        "gpu_launches_per_step": launches / args.steps,
        "host_setup_s": setup_s,
        "l2": "flushed (256 MiB write) before each step",
        "cpu_baseline": cpu,
    }


def run_delaunay(args, local_rank, stream, flush):
    """Irregular batched workload: 64 Delaunay sheets of U(5k, 50k) triangles
    (seeded; density gradient along x, mimicking remeshed output), top
    corners pinned.  Jacobi-PCG and learned-PCG (per-instance Jacobi fallback
    at 2x the instance's last Jacobi count) each time K batched steps from
    the same state after W Jacobi warm-up steps."""
    import numpy as np
    import torch
    import eolc
    import scenes
    t0 = time.perf_counter()
    B = scenes.delaunay_batch(args.delaunay_meshes, tri_lo=5000, tri_hi=50000, seed=5)
    ctx = eolc.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in B["sheets"]])
    ctx.set_instance_materials([eolc.Material(**m) for m in B["mats"]])
    lpc = eolc.LearnedPC(local_rank)
    lpc.set_params(np.load(os.path.join(ROOT, "eol-cloth_gb300", "weights", "lpc.npy")))
    lpc.attach(ctx)
    ctx.state_upload(B["x"], B["X"], B["v"])
    setup_s = time.perf_counter() - t0
    jac = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=eolc.PC_JACOBI)
    lrn = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=eolc.PC_LEARNED,
                         fallback_factor=2)
    chosen, _ = ctx.batch_autotune(GRAV, H, B["fixed"], B["fixed_vel"], jac)
    ctx.step_batched(args.warmup, GRAV, H, B["fixed"], B["fixed_vel"], jac)
    x_w, v_w = ctx.state_download()
    out = {}
    for name, opts in (("jacobi", jac), ("learned", lrn)):
        ctx.state_upload(x_w, B["X"], v_w)
        ctx.step_batched(1, GRAV, H, B["fixed"], B["fixed_vel"], jac)  # per-instance references
        ctx.state_upload(x_w, B["X"], v_w)
        step_ms, iters, fb, worst = [], 0, 0, 0.0
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            tot, _ = ctx.step_batched(1, GRAV, H, B["fixed"], B["fixed_vel"], opts)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            iters += tot.iterations
            fb += tot.n_fallback
            worst = max(worst, tot.max_rel_res)
        total = sum(step_ms)
        out[name] = {"sheet_steps_per_s": len(B["sheets"]) * args.steps / (total / 1e3),
                     "ms_per_batch_step": total / args.steps,
                     "mean_pcg_iters_per_sheet": iters / (args.steps * len(B["sheets"])),
                     "fallbacks": fb, "max_rel_res": worst}
    n_tri = sum(len(s["tri"]) for s in B["sheets"])
    cpu = optional_line(lambda: batch_cpu_baseline(B, x_w, v_w))
    return {"workload": "%d Delaunay sheets, U(5k, 50k) triangles (seed 5), %d triangles and %d "
                        "nodes in total, top corners pinned" % (len(B["sheets"]), n_tri,
                                                                 int(B["node_off"][-1])),
            "arms": out, "learned_vs_jacobi": out["learned"]["sheet_steps_per_s"] /
            out["jacobi"]["sheet_steps_per_s"],
            "autotuned_config": eolc.batch_config_name(chosen), "host_setup_s": setup_s,
            "l2": "flushed (256 MiB write) before each step", "cpu_baseline": cpu}


def run_reference(args, rank):
    import numpy as np
    if rank != 0:
        return
    sc = scene(QUADS)
    x, v = sc["x"].copy(), np.zeros(3 * sc["n"])
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    mat = O.material(**MAT)
    times, iters = [], []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        it, rr = O.step(x, sc["X"], v, sc["tri"], sc["hinge"], mat, GRAV, H, sc["fixed"],
                        sc["fixed_vel"], tol=1e-8)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            iters.append(it)
    total = sum(times)
    val = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "sheet 256x256 quads, 66049 nodes, 131072 tris, 2 corners pinned,"
                               " Jacobi CG to rel-res 1e-8, from rest",
                   "solver": "jacobi-cg", "mean_cg_iters": statistics.mean(iters)},
        "cpu_baseline": {"value": val, "unit": "steps/s", "cores": 1, "kind": "port",
                         "sample": "%d full steps after %d warm-up steps, one thread "
                                   "(the reference is single-threaded)" % (args.steps, args.warmup)},
        "e2e": {"value": val, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


ARM_KERNEL = {"jacobi": "jacobi_resident_kernel", "block": "jacobi_resident_kernel",
              "patch": "patch_resident_kernel", "patch-1l": "patch_resident_kernel",
              "patch-r4": "patch_resident_kernel",
              "learned": "learned_resident_kernel", "learned-1l": "learned_resident_kernel",
              "learned-r4": "learned_resident_kernel", "learned-r2": "learned_resident_kernel",
              "jacobi-streamed": "cg_kernel"}


def arm_opts(eolc, arm, degree):
    base = dict(rel_tol=1e-8, precision=eolc.PREC_MIXED)
    if arm == "jacobi":
        return eolc.SolveOpts(precond=eolc.PC_JACOBI, **base)
    if arm == "jacobi-streamed":
        return eolc.SolveOpts(precond=eolc.PC_JACOBI, streamed=1, **base)
    if arm == "block":
        return eolc.SolveOpts(precond=eolc.PC_BLOCK_JACOBI, **base)
    if arm == "patch":
        return eolc.SolveOpts(precond=eolc.PC_PATCH, degree=degree, **base)
    if arm == "patch-r4":
        return eolc.SolveOpts(precond=eolc.PC_PATCH, degree=degree, **base)
    if arm == "patch-1l":
        return eolc.SolveOpts(precond=eolc.PC_PATCH, degree=degree, no_coarse=1, **base)
    if arm in ("learned", "learned-r2", "learned-r4"):
        return eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=2, **base)
    if arm == "learned-1l":
        return eolc.SolveOpts(precond=eolc.PC_LEARNED, fallback_factor=2, no_coarse=1, **base)
    raise ValueError(arm)


def arm_refresh(arm):
    """(network, coarse) refresh intervals of an arm: learned-rK re-evaluates
    the network every K solves (eolc_set_learned_refresh; learned: every
    solve); learned-r4 updates the coarse inverse every 8 solves, the other
    learned arms and patch-r4 every 4 (eolc_set_coarse_refresh; one update
    costs ~0.3 ms on the 256^2 sheet), the other arms every solve."""
    net = {"learned-r4": 4, "learned-r2": 2}.get(arm, 1)
    if arm == "learned-r4":
        return net, 8
    coarse = 4 if arm.startswith("learned") or arm == "patch-r4" else 1
    return net, coarse


def max_over_ranks(value, world, dev):
    """Largest `value` over the ranks, returned on every rank: the job takes
    as long as its slowest replica.  `dev` holds the tensor the process
    group's backend reduces (the rank's GPU under NCCL, the CPU under gloo)."""
    if world == 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.item()


def job_rate(world, steps, total_ms):
    """Whole-job steps/s: each of `world` replicas runs `steps` steps and
    the job ends with the slowest one, `total_ms` after it started."""
    return world * steps / (total_ms / 1e3)


def shard_instances(sizes, world):
    """Deterministic node-count-balanced split of a batch's instances over
    `world` ranks (the batched configurations shard by instance, with no
    data-path exchange): instances in decreasing size, ties by index, each
    to the rank with the fewest nodes so far, ties to the lower rank.
    Returns every rank's instance indices, ascending."""
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    load, out = [0] * world, [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(k)
        load[r] += int(sizes[k])
    return [sorted(o) for o in out]


def sub_batch(B, idx):
    """The batch of instances idx (ascending) of batch B, in the layout of
    scenes.batch: per-instance scenes and materials, concatenated state and
    global fixed DOFs."""
    import numpy as np
    sheets = [B["sheets"][k] for k in idx]
    mats = [B["mats"][k] for k in idx]
    off = [0]
    for s in sheets:
        off.append(off[-1] + s["n"])
    bo = B["node_off"]
    x = np.concatenate([B["x"][3 * bo[k]:3 * bo[k + 1]] for k in idx])
    X = np.concatenate([B["X"][2 * bo[k]:2 * bo[k + 1]] for k in idx])
    v = np.concatenate([B["v"][3 * bo[k]:3 * bo[k + 1]] for k in idx])
    fixed = np.concatenate([s["fixed"] + 3 * o for s, o in zip(sheets, off[:-1])]).astype(np.int32)
    return dict(sheets=sheets, mats=mats, node_off=np.array(off), x=x, X=X, v=v, fixed=fixed,
                fixed_vel=np.zeros(len(fixed)))


def merge_shards(n_inst, parts):
    """Per-instance results of every rank, parts[r] = [(instance, value), ...],
    merged into instance order; every instance must come exactly once."""
    out = [None] * n_inst
    for part in parts:
        for k, val in part:
            if out[k] is not None:
                raise ValueError("instance %d stepped twice" % k)
            out[k] = val
    missing = [k for k in range(n_inst) if out[k] is None]
    if missing:
        raise ValueError("instances %s not stepped" % missing[:8])
    return out


def run_batched_sharded(args, rank, world, local_rank, stream, flush, dev):
    """Configuration 3 split over the ranks by instance (shard_instances):
    each rank steps its share in one batched launch per step; the job's
    sheet-steps/s is all instances x K over the slowest rank's time."""
    import numpy as np
    import torch
    import eolc
    import scenes
    B = scenes.batch(args.batch_sheets, lo=16, hi=96, seed=3)
    mine = shard_instances([s["n"] for s in B["sheets"]], world)[rank]
    S = sub_batch(B, mine)
    ctx = eolc.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology_batched([(s["n"], s["tri"], s["hinge"]) for s in S["sheets"]])
    ctx.set_instance_materials([eolc.Material(**m) for m in S["mats"]])
    ctx.state_upload(S["x"], S["X"], S["v"])
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=eolc.PC_JACOBI)
    ctx.step_batched(args.warmup, GRAV, H, S["fixed"], S["fixed_vel"], opts)
    torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        ctx.step_batched(1, GRAV, H, S["fixed"], S["fixed_vel"], opts)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    total = max_over_ranks(sum(step_ms), world, dev)
    return {"workload": "%d sheets, side U{16..96} quads (seed 3), split over %d ranks by "
                        "instance (node-count balanced), %d on this rank"
                        % (args.batch_sheets, world, len(mine)),
            "sheet_steps_per_s": args.batch_sheets * args.steps / (total / 1e3),
            "ms_per_batch_step": total / args.steps, "scaling": "strong",
            "note": "unmeasured on hardware until a multi-GPU run happens; no collective on "
                    "the data path (the timed-interval maximum only)"}


def time_arm(ctx, sc, mat, opts, x_w, v_w, steps, stream, flush, world, dev, refresh=(1, 1)):
    """K steps from the post-warm-up state, each bracketed by CUDA events on
    the library's stream with L2 flushed before it; max over ranks."""
    import torch
    ctx.set_learned_refresh(refresh[0])
    ctx.set_coarse_refresh(refresh[1])
    ctx.state_upload(x_w, sc["X"], v_w)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, kern_ms, iters, asm_ms, fallback = [], [], [], [], 0
    launches0 = ctx.launch_count()
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        info = ctx.step_resident(1, mat, GRAV, H, sc["fixed"], sc["fixed_vel"], opts)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        kern_ms.append(info.solve_kernel_ms)
        asm_ms.append(info.assemble_ms)
        iters.append(info.iterations)
        fallback += info.used_fallback
    torch.cuda.synchronize()
    total_ms = max_over_ranks(sum(step_ms), world, dev)
    ctx.set_learned_refresh(1)
    ctx.set_coarse_refresh(1)
    return {"steps_per_s": job_rate(world, steps, total_ms), "ms_per_step": total_ms / steps,
            "mean_pcg_iters": statistics.mean(iters), "pcg_kernel_ms": statistics.mean(kern_ms),
            "assemble_ms": statistics.mean(asm_ms), "fallbacks": fallback,
            "launches": ctx.launch_count() - launches0}


def run_export(ctx, sc, x, stream, frames=10):
    """OBJ frame export of the current state (the two files of
    Cloth::exportBrender): device text generation into host memory and into
    files, against the oracle's sprintf text of the same frame."""
    import tempfile
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # CPU side only: the text the frame must equal
    ctx.state_upload(x, sc["X"], np.zeros_like(x))
    a, b = ctx.export_obj_text(1, H)  # warm-up (buffers)
    t0 = time.perf_counter()
    ra, rb = O.obj_text(x, sc["X"], sc["tri"], frame=1, time=H)
    cpu_s = time.perf_counter() - t0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    text_ms, dev_ms = [], []
    for k in range(frames):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev0.record(stream)
        ctx.export_obj_text(k, k * H)
        ev1.record(stream)
        text_ms.append(1e3 * (time.perf_counter() - t0))
        ev1.synchronize()
        dev_ms.append(ev0.elapsed_time(ev1))
    file_ms = []
    with tempfile.TemporaryDirectory() as d:
        for k in range(frames):
            t0 = time.perf_counter()
            ctx.export_obj(d, k, k * H)
            file_ms.append(1e3 * (time.perf_counter() - t0))
    nbytes = len(a) + len(b)
    med = lambda v: float(np.median(v))
    return {"workload": "2 OBJ files (Cloth2D, Cloth3D) of the 256x256-quad sheet state, "
                        "%d bytes per frame" % nbytes,
            "byte_identical_to_oracle": (a, b) == (ra, rb),
            "frames_per_s_text": 1e3 / med(text_ms), "ms_per_frame_text": med(text_ms),
            "ms_per_frame_device": med(dev_ms), "text_gb_s": nbytes / med(text_ms) / 1e6,
            "ms_per_frame_files": med(file_ms),
            "gpu_launches_per_frame": 4,
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "frames/s", "cores": 1,
                             "kind": "port", "sample": "one frame's text by the oracle "
                                                       "(the reference's sprintf formats)"},
            "note": "text: device formatting + one device-to-host copy into pinned memory + "
                    "copy into the caller's buffer; device: the same on the stream's clock "
                    "(one host round trip for the text size inside); files: text + two "
                    "fwrite calls to a temporary directory"}


def axis_box(eolc, center, dim):
    """Axis-aligned box obstacle (eolc.Box): frame = translation to center,
    stored column-major as the reference's Eigen::Matrix4d."""
    import numpy as np
    E1 = np.eye(4)
    E1[:3, 3] = center
    return eolc.Box(dim, E1.flatten(order="F"))


def run_contacts(args, local_rank, stream, flush, steps=5):
    """Cloth::step with the contact QP (eolc_step_contacts) on the 256x256-quad
    sheet draped over a box (10.6k CD2 contacts), against the plain step on the
    same state; and the QP solve alone on a 24x24-quad drape against the
    oracle's exact active-set QP (the reference's Mosek / Gurobi are not
    available)."""
    import numpy as np
    import torch
    import eolc
    import scenes as S
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # CPU side only: the oracle's CD2 row count and QP below
    import qp_ref
    x0, X, tri, center, snaps = S.drape_positions(QUADS, 40)
    n = len(x0) // 3
    hinge = eolc.mesh_hinges(tri)
    ebox = axis_box(eolc, center, (0.4, 0.4, 0.2))
    box = O.axis_box(center, (0.4, 0.4, 0.2))  # the same box for the oracle's CD2
    ids = eolc.corner_ids(QUADS + 1, QUADS + 1)
    fixed = np.array([3 * ids[k] + c for k in (3, 4) for c in range(3)], np.int32)
    fvel = np.zeros(len(fixed))
    ctx = eolc.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology(n, tri, hinge)
    mat = eolc.Material(**MAT)
    rng = np.random.default_rng(4)
    xs = snaps[14].copy()
    vs = rng.normal(0, 0.02, 3 * n)
    vs[2::3] -= 0.4
    opts = arm_opts(eolc, "patch", args.degree)
    xh = torch.empty(3 * n, dtype=torch.float64).pin_memory().numpy()
    vh = torch.empty(3 * n, dtype=torch.float64).pin_memory().numpy()
    Xh = torch.empty(2 * n, dtype=torch.float64).pin_memory().numpy()
    Xh[:] = X
    out = {}
    for label, contact in (("plain", False), ("contacts", True)):
        ms, infos = [], []
        for k in range(steps + 1):
            xh[:] = xs
            vh[:] = vs
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if contact:
                ctx.clear_contact_multipliers()  # a cold QP every time
                infos.append(ctx.step_contacts(xh, Xh, vh, mat, GRAV, H, fixed, fvel,
                                               boxes=[ebox], threshold=1e-3, opts=opts))
            else:
                infos.append(ctx.step(xh, Xh, vh, mat, GRAV, H, fixed, fvel, opts))
            if k:  # the first call builds plans
                ms.append(1e3 * (time.perf_counter() - t0))
        info = infos[-1]
        out[label] = {"ms_per_step": float(np.median(ms)), "steps_per_s": 1e3 / float(np.median(ms)),
                      "pcg_iterations": info.iterations,
                      "pcg_kernel_ms": round(info.solve_kernel_ms, 4)}
        if contact:
            out[label].update({"qp_solves": info.solves, "multiplier_updates": info.outer,
                               "active_rows": info.n_active,
                               "max_violation": info.max_violation})
    cons = O.cd2(xs, tri, [box], threshold=1e-3)
    out["rows"] = len(qp_ref.contact_rows(cons, n)[1])
    # the same step again on the same context: its QP starts from the
    # multipliers of the first call (what a persisting contact carries from
    # step to step); consecutive steps of this drape are not usable: it is
    # placed kinematically, and after one step its MDK is indefinite (every
    # solver, contacts or not, reports a breakdown)
    warm = []
    for k in range(steps + 1):
        xh[:] = xs
        vh[:] = vs
        if k == 0:
            ctx.clear_contact_multipliers()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        info = ctx.step_contacts(xh, Xh, vh, mat, GRAV, H, fixed, fvel, boxes=[ebox],
                                 threshold=1e-3, opts=opts)
        if k:
            warm.append((1e3 * (time.perf_counter() - t0), info.solves, info.iterations))
    out["carried_multipliers"] = {
        "ms_per_step": round(float(np.median([w[0] for w in warm])), 3),
        "qp_solves": warm[-1][1], "pcg_iterations": warm[-1][2],
        "note": "the same step repeated, the QP starting from the previous call's multipliers"}
    # like for like on a small drape: the QP solve alone, GPU vs the oracle
    q = 24
    x0s, Xs, tris, cs, snapss = S.drape_positions(q, 40)
    ns = len(x0s) // 3
    hs = eolc.mesh_hinges(tris)
    bs = O.axis_box(cs, (0.4, 0.4, 0.2))
    xq = snapss[9]
    F = O.Forces(xq, Xs, tris, hs, O.material(), GRAV, H)
    vq = rng.normal(0, 0.02, 3 * ns)
    vq[2::3] -= 0.4
    bq = F.rhs(vq, H)
    ids = eolc.corner_ids(q + 1, q + 1)
    fq = np.array([3 * ids[k] + c for k in (3, 4) for c in range(3)], np.int32)
    beq = 0.99 * vq[fq]
    C, d = qp_ref.contact_rows(O.cd2(xq, tris, [bs], threshold=1e-3), ns)
    t0 = time.perf_counter()
    vo, lo, _ = qp_ref.solve_qp(F.csr(1), bq, fq, beq, C, d)
    cpu_s = time.perf_counter() - t0
    c2 = eolc.Context(local_rank)
    c2.set_topology(ns, tris, hs)
    c2.forces_fill(xq, Xs, mat, GRAV, H, eolc.PREC_FP64)
    o64 = eolc.SolveOpts(rel_tol=1e-10, precision=eolc.PREC_FP64)
    c2.velocity_solve_ineq(bq, fq, beq, C, d, o64)
    ts = []
    for k in range(5):
        t0 = time.perf_counter()
        vg, lg, ig = c2.velocity_solve_ineq(bq, fq, beq, C, d, o64)
        ts.append(time.perf_counter() - t0)
    out["small_qp"] = {"workload": "24x24-quad drape, %d contact rows, FP64" % C.shape[0],
                       "gpu_ms": 1e3 * float(np.median(ts)), "solves": ig.solves,
                       "v_rel_err_vs_oracle": float(np.abs(vg - vo).max() / np.abs(vo).max()),
                       "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "QP solves/s", "cores": 1,
                                        "kind": "port",
                                        "sample": "the oracle's exact active-set QP (scipy "
                                                  "sparse LU per working-set change) on the "
                                                  "same problem"}}
    out["workload"] = ("256x256-quad sheet draped over a 0.4 x 0.4 box (snapshot 14 of the "
                       "seeded drape), 2 corners pinned, patch-PCG, rel-res 1e-8, host buffers")
    out["trajectory"] = optional_line(lambda: contact_trajectory(args, local_rank, stream))
    return out


def contact_trajectory(args, local_rank, stream, quads=128, steps=80):
    """Consecutive Cloth::steps with contacts: the configuration-2 sheet
    (128x128 quads, positions jittered N(0, 1e-4) from seed 2) dropped flat,
    unpinned, onto the 0.4 x 0.4 x 0.2 box whose top face starts 0.05 m
    below it; every step runs CD2 and the contact QP (eolc_step_contacts,
    multipliers carried from step to step)."""
    import numpy as np
    import torch
    import eolc
    r = quads + 1
    x0, X, tri = eolc.sheet_mesh(r, r)
    n = len(x0) // 3
    hinge = eolc.mesh_hinges(tri)
    x = x0 + np.random.default_rng(2).normal(0.0, 1e-4, x0.size)
    v = np.zeros(3 * n)
    box = axis_box(eolc, [0.5, 0.5, -0.05 - 0.1], (0.4, 0.4, 0.2))
    ctx = eolc.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology(n, tri, hinge)
    mat = eolc.Material(**MAT)
    opts = arm_opts(eolc, "patch", args.degree)
    none = np.zeros(0, np.int32)
    ms, rows, solves, status = [], [], [], "ok"
    for k in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            info = ctx.step_contacts(x, X, v, mat, GRAV, H, none, np.zeros(0), boxes=[box],
                                     threshold=1e-3, opts=opts)
        except Exception as e:  # an indefinite MDK ends the trajectory
            status = "stopped at step %d: %s" % (k, str(e)[:120])
            break
        ms.append(1e3 * (time.perf_counter() - t0))
        rows.append(int(info.n_active))
        solves.append(int(info.solves))
    touch = [k for k, m in enumerate(rows) if m > 0]
    return {"workload": "128x128-quad sheet (16,641 nodes) dropped flat, unpinned, onto the "
                        "0.4 x 0.4 x 0.2 box 0.05 m below; patch-PCG, rel-res 1e-8, host buffers",
            "steps_done": len(ms), "status": status,
            "first_contact_step": touch[0] if touch else None,
            "ms_per_step_free": float(np.median(ms[:touch[0]])) if touch and touch[0] > 0 else None,
            "ms_per_step_contact": float(np.median([ms[k] for k in touch])) if touch else None,
            "max_active_rows": max(rows) if rows else 0,
            "mean_qp_solves_in_contact": float(np.mean([solves[k] for k in touch])) if touch else None}


def run_cd2(args, local_rank, stream, steps=200, cpu_sample=40):
    """CD2 at configuration 2's size: a 128x128-quad sheet (16,641 nodes,
    32,768 triangles) over a 0.4 x 0.4 x 0.2 m box 0.05 m below it, threshold
    1e-3, positions of the seeded 200-step drape (jitter N(0, 1e-4)).  Every
    step is one eolc_cd2 call with host positions in and host contacts out
    (wall clock) and the same call's span on the stream (CUDA events); the
    contact sets of the timed calls are compared with the oracle's bytes.
    CPU baseline: the oracle's CD2 on every fifth step, one thread."""
    import ctypes
    import numpy as np
    import torch
    import eolc
    import scenes as S
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # CPU side only: the contact bytes to match and the baseline
    x0, X, tri, center, snaps = S.drape_positions(128, steps, seed=2024)
    n = len(x0) // 3
    ctx = eolc.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology(n, tri, eolc.mesh_hinges(tri))
    ob = O.axis_box(center, (0.4, 0.4, 0.2))  # the oracle's box (parity check below)
    gb = axis_box(eolc, center, (0.4, 0.4, 0.2))
    ctx.cd2(snaps[0], boxes=[gb], threshold=1e-3)  # edge list and perturbation built
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    wall, dev, raw, launches0 = [], [], [], ctx.launch_count()
    for x in snaps:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev0.record(stream)
        raw.append(ctx.cd2(x, boxes=[gb], threshold=1e-3, raw=True))
        ev1.record(stream)
        wall.append(1e3 * (time.perf_counter() - t0))
        ev1.synchronize()
        dev.append(ev0.elapsed_time(ev1))
    launches = (ctx.launch_count() - launches0) / steps
    size = ctypes.sizeof(eolc.Contact)
    contacts = [len(r) // size for r in raw]
    exact = all(raw[k] == O.cd2(snaps[k], tri, boxes=[ob], threshold=1e-3, raw=True)
                for k in range(0, steps, 10))
    picks = list(range(0, steps, steps // cpu_sample))[:cpu_sample]
    t0 = time.perf_counter()
    for k in picks:
        O.cd2(snaps[k], tri, boxes=[ob], threshold=1e-3)
    cpu_s = (time.perf_counter() - t0) / len(picks)
    med = lambda v: float(np.median(v))
    return {"workload": "CD2, 128x128-quad sheet (16641 nodes, 32768 tris, 49408 edges) over a "
                        "0.4x0.4x0.2 box, threshold 1e-3, 200 drape steps, jitter N(0,1e-4)",
            "ms_per_call": med(wall), "calls_per_s": 1e3 / med(wall),
            "ms_per_call_stream": med(dev), "mean_contacts": float(np.mean(contacts)),
            "max_contacts": int(max(contacts)), "gpu_launches_per_call": launches,
            "bit_exact_vs_oracle": exact,
            "bit_exact_checked": "every 10th of the timed calls (the full 200-step check is "
                                 "tests/test_gpu_c2.py)",
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "calls/s", "cores": 1, "kind": "port",
                             "sample": "the oracle's CD2 on %d of the 200 steps (every %dth)"
                                       % (len(picks), steps // cpu_sample)},
            "note": "ms_per_call: host positions in, host contacts out, through the C ABI "
                    "(eolc_cd2); ms_per_call_stream: the same call on the stream's clock"}


def run_refresh(args, local_rank, stream, sc, reps=3):
    """Topology refresh on the 256x256-quad sheet, as after a remesh: the
    device build (eolc_set_topology), the first step after it (which builds
    the solver's resident plan on the host) and a steady step."""
    import numpy as np
    import torch
    import eolc
    mat = eolc.Material(**MAT)
    out = {}
    for arm in ("patch", "jacobi-streamed"):
        ctx = eolc.Context(local_rank)
        ctx.set_stream(stream.cuda_stream)
        opts = arm_opts(eolc, arm, args.degree)
        topo, first, steady = [], [], []
        for k in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.set_topology(sc["n"], sc["tri"], sc["hinge"])
            t1 = time.perf_counter()
            ctx.state_upload(sc["x"], sc["X"], np.zeros(3 * sc["n"]))
            t2 = time.perf_counter()
            ctx.step_resident(1, mat, GRAV, H, sc["fixed"], sc["fixed_vel"], opts)
            t3 = time.perf_counter()
            # the same step again from the same state, plans reused (the
            # upload is outside both intervals)
            ctx.state_upload(sc["x"], sc["X"], np.zeros(3 * sc["n"]))
            t3b = time.perf_counter()
            ctx.step_resident(1, mat, GRAV, H, sc["fixed"], sc["fixed_vel"], opts)
            t4 = time.perf_counter()
            topo.append(t1 - t0)
            first.append(t3 - t2)
            steady.append(t4 - t3b)
        med = lambda v: round(1e3 * float(np.median(v)), 3)
        out[arm] = {"set_topology_ms": med(topo), "first_step_ms": med(first),
                    "steady_step_ms": med(steady),
                    "plan_ms": round(med(first) - med(steady), 3)}
    out["note"] = ("set_topology: BSR pattern, contribution lists and node-face lists built "
                   "on the GPU (the former host build took 536 ms); plan_ms: the solver's "
                   "per-topology plan (patch partition and shared-memory image layout on "
                   "host threads, or the streamed tiling), built at the first step")
    return out


def run_eol(args, local_rank, stream, sc, reps=5):
    """Forces::fill with EOL nodes (eolc_set_topology_eol): the 256x256-quad
    sheet with its middle row of nodes (257) as EOL nodes, FP64, host
    arrays in and out, against the same fill without EOL nodes and the
    oracle's EOL fill on one core."""
    import numpy as np
    import torch
    import eolc
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # CPU side only: the baseline below
    r = QUADS + 1
    eol = (r // 2) * r + np.arange(r)  # node k = i r + j; the row i = r // 2
    rng = np.random.default_rng(8)
    x = sc["x"] + rng.normal(0, 1e-3, sc["x"].size)
    mat = eolc.Material(**MAT)
    out = {"workload": "256x256-quad sheet, %d EOL nodes (one row), FP64 f, M and MDK "
                       "(host arrays)" % len(eol)}
    for label in ("plain", "eol"):
        ctx = eolc.Context(local_rank)
        ctx.set_stream(stream.cuda_stream)
        if label == "eol":
            ctx.set_topology_eol(sc["n"], sc["tri"], sc["hinge"], eol)
        else:
            ctx.set_topology(sc["n"], sc["tri"], sc["hinge"])
        ctx.forces_fill(x, sc["X"], mat, GRAV, H, eolc.PREC_FP64)
        ts = []
        for k in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.forces_fill(x, sc["X"], mat, GRAV, H, eolc.PREC_FP64)
            ts.append(time.perf_counter() - t0)
        out[label + "_ms"] = round(1e3 * float(np.median(ts)), 3)
        out[label + "_blocks"] = len(ctx.bsr_pattern()[1])
    t0 = time.perf_counter()
    O.ForcesEOL(x, sc["X"], sc["tri"], sc["hinge"], O.material(), GRAV, H, eol)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "fills/s", "cores": 1, "kind": "port",
                           "sample": "one oracle Forces::fill with the same EOL nodes"}
    out["note"] = ("wall time of eolc_forces_fill including the upload of x, X and the "
                   "download of f, M and MDK")
    return out


def run_eol_step(args, local_rank, stream, steps=8, cpu_quads=16, cpu_steps=3):
    """Cloth::step of an EOL mesh: a sheet lying on a box whose edge runs
    under its middle column of nodes (the EOL nodes, on box edge 10), the
    hanging half pulling material over the edge through the Eulerian DOFs.
    Each step is CD2 (eolc_cd2), the rows of Constraints::fill
    (eolc_constraint_rows) and eolc_step_eol (forces with the EOL branches,
    the QP with the EOL equality and inequality rows and the contact rows,
    x += h v, u += h vE; patch PCG inside the QP), host arrays in and out,
    wall clock.  Sheets of 16 and 128 quads per side; CPU baseline: the oracle's step (its restated
    rows, EOL fill and exact active-set QP) on the 16-quad sheet."""
    import numpy as np
    import torch
    import eolc
    import scenes as S
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # CPU side only: the baseline below
    import eol_ref
    mat = eolc.Material(**MAT)
    opts = arm_opts(eolc, "patch", args.degree)
    out = {}
    for q in (cpu_quads, 128):
        sc = S.eol_edge_sheet(q)
        n, ne = sc["n"], len(sc["eol"])
        ctx = eolc.Context(local_rank)
        ctx.set_stream(stream.cuda_stream)
        ctx.set_topology_eol(n, sc["tri"], sc["hinge"], sc["eol"])
        box = axis_box(eolc, sc["box_center"], sc["box_dim"])
        x, u, v = sc["x"].copy(), sc["X"].copy(), np.zeros(3 * (n + ne))
        ts, rows, solves, active = [], [], [], []
        for k in range(steps + 2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            contacts = ctx.cd2(x, [box], threshold=1e-3, array=True)
            E, I = eolc.constraint_rows(x, u, sc["tri"], sc["edges"], sc["eol"], sc["corner"],
                                        sc["cd"], sc["preserve"], [box], None, contacts)
            info = ctx.step_eol(x, u, v, mat, GRAV, H, sc["fixed"], sc["fixed_vel"], E, I, opts)
            if k >= 2:  # the first two steps build the plans and the contact set grows
                ts.append(time.perf_counter() - t0)
                rows.append(E.m + I.m)
                solves.append(info.solves)
                active.append(info.n_active)
        out["sheet_%d" % q] = {"nodes": n, "eol_nodes": ne, "ms_per_step": round(
            1e3 * float(np.median(ts)), 3), "steps_per_s": 1.0 / float(np.median(ts)),
            "rows": int(np.median(rows)), "active_contacts": int(np.median(active)),
            "linear_solves": float(np.mean(solves)),
            "material_flow": float(np.abs(u - sc["X"]).max())}
    sc = S.eol_edge_sheet(cpu_quads)
    ob = O.axis_box(sc["box_center"], sc["box_dim"])
    n, ne = sc["n"], len(sc["eol"])
    x, u, v = sc["x"].copy(), sc["X"].copy(), np.zeros(3 * n + 2 * ne)
    cpu = []
    for k in range(cpu_steps):
        t0 = time.perf_counter()
        c = O.cd2(x, sc["tri"], [ob], threshold=1e-3)
        r = eol_ref.constraint_rows(x, u, sc["tri"], sc["edges"], sc["eol"], sc["corner"],
                                    sc["cd"], sc["preserve"], [ob], None, c)
        eol_ref.step(x, u, v, sc["tri"], sc["hinge"], sc["eol"], O.material(), GRAV, H,
                     sc["fixed"], sc["fixed_vel"], r)
        if k >= 1:
            cpu.append(time.perf_counter() - t0)
    out["workload"] = ("EOL sheet on a box edge (middle node column = EOL nodes), CD2 + "
                       "Constraints::fill rows + Cloth::step with the QP, mixed precision, "
                       "patch PCG inside the QP")
    out["cpu_baseline"] = {"value": 1.0 / float(np.median(cpu)), "unit": "steps/s", "cores": 1,
                           "kind": "port",
                           "sample": "oracle EOL steps 2-%d of the %d-quad sheet (exact "
                                     "active-set QP, scipy sparse LU)" % (cpu_steps, cpu_quads)}
    out["note"] = ("steps 3 onward of each trajectory (the first two build the plans and the "
                   "top half's contact set); host arrays in and out through the C ABI")
    return out


def optional_line(fn):
    """A secondary line of the JSON output: its result, or the error that
    stopped it (the headline line is printed either way)."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    import eolc
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    sc = scene(QUADS)
    ctx = eolc.Context(local_rank)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_topology(sc["n"], sc["tri"], sc["hinge"])
    mat = eolc.Material(**MAT)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2
    n_blocks = len(ctx.bsr_pattern()[1])
    lpc = None
    weights = os.path.join(ROOT, "eol-cloth_gb300", "weights", "lpc.npy")
    arms = args.precond.split(",") if args.precond != "all" else \
        ["jacobi", "jacobi-streamed", "patch", "patch-r4", "patch-1l", "learned", "learned-r2",
         "learned-r4", "learned-1l"]
    if any(a.startswith("learned") for a in arms):
        if os.path.exists(weights):
            lpc = eolc.LearnedPC(local_rank)
            lpc.set_params(np.load(weights))
            lpc.attach(ctx)
        else:
            arms = [a for a in arms if not a.startswith("learned")]

    # warm-up steps with Jacobi from rest; every arm starts from this state
    ctx.state_upload(sc["x"], sc["X"], np.zeros(3 * sc["n"]))
    with ClockSampler(local_rank) as clk:
        ctx.step_resident(args.warmup, mat, GRAV, H, sc["fixed"], sc["fixed_vel"],
                          arm_opts(eolc, "jacobi", args.degree))
        x_w, v_w = ctx.state_download()
        results, failed = {}, {}
        for arm in arms:
            try:
                # one untimed step from the start state right before the arm's
                # timed steps: its plan, network buffers and coarse inverse are
                # built for this state instead of left by the previous arm;
                # time_arm then restarts the refresh counts, so the first timed
                # step evaluates the network and updates the coarse inverse
                ctx.state_upload(x_w, sc["X"], v_w)
                ctx.step_resident(1, mat, GRAV, H, sc["fixed"], sc["fixed_vel"],
                                  arm_opts(eolc, arm, args.degree))
                results[arm] = time_arm(ctx, sc, mat, arm_opts(eolc, arm, args.degree), x_w,
                                        v_w, args.steps, stream, flush, world, dev,
                                        arm_refresh(arm))
            except Exception as e:  # a failed arm is reported, the others still run
                failed[arm] = "%s: %s" % (type(e).__name__, str(e)[:200])
                ctx.set_learned_refresh(1)
                ctx.set_coarse_refresh(1)
    best = max(results, key=lambda a: results[a]["steps_per_s"])
    res = results[best]
    value = res["steps_per_s"]

    # e2e: the best arm through eolc_step with pinned host buffers
    opts = arm_opts(eolc, best, args.degree)
    ctx.set_learned_refresh(arm_refresh(best)[0])
    ctx.set_coarse_refresh(arm_refresh(best)[1])
    xh = torch.empty(3 * sc["n"], dtype=torch.float64).pin_memory().numpy()
    vh = torch.empty(3 * sc["n"], dtype=torch.float64).pin_memory().numpy()
    Xh = torch.empty(2 * sc["n"], dtype=torch.float64).pin_memory().numpy()
    xh[:] = x_w; vh[:] = v_w; Xh[:] = sc["X"]
    if world > 1:
        torch.distributed.barrier()
    e2e_ms = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.step(xh, Xh, vh, mat, GRAV, H, sc["fixed"], sc["fixed_vel"], opts)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = max_over_ranks(sum(e2e_ms), world, dev)
    e2e_val = job_rate(world, args.steps, e2e_total)
    sharded = None
    if world > 1 and not args.no_batch:
        sharded = optional_line(lambda: run_batched_sharded(args, rank, world, local_rank, stream,
                                                            flush, dev))

    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    # Roofline of the dominant kernel, the best arm's resident solve (one
    # launch per step).  Its algorithmic HBM bytes per launch: the matrix
    # (FP32 values, int32 column indices, row pointers) read once, the FP64
    # right-hand side in and the FP64 solution out -- the resident kernels
    # hold the matrix on chip, so no iteration re-reads it.
    n = sc["n"]
    kern_s = res["pcg_kernel_ms"] / 1e3
    alg_bytes = n_blocks * (36 + 4) + (n + 1) * 4 + 2 * 3 * n * 8
    achieved = alg_bytes / kern_s / 1e9
    kernel = ARM_KERNEL[best]
    traffic = None
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "kernel_traffic.json"))) \
            .get(kernel, {}).get("bytes_per_launch")
    except Exception:
        traffic = None
    # What binds it is latency: one grid-wide reduction per iteration.  The
    # resident Jacobi iteration (one product, one reduction) is the floor a
    # one-level method reaches on this GPU.
    us_iter = 1e3 * res["pcg_kernel_ms"] / max(res["mean_pcg_iters"], 1e-9)
    jac = results.get("jacobi")
    jac_us = 1e3 * jac["pcg_kernel_ms"] / max(jac["mean_pcg_iters"], 1e-9) if jac else None
    # bytes an HBM-streamed implementation of the best arm's method would
    # move per iteration (every product's matrix and vectors + CG passes)
    bpi = algorithmic_bytes_per_iter(n, n_blocks)
    if best.startswith("learned"):
        bpi += n_blocks * (36 + 4)  # one more BSR apply (G, pattern of MDK)
    elif best.startswith("patch"):
        bpi += (max(1, args.degree) - 1) * (n_blocks * 36 + 2 * n * 12)
    streamed = bpi * res["mean_pcg_iters"] / kern_s / 1e9
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
        "frac": achieved / hbm, "traffic": traffic, "kernel": kernel,
        "algorithmic_bytes_per_launch": alg_bytes,
        "dram_frac": (traffic / kern_s / 1e9 / hbm) if traffic else None,
        "latency": {"us_per_iter": us_iter, "iters_per_launch": res["mean_pcg_iters"],
                    "jacobi_us_per_iter": jac_us,
                    "note": "the resident solve is bound by one grid-wide reduction per "
                            "iteration, not by HBM: jacobi_us_per_iter is the measured "
                            "one-product floor on this GPU"},
        "streamed_equivalent": {
            "bytes_per_iter": bpi, "achieved": streamed, "frac": streamed / hbm,
            "note": "bytes an HBM-streamed implementation of the same method would move "
                    "per iteration x iterations / kernel time; > 1 means no HBM-streamed "
                    "implementation could match the resident kernel"},
        "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s",
    }
    cpu = None
    if world == 1 and not args.no_cpu:
        secs, cit = cpu_step_seconds(sc, x_w, v_w)
        cpu = {"value": 1.0 / secs, "unit": "steps/s", "cores": 1, "kind": "port",
               "sample": "one full oracle step (triplet assembly + FP64 Jacobi CG, %d iterations)"
                         " on the post-warm-up state, one thread" % cit}
    arms_out = {a: {k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()}
                for a, r in results.items()}
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 dots + f64 refinement residual)", "data": "synthetic",
        "config": {"workload": "sheet 256x256 quads, 66049 nodes, 131072 tris, 196096 hinges,"
                               " 852481 blocks, 2 corners pinned, rel-res 1e-8 (FP64)",
                   "solver": "%s-PCG (fastest arm)" % best,
                   "arms": arms_out,
                   "failed_arms": failed,
                   "learned_vs_jacobi_steps_ratio": {
                       a: results[a]["steps_per_s"] / results["jacobi"]["steps_per_s"]
                       for a in results if a.startswith("learned") and "jacobi" in results},
                   "patch_degree": args.degree,
                   "l2": "flushed (256 MiB write) before each step",
                   "start": "%d Jacobi warm-up steps from rest; every arm times the same "
                            "%d steps from that state" % (args.warmup, args.steps),
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "e2e": {"value": e2e_val, "unit": "steps/s", "h2d_bytes_per_step": 8 * 8 * sc["n"],
                "d2h_bytes_per_step": 6 * 8 * sc["n"]},
        "gpu_launches": res["launches"],
        "roofline": roofline,
        "clocks": clk.summary(),
    }
    # the metric's own comparison at the top level: the fastest learned arm
    # against the resident Jacobi arm, both to the same FP64 residual
    learned_arms = [a for a in results if a.startswith("learned")]
    if learned_arms and "jacobi" in results:
        bl = max(learned_arms, key=lambda a: results[a]["steps_per_s"])
        line["learned_arm"] = bl
        line["learned_steps_per_s"] = results[bl]["steps_per_s"]
        line["jacobi_steps_per_s"] = results["jacobi"]["steps_per_s"]
        line["learned_vs_jacobi"] = results[bl]["steps_per_s"] / results["jacobi"]["steps_per_s"]
    if cpu:
        line["cpu_baseline"] = cpu
    if sharded is not None:
        line["batched_sharded"] = sharded
    if world == 1 and not args.no_cd2:
        line["cd2"] = optional_line(lambda: run_cd2(args, local_rank, stream))
    if world == 1 and not args.no_export:
        line["obj_export"] = optional_line(lambda: run_export(ctx, sc, x_w, stream))
    if world == 1 and not args.no_contacts:
        line["contact_step"] = optional_line(lambda: run_contacts(args, local_rank, stream, flush))
    if world == 1 and not args.no_refresh:
        line["topology_refresh"] = optional_line(lambda: run_refresh(args, local_rank, stream, sc))
    if world == 1 and not args.no_eol:
        line["eol_fill"] = optional_line(lambda: run_eol(args, local_rank, stream, sc))
        line["eol_step"] = optional_line(lambda: run_eol_step(args, local_rank, stream))
    if world == 1 and not args.no_batch:
        line["batched"] = optional_line(lambda: run_batched(args, local_rank, stream, flush))
        line["batched_delaunay_learned"] = optional_line(
            lambda: run_delaunay(args, local_rank, stream, flush))
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precond", default="all",
                    help="comma-separated arms among jacobi, jacobi-streamed, block, patch, "
                         "learned, learned-r4; 'all' times all but block")
    ap.add_argument("--degree", type=int, default=5, help="patch preconditioner degree")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-sheets line")
    ap.add_argument("--no-export", action="store_true", help="skip the OBJ export line")
    ap.add_argument("--no-cd2", action="store_true", help="skip the CD2 (configuration 2) line")
    ap.add_argument("--no-contacts", action="store_true", help="skip the contact-step line")
    ap.add_argument("--no-refresh", action="store_true", help="skip the topology-refresh line")
    ap.add_argument("--no-eol", action="store_true", help="skip the EOL fill and EOL step lines")
    ap.add_argument("--batch-sheets", type=int, default=256)
    ap.add_argument("--delaunay-meshes", type=int, default=64)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
