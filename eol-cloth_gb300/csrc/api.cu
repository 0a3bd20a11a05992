// C ABI of libeolc (include/eolc.h): context, topology, Forces::fill,
// velocity solve and Cloth::step on one GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "internal.h"

using namespace eolc;

namespace {

#define EOLC_CHECK_CUDA(ctx, expr)                                   \
  do {                                                               \
    cudaError_t e_ = (expr);                                         \
    if (e_ != cudaSuccess) {                                         \
      (ctx)->err = std::string(#expr ": ") + cudaGetErrorString(e_); \
      return EOLC_CUDA_ERROR;                                        \
    }                                                                \
  } while (0)

constexpr int kDefaultPatchDegree = 5;  // Chebyshev degree of the patch solves

eolc_status fail(eolc_ctx *ctx, eolc_status s, const char *msg) {
  if (ctx) ctx->err = msg;
  return s;
}

MaterialD make_material(const eolc_material &m, const double g[3], double h) {
  MaterialD d;
  d.rho = m.density;
  d.mu = m.e / (1 + m.nu) / 2;
  d.lam = m.e * m.nu / ((1 + m.nu) * (1 - 2 * m.nu));
  d.beta = m.beta;
  d.dh2 = m.damping_b * h * h;  // ((damping(1) * h) * h), Forces.cpp:105
  d.g[0] = g[0]; d.g[1] = g[1]; d.g[2] = g[2];
  d.h = h;
  return d;
}

// beq_k = (1 - 0.01) v[dof_k] + c_k (addFixed, Constraints.cpp:114-119)
__global__ void pins_kernel(int n_fixed, const int *dofs, const double *c,
                            const double *v, double *beq_full) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_fixed) return;
  int d = dofs[k];
  beq_full[d] = (1 - 0.01) * v[d] + c[k];
}

// node->x = node->x + h * node->v (Cloth.cpp:394-400)
__global__ void integrate_kernel(int n, double h, const double *v, double *x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] + h * v[i];
}

// Cloth.cpp:394-410 on a topology with EOL nodes: x += h v on the n_real
// mesh nodes, and u += h vE for EOL node k (Eulerian velocity at block row
// n_real + k, DOFs 0 and 1).
__global__ void integrate_eol_kernel(int n_real, int n_eol, const int *__restrict__ eol_node,
                                     double h, const double *__restrict__ v, double *__restrict__ x,
                                     double *__restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3 * n_real) x[i] = x[i] + h * v[i];
  if (i < n_eol) {
    const int a = eol_node[i];
    for (int j = 0; j < 2; ++j) u[2 * a + j] = u[2 * a + j] + h * v[3 * (n_real + i) + j];
  }
}

eolc_status need_topology(eolc_ctx *ctx) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!ctx->has_topology) return fail(ctx, EOLC_NO_TOPOLOGY, "no topology set");
  return EOLC_OK;
}

eolc_status check_opts(eolc_ctx *ctx, const eolc_solve_opts *o) {
  if (!o) return fail(ctx, EOLC_BAD_ARG, "null solve options");
  if (!(o->rel_tol > 0) || o->max_iter <= 0)
    return fail(ctx, EOLC_BAD_ARG, "rel_tol must be > 0 and max_iter > 0");
  if (o->precision != EOLC_PREC_FP64 && o->precision != EOLC_PREC_MIXED)
    return fail(ctx, EOLC_BAD_ARG, "unknown precision");
  if (o->precond < EOLC_PC_JACOBI || o->precond > EOLC_PC_PATCH)
    return fail(ctx, EOLC_BAD_ARG, "unknown preconditioner");
  if (o->degree < 0 || o->degree > 64)
    return fail(ctx, EOLC_BAD_ARG, "patch degree must be in 0..64");
  return EOLC_OK;
}

// Uploads the fixed DOF list (and their velocities, when given) and rebuilds
// the 3N-byte pinned mask, on every call: a step may change its pins.
eolc_status set_pins(eolc_ctx *ctx, const int *dofs_h, const double *vel_h,
                     int n_fixed, cudaStream_t s) {
  int n = 3 * ctx->topo.n_nodes;
  if (n_fixed < 0 || (n_fixed > 0 && !dofs_h)) return fail(ctx, EOLC_BAD_ARG, "bad fixed list");
  // the same list as the last upload on this topology: nothing to do (a new
  // topology resets n_fixed_dev)
  if (ctx->n_fixed_dev == n_fixed && int(ctx->pin_dofs_h.size()) == n_fixed &&
      std::equal(dofs_h, dofs_h + n_fixed, ctx->pin_dofs_h.begin()) &&
      (!vel_h || (int(ctx->pin_vel_h.size()) == n_fixed &&
                  std::equal(vel_h, vel_h + n_fixed, ctx->pin_vel_h.begin()))) &&
      ctx->beq_full.n == size_t(n))
    return EOLC_OK;
  std::vector<uint8_t> mask(n, 0);
  for (int k = 0; k < n_fixed; ++k) {
    if (dofs_h[k] < 0 || dofs_h[k] >= n) return fail(ctx, EOLC_BAD_ARG, "fixed dof out of range");
    mask[dofs_h[k]] = 1;
  }
  // the padded third DOF of every Eulerian (EOL) node stays 0
  for (int i = ctx->topo.n_real; i < ctx->topo.n_nodes; ++i) mask[3 * i + 2] = 1;
  EOLC_CHECK_CUDA(ctx, ctx->pinned.upload(mask.data(), n, s));
  EOLC_CHECK_CUDA(ctx, ctx->fixed_dofs.upload(dofs_h, n_fixed, s));
  if (vel_h) EOLC_CHECK_CUDA(ctx, ctx->fixed_vel.upload(vel_h, n_fixed, s));
  ctx->n_fixed_dev = n_fixed;
  ctx->pin_dofs_h.assign(dofs_h, dofs_h + n_fixed);
  if (vel_h) ctx->pin_vel_h.assign(vel_h, vel_h + n_fixed);
  else ctx->pin_vel_h.clear();  // the device copy may be stale: compare next time
  EOLC_CHECK_CUDA(ctx, ctx->beq_full.resize(n));
  return EOLC_OK;
}

// Eulerian node k repeats the position and material coordinates of its EOL
// node (only the resident solver's partition reads them).
__global__ void eol_positions_kernel(int n_real, int n_eol, const int *eol_node, double *x,
                                     double *X) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_eol) return;
  const int v = eol_node[k];
  for (int c = 0; c < 3; ++c) x[3 * (n_real + k) + c] = x[3 * v + c];
  for (int c = 0; c < 2; ++c) X[2 * (n_real + k) + c] = X[2 * v + c];
}

// Positions x (3 n_real) and material coordinates X (2 n_real) of the mesh
// nodes, then the Eulerian nodes' copies.
eolc_status upload_positions(eolc_ctx *ctx, const double *x_h, const double *X_h,
                             cudaStream_t s) {
  const DevTopology &T = ctx->topo;
  const int n = T.n_real;
  if (x_h) EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->x.p, x_h, sizeof(double) * 3 * n,
                                                cudaMemcpyHostToDevice, s));
  if (X_h) EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->X.p, X_h, sizeof(double) * 2 * n,
                                                cudaMemcpyHostToDevice, s));
  if (T.n_eol > 0) {
    eol_positions_kernel<<<(T.n_eol + 127) / 128, 128, 0, s>>>(n, T.n_eol, T.eol_node.p,
                                                               ctx->x.p, ctx->X.p);
    ctx->launches += 1;
    EOLC_CHECK_CUDA(ctx, cudaGetLastError());
  }
  return EOLC_OK;
}

eolc_status ensure_state(eolc_ctx *ctx) {
  size_t n = size_t(ctx->topo.n_nodes) * 3;
  size_t nb9 = size_t(ctx->topo.n_blocks) * 9;
  EOLC_CHECK_CUDA(ctx, ctx->x.resize(n));
  EOLC_CHECK_CUDA(ctx, ctx->v.resize(n));
  EOLC_CHECK_CUDA(ctx, ctx->X.resize(size_t(ctx->topo.n_nodes) * 2));
  EOLC_CHECK_CUDA(ctx, ctx->f.resize(n));
  EOLC_CHECK_CUDA(ctx, ctx->b.resize(n));
  // +16 elements: the solver stages tiles with 16-byte copies whose rounded
  // tail may run past the last block
  EOLC_CHECK_CUDA(ctx, ctx->A32.resize(nb9 + 16));
  EOLC_CHECK_CUDA(ctx, ctx->beq_full.resize(n));
  return EOLC_OK;
}

// The side stream and its fork / join events (created outside any capture).
eolc_status ensure_aux(eolc_ctx *ctx) {
  if (ctx->aux) return EOLC_OK;
  EOLC_CHECK_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
  EOLC_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->aux_fork, cudaEventDisableTiming));
  EOLC_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->aux_join, cudaEventDisableTiming));
  return EOLC_OK;
}

// Assembles MDK (and f, b) for the device state x, X, v.  batched: every
// instance uses its own material from ctx->inst_matd (mat is ignored).
// The FP64 force pass (FP64 pipe) runs on the side stream concurrently with
// the FP32 matrix passes; s waits for it before returning to the caller's
// next work.
eolc_status assemble(eolc_ctx *ctx, const eolc_material &mat, const double g[3],
                     double h, int prec, bool want_M, bool want_b,
                     cudaStream_t s, bool batched = false) {
  MaterialD md = make_material(mat, g, h);
  const MaterialD *mats = batched ? ctx->inst_matd.p : nullptr;
  const int *node_inst = batched ? ctx->node_inst.p : nullptr;
  size_t nb9 = size_t(ctx->topo.n_blocks) * 9;
  const bool eol = ctx->topo.n_eol > 0;
  if (eol && want_b) want_M = true;  // b = -(M v + h f) from the assembled M
  if (prec == EOLC_PREC_FP64) EOLC_CHECK_CUDA(ctx, ctx->A64.resize(nb9 + 16));
  if (want_M) EOLC_CHECK_CUDA(ctx, ctx->Mblk.resize(nb9));
  {
    // the shared-memory assembly's tiles, once per topology and precision
    // (never while the stream is being captured: the build synchronizes;
    // batched steps build them before their capture)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    EOLC_CHECK_CUDA(ctx, cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone) {
      const std::string msg = ensure_assembly_tiles(ctx->topo, prec, s, ctx->launches);
      if (!msg.empty()) {
        ctx->err = msg;
        return EOLC_CUDA_ERROR;
      }
    }
  }
  {
    const size_t need = assemble_scratch_bytes(ctx->topo, prec);
    if (ctx->elem.n < need) EOLC_CHECK_CUDA(ctx, ctx->elem.resize(need));
  }
  eolc_status st = ensure_aux(ctx);
  if (st != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, cudaEventRecord(ctx->aux_fork, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamWaitEvent(ctx->aux, ctx->aux_fork, 0));
  launch_forces_rhs(ctx->topo, ctx->x.p, ctx->X.p, ctx->v.p, md, mats, node_inst, prec,
                    ctx->elem.p, ctx->f.p, want_b ? ctx->b.p : nullptr, ctx->aux);
  EOLC_CHECK_CUDA(ctx, cudaEventRecord(ctx->aux_join, ctx->aux));
  const int nk = launch_assemble_blocks(
      ctx->topo, ctx->x.p, ctx->X.p, md, mats, node_inst, prec, ctx->elem.p,
      prec == EOLC_PREC_FP64 ? ctx->A64.p : nullptr,
      prec == EOLC_PREC_FP64 ? nullptr : ctx->A32.p, want_M ? ctx->Mblk.p : nullptr, s);
  EOLC_CHECK_CUDA(ctx, cudaStreamWaitEvent(s, ctx->aux_join, 0));
  ctx->launches += nk + 2;  // + the two force kernels
  if (eol) {
    ctx->launches += 1;
    if (want_b) {
      launch_bsr_rhs(ctx->topo, ctx->Mblk.p, ctx->v.p, ctx->f.p, h, ctx->b.p, s);
      ctx->launches += 1;
    }
  }
  EOLC_CHECK_CUDA(ctx, cudaGetLastError());
  return EOLC_OK;
}

eolc_status solve_device(eolc_ctx *ctx, const eolc_solve_opts *o,
                         eolc_solve_info *info, cudaStream_t s) {
  return solve_with_args(ctx, o, default_pcg_args(ctx, o), info, s);
}

cudaStream_t stream_of(eolc_ctx *ctx) { return ctx->stream; }

// ---- batches ---------------------------------------------------------------

PcgArgs batch_pcg_args(eolc_ctx *ctx, const eolc_solve_opts *o, double *v) {
  PcgArgs a;
  a.T = &ctx->topo;
  a.A64 = ctx->A64.p;
  a.A32 = ctx->A32.p;
  a.b = ctx->b.p;
  a.pinned = ctx->pinned.p;
  a.beq_full = ctx->beq_full.p;
  a.v = v;
  a.precision = o->precision;
  a.precond = o->precond;
  a.rel_tol = o->rel_tol;
  a.max_iter = o->max_iter;
  a.learned = nullptr;
  a.spin_limit = ctx->spin_limit;
  return a;
}

// Checks shared by the batched entry points; uploads the pins and the
// per-instance material table for (grav, h).
eolc_status batch_begin(eolc_ctx *ctx, const double grav[3], double h, const int *fixed_dofs_h,
                        const double *fixed_vel_h, int n_fixed, const eolc_solve_opts *opts,
                        cudaStream_t s) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = check_opts(ctx, opts)) != EOLC_OK) return st;
  if ((st = refuse_eol(ctx)) != EOLC_OK) return st;
  // host mirrors before any capture (the learned network's graph reads them)
  if (!host_topology(ctx)) return EOLC_CUDA_ERROR;
  if (opts->precond == EOLC_PC_PATCH)
    return fail(ctx, EOLC_BAD_ARG, "batched steps use Jacobi, block Jacobi or the learned preconditioner");
  if (opts->precond == EOLC_PC_LEARNED) {
    if (!ctx->lpc) return fail(ctx, EOLC_BAD_ARG, "no learned preconditioner attached");
    if (opts->precision != EOLC_PREC_MIXED)
      return fail(ctx, EOLC_BAD_ARG, "the learned preconditioner runs on the mixed path");
  }
  if (!grav) return fail(ctx, EOLC_BAD_ARG, "null gravity");
  if (n_fixed > 0 && (!fixed_dofs_h || !fixed_vel_h)) return fail(ctx, EOLC_BAD_ARG, "null fixed list");
  const int n_inst = int(ctx->node_off.size()) - 1;
  if (int(ctx->inst_mat.size()) != n_inst)
    return fail(ctx, EOLC_BAD_ARG, "no per-instance materials set");
  if ((st = set_pins(ctx, fixed_dofs_h, fixed_vel_h, n_fixed, s)) != EOLC_OK) return st;
  ctx->inst_matd_h.resize(n_inst);
  for (int k = 0; k < n_inst; ++k) ctx->inst_matd_h[k] = make_material(ctx->inst_mat[k], grav, h);
  EOLC_CHECK_CUDA(ctx, ctx->inst_matd.upload(ctx->inst_matd_h.data(), n_inst, s));
  if (opts->precision == EOLC_PREC_FP64)
    EOLC_CHECK_CUDA(ctx, ctx->A64.resize(size_t(ctx->topo.n_blocks) * 9 + 16));
  // the captured assembly writes its element blocks here, and forks its
  // force pass onto the side stream
  const size_t need = assemble_scratch_bytes(ctx->topo, opts->precision);
  if (ctx->elem.n < need) EOLC_CHECK_CUDA(ctx, ctx->elem.resize(need));
  return ensure_aux(ctx);
}

// Pins, assembly and right-hand side of one batched step (no allocation, no
// synchronisation: capturable).
eolc_status enqueue_batch_assembly(eolc_ctx *ctx, const double grav[3], double h,
                                   const eolc_solve_opts *o, cudaStream_t s) {
  const int n = 3 * ctx->topo.n_nodes;
  EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->beq_full.p, 0, sizeof(double) * n, s));
  if (ctx->n_fixed_dev > 0) {
    pins_kernel<<<(ctx->n_fixed_dev + 127) / 128, 128, 0, s>>>(
        ctx->n_fixed_dev, ctx->fixed_dofs.p, ctx->fixed_vel.p, ctx->v.p, ctx->beq_full.p);
    ctx->launches += 1;
  }
  eolc_material unused{};
  ctx->last_precision = o->precision;  // the matrix the step leaves on the context
  return assemble(ctx, unused, grav, h, o->precision, false, true, s, true);
}

// One whole batched step: pins, assembly, batched PCG, x += h v.
eolc_status enqueue_batch_step(eolc_ctx *ctx, const double grav[3], double h,
                               const eolc_solve_opts *o, cudaStream_t s) {
  eolc_status st = enqueue_batch_assembly(ctx, grav, h, o, s);
  if (st != EOLC_OK) return st;
  PcgArgs a = batch_pcg_args(ctx, o, ctx->v.p);
  st = batch_enqueue(ctx->bwork, a, s, ctx->err, ctx->launches);
  if (st != EOLC_OK) return st;
  const int n = 3 * ctx->topo.n_nodes;
  integrate_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, h, ctx->v.p, ctx->x.p);
  ctx->launches += 1;
  EOLC_CHECK_CUDA(ctx, cudaGetLastError());
  return EOLC_OK;
}

// Times every configuration of the batched solver on the current state
// (assembled once; solutions go to a scratch vector, the state is unchanged)
// and keeps the fastest.  ms_h (optional): one entry per configuration,
// -1 where the configuration does not apply.
eolc_status batch_autotune(eolc_ctx *ctx, const double grav[3], double h,
                           const eolc_solve_opts *o_in, cudaStream_t s, int *chosen,
                           double *ms_h) {
  // configurations are timed on the Jacobi solve (the learned solve runs on
  // the same tiles and cluster shape)
  eolc_solve_opts oj = *o_in;
  if (oj.precond == EOLC_PC_LEARNED) oj.precond = EOLC_PC_JACOBI;
  const eolc_solve_opts *o = &oj;
  eolc_status st = enqueue_batch_assembly(ctx, grav, h, o, s);
  if (st != EOLC_OK) return st;
  DevBuf<double> scratch;
  EOLC_CHECK_CUDA(ctx, scratch.resize(size_t(3) * ctx->topo.n_nodes));
  PcgArgs a = batch_pcg_args(ctx, o, scratch.p);
  if (!ctx->ev[2]) { cudaEventCreate(&ctx->ev[2]); cudaEventCreate(&ctx->ev[3]); }
  const int nc = batch_num_configs();
  int best = -1;
  double best_ms = 0;
  std::vector<BatchRecord> rec;
  for (int c = 0; c < nc; ++c) {
    double ms = -1;
    std::string msg;
    if (batch_prepare(ctx->bwork, a, ctx->node_off, c, s, msg) == EOLC_OK) {
      bool ok = batch_reset_records(ctx->bwork, s) == EOLC_OK &&
                batch_enqueue(ctx->bwork, a, s, ctx->err, ctx->launches) == EOLC_OK &&
                batch_read_records(ctx->bwork, rec, s) == EOLC_OK;
      for (const BatchRecord &r : rec) ok = ok && r.status == EOLC_OK;
      if (ok) {
        constexpr int kReps = 2;
        cudaEventRecord(ctx->ev[2], s);
        for (int k = 0; k < kReps && ok; ++k)
          ok = batch_enqueue(ctx->bwork, a, s, ctx->err, ctx->launches) == EOLC_OK;
        cudaEventRecord(ctx->ev[3], s);
        EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
        float t = 0.f;
        cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]);
        if (ok) ms = double(t) / kReps;
      }
      EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
    }
    if (ms_h) ms_h[c] = ms;
    if (ms >= 0 && (best < 0 || ms < best_ms)) { best = c; best_ms = ms; }
  }
  if (best < 0) return fail(ctx, EOLC_BAD_ARG, "no batched solver configuration fits this batch");
  std::string msg;
  if ((st = batch_prepare(ctx->bwork, a, ctx->node_off, best, s, msg)) != EOLC_OK)
    return fail(ctx, st, msg.c_str());
  ctx->batch_config = best;
  if (chosen) *chosen = best;
  return EOLC_OK;
}

// Per-instance and total results of a batched call from the device records.
eolc_status batch_results(eolc_ctx *ctx, int n_steps, float ms, cudaStream_t s,
                          eolc_solve_info *inst_info_h, eolc_batch_info *total) {
  std::vector<BatchRecord> rec;
  eolc_status st = batch_read_records(ctx->bwork, rec, s);
  if (st != EOLC_OK) return fail(ctx, st, "batched step failed on the device");
  eolc_batch_info tot{};
  tot.status = EOLC_OK;
  tot.config = ctx->batch_config;
  tot.steps = n_steps;
  tot.step_ms = ms;
  for (size_t k = 0; k < rec.size(); ++k) {
    const BatchRecord &r = rec[k];
    if (r.status != EOLC_OK) {
      if (tot.status == EOLC_OK) tot.status = r.status;
      tot.n_failed += 1;
    }
    tot.iterations += r.iterations;
    tot.max_iterations = std::max(tot.max_iterations, r.max_iterations);
    tot.max_rel_res = std::max(tot.max_rel_res, r.rel_res);
    tot.n_fallback += r.used_fallback;
    if (inst_info_h) {
      eolc_solve_info &o = inst_info_h[k];
      o = eolc_solve_info{};
      o.status = r.status;
      o.iterations = r.iterations;
      o.refinements = r.refinements;
      o.used_fallback = r.used_fallback;
      o.rel_res = r.rel_res;
    }
  }
  if (total) *total = tot;
  if (tot.status != EOLC_OK) ctx->err = "an instance's solve failed (see the per-instance status)";
  return eolc_status(tot.status);
}

// Batched steps with the learned preconditioner: per step the assembly, the
// network's forward pass on the whole batch (block-diagonal G), one learned
// batched launch with per-instance caps and one Jacobi launch over the
// instances it left unconverged, x += h v.  Not captured in a graph (the
// forward pass synchronises).
eolc_status step_batched_learned(eolc_ctx *ctx, int n_steps, const double grav[3], double h,
                                 const eolc_solve_opts *opts, eolc_solve_info *inst_info_h,
                                 eolc_batch_info *total, cudaStream_t s) {
  eolc_status st = batch_reset_records(ctx->bwork, s);
  if (st != EOLC_OK) return fail(ctx, st, "record reset failed");
  if (!ctx->ev[2]) { cudaEventCreate(&ctx->ev[2]); cudaEventCreate(&ctx->ev[3]); }
  EOLC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  const int n = 3 * ctx->topo.n_nodes;
  for (int k = 0; k < n_steps; ++k) {
    if ((st = enqueue_batch_assembly(ctx, grav, h, opts, s)) != EOLC_OK) return st;
    const float *Gm = nullptr;
    std::string msg = learned_forward(ctx->lpc, ctx, ctx->pinned.p, &Gm, s);
    if (!msg.empty()) return fail(ctx, EOLC_CUDA_ERROR, msg.c_str());
    ctx->launches += kLearnedForwardLaunches;
    PcgArgs a = batch_pcg_args(ctx, opts, ctx->v.p);
    if ((st = batch_enqueue_learned(ctx->bwork, a, Gm, opts->fallback_factor, ctx->node_inst.p, s,
                                    ctx->err, ctx->launches)) != EOLC_OK)
      return st;
    integrate_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, h, ctx->v.p, ctx->x.p);
    ctx->launches += 1;
  }
  EOLC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
  return batch_results(ctx, n_steps, ms, s, inst_info_h, total);
}

}  // namespace

namespace eolc {

PcgArgs default_pcg_args(eolc_ctx *ctx, const eolc_solve_opts *o) {
  PcgArgs a;
  a.T = &ctx->topo;
  a.A64 = ctx->A64.p;
  a.A32 = ctx->A32.p;
  a.b = ctx->b.p;
  a.pinned = ctx->pinned.p;
  a.beq_full = ctx->beq_full.p;
  a.v = ctx->v.p;
  a.precision = o->precision;
  a.precond = o->precond;
  a.rel_tol = o->rel_tol;
  a.max_iter = o->max_iter;
  a.learned = nullptr;
  a.X = ctx->X.p;
  a.spin_limit = ctx->spin_limit;
  return a;
}

// The dispatch of eolc_velocity_solve on explicit arguments (matrix, rhs and
// solution buffers of a): learned (with the Jacobi fallback), patch, resident
// or streamed PCG.
eolc_status solve_with_args(eolc_ctx *ctx, const eolc_solve_opts *o, const PcgArgs &a,
                            eolc_solve_info *info, cudaStream_t s) {
  if (o->precision == EOLC_PREC_FP64 && !ctx->A64.p)
    return fail(ctx, EOLC_BAD_ARG, "no FP64 matrix assembled");
  eolc_solve_info local{};
  eolc_solve_info *inf = info ? info : &local;
  if (o->precond == EOLC_PC_LEARNED) {
    if (ctx->topo.n_eol > 0) return refuse_eol(ctx);
    if (!ctx->lpc) return fail(ctx, EOLC_BAD_ARG, "no learned preconditioner attached");
    if (o->precision != EOLC_PREC_MIXED)
      return fail(ctx, EOLC_BAD_ARG, "the learned preconditioner runs on the mixed path");
    const bool resident = !o->streamed && resident_fits(ctx->pwork, ctx->topo, ctx->X.p, s);
    // the resident path keeps the network's G between solves: it is
    // re-evaluated once it has served lpc_refresh solves (1: every solve)
    const bool reuse = resident && ctx->lpc_cached == ctx->lpc && ctx->lpc_uses < ctx->lpc_refresh;
    const float *Gm = nullptr;
    if (!reuse) {
      std::string msg = learned_forward(ctx->lpc, ctx, ctx->pinned.p, &Gm, s);
      if (!msg.empty()) return fail(ctx, EOLC_CUDA_ERROR, msg.c_str());
      ctx->launches += kLearnedForwardLaunches;
      ctx->lpc_cached = resident ? ctx->lpc : nullptr;
      ctx->lpc_uses = 0;
    }
    ctx->lpc_uses += 1;
    // fall back to Jacobi when the learned solve has not converged within
    // fallback_factor x the last Jacobi iteration count
    PcgArgs al = a;
    if (o->fallback_factor > 0 && ctx->last_jacobi_iters > 0)
      al.max_iter = std::min(o->max_iter, o->fallback_factor * ctx->last_jacobi_iters);
    eolc_status st = resident ? run_pcg_resident(ctx->pwork, al, ResidentPC::kLearned, 0, Gm, inf,
                                                 s, ctx->err, ctx->launches, o->no_coarse == 0,
                                                 ctx->coarse_refresh)
                              : run_pcg_learned(ctx->work, al, Gm, inf, s, ctx->err, ctx->launches);
    if (st == EOLC_OK || o->fallback_factor <= 0) return st;
    const double kms = inf->solve_kernel_ms;
    const int its = inf->iterations;
    PcgArgs aj = a;
    aj.precond = EOLC_PC_JACOBI;
    st = resident ? run_pcg_resident(ctx->pwork, aj, ResidentPC::kJacobi, 0, nullptr, inf, s,
                                     ctx->err, ctx->launches)
                  : run_pcg(ctx->work, aj, inf, s, ctx->err, ctx->launches);
    inf->used_fallback = 1;
    inf->iterations += its;
    inf->solve_kernel_ms += kms;
    if (st == EOLC_OK) ctx->last_jacobi_iters = inf->iterations - its;
    return st;
  }
  if (o->precond == EOLC_PC_PATCH)
    return run_pcg_resident(ctx->pwork, a, ResidentPC::kPatch,
                            o->degree > 0 ? o->degree : kDefaultPatchDegree, nullptr, inf, s,
                            ctx->err, ctx->launches, o->no_coarse == 0, ctx->coarse_refresh);
  eolc_status st;
  if (o->precision == EOLC_PREC_MIXED && !o->streamed && resident_fits(ctx->pwork, ctx->topo, ctx->X.p, s))
    st = run_pcg_resident(ctx->pwork, a, ResidentPC::kJacobi, 0, nullptr, inf, s, ctx->err,
                          ctx->launches);
  else
    st = run_pcg(ctx->work, a, inf, s, ctx->err, ctx->launches);
  if (st == EOLC_OK && o->precond == EOLC_PC_JACOBI) ctx->last_jacobi_iters = inf->iterations;
  return st;
}


eolc_status prepare_pins_rhs(eolc_ctx *ctx, const double *b_h, const int *fixed_dofs_h,
                             const double *beq_h, int n_fixed, cudaStream_t s) {
  const int n = 3 * ctx->topo.n_nodes;
  eolc_status st = set_pins(ctx, fixed_dofs_h, nullptr, n_fixed, s);
  if (st != EOLC_OK) return st;
  std::vector<double> beq_full(n, 0.0);
  for (int k = 0; k < n_fixed; ++k) beq_full[fixed_dofs_h[k]] = beq_h[k];
  EOLC_CHECK_CUDA(ctx, ctx->beq_full.upload(beq_full.data(), n, s));
  EOLC_CHECK_CUDA(ctx, ctx->b.upload(b_h, n, s));
  return EOLC_OK;
}

}  // namespace eolc


namespace eolc {

const HostTopology *host_topology(eolc_ctx *ctx) {
  if (ctx->host_valid) return &ctx->host;
  const DevTopology &T = ctx->topo;
  HostTopology &H = ctx->host;
  const int N = T.n_nodes, NB = T.n_blocks;
  cudaStream_t s = ctx->stream;
  H.n_nodes = N;
  H.n_tri = T.n_tri;
  H.n_hinge = T.n_hinge;
  H.n_blocks = NB;
  H.rowptr.resize(size_t(N) + 1);
  H.colidx.resize(NB);
  H.blk_row.resize(NB);
  H.diag.resize(N);
  H.cptr.resize(size_t(NB) + 1);
  H.nf_ptr.resize(size_t(T.n_real) + 1);
  H.nf_list.resize(size_t(3) * T.n_tri);
  auto get = [&](std::vector<int> &dst, const int *src) {
    return cudaMemcpyAsync(dst.data(), src, sizeof(int) * dst.size(), cudaMemcpyDeviceToHost, s);
  };
  cudaError_t e = get(H.rowptr, T.rowptr.p);
  if (e == cudaSuccess) e = get(H.colidx, T.colidx.p);
  if (e == cudaSuccess) e = get(H.blk_row, T.blk_row.p);
  if (e == cudaSuccess) e = get(H.diag, T.diag.p);
  if (e == cudaSuccess) e = get(H.cptr, T.cptr.p);
  if (e == cudaSuccess) e = get(H.nf_ptr, T.nf_ptr.p);
  if (e == cudaSuccess) e = get(H.nf_list, T.nf_list.p);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) {
    H.contrib.resize(H.cptr[NB]);
    e = get(H.contrib, T.contrib.p);
  }
  if (e == cudaSuccess && ctx->host_tri.size() != size_t(3) * T.n_tri) {
    ctx->host_tri.resize(size_t(3) * T.n_tri);
    e = cudaMemcpyAsync(ctx->host_tri.data(), T.tri.p, sizeof(int) * ctx->host_tri.size(),
                        cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    ctx->err = std::string("topology download: ") + cudaGetErrorString(e);
    return nullptr;
  }
  ctx->host_valid = true;
  return &ctx->host;
}

}  // namespace eolc

namespace {

// Builds the BSR pattern, contribution lists and node -> face lists on the
// device from ctx->topo.tri / hinge (already on the device).
eolc_status topology_from_device(eolc_ctx *ctx, int n_nodes, int n_tri, int n_hinge,
                                 cudaStream_t s, int n_eol = 0) {
  ctx->has_topology = false;
  ctx->host_valid = false;
  std::string msg = build_topology_device(ctx->topo_work, n_nodes, ctx->topo.tri.p, n_tri,
                                          n_hinge > 0 ? ctx->topo.hinge.p : nullptr, n_hinge,
                                          ctx->topo, s, ctx->launches, n_eol);
  if (!msg.empty()) return fail(ctx, EOLC_BAD_ARG, msg.c_str());
  return EOLC_OK;
}

// Drops every plan, graph and buffer that depends on the old topology.
eolc_status reset_after_topology(eolc_ctx *ctx, cudaStream_t s) {
  ctx->inst_mat.clear();
  ctx->contact_lambda.clear();
  free_collide_work(ctx->cd_work);
  free_export_work(ctx->ex_work);
  ctx->cd_work = nullptr;
  ctx->ex_work = nullptr;
  ctx->has_topology = true;
  ctx->n_fixed_dev = -1;
  free_solve_work(ctx->work);
  ctx->work = nullptr;
  free_patch_work(ctx->pwork);
  ctx->pwork = nullptr;
  ctx->lpc_cached = nullptr;
  free_batch_work(ctx->bwork);
  ctx->bwork = nullptr;
  ctx->batch_config = -1;
  if (ctx->bgraph) cudaGraphExecDestroy(ctx->bgraph);
  ctx->bgraph = nullptr;
  ctx->bgraph_key.clear();
  ctx->A64.release();
  ctx->Mblk.release();
  ctx->elem.release();
  eolc_status st = ensure_state(ctx);
  if (st != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->v.p, 0, sizeof(double) * ctx->v.n, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  return EOLC_OK;
}

}  // namespace

extern "C" {

int eolc_version(void) { return 1; }

long long eolc_launch_count(const eolc_ctx *ctx) { return ctx ? ctx->launches : 0; }

eolc_status eolc_attach_preconditioner(eolc_ctx *ctx, eolc_lpc *lpc) {
  if (!ctx) return EOLC_BAD_ARG;
  ctx->lpc = lpc;
  ctx->lpc_cached = nullptr;
  return EOLC_OK;
}

eolc_status eolc_set_learned_refresh(eolc_ctx *ctx, int solves) {
  if (!ctx || solves < 1) return EOLC_BAD_ARG;
  ctx->lpc_refresh = solves;
  ctx->lpc_cached = nullptr;  // the count restarts: the next solve runs the network
  ctx->lpc_uses = 0;
  return EOLC_OK;
}

eolc_status eolc_set_coarse_refresh(eolc_ctx *ctx, int solves) {
  if (!ctx || solves < 1) return EOLC_BAD_ARG;
  ctx->coarse_refresh = solves;
  coarse_update_next(ctx->pwork);  // the count restarts at the next solve
  return EOLC_OK;
}

eolc_status eolc_set_wait_limit(eolc_ctx *ctx, long long polls) {
  if (!ctx || polls < 0) return EOLC_BAD_ARG;
  ctx->spin_limit = polls;
  return EOLC_OK;
}

eolc_status eolc_set_jacobi_reference(eolc_ctx *ctx, int iterations) {
  if (!ctx || iterations < 0) return EOLC_BAD_ARG;
  ctx->last_jacobi_iters = iterations;
  return EOLC_OK;
}

eolc_status eolc_create(eolc_ctx **out, int device) {
  if (!out) return EOLC_BAD_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
    return EOLC_CUDA_ERROR;
  auto *ctx = new (std::nothrow) eolc_ctx();
  if (!ctx) return EOLC_CUDA_ERROR;
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return EOLC_CUDA_ERROR;
  }
  ctx->own_stream = true;
  *out = ctx;
  return EOLC_OK;
}

void eolc_destroy(eolc_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_solve_work(ctx->work);
  free_patch_work(ctx->pwork);
  free_collide_work(ctx->cd_work);
  free_export_work(ctx->ex_work);
  free_ineq_work(ctx->iq_work);
  free_topo_scratch(ctx->topo_work);
  free_batch_work(ctx->bwork);
  if (ctx->bgraph) cudaGraphExecDestroy(ctx->bgraph);
  for (cudaEvent_t e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->aux) {
    cudaStreamSynchronize(ctx->aux);
    cudaStreamDestroy(ctx->aux);
    cudaEventDestroy(ctx->aux_fork);
    cudaEventDestroy(ctx->aux_join);
  }
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *eolc_last_error(const eolc_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

eolc_status eolc_set_stream(eolc_ctx *ctx, void *stream) {
  if (!ctx) return EOLC_BAD_ARG;
  cudaSetDevice(ctx->device);
  if (!stream) {
    if (!ctx->own_stream) {
      if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(ctx, EOLC_CUDA_ERROR, "stream creation failed");
      ctx->own_stream = true;
    }
    return EOLC_OK;
  }
  if (ctx->own_stream && ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  ctx->stream = static_cast<cudaStream_t>(stream);
  ctx->own_stream = false;
  return EOLC_OK;
}

eolc_status eolc_set_topology(eolc_ctx *ctx, int n_nodes, const int *tri_h,
                              int n_tri, const int *hinge_h, int n_hinge) {
  if (!ctx) return EOLC_BAD_ARG;
  const int node_off[2] = {0, n_nodes};
  const int tri_off[2] = {0, n_tri};
  const int hinge_off[2] = {0, n_hinge};
  return eolc_set_topology_batched(ctx, 1, node_off, tri_h, tri_off, hinge_h, hinge_off);
}

eolc_status eolc_set_topology_batched(eolc_ctx *ctx, int n_inst, const int *node_off_h,
                                      const int *tri_h, const int *tri_off_h,
                                      const int *hinge_h, const int *hinge_off_h) {
  if (!ctx) return EOLC_BAD_ARG;
  if (n_inst <= 0 || !node_off_h || !tri_off_h || !hinge_off_h)
    return fail(ctx, EOLC_BAD_ARG, "bad instance tables");
  const int n_nodes = node_off_h[n_inst], n_tri = tri_off_h[n_inst],
            n_hinge = hinge_off_h[n_inst];
  if (!tri_h || n_tri <= 0 || (n_hinge > 0 && !hinge_h))
    return fail(ctx, EOLC_BAD_ARG, "null or empty topology");
  if (node_off_h[0] != 0 || tri_off_h[0] != 0 || hinge_off_h[0] != 0)
    return fail(ctx, EOLC_BAD_ARG, "instance tables must start at 0");
  for (int k = 0; k < n_inst; ++k) {
    if (node_off_h[k + 1] <= node_off_h[k] || tri_off_h[k + 1] <= tri_off_h[k] ||
        hinge_off_h[k + 1] < hinge_off_h[k])
      return fail(ctx, EOLC_BAD_ARG, "every instance needs nodes and triangles");
    const int lo = node_off_h[k], hi = node_off_h[k + 1];
    for (int64_t q = int64_t(tri_off_h[k]) * 3; q < int64_t(tri_off_h[k + 1]) * 3; ++q)
      if (tri_h[q] < lo || tri_h[q] >= hi)
        return fail(ctx, EOLC_BAD_ARG, "a triangle references another instance's node");
    for (int64_t q = int64_t(hinge_off_h[k]) * 4; q < int64_t(hinge_off_h[k + 1]) * 4; ++q)
      if (hinge_h[q] < lo || hinge_h[q] >= hi)
        return fail(ctx, EOLC_BAD_ARG, "a hinge references another instance's node");
  }
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  DevTopology &T = ctx->topo;
  EOLC_CHECK_CUDA(ctx, T.tri.upload(tri_h, size_t(n_tri) * 3, s));
  if (n_hinge > 0) EOLC_CHECK_CUDA(ctx, T.hinge.upload(hinge_h, size_t(n_hinge) * 4, s));
  eolc_status st = topology_from_device(ctx, n_nodes, n_tri, n_hinge, s);
  if (st != EOLC_OK) return st;
  std::vector<int> node_inst(n_nodes);
  for (int k = 0; k < n_inst; ++k)
    std::fill(node_inst.begin() + node_off_h[k], node_inst.begin() + node_off_h[k + 1], k);
  EOLC_CHECK_CUDA(ctx, ctx->node_inst.upload(node_inst.data(), node_inst.size(), s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->host_tri.assign(tri_h, tri_h + size_t(n_tri) * 3);
  ctx->node_off.assign(node_off_h, node_off_h + n_inst + 1);
  return reset_after_topology(ctx, s);
}

eolc_status eolc_set_topology_device(eolc_ctx *ctx, int n_nodes, const int *tri_d, int n_tri,
                                     const int *hinge_d, int n_hinge) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!tri_d || n_tri <= 0 || n_nodes <= 0 || n_hinge < 0 || (n_hinge > 0 && !hinge_d))
    return fail(ctx, EOLC_BAD_ARG, "null or empty topology");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  DevTopology &T = ctx->topo;
  EOLC_CHECK_CUDA(ctx, T.tri.resize(size_t(n_tri) * 3));
  EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(T.tri.p, tri_d, sizeof(int) * 3 * size_t(n_tri),
                                       cudaMemcpyDeviceToDevice, s));
  if (n_hinge > 0) {
    EOLC_CHECK_CUDA(ctx, T.hinge.resize(size_t(n_hinge) * 4));
    EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(T.hinge.p, hinge_d, sizeof(int) * 4 * size_t(n_hinge),
                                         cudaMemcpyDeviceToDevice, s));
  }
  eolc_status st = topology_from_device(ctx, n_nodes, n_tri, n_hinge, s);
  if (st != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, ctx->node_inst.resize(n_nodes));
  EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->node_inst.p, 0, sizeof(int) * n_nodes, s));
  ctx->host_tri.clear();  // downloaded on first use
  ctx->node_off.assign({0, n_nodes});
  return reset_after_topology(ctx, s);
}

eolc_status eolc_set_topology_eol(eolc_ctx *ctx, int n_nodes, const int *tri_h, int n_tri,
                                  const int *hinge_h, int n_hinge, const int *eol_nodes_h,
                                  int n_eol) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!tri_h || n_tri <= 0 || n_nodes <= 0 || n_hinge < 0 || (n_hinge > 0 && !hinge_h) ||
      n_eol < 0 || (n_eol > 0 && !eol_nodes_h))
    return fail(ctx, EOLC_BAD_ARG, "null or empty topology");
  std::vector<int> eol(n_nodes, -1);
  for (int k = 0; k < n_eol; ++k) {
    const int v = eol_nodes_h[k];
    if (v < 0 || v >= n_nodes) return fail(ctx, EOLC_BAD_ARG, "EOL node out of range");
    if (eol[v] >= 0) return fail(ctx, EOLC_BAD_ARG, "EOL node listed twice");
    eol[v] = k;
  }
  for (int64_t q = 0; q < int64_t(n_tri) * 3; ++q)
    if (tri_h[q] < 0 || tri_h[q] >= n_nodes)
      return fail(ctx, EOLC_BAD_ARG, "element index out of range");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  DevTopology &T = ctx->topo;
  EOLC_CHECK_CUDA(ctx, T.tri.upload(tri_h, size_t(n_tri) * 3, s));
  if (n_hinge > 0) EOLC_CHECK_CUDA(ctx, T.hinge.upload(hinge_h, size_t(n_hinge) * 4, s));
  if (n_eol > 0) {
    EOLC_CHECK_CUDA(ctx, T.eol.upload(eol.data(), eol.size(), s));
    EOLC_CHECK_CUDA(ctx, T.eol_node.upload(eol_nodes_h, n_eol, s));
  }
  eolc_status st = topology_from_device(ctx, n_nodes, n_tri, n_hinge, s, n_eol);
  if (st != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, ctx->node_inst.resize(T.n_nodes));
  EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->node_inst.p, 0, sizeof(int) * T.n_nodes, s));
  ctx->host_tri.assign(tri_h, tri_h + size_t(n_tri) * 3);
  ctx->node_off.assign({0, T.n_nodes});
  return reset_after_topology(ctx, s);
}

eolc_status eolc_topology_arrays(eolc_ctx *ctx, int *rowptr_h, int *colidx_h, int *cptr_h,
                                 int *contrib_h, int *nf_ptr_h, int *nf_list_h, int sizes[4]) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if (!sizes) return fail(ctx, EOLC_BAD_ARG, "null sizes");
  const DevTopology &T = ctx->topo;
  const int N = T.n_nodes, NB = T.n_blocks;
  int ncon = 0;
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ncon, T.cptr.p + NB, sizeof(int), cudaMemcpyDeviceToHost, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  sizes[0] = N;
  sizes[1] = NB;
  sizes[2] = ncon;
  sizes[3] = 3 * T.n_tri;
  auto get = [&](int *dst, const int *src, size_t n) -> cudaError_t {
    return dst ? cudaMemcpyAsync(dst, src, sizeof(int) * n, cudaMemcpyDeviceToHost, s)
               : cudaSuccess;
  };
  EOLC_CHECK_CUDA(ctx, get(rowptr_h, T.rowptr.p, size_t(N) + 1));
  EOLC_CHECK_CUDA(ctx, get(colidx_h, T.colidx.p, NB));
  EOLC_CHECK_CUDA(ctx, get(cptr_h, T.cptr.p, size_t(NB) + 1));
  EOLC_CHECK_CUDA(ctx, get(contrib_h, T.contrib.p, ncon));
  EOLC_CHECK_CUDA(ctx, get(nf_ptr_h, T.nf_ptr.p, size_t(N) + 1));
  EOLC_CHECK_CUDA(ctx, get(nf_list_h, T.nf_list.p, size_t(3) * T.n_tri));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  return EOLC_OK;
}


eolc_status eolc_bsr_pattern(eolc_ctx *ctx, int *n_blocks, int *rowptr_h,
                             int *colidx_h) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  const HostTopology *H = host_topology(ctx);
  if (!H) return EOLC_CUDA_ERROR;
  if (n_blocks) *n_blocks = H->n_blocks;
  if (rowptr_h) std::memcpy(rowptr_h, H->rowptr.data(), sizeof(int) * H->rowptr.size());
  if (colidx_h) std::memcpy(colidx_h, H->colidx.data(), sizeof(int) * H->colidx.size());
  return EOLC_OK;
}

eolc_status eolc_forces_fill(eolc_ctx *ctx, const double *x_h,
                             const double *X_h, const eolc_material *mat,
                             const double grav[3], double h, int precision,
                             double *f_h, double *M_h, double *MDK_h) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if (!x_h || !X_h || !mat || !grav) return fail(ctx, EOLC_BAD_ARG, "null input");
  if (precision != EOLC_PREC_FP64 && precision != EOLC_PREC_MIXED)
    return fail(ctx, EOLC_BAD_ARG, "unknown precision");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  int N = ctx->topo.n_nodes;
  size_t nb9 = size_t(ctx->topo.n_blocks) * 9;
  if ((st = upload_positions(ctx, x_h, X_h, s)) != EOLC_OK) return st;
  st = assemble(ctx, *mat, grav, h, precision, M_h != nullptr, false, s);
  if (st != EOLC_OK) return st;
  if (f_h) EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(f_h, ctx->f.p, sizeof(double) * 3 * N,
                                                cudaMemcpyDeviceToHost, s));
  if (M_h) EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(M_h, ctx->Mblk.p, sizeof(double) * nb9,
                                                cudaMemcpyDeviceToHost, s));
  std::vector<float> tmp;
  if (MDK_h) {
    if (precision == EOLC_PREC_FP64) {
      EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(MDK_h, ctx->A64.p, sizeof(double) * nb9,
                                           cudaMemcpyDeviceToHost, s));
    } else {
      tmp.resize(nb9);
      EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(tmp.data(), ctx->A32.p, sizeof(float) * nb9,
                                           cudaMemcpyDeviceToHost, s));
    }
  }
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  if (MDK_h && precision != EOLC_PREC_FP64)
    for (size_t k = 0; k < nb9; ++k) MDK_h[k] = tmp[k];
  ctx->last_precision = precision;
  return EOLC_OK;
}

eolc_status eolc_velocity_solve(eolc_ctx *ctx, const double *b_h,
                                const int *fixed_dofs_h, const double *beq_h,
                                int n_fixed, const eolc_solve_opts *opts,
                                double *v_h, eolc_solve_info *info) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = check_opts(ctx, opts)) != EOLC_OK) return st;
  if (!b_h || !v_h || (n_fixed > 0 && !beq_h)) return fail(ctx, EOLC_BAD_ARG, "null input");
  if (ctx->last_precision < 0) return fail(ctx, EOLC_BAD_ARG, "no matrix assembled");
  if (opts->precision != ctx->last_precision)
    return fail(ctx, EOLC_BAD_ARG, "solve precision differs from the assembled matrix");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  int n = 3 * ctx->topo.n_nodes;
  if ((st = set_pins(ctx, fixed_dofs_h, nullptr, n_fixed, s)) != EOLC_OK) return st;
  std::vector<double> beq_full(n, 0.0);
  for (int k = 0; k < n_fixed; ++k) beq_full[fixed_dofs_h[k]] = beq_h[k];
  EOLC_CHECK_CUDA(ctx, ctx->beq_full.upload(beq_full.data(), n, s));
  EOLC_CHECK_CUDA(ctx, ctx->b.upload(b_h, n, s));
  EOLC_CHECK_CUDA(ctx, ctx->v.upload(v_h, n, s));  // initial guess
  st = solve_device(ctx, opts, info, s);
  EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(v_h, ctx->v.p, sizeof(double) * n,
                                       cudaMemcpyDeviceToHost, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  return st;
}

eolc_status eolc_state_upload(eolc_ctx *ctx, const double *x_h,
                              const double *X_h, const double *v_h) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = refuse_eol(ctx)) != EOLC_OK) return st;
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  int N = ctx->topo.n_nodes;
  if (x_h) EOLC_CHECK_CUDA(ctx, ctx->x.upload(x_h, size_t(N) * 3, s));
  if (X_h) EOLC_CHECK_CUDA(ctx, ctx->X.upload(X_h, size_t(N) * 2, s));
  if (v_h) EOLC_CHECK_CUDA(ctx, ctx->v.upload(v_h, size_t(N) * 3, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  return EOLC_OK;
}

eolc_status eolc_state_download(eolc_ctx *ctx, double *x_h, double *v_h) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = refuse_eol(ctx)) != EOLC_OK) return st;
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  int N = ctx->topo.n_nodes;
  if (x_h) EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(x_h, ctx->x.p, sizeof(double) * 3 * N,
                                                cudaMemcpyDeviceToHost, s));
  if (v_h) EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(v_h, ctx->v.p, sizeof(double) * 3 * N,
                                                cudaMemcpyDeviceToHost, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  return EOLC_OK;
}

eolc_status eolc_step_resident(eolc_ctx *ctx, int n_steps,
                               const eolc_material *mat, const double grav[3],
                               double h, const int *fixed_dofs_h,
                               const double *fixed_vel_h, int n_fixed,
                               const eolc_solve_opts *opts,
                               eolc_solve_info *info) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = refuse_eol(ctx)) != EOLC_OK) return st;
  if ((st = check_opts(ctx, opts)) != EOLC_OK) return st;
  if (!mat || !grav || n_steps < 0) return fail(ctx, EOLC_BAD_ARG, "bad step arguments");
  if (n_fixed > 0 && (!fixed_dofs_h || !fixed_vel_h)) return fail(ctx, EOLC_BAD_ARG, "null fixed list");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  int n = 3 * ctx->topo.n_nodes;
  if ((st = set_pins(ctx, fixed_dofs_h, fixed_vel_h, n_fixed, s)) != EOLC_OK) return st;
  eolc_solve_info agg{};
  for (int k = 0; k < n_steps; ++k) {
    // pins from the velocity of the previous step (Constraints.cpp:472-496)
    EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->beq_full.p, 0, sizeof(double) * n, s));
    if (n_fixed > 0) {
      pins_kernel<<<(n_fixed + 127) / 128, 128, 0, s>>>(n_fixed, ctx->fixed_dofs.p,
                                                       ctx->fixed_vel.p, ctx->v.p,
                                                       ctx->beq_full.p);
      ctx->launches += 1;
    }
    if (!ctx->ev[0]) { cudaEventCreate(&ctx->ev[0]); cudaEventCreate(&ctx->ev[1]); }
    cudaEventRecord(ctx->ev[0], s);
    st = assemble(ctx, *mat, grav, h, opts->precision, false, true, s);
    if (st != EOLC_OK) return st;
    cudaEventRecord(ctx->ev[1], s);
    ctx->last_precision = opts->precision;
    eolc_solve_info si{};
    st = solve_device(ctx, opts, &si, s);
    float ams = 0.f;
    cudaEventElapsedTime(&ams, ctx->ev[0], ctx->ev[1]);  // the solve synchronized
    agg.iterations += si.iterations;
    agg.refinements += si.refinements;
    agg.used_fallback |= si.used_fallback;
    agg.rel_res = si.rel_res;
    agg.status = si.status;
    agg.solve_kernel_ms += si.solve_kernel_ms;
    agg.assemble_ms += ams;
    if (st != EOLC_OK) {
      if (info) *info = agg;
      return st;
    }
    integrate_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, h, ctx->v.p, ctx->x.p);
    ctx->launches += 1;
  }
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  if (info) *info = agg;
  return EOLC_OK;
}

eolc_status eolc_step(eolc_ctx *ctx, double *x_h, const double *X_h,
                      double *v_h, const eolc_material *mat,
                      const double grav[3], double h,
                      const int *fixed_dofs_h, const double *fixed_vel_h,
                      int n_fixed, const eolc_solve_opts *opts,
                      eolc_solve_info *info) {
  if (!x_h || !X_h || !v_h) return fail(ctx, EOLC_BAD_ARG, "null state");
  eolc_status st = eolc_state_upload(ctx, x_h, X_h, v_h);
  if (st != EOLC_OK) return st;
  st = eolc_step_resident(ctx, 1, mat, grav, h, fixed_dofs_h, fixed_vel_h,
                          n_fixed, opts, info);
  if (st != EOLC_OK) return st;
  return eolc_state_download(ctx, x_h, v_h);
}

eolc_status eolc_step_contacts(eolc_ctx *ctx, double *x_h, const double *X_h, double *v_h,
                               const eolc_material *mat, const double grav[3], double h,
                               const int *fixed_dofs_h, const double *fixed_vel_h, int n_fixed,
                               const eolc_box *boxes, int n_boxes, const double *points_h,
                               const double *normals_h, int n_points, double threshold,
                               const eolc_solve_opts *opts, eolc_ineq_info *info) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = refuse_eol(ctx)) != EOLC_OK) return st;
  if ((st = check_opts(ctx, opts)) != EOLC_OK) return st;
  if (!x_h || !X_h || !v_h || !mat || !grav) return fail(ctx, EOLC_BAD_ARG, "null state");
  if (n_fixed > 0 && (!fixed_dofs_h || !fixed_vel_h)) return fail(ctx, EOLC_BAD_ARG, "null fixed list");
  if ((st = eolc_state_upload(ctx, x_h, X_h, v_h)) != EOLC_OK) return st;
  cudaStream_t s = stream_of(ctx);
  const int N = ctx->topo.n_nodes, n = 3 * N;
  // Constraints::fill: pins from the previous velocity (Constraints.cpp:
  // 472-496), CD2 on the step's positions and its rows (:422-468)
  if ((st = set_pins(ctx, fixed_dofs_h, fixed_vel_h, n_fixed, s)) != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->beq_full.p, 0, sizeof(double) * n, s));
  if (n_fixed > 0) {
    pins_kernel<<<(n_fixed + 127) / 128, 128, 0, s>>>(n_fixed, ctx->fixed_dofs.p, ctx->fixed_vel.p,
                                                     ctx->v.p, ctx->beq_full.p);
    ctx->launches += 1;
  }
  std::vector<eolc_contact> cons(size_t(4) * N + 64);
  int nc = 0;
  st = eolc_cd2(ctx, x_h, boxes, n_boxes, points_h, normals_h, n_points, threshold, cons.data(),
                int(cons.size()), &nc);
  if (st == EOLC_CAPACITY) {
    cons.resize(nc);
    st = eolc_cd2(ctx, x_h, boxes, n_boxes, points_h, normals_h, n_points, threshold,
                  cons.data(), nc, &nc);
  }
  if (st != EOLC_OK) return st;
  std::vector<int> ptr(nc + 1), col(size_t(9) * std::max(1, nc));
  std::vector<double> val(size_t(9) * std::max(1, nc)), d(std::max(1, nc));
  int m = 0;
  if ((st = eolc_contact_rows(cons.data(), nc, nc, ptr.data(), col.data(), val.data(), d.data(),
                              &m)) != EOLC_OK)
    return fail(ctx, st, "contact rows");
  // Forces::fill, then the QP (GeneralizedSolver::velocitySolve), x += h v
  if ((st = assemble(ctx, *mat, grav, h, opts->precision, false, true, s)) != EOLC_OK) return st;
  ctx->last_precision = opts->precision;
  // warm start: a contact present at the previous step (same obstacle,
  // kind and vertices) starts from that step's multiplier
  std::vector<std::array<int, 9>> keys;
  keys.reserve(m);
  for (int k = 0; k < nc; ++k) {
    const eolc_contact &c = cons[k];
    const bool row = (c.count1 == 3 && c.count2 == 1) || (c.count1 == 2 && c.count2 == 2) ||
                     (c.count1 == 1 && c.count2 == 3);  // the kinds eolc_contact_rows keeps
    if (!row) continue;
    keys.push_back({c.source, c.count1, c.count2, c.verts1[0], c.verts1[1], c.verts1[2],
                    c.verts2[0], c.verts2[1], c.verts2[2]});
  }
  std::vector<double> lam0(std::max(1, m), 0.0), lam(std::max(1, m), 0.0);
  for (int i = 0; i < m; ++i) {
    auto it = ctx->contact_lambda.find(keys[i]);
    if (it != ctx->contact_lambda.end()) lam0[i] = it->second;
  }
  st = ineq_solve_device(ctx, m, ptr.data(), col.data(), val.data(), d.data(), opts, lam.data(),
                         info, lam0.data());
  if (st != EOLC_OK) return st;
  ctx->contact_lambda.clear();
  for (int i = 0; i < m; ++i)
    if (lam[i] > 0) ctx->contact_lambda[keys[i]] = lam[i];
  integrate_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, h, ctx->v.p, ctx->x.p);
  ctx->launches += 1;
  return eolc_state_download(ctx, x_h, v_h);
}

eolc_status eolc_step_eol(eolc_ctx *ctx, double *x_h, double *u_h, double *v_h,
                          const eolc_material *mat, const double grav[3], double h,
                          const int *fixed_dofs_h, const double *fixed_vel_h, int n_fixed,
                          const eolc_rows *eq, const eolc_rows *ineq,
                          const eolc_solve_opts *opts, eolc_ineq_info *info) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if ((st = check_opts(ctx, opts)) != EOLC_OK) return st;
  if (!x_h || !u_h || !v_h || !mat || !grav) return fail(ctx, EOLC_BAD_ARG, "null state");
  if (n_fixed > 0 && (!fixed_dofs_h || !fixed_vel_h)) return fail(ctx, EOLC_BAD_ARG, "null fixed list");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  const DevTopology &T = ctx->topo;
  const int n = 3 * T.n_nodes;
  if ((st = ensure_state(ctx)) != EOLC_OK) return st;
  if ((st = upload_positions(ctx, x_h, u_h, s)) != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, ctx->v.upload(v_h, n, s));
  // pins from the current velocity (Constraints.cpp:472-496)
  if ((st = set_pins(ctx, fixed_dofs_h, fixed_vel_h, n_fixed, s)) != EOLC_OK) return st;
  EOLC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->beq_full.p, 0, sizeof(double) * n, s));
  if (n_fixed > 0) {
    pins_kernel<<<(n_fixed + 127) / 128, 128, 0, s>>>(n_fixed, ctx->fixed_dofs.p, ctx->fixed_vel.p,
                                                     ctx->v.p, ctx->beq_full.p);
    ctx->launches += 1;
  }
  // Forces::fill with the EOL branches and b = -(M v + h f) (Cloth.cpp:345)
  if ((st = assemble(ctx, *mat, grav, h, opts->precision, false, true, s)) != EOLC_OK) return st;
  ctx->last_precision = opts->precision;
  // the QP with the rows of Constraints::fill
  const QpRows none{0, nullptr, nullptr, nullptr, nullptr};
  const QpRows qe = eq ? QpRows{eq->n_rows, eq->ptr, eq->col, eq->val, eq->rhs} : none;
  const QpRows qi = ineq ? QpRows{ineq->n_rows, ineq->ptr, ineq->col, ineq->val, ineq->rhs} : none;
  st = qp_solve_device(ctx, qe, qi, opts, nullptr, nullptr, info);
  if (st != EOLC_OK) return st;
  const int items = std::max(3 * T.n_real, T.n_eol);
  integrate_eol_kernel<<<(items + 255) / 256, 256, 0, s>>>(
      T.n_real, T.n_eol, T.n_eol > 0 ? T.eol_node.p : nullptr, h, ctx->v.p, ctx->x.p, ctx->X.p);
  ctx->launches += 1;
  EOLC_CHECK_CUDA(ctx, cudaGetLastError());
  EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(x_h, ctx->x.p, sizeof(double) * 3 * T.n_real,
                                       cudaMemcpyDeviceToHost, s));
  EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(u_h, ctx->X.p, sizeof(double) * 2 * T.n_real,
                                       cudaMemcpyDeviceToHost, s));
  EOLC_CHECK_CUDA(ctx, cudaMemcpyAsync(v_h, ctx->v.p, sizeof(double) * n,
                                       cudaMemcpyDeviceToHost, s));
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  return EOLC_OK;
}

eolc_status eolc_clear_contact_multipliers(eolc_ctx *ctx) {
  if (!ctx) return EOLC_BAD_ARG;
  ctx->contact_lambda.clear();
  return EOLC_OK;
}

int eolc_batch_num_configs(void) { return batch_num_configs(); }

const char *eolc_batch_config_name(int config) {
  static std::vector<std::string> names;
  static std::mutex m;
  std::lock_guard<std::mutex> lock(m);
  if (names.empty())
    for (int c = 0; c < batch_num_configs(); ++c) names.push_back(batch_config_name(c));
  return (config >= 0 && config < int(names.size())) ? names[config].c_str() : "";
}

eolc_status eolc_set_instance_materials(eolc_ctx *ctx, const eolc_material *mats, int n_inst) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if (!mats || n_inst != int(ctx->node_off.size()) - 1)
    return fail(ctx, EOLC_BAD_ARG, "one material per instance is required");
  ctx->inst_mat.assign(mats, mats + n_inst);
  return EOLC_OK;
}

eolc_status eolc_batch_set_jacobi_reference(eolc_ctx *ctx, const int *iters_h, int n_inst) {
  eolc_status st = need_topology(ctx);
  if (st != EOLC_OK) return st;
  if (!iters_h || n_inst != int(ctx->node_off.size()) - 1)
    return fail(ctx, EOLC_BAD_ARG, "one reference per instance is required");
  if (!ctx->bwork || ctx->batch_config < 0)
    return fail(ctx, EOLC_BAD_ARG, "no batched step has prepared the batch yet");
  return batch_set_jacobi_reference(ctx->bwork, iters_h, n_inst, stream_of(ctx)) == EOLC_OK
             ? EOLC_OK
             : fail(ctx, EOLC_CUDA_ERROR, "reference upload failed");
}

eolc_status eolc_batch_set_config(eolc_ctx *ctx, int config) {
  if (!ctx) return EOLC_BAD_ARG;
  if (config < -1 || config >= batch_num_configs())
    return fail(ctx, EOLC_BAD_ARG, "unknown batch configuration");
  ctx->batch_config = config;
  return EOLC_OK;
}

eolc_status eolc_batch_autotune(eolc_ctx *ctx, const double grav[3], double h,
                                const int *fixed_dofs_h, const double *fixed_vel_h,
                                int n_fixed, const eolc_solve_opts *opts, int *chosen,
                                double *ms_h) {
  if (!ctx) return EOLC_BAD_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  eolc_status st = batch_begin(ctx, grav, h, fixed_dofs_h, fixed_vel_h, n_fixed, opts, s);
  if (st != EOLC_OK) return st;
  return batch_autotune(ctx, grav, h, opts, s, chosen, ms_h);
}

eolc_status eolc_step_batched(eolc_ctx *ctx, int n_steps, const double grav[3], double h,
                              const int *fixed_dofs_h, const double *fixed_vel_h,
                              int n_fixed, const eolc_solve_opts *opts,
                              eolc_solve_info *inst_info_h, eolc_batch_info *total) {
  if (!ctx) return EOLC_BAD_ARG;
  if (n_steps < 0) return fail(ctx, EOLC_BAD_ARG, "negative step count");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream_of(ctx);
  eolc_status st = batch_begin(ctx, grav, h, fixed_dofs_h, fixed_vel_h, n_fixed, opts, s);
  if (st != EOLC_OK) return st;
  if (ctx->batch_config < 0) {
    if ((st = batch_autotune(ctx, grav, h, opts, s, nullptr, nullptr)) != EOLC_OK) return st;
  }
  {
    PcgArgs a = batch_pcg_args(ctx, opts, ctx->v.p);
    if (opts->precond == EOLC_PC_LEARNED) a.precond = EOLC_PC_JACOBI;
    std::string msg;
    if ((st = batch_prepare(ctx->bwork, a, ctx->node_off, ctx->batch_config, s, msg)) != EOLC_OK)
      return fail(ctx, st, msg.c_str());
  }
  {
    // the assembly tiles must exist before a capture records the assembly
    const std::string msg = ensure_assembly_tiles(ctx->topo, opts->precision, s, ctx->launches);
    if (!msg.empty()) return fail(ctx, EOLC_CUDA_ERROR, msg.c_str());
  }
  if (opts->precond == EOLC_PC_LEARNED)
    return step_batched_learned(ctx, n_steps, grav, h, opts, inst_info_h, total, s);
  // the captured graph holds these values and device addresses
  std::vector<double> key = {double(opts->precision), double(opts->precond), opts->rel_tol,
                             double(opts->max_iter), h, grav[0], grav[1], grav[2],
                             double(ctx->n_fixed_dev), double(ctx->batch_config)};
  for (const void *p : {(const void *)ctx->fixed_dofs.p, (const void *)ctx->fixed_vel.p,
                        (const void *)ctx->pinned.p, (const void *)ctx->beq_full.p,
                        (const void *)ctx->A64.p, (const void *)ctx->A32.p,
                        (const void *)ctx->elem.p, (const void *)ctx->inst_matd.p,
                        (const void *)ctx->bwork})
    key.push_back(double(reinterpret_cast<uintptr_t>(p)));
  if (!ctx->bgraph || key != ctx->bgraph_key) {
    if (ctx->bgraph) cudaGraphExecDestroy(ctx->bgraph);
    ctx->bgraph = nullptr;
    const long long before = ctx->launches;
    EOLC_CHECK_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    st = enqueue_batch_step(ctx, grav, h, opts, s);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    ctx->bgraph_launches = int(ctx->launches - before);
    ctx->launches = before;
    if (st != EOLC_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail(ctx, EOLC_CUDA_ERROR, cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(&ctx->bgraph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      ctx->bgraph = nullptr;
      return fail(ctx, EOLC_CUDA_ERROR, cudaGetErrorString(ce));
    }
    ctx->bgraph_key = key;
  }
  if ((st = batch_reset_records(ctx->bwork, s)) != EOLC_OK)
    return fail(ctx, st, "record reset failed");
  if (!ctx->ev[2]) { cudaEventCreate(&ctx->ev[2]); cudaEventCreate(&ctx->ev[3]); }
  EOLC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  for (int k = 0; k < n_steps; ++k) EOLC_CHECK_CUDA(ctx, cudaGraphLaunch(ctx->bgraph, s));
  EOLC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
  ctx->launches += (long long)ctx->bgraph_launches * n_steps;
  EOLC_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
  return batch_results(ctx, n_steps, ms, s, inst_info_h, total);
}

}  // extern "C"
