// Internal declarations of libeolc (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/eolc.h"

namespace eolc {

// ---- device buffer --------------------------------------------------------
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t resize(size_t m) {
    if (m == n && p) return cudaSuccess;
    release();
    if (m == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, m * sizeof(T));
    if (e == cudaSuccess) n = m;
    return e;
  }
  cudaError_t upload(const T *h, size_t m, cudaStream_t s) {
    cudaError_t e = resize(m);
    if (e != cudaSuccess || m == 0) return e;
    return cudaMemcpyAsync(p, h, m * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

// Contribution code of one element to one 3x3 block:
//   bits 0-2: the block's column in the element, bits 3-5: its row — each a
//   local vertex (bits 0-1) plus kVirtual when it is that vertex's Eulerian
//   (EOL) node; bit 6: 0 = triangle (membrane + inertia), 1 = hinge
//   (bending); bits 7-30: element index.
constexpr int kHingeBit = 1 << 6;
constexpr int kVirtual = 4;
__host__ __device__ inline int contrib_code(int elem, bool hinge, int lrow,
                                            int lcol) {
  return (elem << 7) | (hinge ? kHingeBit : 0) | (lrow << 3) | lcol;
}

// ---- topology (device build, topology_gpu.cu; host mirror on demand) -------
struct HostTopology {
  int n_nodes = 0, n_tri = 0, n_hinge = 0, n_blocks = 0;
  std::vector<int> rowptr;   // n_nodes + 1
  std::vector<int> colidx;   // n_blocks
  std::vector<int> blk_row;  // n_blocks
  std::vector<int> diag;     // n_nodes: block index of (i, i)
  std::vector<int> cptr;     // n_blocks + 1
  std::vector<int> contrib;  // contribution codes, faces first then hinges
  std::vector<int> nf_ptr;   // n_nodes + 1
  std::vector<int> nf_list;  // (face << 2) | local vertex
};

// ---- device state -----------------------------------------------------------
// n_nodes rows of the BSR pattern: the n_real mesh nodes, then one Eulerian
// node per EOL node (n_eol; its two Eulerian DOFs and a padded third that
// the solves pin).  eol[node] = EoL_index or -1 (n_real entries) and
// eol_node[k] = the node of EoL_index k, both only when n_eol > 0.
struct DevTopology {
  int n_nodes = 0, n_tri = 0, n_hinge = 0, n_blocks = 0, n_real = 0, n_eol = 0;
  DevBuf<int> tri, hinge, rowptr, colidx, blk_row, diag, cptr, contrib,
      nf_ptr, nf_list, eol, eol_node;
  DevBuf<int> nh_ptr, nh_list;  // node -> hinges (hinge << 2 | local vertex), n_real rows
  // Row tiles of the shared-memory assembly (assemble.cu), per element size
  // (0: FP32, 1: FP64), built on first use: tile boundaries (block rows) and
  // the tile-local shared-memory slot of every contribution (parallel to
  // contrib; bit 15 set for a triangle's).  atiles: tile count, -1 not built,
  // 0 when some row does not fit a tile (the two-pass assembly runs).
  // atask_f/h: each tile's triangle / hinge entries of nf_list / nh_list
  // reordered by local vertex (the warps of a tile then run one specialised
  // row evaluation each); apos_f/h: an entry's position in that order.
  int atiles[2] = {-1, -1};
  DevBuf<int> atile_row[2], atask_f[2], atask_h[2], apos_f[2], apos_h[2];
  DevBuf<unsigned short> aslot[2];
};

struct MaterialD {
  double rho, mu, lam, beta, dh2;  // dh2 = damping_b * h * h
  double g[3];
  double h;
};

// Device build of the same arrays (topology_gpu.cu) from device triangles
// and hinges; T.tri / T.hinge are not touched.  "" on success.
struct TopoScratch;
void free_topo_scratch(TopoScratch *w);
// n_eol > 0: T.eol / T.eol_node hold the EOL tables already (device).
std::string build_topology_device(TopoScratch *&w, int N, const int *tri_d, int n_tri,
                                  const int *hinge_d, int n_hinge, DevTopology &T,
                                  cudaStream_t s, long long &launches, int n_eol = 0);

// CD2's edge list (createEdges, boxTriCollision.cpp:141-231) built on the
// device (topology_gpu.cu): per edge (v0, v1, face, twin face or -1) in the
// reference's order; n_edges gets the count.  "" on success.
struct EdgeScratch;
void free_edge_scratch(EdgeScratch *w);
std::string build_edges_device(EdgeScratch *&w, const int *tri_d, int nf, DevBuf<int4> &edges,
                               int &n_edges, cudaStream_t s, long long &launches);

// Kernel launchers (assemble.cu).  mats/node_inst (both device, may be
// null): per-instance material table and the instance of every node, used
// instead of m for batched topologies.
// elem: device scratch of assemble_scratch_bytes(T, prec) for the element
// blocks.  Launches the triangle pass, the hinge pass and the block gather.
// Returns the number of kernels launched: two (per-step inputs, then the
// shared-memory tiled assembly) on non-EOL topologies whose tiles are built,
// else the two-pass path's three (two without hinges).
int launch_assemble_blocks(const DevTopology &T, const double *x,
                           const double *X, const MaterialD &m,
                           const MaterialD *mats, const int *node_inst,
                           int prec, void *elem, double *A64, float *A32, double *Mblk,
                           cudaStream_t s);
// Builds T's row tiles for precision prec if they are not built yet (a no-op
// for EOL topologies).  "" on success.
std::string ensure_assembly_tiles(DevTopology &T, int prec, cudaStream_t s, long long &launches);
size_t assemble_scratch_bytes(const DevTopology &T, int prec);
// Forces and right-hand side, always in FP64 (the FP64 refinement residual
// of the mixed-precision solve is only as accurate as b): a triangle pass and
// a node gather (two launches).  elem: the assembly scratch of
// assemble_scratch_bytes(T, prec); the force words sit after the blocks.
void launch_forces_rhs(const DevTopology &T, const double *x, const double *X,
                       const double *v, const MaterialD &m,
                       const MaterialD *mats, const int *node_inst, int prec, void *elem,
                       double *f, double *b, cudaStream_t s);

// b = -(M v + h f) from the assembled FP64 M blocks (EOL topologies).
void launch_bsr_rhs(const DevTopology &T, const double *Mblk, const double *v, const double *f,
                    double h, double *b, cudaStream_t s);

// Solver (pcg.cu)
struct SolveWork;
struct PcgArgs {
  const DevTopology *T;
  const double *A64;  // may be null in mixed mode (A32 promoted instead)
  const float *A32;
  const double *b;    // 3N rhs of the unconstrained system (b of Cloth.cpp)
  const uint8_t *pinned;  // 3N mask
  const double *beq_full; // 3N: beq on pinned DOFs, 0 elsewhere
  double *v;          // 3N in: guess, out: solution
  int precision, precond;
  double rel_tol;
  int max_iter;
  const float *learned;  // learned approximate inverse blocks (n_blocks*9)
  const double *X = nullptr;  // material coordinates (2N, device; optional):
                              // partition hint for the resident solvers
  long long spin_limit = 0;   // polls before a device wait gives up (0: default)
};
eolc_status run_pcg(SolveWork *&w, const PcgArgs &a, eolc_solve_info *info,
                    cudaStream_t s, std::string &err, long long &launches);
void free_solve_work(SolveWork *w);

// Batched solver (batch.cu): one persistent launch over many instances.
// Per-instance record, accumulated over the launches of one call.
struct BatchRecord {
  int status;          // first non-OK status, else EOLC_OK
  int iterations;      // summed over launches
  int refinements;
  int max_iterations;  // largest single-launch iteration count
  int steps;           // launches that solved this instance
  int used_fallback;   // a learned solve of this instance fell back to Jacobi
  double rel_res;      // largest final relative residual
};
struct BatchSolveWork;
void free_batch_work(BatchSolveWork *w);
int batch_num_configs();
std::string batch_config_name(int config);
// Builds the per-instance tiling for a configuration (host work and device
// allocations; not capturable).  node_off: n_inst + 1 node offsets.
eolc_status batch_prepare(BatchSolveWork *&w, const PcgArgs &a,
                          const std::vector<int> &node_off, int config,
                          cudaStream_t s, std::string &err);
// Enqueues set-up, the batched CG launch and the finish kernel on s; no
// synchronisation and no allocation, so it can be captured in a graph.
eolc_status batch_enqueue(BatchSolveWork *w, const PcgArgs &a, cudaStream_t s,
                          std::string &err, long long &launches);
// Learned batched solve (mixed precision, a prepared Jacobi configuration):
// the learned launch with per-instance caps of fallback_factor x each
// instance's last Jacobi count, then one Jacobi launch over the instances it
// left unconverged (node_inst: instance of every node, device).
eolc_status batch_enqueue_learned(BatchSolveWork *w, const PcgArgs &a, const float *Gm,
                                  int fallback_factor, const int *node_inst, cudaStream_t s,
                                  std::string &err, long long &launches);
eolc_status batch_reset_records(BatchSolveWork *w, cudaStream_t s);
eolc_status batch_set_jacobi_reference(BatchSolveWork *w, const int *iters_h, int n,
                                       cudaStream_t s);
eolc_status batch_read_records(BatchSolveWork *w, std::vector<BatchRecord> &out,
                               cudaStream_t s);

// Resident solvers (patch.cu), mixed precision only: the matrix is held in
// shared memory for the whole solve.  kJacobi: point / block Jacobi per
// a.precond; kPatch: the patch-local Chebyshev preconditioner of the given
// degree; kLearned: the learned approximate inverse Gm (original block order;
// nullptr reuses the G of the previous learned solve on this topology).
enum class ResidentPC { kJacobi, kPatch, kLearned };
struct PatchWork;
void free_patch_work(PatchWork *w);
// The next resident solve updates the coarse inverse (eolc_set_coarse_refresh).
void coarse_update_next(PatchWork *w);
bool resident_fits(PatchWork *&w, const DevTopology &T, const double *X_d, cudaStream_t s);
eolc_status run_pcg_resident(PatchWork *&w, const PcgArgs &a, ResidentPC mode, int degree,
                             const float *Gm, eolc_solve_info *info, cudaStream_t s,
                             std::string &err, long long &launches,
                             bool coarse = false, int coarse_refresh = 1);

// Collisions (collide.cu)
struct CollideWork;
void free_collide_work(CollideWork *w);

// OBJ export (export.cu)
struct ExportWork;
void free_export_work(ExportWork *w);

// Contact-constrained solve (contact.cu)
struct IneqWork;
void free_ineq_work(IneqWork *w);

// Learned preconditioner (learned.cu / pcg.cu)
eolc_status run_pcg_learned(SolveWork *&w, const PcgArgs &a, const float *Gm,
                            eolc_solve_info *info, cudaStream_t s, std::string &err,
                            long long &launches);

}  // namespace eolc

struct eolc_lpc;
namespace eolc {
// kernel launches of one learned_forward call
constexpr int kLearnedForwardLaunches = 10;
std::string learned_forward(eolc_lpc *P, eolc_ctx *ctx, const uint8_t *pinned_d,
                            const float **G_out, cudaStream_t s);
}

// Solve entry points shared by the C ABI functions (api.cu).
namespace eolc {
// Host copies of the device topology (and of the triangle list), downloaded
// on first use after a topology change; nullptr (with ctx->err set) on a
// CUDA error.
const HostTopology *host_topology(eolc_ctx *ctx);
// PcgArgs on the context's buffers (MDK, b, pins, v) for the options.
PcgArgs default_pcg_args(eolc_ctx *ctx, const eolc_solve_opts *o);
// The solver dispatch of eolc_velocity_solve on explicit arguments.
eolc_status solve_with_args(eolc_ctx *ctx, const eolc_solve_opts *o, const PcgArgs &a,
                            eolc_solve_info *info, cudaStream_t s);
// General rows of the QP in CSR over the DOFs of the topology's block rows.
struct QpRows {
  int m;
  const int *ptr, *col;
  const double *val, *rhs;
};
// The QP (contact.cu) with equality and inequality rows on the device state:
// MDK, b, pins, v (initial guess in, solution out); lambda0_h (optional):
// initial inequality multipliers.
eolc_status qp_solve_device(eolc_ctx *ctx, const QpRows &eq, const QpRows &iq,
                            const eolc_solve_opts *opts, double *lambda_eq_h,
                            double *lambda_h, eolc_ineq_info *info,
                            const double *lambda0_h = nullptr);
// The contact QP: qp_solve_device without equality rows.
eolc_status ineq_solve_device(eolc_ctx *ctx, int n_ineq, const int *ineq_ptr_h,
                              const int *ineq_col_h, const double *ineq_val_h,
                              const double *bineq_h, const eolc_solve_opts *opts,
                              double *lambda_h, eolc_ineq_info *info,
                              const double *lambda0_h = nullptr);
// Uploads the pinned DOFs, their values and the right-hand side b.
eolc_status prepare_pins_rhs(eolc_ctx *ctx, const double *b_h, const int *fixed_dofs_h,
                             const double *beq_h, int n_fixed, cudaStream_t s);
}  // namespace eolc

// ---- the context ------------------------------------------------------------
struct eolc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  bool has_topology = false;
  bool host_valid = false;     // host mirrors of the device topology are current
  eolc::HostTopology host;     // read through eolc::host_topology()
  eolc::TopoScratch *topo_work = nullptr;
  eolc::DevTopology topo;
  // state and per-step buffers
  eolc::DevBuf<double> x, X, v, f, b, A64, Mblk, beq_full;
  eolc::DevBuf<float> A32;
  eolc::DevBuf<unsigned char> elem;  // element blocks of the assembly
  eolc::DevBuf<uint8_t> pinned;
  eolc::DevBuf<int> fixed_dofs;
  eolc::DevBuf<double> fixed_vel;
  // the fixed list of the last upload (host copies), so that an unchanged
  // list is not rebuilt and uploaded again on every step
  std::vector<int> pin_dofs_h;
  std::vector<double> pin_vel_h;
  int n_fixed_dev = -1;
  eolc::SolveWork *work = nullptr;
  eolc::PatchWork *pwork = nullptr;
  int last_jacobi_iters = 0;
  int last_precision = -1;  // precision of the last assembled MDK
  long long launches = 0;   // kernels launched by this context
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // the FP64 force pass runs on aux beside the FP32 matrix passes
  cudaStream_t aux = nullptr;
  cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
  std::vector<int> host_tri;  // triangle list of the current topology
  // multipliers of the last eolc_step_contacts, by contact (source, kinds,
  // obstacle and cloth vertices): the next step's QP starts from them
  std::map<std::array<int, 9>, double> contact_lambda;
  eolc_lpc *lpc = nullptr;    // attached learned preconditioner (not owned)
  const eolc_lpc *lpc_cached = nullptr;  // network whose G the resident solver holds
  int lpc_uses = 0;           // solves that G has served
  int lpc_refresh = 1;        // re-evaluate the network every lpc_refresh solves
  int coarse_refresh = 1;     // rebuild the patch PC's coarse operator every ... solves
  long long spin_limit = 0;   // polls before a device wait gives up (0: the default)
  eolc::CollideWork *cd_work = nullptr;
  eolc::ExportWork *ex_work = nullptr;
  eolc::IneqWork *iq_work = nullptr;
  // batches: instance k owns nodes node_off[k] .. node_off[k+1]
  std::vector<int> node_off;
  eolc::DevBuf<int> node_inst;                // instance of every node
  std::vector<eolc_material> inst_mat;        // per-instance materials
  eolc::DevBuf<eolc::MaterialD> inst_matd;    // device table for a step
  std::vector<eolc::MaterialD> inst_matd_h;   // staging for that table
  eolc::BatchSolveWork *bwork = nullptr;
  int batch_config = -1;                      // -1: autotune on first use
  cudaGraphExec_t bgraph = nullptr;           // captured batched step
  std::vector<double> bgraph_key;             // what the graph was built for
  int bgraph_launches = 0;                    // kernels per replay
};

namespace eolc {
// Entry points that take positions or states of every block row (the plain
// and contact steps, export, batches, the plain contact QP) refuse
// topologies with EOL nodes, whose Eulerian rows have no positions of their
// own; eolc_cd2 runs on the mesh nodes and eolc_step_eol / the general QP
// take the extended layout.
inline eolc_status refuse_eol(eolc_ctx *ctx) {
  if (ctx && ctx->topo.n_eol > 0) {
    ctx->err = "not available on a topology with EOL nodes";
    return EOLC_BAD_ARG;
  }
  return EOLC_OK;
}
}  // namespace eolc
