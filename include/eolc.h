/*
 * eolc.h — C ABI of the GB300-native EOL-Cloth hot path.
 *
 * One library (libeolc.so) replaces, for the non-remeshing path:
 *   Forces::fill                     src/Forces.cpp:912-930   (Forces.h:40)
 *   GeneralizedSolver::velocitySolve src/GeneralizedSolver.cpp:107-173
 *                                    (GeneralizedSolver.h:26-30): pinned DOFs,
 *                                    and the contact QP with inequality rows
 *   Constraints::fill contact rows   src/Constraints.cpp:422-468
 *   Cloth::solve / Cloth::step       src/Cloth.cpp:343-413 (minus dumps),
 *                                    with or without contacts
 *   Forces::fill EOL branches        src/Forces.cpp:127-329, 399-497,
 *                                    541-683, 746-884
 *   Constraints::fill EOL rows and   src/Constraints.cpp:135-468,
 *   Cloth::step of EOL meshes        src/Cloth.cpp:359-413 (no remeshing)
 *   CD2 / btc::boxTriCollision /     src/Collisions.cpp:55-78,
 *   btc::pointTriCollision           src/boxTriCollision.cpp:602-1224
 *   BrenderManager::exportBrender /  src/BrenderManager.cpp:34-84,
 *   Cloth::exportBrender (OBJ)       src/Cloth.cpp:535-590
 *
 * Conventions
 *   - Plain pointers and sizes only.  Arrays suffixed _h are HOST memory
 *     (caller-owned); arrays suffixed _d are DEVICE memory on the context's
 *     device.  Positions are node-major: x[3*i + c].  Material coordinates
 *     are X[2*i + c] (ArcSim Vert::u, mesh.hpp:57-80, z dropped).
 *   - Every call returns an eolc_status; nothing throws or aborts.  The
 *     reference aborts on solver errors (GeneralizedSolver.cpp:139-168); this
 *     library reports them instead.  eolc_last_error() gives a message.
 *   - A context is bound to one device and one stream and is not reentrant.
 *   - Block-sparse matrices are 3x3 BSR in row-major block order; each block
 *     is 9 values, row-major inside the block.  The pattern is the union of
 *     node pairs sharing a triangle or a bending hinge, diagonal included,
 *     columns ascending within a block row.
 */
#ifndef EOLC_H_
#define EOLC_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  EOLC_OK = 0,
  EOLC_NOT_CONVERGED = 1, /* iteration cap reached before the tolerance   */
  EOLC_BREAKDOWN = 2,     /* p'Ap <= 0: matrix not positive definite       */
  EOLC_NONFINITE = 3,     /* NaN/Inf in inputs or iterates                 */
  EOLC_TIMEOUT = 4,       /* a bounded device wait gave up                  */
  EOLC_BAD_ARG = 5,
  EOLC_CUDA_ERROR = 6,
  EOLC_CAPACITY = 7,      /* output buffer too small; *n_out has the need  */
  EOLC_NO_TOPOLOGY = 8,
  EOLC_IO_ERROR = 9       /* a file could not be opened or written         */
} eolc_status;

/* Material of src/Cloth.h:28-35 (dampingA is unused by the reference). */
typedef struct {
  double density;   /* area density rho                      */
  double e;         /* Young's modulus                       */
  double nu;        /* Poisson's ratio                       */
  double beta;      /* bending stiffness                     */
  double damping_a; /* unused (kept for layout parity)       */
  double damping_b; /* stiffness damping: MDK = M + d_B h^2 K */
} eolc_material;

typedef enum {
  EOLC_PREC_FP64 = 0,  /* FP64 element math, FP64 BSR, FP64 PCG          */
  EOLC_PREC_MIXED = 1  /* FP32 matrix element math / BSR / PCG, FP64 dots,
                          FP64 forces and right-hand side, and an FP64
                          iterative-refinement residual                  */
} eolc_precision;

typedef enum {
  EOLC_PC_JACOBI = 0,       /* point Jacobi (Eigen's default for CG)     */
  EOLC_PC_BLOCK_JACOBI = 1, /* inverse of the 3x3 diagonal blocks        */
  EOLC_PC_LEARNED = 2,      /* learned block-sparse approximate inverse  */
  EOLC_PC_PATCH = 3         /* patch-local Chebyshev solves (below)      */
} eolc_precond;

typedef struct {
  double rel_tol;       /* stop when ||b - A v|| <= rel_tol ||b|| (FP64) */
  int max_iter;         /* total inner iterations allowed                */
  int precision;        /* eolc_precision                                */
  int precond;          /* eolc_precond                                  */
  int fallback_factor;  /* learned PC: fall back to Jacobi after
                           fallback_factor * (last Jacobi count) iterations;
                           0 disables the fallback                       */
  int degree;           /* patch PC: Chebyshev degree of the local solves
                           (0: 5)                                        */
  int streamed;         /* Jacobi / block Jacobi on the mixed path: 0 runs
                           the shared-memory-resident kernel when the mesh
                           fits (about 448 nodes per SM), 1 always streams
                           the matrix from memory tile by tile           */
  int no_coarse;        /* patch and learned PCs on the resident path: 0
                           adds the coarse-grid correction on aggregates
                           of patches (default), 1 runs the one-level
                           preconditioner                                */
} eolc_solve_opts;

/* Resident solves (mixed precision): the nodes are split by recursive
 * coordinate (or graph) bisection into one compact patch per SM (at most
 * about 448 nodes each); each SM holds its rows of the FP32 matrix in shared
 * memory for the whole solve and each row's vectors in one thread's
 * registers; every preconditioner runs as a single-grid-barrier
 * Chronopoulos-Gear PCG.
 * EOLC_PC_PATCH (resident only; no counterpart in the reference, whose solve
 * is Eigen's Jacobi CG, GeneralizedSolver.cpp:123-126): a two-level
 * preconditioner.  Local level: a degree-k Chebyshev polynomial of the
 * block-Jacobi-preconditioned, unit-diagonal-scaled principal submatrix of
 * each patch on [l/30, l], l an upper bound of its spectrum (symmetric
 * positive definite), applied with SM-local barriers.  Coarse level (unless
 * no_coarse): the translations of one aggregate per patch (or of compact
 * groups of patches), with the coarse matrix R A R^T assembled on the device
 * and its inverse updated there by Newton-Schulz iterations from the last
 * solve's (see eolc_set_coarse_refresh).  Every solve converges on the same
 * FP64 relative residual.  Meshes too large for the resident image stream the matrix
 * (Jacobi) or are rejected with EOLC_BAD_ARG (EOLC_PC_PATCH). */

typedef struct {
  int status;        /* eolc_status of the solve                          */
  int iterations;    /* inner PCG iterations (all restarts)               */
  int refinements;   /* FP64 true-residual recomputations                 */
  int used_fallback; /* 1 if the learned PC fell back to Jacobi           */
  double rel_res;    /* final FP64 ||b - A v|| / ||b|| on the free DOFs    */
  double solve_kernel_ms; /* device time of the PCG kernel(s), CUDA events */
  double assemble_ms;     /* device time of the assembly kernels          */
} eolc_solve_info;

typedef struct eolc_ctx eolc_ctx;

/* ---- lifetime ---------------------------------------------------------- */
eolc_status eolc_create(eolc_ctx **out, int device);
void eolc_destroy(eolc_ctx *ctx);
const char *eolc_last_error(const eolc_ctx *ctx);
/* stream is a cudaStream_t; NULL selects the context's own stream. */
eolc_status eolc_set_stream(eolc_ctx *ctx, void *stream);
int eolc_version(void);
/* Number of kernels this context has launched so far (telemetry). */
long long eolc_launch_count(const eolc_ctx *ctx);

/* ---- topology (Mesh::add(Face) adjacency, ArcSim mesh.cpp:356-378) -----
 * tri_h:   n_tri x 3 node indices, face vertex order as in Face::v[0..2].
 * hinge_h: n_hinge x 4 (x0, x1, x2, x3) for every edge with two adjacent
 *          faces, in mesh.edges order: x0 = edge->n[0], x1 = edge->n[1],
 *          x2 = other vertex of adjf[0], x3 = other vertex of adjf[1]
 *          (Forces.cpp:687-697).
 * Builds the BSR pattern and the per-block contribution lists once. */
eolc_status eolc_set_topology(eolc_ctx *ctx, int n_nodes, const int *tri_h,
                              int n_tri, const int *hinge_h, int n_hinge);
/* n_blocks = number of 3x3 blocks; rowptr_h has n_nodes + 1 entries. */
eolc_status eolc_bsr_pattern(eolc_ctx *ctx, int *n_blocks, int *rowptr_h,
                             int *colidx_h);

/* Topology refresh from device arrays (e.g. a remesher's output kept on the
 * GPU): same semantics and checks as eolc_set_topology (one instance), the
 * pattern, contribution lists and node -> face lists built on the device;
 * host copies are made only when a host-side routine needs them.  Every
 * eolc_set_topology* call builds on the device. */
eolc_status eolc_set_topology_device(eolc_ctx *ctx, int n_nodes,
                                     const int *tri_d, int n_tri,
                                     const int *hinge_d, int n_hinge);
/* Topology with EOL nodes (Forces.cpp:177-329, 399-497, 580-683, 746-884:
 * the EOL branches of Forces::fill).  eol_nodes_h[k] is the node of
 * EoL_index k.  The block rows are the n_nodes mesh nodes followed by one
 * Eulerian node per EOL node: its DOFs 0 and 1 are the reference's Eulerian
 * DOFs 3 n_nodes + 2k and + 1, DOF 2 is padding (zero in f, M and MDK except
 * a 1 on MDK's diagonal; every solve pins it).  On such a topology
 * eolc_forces_fill takes x_h (3 n_nodes) and X_h (2 n_nodes) and returns f
 * (3 (n_nodes + n_eol)), M and MDK over the extended rows, with the
 * reference's EOL blocks (-F' K, -K F, F' K F with the element's
 * deformation gradient; a hinge's F is the mean of its two faces') and
 * forces (-F' f on the Eulerian DOFs; a hinge with an EOL vertex also adds
 * its bending force); eolc_velocity_solve takes b, v and the fixed DOFs in
 * the extended layout; eolc_cd2 runs on the mesh nodes,
 * eolc_velocity_solve_qp takes the EOL rows of eolc_constraint_rows and
 * eolc_step_eol steps the mesh.  The other steps, export, batches and the
 * learned preconditioner refuse EOL topologies (EOLC_BAD_ARG). */
eolc_status eolc_set_topology_eol(eolc_ctx *ctx, int n_nodes, const int *tri_h,
                                  int n_tri, const int *hinge_h, int n_hinge,
                                  const int *eol_nodes_h, int n_eol);
/* The device topology for inspection: any array pointer may be NULL.
 * sizes: n_nodes, n_blocks, contributions, node -> face entries (3 n_tri).
 * rowptr/colidx: eolc_bsr_pattern's; cptr (n_blocks + 1) and contrib: the
 * element contributions of every block in the reference's insertion order
 * (faces ascending, then hinges; code = element << 7 | hinge << 6 |
 * row << 3 | column, row / column = local vertex, + 4 for its Eulerian
 * node); nf_ptr (n_nodes + 1) / nf_list: each
 * node's faces ascending, code face << 2 | local vertex. */
eolc_status eolc_topology_arrays(eolc_ctx *ctx, int *rowptr_h, int *colidx_h,
                                 int *cptr_h, int *contrib_h, int *nf_ptr_h,
                                 int *nf_list_h, int sizes[4]);

/* ---- Forces::fill (Forces.cpp:912-930, non-EOL branches) ----------------
 * Computes f (3N), M and MDK (BSR values, n_blocks*9 each) for positions
 * x_h and material coordinates X_h.  Any output pointer may be NULL.
 * precision selects FP64 or FP32 element arithmetic for M and MDK; f is
 * always evaluated in FP64 (near rest the FP32 membrane forces are rounding
 * noise of the size of the gravity loads).  Outputs are FP64. */
eolc_status eolc_forces_fill(eolc_ctx *ctx, const double *x_h,
                             const double *X_h, const eolc_material *mat,
                             const double grav[3], double h, int precision,
                             double *f_h, double *M_h, double *MDK_h);

/* ---- GeneralizedSolver::velocitySolve, pinned DOFs, no contacts ---------
 * Solves argmin 1/2 v'MDK v + b'v  s.t. v[fixed_dofs[k]] = beq[k]
 * (GeneralizedSolver.cpp:107-173 semantics with Aeq = unit rows,
 * Constraints.cpp:114-119) using the MDK of the last eolc_forces_fill /
 * eolc_step on this context.  v_h is the initial guess on input and the
 * solution on output (3N values). */
eolc_status eolc_velocity_solve(eolc_ctx *ctx, const double *b_h,
                                const int *fixed_dofs_h, const double *beq_h,
                                int n_fixed, const eolc_solve_opts *opts,
                                double *v_h, eolc_solve_info *info);

/* ---- GeneralizedSolver::velocitySolve with collisions --------------------
 * The QP that the reference hands Mosek or Gurobi (GeneralizedSolver.cpp:
 * 138-170; quadprog convention, QuadProg.h:8-9):
 *   argmin 1/2 v'MDK v + b'v  s.t.  v[fixed_dofs[k]] = beq[k],
 *                                   Aineq v <= bineq,
 * on the MDK of the last eolc_forces_fill / eolc_step.  Aineq: n_ineq rows
 * in CSR over the 3N DOFs (ineq_ptr_h: n_ineq + 1 offsets, ineq_col_h DOF
 * indices, ineq_val_h values; duplicates are summed).  A row may touch up to
 * four nodes, and every pair of them must share a triangle or a hinge (true
 * of the contact rows of Constraints.cpp:422-468; eolc_contact_rows builds
 * them), else EOLC_BAD_ARG.  Solved on the GPU by an augmented Lagrangian
 * with semismooth-Newton active sets; every linear solve is this library's
 * PCG with opts (precision, preconditioner, rel_tol), warm-started
 * (EOLC_PC_LEARNED runs as EOLC_PC_BLOCK_JACOBI here: the network
 * approximates the inverse of MDK, not of the contact-penalised matrix).  Stops
 * when the multipliers change by at most 10 rel_tol max|v| / rho (the
 * remaining infeasibility); EOLC_NOT_CONVERGED after 50 multiplier updates.
 * v_h: initial guess in, solution out (3N); lambda_h (n_ineq, may be NULL):
 * the inequality multipliers (>= 0, MDK v + b + Aineq' lambda = 0 on the
 * free DOFs, Mosek's getDualInequality). */
typedef struct {
  int status;           /* eolc_status of the solve                        */
  int solves;           /* linear solves (semismooth Newton steps)         */
  int outer;            /* multiplier updates                              */
  int iterations;       /* PCG iterations summed over the solves           */
  int n_active;         /* rows with lambda > 0 at the end                 */
  double max_violation; /* max(0, Aineq v - bineq) / max|v| at the end     */
  double rel_res;       /* relative residual of the last linear solve      */
  double solve_kernel_ms; /* device time of the PCG kernels, summed        */
  int fallbacks;        /* linear solves retried with block Jacobi after a
                           breakdown of the requested preconditioner       */
} eolc_ineq_info;
eolc_status eolc_velocity_solve_ineq(eolc_ctx *ctx, const double *b_h,
                                     const int *fixed_dofs_h,
                                     const double *beq_h, int n_fixed,
                                     int n_ineq, const int *ineq_ptr_h,
                                     const int *ineq_col_h,
                                     const double *ineq_val_h,
                                     const double *bineq_h,
                                     const eolc_solve_opts *opts, double *v_h,
                                     double *lambda_h, eolc_ineq_info *info);

/* Constraint rows in CSR over the DOFs of the context's block rows (a
 * topology with EOL nodes: the extended layout of eolc_set_topology_eol,
 * Eulerian DOF j of EOL node k at 3 (n_nodes + k) + j).  As input: n_rows,
 * ptr (n_rows + 1 offsets), col, val (duplicates are summed) and rhs (beq or
 * bineq per row).  As output of eolc_constraint_rows: capacity is the number
 * of rows the arrays hold (ptr capacity + 1 entries, col / val 9 capacity,
 * rhs capacity) and n_rows receives the count. */
typedef struct {
  int n_rows;
  int capacity;
  int *ptr;
  int *col;
  double *val;
  double *rhs;
} eolc_rows;

/* ---- GeneralizedSolver::velocitySolve with equality rows -----------------
 * The whole QP of GeneralizedSolver.cpp:138-170 (quadprog convention,
 * QuadProg.h:8-9):
 *   argmin 1/2 v'MDK v + b'v  s.t.  v[fixed_dofs[k]] = beq[k],
 *                                   Aeq v = beq_rows,  Aineq v <= bineq,
 * on the MDK of the last eolc_forces_fill, on plain and EOL topologies: the
 * rows Constraints::fill builds for an EOL mesh (eolc_constraint_rows) have
 * this form, and the pins stay a DOF list (addFixed's unit rows,
 * Constraints.cpp:114-119).  b_h, v_h: 3 x (block rows) values; a row on a
 * padded Eulerian DOF is EOLC_BAD_ARG.  Same method, stopping test and
 * options as eolc_velocity_solve_ineq, with every equality row always active
 * and its multiplier unclamped.  eq / ineq may be NULL (no rows).
 * lambda_eq_h (eq->n_rows) and lambda_ineq_h (ineq->n_rows) are optional:
 * MDK v + b + Aeq' lambda_eq + Aineq' lambda_ineq = 0 on the free DOFs.
 * info->max_violation covers |Aeq v - beq| as well. */
eolc_status eolc_velocity_solve_qp(eolc_ctx *ctx, const double *b_h,
                                   const int *fixed_dofs_h, const double *beq_h,
                                   int n_fixed, const eolc_rows *eq,
                                   const eolc_rows *ineq,
                                   const eolc_solve_opts *opts, double *v_h,
                                   double *lambda_eq_h, double *lambda_ineq_h,
                                   eolc_ineq_info *info);

/* ---- Cloth::step (Cloth.cpp:359-413, non-EOL, no remeshing, no QP) -----
 * One implicit-Euler step on host buffers: Forces::fill, pinned-corner
 * equality rows beq = 0.99 v + c (Constraints.cpp:114-119,472-496),
 * b = -(M v + h f) (Cloth.cpp:345), velocity solve, x += h v.
 * x_h and v_h (3N each) are updated in place.
 * fixed_dofs_h/fixed_vel_h: n_fixed DOF indices and their scripted
 * velocity offsets c(i+3). */
eolc_status eolc_step(eolc_ctx *ctx, double *x_h, const double *X_h,
                      double *v_h, const eolc_material *mat,
                      const double grav[3], double h,
                      const int *fixed_dofs_h, const double *fixed_vel_h,
                      int n_fixed, const eolc_solve_opts *opts,
                      eolc_solve_info *info);

/* Device-resident stepping: upload the state once, step n_steps times with
 * x, v kept in HBM, download when needed.  Same semantics as eolc_step. */
eolc_status eolc_state_upload(eolc_ctx *ctx, const double *x_h,
                              const double *X_h, const double *v_h);
eolc_status eolc_state_download(eolc_ctx *ctx, double *x_h, double *v_h);
eolc_status eolc_step_resident(eolc_ctx *ctx, int n_steps,
                               const eolc_material *mat, const double grav[3],
                               double h, const int *fixed_dofs_h,
                               const double *fixed_vel_h, int n_fixed,
                               const eolc_solve_opts *opts,
                               eolc_solve_info *info);

/* ---- batches: many independent sheets in one persistent launch -----------
 * No counterpart in the reference, whose Scene holds a single Cloth
 * (Scene.h:56) and steps it once per Scene::step (Scene.cpp:72-98).  Each instance
 * is a Cloth with its own material, stepped exactly as eolc_step_resident
 * steps one sheet; all instances share h and gravity.
 *
 * eolc_set_topology_batched: instance k owns nodes node_off_h[k] ..
 * node_off_h[k+1]-1, triangles tri_off_h[k] .. tri_off_h[k+1]-1 and hinges
 * hinge_off_h[k] .. hinge_off_h[k+1]-1 (each table has n_inst + 1 entries,
 * starting at 0); tri_h/hinge_h hold GLOBAL node indices (node_off + local)
 * and must not reference another instance's nodes.  The state arrays of
 * eolc_state_upload / eolc_state_download and the fixed DOF list are the
 * concatenation over instances.  eolc_set_topology is the one-instance case.
 */
eolc_status eolc_set_topology_batched(eolc_ctx *ctx, int n_inst,
                                      const int *node_off_h, const int *tri_h,
                                      const int *tri_off_h, const int *hinge_h,
                                      const int *hinge_off_h);
/* One material per instance (required before eolc_step_batched). */
eolc_status eolc_set_instance_materials(eolc_ctx *ctx,
                                        const eolc_material *mats, int n_inst);

typedef struct {
  int status;           /* first non-OK instance status (instance order)   */
  int n_failed;         /* instances whose solve did not reach EOLC_OK     */
  int config;           /* batched-solver configuration used               */
  int steps;
  long long iterations; /* PCG iterations summed over instances and steps  */
  int max_iterations;   /* largest iteration count of one instance solve   */
  int n_fallback;       /* instances whose learned solve fell back to Jacobi */
  double max_rel_res;   /* largest final FP64 relative residual            */
  double step_ms;       /* device time of the n_steps steps (CUDA events)  */
} eolc_batch_info;

/* n_steps implicit-Euler steps of every instance on the device-resident
 * state.  One step is one CUDA graph launch (captured on first use and
 * whenever h, gravity, the options, the pins or the configuration change):
 * pins, assembly with per-instance materials, ONE persistent launch of the
 * batched PCG (instances pulled from a work queue, largest first, one CTA
 * cluster each), x += h v.  Preconditioner: EOLC_PC_JACOBI,
 * EOLC_PC_BLOCK_JACOBI or EOLC_PC_LEARNED (mixed precision, a network attached):
 * the network's forward pass on the whole batch, one learned batched launch
 * in which each instance stops at fallback_factor x its last Jacobi iteration
 * count (uncapped until it has one), and one Jacobi launch over the
 * instances it left unconverged (a step per call is then not a single graph:
 * the forward pass synchronises).  inst_info_h (optional, n_inst entries): per-instance
 * status, iterations and refinements summed over the steps and the largest
 * relative residual.  Returns the first non-OK instance status; the other
 * instances' states are advanced regardless.  The first call on a topology
 * runs eolc_batch_autotune unless a configuration was set. */
eolc_status eolc_step_batched(eolc_ctx *ctx, int n_steps, const double grav[3],
                              double h, const int *fixed_dofs_h,
                              const double *fixed_vel_h, int n_fixed,
                              const eolc_solve_opts *opts,
                              eolc_solve_info *inst_info_h,
                              eolc_batch_info *total);
/* Batched-solver configurations: CTA shape (threads, threads per block row,
 * tile rows, CTAs per SM) x cluster size. */
int eolc_batch_num_configs(void);
const char *eolc_batch_config_name(int config);
/* Per-instance Jacobi iteration counts the learned batched solve's caps refer
 * to (set automatically by every converged batched Jacobi solve of an
 * instance); needs a prepared batch (one batched step or autotune). */
eolc_status eolc_batch_set_jacobi_reference(eolc_ctx *ctx, const int *iters_h,
                                            int n_inst);
/* Force a configuration (-1: autotune on the next batched step). */
eolc_status eolc_batch_set_config(eolc_ctx *ctx, int config);
/* Times every configuration on the current state (assembled once; the state
 * is not changed) and keeps the fastest.  ms_h (optional,
 * eolc_batch_num_configs entries): solve time per configuration, -1 where a
 * configuration does not fit the batch. */
eolc_status eolc_batch_autotune(eolc_ctx *ctx, const double grav[3], double h,
                                const int *fixed_dofs_h,
                                const double *fixed_vel_h, int n_fixed,
                                const eolc_solve_opts *opts, int *chosen,
                                double *ms_h);

/* ---- collisions (CD2, Collisions.cpp:55-78) ------------------------------ */

/* Box obstacle: full dimensions dim[3] (Box::dim) and 4x4 frame E1
 * (column-major, Box::E1). */
typedef struct {
  double dim[3];
  double E1[16];
} eolc_box;

/* One contact, mirroring btc::Collision (boxTriCollision.h:49-110). */
typedef struct {
  double dist;
  double nor1[3];
  double nor2[3];
  double pos1[3];
  double pos2[3];
  double pos1_[3];
  double weights1[3];
  double weights2[3];
  double edge_dir[3];
  int count1;
  int count2;
  int verts1[3];
  int verts2[3];
  int tri1;
  int tri2;
  int edge1[3];
  int n_edge1; /* 0, 1 or 3 entries of edge1 are valid */
  int edge2;
  int source;  /* 0: point obstacles, 1 + b: box b */
} eolc_contact;

/* Contact set of CD2 for the current topology: point obstacles first
 * (pointTriCollision, EOL=false), then each box in order
 * (boxTriCollision, EOL=false).  x_h: cloth node positions (3N; on a
 * topology with EOL nodes the N mesh nodes, as Collisions.cpp:55-78 packs
 * them).
 * points_h / normals_h: n_points x 3.  Writes at most capacity contacts;
 * *n_out receives the total count (EOLC_CAPACITY if it exceeds capacity). */
eolc_status eolc_cd2(eolc_ctx *ctx, const double *x_h, const eolc_box *boxes,
                     int n_boxes, const double *points_h,
                     const double *normals_h, int n_points, double threshold,
                     eolc_contact *out_h, int capacity, int *n_out);
/* The cloth edge list CD2 uses (createEdges, boxTriCollision.cpp:141-231),
 * built on the device once per topology: per edge (verts(0), verts(1),
 * face0, face1 or -1), 4 ints, in the reference's order (faces' edges
 * stably sorted by the 32-bit hash kmin + (3 n_tri + 1) kmax, twins
 * paired).  *n_edges gets the count; EOLC_CAPACITY when capacity (edges) is
 * smaller. */
eolc_status eolc_edge_list(eolc_ctx *ctx, int *edges_h, int capacity,
                           int *n_edges);
/* The inequality rows Constraints::fill builds from CD2 contacts of a
 * non-EOL mesh (Constraints.cpp:422-468), in contact order: box face /
 * cloth vertex -> -nor1 on the vertex; edge / edge -> -nor2 weights2[j] on
 * the two cloth vertices; box corner or point / cloth face -> -nor2
 * weights2[j] on the three cloth vertices; bineq = 0.  Other contact kinds
 * give no row.  Host only.  Writes at most cap_rows rows (ineq_ptr_h needs
 * cap_rows + 1 entries, ineq_col_h / ineq_val_h 9 cap_rows) and sets
 * *n_rows; EOLC_CAPACITY when cap_rows is too small. */
eolc_status eolc_contact_rows(const eolc_contact *contacts, int n_contacts,
                              int cap_rows, int *ineq_ptr_h, int *ineq_col_h,
                              double *ineq_val_h, double *bineq_h,
                              int *n_rows);

/* ---- Constraints::fill for an EOL mesh (Constraints.cpp:147-468) ---------
 * The mesh state Constraints::fill reads after EOL preprocessing: positions
 * (Node::x, 3 n_nodes), material coordinates (Vert::u, 2 n_nodes), faces
 * (Face::v, n_tri x 3), the edges in mesh.edges order (Edge::n[0], n[1],
 * n_edges x 2; Node::adje lists a node's edges in this order) with their
 * Edge::preserve flags (may be NULL: none), and per EoL_index k (as
 * eolc_set_topology_eol): the node, Node::cornerID (constraint-table column
 * of the box corner or point obstacle it sits on, or -1) and
 * Node::cdEdges[0] (the column of the box edge, read when cornerID < 0). */
typedef struct {
  int n_nodes;
  const double *x;
  const double *u;
  const int *tri;
  int n_tri;
  const int *edges;
  const int *preserve;
  int n_edges;
  const int *eol_nodes;
  const int *corner_id;
  const int *cd_edge;
  int n_eol;
} eolc_eol_mesh;

/* The equality and inequality rows of Constraints::fill, without the pins
 * (those stay a DOF list): for each EOL node in node order, the rows of
 * :147-415 — at a box corner or point obstacle the normal row (inequality)
 * and its two orthogonal rows (equalities where the node is locally flat or
 * at a point, else inequalities); on a box edge the node-normal inequality
 * and the flat equality, or the edge's two face rows; then one Eulerian
 * equality, across the border at a boundary node, along the preserved edges
 * inside — then the CD2 contact rows of :422-468 (eolc_contact_rows'),
 * skipping contacts on EOL nodes.  The constraint table (:40-105) comes from
 * the point obstacles' normals and the boxes: columns n_points + 20 b + p
 * (corner p) and n_points + 20 b + 8 + e (edge e), the numbering of
 * Box.cpp's tables.  box_velocity_h (may be NULL: boxes at rest): per box
 * Box::v, the angular then the linear velocity (6 values); a node on a
 * moving box gets the right-hand sides of :165-172 and :270-277 (its point's
 * velocity over the step h, Rigid::integrate, dotted with each row's
 * direction); every other right-hand side is 0.  Columns use the extended
 * layout (eolc_rows).  Host only.  EOLC_CAPACITY when eq or ineq is too small
 * (n_rows has the need). */
eolc_status eolc_constraint_rows(const eolc_eol_mesh *mesh, const eolc_box *boxes,
                                 const double *box_velocity_h, int n_boxes,
                                 const double *point_normals_h, int n_points,
                                 const eolc_contact *contacts, int n_contacts,
                                 double h, eolc_rows *eq, eolc_rows *ineq);

/* ---- Cloth::step with collisions (Cloth.cpp:359-413, non-EOL, no remesh) --
 * One implicit-Euler step with the contact QP, on host buffers like
 * eolc_step: pins beq = 0.99 v + c, CD2 of the step's positions against the
 * boxes and point obstacles (as eolc_cd2), the inequality rows of
 * Constraints.cpp:422-468 (eolc_contact_rows), Forces::fill, the QP of
 * eolc_velocity_solve_ineq warm-started from v and, for every contact that
 * the previous call on this context also had (same obstacle, kind and
 * vertices), from its multiplier, x += h v.  info (may be NULL) reports the
 * QP solve. */
/* Forgets the multipliers eolc_step_contacts carries to the next call (after
 * a jump in the scene, or to time cold QP solves). */
eolc_status eolc_clear_contact_multipliers(eolc_ctx *ctx);
eolc_status eolc_step_contacts(eolc_ctx *ctx, double *x_h, const double *X_h,
                               double *v_h, const eolc_material *mat,
                               const double grav[3], double h,
                               const int *fixed_dofs_h,
                               const double *fixed_vel_h, int n_fixed,
                               const eolc_box *boxes, int n_boxes,
                               const double *points_h,
                               const double *normals_h, int n_points,
                               double threshold, const eolc_solve_opts *opts,
                               eolc_ineq_info *info);

/* ---- Cloth::step of an EOL mesh (Cloth.cpp:359-413, no remeshing) --------
 * One implicit-Euler step on host buffers with the rows of Constraints::fill
 * given (eolc_constraint_rows on the step's state): pins beq = 0.99 v + c,
 * Forces::fill with the EOL branches, b = -(M v + h f), the QP of
 * eolc_velocity_solve_qp, x += h v on the mesh nodes and, for every EOL node,
 * u += h vE with its Eulerian velocity (Cloth.cpp:394-410).  x_h (3 n_nodes)
 * and u_h (2 n_nodes, the material coordinates X) are updated in place; v_h
 * has 3 x (block rows) values in the extended layout (the Eulerian
 * velocities at 3 (n_nodes + k)) and is updated in place.  Also runs on a
 * topology without EOL nodes (u is then unchanged). */
eolc_status eolc_step_eol(eolc_ctx *ctx, double *x_h, double *u_h, double *v_h,
                          const eolc_material *mat, const double grav[3],
                          double h, const int *fixed_dofs_h,
                          const double *fixed_vel_h, int n_fixed,
                          const eolc_rows *eq, const eolc_rows *ineq,
                          const eolc_solve_opts *opts, eolc_ineq_info *info);

/* ---- learned preconditioner ------------------------------------------------
 * A 3-layer message-passing network (hidden width 64, BF16 weights, FP32
 * accumulation) on the stencil of MDK that outputs the 3x3 blocks of a
 * symmetric positive definite approximate inverse
 *   G = F (Lambda + sum_e [U_e; V_e][U_e; V_e]^T) F
 * (F: free-DOF mask, Lambda: positive scaled Jacobi, one rank-3 PSD term per
 * stencil edge), applied inside PCG (EOLC_PC_LEARNED).  Inference runs the
 * dense layers on the tensor cores (tcgen05.mma, FP32 activations as three
 * BF16 terms); the resident solve streams G in BF16.  Trained on the GPU by
 * the library's own forward/backward kernels on systems the simulator
 * produces, minimising sum_k |F (G A w_k - w_k)|^2 / |F w_k|^2 over probe
 * vectors w_k.  The reference has no preconditioner beyond Eigen's default
 * Jacobi (GeneralizedSolver.cpp:123-126); point Jacobi stays the fallback
 * (eolc_solve_opts.fallback_factor) and the yardstick (same FP64 residual). */
typedef struct eolc_lpc eolc_lpc;
eolc_status eolc_lpc_create(eolc_lpc **out, int device, unsigned seed);
void eolc_lpc_destroy(eolc_lpc *lpc);
const char *eolc_lpc_last_error(const eolc_lpc *lpc);
int eolc_lpc_num_params(const eolc_lpc *lpc);
eolc_status eolc_lpc_get_params(eolc_lpc *lpc, float *params_h);
eolc_status eolc_lpc_set_params(eolc_lpc *lpc, const float *params_h);
/* Probe loss and its gradient w.r.t. the parameters for the context's last
 * FP32 MDK (eolc_forces_fill / eolc_step with EOLC_PREC_MIXED).
 * probes_h: n_probes x 3N FP32 vectors; grad_h: eolc_lpc_num_params floats. */
eolc_status eolc_lpc_loss_grad(eolc_lpc *lpc, eolc_ctx *ctx,
                               const int *fixed_dofs_h, int n_fixed,
                               const float *probes_h, int n_probes,
                               double *loss, float *grad_h);
/* Stores a copy of the context's current FP32 MDK, its pinned mask and the
 * probes as one training system (all systems share one topology). */
eolc_status eolc_lpc_add_system(eolc_lpc *lpc, eolc_ctx *ctx,
                                const int *fixed_dofs_h, int n_fixed,
                                const float *probes_h, int n_probes);
int eolc_lpc_num_systems(const eolc_lpc *lpc);
/* The approximate inverse G (n_blocks x 9 FP32 values, the BSR pattern of
 * MDK) the network produces for the context's current FP32 MDK with the
 * given pinned DOFs: the blocks EOLC_PC_LEARNED applies (the resident
 * solver applies them rounded to BF16). */
eolc_status eolc_lpc_blocks(eolc_lpc *lpc, eolc_ctx *ctx, const int *fixed_dofs_h,
                            int n_fixed, float *G_h);
eolc_status eolc_lpc_clear_systems(eolc_lpc *lpc);
/* Adam over the stored systems (seeded shuffle); epoch_loss_h[epochs]
 * receives the mean probe loss of each epoch. */
eolc_status eolc_lpc_train(eolc_lpc *lpc, int epochs, float lr, unsigned seed,
                           double *epoch_loss_h);
/* Attach (or detach with NULL) the network used by EOLC_PC_LEARNED solves on
 * this context; the context does not own it. */
eolc_status eolc_attach_preconditioner(eolc_ctx *ctx, eolc_lpc *lpc);
/* Evaluate the attached network every `solves` learned solves (default 1)
 * and keep its G in between (a lagged preconditioner: any symmetric positive
 * definite G leaves PCG exact, and the Jacobi fallback still bounds the
 * iterations).  Applies to the shared-memory-resident solve.  Every call
 * restarts the count: the next solve evaluates the network (as does
 * re-attaching one, eolc_attach_preconditioner). */
eolc_status eolc_set_learned_refresh(eolc_ctx *ctx, int solves);
/* Update the coarse operator of the two-level patch preconditioner (its
 * assembly and the Newton-Schulz update of its inverse) every `solves`
 * EOLC_PC_PATCH solves (default 1) and reuse it in between (a lagged coarse
 * correction: still symmetric positive definite, so PCG stays exact).  Every
 * call restarts the count: the next solve updates the coarse operator.  A
 * new topology starts the inverse again from its block-diagonal guess. */
eolc_status eolc_set_coarse_refresh(eolc_ctx *ctx, int solves);
/* Bound of every device-side wait of this context's solves: the grid
 * barriers of the persistent PCG kernels and the neighbour exchange of the
 * resident kernels poll at most `polls` times, then record EOLC_TIMEOUT;
 * every CTA of the launch then leaves (the others see the status or run out
 * of polls themselves) and the call returns EOLC_TIMEOUT with the context
 * still usable.  0 restores the default (2^25 polls, seconds).  The
 * reference has no device and no wait to bound; this is the library's
 * failure detection for a stalled SM (a small limit makes a healthy solve
 * report EOLC_TIMEOUT, which is how the tests exercise the path). */
eolc_status eolc_set_wait_limit(eolc_ctx *ctx, long long polls);
/* Iteration count of a plain Jacobi solve that the learned solve's fallback
 * cap (fallback_factor x this count) refers to; set automatically by every
 * successful Jacobi solve on the context. */
eolc_status eolc_set_jacobi_reference(eolc_ctx *ctx, int iterations);

/* ---- OBJ frame export (BrenderManager::exportBrender, BrenderManager.cpp:
 * 34-84, with Cloth::exportBrender, Cloth.cpp:535-590) --------------------
 * Writes the two files of one frame from the context's device state (the
 * positions and material coordinates of the last upload or step and the
 * topology's triangles):
 *   <dir>/<frame %06d>_Cloth2D.obj  "v u0 u1 0", "vt u0 u1", "vn 0 0 1"
 *   <dir>/<frame %06d>_Cloth3D.obj  "v x", "vt u0 u1", "vn n" (node normals
 *                                   of ArcSim normal<WS>, geometry.cpp:302-316)
 * each after the header "# frame %06d \n# time %f \n# name <name> \n" and
 * with 1-based faces "f a/a/a b/b/b c/c/c", numbers as C's "%f" prints them
 * (positions, texture coordinates and normals rounded to float first, as the
 * reference's posBuf/texBuf/norBuf).  The text is generated on the GPU.  The
 * caller keeps the frame counter (the reference's BrenderManager increments
 * it after every export).  EOLC_BAD_ARG when a coordinate has magnitude
 * 2^63 or more; EOLC_IO_ERROR when a file cannot be written. */
eolc_status eolc_export_obj(eolc_ctx *ctx, const char *dir, int frame,
                            double time);
/* The same two files' bytes into host memory: the Cloth2D file, then the
 * Cloth3D file, len[0] and len[1] bytes (no terminating NUL).  buf == NULL
 * returns the lengths only; EOLC_CAPACITY when capacity < len[0] + len[1]. */
eolc_status eolc_export_obj_text(eolc_ctx *ctx, int frame, double time,
                                 char *buf, size_t capacity, size_t len[2]);

/* ---- velocity solve without device allocation ----------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * on their step path: an interactive stepping loop (the reference's online
 * mode) cannot afford cudaMalloc/cudaFree, which may synchronize the device
 * and take milliseconds, and a host framework that reserves all device
 * memory in its own pool leaves none for a library allocator.
 * Same mixed-precision Jacobi PCG as eolc_velocity_solve (FP32 matrix and
 * vectors, double-float inner products, FP64 true residual <= rel_tol), with
 * every scratch buffer carved out of one fixed device array inside the
 * library (about 17 MB, held by every GPU that loads the library until the
 * process exits).  No context is needed and nothing is allocated on the
 * device.
 *   rowptr_h/colidx_h: the BSR pattern (host; eolc_bsr_pattern's layout),
 *   mdk_d: FP32 block values (device, 9 per block), b_d: the 3N right-hand
 *   side -(M v + h f) of the implicit-Euler step (device),
 *   fixed_dofs_h/beq_h: pinned DOFs and their values (host), v_d: 3N
 *   solution (device, written).
 * Limits: n_nodes <= EOLC_STATIC_MAX_NODES and n_blocks <=
 * EOLC_STATIC_MAX_BLOCKS, else EOLC_CAPACITY.  The first call on a device
 * looks up the array's device address with that device current.  The call
 * copies its tiling from host memory and synchronizes the stream, so it
 * cannot be made while the stream is being captured into a CUDA graph.
 * Every call shares the array and it keeps the
 * previous call's contents (the call clears what must start at zero), so
 * calls whose GPU work overlaps — two streams, or two threads — race and
 * must be serialized by the caller.  stream: a cudaStream_t (NULL: the
 * legacy default stream); the call synchronizes it before returning. */
#define EOLC_STATIC_MAX_NODES 16384
#define EOLC_STATIC_MAX_BLOCKS 262144
eolc_status eolc_velocity_solve_static(int n_nodes, const int *rowptr_h,
                                       const int *colidx_h, const float *mdk_d,
                                       const double *b_d,
                                       const int *fixed_dofs_h,
                                       const double *beq_h, int n_fixed,
                                       double rel_tol, int max_iter,
                                       double *v_d, eolc_solve_info *info,
                                       void *stream);

#ifdef __cplusplus
}
#endif
#endif /* EOLC_H_ */
