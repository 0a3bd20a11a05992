/*
 * oracle.h — CPU restatement of the reference's hot path.  TEST
 * INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg call it to compare against.  The product library (libeolc.so)
 * never links, loads or calls anything here.
 *
 * Parity pins: the element routines are checked against the reference's own
 * ComputeMembrane/ComputeBending/ComputeInertial and intersect_triangle3_inc
 * compiled in place (oracle/build_ref.sh) through the golden vectors in
 * tests/golden/.  The assembly, solve and collision glue is a line-by-line
 * restatement of the reference's control flow and floating-point evaluation
 * order; the reference itself cannot be built here (Eigen 3.3.4 absent), so
 * that glue is pinned by restatement, not by reference outputs.
 *
 * All arithmetic is IEEE FP64 with FP contraction disabled
 * (-ffp-contract=off), so results are the same on x86-64 and aarch64.
 */
#ifndef EOLC_ORACLE_H_
#define EOLC_ORACLE_H_

#include "../include/eolc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- meshes -------------------------------------------------------------
 * corners: 4 x 5 doubles (x, y, z, X, Y) for p00, p01, p10, p11 in the
 * order load_defclothset parses them (parseParams.cpp:253-270). */

/* Two triangles per quad, (r0 x r1) nodes, node k = i*r1 + j placed as in
 * Cloth::build (Cloth.cpp:63-76); quad (k0, k0+1, k0+r1+1, k0+r1) split
 * along k0--k0+r1+1. */
void orc_grid2_build(int r0, int r1, const double *corners, double *x,
                     double *X, int *tri);
/* The reference's own centre-node grid (Cloth.cpp:63-126): r0*r1 + (r0-1)
 * (r1-1) nodes and 4 (r0-1)(r1-1) triangles. */
void orc_gridc_build(int r0, int r1, const double *corners, double *x,
                     double *X, int *tri);
/* Interior-edge hinges in ArcSim edge order (mesh.cpp:356-378,
 * Forces.cpp:687-697).  Returns the hinge count; writes at most cap. */
int orc_hinges(int n_nodes, const int *tri, int n_tri, int *hinge, int cap);

/* ---- elements (same I/O layout as the reference routines) -------------- */
void orc_face_frame(const double *x9, const double *X6, double *P6,
                    double *Q4);
void orc_membrane(const double *x9, const double *X6, double e, double nu,
                  const double *P6, const double *Q4, double *W, double *f9,
                  double *K81);
void orc_inertial(const double *x9, const double *X6, const double *g,
                  double rho, double *W, double *f9, double *M81);
void orc_bending(const double *x12, const double *X8, double beta, double *W,
                 double *f12, double *K144);
int orc_raytri(const double *orig, const double *dir, const double *v0,
               const double *v1, const double *v2, double *tuv);

/* ---- Forces::fill ------------------------------------------------------- */
typedef struct orc_forces orc_forces;
orc_forces *orc_forces_fill(int n_nodes, const double *x, const double *X,
                            const int *tri, int n_tri, const int *hinge,
                            int n_hinge, const eolc_material *mat,
                            const double *grav, double h);
void orc_forces_free(orc_forces *F);
/* which: 0 = M, 1 = MDK.  Scalar CSR of the 3N x 3N matrix. */
int orc_forces_nnz(const orc_forces *F, int which);
void orc_forces_csr(const orc_forces *F, int which, int *rowptr, int *col,
                    double *val);
void orc_forces_f(const orc_forces *F, double *f);

/* Forces::fill with EOL nodes (Forces.cpp:177-329, 399-497, 580-683,
 * 746-884): eol_index[node] = its EoL_index or -1; the system has
 * 3 n_nodes + 2 n_eol DOFs (Eulerian DOFs of EoL_index k at 3 N + 2 k).
 * Read it with orc_forces_nnz / orc_forces_csr / orc_forces_f. */
orc_forces *orc_forces_fill_eol(int n_nodes, const double *x, const double *X,
                                const int *tri, int n_tri, const int *hinge,
                                int n_hinge, const eolc_material *mat,
                                const double *grav, double h,
                                const int *eol_index, int n_eol);

/* b = -(M v + h f) (Cloth.cpp:345) */
void orc_rhs(const orc_forces *F, const double *v, double h, double *b);

/* Equality-constrained velocity solve with Eigen-style Jacobi CG on the
 * free DOFs (GeneralizedSolver.cpp:123-126 algorithm, rel tol on ||r||).
 * v_out gets the full 3N solution.  Returns iterations; *relres gets the
 * final ||r||/||b|| of the reduced system. */
int orc_velocity_solve(const orc_forces *F, const double *b,
                       const int *fixed_dofs, const double *beq, int n_fixed,
                       double tol, int max_iter, double *v_out,
                       double *relres);

/* Direct FP64 reference for the same reduced system (dense LDL^T on small
 * systems only, n_free <= 6000): the "truth" the CG results are measured against. */
int orc_velocity_solve_direct(const orc_forces *F, const double *b,
                              const int *fixed_dofs, const double *beq,
                              int n_fixed, double *v_out);

/* One Cloth::step (non-EOL): forces, pins, rhs, CG solve, x += h v.
 * Returns CG iterations. */
int orc_step(int n_nodes, double *x, const double *X, double *v,
             const int *tri, int n_tri, const int *hinge, int n_hinge,
             const eolc_material *mat, const double *grav, double h,
             const int *fixed_dofs, const double *fixed_vel, int n_fixed,
             double tol, int max_iter, double *relres);

/* ---- collisions ----------------------------------------------------------
 * CD2 (Collisions.cpp:55-78) with pointTriCollision then boxTriCollision per
 * box.  Returns the contact count; writes at most cap contacts. */
int orc_cd2(int n_nodes, const double *x, const int *tri, int n_tri,
            const eolc_box *boxes, int n_boxes, const double *points,
            const double *normals, int n_points, double threshold,
            eolc_contact *out, int cap);

/* createEdges (boxTriCollision.cpp:141-231): per edge (x0,x1,x2,x3,f0,f1)
 * in output order.  Returns the edge count. */
int orc_create_edges(int n_nodes, const double *x, const int *tri, int n_tri,
                     int *edges6, int cap);

/* ---- OBJ frame export (BrenderManager.cpp:34-84, Cloth.cpp:535-590) -----
 * The Cloth2D file then the Cloth3D file of one frame, as the reference's
 * sprintf calls write them (the 2D file's literal 0 z printed as 0.0), into
 * buf; len[0], len[1] get the two lengths.  buf == NULL: lengths only.
 * Returns 1 when cap is too small, else 0. */
int orc_obj_text(int n_nodes, const double *x, const double *X, const int *tri,
                 int n_tri, int frame, double time, char *buf, long long cap,
                 long long *len);
/* ArcSim normal<WS> of every node (geometry.cpp:302-316), FP64. */
void orc_node_normals(int n_nodes, const double *x, const int *tri, int n_tri,
                      double *out);

#ifdef __cplusplus
}
#endif
#endif
