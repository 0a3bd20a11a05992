// Oracle Forces::fill / Cloth::solve / Cloth::step restatement (test
// infrastructure; see oracle.h).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

struct Trip {
  int r, c;
  double v;
};

// Eigen::SparseMatrix::setFromTriplets semantics: duplicates are summed in
// insertion order.  Output is scalar CSR with ascending columns.
struct Csr {
  int n = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
};

Csr from_triplets(int n, const std::vector<Trip> &t) {
  Csr m;
  m.n = n;
  std::vector<int> cnt(n + 1, 0);
  for (const Trip &x : t) cnt[x.r + 1]++;
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  // bucket by row, keeping insertion order (stable)
  std::vector<int> order(t.size());
  std::vector<int> pos(cnt.begin(), cnt.end() - 1);
  for (size_t k = 0; k < t.size(); ++k) order[pos[t[k].r]++] = int(k);
  m.rowptr.assign(n + 1, 0);
  std::vector<int> slot(n, -1);  // column -> position in current row
  for (int i = 0; i < n; ++i) {
    int start = int(m.col.size());
    for (int q = cnt[i]; q < cnt[i + 1]; ++q) {
      const Trip &x = t[order[q]];
      if (slot[x.c] >= start) {
        m.val[slot[x.c]] += x.v;
      } else {
        slot[x.c] = int(m.col.size());
        m.col.push_back(x.c);
        m.val.push_back(x.v);
      }
    }
    // sort the row by column (values move with their column)
    int end = int(m.col.size());
    std::vector<std::pair<int, double>> row;
    for (int q = start; q < end; ++q) row.push_back({m.col[q], m.val[q]});
    std::sort(row.begin(), row.end(),
              [](auto &a, auto &b) { return a.first < b.first; });
    for (int q = start; q < end; ++q) {
      m.col[q] = row[q - start].first;
      m.val[q] = row[q - start].second;
      slot[m.col[q]] = -1;
    }
    m.rowptr[i + 1] = end;
  }
  return m;
}

void spmv(const Csr &A, const double *x, double *y) {
  for (int i = 0; i < A.n; ++i) {
    double s = 0;
    for (int q = A.rowptr[i]; q < A.rowptr[i + 1]; ++q) s += A.val[q] * x[A.col[q]];
    y[i] = s;
  }
}

}  // namespace

struct orc_forces {
  int n_nodes;
  std::vector<double> f;
  Csr M, MDK;
};

extern "C" {

// Forces::fill, non-EOL branches (Forces.cpp:331-398,498-518 for faces;
// 685-745,885-908 for hinges; 912-930 for the fill itself).
orc_forces *orc_forces_fill(int n_nodes, const double *x, const double *X,
                            const int *tri, int n_tri, const int *hinge,
                            int n_hinge, const eolc_material *mat,
                            const double *grav, double h) {
  auto *F = new orc_forces;
  int n = 3 * n_nodes;
  F->n_nodes = n_nodes;
  F->f.assign(n, 0.0);
  std::vector<Trip> Mt, Kt;
  Mt.reserve(size_t(n_tri) * 81);
  Kt.reserve(size_t(n_tri) * 81 + size_t(n_hinge) * 144);
  const double dh2 = mat->damping_b * h * h;  // ((damping(1) * h) * h)
  for (int t = 0; t < n_tri; ++t) {
    const int *v = tri + 3 * t;
    double x9[9], X6[6], P6[6], Q4[4];
    for (int a = 0; a < 3; ++a) {
      for (int c = 0; c < 3; ++c) x9[3 * a + c] = x[3 * v[a] + c];
      for (int c = 0; c < 2; ++c) X6[2 * a + c] = X[2 * v[a] + c];
    }
    orc_face_frame(x9, X6, P6, Q4);
    double W, fm[9], Km[81], fi[9], Mi[81];
    orc_membrane(x9, X6, mat->e, mat->nu, P6, Q4, &W, fm, Km);
    orc_inertial(x9, X6, grav, mat->density, &W, fi, Mi);
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) F->f[3 * v[a] + c] += fm[3 * a + c] + fi[3 * a + c];
    // Element blocks are read through a column-major Map of K[i*9+j]
    // (Forces.cpp:393-396), i.e. Kme(i, j) = K[j*9 + i].
    auto Kme = [&](int i, int j) { return Km[j * 9 + i]; };
    auto Mie = [&](int i, int j) { return Mi[j * 9 + i]; };
    // fillxMI on the diagonal blocks (Forces.cpp:103-113)
    for (int a = 0; a < 3; ++a) {
      int ia = 3 * v[a];
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          double m = Mie(3 * a + j, 3 * a + k);
          Mt.push_back({ia + j, ia + k, m});
          Kt.push_back({ia + j, ia + k, m + dh2 * Kme(3 * a + j, 3 * a + k)});
        }
    }
    // fillxxMI on (a,b), (a,c), (b,c) (Forces.cpp:115-125)
    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (auto &p : pr) {
      int i0 = 3 * v[p[0]], i1 = 3 * v[p[1]];
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          double m = Mie(3 * p[0] + j, 3 * p[1] + k);
          double mk = m + dh2 * Kme(3 * p[0] + j, 3 * p[1] + k);
          Mt.push_back({i0 + j, i1 + k, m});
          Mt.push_back({i1 + k, i0 + j, m});
          Kt.push_back({i0 + j, i1 + k, mk});
          Kt.push_back({i1 + k, i0 + j, mk});
        }
    }
  }
  for (int e = 0; e < n_hinge; ++e) {
    const int *v = hinge + 4 * e;
    double x12[12], X8[8];
    for (int a = 0; a < 4; ++a) {
      for (int c = 0; c < 3; ++c) x12[3 * a + c] = x[3 * v[a] + c];
      for (int c = 0; c < 2; ++c) X8[2 * a + c] = X[2 * v[a] + c];
    }
    double W, fb[12], Kb[144];
    orc_bending(x12, X8, mat->beta, &W, fb, Kb);
    // Non-EOL hinges add stiffness only, no force (Forces.cpp:885-908).
    auto Kbe = [&](int i, int j) { return Kb[j * 12 + i]; };
    for (int a = 0; a < 4; ++a) {  // fillxB (Forces.cpp:522-529)
      int ia = 3 * v[a];
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k)
          Kt.push_back({ia + j, ia + k, dh2 * Kbe(3 * a + j, 3 * a + k)});
    }
    const int pr[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    for (auto &p : pr) {  // fillxxB (Forces.cpp:531-539)
      int i0 = 3 * v[p[0]], i1 = 3 * v[p[1]];
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          double kk = dh2 * Kbe(3 * p[0] + j, 3 * p[1] + k);
          Kt.push_back({i0 + j, i1 + k, kk});
          Kt.push_back({i1 + k, i0 + j, kk});
        }
    }
  }
  F->M = from_triplets(n, Mt);
  F->MDK = from_triplets(n, Kt);
  return F;
}

void orc_forces_free(orc_forces *F) { delete F; }

int orc_forces_nnz(const orc_forces *F, int which) {
  return int((which ? F->MDK : F->M).col.size());
}

void orc_forces_csr(const orc_forces *F, int which, int *rowptr, int *col,
                    double *val) {
  const Csr &A = which ? F->MDK : F->M;
  std::memcpy(rowptr, A.rowptr.data(), sizeof(int) * (A.n + 1));
  std::memcpy(col, A.col.data(), sizeof(int) * A.col.size());
  std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
}

void orc_forces_f(const orc_forces *F, double *f) {
  std::memcpy(f, F->f.data(), sizeof(double) * F->f.size());
}

// b = -(M v + h f) (Cloth.cpp:345): the sparse product is evaluated into a
// temporary first, then combined elementwise.
void orc_rhs(const orc_forces *F, const double *v, double h, double *b) {
  int n = 3 * F->n_nodes;
  std::vector<double> Mv(n);
  spmv(F->M, v, Mv.data());
  for (int i = 0; i < n; ++i) b[i] = -(Mv[i] + h * F->f[i]);
}

// Equality-constrained optimum of 1/2 v'Av + b'v with v_P = beq: solve
// A_FF v_F = -b_F - A_FP beq by Jacobi-preconditioned CG in the form of
// Eigen's ConjugateGradient (the branch GeneralizedSolver.cpp:123-126 meant
// to take): x0 = 0, threshold tol^2 ||rhs||^2 on ||r||^2, preconditioner =
// inverse diagonal (1 where the diagonal is 0).
int orc_velocity_solve(const orc_forces *F, const double *b,
                       const int *fixed_dofs, const double *beq, int n_fixed,
                       double tol, int max_iter, double *v_out,
                       double *relres) {
  const Csr &A = F->MDK;
  int n = A.n;
  std::vector<int> fixed(n, -1);
  for (int k = 0; k < n_fixed; ++k) fixed[fixed_dofs[k]] = k;
  std::vector<double> rhs(n, 0.0), x(n, 0.0), r(n), p(n), z(n), q(n),
      dinv(n, 1.0);
  for (int i = 0; i < n; ++i) {
    if (fixed[i] >= 0) continue;
    double s = -b[i];
    for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) {
      int j = A.col[k];
      if (fixed[j] >= 0) s -= A.val[k] * beq[fixed[j]];
      if (j == i && A.val[k] != 0.0) dinv[i] = 1.0 / A.val[k];
    }
    rhs[i] = s;
  }
  auto Aff = [&](const std::vector<double> &in, std::vector<double> &out) {
    for (int i = 0; i < n; ++i) {
      if (fixed[i] >= 0) { out[i] = 0; continue; }
      double s = 0;
      for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) {
        int j = A.col[k];
        if (fixed[j] < 0) s += A.val[k] * in[j];
      }
      out[i] = s;
    }
  };
  auto dotp = [&](const std::vector<double> &a, const std::vector<double> &c) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * c[i];
    return s;
  };
  double rhs2 = dotp(rhs, rhs);
  int it = 0;
  double res2 = 0;
  if (rhs2 == 0) {
    std::fill(x.begin(), x.end(), 0.0);
  } else {
    double thr = tol * tol * rhs2;
    r = rhs;  // x0 = 0
    res2 = dotp(r, r);
    if (res2 >= thr) {
      for (int i = 0; i < n; ++i) p[i] = dinv[i] * r[i];
      double absNew = dotp(r, p);
      while (it < max_iter) {
        Aff(p, q);
        double alpha = absNew / dotp(p, q);
        for (int i = 0; i < n; ++i) x[i] += alpha * p[i];
        for (int i = 0; i < n; ++i) r[i] -= alpha * q[i];
        res2 = dotp(r, r);
        if (res2 < thr) { ++it; break; }
        for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
        double absOld = absNew;
        absNew = dotp(r, z);
        double beta = absNew / absOld;
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        ++it;
      }
    }
  }
  if (relres) *relres = rhs2 == 0 ? 0.0 : std::sqrt(res2 / rhs2);
  for (int i = 0; i < n; ++i) v_out[i] = fixed[i] >= 0 ? beq[fixed[i]] : x[i];
  return it;
}

// Dense LDL^T (no pivoting; the reduced system is symmetric) for small
// systems: the FP64 reference solution the iterative results are measured against.
int orc_velocity_solve_direct(const orc_forces *F, const double *b,
                              const int *fixed_dofs, const double *beq,
                              int n_fixed, double *v_out) {
  const Csr &A = F->MDK;
  int n = A.n;
  std::vector<int> fixed(n, -1), fmap(n, -1), free_ids;
  for (int k = 0; k < n_fixed; ++k) fixed[fixed_dofs[k]] = k;
  for (int i = 0; i < n; ++i)
    if (fixed[i] < 0) { fmap[i] = int(free_ids.size()); free_ids.push_back(i); }
  int m = int(free_ids.size());
  if (m > 6000) return -1;
  std::vector<double> D(size_t(m) * m, 0.0), y(m, 0.0);
  for (int a = 0; a < m; ++a) {
    int i = free_ids[a];
    double s = -b[i];
    for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) {
      int j = A.col[k];
      if (fixed[j] >= 0) s -= A.val[k] * beq[fixed[j]];
      else D[size_t(a) * m + fmap[j]] = A.val[k];
    }
    y[a] = s;
  }
  // Band-limited Gaussian elimination without pivoting (the reduced system
  // is symmetric positive definite for the configurations tested); the
  // multipliers l_ik overwrite the strictly lower triangle.
  int bw = 0;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j)
      if (D[size_t(i) * m + j] != 0.0 && std::abs(i - j) > bw) bw = std::abs(i - j);
  for (int k = 0; k < m; ++k) {
    double dk = D[size_t(k) * m + k];
    if (dk == 0) return -2;
    int hi = std::min(m, k + bw + 1);
    const double *rk = &D[size_t(k) * m];
    for (int i = k + 1; i < hi; ++i) {
      double lik = D[size_t(i) * m + k] / dk;
      if (lik == 0) continue;
      double *ri = &D[size_t(i) * m];
      for (int j = k + 1; j < hi; ++j) ri[j] -= lik * rk[j];
      ri[k] = lik;
    }
  }
  for (int i = 0; i < m; ++i)
    for (int k = 0; k < i; ++k) y[i] -= D[size_t(i) * m + k] * y[k];
  for (int i = 0; i < m; ++i) y[i] /= D[size_t(i) * m + i];
  for (int i = m - 1; i >= 0; --i)
    for (int k = i + 1; k < m; ++k) y[i] -= D[size_t(k) * m + i] * y[k];
  for (int i = 0; i < n; ++i) v_out[i] = fixed[i] >= 0 ? beq[fixed[i]] : y[fmap[i]];
  return 0;
}

// Cloth::step, non-EOL without remeshing or contacts (Cloth.cpp:359-413):
// pins beq = (1 - 0.01) v + c (Constraints.cpp:114-119, 472-496), forces,
// rhs, solve, then node->x = node->x + h * node->v.
int orc_step(int n_nodes, double *x, const double *X, double *v,
             const int *tri, int n_tri, const int *hinge, int n_hinge,
             const eolc_material *mat, const double *grav, double h,
             const int *fixed_dofs, const double *fixed_vel, int n_fixed,
             double tol, int max_iter, double *relres) {
  int n = 3 * n_nodes;
  std::vector<double> beq(n_fixed);
  for (int k = 0; k < n_fixed; ++k)
    beq[k] = (1 - 0.01) * v[fixed_dofs[k]] + fixed_vel[k];
  orc_forces *F = orc_forces_fill(n_nodes, x, X, tri, n_tri, hinge, n_hinge,
                                  mat, grav, h);
  std::vector<double> b(n), vn(n);
  orc_rhs(F, v, h, b.data());
  int it = orc_velocity_solve(F, b.data(), fixed_dofs, beq.data(), n_fixed, tol,
                              max_iter, vn.data(), relres);
  orc_forces_free(F);
  for (int i = 0; i < n; ++i) {
    v[i] = vn[i];
    x[i] = x[i] + h * v[i];
  }
  return it;
}

}  // extern "C"

// ---- Forces::fill with EOL nodes ------------------------------------------
// The EOL branches of faceBasedF (Forces.cpp:399-497 with fillEOLInertia /
// fillEOLMembrane, :177-329) and edgeBasedF (:746-884 with fillEOLBending,
// :580-683).  A node with EoL_index k owns two Eulerian DOFs at 3N + 2k.
// With the element's Lagrangian blocks K_vw and, for an EOL vertex v, its
// deformation gradient F_v (3x2; the face's for faces, the mean of the two
// adjacent faces' for hinges), the reference fills
//   (x_v, x_w) = K_vw,  (X_v, x_w) = -F_v' K_vw,  (x_w, X_v) = -K_wv F_v,
//   (X_v, X_w) = F_v' K_vw F_w,  f_X_v = -F_v' f_v,
// in this triplet order: Lagrangian diagonal blocks, Lagrangian pairs,
// Eulerian diagonal blocks, Eulerian pairs, then for each EOL vertex v in
// order the blocks (X_v, x_w) for w >= v followed by (x_u, X_v) for u < v
// (each fill also pushes the transpose).  Faces do this for M and MDK
// (MDK = M + dB h^2 K); hinges for MDK only, and a hinge that touches an EOL
// node also adds its bending force to the Lagrangian DOFs (the non-EOL
// branch adds none).
namespace {

struct F32 {
  double a[3][2];
};

// deform_grad (UtilEOL.cpp:13-28): Dx * inverse(DX), Eigen's 2x2 inverse.
F32 deform_grad(const double *x, const double *X, int i0, int i1, int i2) {
  double Dx[3][2], DX[2][2];
  for (int c = 0; c < 3; ++c) {
    Dx[c][0] = x[3 * i1 + c] - x[3 * i0 + c];
    Dx[c][1] = x[3 * i2 + c] - x[3 * i0 + c];
  }
  for (int c = 0; c < 2; ++c) {
    DX[c][0] = X[2 * i1 + c] - X[2 * i0 + c];
    DX[c][1] = X[2 * i2 + c] - X[2 * i0 + c];
  }
  const double det = DX[0][0] * DX[1][1] - DX[1][0] * DX[0][1];
  const double id = 1.0 / det;
  const double inv[2][2] = {{DX[1][1] * id, -DX[0][1] * id}, {-DX[1][0] * id, DX[0][0] * id}};
  F32 F;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) F.a[r][c] = Dx[r][0] * inv[0][c] + Dx[r][1] * inv[1][c];
  return F;
}

// One element's triplets.  nv vertices with global Lagrangian DOF base
// xi[v] and Eulerian base Xi[v] (-1: not EOL); K(i, j) / M(i, j) read the
// element's 3nv x 3nv matrices; M may be null (hinges).  s = dB h^2.
template <typename KF, typename MF>
void emit_eol_element(int nv, const int *xi, const int *Xi, const F32 *F, KF K, MF M,
                      bool has_m, double s, std::vector<Trip> &Mt, std::vector<Trip> &Kt) {
  auto blk = [&](auto &A, int v, int w, int j, int k) { return A(3 * v + j, 3 * w + k); };
  // value of a transformed block entry: kind 0 x-x, 1 X-x, 2 x-X, 3 X-X
  auto tr = [&](auto &A, int kind, int v, int w, int j, int k) {
    double r = 0;
    if (kind == 0) return blk(A, v, w, j, k);
    if (kind == 1) {  // -F_v' A_vw, (2 x 3)
      for (int p = 0; p < 3; ++p) r += F[v].a[p][j] * blk(A, v, w, p, k);
      return -r;
    }
    if (kind == 2) {  // -A_vw F_w, (3 x 2)
      for (int q = 0; q < 3; ++q) r += blk(A, v, w, j, q) * F[w].a[q][k];
      return -r;
    }
    for (int p = 0; p < 3; ++p) {  // F_v' A_vw F_w, (2 x 2)
      double t = 0;
      for (int q = 0; q < 3; ++q) t += blk(A, v, w, p, q) * F[w].a[q][k];
      r += F[v].a[p][j] * t;
    }
    return r;
  };
  // push block (v, w) of the given kind at rows r0, cols c0, and its
  // transpose when sym
  auto push = [&](int kind, int v, int w, int r0, int c0, bool sym) {
    const int nr = (kind == 1 || kind == 3) ? 2 : 3, nc = (kind == 2 || kind == 3) ? 2 : 3;
    for (int j = 0; j < nr; ++j)
      for (int k = 0; k < nc; ++k) {
        const double m = has_m ? tr(M, kind, v, w, j, k) : 0.0;
        const double kk = has_m ? m + s * tr(K, kind, v, w, j, k) : s * tr(K, kind, v, w, j, k);
        if (has_m) Mt.push_back({r0 + j, c0 + k, m});
        Kt.push_back({r0 + j, c0 + k, kk});
        if (sym) {
          if (has_m) Mt.push_back({c0 + k, r0 + j, m});
          Kt.push_back({c0 + k, r0 + j, kk});
        }
      }
  };
  for (int v = 0; v < nv; ++v) push(0, v, v, xi[v], xi[v], false);
  for (int v = 0; v < nv; ++v)
    for (int w = v + 1; w < nv; ++w) push(0, v, w, xi[v], xi[w], true);
  for (int v = 0; v < nv; ++v)
    if (Xi[v] >= 0) push(3, v, v, Xi[v], Xi[v], false);
  for (int v = 0; v < nv; ++v)
    for (int w = v + 1; w < nv; ++w)
      if (Xi[v] >= 0 && Xi[w] >= 0) push(3, v, w, Xi[v], Xi[w], true);
  for (int v = 0; v < nv; ++v) {
    if (Xi[v] < 0) continue;
    for (int w = v; w < nv; ++w) push(1, v, w, Xi[v], xi[w], true);
    for (int u = 0; u < v; ++u) push(2, u, v, xi[u], Xi[v], true);
  }
}

}  // namespace

extern "C" orc_forces *orc_forces_fill_eol(int n_nodes, const double *x, const double *X,
                                           const int *tri, int n_tri, const int *hinge,
                                           int n_hinge, const eolc_material *mat,
                                           const double *grav, double h, const int *eol_index,
                                           int n_eol) {
  auto *F = new orc_forces;
  const int n = 3 * n_nodes + 2 * n_eol;
  F->n_nodes = n_nodes;
  F->f.assign(n, 0.0);
  std::vector<Trip> Mt, Kt;
  const double dh2 = mat->damping_b * h * h;
  auto Xdof = [&](int node) { return eol_index[node] >= 0 ? 3 * n_nodes + 2 * eol_index[node] : -1; };
  for (int t = 0; t < n_tri; ++t) {
    const int *v = tri + 3 * t;
    double x9[9], X6[6], P6[6], Q4[4];
    for (int a = 0; a < 3; ++a) {
      for (int c = 0; c < 3; ++c) x9[3 * a + c] = x[3 * v[a] + c];
      for (int c = 0; c < 2; ++c) X6[2 * a + c] = X[2 * v[a] + c];
    }
    orc_face_frame(x9, X6, P6, Q4);
    double W, fm[9], Km[81], fi[9], Mi[81];
    orc_membrane(x9, X6, mat->e, mat->nu, P6, Q4, &W, fm, Km);
    orc_inertial(x9, X6, grav, mat->density, &W, fi, Mi);
    auto Kme = [&](int i, int j) { return Km[j * 9 + i]; };
    auto Mie = [&](int i, int j) { return Mi[j * 9 + i]; };
    int xi[3], Xi[3];
    bool eol = false;
    for (int a = 0; a < 3; ++a) {
      xi[a] = 3 * v[a];
      Xi[a] = Xdof(v[a]);
      eol |= Xi[a] >= 0;
    }
    const F32 Fg = deform_grad(x, X, v[0], v[1], v[2]);
    F32 Fv[3] = {Fg, Fg, Fg};
    for (int a = 0; a < 3; ++a) {
      for (int c = 0; c < 3; ++c) F->f[xi[a] + c] += fm[3 * a + c] + fi[3 * a + c];
      if (Xi[a] < 0) continue;
      for (int j = 0; j < 2; ++j) {  // (-F' fm) + (-F' fi), Forces.cpp:206-216,284-294,406-416
        double sm = 0, si = 0;
        for (int p = 0; p < 3; ++p) {
          sm += Fg.a[p][j] * fm[3 * a + p];
          si += Fg.a[p][j] * fi[3 * a + p];
        }
        F->f[Xi[a] + j] += -sm + -si;
      }
    }
    emit_eol_element(3, xi, Xi, Fv, Kme, Mie, true, dh2, Mt, Kt);
    (void)eol;
  }
  for (int e = 0; e < n_hinge; ++e) {
    const int *v = hinge + 4 * e;
    double x12[12], X8[8];
    for (int a = 0; a < 4; ++a) {
      for (int c = 0; c < 3; ++c) x12[3 * a + c] = x[3 * v[a] + c];
      for (int c = 0; c < 2; ++c) X8[2 * a + c] = X[2 * v[a] + c];
    }
    double W, fb[12], Kb[144];
    orc_bending(x12, X8, mat->beta, &W, fb, Kb);
    auto Kbe = [&](int i, int j) { return Kb[j * 12 + i]; };
    auto none = [&](int, int) { return 0.0; };
    int xi[4], Xi[4];
    bool eol = false;
    for (int a = 0; a < 4; ++a) {
      xi[a] = 3 * v[a];
      Xi[a] = Xdof(v[a]);
      eol |= Xi[a] >= 0;
    }
    F32 Fv[4];
    if (eol) {
      // (F1 + F2) / 2 over the two adjacent faces (Forces.cpp:590-596)
      const F32 F1 = deform_grad(x, X, v[0], v[1], v[2]), F2 = deform_grad(x, X, v[0], v[1], v[3]);
      F32 Fm;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 2; ++c) Fm.a[r][c] = (F1.a[r][c] + F2.a[r][c]) / 2;
      for (int a = 0; a < 4; ++a) Fv[a] = Fm;
      for (int a = 0; a < 4; ++a) {  // the EOL branch adds the bending force
        for (int c = 0; c < 3; ++c) F->f[xi[a] + c] += fb[3 * a + c];
        if (Xi[a] < 0) continue;
        for (int j = 0; j < 2; ++j) {
          double sb = 0;
          for (int p = 0; p < 3; ++p) sb += Fm.a[p][j] * fb[3 * a + p];
          F->f[Xi[a] + j] += -sb;
        }
      }
    }
    emit_eol_element(4, xi, Xi, Fv, Kbe, none, false, dh2, Mt, Kt);
  }
  F->M = from_triplets(n, Mt);
  F->MDK = from_triplets(n, Kt);
  return F;
}
