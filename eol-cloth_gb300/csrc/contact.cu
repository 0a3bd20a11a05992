// Contact-constrained velocity solve: the QP that GeneralizedSolver::
// velocitySolve hands Mosek or Gurobi when there are collisions
// (GeneralizedSolver.cpp:138-170, quadprog convention of QuadProg.h:8-9),
//
//     min_v 1/2 v' MDK v + b' v   s.t.  v[pinned] = beq,  C v <= d,
//
// with the inequality rows of Constraints::fill (Constraints.cpp:422-468 for
// the CD2 contacts of a non-EOL mesh: one row per contact over one to three
// cloth nodes), and, for EOL meshes, its general equality rows E v = e
// (Constraints.cpp:147-415: the EOL nodes' rows on their Lagrangian and
// Eulerian DOFs).
//
// Method: augmented Lagrangian (method of multipliers) on the inequality
// rows, each augmented-Lagrangian minimisation by semismooth Newton:
//   W = { i : lam_i + rho_i (C v - d)_i > 0 }
//   (MDK + sum_{i in W} rho_i c_i c_i') v = -(b + sum_{i in W} c_i (lam_i - rho_i d_i))
// repeated until W stops changing, then lam <- max(0, lam + rho (C v - d)),
// until max_i |lam_new - lam|_i / rho_i <= 10 rel_tol max|v|.  Equality rows
// are the same terms with every row always in W and lam <- lam + rho (E v - e)
// unclamped (the method of multipliers for equalities).  At every
// augmented-Lagrangian minimiser MDK v + b + C' lam_new = 0 holds (to the
// linear solve's tolerance), so the stopping test bounds the remaining
// infeasibility and complementarity.  rho_i = 100 x (mean diagonal of MDK over
// the row's nodes) / |c_i|^2; with that scaling the multipliers gain about
// three digits per update.
//
// Every linear solve is the library's PCG (any precision / preconditioner of
// eolc_velocity_solve) on a penalised copy of MDK, warm-started from the
// previous solution.  The penalty terms c_i c_i' couple only nodes of one
// contact (a face or an edge of the mesh), which share BSR blocks, so the
// pattern is unchanged; each touched block and right-hand-side node sums its
// terms in a fixed order (per-block and per-node lists built on the host):
// results are bit-reproducible.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

using namespace eolc;

namespace {

constexpr int kRowNodes = 4;        // nodes a row may touch
constexpr double kKappa = 100.0;    // penalty scale (x mean diagonal / |c|^2)
constexpr int kMaxOuter = 50;       // multiplier updates
constexpr int kMaxInner = 40;       // semismooth Newton steps per update
constexpr double kLooseTol = 1e-4;  // solve tolerance while the active set changes
constexpr int kThreads = 128;

enum { kStatChanges = 0, kStatDlam = 1, kStatViol = 2, kStatActive = 3, kStatVmax = 4,
       kStatWords = 5 };

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *p, double x) {
  atomicMax(p, static_cast<unsigned long long>(__double_as_longlong(x)));
}

// rho_i from the diagonal blocks of the row's nodes (unpenalised MDK): the
// mean diagonal entry over the row's DOFs.  An Eulerian node (block row >=
// n_real) has two DOFs; its padded third diagonal entry (1) is left out.
template <typename T>
__global__ void ineq_setup_kernel(int m, int n_real, const int *__restrict__ rnode,
                                  const double *__restrict__ rg, const int *__restrict__ diag,
                                  const T *__restrict__ A, double *__restrict__ rho) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double tr = 0, g2 = 0;
  int ndof = 0;
  for (int p = 0; p < kRowNodes; ++p) {
    const int a = rnode[kRowNodes * i + p];
    if (a < 0) continue;
    const T *blk = A + size_t(diag[a]) * 9;
    const bool eul = a >= n_real;
    tr += eul ? double(blk[0]) + double(blk[4]) : double(blk[0]) + double(blk[4]) + double(blk[8]);
    for (int c = 0; c < 3; ++c) {
      const double g = rg[(kRowNodes * i + p) * 3 + c];
      g2 += g * g;
    }
    ndof += eul ? 2 : 3;
  }
  rho[i] = ndof > 0 && g2 > 0 ? kKappa * (tr / double(ndof)) / g2 : 0.0;
}

// max |v| over the 3N DOFs; a non-finite entry makes it +inf (fmax alone
// would drop a NaN), which the host reports as EOLC_NONFINITE.
__global__ void absmax_kernel(int n, const double *__restrict__ v, unsigned long long *stat) {
  double mx = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    mx = isfinite(v[k]) ? fmax(mx, fabs(v[k])) : CUDART_INF;
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(stat + kStatVmax, mx);
}

// Per row: r = C_i v - d_i.  update = 1: lam <- max(0, lam + rho r) with the
// largest |change| / rho, violation and active count recorded.  Then the
// active flag for the next solve, lam + rho r > 0, and the count of flags
// that changed.  Rows below m_eq are equalities: lam <- lam + rho r, |r| is
// their violation, and they are always active.
__global__ void ineq_eval_kernel(int m, int m_eq, const int *__restrict__ rnode,
                                 const double *__restrict__ rg, const double *__restrict__ v,
                                 const double *__restrict__ rho, const double *__restrict__ d,
                                 double *__restrict__ lam, uint8_t *__restrict__ act,
                                 double *__restrict__ cv, int update,
                                 unsigned long long *__restrict__ stat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0;
  for (int p = 0; p < kRowNodes; ++p) {
    const int a = rnode[kRowNodes * i + p];
    if (a < 0) continue;
    const double *g = rg + (kRowNodes * i + p) * 3;
    s += g[0] * v[3 * a] + g[1] * v[3 * a + 1] + g[2] * v[3 * a + 2];
  }
  cv[i] = s;
  const double r = s - d[i], ri = rho[i];
  double l = lam[i];
  const bool eq = i < m_eq;
  if (update) {
    const double ln = eq ? l + ri * r : fmax(0.0, l + ri * r);
    if (ri > 0) atomic_max_nonneg(stat + kStatDlam, fabs(ln - l) / ri);
    atomic_max_nonneg(stat + kStatViol, eq ? fabs(r) : fmax(0.0, r));
    if (!eq && ln > 0) atomicAdd(stat + kStatActive, 1ull);
    lam[i] = ln;
    l = ln;
  }
  const uint8_t na = ri > 0 && (eq || l + ri * r > 0);
  if (na != act[i]) {
    atomicAdd(stat + kStatChanges, 1ull);
    act[i] = na;
  }
}

// Penalised blocks: Ap[blk] = A[blk] + sum over the active rows' terms
// rho_i g_pa g_pb' (block (a, b) of the row's nodes pa, pb), summed in FP64
// in list order.
template <typename T>
__global__ void pen_blocks_kernel(int nu, const int *__restrict__ ublk,
                                  const int *__restrict__ uptr, const int *__restrict__ uitem,
                                  const double *__restrict__ rg, const double *__restrict__ rho,
                                  const uint8_t *__restrict__ act, const T *__restrict__ A,
                                  T *__restrict__ Ap) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  const size_t blk = size_t(ublk[u]) * 9;
  double acc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = double(A[blk + k]);
  for (int q = uptr[u]; q < uptr[u + 1]; ++q) {
    const int it = uitem[q];
    const int row = it >> 4, pa = (it >> 2) & 3, pb = it & 3;
    if (!act[row]) continue;
    const double *ga = rg + (kRowNodes * row + pa) * 3, *gb = rg + (kRowNodes * row + pb) * 3;
    const double ri = rho[row];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[3 * r + c] += ri * ga[r] * gb[c];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) Ap[blk + k] = T(acc[k]);
}

// Penalised right-hand side: bp[node] = b[node] + sum over the active rows'
// terms g_p (lam_i - rho_i d_i).
__global__ void pen_rhs_kernel(int nn, const int *__restrict__ unode,
                               const int *__restrict__ nptr, const int *__restrict__ nitem,
                               const double *__restrict__ rg, const double *__restrict__ rho,
                               const double *__restrict__ lam, const double *__restrict__ d,
                               const uint8_t *__restrict__ act, const double *__restrict__ b,
                               double *__restrict__ bp) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nn) return;
  const int a = unode[u];
  double acc[3] = {b[3 * a], b[3 * a + 1], b[3 * a + 2]};
  for (int q = nptr[u]; q < nptr[u + 1]; ++q) {
    const int it = nitem[q];
    const int row = it >> 2, p = it & 3;
    if (!act[row]) continue;
    const double w = lam[row] - rho[row] * d[row];
    const double *g = rg + (kRowNodes * row + p) * 3;
    acc[0] += g[0] * w;
    acc[1] += g[1] * w;
    acc[2] += g[2] * w;
  }
  bp[3 * a] = acc[0];
  bp[3 * a + 1] = acc[1];
  bp[3 * a + 2] = acc[2];
}

// Residual of the current v for the penalised system, per free DOF:
//   rhs = -b - A_fp beq  (the solver's right-hand side),  r = rhs - A_ff v,
// bc = -r (the "b" of the correction solve A d = r, d = 0 on pinned DOFs),
// and per-CTA FP64 partials of |rhs|^2 and |r|^2 (summed on the host in CTA
// order: reproducible).
template <typename T>
__global__ void __launch_bounds__(kThreads)
pen_residual_kernel(int N, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                    const T *__restrict__ A, const double *__restrict__ b,
                    const double *__restrict__ beq, const uint8_t *__restrict__ pinned,
                    const double *__restrict__ v, double *__restrict__ bc,
                    double *__restrict__ part) {
  __shared__ double red[2][kThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double q2 = 0, r2 = 0;
  if (i < N) {
    double rhs[3] = {-b[3 * i], -b[3 * i + 1], -b[3 * i + 2]};
    double av[3] = {0, 0, 0};
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = colidx[k];
      const T *blk = A + size_t(k) * 9;
      for (int c = 0; c < 3; ++c) {
        const bool pj = pinned[3 * j + c];
        const double xv = pj ? beq[3 * j + c] : v[3 * j + c];
        for (int r = 0; r < 3; ++r) {
          const double t = double(blk[3 * r + c]) * xv;
          if (pj) rhs[r] -= t;
          else av[r] += t;
        }
      }
    }
    for (int r = 0; r < 3; ++r) {
      if (pinned[3 * i + r]) {
        bc[3 * i + r] = 0.0;
        continue;
      }
      const double rr = rhs[r] - av[r];
      bc[3 * i + r] = -rr;
      q2 += rhs[r] * rhs[r];
      r2 += rr * rr;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    q2 += __shfl_xor_sync(0xffffffffu, q2, o);
    r2 += __shfl_xor_sync(0xffffffffu, r2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = q2;
    red[1][threadIdx.x >> 5] = r2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, c = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      a += red[0][w];
      c += red[1][w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = c;
  }
}

// v = beq on the pinned DOFs (the initial guess is a free vector).
__global__ void pin_values_kernel(int n, const uint8_t *__restrict__ pinned,
                                  const double *__restrict__ beq, double *__restrict__ v) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && pinned[k]) v[k] = beq[k];
}

// v += d on the free DOFs.
__global__ void add_correction_kernel(int n, const uint8_t *__restrict__ pinned,
                                      const double *__restrict__ dv, double *__restrict__ v) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && !pinned[k]) v[k] += dv[k];
}

int grid(long long n) { return int((n + kThreads - 1) / kThreads); }

}  // namespace

namespace eolc {

struct IneqWork {
  DevBuf<int> rnode, ublk, uptr, uitem, unode, nptr, nitem;
  DevBuf<double> rg, rho, lam, d, cv, bpen, A64, bc, dv, zero, part;
  std::vector<double> part_h;
  DevBuf<float> A32;
  DevBuf<uint8_t> act;
  DevBuf<unsigned long long> stat;
};

void free_ineq_work(IneqWork *w) { delete w; }

}  // namespace eolc

namespace {

#define IQ_CHECK(expr)                                                  \
  do {                                                                  \
    cudaError_t e_ = (expr);                                            \
    if (e_ != cudaSuccess) {                                            \
      ctx->err = std::string(#expr ": ") + cudaGetErrorString(e_);      \
      return EOLC_CUDA_ERROR;                                           \
    }                                                                   \
  } while (0)

eolc_status bad(eolc_ctx *ctx, const std::string &msg) {
  ctx->err = msg;
  return EOLC_BAD_ARG;
}

// Block index of (a, b) in the BSR pattern, or -1.
int find_block(const HostTopology &H, int a, int b) {
  const int *lo = H.colidx.data() + H.rowptr[a], *hi = H.colidx.data() + H.rowptr[a + 1];
  const int *it = std::lower_bound(lo, hi, b);
  return (it != hi && *it == b) ? int(it - H.colidx.data()) : -1;
}

}  // namespace

namespace eolc {

// The QP on the context's device state: MDK (last assembly), b, the pinned
// mask and beq_full, v as the initial guess (overwritten with the solution).
// Rows 0 .. eq.m - 1 of the solve are the equality rows, then the inequality
// rows; lambda0_h (optional) holds initial inequality multipliers.
eolc_status qp_solve_device(eolc_ctx *ctx, const QpRows &eq, const QpRows &iq,
                            const eolc_solve_opts *opts, double *lambda_eq_h,
                            double *lambda_h, eolc_ineq_info *info,
                            const double *lambda0_h) {
  if (eq.m < 0 || (eq.m > 0 && (!eq.ptr || !eq.col || !eq.val || !eq.rhs)))
    return bad(ctx, "null equality rows");
  if (iq.m < 0 || (iq.m > 0 && (!iq.ptr || !iq.col || !iq.val || !iq.rhs)))
    return bad(ctx, "null inequality rows");
  const HostTopology *Hp = host_topology(ctx);
  if (!Hp) return EOLC_CUDA_ERROR;
  const HostTopology &H = *Hp;
  const int N = H.n_nodes, n = 3 * N, m_eq = eq.m, m = eq.m + iq.m;
  const int n_real = ctx->topo.n_real;
  if (eq.m >= (1 << 27) || iq.m >= (1 << 27) || m >= (1 << 27))
    return bad(ctx, "too many constraint rows");
  // rows grouped by node (first-appearance order), columns checked
  std::vector<int> rnode(size_t(kRowNodes) * std::max(1, m), -1);
  std::vector<double> rg(size_t(kRowNodes) * 3 * std::max(1, m), 0.0);
  std::vector<double> d(std::max(1, m), 0.0);
  for (int i = 0; i < m; ++i) {
    const bool is_eq = i < m_eq;
    const QpRows &R = is_eq ? eq : iq;
    const int r = is_eq ? i : i - m_eq;
    const char *kind = is_eq ? "equality" : "inequality";
    if (R.ptr[r + 1] < R.ptr[r]) return bad(ctx, std::string(kind) + " row pointers decrease");
    int cnt = 0;
    for (int q = R.ptr[r]; q < R.ptr[r + 1]; ++q) {
      const int col = R.col[q];
      if (col < 0 || col >= n) return bad(ctx, std::string(kind) + " column out of range");
      if (col / 3 >= n_real && col % 3 == 2)
        return bad(ctx, std::string(kind) + " row on the padded DOF of an Eulerian node");
      if (!std::isfinite(R.val[q])) return bad(ctx, std::string("non-finite ") + kind + " coefficient");
      const int a = col / 3;
      int p = 0;
      while (p < cnt && rnode[kRowNodes * i + p] != a) ++p;
      if (p == cnt) {
        if (cnt == kRowNodes) return bad(ctx, std::string("an ") + kind + " row touches more than 4 nodes");
        rnode[kRowNodes * i + cnt++] = a;
      }
      rg[(size_t(kRowNodes) * i + p) * 3 + col % 3] += R.val[q];
    }
    d[i] = R.rhs[r];
    if (!std::isfinite(d[i])) return bad(ctx, is_eq ? "non-finite beq" : "non-finite bineq");
  }
  // per-block and per-node term lists (blocks of every node pair of a row)
  std::vector<long long> bitems;  // (block << 32) | (row << 4 | pa << 2 | pb)
  std::vector<long long> nitems;  // (node << 32) | (row << 2 | p)
  for (int i = 0; i < m; ++i)
    for (int pa = 0; pa < kRowNodes; ++pa) {
      const int a = rnode[kRowNodes * i + pa];
      if (a < 0) continue;
      nitems.push_back((long long)a << 32 | (i << 2 | pa));
      for (int pb = 0; pb < kRowNodes; ++pb) {
        const int bn = rnode[kRowNodes * i + pb];
        if (bn < 0) continue;
        const int blk = find_block(H, a, bn);
        if (blk < 0)
          return bad(ctx, "a constraint row couples nodes that share no element");
        bitems.push_back((long long)blk << 32 | (i << 4 | pa << 2 | pb));
      }
    }
  std::sort(bitems.begin(), bitems.end());
  std::sort(nitems.begin(), nitems.end());
  std::vector<int> ublk, uptr, uitem, unode, nptr, nitem;
  for (size_t k = 0; k < bitems.size(); ++k) {
    const int blk = int(bitems[k] >> 32);
    if (ublk.empty() || ublk.back() != blk) {
      ublk.push_back(blk);
      uptr.push_back(int(k));
    }
    uitem.push_back(int(bitems[k] & 0xffffffff));
  }
  uptr.push_back(int(bitems.size()));
  for (size_t k = 0; k < nitems.size(); ++k) {
    const int a = int(nitems[k] >> 32);
    if (unode.empty() || unode.back() != a) {
      unode.push_back(a);
      nptr.push_back(int(k));
    }
    nitem.push_back(int(nitems[k] & 0xffffffff));
  }
  nptr.push_back(int(nitems.size()));
  const int nu = int(ublk.size()), nn = int(unode.size());
  // device lists are never empty (one unused entry when there is no row)
  for (std::vector<int> *l : {&ublk, &uitem, &unode, &nitem})
    if (l->empty()) l->push_back(0);

  cudaSetDevice(ctx->device);
  cudaGetLastError();  // a stale error of an earlier call is not this call's
  cudaStream_t s = ctx->stream;
  if (!ctx->iq_work) ctx->iq_work = new IneqWork();
  IneqWork &W = *ctx->iq_work;
  eolc_status st = EOLC_OK;
  const bool fp64 = opts->precision == EOLC_PREC_FP64;
  const size_t nb9 = size_t(H.n_blocks) * 9;
  IQ_CHECK(W.rnode.upload(rnode.data(), rnode.size(), s));
  IQ_CHECK(W.rg.upload(rg.data(), rg.size(), s));
  IQ_CHECK(W.d.upload(d.data(), d.size(), s));
  IQ_CHECK(W.ublk.upload(ublk.data(), ublk.size(), s));
  IQ_CHECK(W.uptr.upload(uptr.data(), uptr.size(), s));
  IQ_CHECK(W.uitem.upload(uitem.data(), uitem.size(), s));
  IQ_CHECK(W.unode.upload(unode.data(), unode.size(), s));
  IQ_CHECK(W.nptr.upload(nptr.data(), nptr.size(), s));
  IQ_CHECK(W.nitem.upload(nitem.data(), nitem.size(), s));
  IQ_CHECK(W.rho.resize(std::max(1, m)));
  IQ_CHECK(W.lam.resize(std::max(1, m)));
  IQ_CHECK(W.cv.resize(std::max(1, m)));
  IQ_CHECK(W.act.resize(std::max(1, m)));
  IQ_CHECK(W.stat.resize(kStatWords));
  IQ_CHECK(W.bpen.resize(n));
  IQ_CHECK(W.bc.resize(n));
  IQ_CHECK(W.dv.resize(n));
  if (W.zero.n != size_t(n)) {
    IQ_CHECK(W.zero.resize(n));
    IQ_CHECK(cudaMemsetAsync(W.zero.p, 0, sizeof(double) * n, s));
  }
  const int nbr = grid(N);
  IQ_CHECK(W.part.resize(size_t(2) * nbr));
  W.part_h.resize(size_t(2) * nbr);
  IQ_CHECK(cudaMemsetAsync(W.lam.p, 0, sizeof(double) * std::max(1, m), s));
  if (lambda0_h && iq.m > 0)  // warm start: the active set starts from these
    IQ_CHECK(cudaMemcpyAsync(W.lam.p + m_eq, lambda0_h, sizeof(double) * iq.m,
                             cudaMemcpyHostToDevice, s));
  IQ_CHECK(cudaMemsetAsync(W.act.p, 0, std::max(1, m), s));
  IQ_CHECK(cudaMemcpyAsync(W.bpen.p, ctx->b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  // the learned network approximates the inverse of MDK, not of the
  // penalised matrix (contact terms up to 100x its diagonal), and the
  // single-reduction PCG breaks down on it: its QP solves use block Jacobi
  eolc_solve_opts qo = *opts;
  if (qo.precond == EOLC_PC_LEARNED) qo.precond = EOLC_PC_BLOCK_JACOBI;
  opts = &qo;
  PcgArgs a = default_pcg_args(ctx, opts);
  a.b = W.bpen.p;
  if (fp64) {
    IQ_CHECK(W.A64.resize(nb9 + 16));
    IQ_CHECK(cudaMemcpyAsync(W.A64.p, ctx->A64.p, sizeof(double) * nb9,
                             cudaMemcpyDeviceToDevice, s));
    a.A64 = W.A64.p;
    if (m > 0)
      ineq_setup_kernel<double><<<grid(m), kThreads, 0, s>>>(m, n_real, W.rnode.p, W.rg.p,
                                                             ctx->topo.diag.p, ctx->A64.p, W.rho.p);
  } else {
    IQ_CHECK(W.A32.resize(nb9 + 16));
    IQ_CHECK(cudaMemcpyAsync(W.A32.p, ctx->A32.p, sizeof(float) * (nb9 + 16),
                             cudaMemcpyDeviceToDevice, s));
    a.A32 = W.A32.p;
    a.A64 = nullptr;
    if (m > 0)
      ineq_setup_kernel<float><<<grid(m), kThreads, 0, s>>>(m, n_real, W.rnode.p, W.rg.p,
                                                            ctx->topo.diag.p, ctx->A32.p, W.rho.p);
  }
  ctx->launches += m > 0 ? 1 : 0;
  unsigned long long stat_h[kStatWords];
  // active set of the initial guess (lam = 0)
  auto eval = [&](int update) -> eolc_status {
    IQ_CHECK(cudaMemsetAsync(W.stat.p, 0, sizeof(unsigned long long) * kStatWords, s));
    if (m > 0) {
      ineq_eval_kernel<<<grid(m), kThreads, 0, s>>>(m, m_eq, W.rnode.p, W.rg.p, ctx->v.p, W.rho.p,
                                                    W.d.p, W.lam.p, W.act.p, W.cv.p, update,
                                                    W.stat.p);
      ++ctx->launches;
    }
    if (update) {
      absmax_kernel<<<152, 256, 0, s>>>(n, ctx->v.p, W.stat.p);
      ++ctx->launches;
    }
    IQ_CHECK(cudaMemcpyAsync(stat_h, W.stat.p, sizeof(stat_h), cudaMemcpyDeviceToHost, s));
    IQ_CHECK(cudaStreamSynchronize(s));
    return EOLC_OK;
  };
  auto as_double = [](unsigned long long u) {
    double x;
    memcpy(&x, &u, 8);
    return x;
  };
  eolc_ineq_info local{};
  eolc_ineq_info &I = info ? *info : local;
  I = eolc_ineq_info{};
  pin_values_kernel<<<grid(n), kThreads, 0, s>>>(n, ctx->pinned.p, ctx->beq_full.p, ctx->v.p);
  ++ctx->launches;
  if ((st = eval(0)) != EOLC_OK) return st;
  const double tol = 10.0 * opts->rel_tol;
  bool converged = false;
  // inexact Newton: while the last evaluation flipped active flags the next
  // solve only needs kLooseTol; a stable active set is confirmed by a solve to
  // rel_tol before the multipliers move
  unsigned long long pending = stat_h[kStatChanges];
  for (int outer = 0; outer < kMaxOuter && !converged; ++outer) {
    for (int inner = 0; inner < kMaxInner; ++inner) {
      const double stol = pending > 0 ? std::max(opts->rel_tol, kLooseTol) : opts->rel_tol;
      if (nu > 0) {
        if (fp64)
          pen_blocks_kernel<double><<<grid(nu), kThreads, 0, s>>>(
              nu, W.ublk.p, W.uptr.p, W.uitem.p, W.rg.p, W.rho.p, W.act.p, ctx->A64.p, W.A64.p);
        else
          pen_blocks_kernel<float><<<grid(nu), kThreads, 0, s>>>(
              nu, W.ublk.p, W.uptr.p, W.uitem.p, W.rg.p, W.rho.p, W.act.p, ctx->A32.p, W.A32.p);
        pen_rhs_kernel<<<grid(nn), kThreads, 0, s>>>(nn, W.unode.p, W.nptr.p, W.nitem.p, W.rg.p,
                                                     W.rho.p, W.lam.p, W.d.p, W.act.p, ctx->b.p,
                                                     W.bpen.p);
        ctx->launches += 2;
      }
      // correction solve from the current v: A d = r(v), tolerance scaled
      // so that the final residual meets rel_tol x |rhs| as a full solve
      if (fp64)
        pen_residual_kernel<double><<<nbr, kThreads, 0, s>>>(
            N, ctx->topo.rowptr.p, ctx->topo.colidx.p, W.A64.p, W.bpen.p, ctx->beq_full.p,
            ctx->pinned.p, ctx->v.p, W.bc.p, W.part.p);
      else
        pen_residual_kernel<float><<<nbr, kThreads, 0, s>>>(
            N, ctx->topo.rowptr.p, ctx->topo.colidx.p, W.A32.p, W.bpen.p, ctx->beq_full.p,
            ctx->pinned.p, ctx->v.p, W.bc.p, W.part.p);
      ++ctx->launches;
      IQ_CHECK(cudaGetLastError());
      IQ_CHECK(cudaMemcpyAsync(W.part_h.data(), W.part.p, sizeof(double) * 2 * nbr,
                               cudaMemcpyDeviceToHost, s));
      IQ_CHECK(cudaStreamSynchronize(s));
      double q2 = 0, r2 = 0;
      for (int k = 0; k < nbr; ++k) {
        q2 += W.part_h[2 * k];
        r2 += W.part_h[2 * k + 1];
      }
      const double qn = std::sqrt(q2), rn = std::sqrt(r2);
      I.solves += 1;
      if (rn > stol * qn) {
        PcgArgs ac = a;
        ac.b = W.bc.p;
        ac.beq_full = W.zero.p;
        ac.v = W.dv.p;
        ac.rel_tol = stol * qn / rn;
        eolc_solve_info si{};
        st = solve_with_args(ctx, opts, ac, &si, s);
        if (st == EOLC_BREAKDOWN && opts->precond != EOLC_PC_BLOCK_JACOBI) {
          // a breakdown of the preconditioned recurrence on a strongly
          // penalised system: the same correction solve once more with block
          // Jacobi (the contact terms sit in its diagonal blocks)
          eolc_solve_opts bj = *opts;
          bj.precond = EOLC_PC_BLOCK_JACOBI;
          PcgArgs ab = ac;
          ab.precond = EOLC_PC_BLOCK_JACOBI;
          I.iterations += si.iterations;
          si = eolc_solve_info{};
          st = solve_with_args(ctx, &bj, ab, &si, s);
          I.fallbacks += 1;
        }
        I.iterations += si.iterations;
        I.rel_res = si.rel_res * rn / std::max(qn, 1e-300);
        I.solve_kernel_ms += si.solve_kernel_ms;
        if (st != EOLC_OK) {
          I.status = st;
          return st;
        }
        add_correction_kernel<<<grid(n), kThreads, 0, s>>>(n, ctx->pinned.p, W.dv.p, ctx->v.p);
        ++ctx->launches;
      } else {
        I.rel_res = rn / std::max(qn, 1e-300);
      }
      if ((st = eval(0)) != EOLC_OK) return st;
      const bool settled = stat_h[kStatChanges] == 0 && stol <= opts->rel_tol;
      pending = stat_h[kStatChanges];
      if (settled) break;
    }
    if ((st = eval(1)) != EOLC_OK) return st;
    pending = stat_h[kStatChanges];
    I.outer = outer + 1;
    const double vmax = as_double(stat_h[kStatVmax]);
    if (!std::isfinite(vmax)) {
      I.status = EOLC_NONFINITE;
      ctx->err = "non-finite velocity in the contact solve";
      return EOLC_NONFINITE;
    }
    I.max_violation = vmax > 0 ? as_double(stat_h[kStatViol]) / vmax : as_double(stat_h[kStatViol]);
    I.n_active = int(stat_h[kStatActive]);
    converged = as_double(stat_h[kStatDlam]) <= tol * std::max(vmax, 1e-300);
  }
  if (lambda_eq_h && m_eq > 0)
    IQ_CHECK(cudaMemcpyAsync(lambda_eq_h, W.lam.p, sizeof(double) * m_eq, cudaMemcpyDeviceToHost,
                             s));
  if (lambda_h && iq.m > 0)
    IQ_CHECK(cudaMemcpyAsync(lambda_h, W.lam.p + m_eq, sizeof(double) * iq.m,
                             cudaMemcpyDeviceToHost, s));
  IQ_CHECK(cudaStreamSynchronize(s));
  I.status = converged ? EOLC_OK : EOLC_NOT_CONVERGED;
  if (!converged) ctx->err = "multiplier updates did not converge";
  return eolc_status(I.status);
}

eolc_status ineq_solve_device(eolc_ctx *ctx, int n_ineq, const int *ineq_ptr_h,
                              const int *ineq_col_h, const double *ineq_val_h,
                              const double *bineq_h, const eolc_solve_opts *opts,
                              double *lambda_h, eolc_ineq_info *info,
                              const double *lambda0_h) {
  const QpRows none{0, nullptr, nullptr, nullptr, nullptr};
  const QpRows iq{n_ineq, ineq_ptr_h, ineq_col_h, ineq_val_h, bineq_h};
  return qp_solve_device(ctx, none, iq, opts, nullptr, lambda_h, info, lambda0_h);
}

}  // namespace eolc

extern "C" eolc_status eolc_velocity_solve_ineq(
    eolc_ctx *ctx, const double *b_h, const int *fixed_dofs_h, const double *beq_h,
    int n_fixed, int n_ineq, const int *ineq_ptr_h, const int *ineq_col_h,
    const double *ineq_val_h, const double *bineq_h, const eolc_solve_opts *opts,
    double *v_h, double *lambda_h, eolc_ineq_info *info) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!ctx->has_topology) {
    ctx->err = "no topology set";
    return EOLC_NO_TOPOLOGY;
  }
  if (!opts) return bad(ctx, "null solve options");
  if (refuse_eol(ctx) != EOLC_OK) return EOLC_BAD_ARG;
  if (!b_h || !v_h || (n_fixed > 0 && !beq_h)) return bad(ctx, "null input");
  if (ctx->last_precision < 0) return bad(ctx, "no matrix assembled");
  if (opts->precision != ctx->last_precision)
    return bad(ctx, "solve precision differs from the assembled matrix");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const int n = 3 * ctx->topo.n_nodes;
  eolc_status st = prepare_pins_rhs(ctx, b_h, fixed_dofs_h, beq_h, n_fixed, s);
  if (st != EOLC_OK) return st;
  IQ_CHECK(ctx->v.upload(v_h, n, s));  // initial guess
  st = ineq_solve_device(ctx, n_ineq, ineq_ptr_h, ineq_col_h, ineq_val_h, bineq_h, opts,
                         lambda_h, info);
  IQ_CHECK(cudaMemcpyAsync(v_h, ctx->v.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  IQ_CHECK(cudaStreamSynchronize(s));
  return st;
}

extern "C" eolc_status eolc_velocity_solve_qp(eolc_ctx *ctx, const double *b_h,
                                              const int *fixed_dofs_h, const double *beq_h,
                                              int n_fixed, const eolc_rows *eq,
                                              const eolc_rows *ineq, const eolc_solve_opts *opts,
                                              double *v_h, double *lambda_eq_h,
                                              double *lambda_ineq_h, eolc_ineq_info *info) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!ctx->has_topology) {
    ctx->err = "no topology set";
    return EOLC_NO_TOPOLOGY;
  }
  if (!opts) return bad(ctx, "null solve options");
  if (!b_h || !v_h || (n_fixed > 0 && !beq_h)) return bad(ctx, "null input");
  if (ctx->last_precision < 0) return bad(ctx, "no matrix assembled");
  if (opts->precision != ctx->last_precision)
    return bad(ctx, "solve precision differs from the assembled matrix");
  const QpRows qe = eq ? QpRows{eq->n_rows, eq->ptr, eq->col, eq->val, eq->rhs}
                       : QpRows{0, nullptr, nullptr, nullptr, nullptr};
  const QpRows qi = ineq ? QpRows{ineq->n_rows, ineq->ptr, ineq->col, ineq->val, ineq->rhs}
                         : QpRows{0, nullptr, nullptr, nullptr, nullptr};
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const int n = 3 * ctx->topo.n_nodes;
  eolc_status st = prepare_pins_rhs(ctx, b_h, fixed_dofs_h, beq_h, n_fixed, s);
  if (st != EOLC_OK) return st;
  IQ_CHECK(ctx->v.upload(v_h, n, s));  // initial guess
  st = qp_solve_device(ctx, qe, qi, opts, lambda_eq_h, lambda_ineq_h, info);
  IQ_CHECK(cudaMemcpyAsync(v_h, ctx->v.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  IQ_CHECK(cudaStreamSynchronize(s));
  return st;
}

extern "C" eolc_status eolc_contact_rows(const eolc_contact *contacts, int n_contacts,
                                         int cap_rows, int *ineq_ptr_h, int *ineq_col_h,
                                         double *ineq_val_h, double *bineq_h, int *n_rows) {
  if (n_contacts < 0 || cap_rows < 0 || !n_rows || (n_contacts > 0 && !contacts) ||
      (cap_rows > 0 && (!ineq_col_h || !ineq_val_h || !bineq_h)) || !ineq_ptr_h)
    return EOLC_BAD_ARG;
  int m = 0, q = 0;
  ineq_ptr_h[0] = 0;
  for (int k = 0; k < n_contacts; ++k) {
    const eolc_contact &c = contacts[k];
    int nv;
    const double *nor;
    bool weighted;
    if (c.count1 == 3 && c.count2 == 1) {  // box face, cloth vertex
      nv = 1, nor = c.nor1, weighted = false;
    } else if (c.count1 == 2 && c.count2 == 2) {  // edge, edge
      nv = 2, nor = c.nor2, weighted = true;
    } else if (c.count1 == 1 && c.count2 == 3) {  // box corner or point, cloth face
      nv = 3, nor = c.nor2, weighted = true;
    } else {
      continue;
    }
    if (m < cap_rows) {
      for (int j = 0; j < nv; ++j)
        for (int a = 0; a < 3; ++a) {
          ineq_col_h[q] = c.verts2[j] * 3 + a;
          ineq_val_h[q] = weighted ? -nor[a] * c.weights2[j] : -nor[a];
          ++q;
        }
      bineq_h[m] = 0.0;
      ineq_ptr_h[m + 1] = q;
    }
    ++m;
  }
  *n_rows = m;
  return m > cap_rows ? EOLC_CAPACITY : EOLC_OK;
}
