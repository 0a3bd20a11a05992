// Preconditioned conjugate gradient on the 3x3 BSR matrix, as ONE persistent
// cooperative kernel per solve.
//
// Replaces the velocity solve of GeneralizedSolver::velocitySolve
// (GeneralizedSolver.cpp:107-173) for the pinned-corner case: the QP
// argmin 1/2 v'Av + b'v s.t. v_P = beq reduces to A_FF v_F = -b_F - A_FP beq.
// The algorithm is Eigen's ConjugateGradient (x0 = 0, stop on
// ||r|| <= tol ||rhs||, Jacobi preconditioner by default) with two
// additions for the mixed-precision path:
//   * inner vectors and matrix in FP32, every dot product accumulated in FP64;
//   * "reliable updates": whenever the iterated residual has dropped by
//     kDelta since the last check (or claims convergence) the FP32 update is
//     folded into an FP64 solution and the TRUE residual rhs - A x is
//     recomputed in FP64 arithmetic.  Convergence is declared only on that
//     FP64 residual, so the reported relative residual is an FP64 one.
// The FP64 path runs the same kernel with T = double.
//
// Layout: every vector is node-major with a padded 4th lane (one 16-byte load
// per node for float).  Rows are split into tiles (<= 256 rows, <= a shared-
// memory budget of blocks); each CTA owns a contiguous range of tiles and
// stages a tile's BSR values and column indices in shared memory with
// coalesced 16-byte loads, then one thread computes one block row.
//
// Per iteration there are two grid-wide barriers:
//   P1  p = z + beta p_old (computed on the fly for every neighbour),
//       q = A p, partial p.q                                  -> barrier
//   P2  alpha, x += alpha p, r -= alpha q, z = M^-1 r, partial r.z, r.r
//                                                             -> barrier
// Barriers spin with an iteration cap; on expiry the kernel records
// EOLC_TIMEOUT and every CTA returns.
#include <cooperative_groups.h>
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <string>
#include <vector>

#include "internal.h"

namespace eolc {

namespace {

constexpr int kThreads = 256;
constexpr int kTileRows = 256;
constexpr int kSmemBytes = 96 * 1024;  // staged values + column indices
constexpr double kDelta = 0.1;          // reliable-update trigger factor
constexpr long long kSpinLimit = 1ll << 24;

template <typename T>
struct alignas(4 * sizeof(T)) V4 {
  T x, y, z, w;
};

struct DevStatus {
  int status;
  int iterations;
  int refinements;
  int pad;
  double rel_res;
  double rhs_norm2;
};

// ---- grid barrier ----------------------------------------------------------
// bar[0] = arrival counter, bar[1] = generation.  Bounded spin: on expiry the
// barrier records EOLC_TIMEOUT and returns false.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned nblocks,
                                             unsigned &gen, DevStatus *st) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(bar[0]);
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> gflag(bar[1]);
    unsigned my_gen = gen;
    int ok = 1;
    __threadfence();
    unsigned arrived = count.fetch_add(1u, cuda::memory_order_acq_rel);
    if (arrived == nblocks - 1) {
      count.store(0u, cuda::memory_order_relaxed);
      gflag.store(my_gen + 1u, cuda::memory_order_release);
    } else {
      long long spins = 0;
      while (gflag.load(cuda::memory_order_acquire) == my_gen) {
        if (++spins > kSpinLimit) {
          atomicCAS(&st->status, EOLC_OK, EOLC_TIMEOUT);
          ok = 0;
          break;
        }
        if (spins > 64) __nanosleep(64);
      }
    }
    __threadfence();
    gen = my_gen + 1u;
    if (ok) {
      cuda::atomic_ref<int, cuda::thread_scope_device> sref(st->status);
      ok = sref.load(cuda::memory_order_relaxed) == EOLC_OK;
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Deterministic CTA-wide FP64 sum (fixed shuffle tree, fixed warp order).
__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
    red[kThreads / 32] = s;
  }
  __syncthreads();
  return red[kThreads / 32];
}

// Every CTA reduces the per-CTA partials of one quantity in the same fixed
// order, so all CTAs take the same branch decisions.
__device__ __forceinline__ double reduce_partials(const double *part, int n,
                                                  double *red) {
  double v = 0;
  for (int k = threadIdx.x; k < n; k += kThreads) v += __ldcg(part + k);
  return block_sum(v, red);
}

template <typename T>
struct Params {
  int n_nodes;
  int n_ctas;
  const int *rowptr;
  const int *colidx;
  const T *A;            // inner matrix (FP32 or FP64), also used promoted
                         // to FP64 for the true residual
  const int *tile_row;   // tile boundaries (n_tiles + 1)
  const int *cta_tile;   // CTA -> first tile (n_ctas + 1)
  const V4<double> *rhs; // masked rhs of the reduced system
  V4<double> *x64;
  V4<T> *r, *z, *pa, *pb, *q, *xacc;
  const T *pc;           // preconditioner: 4 per node (Jacobi) or 9 (block)
  const V4<T> *fmask;    // 1 on free DOFs, 0 on pinned
  double *part;          // 5 x n_ctas partial sums
  unsigned *bar;
  DevStatus *st;
  double tol2;           // tol^2 (scaled by ||rhs||^2 on the device)
  int max_iter;
  int block_pc;          // 0 = point Jacobi, 1 = block Jacobi
};

template <typename T>
__device__ __forceinline__ V4<T> ld4(const V4<T> *p, int i) {
  return p[i];
}

template <typename T>
__device__ __forceinline__ V4<T> apply_pc(const Params<T> &P, int i,
                                          V4<T> r) {
  V4<T> z;
  if (P.block_pc) {
    const T *B = P.pc + size_t(9) * i;
    z.x = B[0] * r.x + B[1] * r.y + B[2] * r.z;
    z.y = B[3] * r.x + B[4] * r.y + B[5] * r.z;
    z.z = B[6] * r.x + B[7] * r.y + B[8] * r.z;
  } else {
    const T *d = P.pc + size_t(4) * i;
    z.x = d[0] * r.x; z.y = d[1] * r.y; z.z = d[2] * r.z;
  }
  z.w = T(0);
  return z;
}

// Stages the BSR values and column indices of tile rows [r0, r1) in shared
// memory.  Returns the block offset of the tile.
template <typename T>
__device__ __forceinline__ int stage_tile(const Params<T> &P, int r0, int r1,
                                          T *sA, int *sC) {
  int b0 = P.rowptr[r0], b1 = P.rowptr[r1];
  int nv = (b1 - b0) * 9;
  const T *src = P.A + size_t(b0) * 9;
  // 16-byte vector loads on the aligned middle part, scalar edges.
  constexpr int VW = 16 / sizeof(T);
  uintptr_t a = reinterpret_cast<uintptr_t>(src);
  int head = int(((16 - (a & 15)) & 15) / sizeof(T));
  if (head > nv) head = nv;
  for (int k = threadIdx.x; k < head; k += kThreads) sA[k] = src[k];
  int nvec = (nv - head) / VW;
  const float4 *s4 = reinterpret_cast<const float4 *>(src + head);
  for (int k = threadIdx.x; k < nvec; k += kThreads) {
    float4 t = __ldcg(s4 + k);
    const T *tp = reinterpret_cast<const T *>(&t);
#pragma unroll
    for (int j = 0; j < VW; ++j) sA[head + k * VW + j] = tp[j];
  }
  for (int k = head + nvec * VW + threadIdx.x; k < nv; k += kThreads) sA[k] = src[k];
  for (int k = threadIdx.x; k < b1 - b0; k += kThreads) sC[k] = __ldg(P.colidx + b0 + k);
  __syncthreads();
  return b0;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
pcg_kernel(Params<T> P) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[kThreads / 32 + 1];
  T *sA = reinterpret_cast<T *>(smem);
  const int cap_blocks = kSmemBytes / (9 * sizeof(T) + sizeof(int));
  int *sC = reinterpret_cast<int *>(smem + size_t(cap_blocks) * 9 * sizeof(T));
  const int cta = blockIdx.x;
  const int G = P.n_ctas;
  double *part_pq = P.part, *part_rz = P.part + G, *part_rr = P.part + 2 * G,
         *part_r64 = P.part + 3 * G;
  unsigned gen = 0;
  const int t0 = P.cta_tile[cta], t1 = P.cta_tile[cta + 1];
  const double tol2 = P.tol2 * __ldcg(&P.st->rhs_norm2);

  double rz = reduce_partials(part_rz, G, red);  // r.z of the initial residual
  double rz_prev = 1.0, rmax2 = reduce_partials(part_rr, G, red);
  int it = 0, nref = 0, status = EOLC_NOT_CONVERGED;
  V4<T> *pold = P.pa, *pnew = P.pb;
  double last_rr64 = rmax2;
  bool converged = rmax2 <= tol2;
  while (!converged && it < P.max_iter) {
    // ---------------- P1: p = z + beta p_old, q = A p -----------------
    const T beta = it == 0 ? T(0) : T(rz / rz_prev);
    double pq = 0;
    for (int tile = t0; tile < t1; ++tile) {
      int r0 = P.tile_row[tile], r1 = P.tile_row[tile + 1];
      int b0 = stage_tile(P, r0, r1, sA, sC);
      int i = r0 + threadIdx.x;
      if (i < r1) {
        V4<T> zi = P.z[i], po = pold[i];
        V4<T> pi{zi.x + beta * po.x, zi.y + beta * po.y, zi.z + beta * po.z, T(0)};
        pnew[i] = pi;
        T a0 = 0, a1 = 0, a2 = 0;
        int q0 = P.rowptr[i], q1 = P.rowptr[i + 1];
        for (int k = q0; k < q1; ++k) {
          int j = sC[k - b0];
          V4<T> zj = P.z[j], pj = pold[j];
          T px = zj.x + beta * pj.x, py = zj.y + beta * pj.y, pz = zj.z + beta * pj.z;
          const T *blk = sA + size_t(k - b0) * 9;
          a0 += blk[0] * px + blk[1] * py + blk[2] * pz;
          a1 += blk[3] * px + blk[4] * py + blk[5] * pz;
          a2 += blk[6] * px + blk[7] * py + blk[8] * pz;
        }
        V4<T> m = P.fmask[i];
        V4<T> qi{a0 * m.x, a1 * m.y, a2 * m.z, T(0)};
        P.q[i] = qi;
        pq += double(pi.x) * double(qi.x) + double(pi.y) * double(qi.y) +
              double(pi.z) * double(qi.z);
      }
      __syncthreads();
    }
    pq = block_sum(pq, red);
    if (threadIdx.x == 0) part_pq[cta] = pq;
    if (!grid_barrier(P.bar, G, gen, P.st)) return;
    ++it;
    // ---------------- P2: update ----------------------------------------
    double pq_all = reduce_partials(part_pq, G, red);
    if (!(pq_all > 0.0)) {
      status = isfinite(pq_all) ? EOLC_BREAKDOWN : EOLC_NONFINITE;
      break;
    }
    const double alpha_d = rz / pq_all;
    const T alpha = T(alpha_d);
    double rzn = 0, rr = 0;
    for (int tile = t0; tile < t1; ++tile) {
      int r0 = P.tile_row[tile], r1 = P.tile_row[tile + 1];
      int i = r0 + threadIdx.x;
      if (i < r1) {
        V4<T> pi = pnew[i], qi = P.q[i], ri = P.r[i], xa = P.xacc[i];
        xa.x += alpha * pi.x; xa.y += alpha * pi.y; xa.z += alpha * pi.z;
        ri.x -= alpha * qi.x; ri.y -= alpha * qi.y; ri.z -= alpha * qi.z;
        P.xacc[i] = xa;
        P.r[i] = ri;
        V4<T> zi = apply_pc(P, i, ri);
        P.z[i] = zi;
        rzn += double(ri.x) * double(zi.x) + double(ri.y) * double(zi.y) +
               double(ri.z) * double(zi.z);
        rr += double(ri.x) * double(ri.x) + double(ri.y) * double(ri.y) +
              double(ri.z) * double(ri.z);
      }
    }
    rzn = block_sum(rzn, red);
    rr = block_sum(rr, red);
    if (threadIdx.x == 0) { part_rz[cta] = rzn; part_rr[cta] = rr; }
    if (!grid_barrier(P.bar, G, gen, P.st)) return;
    rz_prev = rz;
    rz = reduce_partials(part_rz, G, red);
    double rr_all = reduce_partials(part_rr, G, red);
    V4<T> *tmp = pold; pold = pnew; pnew = tmp;
    if (!isfinite(rr_all)) { status = EOLC_NONFINITE; break; }
    bool need_ru = rr_all < kDelta * kDelta * rmax2 || rr_all <= tol2 ||
                   it >= P.max_iter;
    if (!need_ru) continue;
    // ---------------- reliable update --------------------------------------
    // RU1: fold the low-precision update into the FP64 solution.
    for (int tile = t0; tile < t1; ++tile) {
      int r0 = P.tile_row[tile], r1 = P.tile_row[tile + 1];
      int i = r0 + threadIdx.x;
      if (i < r1) {
        V4<T> xa = P.xacc[i];
        V4<double> x = P.x64[i];
        x.x += double(xa.x); x.y += double(xa.y); x.z += double(xa.z);
        P.x64[i] = x;
        P.xacc[i] = V4<T>{T(0), T(0), T(0), T(0)};
      }
    }
    if (!grid_barrier(P.bar, G, gen, P.st)) return;
    // RU2: r64 = rhs - A x64 in FP64 arithmetic; r, z restarted from it.
    double rr64 = 0, rz2 = 0;
    for (int tile = t0; tile < t1; ++tile) {
      int r0 = P.tile_row[tile], r1 = P.tile_row[tile + 1];
      int b0 = stage_tile(P, r0, r1, sA, sC);
      int i = r0 + threadIdx.x;
      if (i < r1) {
        double a0 = 0, a1 = 0, a2 = 0;
        for (int k = P.rowptr[i]; k < P.rowptr[i + 1]; ++k) {
          V4<double> xj = P.x64[sC[k - b0]];
          const T *blk = sA + size_t(k - b0) * 9;
          a0 += double(blk[0]) * xj.x + double(blk[1]) * xj.y + double(blk[2]) * xj.z;
          a1 += double(blk[3]) * xj.x + double(blk[4]) * xj.y + double(blk[5]) * xj.z;
          a2 += double(blk[6]) * xj.x + double(blk[7]) * xj.y + double(blk[8]) * xj.z;
        }
        V4<double> b = P.rhs[i];
        V4<T> m = P.fmask[i];
        double e0 = (b.x - a0) * double(m.x), e1 = (b.y - a1) * double(m.y),
               e2 = (b.z - a2) * double(m.z);
        rr64 += e0 * e0 + e1 * e1 + e2 * e2;
        V4<T> ri{T(e0), T(e1), T(e2), T(0)};
        P.r[i] = ri;
        V4<T> zi = apply_pc(P, i, ri);
        P.z[i] = zi;
        rz2 += double(ri.x) * double(zi.x) + double(ri.y) * double(zi.y) +
               double(ri.z) * double(zi.z);
      }
      __syncthreads();
    }
    rr64 = block_sum(rr64, red);
    rz2 = block_sum(rz2, red);
    if (threadIdx.x == 0) { part_r64[cta] = rr64; part_rz[cta] = rz2; }
    if (!grid_barrier(P.bar, G, gen, P.st)) return;
    ++nref;
    last_rr64 = reduce_partials(part_r64, G, red);
    rz = reduce_partials(part_rz, G, red);
    rmax2 = last_rr64;
    if (!isfinite(last_rr64)) { status = EOLC_NONFINITE; break; }
    if (last_rr64 <= tol2) converged = true;
  }
  if (converged) status = EOLC_OK;
  if (cta == 0 && threadIdx.x == 0) {
    atomicCAS(&P.st->status, EOLC_OK, status);
    P.st->iterations = it;
    P.st->refinements = nref;
    P.st->rel_res = P.st->rhs_norm2 > 0 ? sqrt(last_rr64 / P.st->rhs_norm2) : 0.0;
  }
}

// ---- set-up kernels (one launch each per solve) -----------------------------

// rhs = mask * (-b - A beq_full) in FP64 (A promoted), plus the
// preconditioner, r = rhs, z = M^-1 r, x = 0.
template <typename T>
__global__ void setup_kernel(int n_nodes, const int *rowptr, const int *colidx,
                             const int *diag, const T *A, const double *b,
                             const double *beq_full, const uint8_t *pinned,
                             int block_pc, V4<double> *rhs, V4<double> *x64,
                             V4<T> *r, V4<T> *z, V4<T> *pa, V4<T> *xacc,
                             T *pc, V4<T> *fmask) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  double a[3] = {0, 0, 0};
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    int j = colidx[k];
    const T *blk = A + size_t(k) * 9;
    for (int rr = 0; rr < 3; ++rr)
      for (int c = 0; c < 3; ++c) a[rr] += double(blk[3 * rr + c]) * beq_full[3 * j + c];
  }
  T m[3];
  double e[3];
  for (int c = 0; c < 3; ++c) {
    m[c] = pinned[3 * i + c] ? T(0) : T(1);
    e[c] = pinned[3 * i + c] ? 0.0 : (-b[3 * i + c] - a[c]);
  }
  rhs[i] = V4<double>{e[0], e[1], e[2], 0.0};
  x64[i] = V4<double>{0.0, 0.0, 0.0, 0.0};
  fmask[i] = V4<T>{m[0], m[1], m[2], T(0)};
  const T *D = A + size_t(diag[i]) * 9;
  V4<T> ri{T(e[0]), T(e[1]), T(e[2]), T(0)};
  V4<T> zi;
  if (block_pc) {
    // inverse of the free-free part of the diagonal block (pinned rows and
    // columns replaced by the identity, then masked)
    double M[3][3];
    for (int rr = 0; rr < 3; ++rr)
      for (int c = 0; c < 3; ++c)
        M[rr][c] = (m[rr] == T(0) || m[c] == T(0)) ? (rr == c ? 1.0 : 0.0)
                                                   : double(D[3 * rr + c]);
    double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
    double inv[9];
    if (det != 0.0) {
      double id = 1.0 / det;
      inv[0] = c00 * id;
      inv[1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) * id;
      inv[2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) * id;
      inv[3] = c01 * id;
      inv[4] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) * id;
      inv[5] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) * id;
      inv[6] = c02 * id;
      inv[7] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) * id;
      inv[8] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) * id;
    } else {
      for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }
    for (int rr = 0; rr < 3; ++rr)
      for (int c = 0; c < 3; ++c)
        pc[size_t(9) * i + 3 * rr + c] = T(inv[3 * rr + c] * double(m[rr]) * double(m[c]));
    const T *B = pc + size_t(9) * i;
    zi.x = B[0] * ri.x + B[1] * ri.y + B[2] * ri.z;
    zi.y = B[3] * ri.x + B[4] * ri.y + B[5] * ri.z;
    zi.z = B[6] * ri.x + B[7] * ri.y + B[8] * ri.z;
  } else {
    // Eigen's DiagonalPreconditioner: 1/diag, 1 where the diagonal is 0
    T d[3];
    for (int c = 0; c < 3; ++c) {
      T dd = D[4 * c];
      d[c] = (dd != T(0) ? T(1) / dd : T(1)) * m[c];
      pc[size_t(4) * i + c] = d[c];
    }
    pc[size_t(4) * i + 3] = T(0);
    zi.x = d[0] * ri.x; zi.y = d[1] * ri.y; zi.z = d[2] * ri.z;
  }
  zi.w = T(0);
  r[i] = ri;
  z[i] = zi;
  pa[i] = V4<T>{T(0), T(0), T(0), T(0)};
  xacc[i] = V4<T>{T(0), T(0), T(0), T(0)};
}

// Per-CTA-of-setup partial sums of ||rhs||^2 and r.z, reduced by one block.
template <typename T>
__global__ void init_sums_kernel(int n_nodes, const V4<double> *rhs,
                                 const V4<T> *r, const V4<T> *z, double *part,
                                 int G, DevStatus *st) {
  __shared__ double red[kThreads / 32 + 1];
  double s_rhs = 0, s_rz = 0;
  for (int i = threadIdx.x; i < n_nodes; i += kThreads) {
    V4<double> b = rhs[i];
    V4<T> ri = r[i], zi = z[i];
    s_rhs += b.x * b.x + b.y * b.y + b.z * b.z;
    s_rz += double(ri.x) * double(zi.x) + double(ri.y) * double(zi.y) +
            double(ri.z) * double(zi.z);
  }
  s_rhs = block_sum(s_rhs, red);
  s_rz = block_sum(s_rz, red);
  for (int k = threadIdx.x; k < 5 * G; k += kThreads) part[k] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    part[G] = s_rz;       // part_rz
    part[2 * G] = s_rhs;  // part_rr (initial residual = rhs since x0 = 0)
    st->status = EOLC_OK;
    st->iterations = 0;
    st->refinements = 0;
    st->rel_res = s_rhs > 0 ? 1.0 : 0.0;
    st->rhs_norm2 = s_rhs;
  }
}

template <typename T>
__global__ void finish_kernel(int n_nodes, const V4<double> *x64,
                              const double *beq_full, const uint8_t *pinned,
                              double *v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  V4<double> x = x64[i];
  double xs[3] = {x.x, x.y, x.z};
  for (int c = 0; c < 3; ++c)
    v[3 * i + c] = pinned[3 * i + c] ? beq_full[3 * i + c] : xs[c];
}

}  // namespace

// ---------------------------------------------------------------------------
struct SolveWork {
  int n_nodes = 0, n_blocks = 0, G = 0, prec = -1, block_pc = -1;
  DevBuf<unsigned char> vecs;
  DevBuf<double> part;
  DevBuf<unsigned> bar;
  DevBuf<DevStatus> st;
  DevBuf<int> tile_row, cta_tile;
  DevBuf<unsigned char> pc;
  std::vector<int> h_tile_row, h_cta_tile;
};

void free_solve_work(SolveWork *w) { delete w; }

namespace {

template <typename T>
eolc_status run_pcg_t(SolveWork *&w, const PcgArgs &a, eolc_solve_info *info,
                      cudaStream_t s, std::string &err) {
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes;
  const T *A = std::is_same<T, double>::value
                   ? reinterpret_cast<const T *>(a.A64)
                   : reinterpret_cast<const T *>(a.A32);
  int dev = 0;
  cudaGetDevice(&dev);
  int n_sm = 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int cap_blocks = kSmemBytes / (9 * sizeof(T) + sizeof(int));
  size_t smem = size_t(cap_blocks) * 9 * sizeof(T) + size_t(cap_blocks) * sizeof(int);
  cudaFuncSetAttribute(pcg_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(smem));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_kernel<T>, kThreads, smem);
  if (per_sm < 1) { err = "pcg kernel does not fit on an SM"; return EOLC_CUDA_ERROR; }
  per_sm = std::min(per_sm, 2);
  const int want_G = n_sm * per_sm;
  const int prec = std::is_same<T, double>::value ? 0 : 1;
  if (!w) w = new SolveWork();
  if (w->n_nodes != N || w->n_blocks != Tp.n_blocks || w->prec != prec ||
      w->G != want_G || w->block_pc != (a.precond == EOLC_PC_BLOCK_JACOBI)) {
    // tiles: <= kTileRows rows and <= cap_blocks blocks each
    std::vector<int> rowptr(N + 1);
    cudaMemcpy(rowptr.data(), Tp.rowptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost);
    std::vector<int> tiles{0};
    int start = 0;
    for (int i = 0; i < N; ++i) {
      int rows = i + 1 - start;
      int blocks = rowptr[i + 1] - rowptr[start];
      if (rowptr[i + 1] - rowptr[i] > cap_blocks) { err = "row too long"; return EOLC_BAD_ARG; }
      if (rows > kTileRows || blocks > cap_blocks) {
        tiles.push_back(i);
        start = i;
      }
    }
    tiles.push_back(N);
    int nt = int(tiles.size()) - 1;
    int G = std::min(want_G, nt);
    // contiguous tile ranges balanced by block count
    std::vector<int> cta(G + 1, nt);
    cta[0] = 0;
    long long total = rowptr[N];
    int t = 0;
    for (int c = 1; c < G; ++c) {
      long long target = total * c / G;
      while (t < nt && rowptr[tiles[t]] < target) ++t;
      cta[c] = std::max(t, cta[c - 1] + 1);
      if (cta[c] > nt - (G - c)) cta[c] = nt - (G - c);
    }
    w->h_tile_row = tiles;
    w->h_cta_tile = cta;
    w->G = G;
    w->n_nodes = N;
    w->n_blocks = Tp.n_blocks;
    w->prec = prec;
    w->block_pc = a.precond == EOLC_PC_BLOCK_JACOBI;
    cudaError_t e1 = w->tile_row.upload(tiles.data(), tiles.size(), s);
    cudaError_t e2 = w->cta_tile.upload(cta.data(), cta.size(), s);
    size_t vb = size_t(N) * (sizeof(V4<double>) * 2 + sizeof(V4<T>) * 7);
    cudaError_t e3 = w->vecs.resize(vb);
    cudaError_t e4 = w->part.resize(size_t(5) * G);
    cudaError_t e5 = w->bar.resize(2);
    cudaError_t e6 = w->st.resize(1);
    cudaError_t e7 = w->pc.resize(size_t(N) * 9 * sizeof(T));
    for (cudaError_t e : {e1, e2, e3, e4, e5, e6, e7})
      if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  }
  const int G = w->G;
  unsigned char *vp = w->vecs.p;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<T> *vr = reinterpret_cast<V4<T> *>(vp);
  V4<T> *r = vr, *z = vr + N, *pa = vr + 2 * N, *pb = vr + 3 * N, *q = vr + 4 * N,
        *xacc = vr + 5 * N, *fmask = vr + 6 * N;
  T *pc = reinterpret_cast<T *>(w->pc.p);
  int bpc = a.precond == EOLC_PC_BLOCK_JACOBI ? 1 : 0;
  setup_kernel<T><<<(N + 127) / 128, 128, 0, s>>>(
      N, Tp.rowptr.p, Tp.colidx.p, Tp.diag.p, A, a.b, a.beq_full, a.pinned, bpc,
      rhs, x64, r, z, pa, xacc, pc, fmask);
  init_sums_kernel<T><<<1, kThreads, 0, s>>>(N, rhs, r, z, w->part.p, G, w->st.p);
  cudaMemsetAsync(w->bar.p, 0, sizeof(unsigned) * 2, s);
  Params<T> P;
  P.n_nodes = N;
  P.n_ctas = G;
  P.rowptr = Tp.rowptr.p;
  P.colidx = Tp.colidx.p;
  P.A = A;
  P.tile_row = w->tile_row.p;
  P.cta_tile = w->cta_tile.p;
  P.rhs = rhs;
  P.x64 = x64;
  P.r = r; P.z = z; P.pa = pa; P.pb = pb; P.q = q; P.xacc = xacc;
  P.pc = pc;
  P.fmask = fmask;
  P.part = w->part.p;
  P.bar = w->bar.p;
  P.st = w->st.p;
  P.max_iter = a.max_iter;
  P.block_pc = bpc;
  P.tol2 = a.rel_tol * a.rel_tol;
  DevStatus hs;
  void *args[] = {&P};
  cudaError_t e = cudaLaunchCooperativeKernel((void *)pcg_kernel<T>, dim3(G), dim3(kThreads),
                                  args, smem, s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  finish_kernel<T><<<(N + 127) / 128, 128, 0, s>>>(N, x64, a.beq_full, a.pinned, a.v);
  cudaMemcpyAsync(&hs, w->st.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  if (info) {
    info->status = hs.status;
    info->iterations = hs.iterations;
    info->refinements = hs.refinements;
    info->used_fallback = 0;
    info->rel_res = hs.rel_res;
  }
  if (hs.status != EOLC_OK) {
    err = hs.status == EOLC_TIMEOUT ? "grid barrier timed out"
          : hs.status == EOLC_BREAKDOWN ? "CG breakdown: p'Ap <= 0"
          : hs.status == EOLC_NONFINITE ? "non-finite value in CG"
                                        : "CG did not converge";
  }
  return eolc_status(hs.status);
}

}  // namespace

eolc_status run_pcg(SolveWork *&w, const PcgArgs &a, eolc_solve_info *info,
                    cudaStream_t s, std::string &err) {
  if (a.precision == EOLC_PREC_FP64) return run_pcg_t<double>(w, a, info, s, err);
  return run_pcg_t<float>(w, a, info, s, err);
}

}  // namespace eolc
