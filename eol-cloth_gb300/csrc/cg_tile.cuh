// Tile machinery shared by the persistent CG kernels (pcg.cu: one system
// across all SMs; batch.cu: many systems, one CTA cluster each).
//
// A tile is a run of consecutive block rows whose BSR values, 16-bit
// tile-local column indices and row pointers are staged into shared memory
// with aligned 16-byte copies; its halo (the distinct columns its blocks
// touch, listed once per topology) is staged as one vector window.  Every
// function here is parameterised by a tile configuration C (threads per CTA,
// threads per block row, shared-memory budget for values and windows), so
// the same code runs under each shape the batch autotuner tries.
#pragma once

#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "cg_common.cuh"

namespace eolc {
namespace cgc {
namespace {

// Reliable-update trigger: the iterated residual has dropped by this factor
// since the last true-residual recomputation (convergence is only ever
// declared on a recomputed residual).  kDelta: one recomputation per decade,
// the best for the long Jacobi iterations (at 1e-2 the FP32 recurrence
// drifts enough to cost them ~7% more iterations at 256^2).  The two-level
// kernels' ~115-200 iterations make the FP64 recomputation (an FP64 product,
// about 1/64 of the FP32 rate on this GPU) a large share of the solve:
// kDeltaPatch, one per three decades for the patch-Chebyshev method (the
// same iteration count, 2% faster than one per two decades at 256^2);
// kDeltaLearned, one per two decades for the learned G, whose recurrence
// drifts further (one per three decades left solves unconverged at twice
// Jacobi's iteration count).
constexpr double kDelta = 0.1;
constexpr double kDeltaPatch = 1e-3;
constexpr double kDeltaLearned = 1e-2;

// THREADS threads per CTA, ROWT threads per block row, VALKB KiB of staged
// values + local columns, WINF window nodes per tile in FP32 (3/4 of it in
// FP64, whose window entries are twice as wide).
template <int THREADS, int ROWT, int VALKB, int WINF>
struct TileCfg {
  static constexpr int kThreads = THREADS;
  static constexpr int kRowThreads = ROWT;
  static constexpr int kTileRows = THREADS / ROWT;
  static constexpr int kValBytes = VALKB * 1024;
  static constexpr int kWinMaxF = WINF;
  static constexpr int kWinMaxD = WINF * 3 / 4;
  static_assert(32 % ROWT == 0 && THREADS % 32 == 0, "rows must not straddle warps");
  template <typename T>
  __host__ __device__ static constexpr int win_max() {
    return sizeof(T) == 8 ? kWinMaxD : kWinMaxF;
  }
  // values (9 T) + one 16-bit local column per block, with 16-byte padding
  template <typename T>
  __host__ __device__ static constexpr int cap_blocks() {
    return (kValBytes - 64) / (9 * int(sizeof(T)) + 2);
  }
  // values | local columns | window (an FP64 x window plus an inner-type p
  // window, or the u window)
  template <typename T>
  __host__ __device__ static constexpr size_t smem_bytes() {
    return size_t(kValBytes) + size_t(win_max<T>()) * (sizeof(V4<double>) + sizeof(V4<T>));
  }
};

// Deterministic CTA-wide sums of three accumulators (fixed butterfly tree,
// fixed warp order).  red must hold 3 * (C::kThreads / 32 + 1) accumulators.
template <class C, typename T>
__device__ __forceinline__ void block_sum3(typename Acc<T>::V &a, typename Acc<T>::V &b,
                                           typename Acc<T>::V &c, typename Acc<T>::V *red) {
  using A = Acc<T>;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = A::add(a, A::shfl_xor(a, o));
    b = A::add(b, A::shfl_xor(b, o));
    c = A::add(c, A::shfl_xor(c, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = C::kThreads / 32;
  __syncthreads();
  if (lane == 0) { red[3 * warp] = a; red[3 * warp + 1] = b; red[3 * warp + 2] = c; }
  __syncthreads();
  if (warp == 0) {
    typename A::V x = lane < NW ? red[3 * lane] : A::zero();
    typename A::V y = lane < NW ? red[3 * lane + 1] : A::zero();
    typename A::V z = lane < NW ? red[3 * lane + 2] : A::zero();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      x = A::add(x, A::shfl_xor(x, o));
      y = A::add(y, A::shfl_xor(y, o));
      z = A::add(z, A::shfl_xor(z, o));
    }
    if (lane == 0) { red[3 * NW] = x; red[3 * NW + 1] = y; red[3 * NW + 2] = z; }
  }
  __syncthreads();
  a = red[3 * NW]; b = red[3 * NW + 1]; c = red[3 * NW + 2];
}

// Polls before a bounded device wait (grid barrier, neighbour exchange)
// gives up: the default of eolc_set_wait_limit, seconds of polling.
constexpr long long kDefaultSpinLimit = 1ll << 25;

// ---- grid barrier -----------------------------------------------------------
// Monotonic arrival counter: CTA thread 0 adds 1 with release semantics and
// polls (acquire) until the count reaches n_ctas * epoch.  Bounded spin: after
// `limit` polls the barrier records EOLC_TIMEOUT and returns false.  While it waits
// it reads the status every 1024 polls, so that a CTA that gave up elsewhere
// ends the others' waits early; a barrier that completes does not read it
// (one L2 round trip fewer per barrier).
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned nblocks,
                                             unsigned &epoch, DevStatus *st,
                                             long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(bar[0]);
    epoch += 1u;
    const unsigned target = nblocks * epoch;
    int ok = 1;
    count.fetch_add(1u, cuda::memory_order_release);
    long long spins = 0;
    while (count.load(cuda::memory_order_acquire) < target) {
      ++spins;
      if (spins > limit) {
        atomicCAS(&st->status, EOLC_OK, EOLC_TIMEOUT);
        ok = 0;
        break;
      }
      if ((spins & 1023) == 0) {
        cuda::atomic_ref<int, cuda::thread_scope_device> sref(st->status);
        if (sref.load(cuda::memory_order_relaxed) != EOLC_OK) { ok = 0; break; }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Every CTA reduces the per-CTA partial triples in the same fixed order, so
// all CTAs take the same branch decisions.
template <class C, typename T>
__device__ __forceinline__ void reduce_partials3(const typename Acc<T>::V *part, int G,
                                                 typename Acc<T>::V &a, typename Acc<T>::V &b,
                                                 typename Acc<T>::V &c, typename Acc<T>::V *red) {
  using A = Acc<T>;
  using V = typename A::V;
  a = b = c = A::zero();
  for (int k = threadIdx.x; k < G; k += C::kThreads) {
    const double *pd = reinterpret_cast<const double *>(part + 3 * k);
    double v0 = __ldcg(pd), v1 = __ldcg(pd + 1), v2 = __ldcg(pd + 2);
    a = A::add(a, *reinterpret_cast<V *>(&v0));
    b = A::add(b, *reinterpret_cast<V *>(&v1));
    c = A::add(c, *reinterpret_cast<V *>(&v2));
  }
  block_sum3<C, T>(a, b, c, red);
}

template <typename T>
struct Params {
  int n_nodes;
  int n_ctas;
  const int *rowptr;
  const T *A;               // inner matrix (FP32 or FP64); promoted to FP64
                            // for the true residual
  const uint16_t *lcol;     // tile-local column of every block
  const int *tile_row;      // tile boundaries (n_tiles + 1)
  const int *tile_wptr;     // window list offsets (n_tiles + 1)
  const int *wlist;         // window node ids, per tile
  const int *cta_tile;      // CTA -> first tile (n_ctas + 1)
  const V4<double> *rhs;    // masked rhs of the reduced system
  V4<double> *x64;
  V4<T> *r[2], *w[2], *s[2];
  V4<T> *p, *xacc;
  const T *pc;              // preconditioner: 4 per node (Jacobi) or 9 (block)
  const V4<T> *fmask;       // 1 on free DOFs, 0 on pinned
  double *part;             // partial sums: 2 sets x 3 values x n_ctas
  unsigned *bar;
  DevStatus *st;
  long long spin_limit;     // polls before a grid barrier gives up
  double tol2;              // tol^2 (scaled by ||rhs||^2 on the device)
  int max_iter;
  int block_pc;             // 0 = point Jacobi, 1 = block Jacobi
};

template <typename T>
__device__ __forceinline__ V4<T> apply_pc(const Params<T> &P, int i, V4<T> r) {
  V4<T> z;
  if (P.block_pc) {
    const T *B = P.pc + size_t(9) * i;
    z.x = B[0] * r.x + B[1] * r.y + B[2] * r.z;
    z.y = B[3] * r.x + B[4] * r.y + B[5] * r.z;
    z.z = B[6] * r.x + B[7] * r.y + B[8] * r.z;
  } else {
    V4<T> d = reinterpret_cast<const V4<T> *>(P.pc)[i];
    z.x = d.x * r.x; z.y = d.y * r.y; z.z = d.z * r.z;
  }
  z.w = T(0);
  return z;
}

// Copies n elements (of size E) starting at src into shared memory with
// 16-byte loads and stores; returns the element offset of src inside dst.
// The source allocation is padded so the rounded-up tail stays inside it.
template <class C, typename E>
__device__ __forceinline__ int stage_aligned(const E *src, int n, E *dst) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(src);
  const float4 *s4 = reinterpret_cast<const float4 *>(a & ~uintptr_t(15));
  const int off = int((a & 15) / sizeof(E));
  const int nvec = int((size_t(off + n) * sizeof(E) + 15) / 16);
  float4 *d4 = reinterpret_cast<float4 *>(dst);
  for (int k = threadIdx.x; k < nvec; k += C::kThreads) d4[k] = __ldcg(s4 + k);
  return off;
}

// Per-tile metadata of this CTA, loaded once per solve.
constexpr int kMaxCtaTiles = 64;
struct TileMeta {
  int r0, r1, b0, b1, w0, wn;
};

// Stages a tile's values, local columns and row pointers; returns pointers
// to the tile's first element inside shared memory.
template <class C, typename T>
__device__ __forceinline__ void stage_tile(const Params<T> &P, const TileMeta &tm,
                                           unsigned char *vals, const T *&sA,
                                           const uint16_t *&sL, int *sRow) {
  const int nb = tm.b1 - tm.b0;
  T *dA = reinterpret_cast<T *>(vals);
  const int offA = stage_aligned<C>(P.A + size_t(tm.b0) * 9, nb * 9, dA);
  const size_t abytes = (size_t(offA + nb * 9) * sizeof(T) + 31) & ~size_t(15);
  uint16_t *dL = reinterpret_cast<uint16_t *>(vals + abytes);
  const int offL = stage_aligned<C>(P.lcol + tm.b0, nb, dL);
  for (int k = threadIdx.x; k <= tm.r1 - tm.r0; k += C::kThreads)
    sRow[k] = __ldg(P.rowptr + tm.r0 + k) - tm.b0;
  sA = dA + offA;
  sL = dL + offL;
}

template <typename T>
__device__ __forceinline__ T dot3(V4<T> a, V4<T> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// One CG phase over this CTA's tiles.
//   kInit:  u = M r (current r), w = A u                  -> w[cur]
//   else:   s' = w + beta s, r' = r - alpha s', u = M r' (every halo node),
//           w' = A u, p = M r + beta p, x += alpha p
//           -> r'[nxt], s'[nxt], w'[nxt], p, xacc
// Accumulates (r'.u, w'.u, r'.r') into g, d, rr.
template <class C, typename T, bool kInit>
__device__ __forceinline__ void cg_phase(const Params<T> &P, const TileMeta *tiles,
                                         int ntiles, int cur, T alpha, T beta,
                                         unsigned char *smem, typename Acc<T>::V &g,
                                         typename Acc<T>::V &d, typename Acc<T>::V &rr) {
  using A = Acc<T>;
  const int nxt = cur ^ 1;
  V4<T> *sU = reinterpret_cast<V4<T> *>(smem + C::kValBytes);
  __shared__ V4<T> sRn[C::kTileRows];
  __shared__ int sRow[C::kTileRows + 1];
  const int lrow = threadIdx.x / C::kRowThreads, quarter = threadIdx.x % C::kRowThreads;
  for (int t = 0; t < ntiles; ++t) {
    const TileMeta tm = tiles[t];
    const int i = tm.r0 + lrow;
    const bool owner = i < tm.r1 && quarter == 0;
    // epilogue operands, prefetched so their latency overlaps the staging
    V4<T> m{}, ro{}, po{}, xa{};
    if (owner) {
      m = P.fmask[i];
      if (!kInit) { ro = P.r[cur][i]; po = P.p[i]; xa = P.xacc[i]; }
    }
    const T *sA;
    const uint16_t *sL;
    stage_tile<C>(P, tm, smem, sA, sL, sRow);
    for (int j = threadIdx.x; j < tm.wn; j += C::kThreads) {
      const int node = __ldg(P.wlist + tm.w0 + j);
      V4<T> rn = P.r[cur][node];
      if (!kInit) {
        const V4<T> so = P.s[cur][node], wo = P.w[cur][node];
        const V4<T> sn{wo.x + beta * so.x, wo.y + beta * so.y, wo.z + beta * so.z, T(0)};
        rn = V4<T>{rn.x - alpha * sn.x, rn.y - alpha * sn.y, rn.z - alpha * sn.z, T(0)};
        if (node >= tm.r0 && node < tm.r1) {
          P.s[nxt][node] = sn;
          P.r[nxt][node] = rn;
        }
      }
      if (node >= tm.r0 && node < tm.r1) sRn[node - tm.r0] = rn;
      sU[j] = apply_pc(P, node, rn);
    }
    __syncthreads();
    T a0 = 0, a1 = 0, a2 = 0;
    if (i < tm.r1) {
      const int q0 = sRow[lrow], q1 = sRow[lrow + 1];
#pragma unroll 2
      for (int k = q0 + quarter; k < q1; k += C::kRowThreads) {
        const V4<T> u = sU[sL[k]];
        const T *blk = sA + size_t(k) * 9;
        a0 += blk[0] * u.x + blk[1] * u.y + blk[2] * u.z;
        a1 += blk[3] * u.x + blk[4] * u.y + blk[5] * u.z;
        a2 += blk[6] * u.x + blk[7] * u.y + blk[8] * u.z;
      }
    }
#pragma unroll
    for (int o = 1; o < C::kRowThreads; o <<= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (owner) {
      const V4<T> wn4{a0 * m.x, a1 * m.y, a2 * m.z, T(0)};
      const V4<T> rn = sRn[lrow];
      const V4<T> un = apply_pc(P, i, rn);
      if (kInit) {
        P.w[cur][i] = wn4;
      } else {
        P.w[nxt][i] = wn4;
        // p = M r_old + beta p ; x += alpha p
        const V4<T> uo = apply_pc(P, i, ro);
        const V4<T> pi{uo.x + beta * po.x, uo.y + beta * po.y, uo.z + beta * po.z, T(0)};
        P.p[i] = pi;
        xa.x += alpha * pi.x; xa.y += alpha * pi.y; xa.z += alpha * pi.z;
        P.xacc[i] = xa;
      }
      g = A::addf(g, dot3(rn, un));
      d = A::addf(d, dot3(wn4, un));
      rr = A::addf(rr, dot3(rn, rn));
    }
    __syncthreads();
  }
}

// Reliable update, second step: r = rhs - A x64 (FP64 arithmetic) and
// s = A p, written to r[cur], s[cur].  Accumulates r.r (FP64) into rr64.
template <class C, typename T>
__device__ __forceinline__ void ru_residual(const Params<T> &P, const TileMeta *tiles,
                                           int ntiles, int cur, unsigned char *smem,
                                           double &rr64) {
  V4<double> *sX = reinterpret_cast<V4<double> *>(smem + C::kValBytes);
  V4<T> *sP = reinterpret_cast<V4<T> *>(smem + C::kValBytes +
                                         size_t(C::template win_max<T>()) * sizeof(V4<double>));
  __shared__ int sRow[C::kTileRows + 1];
  const int lrow = threadIdx.x / C::kRowThreads, quarter = threadIdx.x % C::kRowThreads;
  for (int t = 0; t < ntiles; ++t) {
    const TileMeta tm = tiles[t];
    const T *sA;
    const uint16_t *sL;
    stage_tile<C>(P, tm, smem, sA, sL, sRow);
    for (int j = threadIdx.x; j < tm.wn; j += C::kThreads) {
      const int node = __ldg(P.wlist + tm.w0 + j);
      sX[j] = P.x64[node];
      sP[j] = P.p[node];
    }
    __syncthreads();
    const int i = tm.r0 + lrow;
    double a0 = 0, a1 = 0, a2 = 0;
    T c0 = 0, c1 = 0, c2 = 0;
    if (i < tm.r1) {
      const int q0 = sRow[lrow], q1 = sRow[lrow + 1];
      for (int k = q0 + quarter; k < q1; k += C::kRowThreads) {
        const V4<double> xj = sX[sL[k]];
        const V4<T> pj = sP[sL[k]];
        const T *blk = sA + size_t(k) * 9;
        a0 += double(blk[0]) * xj.x + double(blk[1]) * xj.y + double(blk[2]) * xj.z;
        a1 += double(blk[3]) * xj.x + double(blk[4]) * xj.y + double(blk[5]) * xj.z;
        a2 += double(blk[6]) * xj.x + double(blk[7]) * xj.y + double(blk[8]) * xj.z;
        c0 += blk[0] * pj.x + blk[1] * pj.y + blk[2] * pj.z;
        c1 += blk[3] * pj.x + blk[4] * pj.y + blk[5] * pj.z;
        c2 += blk[6] * pj.x + blk[7] * pj.y + blk[8] * pj.z;
      }
    }
#pragma unroll
    for (int o = 1; o < C::kRowThreads; o <<= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
      c0 += __shfl_xor_sync(0xffffffffu, c0, o);
      c1 += __shfl_xor_sync(0xffffffffu, c1, o);
      c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    }
    if (i < tm.r1 && quarter == 0) {
      const V4<double> b = P.rhs[i];
      const V4<T> m = P.fmask[i];
      const double e0 = (b.x - a0) * double(m.x), e1 = (b.y - a1) * double(m.y),
                   e2 = (b.z - a2) * double(m.z);
      rr64 += e0 * e0 + e1 * e1 + e2 * e2;
      P.r[cur][i] = V4<T>{T(e0), T(e1), T(e2), T(0)};
      P.s[cur][i] = V4<T>{c0 * m.x, c1 * m.y, c2 * m.z, T(0)};
    }
    __syncthreads();
  }
}

// ---- tile phases of PCG with a non-local preconditioner G (pattern of A) ----
template <class C, typename T>
__device__ __forceinline__ void stage_matrix(const T *M, const uint16_t *lcol, const int *rowptr,
                                             const TileMeta &tm, unsigned char *vals,
                                             const T *&sA, const uint16_t *&sL, int *sRow) {
  const int nb = tm.b1 - tm.b0;
  T *dA = reinterpret_cast<T *>(vals);
  const int offA = stage_aligned<C>(M + size_t(tm.b0) * 9, nb * 9, dA);
  const size_t abytes = (size_t(offA + nb * 9) * sizeof(T) + 31) & ~size_t(15);
  uint16_t *dL = reinterpret_cast<uint16_t *>(vals + abytes);
  const int offL = stage_aligned<C>(lcol + tm.b0, nb, dL);
  for (int k = threadIdx.x; k <= tm.r1 - tm.r0; k += C::kThreads)
    sRow[k] = __ldg(rowptr + tm.r0 + k) - tm.b0;
  sA = dA + offA;
  sL = dL + offL;
}

enum GenMode { kGenZ = 0, kGenP = 1, kGenR = 2 };

template <class C, typename T, int kMode>
__device__ __forceinline__ void gen_phase(const Params<T> &P, const T *Gm, const TileMeta *tiles,
                                          int ntiles, int rcur, int pold, T alpha, T beta,
                                          unsigned char *smem, typename Acc<T>::V &a1,
                                          typename Acc<T>::V &a2) {
  using A = Acc<T>;
  V4<T> *sU = reinterpret_cast<V4<T> *>(smem + C::kValBytes);
  __shared__ V4<T> sOwn[C::kTileRows];
  __shared__ int sRow[C::kTileRows + 1];
  const int lrow = threadIdx.x / C::kRowThreads, quarter = threadIdx.x % C::kRowThreads;
  V4<T> *z = P.w[0], *q = P.w[1];
  V4<T> *po = P.s[pold], *pn = P.s[pold ^ 1];
  const T *M = kMode == kGenP ? P.A : Gm;
  for (int t = 0; t < ntiles; ++t) {
    const TileMeta tm = tiles[t];
    const int i = tm.r0 + lrow;
    const bool owner = i < tm.r1 && quarter == 0;
    V4<T> m{}, xa{}, pv{};
    if (owner) {
      m = P.fmask[i];
      if (kMode == kGenR) { xa = P.xacc[i]; pv = pn[i]; }
    }
    const T *sA;
    const uint16_t *sL;
    stage_matrix<C>(M, P.lcol, P.rowptr, tm, smem, sA, sL, sRow);
    for (int j = threadIdx.x; j < tm.wn; j += C::kThreads) {
      const int node = __ldg(P.wlist + tm.w0 + j);
      V4<T> u;
      if (kMode == kGenZ) {
        u = P.r[rcur][node];
      } else if (kMode == kGenP) {
        const V4<T> zj = z[node], pj = po[node];
        u = V4<T>{zj.x + beta * pj.x, zj.y + beta * pj.y, zj.z + beta * pj.z, T(0)};
      } else {
        const V4<T> rj = P.r[rcur][node], qj = q[node];
        u = V4<T>{rj.x - alpha * qj.x, rj.y - alpha * qj.y, rj.z - alpha * qj.z, T(0)};
      }
      if (node >= tm.r0 && node < tm.r1) sOwn[node - tm.r0] = u;
      sU[j] = u;
    }
    __syncthreads();
    T c0 = 0, c1 = 0, c2 = 0;
    if (i < tm.r1) {
      const int q0 = sRow[lrow], q1 = sRow[lrow + 1];
#pragma unroll 2
      for (int k = q0 + quarter; k < q1; k += C::kRowThreads) {
        const V4<T> u = sU[sL[k]];
        const T *blk = sA + size_t(k) * 9;
        c0 += blk[0] * u.x + blk[1] * u.y + blk[2] * u.z;
        c1 += blk[3] * u.x + blk[4] * u.y + blk[5] * u.z;
        c2 += blk[6] * u.x + blk[7] * u.y + blk[8] * u.z;
      }
    }
#pragma unroll
    for (int o = 1; o < C::kRowThreads; o <<= 1) {
      c0 += __shfl_xor_sync(0xffffffffu, c0, o);
      c1 += __shfl_xor_sync(0xffffffffu, c1, o);
      c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    }
    if (owner) {
      const V4<T> res{c0 * m.x, c1 * m.y, c2 * m.z, T(0)};
      const V4<T> own = sOwn[lrow];
      if (kMode == kGenZ) {
        z[i] = res;
        a1 = A::addf(a1, dot3(own, res));
        a2 = A::addf(a2, dot3(own, own));
      } else if (kMode == kGenP) {
        pn[i] = own;
        q[i] = res;
        a1 = A::addf(a1, dot3(own, res));
      } else {
        P.r[rcur ^ 1][i] = own;
        z[i] = res;
        xa.x += alpha * pv.x; xa.y += alpha * pv.y; xa.z += alpha * pv.z;
        P.xacc[i] = xa;
        a1 = A::addf(a1, dot3(own, res));
        a2 = A::addf(a2, dot3(own, own));
      }
    }
    __syncthreads();
  }
}

// Reliable update: r[rcur] = rhs - A x64 in FP64 arithmetic.
template <class C, typename T>
__device__ __forceinline__ void gen_ru_residual(const Params<T> &P, const TileMeta *tiles,
                                               int ntiles, int rcur, unsigned char *smem,
                                               double &rr64) {
  V4<double> *sX = reinterpret_cast<V4<double> *>(smem + C::kValBytes);
  __shared__ int sRow[C::kTileRows + 1];
  const int lrow = threadIdx.x / C::kRowThreads, quarter = threadIdx.x % C::kRowThreads;
  for (int t = 0; t < ntiles; ++t) {
    const TileMeta tm = tiles[t];
    const T *sA;
    const uint16_t *sL;
    stage_matrix<C>(P.A, P.lcol, P.rowptr, tm, smem, sA, sL, sRow);
    for (int j = threadIdx.x; j < tm.wn; j += C::kThreads) sX[j] = P.x64[__ldg(P.wlist + tm.w0 + j)];
    __syncthreads();
    const int i = tm.r0 + lrow;
    double a0 = 0, a1 = 0, a2 = 0;
    if (i < tm.r1) {
      for (int k = sRow[lrow] + quarter; k < sRow[lrow + 1]; k += C::kRowThreads) {
        const V4<double> xj = sX[sL[k]];
        const T *blk = sA + size_t(k) * 9;
        a0 += double(blk[0]) * xj.x + double(blk[1]) * xj.y + double(blk[2]) * xj.z;
        a1 += double(blk[3]) * xj.x + double(blk[4]) * xj.y + double(blk[5]) * xj.z;
        a2 += double(blk[6]) * xj.x + double(blk[7]) * xj.y + double(blk[8]) * xj.z;
      }
    }
#pragma unroll
    for (int o = 1; o < C::kRowThreads; o <<= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (i < tm.r1 && quarter == 0) {
      const V4<double> b = P.rhs[i];
      const V4<T> m = P.fmask[i];
      const double e0 = (b.x - a0) * double(m.x), e1 = (b.y - a1) * double(m.y),
                   e2 = (b.z - a2) * double(m.z);
      rr64 += e0 * e0 + e1 * e1 + e2 * e2;
      P.r[rcur][i] = V4<T>{T(e0), T(e1), T(e2), T(0)};
    }
    __syncthreads();
  }
}

// rhs = mask * (-b - A beq_full) in FP64 (A promoted), the preconditioner,
// r = rhs, x = 0, p = s = 0.
template <typename T>
__device__ void setup_node(int i, const int *rowptr, const int *colidx,
                           const int *diag, const T *A, const double *b,
                           const double *beq_full, const uint8_t *pinned,
                           int block_pc, V4<double> *rhs, V4<double> *x64,
                           V4<T> *r, V4<T> *p, V4<T> *s, V4<T> *xacc, T *pc,
                           V4<T> *fmask) {
  // a = (A beq)_i.  beq is zero off the pinned DOFs, and a column block
  // whose three beq entries are zero adds exact zeros (finite blocks), so it
  // is skipped without reading the block: same sums, same order.
  double a[3] = {0, 0, 0};
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int j = colidx[k];
    const double q[3] = {beq_full[3 * j], beq_full[3 * j + 1], beq_full[3 * j + 2]};
    if (((__double_as_longlong(q[0]) | __double_as_longlong(q[1]) | __double_as_longlong(q[2]))
         << 1) == 0)
      continue;
    const T *blk = A + size_t(k) * 9;
    for (int rr = 0; rr < 3; ++rr)
      for (int c = 0; c < 3; ++c) a[rr] += double(blk[3 * rr + c]) * q[c];
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
  } else {
    // Eigen's DiagonalPreconditioner: 1/diag, 1 where the diagonal is 0
    for (int c = 0; c < 3; ++c) {
      T dd = D[4 * c];
      pc[size_t(4) * i + c] = (dd != T(0) ? T(1) / dd : T(1)) * m[c];
    }
    pc[size_t(4) * i + 3] = T(0);
  }
  const V4<T> zero{T(0), T(0), T(0), T(0)};
  r[i] = V4<T>{T(e[0]), T(e[1]), T(e[2]), T(0)};
  p[i] = zero;
  s[i] = zero;
  xacc[i] = zero;
}

template <typename T>
__global__ void setup_kernel(int n_nodes, const int *rowptr, const int *colidx,
                             const int *diag, const T *A, const double *b,
                             const double *beq_full, const uint8_t *pinned,
                             int block_pc, V4<double> *rhs, V4<double> *x64,
                             V4<T> *r, V4<T> *p, V4<T> *s, V4<T> *xacc, T *pc,
                             V4<T> *fmask) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  setup_node<T>(i, rowptr, colidx, diag, A, b, beq_full, pinned, block_pc, rhs, x64, r, p, s,
                xacc, pc, fmask);
}

// setup_kernel (128 threads per block) plus each block's FP64 partial of
// ||rhs||^2 (warp trees, then the four warps in order).
template <typename T>
__global__ void __launch_bounds__(128)
    setup_norm_kernel(int n_nodes, const int *rowptr, const int *colidx, const int *diag,
                      const T *A, const double *b, const double *beq_full,
                      const uint8_t *pinned, int block_pc, V4<double> *rhs, V4<double> *x64,
                      V4<T> *r, V4<T> *p, V4<T> *s, V4<T> *xacc, T *pc, V4<T> *fmask,
                      double *part) {
  __shared__ double red[4];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double s2 = 0.0;
  if (i < n_nodes) {
    setup_node<T>(i, rowptr, colidx, diag, A, b, beq_full, pinned, block_pc, rhs, x64, r, p, s,
                  xacc, pc, fmask);
    const V4<double> q = rhs[i];
    s2 = q.x * q.x + q.y * q.y + q.z * q.z;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s2;
  __syncthreads();
  if (threadIdx.x == 0) part[blockIdx.x] = (red[0] + red[1]) + (red[2] + red[3]);
}

// ||rhs||^2 from the nb partials of setup_norm_kernel (one CTA of 256
// threads, a fixed order); resets the status record.
__global__ void __launch_bounds__(256) norm_finish_kernel(int nb, const double *part,
                                                          DevStatus *st) {
  __shared__ double red[8];
  double s2 = 0.0;
  for (int k = threadIdx.x; k < nb; k += 256) s2 += part[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < 8; ++w) v += red[w];
    st->status = EOLC_OK;
    st->iterations = 0;
    st->refinements = 0;
    st->rel_res = v > 0 ? 1.0 : 0.0;
    st->rhs_norm2 = v;
  }
}

// ||rhs||^2 by one CTA; resets the status record.
template <class C>
__global__ void __launch_bounds__(C::kThreads) init_sums_kernel(int n_nodes, const V4<double> *rhs,
                                                             DevStatus *st) {
  __shared__ double red[3 * (C::kThreads / 32 + 1)];
  double s_rhs = 0, d0 = 0, d1 = 0;
  for (int i = threadIdx.x; i < n_nodes; i += C::kThreads) {
    V4<double> b = rhs[i];
    s_rhs += b.x * b.x + b.y * b.y + b.z * b.z;
  }
  block_sum3<C, double>(s_rhs, d0, d1, red);
  if (threadIdx.x == 0) {
    st->status = EOLC_OK;
    st->iterations = 0;
    st->refinements = 0;
    st->rel_res = s_rhs > 0 ? 1.0 : 0.0;
    st->rhs_norm2 = s_rhs;
  }
}

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


// Tiles of <= tile_rows rows whose staged values, local columns and halo fit
// the shared-memory budget; the halo list and tile-local columns are built
// here once per topology.
// breaks: optional ascending row indices that no tile may straddle (the
// first row of every instance of a batch).
inline std::string build_tiles(int N, const std::vector<int> &rowptr,
                               const std::vector<int> &colidx, int cap, int win_cap,
                               int tile_rows, std::vector<int> &tiles, std::vector<int> &wptr,
                               std::vector<int> &wlist, std::vector<uint16_t> &lcol,
                               const std::vector<int> *breaks = nullptr) {
  tiles.assign(1, 0);
  wptr.assign(1, 0);
  wlist.clear();
  lcol.assign(colidx.size(), 0);
  std::vector<int> stamp(N, -1), local(N, 0);
  int start = 0;
  size_t nb = 0;  // next break index
  std::vector<int> win;
  while (start < N) {
    while (breaks && nb < breaks->size() && (*breaks)[nb] <= start) ++nb;
    const int limit = (breaks && nb < breaks->size()) ? (*breaks)[nb] : N;
    int end = start;
    win.clear();
    // grow the tile row by row while it fits
    while (end < limit && end - start < tile_rows) {
      if (rowptr[end + 1] - rowptr[start] > cap) break;
      int added = 0;
      for (int k = rowptr[end]; k < rowptr[end + 1]; ++k)
        if (stamp[colidx[k]] != start) added++;
      if (int(win.size()) + added > win_cap) break;
      for (int k = rowptr[end]; k < rowptr[end + 1]; ++k)
        if (stamp[colidx[k]] != start) { stamp[colidx[k]] = start; win.push_back(colidx[k]); }
      ++end;
    }
    if (end == start) return "a block row does not fit the shared-memory tile";
    // every own row is in its window (the diagonal block is always present)
    std::sort(win.begin(), win.end());
    for (int j = 0; j < int(win.size()); ++j) local[win[j]] = j;
    for (int k = rowptr[start]; k < rowptr[end]; ++k) lcol[k] = uint16_t(local[colidx[k]]);
    wlist.insert(wlist.end(), win.begin(), win.end());
    wptr.push_back(int(wlist.size()));
    tiles.push_back(end);
    start = end;
  }
  return "";
}


}  // namespace
}  // namespace cgc
}  // namespace eolc
