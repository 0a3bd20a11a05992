// Batched PCG: many independent cloth instances of uneven size, solved in ONE
// persistent launch.
//
// The instances are concatenated into one block-diagonal BSR system (global
// node numbering, instance k owns rows node_off[k] .. node_off[k+1]).  Tiles
// never straddle an instance boundary.  A persistent grid of CTA clusters
// pulls instances from a work queue (largest first); the CTAs of a cluster
// split the instance's tiles and run the same single-reduction CG iteration
// as the one-system kernel (pcg.cu: Chronopoulos-Gear, halo residual
// recomputed per tile, FP64 reliable updates), but synchronise with the
// hardware cluster barrier and exchange their partial inner products through
// distributed shared memory.  No grid-wide barrier and no spin-wait: an
// instance's iteration costs one cluster barrier instead of a grid barrier.
//
// Every CTA of a cluster reduces the same partials in the same rank order,
// so all of them take the same branches and reach the same barriers.
//
// Shapes (threads per CTA, threads per block row, shared-memory split) and
// the cluster size are chosen by an autotuner that times each candidate on
// the caller's batch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "cg_common.cuh"
#include "cg_tile.cuh"
#include "internal.h"

namespace eolc {

namespace {
using namespace cgc;
namespace cgr = cooperative_groups;

constexpr int kMaxBatchTiles = 160;  // tiles of one instance held by one CTA

struct BatchArgs {
  int n_inst;
  const int *n_inst_d;   // if set: the queue length, read on the device
  const int *inst_tile;  // n_inst + 1: first tile of every instance
  const int *order;      // queue position -> instance (largest first)
  unsigned *queue;       // next queue position; zero before each launch
  BatchRecord *rec;      // per instance, accumulated over launches
  const int *cap;        // if set: per-instance iteration cap (else max_iter)
  int *last_status;      // if set: per-instance status of this launch
  int *jac_iters;        // if set: Jacobi iterations of each converged instance
  int fallback;          // 1: this launch re-solves instances a learned solve left
  double tol2;           // rel_tol^2
  int max_iter;
};

// Per-instance bookkeeping at the end of an instance's solve (rank 0,
// thread 0 of its cluster).  A learned solve that stopped at its cap leaves
// the status to the Jacobi re-solve that follows.
__device__ __forceinline__ void record_instance(const BatchArgs &B, int inst, int status, int it,
                                                int nref, double last_rr64, double rhs2,
                                                bool learned) {
  BatchRecord r = B.rec[inst];
  const bool deferred = learned && status == EOLC_NOT_CONVERGED;
  if (r.status == EOLC_OK && !deferred) r.status = status;
  r.iterations += it;
  r.refinements += nref;
  r.max_iterations = max(r.max_iterations, it);
  if (!deferred) r.steps += 1;
  if (B.fallback) r.used_fallback = 1;
  const double rel = rhs2 > 0 ? sqrt(last_rr64 / rhs2) : 0.0;
  if (!deferred) r.rel_res = fmax(r.rel_res, rel);
  B.rec[inst] = r;
  if (B.last_status) B.last_status[inst] = status;
  if (B.jac_iters && !learned && status == EOLC_OK) B.jac_iters[inst] = it;
}

__device__ __forceinline__ void cluster_barrier() {
  // Every thread of every CTA of the cluster arrives.  release: this thread's
  // global and shared writes become visible to the cluster; acquire: writes
  // released by the other CTAs are visible after it.  (Not the .aligned form:
  // a warp may reach it just after a divergent branch.)
  asm volatile(
      "barrier.cluster.arrive.release;\n\t"
      "barrier.cluster.wait.acquire;\n" ::: "memory");
}

// Sum of (a, b, c) over every thread of every CTA of the cluster, in a fixed
// order.  xch: this CTA's exchange slots, double-buffered by pset, so that a
// slot is rewritten only after a later barrier has retired its readers.
template <class C, typename U>
__device__ __forceinline__ void cluster_sum3(cgr::cluster_group &cl, int csize,
                                             typename Acc<U>::V &a, typename Acc<U>::V &b,
                                             typename Acc<U>::V &c, typename Acc<U>::V *red,
                                             double (*xch)[3], int &pset) {
  using A = Acc<U>;
  using V = typename A::V;
  static_assert(sizeof(V) == sizeof(double), "exchange slots hold 8-byte values");
  block_sum3<C, U>(a, b, c, red);
  if (csize == 1) return;
  if (threadIdx.x == 0) {
    V *slot = reinterpret_cast<V *>(xch[pset]);
    slot[0] = a; slot[1] = b; slot[2] = c;
  }
  cluster_barrier();
  a = b = c = A::zero();
  for (int r = 0; r < csize; ++r) {
    const V *rem = reinterpret_cast<const V *>(cl.map_shared_rank(&xch[pset][0], r));
    a = A::add(a, rem[0]);
    b = A::add(b, rem[1]);
    c = A::add(c, rem[2]);
  }
  pset ^= 1;
}

template <typename T, class C, int kMinBlocks>
__global__ void __launch_bounds__(C::kThreads, kMinBlocks)
batch_cg_kernel(Params<T> P, BatchArgs B) {
  using A = Acc<T>;
  using V = typename A::V;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ V red[3 * (C::kThreads / 32 + 1)];
  __shared__ TileMeta tiles[kMaxBatchTiles];
  __shared__ double xch[2][3];
  __shared__ int s_inst;
  cgr::cluster_group cl = cgr::this_cluster();
  const int crank = int(cl.block_rank()), csize = int(cl.num_blocks());
  int pset = 0;
  const V delta2 = A::from_d(kDelta * kDelta);
  double *redd = reinterpret_cast<double *>(red);
  for (;;) {
    if (crank == 0 && threadIdx.x == 0) s_inst = int(atomicAdd(B.queue, 1u));
    cluster_barrier();
    const int q = *cl.map_shared_rank(&s_inst, 0);
    const int n_queue = B.n_inst_d ? *B.n_inst_d : B.n_inst;
    if (q >= n_queue) {
      cluster_barrier();  // nobody leaves while the leader's slot may be read
      return;
    }
    const int inst = B.order[q];
    const int max_iter = B.cap ? B.cap[inst] : B.max_iter;
    const int it0 = B.inst_tile[inst];
    const int nt = B.inst_tile[inst + 1] - it0;
    const int c0 = it0 + int((long long)nt * crank / csize);
    const int c1 = it0 + int((long long)nt * (crank + 1) / csize);
    const int ntiles = c1 - c0;
    for (int t = threadIdx.x; t < ntiles; t += C::kThreads) {
      TileMeta tm;
      tm.r0 = P.tile_row[c0 + t];
      tm.r1 = P.tile_row[c0 + t + 1];
      tm.b0 = P.rowptr[tm.r0];
      tm.b1 = P.rowptr[tm.r1];
      tm.w0 = P.tile_wptr[c0 + t];
      tm.wn = P.tile_wptr[c0 + t + 1] - tm.w0;
      tiles[t] = tm;
    }
    __syncthreads();
    // ||rhs||^2 of this instance (FP64)
    double n0 = 0, n1 = 0, n2 = 0;
    for (int t = 0; t < ntiles; ++t)
      for (int i = tiles[t].r0 + threadIdx.x; i < tiles[t].r1; i += C::kThreads) {
        const V4<double> b = P.rhs[i];
        n0 += b.x * b.x + b.y * b.y + b.z * b.z;
      }
    cluster_sum3<C, double>(cl, csize, n0, n1, n2, redd, xch, pset);
    const double rhs2 = n0;
    const V tol2 = A::from_d(B.tol2 * rhs2);

    int cur = 0;
    V gam = A::zero(), del = A::zero(), rr = A::zero();
    cg_phase<C, T, true>(P, tiles, ntiles, cur, T(0), T(0), smem, gam, del, rr);
    cluster_sum3<C, T>(cl, csize, gam, del, rr, red, xch, pset);
    V rmax2 = rr;
    double last_rr64 = A::to_d(rr);
    int it = 0, nref = 0, status = EOLC_NOT_CONVERGED;
    bool converged = A::finite(rr) && A::le(rr, tol2);
    if (!A::finite(rr)) status = EOLC_NONFINITE;
    V gam_old = A::from_d(1.0), alpha_old = A::from_d(1.0);
    bool restart = true;
    while (!converged && status != EOLC_NONFINITE && it < max_iter) {
      const V beta = restart ? A::zero() : A::div(gam, gam_old);
      const V denom =
          restart ? del : A::add(del, A::neg(A::div(A::mul(beta, gam), alpha_old)));
      if (!A::pos(denom) || !A::pos(gam)) {
        status = (A::finite(denom) && A::finite(gam)) ? EOLC_BREAKDOWN : EOLC_NONFINITE;
        break;
      }
      const V alpha = A::div(gam, denom);
      restart = false;
      V g2 = A::zero(), d2 = A::zero(), rr2 = A::zero();
      cg_phase<C, T, false>(P, tiles, ntiles, cur, T(A::to_t(alpha)), T(A::to_t(beta)), smem,
                            g2, d2, rr2);
      cluster_sum3<C, T>(cl, csize, g2, d2, rr2, red, xch, pset);
      ++it;
      cur ^= 1;
      gam_old = gam;
      alpha_old = alpha;
      gam = g2;
      del = d2;
      rr = rr2;
      if (!A::finite(rr) || !A::finite(gam) || !A::finite(del)) { status = EOLC_NONFINITE; break; }
      if (!(A::lt(rr, A::mul(delta2, rmax2)) || A::le(rr, tol2) || it >= max_iter)) continue;
      // reliable update: fold the FP32 increment into the FP64 solution ...
      for (int t = 0; t < ntiles; ++t)
        for (int i = tiles[t].r0 + threadIdx.x; i < tiles[t].r1; i += C::kThreads) {
          const V4<T> xa = P.xacc[i];
          V4<double> x = P.x64[i];
          x.x += double(xa.x); x.y += double(xa.y); x.z += double(xa.z);
          P.x64[i] = x;
          P.xacc[i] = V4<T>{T(0), T(0), T(0), T(0)};
        }
      if (csize > 1) cluster_barrier(); else __syncthreads();
      // ... recompute the true residual in FP64, and s = A p
      double rr64d = 0, z0 = 0, z1 = 0;
      ru_residual<C>(P, tiles, ntiles, cur, smem, rr64d);
      cluster_sum3<C, double>(cl, csize, rr64d, z0, z1, redd, xch, pset);
      ++nref;
      last_rr64 = rr64d;
      rmax2 = A::from_d(rr64d);
      if (!isfinite(rr64d)) { status = EOLC_NONFINITE; break; }
      if (A::le(A::from_d(rr64d), tol2)) { converged = true; break; }
      // u = M r, w = A u for the replaced residual
      V g3 = A::zero(), d3 = A::zero(), rr3 = A::zero();
      cg_phase<C, T, true>(P, tiles, ntiles, cur, T(0), T(0), smem, g3, d3, rr3);
      cluster_sum3<C, T>(cl, csize, g3, d3, rr3, red, xch, pset);
      gam = g3;
      del = d3;
    }
    if (converged) status = EOLC_OK;
    if (crank == 0 && threadIdx.x == 0)
      record_instance(B, inst, status, it, nref, last_rr64, rhs2, false);
    __syncthreads();
  }
}


// Batched PCG with the learned approximate inverse G (FP32, pattern of A):
// standard PCG per instance, two cluster reductions per iteration (p'q after
// q = A p; r'z and r'r after z = G r), the halo values recomputed on the fly
// as in pcg_general_kernel (pcg.cu).  An instance stops at its cap
// (B.cap: fallback_factor x its last Jacobi count) and is left to the Jacobi
// re-solve that follows in the same step.
template <class C, int kMinBlocks>
__global__ void __launch_bounds__(C::kThreads, kMinBlocks)
batch_gen_kernel(Params<float> P, BatchArgs B, const float *Gm) {
  using T = float;
  using A = Acc<T>;
  using V = typename A::V;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ V red[3 * (C::kThreads / 32 + 1)];
  __shared__ TileMeta tiles[kMaxBatchTiles];
  __shared__ double xch[2][3];
  __shared__ int s_inst;
  cgr::cluster_group cl = cgr::this_cluster();
  const int crank = int(cl.block_rank()), csize = int(cl.num_blocks());
  int pset = 0;
  const V delta2 = A::from_d(kDelta * kDelta);
  double *redd = reinterpret_cast<double *>(red);
  for (;;) {
    if (crank == 0 && threadIdx.x == 0) s_inst = int(atomicAdd(B.queue, 1u));
    cluster_barrier();
    const int q = *cl.map_shared_rank(&s_inst, 0);
    const int n_queue = B.n_inst_d ? *B.n_inst_d : B.n_inst;
    if (q >= n_queue) {
      cluster_barrier();
      return;
    }
    const int inst = B.order[q];
    const int max_iter = B.cap ? B.cap[inst] : B.max_iter;
    const int it0 = B.inst_tile[inst];
    const int nt = B.inst_tile[inst + 1] - it0;
    const int c0 = it0 + int((long long)nt * crank / csize);
    const int c1 = it0 + int((long long)nt * (crank + 1) / csize);
    const int ntiles = c1 - c0;
    for (int t = threadIdx.x; t < ntiles; t += C::kThreads) {
      TileMeta tm;
      tm.r0 = P.tile_row[c0 + t];
      tm.r1 = P.tile_row[c0 + t + 1];
      tm.b0 = P.rowptr[tm.r0];
      tm.b1 = P.rowptr[tm.r1];
      tm.w0 = P.tile_wptr[c0 + t];
      tm.wn = P.tile_wptr[c0 + t + 1] - tm.w0;
      tiles[t] = tm;
    }
    __syncthreads();
    double n0 = 0, n1 = 0, n2 = 0;
    for (int t = 0; t < ntiles; ++t)
      for (int i = tiles[t].r0 + threadIdx.x; i < tiles[t].r1; i += C::kThreads) {
        const V4<double> b = P.rhs[i];
        n0 += b.x * b.x + b.y * b.y + b.z * b.z;
      }
    cluster_sum3<C, double>(cl, csize, n0, n1, n2, redd, xch, pset);
    const double rhs2 = n0;
    const V tol2 = A::from_d(B.tol2 * rhs2);
    int rcur = 0, pold = 0;
    V rz = A::zero(), rr = A::zero(), zz = A::zero();
    gen_phase<C, T, kGenZ>(P, Gm, tiles, ntiles, rcur, pold, T(0), T(0), smem, rz, rr);
    cluster_sum3<C, T>(cl, csize, rz, rr, zz, red, xch, pset);
    V rmax2 = rr;
    double last_rr64 = A::to_d(rr);
    int it = 0, nref = 0, status = A::finite(rr) ? EOLC_NOT_CONVERGED : EOLC_NONFINITE;
    bool converged = A::finite(rr) && A::le(rr, tol2);
    V rz_prev = A::from_d(1.0);
    bool restart = true;
    while (!converged && status != EOLC_NONFINITE && it < max_iter) {
      const V beta = restart ? A::zero() : A::div(rz, rz_prev);
      restart = false;
      V pq = A::zero(), d1 = A::zero(), d2 = A::zero();
      gen_phase<C, T, kGenP>(P, Gm, tiles, ntiles, rcur, pold, T(0), T(A::to_t(beta)), smem, pq,
                             d1);
      cluster_sum3<C, T>(cl, csize, pq, d1, d2, red, xch, pset);
      if (!A::pos(pq) || !A::pos(rz)) {
        status = (A::finite(pq) && A::finite(rz)) ? EOLC_BREAKDOWN : EOLC_NONFINITE;
        break;
      }
      const V alpha = A::div(rz, pq);
      V rz2 = A::zero(), rr2 = A::zero(), d3 = A::zero();
      gen_phase<C, T, kGenR>(P, Gm, tiles, ntiles, rcur, pold, T(A::to_t(alpha)), T(0), smem,
                             rz2, rr2);
      cluster_sum3<C, T>(cl, csize, rz2, rr2, d3, red, xch, pset);
      ++it;
      rcur ^= 1;
      pold ^= 1;
      rz_prev = rz;
      rz = rz2;
      rr = rr2;
      if (!A::finite(rr) || !A::finite(rz)) { status = EOLC_NONFINITE; break; }
      if (!(A::lt(rr, A::mul(delta2, rmax2)) || A::le(rr, tol2) || it >= max_iter)) continue;
      for (int t = 0; t < ntiles; ++t)
        for (int i = tiles[t].r0 + threadIdx.x; i < tiles[t].r1; i += C::kThreads) {
          const V4<T> xa = P.xacc[i];
          V4<double> x = P.x64[i];
          x.x += double(xa.x); x.y += double(xa.y); x.z += double(xa.z);
          P.x64[i] = x;
          P.xacc[i] = V4<T>{T(0), T(0), T(0), T(0)};
        }
      if (csize > 1) cluster_barrier(); else __syncthreads();
      double rr64d = 0, z0 = 0, z1 = 0;
      gen_ru_residual<C>(P, tiles, ntiles, rcur, smem, rr64d);
      cluster_sum3<C, double>(cl, csize, rr64d, z0, z1, redd, xch, pset);
      ++nref;
      last_rr64 = rr64d;
      rmax2 = A::from_d(rr64d);
      if (!isfinite(rr64d)) { status = EOLC_NONFINITE; break; }
      if (A::le(A::from_d(rr64d), tol2)) { converged = true; break; }
      V rz3 = A::zero(), rr3 = A::zero(), e3 = A::zero();
      gen_phase<C, T, kGenZ>(P, Gm, tiles, ntiles, rcur, pold, T(0), T(0), smem, rz3, rr3);
      cluster_sum3<C, T>(cl, csize, rz3, rr3, e3, red, xch, pset);
      rz = rz3;
    }
    if (converged) status = EOLC_OK;
    if (crank == 0 && threadIdx.x == 0)
      record_instance(B, inst, status, it, nref, last_rr64, rhs2, true);
    __syncthreads();
  }
}

// Iteration caps of a learned batched solve: fallback_factor x each
// instance's last Jacobi count (uncapped where there is none yet).
__global__ void caps_kernel(int n_inst, const int *jac_iters, int factor, int max_iter, int *cap) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_inst) return;
  const int j = jac_iters[k];
  cap[k] = (factor > 0 && j > 0) ? min(max_iter, factor * j) : max_iter;
}

// The instances a learned launch left unconverged, in queue order (one CTA,
// fixed order): order_out[0 .. *count), and a flag per instance.
__global__ void collect_failed_kernel(int n_inst, const int *order, const int *last_status,
                                      int *order_out, int *count, int *flag) {
  __shared__ int s_base;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < n_inst; c0 += blockDim.x) {
    const int q = c0 + threadIdx.x;
    const int inst = q < n_inst ? order[q] : -1;
    const int f = (inst >= 0 && last_status[inst] == EOLC_NOT_CONVERGED) ? 1 : 0;
    if (inst >= 0) flag[inst] = f;
    // block-wide exclusive scan of f in thread order
    const unsigned ballot = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ int s_warp[32];
    if (lane == 0) s_warp[warp] = __popc(ballot);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += s_warp[w];
    const int pos = s_base + before + __popc(ballot & ((1u << lane) - 1u));
    if (f) order_out[pos] = inst;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < int(blockDim.x) / 32; ++w) tot += s_warp[w];
      s_base += tot;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = s_base;
}

// Set-up / finish restricted to the nodes of flagged instances.
__global__ void setup_flagged_kernel(int n_nodes, const int *node_inst, const int *flag,
                                     const int *rowptr, const int *colidx, const int *diag,
                                     const float *A, const double *b, const double *beq_full,
                                     const uint8_t *pinned, V4<double> *rhs, V4<double> *x64,
                                     V4<float> *r, V4<float> *p, V4<float> *s, V4<float> *xacc,
                                     float *pc, V4<float> *fmask) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes || !flag[node_inst[i]]) return;
  setup_node<float>(i, rowptr, colidx, diag, A, b, beq_full, pinned, 0, rhs, x64, r, p, s, xacc,
                    pc, fmask);
}

__global__ void finish_flagged_kernel(int n_nodes, const int *node_inst, const int *flag,
                                      const V4<double> *x64, const double *beq_full,
                                      const uint8_t *pinned, double *v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes || !flag[node_inst[i]]) return;
  const V4<double> x = x64[i];
  const double xs[3] = {x.x, x.y, x.z};
  for (int c = 0; c < 3; ++c) v[3 * i + c] = pinned[3 * i + c] ? beq_full[3 * i + c] : xs[c];
}

// ---- configurations ---------------------------------------------------------
using K0 = TileCfg<512, 4, 112, 2048>;  // 128-row tiles, one CTA per SM
using K1 = TileCfg<512, 8, 112, 2048>;  // 64-row tiles, 8 threads per row
using K2 = TileCfg<256, 4, 52, 1024>;   // 64-row tiles, two CTAs per SM
using K3 = TileCfg<256, 2, 52, 1024>;   // 128-row tiles, two CTAs per SM

struct ShapeInfo {
  int threads, tile_rows, min_blocks;
  size_t smem_f, smem_d;
  int cap_f, cap_d, win_f, win_d;
  const char *name;
};

template <class C, int kMin>
ShapeInfo shape_info(const char *name) {
  return {C::kThreads,
          C::kTileRows,
          kMin,
          C::template smem_bytes<float>(),
          C::template smem_bytes<double>(),
          C::template cap_blocks<float>(),
          C::template cap_blocks<double>(),
          C::template win_max<float>(),
          C::template win_max<double>(),
          name};
}

constexpr int kNumShapes = 4;
constexpr int kClusterSizes[] = {1, 2, 4, 8};  // 8: the portable maximum
constexpr int kNumCluster = 4;

const ShapeInfo &shape(int k) {
  static const ShapeInfo s[kNumShapes] = {
      shape_info<K0, 1>("512 threads, 4 per row, 128-row tiles, 1 CTA/SM"),
      shape_info<K1, 1>("512 threads, 8 per row, 64-row tiles, 1 CTA/SM"),
      shape_info<K2, 2>("256 threads, 4 per row, 64-row tiles, 2 CTAs/SM"),
      shape_info<K3, 2>("256 threads, 2 per row, 128-row tiles, 2 CTAs/SM")};
  return s[k];
}

template <typename T>
const void *kernel_of(int k) {
  switch (k) {
    case 0: return reinterpret_cast<const void *>(batch_cg_kernel<T, K0, 1>);
    case 1: return reinterpret_cast<const void *>(batch_cg_kernel<T, K1, 1>);
    case 2: return reinterpret_cast<const void *>(batch_cg_kernel<T, K2, 2>);
    default: return reinterpret_cast<const void *>(batch_cg_kernel<T, K3, 2>);
  }
}

const void *gen_kernel_of(int k) {
  switch (k) {
    case 0: return reinterpret_cast<const void *>(batch_gen_kernel<K0, 1>);
    case 1: return reinterpret_cast<const void *>(batch_gen_kernel<K1, 1>);
    case 2: return reinterpret_cast<const void *>(batch_gen_kernel<K2, 2>);
    default: return reinterpret_cast<const void *>(batch_gen_kernel<K3, 2>);
  }
}

}  // namespace

int batch_num_configs() { return kNumShapes * kNumCluster; }

std::string batch_config_name(int config) {
  if (config < 0 || config >= batch_num_configs()) return "";
  const int k = config / kNumCluster, cs = kClusterSizes[config % kNumCluster];
  return std::string(shape(k).name) + ", cluster of " + std::to_string(cs);
}

struct BatchSolveWork {
  int config = -1, prec = -1, block_pc = -1;
  int n_nodes = 0, n_blocks = 0, n_inst = 0;
  int grid = 0, gen_grid = 0;
  size_t smem = 0;
  // learned solves: per-instance caps, statuses, Jacobi references (kept
  // across configurations of one topology), the fallback queue
  DevBuf<int> cap, last_status, jac_iters, flag, order2, count;
  DevBuf<unsigned char> vecs, pc;
  DevBuf<int> tile_row, tile_wptr, wlist, inst_tile, order;
  DevBuf<uint16_t> lcol;
  DevBuf<unsigned> queue;
  DevBuf<BatchRecord> rec;
  std::vector<int> rowptr, colidx;  // host copy of the pattern
};

void free_batch_work(BatchSolveWork *w) { delete w; }

eolc_status batch_prepare(BatchSolveWork *&w, const PcgArgs &a, const std::vector<int> &node_off,
                          int config, cudaStream_t s, std::string &err) {
  if (config < 0 || config >= batch_num_configs()) {
    err = "unknown batch configuration";
    return EOLC_BAD_ARG;
  }
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes;
  const int n_inst = int(node_off.size()) - 1;
  const bool fp64 = a.precision == EOLC_PREC_FP64;
  const int prec = fp64 ? 0 : 1;
  const int bpc = a.precond == EOLC_PC_BLOCK_JACOBI ? 1 : 0;
  if (!w) w = new BatchSolveWork();
  if (w->config == config && w->prec == prec && w->block_pc == bpc && w->n_nodes == N &&
      w->n_blocks == Tp.n_blocks && w->n_inst == n_inst)
    return EOLC_OK;
  const int k = config / kNumCluster, csize = kClusterSizes[config % kNumCluster];
  const ShapeInfo &sh = shape(k);
  if (int(w->rowptr.size()) != N + 1 || int(w->colidx.size()) != Tp.n_blocks) {
    w->rowptr.resize(N + 1);
    w->colidx.resize(Tp.n_blocks);
    cudaMemcpy(w->rowptr.data(), Tp.rowptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost);
    cudaMemcpy(w->colidx.data(), Tp.colidx.p, sizeof(int) * Tp.n_blocks, cudaMemcpyDeviceToHost);
  }
  std::vector<int> breaks(node_off.begin() + 1, node_off.end() - 1);
  std::vector<int> tiles, wptr, wlist;
  std::vector<uint16_t> lcol;
  std::string msg = build_tiles(N, w->rowptr, w->colidx, fp64 ? sh.cap_d : sh.cap_f,
                                fp64 ? sh.win_d : sh.win_f, sh.tile_rows, tiles, wptr, wlist,
                                lcol, &breaks);
  if (!msg.empty()) { err = msg; return EOLC_BAD_ARG; }
  // first tile of every instance
  std::vector<int> inst_tile(n_inst + 1, 0);
  {
    int t = 0;
    for (int q = 0; q <= n_inst; ++q) {
      while (t < int(tiles.size()) - 1 && tiles[t] < node_off[q]) ++t;
      inst_tile[q] = t;
    }
    inst_tile[n_inst] = int(tiles.size()) - 1;
  }
  for (int q = 0; q < n_inst; ++q) {
    const int nt = inst_tile[q + 1] - inst_tile[q];
    if ((nt + csize - 1) / csize > kMaxBatchTiles) {
      err = "an instance has too many tiles for this cluster size";
      return EOLC_BAD_ARG;
    }
  }
  // largest instances first
  std::vector<int> order(n_inst);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return w->rowptr[node_off[x + 1]] - w->rowptr[node_off[x]] >
           w->rowptr[node_off[y + 1]] - w->rowptr[node_off[y]];
  });
  // launch shape: as many co-resident clusters as fit
  const void *fn = fp64 ? kernel_of<double>(k) : kernel_of<float>(k);
  const size_t smem = fp64 ? sh.smem_d : sh.smem_f;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3(csize);
  lc.blockDim = dim3(sh.threads);
  lc.dynamicSmemBytes = smem;
  lc.attrs = attr;
  lc.numAttrs = 1;
  int n_clusters = 0;
  e = cudaOccupancyMaxActiveClusters(&n_clusters, fn, &lc);
  if (e != cudaSuccess || n_clusters < 1) {
    err = e != cudaSuccess ? cudaGetErrorString(e) : "batch kernel does not fit on the device";
    return EOLC_CUDA_ERROR;
  }
  // the learned kernel of this shape (mixed precision only)
  int gen_clusters = 0;
  if (!fp64) {
    const void *gfn = gen_kernel_of(k);
    e = cudaFuncSetAttribute(gfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&gen_clusters, gfn, &lc);
    if (e != cudaSuccess || gen_clusters < 1) {
      err = e != cudaSuccess ? cudaGetErrorString(e) : "batch kernel does not fit on the device";
      return EOLC_CUDA_ERROR;
    }
  }
  if (int(w->jac_iters.n) != std::max(n_inst, 1)) {
    if (w->jac_iters.resize(std::max(n_inst, 1)) != cudaSuccess ||
        cudaMemsetAsync(w->jac_iters.p, 0, sizeof(int) * w->jac_iters.n, s) != cudaSuccess) {
      err = "device allocation failed";
      return EOLC_CUDA_ERROR;
    }
  }
  lcol.resize(lcol.size() + 8, 0);
  const size_t vt = fp64 ? sizeof(V4<double>) : sizeof(V4<float>);
  cudaError_t es[] = {
      w->tile_row.upload(tiles.data(), tiles.size(), s),
      w->tile_wptr.upload(wptr.data(), wptr.size(), s),
      w->wlist.upload(wlist.data(), std::max<size_t>(wlist.size(), 1), s),
      w->lcol.upload(lcol.data(), lcol.size(), s),
      w->inst_tile.upload(inst_tile.data(), inst_tile.size(), s),
      w->order.upload(order.data(), order.size(), s),
      w->vecs.resize(size_t(N) * (sizeof(V4<double>) * 2 + vt * 9)),
      w->pc.resize(size_t(N) * 9 * (fp64 ? sizeof(double) : sizeof(float))),
      w->queue.resize(1),
      w->rec.resize(std::max(n_inst, 1)),
      w->cap.resize(std::max(n_inst, 1)),
      w->last_status.resize(std::max(n_inst, 1)),
      w->flag.resize(std::max(n_inst, 1)),
      w->order2.resize(std::max(n_inst, 1)),
      w->count.resize(1),
      cudaStreamSynchronize(s)};
  for (cudaError_t x : es)
    if (x != cudaSuccess) { err = cudaGetErrorString(x); return EOLC_CUDA_ERROR; }
  w->config = config;
  w->prec = prec;
  w->block_pc = bpc;
  w->n_nodes = N;
  w->n_blocks = Tp.n_blocks;
  w->n_inst = n_inst;
  w->grid = n_clusters * csize;
  w->gen_grid = gen_clusters * csize;
  w->smem = smem;
  return EOLC_OK;
}

namespace {

template <typename T>
eolc_status batch_enqueue_t(BatchSolveWork *w, const PcgArgs &a, cudaStream_t s,
                            std::string &err, long long &launches) {
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes;
  const T *A = std::is_same<T, double>::value ? reinterpret_cast<const T *>(a.A64)
                                              : reinterpret_cast<const T *>(a.A32);
  unsigned char *vp = w->vecs.p;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<T> *vr = reinterpret_cast<V4<T> *>(vp);
  Params<T> P{};
  P.r[0] = vr; P.r[1] = vr + N;
  P.w[0] = vr + 2 * N; P.w[1] = vr + 3 * N;
  P.s[0] = vr + 4 * N; P.s[1] = vr + 5 * N;
  P.p = vr + 6 * N;
  P.xacc = vr + 7 * N;
  V4<T> *fmask = vr + 8 * N;
  T *pc = reinterpret_cast<T *>(w->pc.p);
  setup_kernel<T><<<(N + 127) / 128, 128, 0, s>>>(
      N, Tp.rowptr.p, Tp.colidx.p, Tp.diag.p, A, a.b, a.beq_full, a.pinned, w->block_pc, rhs,
      x64, P.r[0], P.p, P.s[0], P.xacc, pc, fmask);
  cudaMemsetAsync(w->queue.p, 0, sizeof(unsigned), s);
  P.n_nodes = N;
  P.rowptr = Tp.rowptr.p;
  P.A = A;
  P.lcol = w->lcol.p;
  P.tile_row = w->tile_row.p;
  P.tile_wptr = w->tile_wptr.p;
  P.wlist = w->wlist.p;
  P.rhs = rhs;
  P.x64 = x64;
  P.pc = pc;
  P.fmask = fmask;
  P.max_iter = a.max_iter;
  P.block_pc = w->block_pc;
  P.tol2 = a.rel_tol * a.rel_tol;
  BatchArgs B{};
  B.n_inst = w->n_inst;
  B.inst_tile = w->inst_tile.p;
  B.order = w->order.p;
  B.queue = w->queue.p;
  B.rec = w->rec.p;
  B.last_status = w->last_status.p;
  B.jac_iters = (w->block_pc == 0) ? w->jac_iters.p : nullptr;
  B.tol2 = a.rel_tol * a.rel_tol;
  B.max_iter = a.max_iter;
  const int k = w->config / kNumCluster, csize = kClusterSizes[w->config % kNumCluster];
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3(w->grid);
  lc.blockDim = dim3(shape(k).threads);
  lc.dynamicSmemBytes = w->smem;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  void *args[] = {&P, &B};
  cudaError_t e = cudaLaunchKernelExC(&lc, kernel_of<T>(k), args);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  finish_kernel<<<(N + 127) / 128, 128, 0, s>>>(N, x64, a.beq_full, a.pinned, a.v);
  launches += 3;  // setup, batched CG, finish
  e = cudaGetLastError();
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  return EOLC_OK;
}

}  // namespace

// One learned batched solve with the per-instance Jacobi fallback, all on the
// device: set-up, caps, the learned launch, finish, the list of instances it
// left at their cap, their set-up, one Jacobi launch over that list, their
// finish.  No host synchronisation.
eolc_status batch_enqueue_learned(BatchSolveWork *w, const PcgArgs &a, const float *Gm,
                                  int fallback_factor, const int *node_inst, cudaStream_t s,
                                  std::string &err, long long &launches) {
  if (!w || w->config < 0 || w->prec != 1 || w->block_pc != 0) {
    err = "batch solver not prepared for mixed-precision Jacobi";
    return EOLC_BAD_ARG;
  }
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes;
  const float *A = a.A32;
  unsigned char *vp = w->vecs.p;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<float> *vr = reinterpret_cast<V4<float> *>(vp);
  Params<float> P{};
  P.r[0] = vr; P.r[1] = vr + N;
  P.w[0] = vr + 2 * N; P.w[1] = vr + 3 * N;  // learned: z, q
  P.s[0] = vr + 4 * N; P.s[1] = vr + 5 * N;  // learned: p ping-pong
  P.p = vr + 6 * N;
  P.xacc = vr + 7 * N;
  V4<float> *fmask = vr + 8 * N;
  float *pc = reinterpret_cast<float *>(w->pc.p);
  const int nn = (N + 127) / 128;
  setup_kernel<float><<<nn, 128, 0, s>>>(N, Tp.rowptr.p, Tp.colidx.p, Tp.diag.p, A, a.b,
                                         a.beq_full, a.pinned, 0, rhs, x64, P.r[0], P.p, P.s[0],
                                         P.xacc, pc, fmask);
  caps_kernel<<<(w->n_inst + 127) / 128, 128, 0, s>>>(w->n_inst, w->jac_iters.p, fallback_factor,
                                                      a.max_iter, w->cap.p);
  cudaMemsetAsync(w->queue.p, 0, sizeof(unsigned), s);
  P.n_nodes = N;
  P.rowptr = Tp.rowptr.p;
  P.A = A;
  P.lcol = w->lcol.p;
  P.tile_row = w->tile_row.p;
  P.tile_wptr = w->tile_wptr.p;
  P.wlist = w->wlist.p;
  P.rhs = rhs;
  P.x64 = x64;
  P.pc = pc;
  P.fmask = fmask;
  P.max_iter = a.max_iter;
  P.block_pc = 0;
  P.tol2 = a.rel_tol * a.rel_tol;
  BatchArgs B{};
  B.n_inst = w->n_inst;
  B.inst_tile = w->inst_tile.p;
  B.order = w->order.p;
  B.queue = w->queue.p;
  B.rec = w->rec.p;
  B.cap = w->cap.p;
  B.last_status = w->last_status.p;
  B.tol2 = a.rel_tol * a.rel_tol;
  B.max_iter = a.max_iter;
  const int k = w->config / kNumCluster, csize = kClusterSizes[w->config % kNumCluster];
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3(w->gen_grid);
  lc.blockDim = dim3(shape(k).threads);
  lc.dynamicSmemBytes = w->smem;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  {
    void *args[] = {&P, &B, &Gm};
    cudaError_t e = cudaLaunchKernelExC(&lc, gen_kernel_of(k), args);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  }
  finish_kernel<<<nn, 128, 0, s>>>(N, x64, a.beq_full, a.pinned, a.v);
  // Jacobi re-solve of the instances the learned launch left at their cap
  collect_failed_kernel<<<1, 1024, 0, s>>>(w->n_inst, w->order.p, w->last_status.p, w->order2.p,
                                           w->count.p, w->flag.p);
  setup_flagged_kernel<<<nn, 128, 0, s>>>(N, node_inst, w->flag.p, Tp.rowptr.p, Tp.colidx.p,
                                          Tp.diag.p, A, a.b, a.beq_full, a.pinned, rhs, x64,
                                          P.r[0], P.p, P.s[0], P.xacc, pc, fmask);
  cudaMemsetAsync(w->queue.p, 0, sizeof(unsigned), s);
  BatchArgs J = B;
  J.n_inst_d = w->count.p;
  J.order = w->order2.p;
  J.cap = nullptr;
  J.jac_iters = w->jac_iters.p;
  J.fallback = 1;
  lc.gridDim = dim3(w->grid);
  {
    void *args[] = {&P, &J};
    cudaError_t e = cudaLaunchKernelExC(&lc, kernel_of<float>(k), args);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  }
  finish_flagged_kernel<<<nn, 128, 0, s>>>(N, node_inst, w->flag.p, x64, a.beq_full, a.pinned,
                                           a.v);
  launches += 8;  // setup, caps, learned, finish, collect, setup, Jacobi, finish
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  return EOLC_OK;
}

eolc_status batch_enqueue(BatchSolveWork *w, const PcgArgs &a, cudaStream_t s, std::string &err,
                          long long &launches) {
  if (!w || w->config < 0) { err = "batch solver not prepared"; return EOLC_BAD_ARG; }
  if (a.precision == EOLC_PREC_FP64) return batch_enqueue_t<double>(w, a, s, err, launches);
  return batch_enqueue_t<float>(w, a, s, err, launches);
}

eolc_status batch_set_jacobi_reference(BatchSolveWork *w, const int *iters_h, int n,
                                       cudaStream_t s) {
  if (!w || int(w->jac_iters.n) < n) return EOLC_BAD_ARG;
  if (cudaMemcpyAsync(w->jac_iters.p, iters_h, sizeof(int) * n, cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  return EOLC_OK;
}

eolc_status batch_reset_records(BatchSolveWork *w, cudaStream_t s) {
  if (!w || !w->rec.p) return EOLC_BAD_ARG;
  return cudaMemsetAsync(w->rec.p, 0, sizeof(BatchRecord) * w->rec.n, s) == cudaSuccess
             ? EOLC_OK
             : EOLC_CUDA_ERROR;
}

eolc_status batch_read_records(BatchSolveWork *w, std::vector<BatchRecord> &out, cudaStream_t s) {
  if (!w || !w->rec.p) return EOLC_BAD_ARG;
  out.resize(w->n_inst);
  if (cudaMemcpyAsync(out.data(), w->rec.p, sizeof(BatchRecord) * w->n_inst,
                      cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  return EOLC_OK;
}

}  // namespace eolc
