// Preconditioned conjugate gradient on the 3x3 BSR matrix as ONE persistent
// cooperative kernel per solve, with one grid-wide barrier per iteration.
//
// Replaces the velocity solve of GeneralizedSolver::velocitySolve
// (GeneralizedSolver.cpp:107-173) for the pinned-corner case: the QP
// argmin 1/2 v'Av + b'v s.t. v_P = beq reduces to A_FF v_F = -b_F - A_FP beq.
// The iteration is Eigen's preconditioned CG (x0 = 0, stop on
// ||r|| <= tol ||rhs||, Jacobi preconditioner by default, the branch
// GeneralizedSolver.cpp:123-126 meant to take) written in the
// single-reduction form of Chronopoulos and Gear:
//     u = M r, w = A u, gamma = (r,u), delta = (w,u)
//     beta = gamma/gamma_old, alpha = gamma/(delta - beta gamma/alpha_old)
//     p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s
// so that the two inner products of an iteration are reduced together.
// Each neighbour's u = M (r - alpha (w + beta s)) is recomputed from its
// previous r, w, s when a tile's halo is staged, so an iteration needs ONE
// grid barrier (the reductions) instead of three.
//
// Mixed precision: inner vectors and matrix in FP32, every inner product
// accumulated in FP64, and "reliable updates": whenever the iterated residual
// has dropped by kDelta since the last check (or claims convergence), the
// FP32 solution increment is folded into an FP64 solution and the TRUE
// residual rhs - A x is recomputed in FP64 arithmetic, together with s = A p
// and w = A M r.  Convergence is declared only on that FP64 residual.  The
// FP64 path runs the same kernel with T = double.
//
// Layout: vectors are node-major with a padded 4th lane (one 16-byte load per
// node in FP32).  Rows are cut into tiles; a tile's BSR values and its
// tile-local 16-bit column indices are staged in shared memory with aligned
// 16-byte copies, and the tile's halo (the distinct columns it touches, a
// list built once per topology) is staged as one vector window.
// Barriers spin with an iteration cap; on expiry the kernel records
// EOLC_TIMEOUT and every CTA returns.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "cg_common.cuh"
#include "cg_tile.cuh"
#include "internal.h"

namespace eolc {

namespace {
using namespace cgc;

using C0 = TileCfg<512, 4, 112, 2048>;  // one CTA of 512 threads per SM
constexpr int kThreads = C0::kThreads;
constexpr int kValBytes = C0::kValBytes;
constexpr int kTileRows = C0::kTileRows;
constexpr int kRowThreads = C0::kRowThreads;

template <typename T>
constexpr int win_max() { return C0::win_max<T>(); }
template <typename T>
constexpr int cap_blocks() { return C0::cap_blocks<T>(); }
template <typename T>
constexpr size_t smem_bytes() { return C0::smem_bytes<T>(); }


template <typename T>
__global__ void __launch_bounds__(kThreads, 1)
cg_kernel(Params<T> P) {
  using A = Acc<T>;
  using V = typename A::V;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ V red[3 * (kThreads / 32 + 1)];
  __shared__ TileMeta tiles[kMaxCtaTiles];
  const int cta = blockIdx.x;
  const int G = P.n_ctas;
  unsigned epoch = 0;
  const int t0 = P.cta_tile[cta], t1 = P.cta_tile[cta + 1];
  const int ntiles = t1 - t0;
  for (int t = threadIdx.x; t < ntiles; t += kThreads) {
    TileMeta tm;
    tm.r0 = P.tile_row[t0 + t];
    tm.r1 = P.tile_row[t0 + t + 1];
    tm.b0 = P.rowptr[tm.r0];
    tm.b1 = P.rowptr[tm.r1];
    tm.w0 = P.tile_wptr[t0 + t];
    tm.wn = P.tile_wptr[t0 + t + 1] - tm.w0;
    tiles[t] = tm;
  }
  __syncthreads();
  const V tol2 = A::from_d(P.tol2 * __ldcg(&P.st->rhs_norm2));
  const V delta2 = A::from_d(kDelta * kDelta);
  V *partbuf = reinterpret_cast<V *>(P.part);
  int pset = 0;  // partial-sum buffers alternate between barriers

  int cur = 0;
  // initial residual r = rhs (x0 = 0): u = M r, w = A u
  V gam = A::zero(), del = A::zero(), rr = A::zero();
  cg_phase<C0, T, true>(P, tiles, ntiles, cur, T(0), T(0), smem, gam, del, rr);
#define EOLC_PUBLISH_AND_SYNC(a, b, c)                                  \
  do {                                                                  \
    block_sum3<C0, T>(a, b, c, red);                                        \
    V *pp = partbuf + size_t(3) * G * pset;                             \
    if (threadIdx.x == 0) {                                             \
      pp[3 * cta] = a; pp[3 * cta + 1] = b; pp[3 * cta + 2] = c;        \
    }                                                                   \
    if (!grid_barrier(P.bar, G, epoch, P.st, P.spin_limit)) return;                   \
    reduce_partials3<C0, T>(pp, G, a, b, c, red);                           \
    pset ^= 1;                                                          \
  } while (0)
  EOLC_PUBLISH_AND_SYNC(gam, del, rr);
  V rmax2 = rr;
  double last_rr64 = A::to_d(rr);
  int it = 0, nref = 0, status = EOLC_NOT_CONVERGED;
  bool converged = A::finite(rr) && A::le(rr, tol2);
  if (!A::finite(rr)) status = EOLC_NONFINITE;
  V gam_old = A::from_d(1.0), alpha_old = A::from_d(1.0);
  bool restart = true;  // beta = 0 on the first step
  while (!converged && status != EOLC_NONFINITE && it < P.max_iter) {
    const V beta = restart ? A::zero() : A::div(gam, gam_old);
    const V denom = restart ? del : A::add(del, A::neg(A::div(A::mul(beta, gam), alpha_old)));
    if (!A::pos(denom) || !A::pos(gam)) {
      status = (A::finite(denom) && A::finite(gam)) ? EOLC_BREAKDOWN : EOLC_NONFINITE;
      break;
    }
    const V alpha = A::div(gam, denom);
    restart = false;
    V g2 = A::zero(), d2 = A::zero(), rr2 = A::zero();
    cg_phase<C0, T, false>(P, tiles, ntiles, cur, T(A::to_t(alpha)), T(A::to_t(beta)), smem, g2,
                       d2, rr2);
    EOLC_PUBLISH_AND_SYNC(g2, d2, rr2);
    ++it;
    cur ^= 1;
    gam_old = gam;
    alpha_old = alpha;
    gam = g2;
    del = d2;
    rr = rr2;
    if (!A::finite(rr) || !A::finite(gam) || !A::finite(del)) { status = EOLC_NONFINITE; break; }
    if (!(A::lt(rr, A::mul(delta2, rmax2)) || A::le(rr, tol2) || it >= P.max_iter)) continue;
    // ---------------- reliable update ----------------------------------------
    // RU1: fold the low-precision increment into the FP64 solution.
    for (int t = 0; t < ntiles; ++t)
      for (int i = tiles[t].r0 + threadIdx.x; i < tiles[t].r1; i += kThreads) {
        const V4<T> xa = P.xacc[i];
        V4<double> x = P.x64[i];
        x.x += double(xa.x); x.y += double(xa.y); x.z += double(xa.z);
        P.x64[i] = x;
        P.xacc[i] = V4<T>{T(0), T(0), T(0), T(0)};
      }
    if (!grid_barrier(P.bar, G, epoch, P.st, P.spin_limit)) return;
    // RU2: r = rhs - A x64 (FP64), s = A p
    double rr64d = 0;
    ru_residual<C0>(P, tiles, ntiles, cur, smem, rr64d);
    V rr64 = A::from_d(rr64d), z0 = A::zero(), z1 = A::zero();
    EOLC_PUBLISH_AND_SYNC(rr64, z0, z1);
    ++nref;
    last_rr64 = A::to_d(rr64);
    rmax2 = rr64;
    if (!A::finite(rr64)) { status = EOLC_NONFINITE; break; }
    if (A::le(rr64, tol2)) { converged = true; break; }
    // RU3: u = M r, w = A u for the replaced residual
    V g3 = A::zero(), d3 = A::zero(), rr3 = A::zero();
    cg_phase<C0, T, true>(P, tiles, ntiles, cur, T(0), T(0), smem, g3, d3, rr3);
    EOLC_PUBLISH_AND_SYNC(g3, d3, rr3);
    gam = g3;
    del = d3;
  }
#undef EOLC_PUBLISH_AND_SYNC
  if (converged) status = EOLC_OK;
  if (cta == 0 && threadIdx.x == 0) {
    atomicCAS(&P.st->status, EOLC_OK, status);
    P.st->iterations = it;
    P.st->refinements = nref;
    P.st->rel_res = P.st->rhs_norm2 > 0 ? sqrt(last_rr64 / P.st->rhs_norm2) : 0.0;
  }
}

// ---- PCG with a non-local preconditioner (learned approximate inverse) ------
// Standard PCG with two grid barriers per iteration:
//   P1  p = z + beta p_old (halo on the fly), q = A p        -> barrier (p.q)
//   P2  r' = r - alpha q (halo on the fly), z = G r', x += alpha p
//                                                          -> barrier (r'.z, r'.r')
// G has the pattern of A, so both products reuse the tiles, local columns
// and halo lists.  Buffers (reusing Params fields): r[2] ping-pong r,
// w[0] = z, w[1] = q, s[0]/s[1] ping-pong p, xacc, x64.
template <typename T>
__global__ void __launch_bounds__(kThreads, 1)
pcg_general_kernel(Params<T> P, const T *Gm) {
  using A = Acc<T>;
  using V = typename A::V;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ V red[3 * (kThreads / 32 + 1)];
  __shared__ TileMeta tiles[kMaxCtaTiles];
  const int cta = blockIdx.x;
  const int G = P.n_ctas;
  unsigned epoch = 0;
  const int t0 = P.cta_tile[cta], t1 = P.cta_tile[cta + 1];
  const int ntiles = t1 - t0;
  for (int t = threadIdx.x; t < ntiles; t += kThreads) {
    TileMeta tm;
    tm.r0 = P.tile_row[t0 + t];
    tm.r1 = P.tile_row[t0 + t + 1];
    tm.b0 = P.rowptr[tm.r0];
    tm.b1 = P.rowptr[tm.r1];
    tm.w0 = P.tile_wptr[t0 + t];
    tm.wn = P.tile_wptr[t0 + t + 1] - tm.w0;
    tiles[t] = tm;
  }
  __syncthreads();
  const V tol2 = A::from_d(P.tol2 * __ldcg(&P.st->rhs_norm2));
  const V delta2 = A::from_d(kDelta * kDelta);
  V *partbuf = reinterpret_cast<V *>(P.part);
  int pset = 0;
#define EOLC_SYNC3(a, b, c)                                             \
  do {                                                                  \
    block_sum3<C0, T>(a, b, c, red);                                        \
    V *pp = partbuf + size_t(3) * G * pset;                             \
    if (threadIdx.x == 0) {                                             \
      pp[3 * cta] = a; pp[3 * cta + 1] = b; pp[3 * cta + 2] = c;        \
    }                                                                   \
    if (!grid_barrier(P.bar, G, epoch, P.st, P.spin_limit)) return;                   \
    reduce_partials3<C0, T>(pp, G, a, b, c, red);                           \
    pset ^= 1;                                                          \
  } while (0)
  int rcur = 0, pold = 0;
  V rz = A::zero(), rr = A::zero(), zz = A::zero();
  gen_phase<C0, T, kGenZ>(P, Gm, tiles, ntiles, rcur, pold, T(0), T(0), smem, rz, rr);
  EOLC_SYNC3(rz, rr, zz);
  V rmax2 = rr;
  double last_rr64 = A::to_d(rr);
  int it = 0, nref = 0, status = A::finite(rr) ? EOLC_NOT_CONVERGED : EOLC_NONFINITE;
  bool converged = A::finite(rr) && A::le(rr, tol2);
  V rz_prev = A::from_d(1.0);
  bool restart = true;
  while (!converged && status != EOLC_NONFINITE && it < P.max_iter) {
    const V beta = restart ? A::zero() : A::div(rz, rz_prev);
    restart = false;
    V pq = A::zero(), d1 = A::zero(), d2 = A::zero();
    gen_phase<C0, T, kGenP>(P, Gm, tiles, ntiles, rcur, pold, T(0), T(A::to_t(beta)), smem, pq, d1);
    EOLC_SYNC3(pq, d1, d2);
    if (!A::pos(pq) || !A::pos(rz)) {
      status = (A::finite(pq) && A::finite(rz)) ? EOLC_BREAKDOWN : EOLC_NONFINITE;
      break;
    }
    const V alpha = A::div(rz, pq);
    V rz2 = A::zero(), rr2 = A::zero(), d3 = A::zero();
    gen_phase<C0, T, kGenR>(P, Gm, tiles, ntiles, rcur, pold, T(A::to_t(alpha)), T(0), smem, rz2, rr2);
    EOLC_SYNC3(rz2, rr2, d3);
    ++it;
    rcur ^= 1;
    pold ^= 1;
    rz_prev = rz;
    rz = rz2;
    rr = rr2;
    if (!A::finite(rr) || !A::finite(rz)) { status = EOLC_NONFINITE; break; }
    if (!(A::lt(rr, A::mul(delta2, rmax2)) || A::le(rr, tol2) || it >= P.max_iter)) continue;
    for (int t = 0; t < ntiles; ++t)
      for (int i = tiles[t].r0 + threadIdx.x; i < tiles[t].r1; i += kThreads) {
        const V4<T> xa = P.xacc[i];
        V4<double> x = P.x64[i];
        x.x += double(xa.x); x.y += double(xa.y); x.z += double(xa.z);
        P.x64[i] = x;
        P.xacc[i] = V4<T>{T(0), T(0), T(0), T(0)};
      }
    if (!grid_barrier(P.bar, G, epoch, P.st, P.spin_limit)) return;
    double rr64d = 0;
    gen_ru_residual<C0>(P, tiles, ntiles, rcur, smem, rr64d);
    V rr64 = A::from_d(rr64d), e1 = A::zero(), e2 = A::zero();
    EOLC_SYNC3(rr64, e1, e2);
    ++nref;
    last_rr64 = A::to_d(rr64);
    rmax2 = rr64;
    if (!A::finite(rr64)) { status = EOLC_NONFINITE; break; }
    if (A::le(rr64, tol2)) { converged = true; break; }
    V rz3 = A::zero(), rr3 = A::zero(), e3 = A::zero();
    gen_phase<C0, T, kGenZ>(P, Gm, tiles, ntiles, rcur, pold, T(0), T(0), smem, rz3, rr3);
    EOLC_SYNC3(rz3, rr3, e3);
    rz = rz3;
  }
#undef EOLC_SYNC3
  if (converged) status = EOLC_OK;
  if (cta == 0 && threadIdx.x == 0) {
    atomicCAS(&P.st->status, EOLC_OK, status);
    P.st->iterations = it;
    P.st->refinements = nref;
    P.st->rel_res = P.st->rhs_norm2 > 0 ? sqrt(last_rr64 / P.st->rhs_norm2) : 0.0;
  }
}

// ---- set-up kernels (one launch each per solve) -----------------------------


}  // namespace

// ---------------------------------------------------------------------------
struct SolveWork {
  int n_nodes = 0, n_blocks = 0, G = 0, prec = -1, block_pc = -1;
  DevBuf<unsigned char> vecs;
  DevBuf<double> part;
  DevBuf<unsigned> bar;
  DevBuf<DevStatus> st;
  DevBuf<int> tile_row, tile_wptr, wlist, cta_tile;
  DevBuf<uint16_t> lcol;
  DevBuf<unsigned char> pc;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~SolveWork() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

void free_solve_work(SolveWork *w) { delete w; }

namespace {

template <typename T>
eolc_status run_pcg_t(SolveWork *&w, const PcgArgs &a, eolc_solve_info *info,
                      cudaStream_t s, std::string &err, long long &launches) {
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes;
  const T *A = std::is_same<T, double>::value ? reinterpret_cast<const T *>(a.A64)
                                              : reinterpret_cast<const T *>(a.A32);
  int dev = 0;
  cudaGetDevice(&dev);
  int n_sm = 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = smem_bytes<T>();
  cudaFuncSetAttribute(cg_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_kernel<T>, kThreads, smem);
  if (per_sm < 1) { err = "cg kernel does not fit on an SM"; return EOLC_CUDA_ERROR; }
  const int want_G = n_sm;  // one CTA per SM
  const int prec = std::is_same<T, double>::value ? 0 : 1;
  const int bpc = a.precond == EOLC_PC_BLOCK_JACOBI ? 1 : 0;
  if (!w) w = new SolveWork();
  if (w->n_nodes != N || w->n_blocks != Tp.n_blocks || w->prec != prec || w->block_pc != bpc) {
    std::vector<int> rowptr(N + 1), colidx(Tp.n_blocks);
    cudaMemcpy(rowptr.data(), Tp.rowptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost);
    cudaMemcpy(colidx.data(), Tp.colidx.p, sizeof(int) * Tp.n_blocks, cudaMemcpyDeviceToHost);
    std::vector<int> tiles, wptr, wlist;
    std::vector<uint16_t> lcol;
    std::string msg = build_tiles(N, rowptr, colidx, cap_blocks<T>(), win_max<T>(), kTileRows, tiles, wptr,
                                  wlist, lcol);
    if (!msg.empty()) { err = msg; return EOLC_BAD_ARG; }
    const int nt = int(tiles.size()) - 1;
    const int G = std::min(want_G, nt);
    if ((nt + G - 1) / G > kMaxCtaTiles / 2) { err = "matrix too large for one solve"; return EOLC_BAD_ARG; }
    // contiguous tile ranges per CTA, balanced by block count
    std::vector<int> cta(G + 1, nt);
    cta[0] = 0;
    const long long total = rowptr[N];
    int t = 0;
    for (int c = 1; c < G; ++c) {
      long long target = total * c / G;
      while (t < nt && rowptr[tiles[t]] < target) ++t;
      cta[c] = std::max(t, cta[c - 1] + 1);
      if (cta[c] > nt - (G - c)) cta[c] = nt - (G - c);
    }
    for (int c = 0; c < G; ++c)
      if (cta[c + 1] - cta[c] > kMaxCtaTiles) { err = "tile partition too uneven"; return EOLC_BAD_ARG; }
    // local columns are padded by 8 entries for the 16-byte staging tail
    lcol.resize(lcol.size() + 8, 0);
    w->G = G;
    w->n_nodes = N;
    w->n_blocks = Tp.n_blocks;
    w->prec = prec;
    w->block_pc = bpc;
    cudaError_t es[] = {
        w->tile_row.upload(tiles.data(), tiles.size(), s),
        w->tile_wptr.upload(wptr.data(), wptr.size(), s),
        w->wlist.upload(wlist.data(), std::max<size_t>(wlist.size(), 1), s),
        w->lcol.upload(lcol.data(), lcol.size(), s),
        w->cta_tile.upload(cta.data(), cta.size(), s),
        w->vecs.resize(size_t(N) * (sizeof(V4<double>) * 2 + sizeof(V4<T>) * 9)),
        w->part.resize(size_t(6) * G),
        w->bar.resize(2),
        w->st.resize(1),
        w->pc.resize(size_t(N) * 9 * sizeof(T)),
        cudaStreamSynchronize(s)};
    for (cudaError_t e : es)
      if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  }
  const int G = w->G;
  unsigned char *vp = w->vecs.p;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<T> *vr = reinterpret_cast<V4<T> *>(vp);
  Params<T> P;
  P.r[0] = vr; P.r[1] = vr + N;
  P.w[0] = vr + 2 * N; P.w[1] = vr + 3 * N;
  P.s[0] = vr + 4 * N; P.s[1] = vr + 5 * N;
  P.p = vr + 6 * N;
  P.xacc = vr + 7 * N;
  V4<T> *fmask = vr + 8 * N;
  T *pc = reinterpret_cast<T *>(w->pc.p);
  setup_kernel<T><<<(N + 127) / 128, 128, 0, s>>>(
      N, Tp.rowptr.p, Tp.colidx.p, Tp.diag.p, A, a.b, a.beq_full, a.pinned, bpc, rhs, x64,
      P.r[0], P.p, P.s[0], P.xacc, pc, fmask);
  init_sums_kernel<C0><<<1, kThreads, 0, s>>>(N, rhs, w->st.p);
  cudaMemsetAsync(w->bar.p, 0, sizeof(unsigned) * 2, s);
  P.n_nodes = N;
  P.n_ctas = G;
  P.rowptr = Tp.rowptr.p;
  P.A = A;
  P.lcol = w->lcol.p;
  P.tile_row = w->tile_row.p;
  P.tile_wptr = w->tile_wptr.p;
  P.wlist = w->wlist.p;
  P.cta_tile = w->cta_tile.p;
  P.rhs = rhs;
  P.x64 = x64;
  P.pc = pc;
  P.fmask = fmask;
  P.part = w->part.p;
  P.bar = w->bar.p;
  P.st = w->st.p;
  P.max_iter = a.max_iter;
  P.block_pc = bpc;
  P.spin_limit = a.spin_limit > 0 ? a.spin_limit : kDefaultSpinLimit;
  P.tol2 = a.rel_tol * a.rel_tol;
  void *args[] = {&P};
  if (!w->ev0) { cudaEventCreate(&w->ev0); cudaEventCreate(&w->ev1); }
  cudaEventRecord(w->ev0, s);
  cudaError_t e = cudaLaunchCooperativeKernel((void *)cg_kernel<T>, dim3(G), dim3(kThreads),
                                              args, smem, s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  cudaEventRecord(w->ev1, s);
  finish_kernel<<<(N + 127) / 128, 128, 0, s>>>(N, x64, a.beq_full, a.pinned, a.v);
  launches += 4;  // setup, init_sums, cg, finish
  DevStatus hs;
  cudaMemcpyAsync(&hs, w->st.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  float kms = 0.f;
  cudaEventElapsedTime(&kms, w->ev0, w->ev1);
  if (info) {
    info->status = hs.status;
    info->iterations = hs.iterations;
    info->refinements = hs.refinements;
    info->used_fallback = 0;
    info->rel_res = hs.rel_res;
    info->solve_kernel_ms = kms;
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
                    cudaStream_t s, std::string &err, long long &launches) {
  if (a.precision == EOLC_PREC_FP64) return run_pcg_t<double>(w, a, info, s, err, launches);
  return run_pcg_t<float>(w, a, info, s, err, launches);
}

namespace {

// PCG with the preconditioner matrix G (FP32, pattern of A) on the mixed path.
eolc_status run_pcg_general_f(SolveWork *&w, const PcgArgs &a, const float *Gm,
                              eolc_solve_info *info, cudaStream_t s, std::string &err,
                              long long &launches) {
  using T = float;
  // the tiling and vectors are the point-Jacobi layout's
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes;
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = smem_bytes<T>();
  cudaFuncSetAttribute(pcg_general_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  // build (or reuse) the tiling through the Jacobi path's bookkeeping
  if (!w || w->n_nodes != N || w->n_blocks != Tp.n_blocks || w->prec != 1 || w->block_pc != 0) {
    std::vector<int> rowptr(N + 1), colidx(Tp.n_blocks);
    cudaMemcpy(rowptr.data(), Tp.rowptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost);
    cudaMemcpy(colidx.data(), Tp.colidx.p, sizeof(int) * Tp.n_blocks, cudaMemcpyDeviceToHost);
    std::vector<int> tiles, wptr, wlist;
    std::vector<uint16_t> lcol;
    std::string msg = build_tiles(N, rowptr, colidx, cap_blocks<T>(), win_max<T>(), kTileRows, tiles, wptr,
                                  wlist, lcol);
    if (!msg.empty()) { err = msg; return EOLC_BAD_ARG; }
    const int nt = int(tiles.size()) - 1;
    const int G = std::min(n_sm, nt);
    if ((nt + G - 1) / G > kMaxCtaTiles / 2) { err = "matrix too large for one solve"; return EOLC_BAD_ARG; }
    std::vector<int> cta(G + 1, nt);
    cta[0] = 0;
    const long long total = rowptr[N];
    int t = 0;
    for (int c = 1; c < G; ++c) {
      long long target = total * c / G;
      while (t < nt && rowptr[tiles[t]] < target) ++t;
      cta[c] = std::max(t, cta[c - 1] + 1);
      if (cta[c] > nt - (G - c)) cta[c] = nt - (G - c);
    }
    lcol.resize(lcol.size() + 8, 0);
    if (!w) w = new SolveWork();
    w->G = G; w->n_nodes = N; w->n_blocks = Tp.n_blocks; w->prec = 1; w->block_pc = 0;
    cudaError_t es[] = {
        w->tile_row.upload(tiles.data(), tiles.size(), s),
        w->tile_wptr.upload(wptr.data(), wptr.size(), s),
        w->wlist.upload(wlist.data(), std::max<size_t>(wlist.size(), 1), s),
        w->lcol.upload(lcol.data(), lcol.size(), s),
        w->cta_tile.upload(cta.data(), cta.size(), s),
        w->vecs.resize(size_t(N) * (sizeof(V4<double>) * 2 + sizeof(V4<T>) * 9)),
        w->part.resize(size_t(6) * G), w->bar.resize(2), w->st.resize(1),
        w->pc.resize(size_t(N) * 9 * sizeof(T)), cudaStreamSynchronize(s)};
    for (cudaError_t e : es)
      if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  }
  const int G = w->G;
  unsigned char *vp = w->vecs.p;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<T> *vr = reinterpret_cast<V4<T> *>(vp);
  Params<T> P;
  P.r[0] = vr; P.r[1] = vr + N;
  P.w[0] = vr + 2 * N; P.w[1] = vr + 3 * N;   // z, q
  P.s[0] = vr + 4 * N; P.s[1] = vr + 5 * N;   // p ping-pong
  P.p = vr + 6 * N;
  P.xacc = vr + 7 * N;
  V4<T> *fmask = vr + 8 * N;
  T *pc = reinterpret_cast<T *>(w->pc.p);
  const T *Amat = a.A32;
  setup_kernel<T><<<(N + 127) / 128, 128, 0, s>>>(N, Tp.rowptr.p, Tp.colidx.p, Tp.diag.p, Amat,
                                                   a.b, a.beq_full, a.pinned, 0, rhs, x64, P.r[0],
                                                   P.p, P.s[0], P.xacc, pc, fmask);
  init_sums_kernel<C0><<<1, kThreads, 0, s>>>(N, rhs, w->st.p);
  cudaMemsetAsync(w->bar.p, 0, sizeof(unsigned) * 2, s);
  cudaMemsetAsync(P.s[0], 0, sizeof(V4<T>) * N, s);
  P.n_nodes = N; P.n_ctas = G; P.rowptr = Tp.rowptr.p; P.A = Amat; P.lcol = w->lcol.p;
  P.tile_row = w->tile_row.p; P.tile_wptr = w->tile_wptr.p; P.wlist = w->wlist.p;
  P.cta_tile = w->cta_tile.p; P.rhs = rhs; P.x64 = x64; P.pc = pc; P.fmask = fmask;
  P.part = w->part.p; P.bar = w->bar.p; P.st = w->st.p; P.max_iter = a.max_iter; P.block_pc = 0;
  P.spin_limit = a.spin_limit > 0 ? a.spin_limit : kDefaultSpinLimit;
  P.tol2 = a.rel_tol * a.rel_tol;
  void *args[] = {&P, &Gm};
  if (!w->ev0) { cudaEventCreate(&w->ev0); cudaEventCreate(&w->ev1); }
  cudaEventRecord(w->ev0, s);
  cudaError_t e = cudaLaunchCooperativeKernel((void *)pcg_general_kernel<T>, dim3(G),
                                              dim3(kThreads), args, smem, s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  cudaEventRecord(w->ev1, s);
  finish_kernel<<<(N + 127) / 128, 128, 0, s>>>(N, x64, a.beq_full, a.pinned, a.v);
  launches += 4;
  DevStatus hs;
  cudaMemcpyAsync(&hs, w->st.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  float kms = 0.f;
  cudaEventElapsedTime(&kms, w->ev0, w->ev1);
  if (info) {
    info->status = hs.status;
    info->iterations = hs.iterations;
    info->refinements = hs.refinements;
    info->used_fallback = 0;
    info->rel_res = hs.rel_res;
    info->solve_kernel_ms = kms;
  }
  if (hs.status != EOLC_OK)
    err = hs.status == EOLC_BREAKDOWN ? "PCG breakdown" : hs.status == EOLC_NONFINITE
                                                              ? "non-finite value in PCG"
                                                              : "PCG did not converge";
  return eolc_status(hs.status);
}

}  // namespace

eolc_status run_pcg_learned(SolveWork *&w, const PcgArgs &a, const float *Gm,
                            eolc_solve_info *info, cudaStream_t s, std::string &err,
                            long long &launches) {
  if (a.precision != EOLC_PREC_MIXED) {
    err = "the learned preconditioner runs on the mixed-precision path";
    return EOLC_BAD_ARG;
  }
  return run_pcg_general_f(w, a, Gm, info, s, err, launches);
}

}  // namespace eolc

// ===========================================================================
// Velocity solve that allocates nothing on the device.
//
// For callers that cannot call cudaMalloc on their step path: an interactive
// stepping thread (the reference's online mode steps and renders every frame)
// cannot afford cudaMalloc/cudaFree, which may synchronize the device and take
// milliseconds, and a host framework that reserves all device memory in its
// own pool leaves nothing for a library allocator.  This entry point runs the
// same mixed-precision Jacobi PCG kernels as eolc_velocity_solve, with every
// scratch buffer carved out of one file-scope device array of fixed size.
// The caller passes the matrix, right-hand side and solution in its own
// device buffers.  Limits: EOLC_STATIC_MAX_NODES block rows and
// EOLC_STATIC_MAX_BLOCKS 3x3 blocks.
// ===========================================================================
namespace eolc {
namespace {

constexpr size_t kStaticMaxCtas = 1024;

constexpr size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct StaticLayout {
  size_t A, rowptr, colidx, diag, lcol, wlist, tile_row, tile_wptr, cta_tile, pinned,
      beq, vecs, pc, part, bar, st, total;
};

constexpr StaticLayout static_layout() {
  StaticLayout L{};
  const size_t N = EOLC_STATIC_MAX_NODES, NB = EOLC_STATIC_MAX_BLOCKS;
  size_t o = 0;
  L.A = o;         o += al256((NB * 9 + 16) * sizeof(float));
  L.rowptr = o;    o += al256((N + 1) * sizeof(int));
  L.colidx = o;    o += al256(NB * sizeof(int));
  L.diag = o;      o += al256(N * sizeof(int));
  L.lcol = o;      o += al256((NB + 8) * sizeof(uint16_t));
  L.wlist = o;     o += al256(NB * sizeof(int));  // windows never exceed the blocks
  L.tile_row = o;  o += al256((N + 1) * sizeof(int));
  L.tile_wptr = o; o += al256((N + 1) * sizeof(int));
  L.cta_tile = o;  o += al256((kStaticMaxCtas + 1) * sizeof(int));
  L.pinned = o;    o += al256(3 * N);
  L.beq = o;       o += al256(3 * N * sizeof(double));
  L.vecs = o;      o += al256(N * (2 * sizeof(V4<double>) + 9 * sizeof(V4<float>)));
  L.pc = o;        o += al256(N * 4 * sizeof(float));
  L.part = o;      o += al256(6 * kStaticMaxCtas * sizeof(double));
  L.bar = o;       o += al256(2 * sizeof(unsigned));
  L.st = o;        o += al256(sizeof(DevStatus));
  L.total = o;
  return L;
}

constexpr StaticLayout kStatic = static_layout();

}  // namespace
}  // namespace eolc

// The scratch itself: every GPU that loads this library holds it until exit.
static __device__ __align__(256) unsigned char g_eolc_static_scratch[eolc::kStatic.total];

namespace {
std::mutex g_static_mutex;
void *g_static_addr[64] = {nullptr};  // symbol address per device, set once
}  // namespace

extern "C" eolc_status eolc_velocity_solve_static(
    int n_nodes, const int *rowptr_h, const int *colidx_h, const float *mdk_d,
    const double *b_d, const int *fixed_dofs_h, const double *beq_h, int n_fixed,
    double rel_tol, int max_iter, double *v_d, eolc_solve_info *info, void *stream) {
  using namespace eolc;
  using T = float;
  if (n_nodes <= 0 || !rowptr_h || !colidx_h || !mdk_d || !b_d || !v_d ||
      (n_fixed > 0 && (!fixed_dofs_h || !beq_h)) || n_fixed < 0 || !(rel_tol > 0) ||
      max_iter <= 0)
    return EOLC_BAD_ARG;
  if (n_nodes > EOLC_STATIC_MAX_NODES) return EOLC_CAPACITY;
  const int nb = rowptr_h[n_nodes];
  if (nb <= 0 || nb > EOLC_STATIC_MAX_BLOCKS) return EOLC_CAPACITY;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return EOLC_CUDA_ERROR;
  unsigned char *base = nullptr;
  {
    // one-time set-up per device, with that device current
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_addr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_eolc_static_scratch) != cudaSuccess || !p)
        return EOLC_CUDA_ERROR;
      g_static_addr[dev] = p;
    }
    base = static_cast<unsigned char *>(g_static_addr[dev]);
  }
  // pattern checks and host-side tiling (host memory only)
  std::vector<int> rowptr(rowptr_h, rowptr_h + n_nodes + 1), colidx(colidx_h, colidx_h + nb);
  std::vector<int> diag(n_nodes, -1);
  for (int i = 0; i < n_nodes; ++i) {
    if (rowptr[i + 1] < rowptr[i]) return EOLC_BAD_ARG;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      if (colidx[k] < 0 || colidx[k] >= n_nodes) return EOLC_BAD_ARG;
      if (colidx[k] == i) diag[i] = k;
    }
    if (diag[i] < 0) return EOLC_BAD_ARG;
  }
  std::vector<int> tiles, wptr, wlist;
  std::vector<uint16_t> lcol;
  if (!build_tiles(n_nodes, rowptr, colidx, cap_blocks<T>(), win_max<T>(), kTileRows, tiles, wptr, wlist,
                   lcol).empty())
    return EOLC_BAD_ARG;
  lcol.resize(lcol.size() + 8, 0);
  // the tiling's arrays must fit their fixed slots of the scratch array
  // (windows never exceed the blocks and tiles never exceed the rows, but a
  // broken invariant must not write past a slot)
  if (wlist.size() > size_t(EOLC_STATIC_MAX_BLOCKS) || tiles.size() > size_t(n_nodes) + 1 ||
      wptr.size() > size_t(n_nodes) + 1 || lcol.size() > size_t(EOLC_STATIC_MAX_BLOCKS) + 8)
    return EOLC_CAPACITY;
  const int nt = int(tiles.size()) - 1;
  int n_sm = 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int G = std::min({n_sm, nt, int(kStaticMaxCtas)});
  if ((nt + G - 1) / G > kMaxCtaTiles / 2) return EOLC_CAPACITY;
  std::vector<int> cta(G + 1, nt);
  cta[0] = 0;
  {
    const long long total = rowptr[n_nodes];
    int t = 0;
    for (int c = 1; c < G; ++c) {
      long long target = total * c / G;
      while (t < nt && rowptr[tiles[t]] < target) ++t;
      cta[c] = std::max(t, cta[c - 1] + 1);
      if (cta[c] > nt - (G - c)) cta[c] = nt - (G - c);
    }
  }
  for (int c = 0; c < G; ++c)
    if (cta[c + 1] - cta[c] > kMaxCtaTiles) return EOLC_CAPACITY;
  std::vector<uint8_t> pinned(size_t(3) * n_nodes, 0);
  std::vector<double> beq_full(size_t(3) * n_nodes, 0.0);
  for (int k = 0; k < n_fixed; ++k) {
    if (fixed_dofs_h[k] < 0 || fixed_dofs_h[k] >= 3 * n_nodes) return EOLC_BAD_ARG;
    pinned[fixed_dofs_h[k]] = 1;
    beq_full[fixed_dofs_h[k]] = beq_h[k];
  }
  const StaticLayout &L = kStatic;
  T *A = reinterpret_cast<T *>(base + L.A);
  int *d_rowptr = reinterpret_cast<int *>(base + L.rowptr);
  int *d_colidx = reinterpret_cast<int *>(base + L.colidx);
  int *d_diag = reinterpret_cast<int *>(base + L.diag);
  uint16_t *d_lcol = reinterpret_cast<uint16_t *>(base + L.lcol);
  int *d_wlist = reinterpret_cast<int *>(base + L.wlist);
  int *d_tile_row = reinterpret_cast<int *>(base + L.tile_row);
  int *d_tile_wptr = reinterpret_cast<int *>(base + L.tile_wptr);
  int *d_cta = reinterpret_cast<int *>(base + L.cta_tile);
  uint8_t *d_pinned = base + L.pinned;
  double *d_beq = reinterpret_cast<double *>(base + L.beq);
  double *d_part = reinterpret_cast<double *>(base + L.part);
  unsigned *d_bar = reinterpret_cast<unsigned *>(base + L.bar);
  DevStatus *d_st = reinterpret_cast<DevStatus *>(base + L.st);
  const int N = n_nodes;
  unsigned char *vp = base + L.vecs;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<T> *vr = reinterpret_cast<V4<T> *>(vp);
  T *pc = reinterpret_cast<T *>(base + L.pc);
  cudaError_t es[] = {
      cudaMemcpyAsync(A, mdk_d, sizeof(T) * size_t(nb) * 9, cudaMemcpyDeviceToDevice, s),
      cudaMemsetAsync(A + size_t(nb) * 9, 0, sizeof(T) * 16, s),
      cudaMemcpyAsync(d_rowptr, rowptr.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_colidx, colidx.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_diag, diag.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_lcol, lcol.data(), sizeof(uint16_t) * lcol.size(), cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_wlist, wlist.data(), sizeof(int) * std::max<size_t>(wlist.size(), 1),
                      cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_tile_row, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_tile_wptr, wptr.data(), sizeof(int) * wptr.size(), cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_cta, cta.data(), sizeof(int) * cta.size(), cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_pinned, pinned.data(), pinned.size(), cudaMemcpyHostToDevice, s),
      cudaMemcpyAsync(d_beq, beq_full.data(), sizeof(double) * beq_full.size(),
                      cudaMemcpyHostToDevice, s),
      // the array keeps the previous call's contents: the barrier counter and
      // the partial sums must start at zero
      cudaMemsetAsync(d_bar, 0, sizeof(unsigned) * 2, s),
      cudaMemsetAsync(d_part, 0, sizeof(double) * 6 * G, s)};
  for (cudaError_t e : es)
    if (e != cudaSuccess) return EOLC_CUDA_ERROR;
  Params<T> P;
  P.r[0] = vr; P.r[1] = vr + N;
  P.w[0] = vr + 2 * N; P.w[1] = vr + 3 * N;
  P.s[0] = vr + 4 * N; P.s[1] = vr + 5 * N;
  P.p = vr + 6 * N;
  P.xacc = vr + 7 * N;
  V4<T> *fmask = vr + 8 * N;
  setup_kernel<T><<<(N + 127) / 128, 128, 0, s>>>(N, d_rowptr, d_colidx, d_diag, A, b_d, d_beq,
                                                   d_pinned, 0, rhs, x64, P.r[0], P.p, P.s[0],
                                                   P.xacc, pc, fmask);
  init_sums_kernel<C0><<<1, kThreads, 0, s>>>(N, rhs, d_st);
  P.n_nodes = N;
  P.n_ctas = G;
  P.rowptr = d_rowptr;
  P.A = A;
  P.lcol = d_lcol;
  P.tile_row = d_tile_row;
  P.tile_wptr = d_tile_wptr;
  P.wlist = d_wlist;
  P.cta_tile = d_cta;
  P.rhs = rhs;
  P.x64 = x64;
  P.pc = pc;
  P.fmask = fmask;
  P.part = d_part;
  P.bar = d_bar;
  P.st = d_st;
  P.max_iter = max_iter;
  P.block_pc = 0;
  P.spin_limit = kDefaultSpinLimit;
  P.tol2 = rel_tol * rel_tol;
  const size_t smem = smem_bytes<T>();
  if (cudaFuncSetAttribute(cg_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           int(smem)) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  void *args[] = {&P};
  if (cudaLaunchCooperativeKernel((void *)cg_kernel<T>, dim3(G), dim3(kThreads), args, smem, s) !=
      cudaSuccess)
    return EOLC_CUDA_ERROR;
  finish_kernel<<<(N + 127) / 128, 128, 0, s>>>(N, x64, d_beq, d_pinned, v_d);
  DevStatus hs;
  if (cudaMemcpyAsync(&hs, d_st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  if (info) {
    info->status = hs.status;
    info->iterations = hs.iterations;
    info->refinements = hs.refinements;
    info->used_fallback = 0;
    info->rel_res = hs.rel_res;
    info->solve_kernel_ms = 0.0;
    info->assemble_ms = 0.0;
  }
  return eolc_status(hs.status);
}
