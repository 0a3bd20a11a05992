// PCG with a patch-local preconditioner whose matrices live in shared memory.
//
// The velocity solve on this GPU is bound by synchronisation latency, not by
// bytes: a Jacobi-PCG iteration costs one grid barrier plus one pass over
// the matrix, and the 256^2 sheet needs ~800 of them.  This preconditioner
// spends on-chip work instead of grid barriers:
//
//   * the nodes are reordered by recursive graph bisection into one compact
//     patch per CTA (one CTA per SM), so a CTA owns a contiguous range of
//     rows of the permuted system;
//   * each CTA keeps the principal submatrix of its patch, symmetrically
//     scaled to unit diagonal (A^ = S A S, S = diag^-1/2) and stored in FP16,
//     resident in shared memory for the whole solve (~100 KB at 435 rows);
//   * the preconditioner is M = blockdiag_p( S q_p(B^ A^_pp) B^ S ), a
//     degree-k Chebyshev polynomial in the block-Jacobi-preconditioned patch
//     matrix (B^ = inverse 3x3 diagonal blocks of A^), applied with CTA
//     barriers only.  Its interval [l/30, l] takes l from the infinity norm
//     of B^ A^_pp (an upper bound of its spectrum), so q_p > 0 on the whole
//     spectrum and M is symmetric positive definite: plain PCG applies.
//
// An iteration has two grid barriers: one for p'q after q = A p (the p halo
// is recomputed from z and the previous p, so no exchange barrier), one for
// r'z and r'r after the local solves.  The outer matrix product uses the
// FP32 BSR matrix staged tile by tile; inner products are double-float;
// convergence is declared on an FP64 true residual (reliable updates, as in
// the Jacobi kernel), so the result meets the same FP64 criterion.
//
// No counterpart in the reference, whose solve is Eigen's Jacobi CG
// (GeneralizedSolver.cpp:123-126); the judge of every result is the same
// FP64 relative residual.
#include <cuda/atomic>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "cg_common.cuh"
#include "cg_tile.cuh"
#include "internal.h"

namespace eolc {

namespace {
using namespace cgc;

using CA = TileCfg<512, 8, 30, 512>;  // outer product: 64-row tiles, 8 threads per row
constexpr int kPThreads = CA::kThreads;
constexpr int kMaxPatchRows = 464;     // rows of one patch (one thread each)
constexpr int kMaxLocalBlocks = 6016;  // blocks of one patch's principal submatrix
constexpr int kWinA = CA::kWinMaxF;    // halo nodes of an outer-product tile
constexpr float kLoFrac = 30.f;        // Chebyshev interval [lmax / 30, lmax]
constexpr float kBoundMargin = 1.02f;  // FP16 rounding margin on the norm bound
constexpr int kLeafRows = CA::kTileRows;
static_assert(kMaxPatchRows <= kPThreads, "one thread per patch row");

constexpr size_t al16(size_t x) { return (x + 15) & ~size_t(15); }
// shared-memory layout (bytes)
constexpr size_t kOffVals = 0;  // 10 halves per block (9 used)
constexpr size_t kOffLc = al16(kOffVals + size_t(kMaxLocalBlocks) * 20);
constexpr size_t kOffLp = al16(kOffLc + size_t(kMaxLocalBlocks) * 2);
constexpr size_t kOffB = al16(kOffLp + size_t(kMaxPatchRows + 1) * 2);
constexpr size_t kOffS = al16(kOffB + size_t(kMaxPatchRows) * 9 * 4);
constexpr size_t kOffVec = al16(kOffS + size_t(kMaxPatchRows) * 16);  // y, res, d
constexpr size_t kVecBytes = size_t(kMaxPatchRows) * 16 * 3;
constexpr size_t kOffA = al16(kOffVec + kVecBytes);                    // tile values + cols
constexpr size_t kOffW = kOffA + size_t(CA::kValBytes);                // p window
constexpr size_t kPatchSmem = kOffW + size_t(kWinA) * 16;
static_assert(size_t(kWinA) * sizeof(V4<double>) <= kVecBytes,
              "the FP64 residual window overlays the Chebyshev vectors");
static_assert(kPatchSmem <= 220 * 1024, "patch solver exceeds shared memory");

struct PatchParams {
  Params<float> Q;        // permuted system: rowptr, A, lcol, tiles, vectors
  const int *diag;        // diagonal block of every permuted row
  const int *tr;          // block (j, i) of every block (i, j)
  const int *patch_row;   // n_ctas + 1 row boundaries
  const int *lptr;        // n_nodes + 1: first local block of every row
  const int *lblk;        // permuted block of every local block
  const uint16_t *llc;    // patch-local column of every local block
  V4<float> *z, *q;
  V4<float> *pp[2];       // search direction, ping-pong
  int degree;             // Chebyshev degree
};

__device__ __forceinline__ void load9(const float *p, float (&m)[9]) {
#pragma unroll
  for (int k = 0; k < 9; ++k) m[k] = __ldg(p + k);
}

// Inverse of a symmetric 3x3 block in FP64 (pinned axes: identity, then
// masked out), returned in FP32.
__device__ void inverse3_masked(const float (&D)[9], const float (&m)[3], float (&out)[9]) {
  double M[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      M[r][c] = (m[r] == 0.f || m[c] == 0.f) ? (r == c ? 1.0 : 0.0) : double(D[3 * r + c]);
  const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
  const double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
  const double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
  const double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
  double inv[9];
  if (det > 0.0) {
    const double id = 1.0 / det;
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
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[3 * r + c] = float(inv[3 * r + c] * double(m[r]) * double(m[c]));
}

__device__ __forceinline__ float3 mul3(const float *B, float x, float y, float z) {
  return make_float3(B[0] * x + B[1] * y + B[2] * z, B[3] * x + B[4] * y + B[5] * z,
                     B[6] * x + B[7] * y + B[8] * z);
}

struct PatchSmem {
  __half2 *vals;
  uint16_t *lc, *lp;
  float *B;
  float4 *S, *Y, *R, *D;
  unsigned char *tileA;
};

// Local solve on the patch: Y = q(B^ A^) B^ R by k Chebyshev steps on
// [lmax / kLoFrac, lmax] (R is overwritten by the local residual).
__device__ void patch_chebyshev(const PatchSmem &sm, int np, int k, float lmax) {
  const int i = threadIdx.x;
  const float lo = lmax / kLoFrac;
  const float theta = 0.5f * (lmax + lo), delta = 0.5f * (lmax - lo);
  const float sigma = theta / delta;
  float rho = 1.f / sigma;
  float4 y = make_float4(0.f, 0.f, 0.f, 0.f), d = y, res = y;
  const float *Bi = sm.B + 9 * i;
  if (i < np) {
    res = sm.R[i];
    const float3 t = mul3(Bi, res.x, res.y, res.z);
    d = make_float4(t.x / theta, t.y / theta, t.z / theta, 0.f);
    sm.D[i] = d;
  }
  for (int s = 0; s < k; ++s) {
    y.x += d.x; y.y += d.y; y.z += d.z;
    if (s == k - 1) break;
    __syncthreads();  // d complete
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (i < np) {
      for (int b = sm.lp[i]; b < sm.lp[i + 1]; ++b) {
        const float4 dj = sm.D[sm.lc[b]];
        const __half2 *h = sm.vals + 5 * b;
        const float2 m01 = __half22float2(h[0]), m23 = __half22float2(h[1]),
                     m45 = __half22float2(h[2]), m67 = __half22float2(h[3]),
                     m8 = __half22float2(h[4]);
        a0 += m01.x * dj.x + m01.y * dj.y + m23.x * dj.z;
        a1 += m23.y * dj.x + m45.x * dj.y + m45.y * dj.z;
        a2 += m67.x * dj.x + m67.y * dj.y + m8.x * dj.z;
      }
    }
    __syncthreads();  // every read of d done
    const float rho1 = 1.f / (2.f * sigma - rho);
    if (i < np) {
      res.x -= a0; res.y -= a1; res.z -= a2;
      const float3 t = mul3(Bi, res.x, res.y, res.z);
      const float c1 = rho1 * rho, c2 = 2.f * rho1 / delta;
      d = make_float4(c1 * d.x + c2 * t.x, c1 * d.y + c2 * t.y, c1 * d.z + c2 * t.z, 0.f);
      sm.D[i] = d;
    }
    rho = rho1;
  }
  if (i < np) sm.Y[i] = y;
  __syncthreads();
}

// Own rows of the patch: [r -= alpha q, x += alpha p], z = M r.
// Accumulates r'z and r'r.
__device__ void patch_precond(const PatchParams &P, const PatchSmem &sm, int p0, int np,
                              bool update, float alpha, int pnew, float lmax,
                              Acc<float>::V &g, Acc<float>::V &rr) {
  using A = Acc<float>;
  const int i = threadIdx.x;
  V4<float> r{};
  float4 S = make_float4(0.f, 0.f, 0.f, 0.f);
  if (i < np) {
    const int row = p0 + i;
    r = P.Q.r[0][row];
    if (update) {
      const V4<float> q = P.q[row], pn = P.pp[pnew][row];
      V4<float> xa = P.Q.xacc[row];
      r.x -= alpha * q.x; r.y -= alpha * q.y; r.z -= alpha * q.z;
      xa.x += alpha * pn.x; xa.y += alpha * pn.y; xa.z += alpha * pn.z;
      P.Q.xacc[row] = xa;
      P.Q.r[0][row] = r;
    }
    rr = A::addf(rr, dot3(r, r));
    S = sm.S[i];
    sm.R[i] = make_float4(S.x * r.x, S.y * r.y, S.z * r.z, 0.f);
  }
  __syncthreads();
  patch_chebyshev(sm, np, P.degree, lmax);
  if (i < np) {
    const float4 y = sm.Y[i];
    const V4<float> z{S.x * y.x, S.y * y.y, S.z * y.z, 0.f};
    P.z[p0 + i] = z;
    g = A::addf(g, dot3(r, z));
  }
}

// q = A p over this CTA's tiles, with p = z + beta p_old recomputed on every
// halo node (written for own rows to pp[cur ^ 1]).  Accumulates p'q.
__device__ void patch_apass(const PatchParams &P, const PatchSmem &sm, const TileMeta *tiles,
                            int ntiles, int cur, float beta, Acc<float>::V &pq) {
  using A = Acc<float>;
  V4<float> *sU = reinterpret_cast<V4<float> *>(sm.tileA + CA::kValBytes);
  __shared__ V4<float> sOwn[CA::kTileRows];
  __shared__ int sRow[CA::kTileRows + 1];
  const int lrow = threadIdx.x / CA::kRowThreads, part = threadIdx.x % CA::kRowThreads;
  const V4<float> *po = P.pp[cur];
  V4<float> *pn = P.pp[cur ^ 1];
  for (int t = 0; t < ntiles; ++t) {
    const TileMeta tm = tiles[t];
    const int i = tm.r0 + lrow;
    const bool owner = i < tm.r1 && part == 0;
    V4<float> m{};
    if (owner) m = P.Q.fmask[i];
    const float *sA;
    const uint16_t *sL;
    stage_tile<CA>(P.Q, tm, sm.tileA, sA, sL, sRow);
    for (int j = threadIdx.x; j < tm.wn; j += kPThreads) {
      const int node = __ldg(P.Q.wlist + tm.w0 + j);
      const V4<float> zj = P.z[node], pj = po[node];
      const V4<float> u{zj.x + beta * pj.x, zj.y + beta * pj.y, zj.z + beta * pj.z, 0.f};
      sU[j] = u;
      if (node >= tm.r0 && node < tm.r1) {
        sOwn[node - tm.r0] = u;
        pn[node] = u;
      }
    }
    __syncthreads();
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (i < tm.r1) {
      const int q0 = sRow[lrow], q1 = sRow[lrow + 1];
      for (int k = q0 + part; k < q1; k += CA::kRowThreads) {
        const V4<float> u = sU[sL[k]];
        const float *blk = sA + size_t(k) * 9;
        a0 += blk[0] * u.x + blk[1] * u.y + blk[2] * u.z;
        a1 += blk[3] * u.x + blk[4] * u.y + blk[5] * u.z;
        a2 += blk[6] * u.x + blk[7] * u.y + blk[8] * u.z;
      }
    }
#pragma unroll
    for (int o = 1; o < CA::kRowThreads; o <<= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (owner) {
      const V4<float> qv{a0 * m.x, a1 * m.y, a2 * m.z, 0.f};
      P.q[i] = qv;
      pq = A::addf(pq, dot3(sOwn[lrow], qv));
    }
    __syncthreads();
  }
}

// Reliable update: r = rhs - A x64 in FP64 arithmetic over this CTA's tiles.
__device__ void patch_true_residual(const PatchParams &P, const PatchSmem &sm,
                                    const TileMeta *tiles, int ntiles, double &rr64) {
  V4<double> *sX = reinterpret_cast<V4<double> *>(sm.Y);  // overlays the Chebyshev vectors
  __shared__ int sRow[CA::kTileRows + 1];
  const int lrow = threadIdx.x / CA::kRowThreads, part = threadIdx.x % CA::kRowThreads;
  for (int t = 0; t < ntiles; ++t) {
    const TileMeta tm = tiles[t];
    const float *sA;
    const uint16_t *sL;
    stage_tile<CA>(P.Q, tm, sm.tileA, sA, sL, sRow);
    for (int j = threadIdx.x; j < tm.wn; j += kPThreads)
      sX[j] = P.Q.x64[__ldg(P.Q.wlist + tm.w0 + j)];
    __syncthreads();
    const int i = tm.r0 + lrow;
    double a0 = 0, a1 = 0, a2 = 0;
    if (i < tm.r1) {
      for (int k = sRow[lrow] + part; k < sRow[lrow + 1]; k += CA::kRowThreads) {
        const V4<double> xj = sX[sL[k]];
        const float *blk = sA + size_t(k) * 9;
        a0 += double(blk[0]) * xj.x + double(blk[1]) * xj.y + double(blk[2]) * xj.z;
        a1 += double(blk[3]) * xj.x + double(blk[4]) * xj.y + double(blk[5]) * xj.z;
        a2 += double(blk[6]) * xj.x + double(blk[7]) * xj.y + double(blk[8]) * xj.z;
      }
    }
#pragma unroll
    for (int o = 1; o < CA::kRowThreads; o <<= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (i < tm.r1 && part == 0) {
      const V4<double> b = P.Q.rhs[i];
      const V4<float> m = P.Q.fmask[i];
      const double e0 = (b.x - a0) * double(m.x), e1 = (b.y - a1) * double(m.y),
                   e2 = (b.z - a2) * double(m.z);
      rr64 += e0 * e0 + e1 * e1 + e2 * e2;
      P.Q.r[0][i] = V4<float>{float(e0), float(e1), float(e2), 0.f};
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kPThreads, 1) patch_pcg_kernel(PatchParams P) {
  using A = Acc<float>;
  using V = A::V;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ V red[3 * (kPThreads / 32 + 1)];
  __shared__ TileMeta tiles[kMaxCtaTiles];
  __shared__ float s_max[kPThreads / 32];
  PatchSmem sm;
  sm.vals = reinterpret_cast<__half2 *>(smem + kOffVals);
  sm.lc = reinterpret_cast<uint16_t *>(smem + kOffLc);
  sm.lp = reinterpret_cast<uint16_t *>(smem + kOffLp);
  sm.B = reinterpret_cast<float *>(smem + kOffB);
  sm.S = reinterpret_cast<float4 *>(smem + kOffS);
  sm.Y = reinterpret_cast<float4 *>(smem + kOffVec);
  sm.R = sm.Y + kMaxPatchRows;
  sm.D = sm.R + kMaxPatchRows;
  sm.tileA = smem + kOffA;
  const int cta = blockIdx.x;
  const int G = P.Q.n_ctas;
  unsigned epoch = 0;
  const int p0 = P.patch_row[cta], np = P.patch_row[cta + 1] - p0;
  const int t0 = P.Q.cta_tile[cta], ntiles = P.Q.cta_tile[cta + 1] - t0;
  for (int t = threadIdx.x; t < ntiles; t += kPThreads) {
    TileMeta tm;
    tm.r0 = P.Q.tile_row[t0 + t];
    tm.r1 = P.Q.tile_row[t0 + t + 1];
    tm.b0 = P.Q.rowptr[tm.r0];
    tm.b1 = P.Q.rowptr[tm.r1];
    tm.w0 = P.Q.tile_wptr[t0 + t];
    tm.wn = P.Q.tile_wptr[t0 + t + 1] - tm.w0;
    tiles[t] = tm;
  }
  // ---- patch set-up: scaling, block-Jacobi inverses, FP16 submatrix, bound
  const int i = threadIdx.x;
  float lmax_row = 0.f;
  if (i < np) {
    const int row = p0 + i;
    float D[9];
    load9(P.Q.A + size_t(P.diag[row]) * 9, D);
    const V4<float> fm = P.Q.fmask[row];
    const float m[3] = {fm.x, fm.y, fm.z};
    float s[3];
    for (int c = 0; c < 3; ++c) s[c] = (m[c] != 0.f && D[4 * c] > 0.f) ? 1.f / sqrtf(D[4 * c]) : 0.f;
    sm.S[i] = make_float4(s[0], s[1], s[2], 0.f);
    float Dh[9];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) Dh[3 * r + c] = (0.5f * (D[3 * r + c] + D[3 * c + r])) * (s[r] * s[c]);
    float Bi[9];
    inverse3_masked(Dh, m, Bi);
    for (int k = 0; k < 9; ++k) sm.B[9 * i + k] = Bi[k];
  }
  __syncthreads();
  if (i < np) {
    const int row = p0 + i;
    const int base = P.lptr[p0];
    const int b0 = P.lptr[row] - base, b1 = P.lptr[row + 1] - base;
    sm.lp[i] = uint16_t(b0);
    if (i == np - 1) sm.lp[np] = uint16_t(b1);
    const float4 si = sm.S[i];
    const float Si[3] = {si.x, si.y, si.z};
    const float *Bi = sm.B + 9 * i;
    float acc[3] = {0.f, 0.f, 0.f};
    for (int b = b0; b < b1; ++b) {
      const int k = P.lblk[base + b];
      const int jl = P.llc[base + b];
      float Aij[9], Aji[9];
      load9(P.Q.A + size_t(k) * 9, Aij);
      load9(P.Q.A + size_t(P.tr[k]) * 9, Aji);
      const float4 sj = sm.S[jl];
      const float Sj[3] = {sj.x, sj.y, sj.z};
      float h[9];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          h[3 * r + c] = (0.5f * (Aij[3 * r + c] + Aji[3 * c + r])) * (Si[r] * Sj[c]);
      __half2 *dst = sm.vals + 5 * b;
      dst[0] = __floats2half2_rn(h[0], h[1]);
      dst[1] = __floats2half2_rn(h[2], h[3]);
      dst[2] = __floats2half2_rn(h[4], h[5]);
      dst[3] = __floats2half2_rn(h[6], h[7]);
      dst[4] = __floats2half2_rn(h[8], 0.f);
      sm.lc[b] = uint16_t(jl);
      // row sums of |B_i A^_ij| (infinity norm of B^ A^_pp)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          acc[r] += fabsf(Bi[3 * r] * h[c] + Bi[3 * r + 1] * h[3 + c] + Bi[3 * r + 2] * h[6 + c]);
    }
    lmax_row = fmaxf(acc[0], fmaxf(acc[1], acc[2]));
  }
  for (int o = 16; o > 0; o >>= 1) lmax_row = fmaxf(lmax_row, __shfl_xor_sync(0xffffffffu, lmax_row, o));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = lmax_row;
  __syncthreads();
  float lmax = 0.f;
  for (int w = 0; w < kPThreads / 32; ++w) lmax = fmaxf(lmax, s_max[w]);
  lmax = fmaxf(kBoundMargin * lmax, 1e-30f);

  V *partbuf = reinterpret_cast<V *>(P.Q.part);
  int pset = 0;
#define EOLC_PATCH_SYNC(a, b, c)                                        \
  do {                                                                  \
    block_sum3<CA, float>(a, b, c, red);                                \
    V *pp_ = partbuf + size_t(3) * G * pset;                            \
    if (threadIdx.x == 0) {                                             \
      pp_[3 * cta] = a; pp_[3 * cta + 1] = b; pp_[3 * cta + 2] = c;     \
    }                                                                   \
    if (!grid_barrier(P.Q.bar, G, epoch, P.Q.st)) return;               \
    reduce_partials3<CA, float>(pp_, G, a, b, c, red);                  \
    pset ^= 1;                                                          \
  } while (0)

  // ||rhs||^2 (FP64) and the first preconditioned residual
  double n0 = 0;
  if (i < np) {
    const V4<double> b = P.Q.rhs[p0 + i];
    n0 = b.x * b.x + b.y * b.y + b.z * b.z;
  }
  V gam = A::zero(), rr = A::zero();
  patch_precond(P, sm, p0, np, false, 0.f, 0, lmax, gam, rr);
  V nrm = A::from_d(n0);  // this thread's share of ||rhs||^2
  EOLC_PATCH_SYNC(gam, rr, nrm);
  const double rhs2 = A::to_d(nrm);
  const V tol2 = A::from_d(P.Q.tol2 * rhs2);
  const V delta2 = A::from_d(kDelta * kDelta);
  V rmax2 = rr;
  double last_rr64 = A::to_d(rr);
  int it = 0, nref = 0, status = EOLC_NOT_CONVERGED;
  bool converged = A::finite(rr) && A::le(rr, tol2);
  if (!A::finite(rr) || !A::finite(gam)) status = EOLC_NONFINITE;
  V gam_old = A::from_d(1.0);
  bool restart = true;
  int cur = 0;  // pp[cur] holds the current search direction's predecessor
  while (!converged && status != EOLC_NONFINITE && it < P.Q.max_iter) {
    const V beta = restart ? A::zero() : A::div(gam, gam_old);
    restart = false;
    V pq = A::zero(), e1 = A::zero(), e2 = A::zero();
    patch_apass(P, sm, tiles, ntiles, cur, float(A::to_t(beta)), pq);
    EOLC_PATCH_SYNC(pq, e1, e2);
    if (!A::pos(pq) || !A::pos(gam)) {
      status = (A::finite(pq) && A::finite(gam)) ? EOLC_BREAKDOWN : EOLC_NONFINITE;
      break;
    }
    const V alpha = A::div(gam, pq);
    V g2 = A::zero(), rr2 = A::zero(), e3 = A::zero();
    patch_precond(P, sm, p0, np, true, float(A::to_t(alpha)), cur ^ 1, lmax, g2, rr2);
    EOLC_PATCH_SYNC(g2, rr2, e3);
    ++it;
    cur ^= 1;
    gam_old = gam;
    gam = g2;
    rr = rr2;
    if (!A::finite(rr) || !A::finite(gam)) { status = EOLC_NONFINITE; break; }
    if (!(A::lt(rr, A::mul(delta2, rmax2)) || A::le(rr, tol2) || it >= P.Q.max_iter)) continue;
    // reliable update: fold the FP32 increment into the FP64 solution, then
    // replace r by the FP64 true residual and z by M r
    if (i < np) {
      const int row = p0 + i;
      const V4<float> xa = P.Q.xacc[row];
      V4<double> x = P.Q.x64[row];
      x.x += double(xa.x); x.y += double(xa.y); x.z += double(xa.z);
      P.Q.x64[row] = x;
      P.Q.xacc[row] = V4<float>{0.f, 0.f, 0.f, 0.f};
    }
    if (!grid_barrier(P.Q.bar, G, epoch, P.Q.st)) return;
    double rr64d = 0;
    patch_true_residual(P, sm, tiles, ntiles, rr64d);
    V g3 = A::zero(), rr3 = A::zero();
    patch_precond(P, sm, p0, np, false, 0.f, 0, lmax, g3, rr3);
    V rr64 = A::from_d(rr64d);
    EOLC_PATCH_SYNC(rr64, g3, rr3);
    ++nref;
    last_rr64 = A::to_d(rr64);
    rmax2 = rr64;
    gam = g3;
    if (!A::finite(rr64) || !A::finite(gam)) { status = EOLC_NONFINITE; break; }
    if (A::le(rr64, tol2)) { converged = true; break; }
  }
#undef EOLC_PATCH_SYNC
  if (converged) status = EOLC_OK;
  if (cta == 0 && threadIdx.x == 0) {
    atomicCAS(&P.Q.st->status, EOLC_OK, status);
    P.Q.st->iterations = it;
    P.Q.st->refinements = nref;
    P.Q.st->rhs_norm2 = rhs2;
    P.Q.st->rel_res = rhs2 > 0 ? sqrt(last_rr64 / rhs2) : 0.0;
  }
}

// ---- per-solve permutation kernels --------------------------------------------
__global__ void permute_blocks_kernel(int nb, const int *__restrict__ src,
                                      const float *__restrict__ A, float *__restrict__ Ap) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const float *s = A + size_t(src[k]) * 9;
  float *d = Ap + size_t(k) * 9;
#pragma unroll
  for (int c = 0; c < 9; ++c) d[c] = __ldg(s + c);
}

__global__ void permute_vectors_kernel(int n, const int *__restrict__ perm,
                                       const double *__restrict__ b, const double *__restrict__ beq,
                                       const uint8_t *__restrict__ pinned, double *__restrict__ bp,
                                       double *__restrict__ beqp, uint8_t *__restrict__ pinp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  for (int c = 0; c < 3; ++c) {
    bp[3 * i + c] = b[3 * o + c];
    beqp[3 * i + c] = beq[3 * o + c];
    pinp[3 * i + c] = pinned[3 * o + c];
  }
}

__global__ void unpermute_finish_kernel(int n, const int *__restrict__ perm,
                                        const V4<double> *__restrict__ x64,
                                        const double *__restrict__ beq,
                                        const uint8_t *__restrict__ pinned, double *__restrict__ v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  const V4<double> x = x64[i];
  const double xs[3] = {x.x, x.y, x.z};
  for (int c = 0; c < 3; ++c) v[3 * o + c] = pinned[3 * o + c] ? beq[3 * o + c] : xs[c];
}

// ---- host: patches by recursive graph bisection -------------------------------
struct Bisector {
  const std::vector<int> &rowptr, &colidx;
  std::vector<int> mark, dist, queue;
  int stamp = 0;
  Bisector(const std::vector<int> &rp, const std::vector<int> &ci)
      : rowptr(rp), colidx(ci), mark(rp.size() - 1, -1), dist(rp.size() - 1, 0) {}

  // BFS over the subgraph induced by `set` from src; unreached nodes of the
  // set follow in set order.
  void bfs(const std::vector<int> &set, int src, std::vector<int> &order) {
    ++stamp;
    for (int v : set) mark[v] = stamp;
    order.clear();
    order.push_back(src);
    mark[src] = -stamp;
    for (size_t h = 0; h < order.size(); ++h) {
      const int u = order[h];
      for (int k = rowptr[u]; k < rowptr[u + 1]; ++k) {
        const int v = colidx[k];
        if (mark[v] == stamp) { mark[v] = -stamp; order.push_back(v); }
      }
      if (h + 1 == order.size() && order.size() < set.size()) {
        for (int v : set)
          if (mark[v] == stamp) { mark[v] = -stamp; order.push_back(v); break; }
      }
    }
  }

  // Splits set into `parts` pieces of near-equal size (BFS prefixes from a
  // pseudo-peripheral node); leaves are ordered the same way down to
  // `leaf` nodes.  Appends the ordered nodes to out and, at depth `parts`,
  // the piece boundaries to bounds.
  void split(const std::vector<int> &set, int parts, int leaf, std::vector<int> &out,
             std::vector<int> *bounds) {
    if (set.empty() || (parts <= 1 && int(set.size()) <= leaf)) {
      out.insert(out.end(), set.begin(), set.end());
      if (bounds) bounds->push_back(int(out.size()));
      return;
    }
    std::vector<int> order;
    bfs(set, set[0], order);
    bfs(set, order.back(), order);
    if (parts <= 1) {
      const size_t half = order.size() / 2;
      std::vector<int> a(order.begin(), order.begin() + half), b(order.begin() + half, order.end());
      split(a, 1, leaf, out, nullptr);
      split(b, 1, leaf, out, nullptr);
      if (bounds) bounds->push_back(int(out.size()));
      return;
    }
    const int pl = parts / 2, pr = parts - pl;
    const size_t cut = size_t((long long)order.size() * pl / parts);
    std::vector<int> a(order.begin(), order.begin() + cut), b(order.begin() + cut, order.end());
    split(a, pl, leaf, out, bounds);
    split(b, pr, leaf, out, bounds);
  }
};

}  // namespace

struct PatchPlan {
  int G = 0;
  std::vector<int> perm, rowptr, colidx, src, tr, diag, patch_row, tile_row, tile_wptr, wlist,
      cta_tile, lptr, lblk;
  std::vector<uint16_t> lcol, llc;
};

struct PatchWork {
  int n_nodes = 0, n_blocks = 0, G = 0;
  bool ok = false;
  std::string why;
  DevBuf<int> perm, rowptr, colidx, diag, tr, src, tile_row, tile_wptr, wlist, cta_tile,
      patch_row, lptr, lblk;
  DevBuf<uint16_t> lcol, llc;
  DevBuf<float> Ap;
  DevBuf<unsigned char> vecs, pc, pinp;
  DevBuf<double> bp, beqp, part;
  DevBuf<unsigned> bar;
  DevBuf<DevStatus> st;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~PatchWork() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

void free_patch_work(PatchWork *w) { delete w; }

// Host plan of the patch solver for a BSR pattern: permutation, permuted
// pattern with source and transpose blocks, patch and tile boundaries, and
// the patch-internal block lists.  Returns "" or the reason it does not fit.
std::string build_patch_plan(int N, const std::vector<int> &rowptr,
                             const std::vector<int> &colidx, int n_sm, PatchPlan &out) {
  const int NB = int(colidx.size());
  // patches: as many as SMs, but at least ~256 rows each on small meshes
  const int G = std::max(1, std::min(n_sm, (N + 255) / 256));
  if ((N + G - 1) / G > kMaxPatchRows) {
    return "mesh too large for shared-memory patches on this device";
  }
  std::vector<int> all(N), perm, bounds;
  for (int k = 0; k < N; ++k) all[k] = k;
  perm.reserve(N);
  Bisector bis(rowptr, colidx);
  bis.split(all, G, kLeafRows, perm, &bounds);
  if (int(perm.size()) != N || int(bounds.size()) != G) {
    return "patch partition failed";
  }
  std::vector<int> iperm(N);
  for (int k = 0; k < N; ++k) iperm[perm[k]] = k;
  // permuted pattern, source blocks, transposes, diagonals
  std::vector<int> prow(N + 1, 0), pcol(NB), psrc(NB), ptr(NB), pdiag(N, -1);
  for (int i = 0; i < N; ++i) prow[i + 1] = prow[i] + rowptr[perm[i] + 1] - rowptr[perm[i]];
  std::vector<std::pair<int, int>> tmp;
  for (int i = 0; i < N; ++i) {
    const int o = perm[i];
    tmp.clear();
    for (int k = rowptr[o]; k < rowptr[o + 1]; ++k) tmp.push_back({iperm[colidx[k]], k});
    std::sort(tmp.begin(), tmp.end());
    for (size_t q = 0; q < tmp.size(); ++q) {
      pcol[prow[i] + q] = tmp[q].first;
      psrc[prow[i] + q] = tmp[q].second;
      if (tmp[q].first == i) pdiag[i] = prow[i] + int(q);
    }
  }
  for (int i = 0; i < N; ++i)
    for (int k = prow[i]; k < prow[i + 1]; ++k) {
      const int j = pcol[k];
      const int *b = pcol.data() + prow[j], *e = pcol.data() + prow[j + 1];
      const int *f = std::lower_bound(b, e, i);
      if (f == e || *f != i) return "matrix pattern is not symmetric";
      ptr[k] = int(f - pcol.data());
    }
  std::vector<int> patch_row(G + 1, 0);
  for (int c = 0; c < G; ++c) patch_row[c + 1] = bounds[c];
  // outer-product tiles inside each patch
  std::vector<int> breaks(patch_row.begin() + 1, patch_row.end() - 1);
  std::vector<int> tiles, wptr, wlist;
  std::vector<uint16_t> lcol;
  std::string msg = build_tiles(N, prow, pcol, CA::cap_blocks<float>(), kWinA, CA::kTileRows,
                                tiles, wptr, wlist, lcol, &breaks);
  if (!msg.empty()) return msg;
  std::vector<int> cta(G + 1, 0);
  {
    int t = 0;
    for (int c = 0; c <= G; ++c) {
      while (t < int(tiles.size()) - 1 && tiles[t] < patch_row[c]) ++t;
      cta[c] = t;
    }
    cta[G] = int(tiles.size()) - 1;
  }
  for (int c = 0; c < G; ++c)
    if (cta[c + 1] - cta[c] > kMaxCtaTiles) return "patch has too many tiles";
  // local (patch-internal) blocks
  std::vector<int> lptr(N + 1, 0), lblk;
  std::vector<uint16_t> llc;
  for (int c = 0; c < G; ++c) {
    const int r0 = patch_row[c], r1 = patch_row[c + 1];
    if (r1 - r0 > kMaxPatchRows) return "patch too large";
    const size_t first = lblk.size();
    for (int i = r0; i < r1; ++i) {
      lptr[i] = int(lblk.size());
      for (int k = prow[i]; k < prow[i + 1]; ++k)
        if (pcol[k] >= r0 && pcol[k] < r1) {
          lblk.push_back(k);
          llc.push_back(uint16_t(pcol[k] - r0));
        }
    }
    if (lblk.size() - first > size_t(kMaxLocalBlocks))
      return "patch submatrix exceeds shared memory";
  }
  lptr[N] = int(lblk.size());
  lcol.resize(lcol.size() + 8, 0);
  out.G = G;
  out.perm = std::move(perm);
  out.rowptr = std::move(prow);
  out.colidx = std::move(pcol);
  out.src = std::move(psrc);
  out.tr = std::move(ptr);
  out.diag = std::move(pdiag);
  out.patch_row = std::move(patch_row);
  out.tile_row = std::move(tiles);
  out.tile_wptr = std::move(wptr);
  out.wlist = std::move(wlist);
  out.lcol = std::move(lcol);
  out.cta_tile = std::move(cta);
  out.lptr = std::move(lptr);
  out.lblk = std::move(lblk);
  out.llc = std::move(llc);
  return "";
}

namespace {

eolc_status patch_plan(PatchWork *w, const DevTopology &Tp, int n_sm, cudaStream_t s,
                       std::string &err) {
  const int N = Tp.n_nodes, NB = Tp.n_blocks;
  std::vector<int> rowptr(N + 1), colidx(NB);
  cudaMemcpy(rowptr.data(), Tp.rowptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost);
  cudaMemcpy(colidx.data(), Tp.colidx.p, sizeof(int) * NB, cudaMemcpyDeviceToHost);
  PatchPlan L;
  err = build_patch_plan(N, rowptr, colidx, n_sm, L);
  if (!err.empty()) return EOLC_BAD_ARG;
  const int G = L.G;
  const std::vector<int> &perm = L.perm, &prow = L.rowptr, &pcol = L.colidx, &pdiag = L.diag,
                         &ptr = L.tr, &psrc = L.src, &tiles = L.tile_row, &wptr = L.tile_wptr,
                         &wlist = L.wlist, &cta = L.cta_tile, &patch_row = L.patch_row,
                         &lptr = L.lptr, &lblk = L.lblk;
  const std::vector<uint16_t> &lcol = L.lcol, &llc = L.llc;
  cudaError_t es[] = {
      w->perm.upload(perm.data(), N, s),
      w->rowptr.upload(prow.data(), N + 1, s),
      w->colidx.upload(pcol.data(), NB, s),
      w->diag.upload(pdiag.data(), N, s),
      w->tr.upload(ptr.data(), NB, s),
      w->src.upload(psrc.data(), NB, s),
      w->tile_row.upload(tiles.data(), tiles.size(), s),
      w->tile_wptr.upload(wptr.data(), wptr.size(), s),
      w->wlist.upload(wlist.data(), std::max<size_t>(wlist.size(), 1), s),
      w->cta_tile.upload(cta.data(), cta.size(), s),
      w->patch_row.upload(patch_row.data(), patch_row.size(), s),
      w->lptr.upload(lptr.data(), lptr.size(), s),
      w->lblk.upload(lblk.data(), std::max<size_t>(lblk.size(), 1), s),
      w->lcol.upload(lcol.data(), lcol.size(), s),
      w->llc.upload(llc.data(), std::max<size_t>(llc.size(), 1), s),
      w->Ap.resize(size_t(NB) * 9 + 16),
      w->vecs.resize(size_t(N) * (sizeof(V4<double>) * 2 + sizeof(V4<float>) * 9)),
      w->pc.resize(size_t(N) * 4 * sizeof(float)),
      w->pinp.resize(size_t(N) * 3),
      w->bp.resize(size_t(N) * 3),
      w->beqp.resize(size_t(N) * 3),
      w->part.resize(size_t(6) * G),
      w->bar.resize(2),
      w->st.resize(1),
      cudaMemsetAsync(w->Ap.p + size_t(NB) * 9, 0, sizeof(float) * 16, s),
      cudaStreamSynchronize(s)};
  for (cudaError_t e : es)
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  w->n_nodes = N;
  w->n_blocks = NB;
  w->G = G;
  return EOLC_OK;
}

}  // namespace

eolc_status run_pcg_patch(PatchWork *&w, const PcgArgs &a, int degree, eolc_solve_info *info,
                          cudaStream_t s, std::string &err, long long &launches) {
  if (a.precision != EOLC_PREC_MIXED) {
    err = "the patch preconditioner runs on the mixed-precision path";
    return EOLC_BAD_ARG;
  }
  const DevTopology &Tp = *a.T;
  const int N = Tp.n_nodes, NB = Tp.n_blocks;
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  if (!w) w = new PatchWork();
  if (w->n_nodes != N || w->n_blocks != NB) {
    w->n_nodes = 0;
    eolc_status st = patch_plan(w, Tp, n_sm, s, err);
    if (st != EOLC_OK) return st;
  }
  cudaFuncSetAttribute(patch_pcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(kPatchSmem));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, patch_pcg_kernel, kPThreads, kPatchSmem);
  if (per_sm < 1 || w->G > per_sm * n_sm) {
    err = "patch kernel does not fit on the device";
    return EOLC_CUDA_ERROR;
  }
  const int G = w->G;
  unsigned char *vp = w->vecs.p;
  V4<double> *rhs = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<double> *x64 = reinterpret_cast<V4<double> *>(vp); vp += sizeof(V4<double>) * N;
  V4<float> *vr = reinterpret_cast<V4<float> *>(vp);
  PatchParams P{};
  P.Q.r[0] = vr;
  P.z = vr + N;
  P.pp[0] = vr + 2 * N;
  P.pp[1] = vr + 3 * N;
  P.q = vr + 4 * N;
  P.Q.xacc = vr + 5 * N;
  V4<float> *fmask = vr + 6 * N;
  V4<float> *scratch = vr + 7 * N;  // setup_kernel's s output (unused here)
  const int nb_blocks = (NB + 255) / 256, nn = (N + 127) / 128;
  permute_blocks_kernel<<<nb_blocks, 256, 0, s>>>(NB, w->src.p, a.A32, w->Ap.p);
  permute_vectors_kernel<<<nn, 128, 0, s>>>(N, w->perm.p, a.b, a.beq_full, a.pinned, w->bp.p,
                                             w->beqp.p, w->pinp.p);
  setup_kernel<float><<<nn, 128, 0, s>>>(N, w->rowptr.p, w->colidx.p, w->diag.p, w->Ap.p, w->bp.p,
                                         w->beqp.p, w->pinp.p, 0, rhs, x64, P.Q.r[0], P.pp[0],
                                         scratch, P.Q.xacc, reinterpret_cast<float *>(w->pc.p),
                                         fmask);
  cudaMemsetAsync(w->bar.p, 0, sizeof(unsigned) * 2, s);
  DevStatus st0{};
  st0.status = EOLC_OK;
  cudaMemcpyAsync(w->st.p, &st0, sizeof(DevStatus), cudaMemcpyHostToDevice, s);
  P.Q.n_nodes = N;
  P.Q.n_ctas = G;
  P.Q.rowptr = w->rowptr.p;
  P.Q.A = w->Ap.p;
  P.Q.lcol = w->lcol.p;
  P.Q.tile_row = w->tile_row.p;
  P.Q.tile_wptr = w->tile_wptr.p;
  P.Q.wlist = w->wlist.p;
  P.Q.cta_tile = w->cta_tile.p;
  P.Q.rhs = rhs;
  P.Q.x64 = x64;
  P.Q.fmask = fmask;
  P.Q.part = w->part.p;
  P.Q.bar = w->bar.p;
  P.Q.st = w->st.p;
  P.Q.max_iter = a.max_iter;
  P.Q.tol2 = a.rel_tol * a.rel_tol;
  P.diag = w->diag.p;
  P.tr = w->tr.p;
  P.patch_row = w->patch_row.p;
  P.lptr = w->lptr.p;
  P.lblk = w->lblk.p;
  P.llc = w->llc.p;
  P.degree = std::max(1, std::min(degree, 64));
  void *args[] = {&P};
  if (!w->ev0) { cudaEventCreate(&w->ev0); cudaEventCreate(&w->ev1); }
  cudaEventRecord(w->ev0, s);
  cudaError_t e = cudaLaunchCooperativeKernel((void *)patch_pcg_kernel, dim3(G), dim3(kPThreads),
                                              args, kPatchSmem, s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  cudaEventRecord(w->ev1, s);
  unpermute_finish_kernel<<<nn, 128, 0, s>>>(N, w->perm.p, x64, a.beq_full, a.pinned, a.v);
  launches += 5;  // permute x2, setup, patch PCG, finish
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
    err = hs.status == EOLC_TIMEOUT     ? "grid barrier timed out"
          : hs.status == EOLC_BREAKDOWN ? "PCG breakdown"
          : hs.status == EOLC_NONFINITE ? "non-finite value in PCG"
                                        : "PCG did not converge";
  return eolc_status(hs.status);
}

}  // namespace eolc
