// Assembly of MDK (and optionally M) into the fixed 3x3 BSR pattern, and of
// the force / right-hand side vectors.
//
// Replaces the triplet loops of faceBasedF / edgeBasedF and the two
// setFromTriplets calls (Forces.cpp:331-930) plus b = -(M v + h f)
// (Cloth.cpp:345).
//
// Matrix blocks, one launch (tile_blocks_kernel): the block rows are cut into
// tiles of consecutive rows whose element blocks fit in shared memory.  A CTA
// takes one tile.  Every (element, local vertex) pair whose vertex is a row
// of the tile is a task: it evaluates that row's blocks of the element (3 for
// a triangle, d_B h^2 K_e plus the mass t8/12 or t8/24; 4 for a hinge,
// d_B h^2 K_b) into shared memory.  Then each output value (block, entry) of
// the tile sums the contributions that land in its block, in the reference's
// insertion order (faces ascending with their mass terms, then hinges
// ascending), from shared memory, and is stored once: consecutive threads
// store consecutive words, so the BSR is written with full-sector coalesced
// stores and nothing but the BSR goes to memory.  No atomics: bit-
// reproducible.  Element matrices are symmetric: a block (a, b) with a > b is
// the transpose of the evaluated (b, a), and a block and its partner sum the
// same elements in the same order.  The block formulas are compiled once per
// local row (vertex selections folded to constants), so the two evaluations
// of an element block may contract their multiply-adds differently: the
// matrix is symmetric to the last bit of its precision, not exactly.
//
// EOL topologies (and meshes whose rows do not fit a tile) take the two-pass
// path: an element pass (one thread per triangle, one per hinge) writes every
// element block to a contribution buffer and one thread per BSR block sums
// them in the same order.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "elements.cuh"
#include "internal.h"

namespace eolc {

namespace {

// Element pass, triangles: d_B h^2 K_e block (la, lb) of face t at
// Kt[((t * 3 + la) * 3 + lb) * 9 ...] (fillxxMI, Forces.cpp:103-125), and
// t8 = rho 2 A (ComputeInertial.cpp:33).  K_e is symmetric: the blocks with
// la <= lb are evaluated and (lb, la) gets the transpose.
template <typename T>
__global__ void __launch_bounds__(128)
tri_blocks_kernel(int n_tri, const int *__restrict__ tri, const double *__restrict__ x,
                  const double *__restrict__ X, MaterialD m,
                  const MaterialD *__restrict__ mats, const int *__restrict__ node_inst,
                  T *__restrict__ Kt, T *__restrict__ t8) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tri) return;
  const int a = __ldg(tri + 3 * t), b = __ldg(tri + 3 * t + 1), c = __ldg(tri + 3 * t + 2);
  if (mats) m = mats[node_inst[a]];  // batched: the element's instance
  const Tri<T> q = make_tri<T>(x, X, a, b, c);
  const T mu = T(m.mu), lam = T(m.lam), dh2 = T(m.dh2);
  T *out = Kt + size_t(t) * 81;
#pragma unroll 1
  for (int la = 0; la < 3; ++la)
#pragma unroll 1
    for (int lb = la; lb < 3; ++lb) {
      T blk[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) blk[k] = T(0);
      add_membrane_block<T, T>(q, la, lb, mu, lam, dh2, blk);
#pragma unroll
      for (int k = 0; k < 9; ++k) out[(3 * la + lb) * 9 + k] = blk[k];
      if (lb != la)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) out[(3 * lb + la) * 9 + 3 * c + r] = blk[3 * r + c];
    }
  t8[t] = T(m.rho) * T(2) * q.A;
}

// Element pass, hinges: d_B h^2 K_b block (la, lb) of hinge e at
// Kh[((e * 4 + la) * 4 + lb) * 9 ...] (fillxxB, Forces.cpp:522-539, 885-908).
// K_b is a Hessian: the blocks with la <= lb are evaluated and (lb, la) gets
// the transpose.
template <typename T>
__global__ void __launch_bounds__(128)
hinge_blocks_kernel(int n_hinge, const int *__restrict__ hinge, const double *__restrict__ x,
                    const double *__restrict__ X, MaterialD m,
                    const MaterialD *__restrict__ mats, const int *__restrict__ node_inst,
                    T *__restrict__ Kh) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_hinge) return;
  const int *hv = hinge + 4 * e;
  const int v0 = __ldg(hv), v1 = __ldg(hv + 1), v2 = __ldg(hv + 2), v3n = __ldg(hv + 3);
  if (mats) m = mats[node_inst[v0]];
  const Hinge<T> H = make_hinge<T>(x, X, v0, v1, v2, v3n, T(m.beta));
  const T dh2 = T(m.dh2);
  T *out = Kh + size_t(e) * 144;
#pragma unroll 1
  for (int la = 0; la < 4; ++la)
#pragma unroll 1
    for (int lb = la; lb < 4; ++lb) {
      T blk[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) blk[k] = T(0);
      add_bending_block<T, T>(H, la, lb, dh2, blk);
#pragma unroll
      for (int k = 0; k < 9; ++k) out[(4 * la + lb) * 9 + k] = blk[k];
      if (lb != la)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) out[(4 * lb + la) * 9 + 3 * c + r] = blk[3 * r + c];
    }
}

// Deformation gradient of a face (UtilEOL.cpp:13-28, deform_grad): Dx times
// the inverse of DX, vertices (i0, i1, i2).
__device__ __forceinline__ void face_grad(const double *__restrict__ x,
                                          const double *__restrict__ X, int i0, int i1, int i2,
                                          double F[3][2]) {
  double DX00 = X[2 * i1] - X[2 * i0], DX01 = X[2 * i2] - X[2 * i0];
  double DX10 = X[2 * i1 + 1] - X[2 * i0 + 1], DX11 = X[2 * i2 + 1] - X[2 * i0 + 1];
  const double id = 1.0 / (DX00 * DX11 - DX10 * DX01);
  const double inv[2][2] = {{DX11 * id, -DX01 * id}, {-DX10 * id, DX00 * id}};
  for (int r = 0; r < 3; ++r) {
    const double d0 = x[3 * i1 + r] - x[3 * i0 + r], d1 = x[3 * i2 + r] - x[3 * i0 + r];
    F[r][0] = d0 * inv[0][0] + d1 * inv[1][0];
    F[r][1] = d0 * inv[0][1] + d1 * inv[1][1];
  }
}

// The F that an element's EOL vertices use: the face's, or for a hinge the
// mean of its two faces' (Forces.cpp:590-596).
__device__ __forceinline__ void element_grad(bool hinge, int e, const int *__restrict__ tri,
                                             const int *__restrict__ hin,
                                             const double *__restrict__ x,
                                             const double *__restrict__ X, double F[3][2]) {
  if (!hinge) {
    face_grad(x, X, tri[3 * e], tri[3 * e + 1], tri[3 * e + 2], F);
    return;
  }
  const int *v = hin + 4 * e;
  double F1[3][2], F2[3][2];
  face_grad(x, X, v[0], v[1], v[2], F1);
  face_grad(x, X, v[0], v[1], v[3], F2);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) F[r][c] = (F1[r][c] + F2[r][c]) / 2;
}

// out = R' B C with R = -F on an Eulerian row (else I) and C = -F on an
// Eulerian column: -F'B, -BF or F'BF (fillEOLInertia / fillEOLMembrane /
// fillEOLBending, Forces.cpp:177-329, 580-683); padded rows / columns 0.
template <typename T>
__device__ __forceinline__ void eol_transform(const T B[9], bool vr, bool vc, const double F[3][2],
                                              T out[9]) {
  double L[3][3];  // B C
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      if (!vc) {
        L[r][c] = double(B[3 * r + c]);
      } else if (c < 2) {
        L[r][c] = -(double(B[3 * r]) * F[0][c] + double(B[3 * r + 1]) * F[1][c] +
                    double(B[3 * r + 2]) * F[2][c]);
      } else {
        L[r][c] = 0.0;
      }
    }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double v;
      if (!vr) v = L[r][c];
      else if (r < 2) v = -(F[0][r] * L[0][c] + F[1][r] * L[1][c] + F[2][r] * L[2][c]);
      else v = 0.0;
      out[3 * r + c] = T(v);
    }
}

// Block gather: each BSR block sums its element contributions (cptr/contrib)
// in the reference's insertion order: per face, MDK += d_B h^2 K_e then the
// mass M_e (t8/12 on the diagonal, t8/24 off it, times I); per hinge,
// MDK += d_B h^2 K_b.  A contribution to an Eulerian row or column (EOL)
// is the same element block transformed by the element's F (eol_transform).
// n_real < n_nodes: the padded third DOF of each Eulerian node gets 1 on the
// MDK diagonal (the solves pin it).
template <typename T>
__global__ void __launch_bounds__(128)
gather_blocks_kernel(int n_blocks, const int *__restrict__ cptr, const int *__restrict__ contrib,
                     const T *__restrict__ Kt, const T *__restrict__ t8,
                     const T *__restrict__ Kh, double *__restrict__ A64,
                     float *__restrict__ A32, double *__restrict__ Mblk,
                     int n_real, int n_nodes, const int *__restrict__ blk_row,
                     const int *__restrict__ colidx, const int *__restrict__ tri,
                     const int *__restrict__ hin, const double *__restrict__ x,
                     const double *__restrict__ X) {
  const int bidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (bidx >= n_blocks) return;
  T acc[9], macc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { acc[k] = T(0); macc[k] = T(0); }
  const int c0 = cptr[bidx], c1 = cptr[bidx + 1];
  for (int q = c0; q < c1; ++q) {
    const int code = __ldg(contrib + q);
    const int lb = code & 3, la = (code >> 3) & 3, e = code >> 7;
    const bool hinge = (code & kHingeBit) != 0;
    const bool vr = (code >> 3) & kVirtual, vc = code & kVirtual;
    const T *blk = hinge ? Kh + size_t(e) * 144 + (4 * la + lb) * 9
                         : Kt + size_t(e) * 81 + (3 * la + lb) * 9;
    T mm = T(0);
    if (!hinge) {
      const T te = __ldg(t8 + e);
      mm = la == lb ? te / T(12) : te / T(24);
    }
    if (!vr && !vc) {
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] += __ldg(blk + k);
      if (!hinge) {
        acc[0] += mm; acc[4] += mm; acc[8] += mm;
        macc[0] += mm; macc[4] += mm; macc[8] += mm;
      }
      continue;
    }
    double F[3][2];
    element_grad(hinge, e, tri, hin, x, X, F);
    T B[9], Bt[9];
    for (int k = 0; k < 9; ++k) B[k] = __ldg(blk + k);
    eol_transform(B, vr, vc, F, Bt);
    for (int k = 0; k < 9; ++k) acc[k] += Bt[k];
    if (!hinge) {
      T Mm[9] = {mm, T(0), T(0), T(0), mm, T(0), T(0), T(0), mm};
      eol_transform(Mm, vr, vc, F, Bt);
      for (int k = 0; k < 9; ++k) {
        acc[k] += Bt[k];
        macc[k] += Bt[k];
      }
    }
  }
  if (n_real < n_nodes && blk_row[bidx] >= n_real && colidx[bidx] == blk_row[bidx])
    acc[8] += T(1);  // padded DOF of an Eulerian node
  if (A64) {
#pragma unroll
    for (int k = 0; k < 9; ++k) A64[size_t(bidx) * 9 + k] = double(acc[k]);
  }
  if (A32) {
#pragma unroll
    for (int k = 0; k < 9; ++k) A32[size_t(bidx) * 9 + k] = float(acc[k]);
  }
  if (Mblk) {
#pragma unroll
    for (int k = 0; k < 9; ++k) Mblk[size_t(bidx) * 9 + k] = double(macc[k]);
  }
}

// ---- shared-memory tiled assembly ---------------------------------------------
constexpr int kTileThreads = 256;
constexpr int kTileBytes = 112640;  // two CTAs per SM
// slots (3x3 blocks + a mass word) of one tile
template <typename T>
__host__ __device__ constexpr int tile_slots() {
  // slots of 9 values + a mass word, and 4 bytes per slot for the staged
  // gather lists (a 16-bit slot per contribution — one per slot — and a
  // 16-bit contribution offset per block — at most one block per slot)
  return (kTileBytes - 16) / (10 * int(sizeof(T)) + 4);
}
template <typename T>
__host__ __device__ constexpr size_t tile_smem_bytes() {
  return size_t(tile_slots<T>()) * (10 * sizeof(T) + 4) + 16;
}

// Row blocks (la, 0..n-1) of element e into shared memory at base: a block
// (la, lb) with la <= lb is evaluated, (la, lb) with la > lb is the
// transpose of the evaluated (lb, la).
template <typename T>
__device__ __forceinline__ void store_block(T *sk, int slot, const T blk[9], bool transpose) {
  T *o = sk + size_t(slot) * 9;
  if (!transpose) {
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = blk[k];
  } else {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) o[3 * c + r] = blk[3 * r + c];
  }
}

// Per-step inputs of the tiled kernel, one launch (prep_kernel), written to
// the assembly scratch:
//   xhl   FP32 path: every node's position split into float hi / lo words,
//         (hi.xyz, lo.xyz) as two float4, so that an edge vector is
//         (hi_b - hi_a) + (lo_b - lo_a) in FP32 — the FP64 difference to FP32
//         precision without FP64 arithmetic in the element loop;
//   fgeo  per triangle the material-space part (signed area, shape-function
//         gradients; 8 words), hgeo per hinge 3 |X1 - X0|^2 / cross2(...) —
//         X only, in the element's precision.
template <typename T>
__global__ void prep_kernel(int n_nodes, int n_tri, int n_hinge, const double *__restrict__ x,
                            const double *__restrict__ X, const int *__restrict__ tri,
                            const int *__restrict__ hinge, float4 *__restrict__ xhl,
                            T *__restrict__ fgeo, T *__restrict__ hgeo) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (xhl && k < n_nodes) {
    float h[3], l[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double v = x[3 * size_t(k) + c];
      h[c] = __double2float_rn(v);
      l[c] = __double2float_rn(v - double(h[c]));
    }
    xhl[2 * size_t(k)] = make_float4(h[0], h[1], h[2], 0.f);
    xhl[2 * size_t(k) + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
  if (k < n_tri) {
    const TriGeo<T> g = make_tri_geo<T>(X, tri[3 * k], tri[3 * k + 1], tri[3 * k + 2]);
    T *o = fgeo + 8 * size_t(k);
    o[0] = g.A;
    o[1] = g.g[0][0]; o[2] = g.g[0][1];
    o[3] = g.g[1][0]; o[4] = g.g[1][1];
    o[5] = g.g[2][0]; o[6] = g.g[2][1];
    o[7] = T(0);
  }
  if (k < n_hinge) {
    const int *v = hinge + 4 * k;
    hgeo[k] = hinge_geo<T>(X, v[0], v[1], v[2], v[3]);
  }
}

// x_i - x_j in the element's precision: from the hi / lo split (FP32) or
// the FP64 positions.
struct PosHL {
  const float4 *hl;
  __device__ __forceinline__ void load(int i, float4 &h, float4 &l) const {
    h = __ldg(hl + 2 * size_t(i));
    l = __ldg(hl + 2 * size_t(i) + 1);
  }
};
__device__ __forceinline__ v3<float> hl_diff(const float4 &hi, const float4 &li, const float4 &hj,
                                             const float4 &lj) {
  return mk3<float>((hi.x - hj.x) + (li.x - lj.x), (hi.y - hj.y) + (li.y - lj.y),
                    (hi.z - hj.z) + (li.z - lj.z));
}

// The row blocks (LA, 0..2) of a triangle / (LA, 0..3) of a hinge into
// shared memory, block LB at slot base + LB stride (consecutive tasks in
// consecutive slots: a 9-word stride between the threads of a warp, free of
// bank conflicts).  LA is a compile-time row (one instance per
// local vertex), so the vertex selections of the block formulas fold to
// constants; a block (LA, LB) with LA > LB is the transpose of the evaluated
// (LB, LA).
template <typename T, int LA>
__device__ __forceinline__ void face_row(const Tri<T> &q, T mu, T lam, T dh2, T t8, T *sk,
                                         T *smass, int base, int stride) {
#pragma unroll
  for (int lb = 0; lb < 3; ++lb) {
    T blk[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) blk[j] = T(0);
    add_membrane_block<T, T>(q, LA < lb ? LA : lb, LA < lb ? lb : LA, mu, lam, dh2, blk);
    store_block(sk, base + lb * stride, blk, LA > lb);
    smass[base + lb * stride] = LA == lb ? t8 / T(12) : t8 / T(24);
  }
}
// Hinge blocks by the grouped form of the bending Hessian (bend_block: eight
// outer products per block on per-vertex vectors the compiler computes once
// per task).
template <typename T, int LA, int LB>
__device__ __forceinline__ void hinge_pair(const Hinge<T> &H, T dh2, T *sk, int slot) {
  constexpr int V = LA < LB ? LA : LB, W = LA < LB ? LB : LA;
  T blk[9];
  bend_block<T, V, W>(H, bend_left<T, V>(H), bend_right<T, W>(H), dh2, blk);
  store_block(sk, slot, blk, LA > LB);
}
template <typename T, int LA>
__device__ __forceinline__ void hinge_row(const Hinge<T> &H, T dh2, T *sk, int base, int stride) {
  hinge_pair<T, LA, 0>(H, dh2, sk, base);
  hinge_pair<T, LA, 1>(H, dh2, sk, base + stride);
  hinge_pair<T, LA, 2>(H, dh2, sk, base + 2 * stride);
  hinge_pair<T, LA, 3>(H, dh2, sk, base + 3 * stride);
}

// FP32: two CTAs per SM (128 registers); FP64: one, without spills
template <typename T, bool WANT_M>
__global__ void __launch_bounds__(kTileThreads, sizeof(T) == 4 ? 2 : 1)
tile_blocks_kernel(const int *__restrict__ tile_row, const int *__restrict__ rowptr,
                   const int *__restrict__ cptr, const unsigned short *__restrict__ aslot,
                   const int *__restrict__ nf_ptr, const int *__restrict__ task_f,
                   const int *__restrict__ nh_ptr, const int *__restrict__ task_h,
                   const int *__restrict__ tri, const int *__restrict__ hinge,
                   const double *__restrict__ x, const float4 *__restrict__ xhl,
                   const T *__restrict__ fgeo, const T *__restrict__ hgeo, MaterialD m0,
                   const MaterialD *__restrict__ mats, const int *__restrict__ node_inst,
                   double *__restrict__ A64, float *__restrict__ A32,
                   double *__restrict__ Mblk) {
  extern __shared__ __align__(16) unsigned char tsm[];
  constexpr int kSlots = tile_slots<T>();
  constexpr bool kHL = sizeof(T) == 4;  // FP32: positions from the hi / lo split
  T *sk = reinterpret_cast<T *>(tsm);  // kSlots x 9
  T *smass = sk + size_t(kSlots) * 9;  // kSlots
  // the tile's gather lists, staged with one coalesced sweep: the slot of
  // every contribution and every block's first contribution, tile-relative
  unsigned short *s_slot = reinterpret_cast<unsigned short *>(smass + kSlots);
  unsigned short *s_cptr = s_slot + kSlots;  // kSlots + 1 entries
  const PosHL P{xhl};
  const int r0 = tile_row[blockIdx.x], r1 = tile_row[blockIdx.x + 1];
  const int b0 = rowptr[r0], nb = rowptr[r1] - b0;
  const int cb = __ldg(cptr + b0), nc = __ldg(cptr + b0 + nb) - cb;
  for (int q = threadIdx.x; q < nc; q += kTileThreads) s_slot[q] = __ldg(aslot + cb + q);
  for (int q = threadIdx.x; q <= nb; q += kTileThreads)
    s_cptr[q] = (unsigned short)(__ldg(cptr + b0 + q) - cb);
  const int fa = nf_ptr[r0], nf = nf_ptr[r1] - fa;
  const int ha = nh_ptr[r0], nh = nh_ptr[r1] - ha;
  // triangle task k: slots k + lb nf; hinge task k: 3 nf + k + lb nh
  for (int k = threadIdx.x; k < nf; k += kTileThreads) {
    const int code = __ldg(task_f + fa + k);
    const int e = code >> 2, la = code & 3;
    const int a = __ldg(tri + 3 * e), b = __ldg(tri + 3 * e + 1), c = __ldg(tri + 3 * e + 2);
    MaterialD m = m0;
    if (mats) m = mats[node_inst[a]];  // batched: the element's instance
    TriGeo<T> geo;
    const T *gp = fgeo + 8 * size_t(e);
    geo.A = gp[0];
    geo.g[0][0] = gp[1]; geo.g[0][1] = gp[2];
    geo.g[1][0] = gp[3]; geo.g[1][1] = gp[4];
    geo.g[2][0] = gp[5]; geo.g[2][1] = gp[6];
    v3<T> e0, e1;
    if constexpr (kHL) {
      float4 ha4, la4, hb4, lb4, hc4, lc4;
      P.load(a, ha4, la4); P.load(b, hb4, lb4); P.load(c, hc4, lc4);
      e0 = hl_diff(hb4, lb4, ha4, la4);
      e1 = hl_diff(hc4, lc4, ha4, la4);
    } else {
      e0 = dpos<T>(x, b, a);
      e1 = dpos<T>(x, c, a);
    }
    const Tri<T> q = make_tri_from<T>(e0, e1, geo);
    const T mu = T(m.mu), lam = T(m.lam), dh2 = T(m.dh2);
    const T t8 = T(m.rho) * T(2) * q.A;
    switch (la) {
      case 0: face_row<T, 0>(q, mu, lam, dh2, t8, sk, smass, k, nf); break;
      case 1: face_row<T, 1>(q, mu, lam, dh2, t8, sk, smass, k, nf); break;
      default: face_row<T, 2>(q, mu, lam, dh2, t8, sk, smass, k, nf); break;
    }
  }
  for (int k = threadIdx.x; k < nh; k += kTileThreads) {
    const int code = __ldg(task_h + ha + k);
    const int e = code >> 2, la = code & 3;
    const int *hv = hinge + 4 * e;
    const int v0 = __ldg(hv), v1 = __ldg(hv + 1), v2 = __ldg(hv + 2), v3n = __ldg(hv + 3);
    MaterialD m = m0;
    if (mats) m = mats[node_inst[v0]];
    v3<T> pp, qv, qq;
    if constexpr (kHL) {
      float4 h0, l0, h1, l1, h2, l2, h3, l3;
      P.load(v0, h0, l0); P.load(v1, h1, l1); P.load(v2, h2, l2); P.load(v3n, h3, l3);
      pp = hl_diff(h1, l1, h0, l0);
      qv = hl_diff(h2, l2, h0, l0);
      qq = hl_diff(h3, l3, h1, l1);
    } else {
      pp = dpos<T>(x, v1, v0);
      qv = dpos<T>(x, v2, v0);
      qq = dpos<T>(x, v3n, v1);
    }
    const Hinge<T> H = make_hinge_from<T>(pp, qv, qq, hgeo[e] * T(m.beta));
    const T dh2 = T(m.dh2);
    const int base = 3 * nf + k;
    switch (la) {
      case 0: hinge_row<T, 0>(H, dh2, sk, base, nh); break;
      case 1: hinge_row<T, 1>(H, dh2, sk, base, nh); break;
      case 2: hinge_row<T, 2>(H, dh2, sk, base, nh); break;
      default: hinge_row<T, 3>(H, dh2, sk, base, nh); break;
    }
  }
  __syncthreads();
  // one thread per (block, entry) of the tile: the contributions in insertion
  // order; consecutive threads write consecutive words
  const int nv = nb * 9;
  for (int idx = threadIdx.x; idx < nv; idx += kTileThreads) {
    const int bt = idx / 9, j = idx - bt * 9;
    const bool on_diag = j == 0 || j == 4 || j == 8;
    T acc = T(0), macc = T(0);
    const int c0 = s_cptr[bt], c1 = s_cptr[bt + 1];
    for (int q = c0; q < c1; ++q) {
      const unsigned sl = s_slot[q];
      const unsigned sidx = sl & 0x7fffu;
      acc += sk[size_t(sidx) * 9 + j];
      if ((sl & 0x8000u) && on_diag) {  // a triangle's mass term
        const T mm = smass[sidx];
        acc += mm;
        if (WANT_M) macc += mm;
      }
    }
    const size_t o = size_t(b0) * 9 + idx;
    if (A64) A64[o] = double(acc);
    if (A32) A32[o] = float(acc);
    if (WANT_M) Mblk[o] = double(macc);
  }
}

// Slot of every contribution: thread per block b (row i); the contribution
// (element e, local row la, local column lb) lands in block lb of the task
// (e, la) of row i: its entry p in i's triangle or hinge list has position
// k = pos[p] in the tile's task order, slot k + lb nf for a triangle, 3 nf +
// k + lb nh for a hinge (nf, nh: the tile's task counts).
__global__ void tile_slots_kernel(int n_blocks, const int *__restrict__ blk_row,
                                  const int *__restrict__ cptr, const int *__restrict__ contrib,
                                  const int *__restrict__ row_tile, const int *__restrict__ tile_row,
                                  const int *__restrict__ nf_ptr, const int *__restrict__ nf_list,
                                  const int *__restrict__ nh_ptr, const int *__restrict__ nh_list,
                                  const int *__restrict__ pos_f, const int *__restrict__ pos_h,
                                  unsigned short *__restrict__ aslot, int *__restrict__ err) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_blocks) return;
  const int i = blk_row[b], t = row_tile[i], r0 = tile_row[t], r1 = tile_row[t + 1];
  const int nft = nf_ptr[r1] - nf_ptr[r0], nht = nh_ptr[r1] - nh_ptr[r0];
  for (int q = cptr[b]; q < cptr[b + 1]; ++q) {
    const int code = contrib[q];
    const int e = code >> 7, la = (code >> 3) & 3, lb = code & 3;
    const bool h = (code & kHingeBit) != 0;
    const int want = (e << 2) | la;
    const int *lst = h ? nh_list : nf_list;
    const int p0 = h ? nh_ptr[i] : nf_ptr[i], p1 = h ? nh_ptr[i + 1] : nf_ptr[i + 1];
    int p = p0;
    while (p < p1 && lst[p] != want) ++p;
    if (p == p1) { atomicOr(err, 1); continue; }
    const int slot = h ? 3 * nft + pos_h[p] + lb * nht : pos_f[p] + lb * nft;
    aslot[q] = (unsigned short)(slot | (h ? 0 : 0x8000));
  }
}

// Forces, FP64 in every precision mode (the FP64 refinement residual of the
// mixed solve is only as accurate as b; near rest FP32 membrane forces are
// rounding noise as large as the gravity loads).  Two passes, so that each
// triangle is evaluated once:
//   tri_forces_kernel    per triangle: the membrane force on each of its
//                        vertices and t8 = rho 2 A, at Ft[10 t ...];
//   forces_rhs_kernel    per node: f_i = sum over incident faces of membrane
//                        + gravity forces in face order (faceBasedF non-EOL,
//                        Forces.cpp:498-501; bending adds no force there,
//                        Forces.cpp:885-908), then b_i = -((M v)_i + h f_i)
//                        (Cloth.cpp:345).
// Per-triangle words of the force pass: the membrane force on each vertex
// (9), t8, and the terms every incident node would otherwise divide out
// again (FP64 division is a long software sequence on this GPU's FP64 pipe):
// the gravity force t8 g / 6 (3) and the mass entries t8 / 12, t8 / 24 —
// the same expressions, evaluated once per triangle instead of once per
// (node, triangle) pair.
constexpr int kForceWords = 16;
constexpr int kFwT8 = 9, kFwGrav = 10, kFwMdiag = 13, kFwMoff = 14;

__global__ void __launch_bounds__(128)
tri_forces_kernel(int n_tri, const int *__restrict__ tri, const double *__restrict__ x,
                  const double *__restrict__ X, MaterialD m,
                  const MaterialD *__restrict__ mats, const int *__restrict__ node_inst,
                  double *__restrict__ Ft) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tri) return;
  const int a = __ldg(tri + 3 * t), b = __ldg(tri + 3 * t + 1), c = __ldg(tri + 3 * t + 2);
  if (mats) m = mats[node_inst[a]];  // batched: the element's instance
  const Tri<double> q = make_tri<double>(x, X, a, b, c);
  double *out = Ft + size_t(t) * kForceWords;
#pragma unroll
  for (int la = 0; la < 3; ++la) {
    const v3<double> fm = membrane_force(q, la, m.mu, m.lam);
    out[3 * la] = fm.x;
    out[3 * la + 1] = fm.y;
    out[3 * la + 2] = fm.z;
  }
  const double t8 = m.rho * 2.0 * q.A;
  out[kFwT8] = t8;
  out[kFwGrav] = t8 * m.g[0] / 6.0;
  out[kFwGrav + 1] = t8 * m.g[1] / 6.0;
  out[kFwGrav + 2] = t8 * m.g[2] / 6.0;
  out[kFwMdiag] = t8 / 12.0;
  out[kFwMoff] = t8 / 24.0;
  out[15] = 0.0;
}

__global__ void __launch_bounds__(128)
forces_rhs_kernel(int n_nodes, const int *__restrict__ nf_ptr,
                  const int *__restrict__ nf_list, const int *__restrict__ tri,
                  const double *__restrict__ Ft, const double *__restrict__ v, MaterialD m,
                  const MaterialD *__restrict__ mats, const int *__restrict__ node_inst,
                  double *__restrict__ f, double *__restrict__ b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  if (mats) m = mats[node_inst[i]];  // batched: the node's instance
  double fx = 0, fy = 0, fz = 0;
  double mvx = 0, mvy = 0, mvz = 0;
  for (int q = nf_ptr[i]; q < nf_ptr[i + 1]; ++q) {
    const int code = __ldg(nf_list + q);
    const int e = code >> 2, la = code & 3;
    const double *fe = Ft + size_t(e) * kForceWords;
    fx += __ldg(fe + 3 * la) + __ldg(fe + kFwGrav);
    fy += __ldg(fe + 3 * la + 1) + __ldg(fe + kFwGrav + 1);
    fz += __ldg(fe + 3 * la + 2) + __ldg(fe + kFwGrav + 2);
    if (b) {
      const double mdiag = __ldg(fe + kFwMdiag), moff = __ldg(fe + kFwMoff);
#pragma unroll
      for (int w = 0; w < 3; ++w) {
        const int vw = __ldg(tri + 3 * e + w);
        const double mm = w == la ? mdiag : moff;
        mvx += mm * v[3 * vw];
        mvy += mm * v[3 * vw + 1];
        mvz += mm * v[3 * vw + 2];
      }
    }
  }
  if (f) {
    f[3 * i] = fx; f[3 * i + 1] = fy; f[3 * i + 2] = fz;
  }
  if (b) {
    b[3 * i] = -(mvx + m.h * fx);
    b[3 * i + 1] = -(mvy + m.h * fy);
    b[3 * i + 2] = -(mvz + m.h * fz);
  }
}

}  // namespace

constexpr size_t al256(size_t b) { return (b + 255) / 256 * 256; }

// Scratch of the tiled path (prep_kernel's outputs): xhl (FP32 path), fgeo,
// hgeo, each 256-byte aligned.
size_t tiled_prep_bytes(const DevTopology &T, int prec) {
  const size_t e = prec == EOLC_PREC_FP64 ? sizeof(double) : sizeof(float);
  const size_t xhl = prec == EOLC_PREC_FP64 ? 0 : al256(size_t(T.n_nodes) * 2 * sizeof(float4));
  return xhl + al256(size_t(T.n_tri) * 8 * e) + al256(size_t(std::max(1, T.n_hinge)) * e);
}

template <typename E>
void launch_tiled(const DevTopology &T, int w, const double *x, const double *X,
                  const MaterialD &m, const MaterialD *mats, const int *node_inst, void *elem,
                  double *A64, float *A32, double *Mblk, cudaStream_t s) {
  char *sp = static_cast<char *>(elem);
  float4 *xhl = nullptr;
  if (sizeof(E) == 4) {
    xhl = reinterpret_cast<float4 *>(sp);
    sp += al256(size_t(T.n_nodes) * 2 * sizeof(float4));
  }
  E *fgeo = reinterpret_cast<E *>(sp);
  sp += al256(size_t(T.n_tri) * 8 * sizeof(E));
  E *hgeo = reinterpret_cast<E *>(sp);
  const int np = std::max(T.n_nodes, std::max(T.n_tri, T.n_hinge));
  prep_kernel<E><<<(np + 255) / 256, 256, 0, s>>>(T.n_nodes, T.n_tri, T.n_hinge, x, X, T.tri.p,
                                                  T.hinge.p, xhl, fgeo, hgeo);
  const size_t smem = tile_smem_bytes<E>();
  if (Mblk) {
    tile_blocks_kernel<E, true><<<T.atiles[w], kTileThreads, smem, s>>>(
        T.atile_row[w].p, T.rowptr.p, T.cptr.p, T.aslot[w].p, T.nf_ptr.p, T.atask_f[w].p,
        T.nh_ptr.p, T.atask_h[w].p, T.tri.p, T.hinge.p, x, xhl, fgeo, hgeo, m, mats, node_inst,
        A64, A32, Mblk);
  } else {
    tile_blocks_kernel<E, false><<<T.atiles[w], kTileThreads, smem, s>>>(
        T.atile_row[w].p, T.rowptr.p, T.cptr.p, T.aslot[w].p, T.nf_ptr.p, T.atask_f[w].p,
        T.nh_ptr.p, T.atask_h[w].p, T.tri.p, T.hinge.p, x, xhl, fgeo, hgeo, m, mats, node_inst,
        A64, A32, nullptr);
  }
}

std::string ensure_assembly_tiles(DevTopology &T, int prec, cudaStream_t s, long long &launches) {
  const int w = prec == EOLC_PREC_FP64 ? 1 : 0;
  if (T.n_eol > 0 || T.atiles[w] >= 0) return "";
  const int N = T.n_nodes;
  const int cap = w ? tile_slots<double>() : tile_slots<float>();
#define AT(expr)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (expr);                                                        \
    if (e_ != cudaSuccess) return std::string(#expr ": ") + cudaGetErrorString(e_); \
  } while (0)
  std::vector<int> nf(N + 1), nh(N + 1);
  AT(cudaMemcpyAsync(nf.data(), T.nf_ptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, s));
  AT(cudaMemcpyAsync(nh.data(), T.nh_ptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, s));
  AT(cudaStreamSynchronize(s));
  // greedy: grow each tile row by row while its slots fit
  std::vector<int> tile_row(1, 0), row_tile(N);
  int start = 0;
  while (start < N) {
    int end = start;
    while (end < N) {
      const long long slots = 3ll * (nf[end + 1] - nf[start]) + 4ll * (nh[end + 1] - nh[start]);
      if (slots > cap) break;
      ++end;
    }
    if (end == start) {  // one row's blocks exceed a tile: the two-pass path
      T.atiles[w] = 0;
      return "";
    }
    for (int i = start; i < end; ++i) row_tile[i] = int(tile_row.size()) - 1;
    tile_row.push_back(end);
    start = end;
  }
  // every tile's tasks reordered by local vertex (stable), and each list
  // entry's position in its tile's order
  const size_t nfl = size_t(nf[N]), nhl = size_t(nh[N]);
  std::vector<int> fl(std::max<size_t>(nfl, 1)), hl(std::max<size_t>(nhl, 1));
  AT(cudaMemcpyAsync(fl.data(), T.nf_list.p, sizeof(int) * nfl, cudaMemcpyDeviceToHost, s));
  if (nhl > 0)
    AT(cudaMemcpyAsync(hl.data(), T.nh_list.p, sizeof(int) * nhl, cudaMemcpyDeviceToHost, s));
  AT(cudaStreamSynchronize(s));
  std::vector<int> tf(fl.size()), th(hl.size()), pf(fl.size()), ph(hl.size());
  auto reorder = [](const std::vector<int> &lst, int a, int b, int nv, std::vector<int> &task,
                    std::vector<int> &pos) {
    int k = 0;
    for (int v = 0; v < nv; ++v)
      for (int p = a; p < b; ++p)
        if ((lst[p] & 3) == v) {
          task[a + k] = lst[p];
          pos[p] = k++;
        }
  };
  for (size_t t = 0; t + 1 < tile_row.size(); ++t) {
    reorder(fl, nf[tile_row[t]], nf[tile_row[t + 1]], 3, tf, pf);
    reorder(hl, nh[tile_row[t]], nh[tile_row[t + 1]], 4, th, ph);
  }
  AT(T.atask_f[w].upload(tf.data(), tf.size(), s));
  AT(T.atask_h[w].upload(th.data(), th.size(), s));
  AT(T.apos_f[w].upload(pf.data(), pf.size(), s));
  AT(T.apos_h[w].upload(ph.data(), ph.size(), s));
  DevBuf<int> drt, derr;
  const size_t ncon = T.contrib.n;
  AT(T.atile_row[w].upload(tile_row.data(), tile_row.size(), s));
  AT(drt.upload(row_tile.data(), row_tile.size(), s));
  AT(T.aslot[w].resize(std::max<size_t>(ncon, 1)));
  AT(derr.resize(1));
  AT(cudaMemsetAsync(derr.p, 0, sizeof(int), s));
  tile_slots_kernel<<<(T.n_blocks + 127) / 128, 128, 0, s>>>(
      T.n_blocks, T.blk_row.p, T.cptr.p, T.contrib.p, drt.p, T.atile_row[w].p, T.nf_ptr.p,
      T.nf_list.p, T.nh_ptr.p, T.nh_list.p, T.apos_f[w].p, T.apos_h[w].p, T.aslot[w].p, derr.p);
  launches += 1;
  int err = 0;
  AT(cudaGetLastError());
  AT(cudaMemcpyAsync(&err, derr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  AT(cudaStreamSynchronize(s));
  if (err) return "assembly tiles: a contribution without its element task";
  // the kernels' shared-memory size, once per topology and device
  if (w) {
    AT(cudaFuncSetAttribute(tile_blocks_kernel<double, true>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                            int(tile_smem_bytes<double>())));
    AT(cudaFuncSetAttribute(tile_blocks_kernel<double, false>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                            int(tile_smem_bytes<double>())));
  } else {
    AT(cudaFuncSetAttribute(tile_blocks_kernel<float, true>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                            int(tile_smem_bytes<float>())));
    AT(cudaFuncSetAttribute(tile_blocks_kernel<float, false>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                            int(tile_smem_bytes<float>())));
  }
#undef AT
  T.atiles[w] = int(tile_row.size()) - 1;
  return "";
}

int launch_assemble_blocks(const DevTopology &T, const double *x,
                           const double *X, const MaterialD &m,
                           const MaterialD *mats, const int *node_inst,
                           int prec, void *elem, double *A64, float *A32, double *Mblk,
                           cudaStream_t s) {
  const int nb = T.n_blocks, nt = T.n_tri, nh = T.n_hinge;
  const int w = prec == EOLC_PREC_FP64 ? 1 : 0;
  if (T.n_eol == 0 && T.atiles[w] > 0) {
    if (w) launch_tiled<double>(T, w, x, X, m, mats, node_inst, elem, A64, A32, Mblk, s);
    else launch_tiled<float>(T, w, x, X, m, mats, node_inst, elem, A64, A32, Mblk, s);
    return 2;
  }
  if (prec == EOLC_PREC_FP64) {
    double *Kt = static_cast<double *>(elem), *t8 = Kt + size_t(nt) * 81, *Kh = t8 + nt;
    tri_blocks_kernel<double><<<(nt + 127) / 128, 128, 0, s>>>(nt, T.tri.p, x, X, m, mats,
                                                               node_inst, Kt, t8);
    if (nh > 0)
      hinge_blocks_kernel<double><<<(nh + 127) / 128, 128, 0, s>>>(nh, T.hinge.p, x, X, m, mats,
                                                                   node_inst, Kh);
    gather_blocks_kernel<double><<<(nb + 127) / 128, 128, 0, s>>>(
        nb, T.cptr.p, T.contrib.p, Kt, t8, Kh, A64, A32, Mblk, T.n_real, T.n_nodes,
        T.blk_row.p, T.colidx.p, T.tri.p, T.hinge.p, x, X);
  } else {
    float *Kt = static_cast<float *>(elem), *t8 = Kt + size_t(nt) * 81, *Kh = t8 + nt;
    tri_blocks_kernel<float><<<(nt + 127) / 128, 128, 0, s>>>(nt, T.tri.p, x, X, m, mats,
                                                              node_inst, Kt, t8);
    if (nh > 0)
      hinge_blocks_kernel<float><<<(nh + 127) / 128, 128, 0, s>>>(nh, T.hinge.p, x, X, m, mats,
                                                                  node_inst, Kh);
    gather_blocks_kernel<float><<<(nb + 127) / 128, 128, 0, s>>>(
        nb, T.cptr.p, T.contrib.p, Kt, t8, Kh, A64, A32, Mblk, T.n_real, T.n_nodes,
        T.blk_row.p, T.colidx.p, T.tri.p, T.hinge.p, x, X);
  }
  return nh > 0 ? 3 : 2;
}

// Bending force of hinge e on its local vertex a: c (a x s0_v + b x s1_v),
// the gradient of c (1 - n0^.n1^) (ComputeBending's f, oracle orc_bending).
__device__ __forceinline__ v3<double> bending_force(const int *__restrict__ hin, int e, int a,
                                                    const double *__restrict__ x,
                                                    const double *__restrict__ X, double beta) {
  const int *v = hin + 4 * e;
  const Hinge<double> Hg = make_hinge<double>(x, X, v[0], v[1], v[2], v[3], beta);
  const v3<double> g = cross(Hg.a, hinge_s0(Hg, a)) + cross(Hg.b, hinge_s1(Hg, a));
  return mk3<double>(Hg.c * g.x, Hg.c * g.y, Hg.c * g.z);
}

// EOL forces, after forces_rhs_kernel has summed the face forces of the
// mesh nodes (edgeBasedF follows faceBasedF, Forces.cpp:912-930):
//   node row i: + the bending force of every hinge of i that has an EOL
//     vertex (the EOL branch adds it, Forces.cpp:750-760; the other hinges
//     add none);
//   Eulerian row of EOL node v: sum over v's faces of (-F' fm_v) + (-F' fi_v)
//     (F the face's), then over v's hinges of -Fm' fb_v (Fm the mean of the
//     hinge's faces'); the padded third DOF is 0.
__global__ void __launch_bounds__(128)
eol_forces_kernel(int n_nodes, int n_real, const int *__restrict__ eol,
                  const int *__restrict__ eol_node, const int *__restrict__ nf_ptr,
                  const int *__restrict__ nf_list, const int *__restrict__ nh_ptr,
                  const int *__restrict__ nh_list, const int *__restrict__ tri,
                  const int *__restrict__ hin, const double *__restrict__ x,
                  const double *__restrict__ X, const double *__restrict__ Ft, MaterialD m,
                  double *__restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  if (i < n_real) {
    for (int q = nh_ptr[i]; q < nh_ptr[i + 1]; ++q) {
      const int e = nh_list[q] >> 2, a = nh_list[q] & 3;
      bool touches = false;
      for (int b = 0; b < 4; ++b) touches |= eol[hin[4 * e + b]] >= 0;
      if (!touches) continue;
      const v3<double> fb = bending_force(hin, e, a, x, X, m.beta);
      f[3 * i] += fb.x;
      f[3 * i + 1] += fb.y;
      f[3 * i + 2] += fb.z;
    }
    return;
  }
  const int v = eol_node[i - n_real];
  double fx[2] = {0.0, 0.0};
  for (int q = nf_ptr[v]; q < nf_ptr[v + 1]; ++q) {
    const int t = nf_list[q] >> 2, a = nf_list[q] & 3;
    double F[3][2];
    face_grad(x, X, tri[3 * t], tri[3 * t + 1], tri[3 * t + 2], F);
    const double *fe = Ft + size_t(t) * kForceWords;
    const double t8 = fe[kFwT8];
    for (int j = 0; j < 2; ++j) {
      double sm = 0, si = 0;
      for (int p = 0; p < 3; ++p) {
        sm += F[p][j] * fe[3 * a + p];
        si += F[p][j] * (t8 * m.g[p] / 6.0);
      }
      fx[j] += -sm + -si;
    }
  }
  for (int q = nh_ptr[v]; q < nh_ptr[v + 1]; ++q) {
    const int e = nh_list[q] >> 2, a = nh_list[q] & 3;
    double F[3][2];
    element_grad(true, e, tri, hin, x, X, F);
    const v3<double> fb = bending_force(hin, e, a, x, X, m.beta);
    for (int j = 0; j < 2; ++j) fx[j] += -(F[0][j] * fb.x + F[1][j] * fb.y + F[2][j] * fb.z);
  }
  f[3 * i] = fx[0];
  f[3 * i + 1] = fx[1];
  f[3 * i + 2] = 0.0;
}

// b = -(M v + h f) with the assembled FP64 M blocks (the EOL path, where M
// couples Eulerian DOFs; the product first, Cloth.cpp:345).
__global__ void __launch_bounds__(128)
bsr_rhs_kernel(int n_nodes, const int *__restrict__ rowptr, const int *__restrict__ colidx,
               const double *__restrict__ Mblk, const double *__restrict__ v,
               const double *__restrict__ f, double h, double *__restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  double mv[3] = {0.0, 0.0, 0.0};
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const double *B = Mblk + size_t(k) * 9;
    const int j = colidx[k];
    for (int r = 0; r < 3; ++r)
      mv[r] += B[3 * r] * v[3 * j] + B[3 * r + 1] * v[3 * j + 1] + B[3 * r + 2] * v[3 * j + 2];
  }
  for (int r = 0; r < 3; ++r) b[3 * i + r] = -(mv[r] + h * f[3 * i + r]);
}

// The force pass's per-triangle words follow the element blocks of the
// two-pass assembly, or the tiled path's per-step inputs, 256-byte aligned.
size_t forces_scratch_offset(const DevTopology &T, int prec) {
  const int w = prec == EOLC_PREC_FP64 ? 1 : 0;
  if (T.n_eol == 0 && T.atiles[w] > 0) return tiled_prep_bytes(T, prec);
  const size_t e = prec == EOLC_PREC_FP64 ? sizeof(double) : sizeof(float);
  return (e * (size_t(T.n_tri) * 82 + size_t(T.n_hinge) * 144) + 255) / 256 * 256;
}

size_t assemble_scratch_bytes(const DevTopology &T, int prec) {
  return forces_scratch_offset(T, prec) + sizeof(double) * kForceWords * size_t(T.n_tri);
}

void launch_forces_rhs(const DevTopology &T, const double *x, const double *X,
                       const double *v, const MaterialD &m,
                       const MaterialD *mats, const int *node_inst, int prec, void *elem,
                       double *f, double *b, cudaStream_t s) {
  const int n = T.n_real, nt = T.n_tri;
  double *Ft = reinterpret_cast<double *>(static_cast<char *>(elem) +
                                          forces_scratch_offset(T, prec));
  tri_forces_kernel<<<(nt + 127) / 128, 128, 0, s>>>(nt, T.tri.p, x, X, m, mats, node_inst, Ft);
  forces_rhs_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, T.nf_ptr.p, T.nf_list.p, T.tri.p, Ft, v,
                                                    m, mats, node_inst, f,
                                                    T.n_eol > 0 ? nullptr : b);
  if (T.n_eol > 0)
    eol_forces_kernel<<<(T.n_nodes + 127) / 128, 128, 0, s>>>(
        T.n_nodes, n, T.eol.p, T.eol_node.p, T.nf_ptr.p, T.nf_list.p, T.nh_ptr.p, T.nh_list.p,
        T.tri.p, T.hinge.p, x, X, Ft, m, f);
}

void launch_bsr_rhs(const DevTopology &T, const double *Mblk, const double *v, const double *f,
                    double h, double *b, cudaStream_t s) {
  bsr_rhs_kernel<<<(T.n_nodes + 127) / 128, 128, 0, s>>>(T.n_nodes, T.rowptr.p, T.colidx.p,
                                                         Mblk, v, f, h, b);
}

}  // namespace eolc
