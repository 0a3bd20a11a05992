// Assembly of MDK (and optionally M) into the fixed 3x3 BSR pattern, and of
// the force / right-hand side vectors.
//
// Replaces the triplet loops of faceBasedF / edgeBasedF and the two
// setFromTriplets calls (Forces.cpp:331-930) plus b = -(M v + h f)
// (Cloth.cpp:345).  Design: an element pass (one thread per triangle, one
// per hinge) evaluates each element once and writes its 3x3 blocks (9 per
// triangle: d_B h^2 K_e; 16 per hinge: d_B h^2 K_b) and the triangle's mass
// t8 to a contribution buffer; then one thread per BSR block sums the
// contributions that land in it in the reference's insertion order (faces
// ascending, then hinges ascending) and writes the block once.  No atomics:
// results are bit-reproducible run to run.
#include <cuda_runtime.h>

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
constexpr int kForceWords = 10;  // 3 x 3 vertex forces + t8

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
  out[9] = m.rho * 2.0 * q.A;
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
    const double t8 = __ldg(fe + 9);
    fx += __ldg(fe + 3 * la) + t8 * m.g[0] / 6.0;
    fy += __ldg(fe + 3 * la + 1) + t8 * m.g[1] / 6.0;
    fz += __ldg(fe + 3 * la + 2) + t8 * m.g[2] / 6.0;
    if (b) {
#pragma unroll
      for (int w = 0; w < 3; ++w) {
        const int vw = __ldg(tri + 3 * e + w);
        const double mm = w == la ? t8 / 12.0 : t8 / 24.0;
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

void launch_assemble_blocks(const DevTopology &T, const double *x,
                            const double *X, const MaterialD &m,
                            const MaterialD *mats, const int *node_inst,
                            int prec, void *elem, double *A64, float *A32, double *Mblk,
                            cudaStream_t s) {
  const int nb = T.n_blocks, nt = T.n_tri, nh = T.n_hinge;
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
    const double t8 = fe[9];
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

// The force pass's per-triangle words follow the element blocks, 256-byte
// aligned.
size_t forces_scratch_offset(const DevTopology &T, int prec) {
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
