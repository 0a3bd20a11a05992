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

// Block gather: MDK (and M) of every BSR block from the element blocks, in
// the reference's insertion order: per face, MDK += d_B h^2 K_e then the mass
// M_e (t8/12 on the diagonal, t8/24 off it, times I); per hinge,
// MDK += d_B h^2 K_b.
template <typename T>
__global__ void __launch_bounds__(128)
gather_blocks_kernel(int n_blocks, const int *__restrict__ cptr, const int *__restrict__ contrib,
                     const T *__restrict__ Kt, const T *__restrict__ t8,
                     const T *__restrict__ Kh, double *__restrict__ A64,
                     float *__restrict__ A32, double *__restrict__ Mblk) {
  const int bidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (bidx >= n_blocks) return;
  T acc[9], macc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { acc[k] = T(0); macc[k] = T(0); }
  const int c0 = cptr[bidx], c1 = cptr[bidx + 1];
  for (int q = c0; q < c1; ++q) {
    const int code = __ldg(contrib + q);
    const int lb = code & 3, la = (code >> 2) & 3, e = code >> 5;
    if (!(code & kHingeBit)) {
      const T *blk = Kt + size_t(e) * 81 + (3 * la + lb) * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] += __ldg(blk + k);
      const T te = __ldg(t8 + e);
      const T mm = la == lb ? te / T(12) : te / T(24);
      acc[0] += mm; acc[4] += mm; acc[8] += mm;
      macc[0] += mm; macc[4] += mm; macc[8] += mm;
    } else {
      const T *blk = Kh + size_t(e) * 144 + (4 * la + lb) * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] += __ldg(blk + k);
    }
  }
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
        nb, T.cptr.p, T.contrib.p, Kt, t8, Kh, A64, A32, Mblk);
  } else {
    float *Kt = static_cast<float *>(elem), *t8 = Kt + size_t(nt) * 81, *Kh = t8 + nt;
    tri_blocks_kernel<float><<<(nt + 127) / 128, 128, 0, s>>>(nt, T.tri.p, x, X, m, mats,
                                                              node_inst, Kt, t8);
    if (nh > 0)
      hinge_blocks_kernel<float><<<(nh + 127) / 128, 128, 0, s>>>(nh, T.hinge.p, x, X, m, mats,
                                                                  node_inst, Kh);
    gather_blocks_kernel<float><<<(nb + 127) / 128, 128, 0, s>>>(
        nb, T.cptr.p, T.contrib.p, Kt, t8, Kh, A64, A32, Mblk);
  }
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
  const int n = T.n_nodes, nt = T.n_tri;
  double *Ft = reinterpret_cast<double *>(static_cast<char *>(elem) +
                                          forces_scratch_offset(T, prec));
  tri_forces_kernel<<<(nt + 127) / 128, 128, 0, s>>>(nt, T.tri.p, x, X, m, mats, node_inst, Ft);
  forces_rhs_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, T.nf_ptr.p, T.nf_list.p, T.tri.p, Ft, v,
                                                    m, mats, node_inst, f, b);
}

}  // namespace eolc
