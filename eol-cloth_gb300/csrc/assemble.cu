// Assembly of MDK (and optionally M) into the fixed 3x3 BSR pattern, and of
// the force / right-hand side vectors.
//
// Replaces the triplet loops of faceBasedF / edgeBasedF and the two
// setFromTriplets calls (Forces.cpp:331-930) plus b = -(M v + h f)
// (Cloth.cpp:345).  Design: one thread per BSR block gathers the element
// terms that land in its block, in the reference's insertion order (faces
// ascending, then hinges ascending), and writes the block once.  No atomics,
// no staging buffer: results are bit-reproducible run to run and the only
// HBM writes are the BSR values themselves.
#include <cuda_runtime.h>

#include "elements.cuh"
#include "internal.h"

namespace eolc {

namespace {

template <typename T, typename Acc>
__global__ void __launch_bounds__(128)
assemble_blocks_kernel(int n_blocks, const int *__restrict__ cptr,
                       const int *__restrict__ contrib,
                       const int *__restrict__ tri,
                       const int *__restrict__ hinge,
                       const double *__restrict__ x,
                       const double *__restrict__ X, MaterialD m,
                       const MaterialD *__restrict__ mats,
                       const int *__restrict__ node_inst,
                       const int *__restrict__ blk_row,
                       double *__restrict__ A64, float *__restrict__ A32,
                       double *__restrict__ Mblk) {
  int bidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (bidx >= n_blocks) return;
  if (mats) m = mats[node_inst[blk_row[bidx]]];  // batched: the row's instance
  Acc acc[9], macc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { acc[k] = Acc(0); macc[k] = Acc(0); }
  const T mu = T(m.mu), lam = T(m.lam), dh2 = T(m.dh2), beta = T(m.beta);
  int c0 = cptr[bidx], c1 = cptr[bidx + 1];
  for (int q = c0; q < c1; ++q) {
    int code = __ldg(contrib + q);
    int lb = code & 3, la = (code >> 2) & 3, e = code >> 5;
    if (!(code & kHingeBit)) {
      int a = __ldg(tri + 3 * e), b = __ldg(tri + 3 * e + 1),
          c = __ldg(tri + 3 * e + 2);
      Tri<T> t = make_tri<T>(x, X, a, b, c);
      // MDK += M_e + dh2 K_e (fillxMI / fillxxMI, Forces.cpp:103-125)
      add_membrane_block<T, Acc>(t, la, lb, mu, lam, dh2, acc);
      T t8 = T(m.rho) * T(2) * t.A;
      T mm = la == lb ? t8 / T(12) : t8 / T(24);
      acc[0] += Acc(mm); acc[4] += Acc(mm); acc[8] += Acc(mm);
      macc[0] += Acc(mm); macc[4] += Acc(mm); macc[8] += Acc(mm);
    } else {
      const int *hv = hinge + 4 * e;
      Hinge<T> H = make_hinge<T>(x, X, __ldg(hv), __ldg(hv + 1), __ldg(hv + 2),
                                 __ldg(hv + 3), beta);
      // MDK += dh2 Kb (fillxB / fillxxB, Forces.cpp:522-539, 885-908)
      add_bending_block<T, Acc>(H, la, lb, dh2, acc);
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

// Per node: f_i = sum over incident faces of membrane + gravity forces
// (faceBasedF non-EOL, Forces.cpp:498-501; bending adds no force there,
// Forces.cpp:885-908), then b_i = -((M v)_i + h f_i) (Cloth.cpp:345).
template <typename T>
__global__ void __launch_bounds__(128)
forces_rhs_kernel(int n_nodes, const int *__restrict__ nf_ptr,
                  const int *__restrict__ nf_list, const int *__restrict__ tri,
                  const double *__restrict__ x, const double *__restrict__ X,
                  const double *__restrict__ v, MaterialD m,
                  const MaterialD *__restrict__ mats,
                  const int *__restrict__ node_inst,
                  double *__restrict__ f, double *__restrict__ b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  if (mats) m = mats[node_inst[i]];  // batched: the node's instance
  const T mu = T(m.mu), lam = T(m.lam);
  T fx = 0, fy = 0, fz = 0;
  double mvx = 0, mvy = 0, mvz = 0;
  for (int q = nf_ptr[i]; q < nf_ptr[i + 1]; ++q) {
    int code = __ldg(nf_list + q);
    int e = code >> 2, la = code & 3;
    int vv[3] = {__ldg(tri + 3 * e), __ldg(tri + 3 * e + 1), __ldg(tri + 3 * e + 2)};
    Tri<T> t = make_tri<T>(x, X, vv[0], vv[1], vv[2]);
    v3<T> fm = membrane_force(t, la, mu, lam);
    T t8 = T(m.rho) * T(2) * t.A;
    fx += fm.x + t8 * T(m.g[0]) / T(6);
    fy += fm.y + t8 * T(m.g[1]) / T(6);
    fz += fm.z + t8 * T(m.g[2]) / T(6);
    if (b) {
#pragma unroll
      for (int w = 0; w < 3; ++w) {
        double mm = double(w == la ? t8 / T(12) : t8 / T(24));
        mvx += mm * v[3 * vv[w]];
        mvy += mm * v[3 * vv[w] + 1];
        mvz += mm * v[3 * vv[w] + 2];
      }
    }
  }
  if (f) {
    f[3 * i] = double(fx); f[3 * i + 1] = double(fy); f[3 * i + 2] = double(fz);
  }
  if (b) {
    b[3 * i] = -(mvx + m.h * double(fx));
    b[3 * i + 1] = -(mvy + m.h * double(fy));
    b[3 * i + 2] = -(mvz + m.h * double(fz));
  }
}

}  // namespace

void launch_assemble_blocks(const DevTopology &T, const double *x,
                            const double *X, const MaterialD &m,
                            const MaterialD *mats, const int *node_inst,
                            int prec, double *A64, float *A32, double *Mblk,
                            cudaStream_t s) {
  int nb = T.n_blocks;
  dim3 block(128), grid((nb + 127) / 128);
  if (prec == EOLC_PREC_FP64)
    assemble_blocks_kernel<double, double><<<grid, block, 0, s>>>(
        nb, T.cptr.p, T.contrib.p, T.tri.p, T.hinge.p, x, X, m, mats, node_inst, T.blk_row.p,
        A64, A32, Mblk);
  else
    assemble_blocks_kernel<float, float><<<grid, block, 0, s>>>(
        nb, T.cptr.p, T.contrib.p, T.tri.p, T.hinge.p, x, X, m, mats, node_inst, T.blk_row.p,
        A64, A32, Mblk);
}

void launch_forces_rhs(const DevTopology &T, const double *x, const double *X,
                       const double *v, const MaterialD &m,
                       const MaterialD *mats, const int *node_inst, int prec,
                       double *f, double *b, cudaStream_t s) {
  int n = T.n_nodes;
  dim3 block(128), grid((n + 127) / 128);
  if (prec == EOLC_PREC_FP64)
    forces_rhs_kernel<double><<<grid, block, 0, s>>>(
        n, T.nf_ptr.p, T.nf_list.p, T.tri.p, x, X, v, m, mats, node_inst, f, b);
  else
    forces_rhs_kernel<float><<<grid, block, 0, s>>>(
        n, T.nf_ptr.p, T.nf_list.p, T.tri.p, x, X, v, m, mats, node_inst, f, b);
}

}  // namespace eolc
