// Learned block-sparse approximate inverse for the velocity solve.
//
// A message-passing network on the stencil of MDK (nodes = block rows,
// edges = off-diagonal block pairs i < j) maps local stiffness features to an
// approximate inverse G with the sparsity of MDK that is symmetric positive
// definite by construction:
//     G = F ( Lambda + sum_e [U_e; V_e][U_e; V_e]^T ) F
// Lambda_i = diag(softplus(theta_i) / d_i) (d_i = diagonal of MDK_ii, so
// theta = softplus^-1(1) reproduces Jacobi), U_e = S_i Ut_e, V_e = S_j Vt_e
// with S = diag(d)^-1/2 and Ut, Vt 3x3 network outputs, and F the free-DOF
// mask.  Each edge adds a rank-3 positive semidefinite 6x6 term, so G >= F
// Lambda F > 0 on the free DOFs whatever the weights.
//
// Network (width H = 64, weights rounded to BF16 in the forward pass, FP32
// accumulation):
//   h0 = relu(Wn f + bn)                        f: 8 node features
//   g  = sigmoid(Wg x + bg)                     x: 9 edge features
//   h^l = relu([h^{l-1}, agg^l] Wl + bl), l = 1..3,
//         agg^l_i = mean over edges e of i of g_e * h^{l-1}_other(e)
//   theta = h3 Wt + bt                          (3 per node)
//   o_e   = [h3_i, h3_j, x_e] Wo + bo           (18 per edge -> Ut, Vt)
// Training minimises the probe loss  sum_k |F (G A w_k - w_k)|^2 / |F w_k|^2
// over linear systems produced by the simulator (w_k: their solutions and
// seeded smooth random fields), with hand-written forward and backward
// kernels and Adam.  All reductions are deterministic (fixed-order two-stage
// sums), so training is bit-reproducible.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "tc.cuh"

namespace eolc {
namespace lpc {

constexpr int kH = 64, kFN = 8, kFE = 9, kOE = 18, kON = 3, kLayers = 3;
constexpr int kEdgeIn = 2 * kH + kFE;  // 137

// Parameter layout (offsets into one FP32 vector)
struct Layout {
  int Wn, bn, Wg, bg, Wl[kLayers], bl[kLayers], Wt, bt, Wo, bo, total;
};
inline Layout layout() {
  Layout L;
  int o = 0;
  L.Wn = o; o += kFN * kH;
  L.bn = o; o += kH;
  L.Wg = o; o += kFE * kH;
  L.bg = o; o += kH;
  for (int l = 0; l < kLayers; ++l) {
    L.Wl[l] = o; o += 2 * kH * kH;
    L.bl[l] = o; o += kH;
  }
  L.Wt = o; o += kH * kON;
  L.bt = o; o += kON;
  L.Wo = o; o += kEdgeIn * kOE;
  L.bo = o; o += kOE;
  L.total = o;
  return L;
}

// ---- device helpers ------------------------------------------------------------
__device__ __forceinline__ float bf16r(float w) {
  return __bfloat162float(__float2bfloat16(w));
}
__device__ __forceinline__ float softplus(float x) {
  return x > 20.f ? x : log1pf(expf(x));
}
__device__ __forceinline__ float sigm(float x) { return __fdividef(1.f, 1.f + __expf(-x)); }

enum Act { kNone = 0, kRelu = 1, kSigmoid = 2 };

// Y[r][c] = act(sum_k X[r][k] W[k][c] + b[c]); W is read through BF16.
// One CTA handles 64 rows x all columns (out <= 64); W staged in shared memory.
__global__ void dense_fwd_kernel(int rows, int in, int out, const float *__restrict__ X,
                                 const float *__restrict__ W, const float *__restrict__ b,
                                 int act, float *__restrict__ Y) {
  extern __shared__ float sW[];  // in*out + out
  for (int k = threadIdx.x; k < in * out; k += blockDim.x) sW[k] = bf16r(W[k]);
  for (int k = threadIdx.x; k < out; k += blockDim.x) sW[in * out + k] = b[k];
  __syncthreads();
  const int c = threadIdx.x % out;
  const int rsub = threadIdx.x / out, rstep = blockDim.x / out;
  if (rsub >= rstep) return;
  for (int r = blockIdx.x * 64 + rsub; r < min(rows, blockIdx.x * 64 + 64); r += rstep) {
    const float *x = X + size_t(r) * in;
    float acc = sW[in * out + c];
    for (int k = 0; k < in; ++k) acc += x[k] * sW[k * out + c];
    if (act == kRelu) acc = fmaxf(acc, 0.f);
    else if (act == kSigmoid) acc = sigm(acc);
    Y[size_t(r) * out + c] = acc;
  }
}

// dZ = dY * act'(Y) (in place into dY), dX = dZ W^T (optional), and per-CTA
// partial sums of dW = X^T dZ and db = sum dZ over this CTA's 64 rows.
__global__ void dense_bwd_kernel(int rows, int in, int out, const float *__restrict__ X,
                                 const float *__restrict__ W, const float *__restrict__ Y,
                                 float *__restrict__ dY, int act, float *__restrict__ dX,
                                 float *__restrict__ dWpart) {
  extern __shared__ float sm[];
  float *sW = sm;                   // in*out (BF16-rounded)
  float *sZ = sm + in * out;        // 64*out
  float *sX = sZ + 64 * out;        // 64*in
  const int r0 = blockIdx.x * 64, nr = min(64, rows - r0);
  for (int k = threadIdx.x; k < in * out; k += blockDim.x) sW[k] = bf16r(W[k]);
  for (int k = threadIdx.x; k < 64 * out; k += blockDim.x) {
    int r = k / out, c = k % out;
    float z = 0.f;
    if (r < nr) {
      float dy = dY[size_t(r0 + r) * out + c], y = Y[size_t(r0 + r) * out + c];
      z = act == kRelu ? (y > 0.f ? dy : 0.f) : (act == kSigmoid ? dy * y * (1.f - y) : dy);
      dY[size_t(r0 + r) * out + c] = z;
    }
    sZ[k] = z;
  }
  for (int k = threadIdx.x; k < 64 * in; k += blockDim.x) {
    int r = k / in;
    sX[k] = r < nr ? X[size_t(r0 + r) * in + (k % in)] : 0.f;
  }
  __syncthreads();
  if (dX) {
    for (int k = threadIdx.x; k < nr * in; k += blockDim.x) {
      int r = k / in, i = k % in;
      float acc = 0.f;
      for (int c = 0; c < out; ++c) acc += sZ[r * out + c] * sW[i * out + c];
      dX[size_t(r0 + r) * in + i] = acc;
    }
  }
  // dW partial: (in x out) + db (out)
  float *dst = dWpart + size_t(blockIdx.x) * (in * out + out);
  for (int k = threadIdx.x; k < in * out + out; k += blockDim.x) {
    float acc = 0.f;
    if (k < in * out) {
      int i = k / out, c = k % out;
      for (int r = 0; r < nr; ++r) acc += sX[r * in + i] * sZ[r * out + c];
    } else {
      int c = k - in * out;
      for (int r = 0; r < nr; ++r) acc += sZ[r * out + c];
    }
    dst[k] = acc;
  }
}

// grad[k] += sum over parts (fixed order) of part[p][k]
__global__ void reduce_parts_kernel(int nparts, int n, const float *__restrict__ parts,
                                    float *__restrict__ grad) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float acc = 0.f;
  for (int p = 0; p < nparts; ++p) acc += parts[size_t(p) * n + k];
  grad[k] += acc;
}

// ---- graph structure ------------------------------------------------------------
// Edges: off-diagonal block pairs (i < j) of the pattern; node incidence CSR
// lists (edge, side) with side 0 when the node is i.
struct Graph {
  int n = 0, m = 0, nb = 0;
  DevBuf<int> ei, ej, bij, bji, inc_ptr, inc, diag, rowptr, colidx;
  DevBuf<int> inc_o;     // per incidence entry: the edge's other node
  DevBuf<int> blk_edge;  // per block: edge id (off-diagonal) or -1
  DevBuf<float> deg_inv;
};

std::string build_graph(const HostTopology &H, Graph &G, cudaStream_t s) {
  const int n = H.n_nodes, nb = H.n_blocks;
  std::vector<int> ei, ej, bij, bji, blk_edge(nb, -1);
  for (int i = 0; i < n; ++i)
    for (int k = H.rowptr[i]; k < H.rowptr[i + 1]; ++k) {
      int j = H.colidx[k];
      if (j <= i) continue;
      // transpose block (j, i)
      int t = -1;
      for (int q = H.rowptr[j]; q < H.rowptr[j + 1]; ++q)
        if (H.colidx[q] == i) { t = q; break; }
      if (t < 0) return "pattern is not symmetric";
      blk_edge[k] = int(ei.size());
      blk_edge[t] = int(ei.size());
      ei.push_back(i); ej.push_back(j); bij.push_back(k); bji.push_back(t);
    }
  const int m = int(ei.size());
  std::vector<int> ptr(n + 1, 0), inc(2 * size_t(m));
  for (int e = 0; e < m; ++e) { ptr[ei[e] + 1]++; ptr[ej[e] + 1]++; }
  for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  std::vector<int> pos(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < m; ++e) {
    inc[pos[ei[e]]++] = 2 * e;
    inc[pos[ej[e]]++] = 2 * e + 1;
  }
  std::vector<int> inc_o(inc.size());
  for (size_t q = 0; q < inc.size(); ++q) {
    const int e = inc[q] >> 1;
    inc_o[q] = (inc[q] & 1) ? ei[e] : ej[e];
  }
  std::vector<float> dinv(n);
  for (int i = 0; i < n; ++i) dinv[i] = ptr[i + 1] > ptr[i] ? 1.f / float(ptr[i + 1] - ptr[i]) : 0.f;
  G.n = n; G.m = m; G.nb = nb;
  cudaError_t es[] = {G.ei.upload(ei.data(), m, s), G.ej.upload(ej.data(), m, s),
                      G.bij.upload(bij.data(), m, s), G.bji.upload(bji.data(), m, s),
                      G.inc_ptr.upload(ptr.data(), n + 1, s), G.inc.upload(inc.data(), inc.size(), s),
                      G.inc_o.upload(inc_o.data(), inc_o.size(), s),
                      G.diag.upload(H.diag.data(), n, s), G.rowptr.upload(H.rowptr.data(), n + 1, s),
                      G.colidx.upload(H.colidx.data(), nb, s),
                      G.blk_edge.upload(blk_edge.data(), nb, s),
                      G.deg_inv.upload(dinv.data(), n, s), cudaStreamSynchronize(s)};
  for (cudaError_t e : es)
    if (e != cudaSuccess) return cudaGetErrorString(e);
  return "";
}

// ---- features ---------------------------------------------------------------
// node: [log(sum of off-diagonal block norms / diagonal block norm), A_ii
//        normalised by its mean diagonal (6 unique entries), pinned fraction];
//        d = diag(A_ii) (3)
// edge: A_ij / sqrt(m_i m_j) (9), m = mean diagonal
// Node rows: eight lanes per node, each lane the norms of every eighth block
// of the row (consecutive lanes read consecutive blocks), summed by a fixed
// shuffle tree; then one thread per edge.
__global__ void features_kernel(int n, int m, const int *rowptr, const int *diag, const float *A,
                                const uint8_t *pinned, const int *ei, const int *ej,
                                const int *bij, float *fN, float *dvec, float *fE) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int node = t >> 3, sub = t & 7;
  float off = 0.f;
  int dk = 0;
  if (node < n) {
    dk = diag[node];
    for (int k = rowptr[node] + sub; k < rowptr[node + 1]; k += 8) {
      if (k == dk) continue;
      const float *B = A + size_t(k) * 9;
      float b2 = 0.f;
      for (int q = 0; q < 9; ++q) b2 += B[q] * B[q];
      off += sqrtf(b2);
    }
  }
  off += __shfl_xor_sync(0xffffffffu, off, 4);  // every lane of the warp takes part
  off += __shfl_xor_sync(0xffffffffu, off, 2);
  off += __shfl_xor_sync(0xffffffffu, off, 1);
  if (node < n) {
    if (sub == 0) {
      const float *D = A + size_t(dk) * 9;
      const float mdiag = (D[0] + D[4] + D[8]) / 3.f;
      float *f = fN + size_t(node) * kFN;
      // scale-free coupling strength: sum of off-diagonal block norms over
      // the diagonal block's norm (large when stiffness dominates mass)
      float dn = 0.f;
      for (int k = 0; k < 9; ++k) dn += D[k] * D[k];
      f[0] = logf(1e-12f + off / sqrtf(dn));
      f[1] = D[0] / mdiag; f[2] = D[4] / mdiag; f[3] = D[8] / mdiag;
      f[4] = D[1] / mdiag; f[5] = D[2] / mdiag; f[6] = D[5] / mdiag;
      f[7] = (pinned[3 * node] + pinned[3 * node + 1] + pinned[3 * node + 2]) / 3.f;
      dvec[3 * node] = D[0]; dvec[3 * node + 1] = D[4]; dvec[3 * node + 2] = D[8];
    }
  }
  if (t < m) {
    const int i = ei[t], j = ej[t];
    const float *Di = A + size_t(diag[i]) * 9, *Dj = A + size_t(diag[j]) * 9;
    float mi = (Di[0] + Di[4] + Di[8]) / 3.f, mj = (Dj[0] + Dj[4] + Dj[8]) / 3.f;
    float sc = rsqrtf(mi * mj);
    const float *B = A + size_t(bij[t]) * 9;
    float *f = fE + size_t(t) * kFE;
    for (int k = 0; k < 9; ++k) f[k] = B[k] * sc;
  }
}

// agg_i = deg_inv_i * sum_{(e,side) in inc(i)} g_e * h_other
__global__ void aggregate_fwd_kernel(int n, const int *inc_ptr, const int *inc, const int *ei,
                                     const int *ej, const float *deg_inv, const float *g,
                                     const float *h, float *agg_cat /* n x 2H, writes cols H.. */) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int i = t / kH, c = t % kH;
  if (i >= n) return;
  float acc = 0.f;
  for (int q = inc_ptr[i]; q < inc_ptr[i + 1]; ++q) {
    int e = inc[q] >> 1, side = inc[q] & 1;
    int o = side ? ei[e] : ej[e];
    acc += g[size_t(e) * kH + c] * h[size_t(o) * kH + c];
  }
  agg_cat[size_t(i) * 2 * kH + kH + c] = acc * deg_inv[i];
}

// dst[r][c] = src[r * ld + col0 + c] for c < w
__global__ void take_cols_kernel(int rows, int w, const float *src, int ld, int col0, float *dst) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * w) return;
  int r = t / w, c = t % w;
  dst[size_t(r) * w + c] = src[size_t(r) * ld + col0 + c];
}

// copy h into the first H columns of the [h, agg] input matrix
__global__ void copy_cols_kernel(int rows, int w, const float *src, int ld, int col0, float *dst) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * w) return;
  int r = t / w, c = t % w;
  dst[size_t(r) * ld + col0 + c] = src[size_t(r) * w + c];
}

// backward of aggregation: dh_j += sum over incident edges of dagg_other * g_e * deg_inv_other
// dg_e = dagg_i * h_j * deg_inv_i + dagg_j * h_i * deg_inv_j
__global__ void aggregate_bwd_h_kernel(int n, const int *inc_ptr, const int *inc, const int *ei,
                                       const int *ej, const float *deg_inv, const float *g,
                                       const float *dcat /* n x 2H */, float *dh /* += */) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int j = t / kH, c = t % kH;
  if (j >= n) return;
  float acc = 0.f;
  for (int q = inc_ptr[j]; q < inc_ptr[j + 1]; ++q) {
    int e = inc[q] >> 1, side = inc[q] & 1;
    int o = side ? ei[e] : ej[e];  // the node whose aggregate used h_j
    acc += dcat[size_t(o) * 2 * kH + kH + c] * g[size_t(e) * kH + c] * deg_inv[o];
  }
  dh[size_t(j) * kH + c] += acc;
}
__global__ void aggregate_bwd_g_kernel(int m, const int *ei, const int *ej, const float *deg_inv,
                                       const float *h, const float *dcat, float *dg /* += */) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int e = t / kH, c = t % kH;
  if (e >= m) return;
  int i = ei[e], j = ej[e];
  dg[size_t(e) * kH + c] += dcat[size_t(i) * 2 * kH + kH + c] * h[size_t(j) * kH + c] * deg_inv[i] +
                            dcat[size_t(j) * 2 * kH + kH + c] * h[size_t(i) * kH + c] * deg_inv[j];
}

// edge head input [h3_i, h3_j, x_e]
__global__ void edge_concat_kernel(int m, const int *ei, const int *ej, const float *h,
                                   const float *fE, float *X) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int e = t / kEdgeIn, c = t % kEdgeIn;
  if (e >= m) return;
  float v;
  if (c < kH) v = h[size_t(ei[e]) * kH + c];
  else if (c < 2 * kH) v = h[size_t(ej[e]) * kH + c - kH];
  else v = fE[size_t(e) * kFE + c - 2 * kH];
  X[size_t(e) * kEdgeIn + c] = v;
}
// backward: dh3 += contributions (gather per node over incident edges)
__global__ void edge_concat_bwd_kernel(int n, const int *inc_ptr, const int *inc,
                                       const float *dX, float *dh /* += */) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int i = t / kH, c = t % kH;
  if (i >= n) return;
  float acc = 0.f;
  for (int q = inc_ptr[i]; q < inc_ptr[i + 1]; ++q) {
    int e = inc[q] >> 1, side = inc[q] & 1;
    acc += dX[size_t(e) * kEdgeIn + side * kH + c];
  }
  dh[size_t(i) * kH + c] += acc;
}

// ---- inference forward: edge gates and the input layer ----------------------------
// Per (edge, four channels): gate_e = sigmoid(x_e Wg + bg), shared by the
// three message-passing layers; then per (node, four channels):
// h0_i = relu(f_i Wn + bn).  Both summed in the order of dense_fwd_kernel;
// the BF16-rounded weights sit in shared memory, and each thread takes
// kGateItems items so the staging is paid once per 2,048 items.
constexpr int kGateItems = 8;
__global__ void __launch_bounds__(256)
gate_h0_kernel(int m, int n, const float *__restrict__ fE, const float *__restrict__ Wg,
               const float *__restrict__ fN, const float *__restrict__ Wn,
               float *__restrict__ gate, float *__restrict__ h0) {
  __shared__ float4 sg[kFE + 1][kH / 4], sn[kFN + 1][kH / 4];
  for (int q = threadIdx.x; q < (kFE + 1) * kH; q += blockDim.x) {
    const float w = q < kFE * kH ? bf16r(Wg[q]) : Wg[q];
    reinterpret_cast<float *>(sg)[q] = w;
  }
  for (int q = threadIdx.x; q < (kFN + 1) * kH; q += blockDim.x) {
    const float w = q < kFN * kH ? bf16r(Wn[q]) : Wn[q];
    reinterpret_cast<float *>(sn)[q] = w;
  }
  __syncthreads();
  const int groups = kH / 4;
  const int t0 = blockIdx.x * blockDim.x * kGateItems + threadIdx.x;
  for (int t = t0; t < min(t0 + blockDim.x * kGateItems, (m + n) * groups); t += blockDim.x) {
  if (t < m * groups) {
    const int e = t / groups, c = t % groups;
    float4 g = sg[kFE][c];
#pragma unroll
    for (int k = 0; k < kFE; ++k) {
      const float x = __ldg(fE + size_t(e) * kFE + k);
      const float4 w = sg[k][c];
      g.x += x * w.x; g.y += x * w.y; g.z += x * w.z; g.w += x * w.w;
    }
    reinterpret_cast<float4 *>(gate)[t] = make_float4(sigm(g.x), sigm(g.y), sigm(g.z), sigm(g.w));
  } else if (t < (m + n) * groups) {
    const int u = t - m * groups;
    const int i = u / groups, c = u % groups;
    float4 a = sn[kFN][c];
#pragma unroll
    for (int k = 0; k < kFN; ++k) {
      const float x = __ldg(fN + size_t(i) * kFN + k);
      const float4 w = sn[k][c];
      a.x += x * w.x; a.y += x * w.y; a.z += x * w.z; a.w += x * w.w;
    }
    reinterpret_cast<float4 *>(h0)[u] =
        make_float4(fmaxf(a.x, 0.f), fmaxf(a.y, 0.f), fmaxf(a.z, 0.f), fmaxf(a.w, 0.f));
  }
  }
}

// agg_i = deg_inv_i * sum over the incidence entries of i (in order) of
// gate_e * h_other: a half-warp per node, four channels per lane.  The
// node's entries (edge, other node) are read by its lanes at once and
// broadcast, so the per-edge loads of the gate and of the neighbour's h row
// are independent of each other; no shared memory, so the SM keeps 64
// warps of gathers in flight.  The sums are those of aggregate_fwd_kernel.
__global__ void __launch_bounds__(256)
aggregate_kernel(int n, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                 const int *__restrict__ inc_o, const float *__restrict__ deg_inv,
                 const float *__restrict__ gate, const float *__restrict__ h_in,
                 float *__restrict__ agg) {
  const int lane = threadIdx.x & 31, hl = lane & 15, c4 = 4 * hl;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
  float a[4] = {0.f, 0.f, 0.f, 0.f};
  int q0 = 0, deg = 0;
  if (i < n) {
    q0 = inc_ptr[i];
    deg = inc_ptr[i + 1] - q0;
  }
  const int maxdeg = max(deg, __shfl_xor_sync(0xffffffffu, deg, 16));
  for (int base = 0; base < maxdeg; base += 16) {
    int me = 0, mo = 0;
    if (base + hl < deg) {
      me = inc[q0 + base + hl] >> 1;
      mo = inc_o[q0 + base + hl];
    }
    const int cnt = min(16, maxdeg - base);
#pragma unroll 4
    for (int t = 0; t < cnt; ++t) {
      const int e = __shfl_sync(0xffffffffu, me, t, 16);
      const int o = __shfl_sync(0xffffffffu, mo, t, 16);
      if (base + t < deg) {
        const float4 g = __ldg(reinterpret_cast<const float4 *>(gate + size_t(e) * kH + c4));
        const float4 ho = __ldg(reinterpret_cast<const float4 *>(h_in + size_t(o) * kH + c4));
        a[0] += g.x * ho.x;
        a[1] += g.y * ho.y;
        a[2] += g.z * ho.z;
        a[3] += g.w * ho.w;
      }
    }
  }
  if (i < n) {
    const float d = deg_inv[i];
    reinterpret_cast<float4 *>(agg)[size_t(i) * (kH / 4) + hl] =
        make_float4(a[0] * d, a[1] * d, a[2] * d, a[3] * d);
  }
}

// ---- inference forward on the tensor cores --------------------------------------
// One message-passing layer per launch.  A CTA takes kTcM = 128 nodes (the
// MMA's M): its rows of [h, agg] (agg from aggregate_kernel) go as three
// BF16 terms into K-major shared-memory tiles; one
// thread then issues the 128 x 64 x 128 product with W (BF16) as
// 8 K-steps x 3 terms of tcgen05.mma into a TMEM accumulator, and the eight
// warps read it back (warp w: rows 32 (w % 4) .., columns 32 (w / 4) ..),
// add the bias and apply relu.  The last layer keeps h3 on chip: its rows go
// back into shared memory as the A operand of a second product with
// [Wo_i | Wo_j | Wt] (64 x 39, padded to 48), which gives every node's share
// of the edge head (h3_i Wo_i, h3_j Wo_j) and theta = h3 Wt + bt.
// The training forward (dense_fwd_kernel, aggregate_fwd_kernel) computes the
// same network on the CUDA cores; the two agree to FP32 rounding.
constexpr int kTcM = 128;
constexpr int kTcThreads = 256;
constexpr int kLayerK = 2 * kH;                      // [h, agg]
constexpr int kLayerPart = kTcM * kLayerK * 2;       // one BF16 term tile (32 KB)
constexpr int kLayerB = kH * kLayerK * 2;            // W^T (16 KB)
constexpr int kHeadN = 48;                           // [Wo_i | Wo_j | Wt] padded
constexpr int kHeadCols = 2 * kOE + kON;             // 39 used head columns
constexpr int kLayerSmem = tc::kSplit * kLayerPart + kLayerB + 16;  // two CTAs per SM
constexpr long long kTcWaitLimit = 1ll << 20;
// MMA completions that did not arrive within kTcWaitLimit polls (their rows
// are written as NaN, which the solve reports as non-finite)
__device__ unsigned int g_tc_timeouts = 0;

template <bool LAST>
__global__ void __launch_bounds__(kTcThreads, 2)
layer_tc_kernel(int n, const float *__restrict__ agg, const float *__restrict__ Wl,
                const float *__restrict__ Wo, const float *__restrict__ Wt,
                const float *__restrict__ h_in, float *__restrict__ h_out,
                float *__restrict__ head, float *__restrict__ theta) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  uint8_t *sA = tc_smem;                             // kSplit tiles, 128 x 128
  uint8_t *sB = tc_smem + tc::kSplit * kLayerPart;        // W^T, 64 x 128
  uint64_t *bar = reinterpret_cast<uint64_t *>(sB + kLayerB);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
  constexpr uint32_t kCols = LAST ? 128 : 64;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int node0 = blockIdx.x * kTcM;
  if (warp == 0) tc::tmem_alloc(tslot, kCols);
  if (threadIdx.x == 32) tc::mbar_init(bar, 1);
  for (int q = threadIdx.x; q < kLayerK * kH; q += kTcThreads) {
    const int k = q / kH, c = q % kH;
    *reinterpret_cast<__nv_bfloat16 *>(sB + tc::tile_off(c, k, kLayerK)) =
        __float2bfloat16_rn(Wl[q]);
  }
  // [h, agg] rows of the tile (zero past n): a half-warp per row, four
  // channels per lane, as three BF16 terms
  // (the loads of four row pairs are issued before their stores)
  const int half = lane >> 4, hl = lane & 15, c4 = 4 * hl;
  constexpr int kPairIters = kTcM / 2 / (kTcThreads / 32), kBatch = 4;
  static_assert(kPairIters % kBatch == 0, "row batches");
  for (int b0 = 0; b0 < kPairIters; b0 += kBatch) {
    float4 hv[kBatch], av[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int i = node0 + 2 * (warp + (kTcThreads / 32) * (b0 + u)) + half;
      hv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      av[u] = hv[u];
      if (i < n) {
        hv[u] = __ldg(reinterpret_cast<const float4 *>(h_in + size_t(i) * kH + c4));
        av[u] = __ldg(reinterpret_cast<const float4 *>(agg + size_t(i) * kH + c4));
      }
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int ln = 2 * (warp + (kTcThreads / 32) * (b0 + u)) + half;
      tc::put3x4(sA, kLayerPart, ln, c4, kLayerK, hv[u].x, hv[u].y, hv[u].z, hv[u].w);
      tc::put3x4(sA, kLayerPart, ln, kH + c4, kLayerK, av[u].x, av[u].y, av[u].z, av[u].w);
    }
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t a_base = tc::smem_u32(sA), b_base = tc::smem_u32(sB);
  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = tc::idesc_bf16(kTcM, kH);
    for (int s = 0; s < kLayerK / 16; ++s)
      for (int p = 0; p < tc::kSplit; ++p)
        tc::mma_bf16(tmem, tc::smem_desc(a_base + p * kLayerPart + 256 * s, 128, kLayerK * 16),
                     tc::smem_desc(b_base + 256 * s, 128, kLayerK * 16), idesc,
                     uint32_t(s | p));
    tc::mma_commit(bar);
  }
  const bool ok0 = __all_sync(0xffffffffu, tc::mbar_wait(bar, 0, kTcWaitLimit));
  bool ok = ok0;
  tc::fence_after_sync();
  const int row = 32 * (warp & 3) + lane, c0 = 32 * (warp >> 2);
  const int i = node0 + row;
  const uint32_t lane_addr = uint32_t(32 * (warp & 3)) << 16;
  float v[32];
  if (ok) tc::tmem_ld32(tmem + lane_addr + c0, v);
  const float *bias = Wl + 2 * kH * kH;
#pragma unroll
  for (int k = 0; k < 32; ++k)
    v[k] = ok ? fmaxf(v[k] + __ldg(bias + c0 + k), 0.f) : __int_as_float(0x7fc00000);
  if (!LAST) {
    if (i < n) {
      float4 *dst = reinterpret_cast<float4 *>(h_out + size_t(i) * kH + c0);
#pragma unroll
      for (int k = 0; k < 8; ++k) dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    }
  } else {
    // the layer product has completed: h3 rows (zero past n) go into the
    // first kSplit x 16 KB of the A tiles as the 128 x 64 A operand of the
    // head product, the head weights^T (48 x 64) after them
    constexpr int kPart2 = kTcM * kH * 2;
    uint8_t *sH = sA + tc::kSplit * kPart2;
#pragma unroll
    for (int k = 0; k < 32; k += 4)
      tc::put3x4(sA, kPart2, row, c0 + k, kH, i < n ? v[k] : 0.f, i < n ? v[k + 1] : 0.f,
                 i < n ? v[k + 2] : 0.f, i < n ? v[k + 3] : 0.f);
    for (int q = threadIdx.x; q < kHeadN * kH; q += kTcThreads) {
      const int k = q / kHeadN, c = q % kHeadN;
      float w = 0.f;
      if (c < kOE) w = Wo[k * kOE + c];                         // h3_i rows of Wo
      else if (c < 2 * kOE) w = Wo[(kH + k) * kOE + c - kOE];   // h3_j rows of Wo
      else if (c < kHeadCols) w = Wt[k * kON + c - 2 * kOE];
      *reinterpret_cast<__nv_bfloat16 *>(sH + tc::tile_off(c, k, kH)) = __float2bfloat16_rn(w);
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0 && ok0) {
      constexpr uint32_t idesc = tc::idesc_bf16(kTcM, kHeadN);
      const uint32_t h_base = tc::smem_u32(sH);
      for (int s = 0; s < kH / 16; ++s)
        for (int p = 0; p < tc::kSplit; ++p)
          tc::mma_bf16(tmem + kH, tc::smem_desc(a_base + p * kPart2 + 256 * s, 128, kH * 16),
                       tc::smem_desc(h_base + 256 * s, 128, kH * 16), idesc, uint32_t(s | p));
      tc::mma_commit(bar);
    }
    ok = ok && __all_sync(0xffffffffu, tc::mbar_wait(bar, 1, kTcWaitLimit));
    tc::fence_after_sync();
    if (ok) tc::tmem_ld32(tmem + lane_addr + kH + c0, v);
    if (!ok)
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = __int_as_float(0x7fc00000);
    if (i < n) {
      // head row: 36 floats (144 bytes, 16-byte aligned) as float4 stores;
      // columns 36..38 are theta
      float4 *hrow = reinterpret_cast<float4 *>(head + size_t(i) * 2 * kOE);
      if (c0 == 0) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
          hrow[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
      } else {
        hrow[8] = make_float4(v[0], v[1], v[2], v[3]);
#pragma unroll
        for (int k = 0; k < kON; ++k)
          theta[size_t(i) * kON + k] = v[4 + k] + __ldg(Wt + kH * kON + k);
      }
    }
  }
  if (!ok) {
    if (lane == 0) atomicAdd(&g_tc_timeouts, 1u);
    tc::mbar_wait(bar, ok0 ? 1 : 0, kTcWaitLimit);  // let an MMA in flight land
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---- G assembly -----------------------------------------------------------------
// 3x3 helpers, row-major
__device__ __forceinline__ void mmT(const float *P, const float *Q, float *R) {  // R = P Q^T
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      R[3 * a + b] = P[3 * a] * Q[3 * b] + P[3 * a + 1] * Q[3 * b + 1] + P[3 * a + 2] * Q[3 * b + 2];
}

// U_e = S_i Ut_e (rows scaled by d_i^-1/2), V_e = S_j Vt_e
__device__ __forceinline__ void edge_UV(int e, const int *ei, const int *ej, const float *o,
                                        const float *dvec, float *U, float *V) {
  const int i = ei[e], j = ej[e];
  const float *oe = o + size_t(e) * kOE;
  for (int a = 0; a < 3; ++a) {
    float si = rsqrtf(dvec[3 * i + a]), sj = rsqrtf(dvec[3 * j + a]);
    for (int b = 0; b < 3; ++b) {
      U[3 * a + b] = si * oe[3 * a + b];
      V[3 * a + b] = sj * oe[9 + 3 * a + b];
    }
  }
}

// One thread per BSR block of G (same pattern as MDK).
__global__ void g_assemble_kernel(int nb, const int *blk_row, const int *colidx, const int *blk_edge,
                                  const int *inc_ptr, const int *inc, const int *ei, const int *ej,
                                  const float *o, const float *theta, const float *dvec,
                                  const uint8_t *pinned, float *Gv) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int i = blk_row[b], j = colidx[b];
  float acc[9];
  for (int k = 0; k < 9; ++k) acc[k] = 0.f;
  float U[9], V[9], R[9];
  if (i == j) {
    for (int a = 0; a < 3; ++a) acc[4 * a] = softplus(theta[3 * i + a]) / dvec[3 * i + a];
    for (int q = inc_ptr[i]; q < inc_ptr[i + 1]; ++q) {
      int e = inc[q] >> 1, side = inc[q] & 1;
      edge_UV(e, ei, ej, o, dvec, U, V);
      if (side == 0) mmT(U, U, R); else mmT(V, V, R);
      for (int k = 0; k < 9; ++k) acc[k] += R[k];
    }
  } else {
    int e = blk_edge[b];
    edge_UV(e, ei, ej, o, dvec, U, V);
    if (i == ei[e]) mmT(U, V, acc); else mmT(V, U, acc);
  }
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) {
      bool free_ac = !pinned[3 * i + a] && !pinned[3 * j + c];
      Gv[size_t(b) * 9 + 3 * a + c] = free_ac ? acc[3 * a + c] : 0.f;
    }
}

// Inference G assembly in two passes over the graph instead of one thread
// per block.  edge_blocks_kernel, one thread per edge e = (i, j): the edge
// head o_e = h3_i Wo_i + h3_j Wo_j + (bo + x_e Wo_x) from the per-node
// shares of layer_tc_kernel<true>, U_e and V_e (kept for the diagonal pass)
// and the two off-diagonal blocks G_ij = U V^T, G_ji = V U^T.
// node_blocks_kernel, one thread per node: G_ii = Lambda_i + the U U^T or
// V V^T terms of its incident edges, in incidence order.  The blocks are the
// ones g_assemble_kernel forms from the same o and theta.
__global__ void __launch_bounds__(128)
edge_blocks_kernel(int m, const int *__restrict__ ei, const int *__restrict__ ej,
                   const int *__restrict__ bij, const int *__restrict__ bji,
                   const float *__restrict__ head, const float *__restrict__ fE,
                   const float *__restrict__ Wo, const float *__restrict__ dvec,
                   const uint8_t *__restrict__ pinned, float *__restrict__ uv,
                   float *__restrict__ Gv) {
  __shared__ float sW[kFE * kOE + kOE];
  // per warp: its 32 edges' U, V (18 each) and two blocks (9 each), written
  // back to global memory lane-contiguously
  __shared__ float sOut[4][32 * 36];
  for (int k = threadIdx.x; k < kFE * kOE; k += blockDim.x) sW[k] = bf16r(Wo[2 * kH * kOE + k]);
  for (int k = threadIdx.x; k < kOE; k += blockDim.x) sW[kFE * kOE + k] = Wo[kEdgeIn * kOE + k];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e0 = blockIdx.x * blockDim.x + 32 * warp, e = e0 + lane;
  float *so = sOut[warp];
  if (e < m) {
    const int i = ei[e], j = ej[e];
    float acc[kOE];
#pragma unroll
    for (int c = 0; c < kOE; ++c) acc[c] = sW[kFE * kOE + c];
    for (int k = 0; k < kFE; ++k) {
      const float x = __ldg(fE + size_t(e) * kFE + k);
#pragma unroll
      for (int c = 0; c < kOE; ++c) acc[c] += x * sW[k * kOE + c];
    }
    const float *hi = head + size_t(i) * 2 * kOE, *hj = head + size_t(j) * 2 * kOE + kOE;
    float U[9], V[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float si = rsqrtf(dvec[3 * i + a]), sj = rsqrtf(dvec[3 * j + a]);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        U[3 * a + b] = si * ((__ldg(hi + 3 * a + b) + __ldg(hj + 3 * a + b)) + acc[3 * a + b]);
        V[3 * a + b] = sj * ((__ldg(hi + 9 + 3 * a + b) + __ldg(hj + 9 + 3 * a + b)) +
                             acc[9 + 3 * a + b]);
      }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      so[18 * lane + k] = U[k];
      so[18 * lane + 9 + k] = V[k];
    }
    float R[9];
    mmT(U, V, R);
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c)
        so[576 + 9 * lane + 3 * a + c] =
            (!pinned[3 * i + a] && !pinned[3 * j + c]) ? R[3 * a + c] : 0.f;
    mmT(V, U, R);
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c)
        so[864 + 9 * lane + 3 * a + c] =
            (!pinned[3 * j + a] && !pinned[3 * i + c]) ? R[3 * a + c] : 0.f;
  }
  __syncwarp();
  const int ne = min(32, m - e0);
  if (ne <= 0) return;
  for (int t = lane; t < 18 * ne; t += 32) uv[size_t(e0) * 18 + t] = so[t];
  for (int t = lane; t < 9 * ne; t += 32) {
    const int q = t / 9, c = t - 9 * q;
    Gv[size_t(__ldg(bij + e0 + q)) * 9 + c] = so[576 + t];
    Gv[size_t(__ldg(bji + e0 + q)) * 9 + c] = so[864 + t];
  }
}

__global__ void __launch_bounds__(128)
node_blocks_kernel(int n, const int *__restrict__ diag, const int *__restrict__ inc_ptr,
                   const int *__restrict__ inc, const float *__restrict__ uv,
                   const float *__restrict__ theta, const float *__restrict__ dvec,
                   const uint8_t *__restrict__ pinned, float *__restrict__ Gv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float acc[9];
  for (int k = 0; k < 9; ++k) acc[k] = 0.f;
  for (int a = 0; a < 3; ++a) acc[4 * a] = softplus(theta[3 * i + a]) / dvec[3 * i + a];
  for (int q = inc_ptr[i]; q < inc_ptr[i + 1]; ++q) {
    const int e = inc[q] >> 1, side = inc[q] & 1;
    float P[9], R[9];
    for (int k = 0; k < 9; ++k) P[k] = __ldg(uv + size_t(e) * 18 + 9 * side + k);
    mmT(P, P, R);
    for (int k = 0; k < 9; ++k) acc[k] += R[k];
  }
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c)
      Gv[size_t(diag[i]) * 9 + 3 * a + c] =
          (!pinned[3 * i + a] && !pinned[3 * i + c]) ? acc[3 * a + c] : 0.f;
}

// dG (masked) -> d o_e (18) per edge and d theta per node.
__global__ void g_assemble_bwd_edges_kernel(int m, const int *ei, const int *ej, const int *bij,
                                            const int *bji, const int *diag, const float *o,
                                            const float *dvec, const uint8_t *pinned,
                                            const float *dG, float *dO) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  const int i = ei[e], j = ej[e];
  float U[9], V[9];
  edge_UV(e, ei, ej, o, dvec, U, V);
  float Gij[9], Gji[9], Gii[9], Gjj[9];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) {
      float mij = (!pinned[3 * i + a] && !pinned[3 * j + c]) ? 1.f : 0.f;
      float mji = (!pinned[3 * j + a] && !pinned[3 * i + c]) ? 1.f : 0.f;
      float mii = (!pinned[3 * i + a] && !pinned[3 * i + c]) ? 1.f : 0.f;
      float mjj = (!pinned[3 * j + a] && !pinned[3 * j + c]) ? 1.f : 0.f;
      Gij[3 * a + c] = mij * dG[size_t(bij[e]) * 9 + 3 * a + c];
      Gji[3 * a + c] = mji * dG[size_t(bji[e]) * 9 + 3 * a + c];
      Gii[3 * a + c] = mii * dG[size_t(diag[i]) * 9 + 3 * a + c];
      Gjj[3 * a + c] = mjj * dG[size_t(diag[j]) * 9 + 3 * a + c];
    }
  // dU = dGij V + dGji^T V + (dGii + dGii^T) U ; dV = dGij^T U + dGji U + (dGjj + dGjj^T) V
  float dU[9], dV[9];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      float su = 0.f, sv = 0.f;
      for (int k = 0; k < 3; ++k) {
        su += Gij[3 * a + k] * V[3 * k + b] + Gji[3 * k + a] * V[3 * k + b] +
              (Gii[3 * a + k] + Gii[3 * k + a]) * U[3 * k + b];
        sv += Gij[3 * k + a] * U[3 * k + b] + Gji[3 * a + k] * U[3 * k + b] +
              (Gjj[3 * a + k] + Gjj[3 * k + a]) * V[3 * k + b];
      }
      dU[3 * a + b] = su;
      dV[3 * a + b] = sv;
    }
  float *d = dO + size_t(e) * kOE;
  for (int a = 0; a < 3; ++a) {
    float si = rsqrtf(dvec[3 * i + a]), sj = rsqrtf(dvec[3 * j + a]);
    for (int b = 0; b < 3; ++b) {
      d[3 * a + b] = si * dU[3 * a + b];
      d[9 + 3 * a + b] = sj * dV[3 * a + b];
    }
  }
}
__global__ void g_assemble_bwd_nodes_kernel(int n, const int *diag, const float *theta,
                                            const float *dvec, const uint8_t *pinned,
                                            const float *dG, float *dtheta) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int a = 0; a < 3; ++a) {
    float g = pinned[3 * i + a] ? 0.f : dG[size_t(diag[i]) * 9 + 4 * a];
    dtheta[3 * i + a] = g * sigm(theta[3 * i + a]) / dvec[3 * i + a];
  }
}

// ---- loss -------------------------------------------------------------------------
// z = G y for one probe, r = F (z - w); per-row r and partial |r|^2 in FP64
__global__ void probe_residual_kernel(int n, const int *rowptr, const int *colidx, const float *Gv,
                                      const float *y, const float *w, const uint8_t *pinned,
                                      float *r, double *part) {
  __shared__ double red[256];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0;
  if (i < n) {
    float z[3] = {0.f, 0.f, 0.f};
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = colidx[k];
      const float *B = Gv + size_t(k) * 9;
      for (int a = 0; a < 3; ++a)
        z[a] += B[3 * a] * y[3 * j] + B[3 * a + 1] * y[3 * j + 1] + B[3 * a + 2] * y[3 * j + 2];
    }
    for (int a = 0; a < 3; ++a) {
      float v = pinned[3 * i + a] ? 0.f : z[a] - w[3 * i + a];
      r[3 * i + a] = v;
      acc += double(v) * double(v);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// dG_b += scale * r[i] y[j]^T for every block b = (i, j)
__global__ void probe_grad_kernel(int nb, const int *blk_row, const int *colidx, const float *r,
                                  const float *y, float scale, float *dG) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  int i = blk_row[b], j = colidx[b];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) dG[size_t(b) * 9 + 3 * a + c] += scale * r[3 * i + a] * y[3 * j + c];
}

// y = A w (FP32 SpMV)
__global__ void spmv_kernel(int n, const int *rowptr, const int *colidx, const float *A,
                            const float *w, float *y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float z[3] = {0.f, 0.f, 0.f};
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    int j = colidx[k];
    const float *B = A + size_t(k) * 9;
    for (int a = 0; a < 3; ++a)
      z[a] += B[3 * a] * w[3 * j] + B[3 * a + 1] * w[3 * j + 1] + B[3 * a + 2] * w[3 * j + 2];
  }
  for (int a = 0; a < 3; ++a) y[3 * i + a] = z[a];
}

// *out += weight * sum of the parts (one thread, fixed order)
__global__ void accumulate_kernel(int n, const double *part, double weight, double *out) {
  if (threadIdx.x || blockIdx.x) return;
  double s = 0;
  for (int k = 0; k < n; ++k) s += part[k];
  *out += weight * s;
}

// Adam, one thread per parameter
__global__ void adam_kernel(int n, float *p, const float *g, float *m1, float *m2, float lr,
                            float b1, float b2, float eps, float bc1, float bc2, float clip) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float gk = fminf(fmaxf(g[k], -clip), clip);
  m1[k] = b1 * m1[k] + (1.f - b1) * gk;
  m2[k] = b2 * m2[k] + (1.f - b2) * gk * gk;
  p[k] -= lr * (m1[k] / bc1) / (sqrtf(m2[k] / bc2) + eps);
}

}  // namespace lpc

// ---------------------------------------------------------------------------
// Network state, activations and training storage.
struct LearnedPC {
  int device = 0;
  lpc::Layout L;
  std::vector<float> h_params;
  DevBuf<float> params, grad, m1, m2, parts;
  DevBuf<double> dpart, dloss;
  int adam_t = 0;
  // graph + activations for the current topology
  const void *topo_key = nullptr;
  int topo_n = -1, topo_nb = -1;
  bool topo_train = false;  // training buffers allocated for this topology
  lpc::Graph G;
  DevBuf<float> fN, dvec, fE, h[4], cat[3], gate, eX, o, theta;
  DevBuf<float> head;  // inference: per-node shares of the edge head (2 x 18)
  DevBuf<float> uv;    // inference: U_e, V_e per edge (2 x 9)
  DevBuf<float> agg;   // inference: a layer's aggregated neighbour rows
  DevBuf<float> dh, dcat, dgate, deX, dO, dtheta, dGv, tmpX;
  DevBuf<float> Gv;
  // training set: one topology, many systems
  HostTopology train_topo;
  bool has_train_topo = false;
  std::vector<DevBuf<float> *> sys_A;
  std::vector<DevBuf<uint8_t> *> sys_pin;
  std::vector<DevBuf<float> *> sys_w;  // probe vectors (3N each, k per system)
  std::vector<int> sys_nprobe;
  DevBuf<float> y, r;
  std::string err;
  ~LearnedPC() {
    for (auto *p : sys_A) delete p;
    for (auto *p : sys_pin) delete p;
    for (auto *p : sys_w) delete p;
  }
};

namespace lpc {

// Glorot-style deterministic initialisation (LCG), heads started near Jacobi:
// Wo small, theta bias = softplus^-1(1).
void init_params(LearnedPC &P, unsigned seed) {
  const Layout &L = P.L;
  P.h_params.assign(L.total, 0.f);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
  auto rnd = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return float((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
  };
  auto fill = [&](int off, int fan_in, int fan_out, float gain) {
    float a = gain * std::sqrt(6.f / float(fan_in + fan_out));
    for (int k = 0; k < fan_in * fan_out; ++k) P.h_params[off + k] = a * rnd();
  };
  fill(L.Wn, kFN, kH, 1.f);
  fill(L.Wg, kFE, kH, 1.f);
  for (int l = 0; l < kLayers; ++l) fill(L.Wl[l], 2 * kH, kH, 1.f);
  fill(L.Wt, kH, kON, 0.1f);
  fill(L.Wo, kEdgeIn, kOE, 0.05f);
  for (int a = 0; a < kON; ++a) P.h_params[L.bt + a] = std::log(std::exp(1.f) - 1.f);
}

struct Ptrs {
  const float *A;
  const uint8_t *pinned;
};

inline int nblk(int rows, int per) { return (rows + per - 1) / per; }

// Forward pass over the context-independent graph G; fills P.o, P.theta,
// P.Gv.  Returns "" or a message.
std::string forward(LearnedPC &P, const Graph &G, const int *blk_row, const float *A,
                    const uint8_t *pinned, cudaStream_t s) {
  const Layout &L = P.L;
  const float *W = P.params.p;
  const int n = G.n, m = G.m;
  features_kernel<<<nblk(std::max(8 * n, m), 256), 256, 0, s>>>(n, m, G.rowptr.p, G.diag.p, A, pinned,
                                                          G.ei.p, G.ej.p, G.bij.p, P.fN.p,
                                                          P.dvec.p, P.fE.p);
  auto dense = [&](int rows, int in, int out, const float *X, int woff, int boff, int act, float *Y) {
    // W and b are adjacent in the layout (W then b)
    (void)boff;
    size_t smem = size_t(in * out + out) * sizeof(float);
    dense_fwd_kernel<<<nblk(rows, 64), 256, smem, s>>>(rows, in, out, X, W + woff, W + woff + in * out,
                                                       act, Y);
  };
  dense(n, kFN, kH, P.fN.p, L.Wn, L.bn, kRelu, P.h[0].p);
  dense(m, kFE, kH, P.fE.p, L.Wg, L.bg, kSigmoid, P.gate.p);
  for (int l = 0; l < kLayers; ++l) {
    copy_cols_kernel<<<nblk(n * kH, 256), 256, 0, s>>>(n, kH, P.h[l].p, 2 * kH, 0, P.cat[l].p);
    aggregate_fwd_kernel<<<nblk(n * kH, 256), 256, 0, s>>>(n, G.inc_ptr.p, G.inc.p, G.ei.p, G.ej.p,
                                                         G.deg_inv.p, P.gate.p, P.h[l].p,
                                                         P.cat[l].p);
    dense(n, 2 * kH, kH, P.cat[l].p, L.Wl[l], L.bl[l], kRelu, P.h[l + 1].p);
  }
  dense(n, kH, kON, P.h[3].p, L.Wt, L.bt, kNone, P.theta.p);
  edge_concat_kernel<<<nblk(m * kEdgeIn, 256), 256, 0, s>>>(m, G.ei.p, G.ej.p, P.h[3].p, P.fE.p,
                                                          P.eX.p);
  dense(m, kEdgeIn, kOE, P.eX.p, L.Wo, L.bo, kNone, P.o.p);
  g_assemble_kernel<<<nblk(G.nb, 128), 128, 0, s>>>(G.nb, blk_row, G.colidx.p, G.blk_edge.p,
                                                   G.inc_ptr.p, G.inc.p, G.ei.p, G.ej.p, P.o.p,
                                                   P.theta.p, P.dvec.p, pinned, P.Gv.p);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? "" : cudaGetErrorString(e);
}

// Backward from dGv (in P.dGv) to P.grad (accumulated).
std::string backward(LearnedPC &P, const Graph &G, const uint8_t *pinned, cudaStream_t s) {
  const Layout &L = P.L;
  const float *W = P.params.p;
  const int n = G.n, m = G.m;
  g_assemble_bwd_edges_kernel<<<nblk(m, 128), 128, 0, s>>>(m, G.ei.p, G.ej.p, G.bij.p, G.bji.p,
                                                          G.diag.p, P.o.p, P.dvec.p, pinned,
                                                          P.dGv.p, P.dO.p);
  g_assemble_bwd_nodes_kernel<<<nblk(n, 128), 128, 0, s>>>(n, G.diag.p, P.theta.p, P.dvec.p,
                                                          pinned, P.dGv.p, P.dtheta.p);
  auto dense_b = [&](int rows, int in, int out, const float *X, int woff, const float *Y, float *dY,
                     int act, float *dX) {
    int nb = nblk(rows, 64);
    size_t smem = size_t(in * out + 64 * out + 64 * in) * sizeof(float);
    dense_bwd_kernel<<<nb, 256, smem, s>>>(rows, in, out, X, W + woff, Y, dY, act, dX, P.parts.p);
    int nw = in * out + out;
    reduce_parts_kernel<<<nblk(nw, 256), 256, 0, s>>>(nb, nw, P.parts.p, P.grad.p + woff);
  };
  // heads
  dense_b(m, kEdgeIn, kOE, P.eX.p, L.Wo, P.o.p, P.dO.p, kNone, P.deX.p);
  cudaMemsetAsync(P.dh.p, 0, sizeof(float) * size_t(n) * kH, s);
  dense_b(n, kH, kON, P.h[3].p, L.Wt, P.theta.p, P.dtheta.p, kNone, P.tmpX.p);
  copy_cols_kernel<<<nblk(n * kH, 256), 256, 0, s>>>(n, kH, P.tmpX.p, kH, 0, P.dh.p);
  edge_concat_bwd_kernel<<<nblk(n * kH, 256), 256, 0, s>>>(n, G.inc_ptr.p, G.inc.p, P.deX.p, P.dh.p);
  cudaMemsetAsync(P.dgate.p, 0, sizeof(float) * size_t(m) * kH, s);
  for (int l = kLayers - 1; l >= 0; --l) {
    // dh currently holds d h^{l+1}; through relu dense -> dcat
    dense_b(n, 2 * kH, kH, P.cat[l].p, L.Wl[l], P.h[l + 1].p, P.dh.p, kRelu, P.dcat.p);
    // d h^l = dcat[:, :H] + aggregation backward
    cudaMemsetAsync(P.dh.p, 0, sizeof(float) * size_t(n) * kH, s);
    take_cols_kernel<<<nblk(n * kH, 256), 256, 0, s>>>(n, kH, P.dcat.p, 2 * kH, 0, P.dh.p);
    aggregate_bwd_h_kernel<<<nblk(n * kH, 256), 256, 0, s>>>(n, G.inc_ptr.p, G.inc.p, G.ei.p,
                                                           G.ej.p, G.deg_inv.p, P.gate.p, P.dcat.p,
                                                           P.dh.p);
    aggregate_bwd_g_kernel<<<nblk(m * kH, 256), 256, 0, s>>>(m, G.ei.p, G.ej.p, G.deg_inv.p,
                                                           P.h[l].p, P.dcat.p, P.dgate.p);
  }
  dense_b(n, kFN, kH, P.fN.p, L.Wn, P.h[0].p, P.dh.p, kRelu, nullptr);
  dense_b(m, kFE, kH, P.fE.p, L.Wg, P.gate.p, P.dgate.p, kSigmoid, nullptr);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? "" : cudaGetErrorString(e);
}

}  // namespace lpc
}  // namespace eolc

// ===========================================================================
// Host-side management and C ABI
// ===========================================================================
namespace eolc {
namespace lpc {

// Inference forward (kLearnedForwardLaunches = 10 launches): features, edge
// gates with h0, three (aggregation, layer) pairs -- the last layer with the
// node-side heads --, the edge head with the off-diagonal blocks of G, the
// diagonal blocks.  Fills
// P.Gv; the network of forward() to FP32 rounding.
std::string forward_fused(LearnedPC &P, const Graph &G, const int *blk_row, const float *A,
                          const uint8_t *pinned, cudaStream_t s) {
  const Layout &L = P.L;
  const float *W = P.params.p;
  const int n = G.n, m = G.m;
  int dev = 0;
  cudaGetDevice(&dev);
  static bool attr_set[2][64] = {};
  if (dev < 64 && !attr_set[0][dev]) {
    cudaFuncSetAttribute(layer_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kLayerSmem);
    cudaFuncSetAttribute(layer_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kLayerSmem);
    attr_set[0][dev] = true;
  }
  features_kernel<<<nblk(std::max(8 * n, m), 256), 256, 0, s>>>(n, m, G.rowptr.p, G.diag.p, A, pinned,
                                                          G.ei.p, G.ej.p, G.bij.p, P.fN.p,
                                                          P.dvec.p, P.fE.p);
  const int gh = (m + n) * (kH / 4);
  gate_h0_kernel<<<(gh + 256 * kGateItems - 1) / (256 * kGateItems), 256, 0, s>>>(
      m, n, P.fE.p, W + L.Wg, P.fN.p, W + L.Wn, P.gate.p, P.h[0].p);
  const int grid = nblk(n, kTcM), agrid = nblk(16 * n, 256);
  for (int l = 0; l + 1 < kLayers; ++l) {
    aggregate_kernel<<<agrid, 256, 0, s>>>(n, G.inc_ptr.p, G.inc.p, G.inc_o.p, G.deg_inv.p,
                                          P.gate.p, P.h[l].p, P.agg.p);
    layer_tc_kernel<false><<<grid, kTcThreads, kLayerSmem, s>>>(
        n, P.agg.p, W + L.Wl[l], W + L.Wo, W + L.Wt, P.h[l].p, P.h[l + 1].p, nullptr, nullptr);
  }
  aggregate_kernel<<<agrid, 256, 0, s>>>(n, G.inc_ptr.p, G.inc.p, G.inc_o.p, G.deg_inv.p,
                                        P.gate.p, P.h[kLayers - 1].p, P.agg.p);
  layer_tc_kernel<true><<<grid, kTcThreads, kLayerSmem, s>>>(
      n, P.agg.p, W + L.Wl[kLayers - 1], W + L.Wo, W + L.Wt, P.h[kLayers - 1].p, nullptr, P.head.p,
      P.theta.p);
  (void)blk_row;
  edge_blocks_kernel<<<nblk(m, 128), 128, 0, s>>>(m, G.ei.p, G.ej.p, G.bij.p, G.bji.p, P.head.p,
                                                  P.fE.p, W + L.Wo, P.dvec.p, pinned, P.uv.p,
                                                  P.Gv.p);
  node_blocks_kernel<<<nblk(n, 128), 128, 0, s>>>(n, G.diag.p, G.inc_ptr.p, G.inc.p, P.uv.p,
                                                  P.theta.p, P.dvec.p, pinned, P.Gv.p);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? "" : cudaGetErrorString(e);
}

// Buffers of the inference forward; with train, also those of the training
// forward and backward (the per-edge gate and concat matrices and all
// gradients), allocated only when a training call needs them.
std::string ensure_buffers(LearnedPC &P, int n, int m, int nb, bool train) {
  const size_t N = size_t(n), M = size_t(m);
  {
    cudaError_t es[] = {
        P.fN.resize(N * kFN), P.dvec.resize(N * 3), P.fE.resize(M * kFE),
        P.h[0].resize(N * kH), P.h[1].resize(N * kH), P.h[2].resize(N * kH),
        P.h[3].resize(N * kH), P.o.resize(M * kOE), P.theta.resize(N * kON),
        P.head.resize(N * 2 * kOE), P.gate.resize(M * kH), P.uv.resize(M * 18),
        P.agg.resize(N * kH),
        P.Gv.resize(size_t(nb) * 9 + 16)};
    for (cudaError_t e : es)
      if (e != cudaSuccess) return cudaGetErrorString(e);
  }
  if (!train) return "";
  cudaError_t es[] = {
      P.cat[0].resize(N * 2 * kH), P.cat[1].resize(N * 2 * kH), P.cat[2].resize(N * 2 * kH),
      P.eX.resize(M * kEdgeIn),
      P.dh.resize(N * kH), P.dcat.resize(N * 2 * kH),
      P.dgate.resize(M * kH), P.deX.resize(M * kEdgeIn), P.dO.resize(M * kOE),
      P.dtheta.resize(N * kON), P.dGv.resize(size_t(nb) * 9), P.tmpX.resize(N * kH),
      P.y.resize(N * 3), P.r.resize(N * 3),
      P.dpart.resize((N + 255) / 256 + 1), P.dloss.resize(2),
      // dense-backward partials: largest (rows/64) x (in*out + out)
      P.parts.resize(std::max(((M + 63) / 64) * size_t(kEdgeIn * kOE + kOE),
                              ((std::max(N, M) + 63) / 64) * size_t(2 * kH * kH + kH)))};
  for (cudaError_t e : es)
    if (e != cudaSuccess) return cudaGetErrorString(e);
  return "";
}

std::string use_topology(LearnedPC &P, const HostTopology &H, DevBuf<int> &blk_row_out,
                         cudaStream_t s, bool train = true) {
  (void)blk_row_out;
  if (P.topo_n != H.n_nodes || P.topo_nb != H.n_blocks || P.topo_key != &H) {
    std::string msg = build_graph(H, P.G, s);
    if (!msg.empty()) return msg;
    P.topo_n = H.n_nodes;
    P.topo_nb = H.n_blocks;
    P.topo_key = &H;
    P.topo_train = false;
  }
  if (train && P.topo_train) return "";
  std::string msg = ensure_buffers(P, H.n_nodes, P.G.m, H.n_blocks, train);
  if (!msg.empty()) return msg;
  if (train) P.topo_train = true;
  return "";
}

// Loss and parameter gradient (accumulated into P.grad) for one system.
// probes: k device vectors of 3N floats; norms: |F w_q|^2 on the host.
std::string loss_grad_system(LearnedPC &P, const int *blk_row, const float *A,
                             const uint8_t *pinned, const float *probes, int k,
                             const std::vector<double> &norms, cudaStream_t s) {
  const Graph &G = P.G;
  std::string msg = forward(P, G, blk_row, A, pinned, s);
  if (!msg.empty()) return msg;
  cudaMemsetAsync(P.dGv.p, 0, sizeof(float) * size_t(G.nb) * 9, s);
  const int n = G.n;
  const int nparts = nblk(n, 256);
  for (int q = 0; q < k; ++q) {
    const float *w = probes + size_t(q) * 3 * n;
    spmv_kernel<<<nblk(n, 128), 128, 0, s>>>(n, G.rowptr.p, G.colidx.p, A, w, P.y.p);
    probe_residual_kernel<<<nparts, 256, 0, s>>>(n, G.rowptr.p, G.colidx.p, P.Gv.p, P.y.p, w,
                                                pinned, P.r.p, P.dpart.p);
    double wt = 1.0 / (double(k) * std::max(norms[q], 1e-300));
    accumulate_kernel<<<1, 1, 0, s>>>(nparts, P.dpart.p, wt, P.dloss.p);
    probe_grad_kernel<<<nblk(G.nb, 128), 128, 0, s>>>(G.nb, blk_row, G.colidx.p, P.r.p, P.y.p,
                                                     float(2.0 * wt), P.dGv.p);
  }
  return backward(P, G, pinned, s);
}

}  // namespace lpc
}  // namespace eolc

struct eolc_lpc : eolc::LearnedPC {
  eolc::DevBuf<int> train_blk_row;
  std::vector<std::vector<double>> sys_norms;
  cudaStream_t stream = nullptr;
};

namespace {
using namespace eolc;

std::vector<uint8_t> pin_mask(int n_nodes, const int *dofs, int n_fixed) {
  std::vector<uint8_t> m(size_t(3) * n_nodes, 0);
  for (int k = 0; k < n_fixed; ++k)
    if (dofs[k] >= 0 && dofs[k] < 3 * n_nodes) m[dofs[k]] = 1;
  return m;
}

std::vector<double> probe_norms(int n_nodes, const std::vector<uint8_t> &mask, const float *probes,
                                int k) {
  std::vector<double> out(k, 0.0);
  for (int q = 0; q < k; ++q)
    for (int i = 0; i < 3 * n_nodes; ++i)
      if (!mask[i]) out[q] += double(probes[size_t(q) * 3 * n_nodes + i]) *
                              double(probes[size_t(q) * 3 * n_nodes + i]);
  return out;
}

eolc_status ctx_mixed_matrix(eolc_ctx *ctx) {
  if (!ctx || !ctx->has_topology) return EOLC_NO_TOPOLOGY;
  if (ctx->last_precision != EOLC_PREC_MIXED) {
    ctx->err = "the context holds no FP32 matrix (assemble with EOLC_PREC_MIXED first)";
    return EOLC_BAD_ARG;
  }
  return EOLC_OK;
}

}  // namespace

extern "C" {

eolc_status eolc_lpc_create(eolc_lpc **out, int device, unsigned seed) {
  if (!out) return EOLC_BAD_ARG;
  *out = nullptr;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || device < 0 || device >= nd) return EOLC_CUDA_ERROR;
  cudaSetDevice(device);
  auto *P = new eolc_lpc();
  P->device = device;
  P->L = lpc::layout();
  lpc::init_params(*P, seed);
  const size_t np = P->L.total;
  std::vector<float> zeros(np, 0.f);
  if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess ||
      P->params.upload(P->h_params.data(), np, P->stream) != cudaSuccess ||
      P->grad.upload(zeros.data(), np, P->stream) != cudaSuccess ||
      P->m1.upload(zeros.data(), np, P->stream) != cudaSuccess ||
      P->m2.upload(zeros.data(), np, P->stream) != cudaSuccess ||
      cudaStreamSynchronize(P->stream) != cudaSuccess) {
    delete P;
    return EOLC_CUDA_ERROR;
  }
  // dense backward uses up to ~100 KB of shared memory
  cudaFuncSetAttribute(lpc::dense_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       120 * 1024);
  cudaFuncSetAttribute(lpc::dense_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       64 * 1024);
  *out = P;
  return EOLC_OK;
}

void eolc_lpc_destroy(eolc_lpc *P) {
  if (!P) return;
  cudaSetDevice(P->device);
  if (P->stream) {
    cudaStreamSynchronize(P->stream);
    cudaStreamDestroy(P->stream);
  }
  delete P;
}

int eolc_lpc_num_params(const eolc_lpc *P) { return P ? P->L.total : 0; }

eolc_status eolc_lpc_get_params(eolc_lpc *P, float *out_h) {
  if (!P || !out_h) return EOLC_BAD_ARG;
  cudaSetDevice(P->device);
  if (cudaMemcpy(out_h, P->params.p, sizeof(float) * P->L.total, cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return EOLC_CUDA_ERROR;
  return EOLC_OK;
}

eolc_status eolc_lpc_set_params(eolc_lpc *P, const float *in_h) {
  if (!P || !in_h) return EOLC_BAD_ARG;
  cudaSetDevice(P->device);
  if (cudaMemcpy(P->params.p, in_h, sizeof(float) * P->L.total, cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return EOLC_CUDA_ERROR;
  std::vector<float> zeros(P->L.total, 0.f);
  cudaMemcpy(P->m1.p, zeros.data(), sizeof(float) * P->L.total, cudaMemcpyHostToDevice);
  cudaMemcpy(P->m2.p, zeros.data(), sizeof(float) * P->L.total, cudaMemcpyHostToDevice);
  P->adam_t = 0;
  return EOLC_OK;
}

eolc_status eolc_lpc_loss_grad(eolc_lpc *P, eolc_ctx *ctx, const int *fixed_dofs_h, int n_fixed,
                               const float *probes_h, int n_probes, double *loss,
                               float *grad_h) {
  if (!P || !probes_h || n_probes <= 0 || (n_fixed > 0 && !fixed_dofs_h)) return EOLC_BAD_ARG;
  eolc_status st = ctx_mixed_matrix(ctx);
  if (st != EOLC_OK) return st;
  cudaSetDevice(P->device);
  cudaStream_t s = P->stream;
  cudaStreamSynchronize(ctx->stream);
  const int n = ctx->topo.n_nodes;
  const HostTopology *H = host_topology(ctx);
  if (!H) { P->err = ctx->err; return EOLC_CUDA_ERROR; }
  std::string msg = lpc::use_topology(*P, *H, P->train_blk_row, s);
  if (!msg.empty()) { P->err = msg; return EOLC_BAD_ARG; }
  auto mask = pin_mask(n, fixed_dofs_h, n_fixed);
  auto norms = probe_norms(n, mask, probes_h, n_probes);
  DevBuf<uint8_t> dmask;
  DevBuf<float> dprobes;
  if (dmask.upload(mask.data(), mask.size(), s) != cudaSuccess ||
      dprobes.upload(probes_h, size_t(n_probes) * 3 * n, s) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  cudaMemsetAsync(P->grad.p, 0, sizeof(float) * P->L.total, s);
  cudaMemsetAsync(P->dloss.p, 0, sizeof(double), s);
  msg = lpc::loss_grad_system(*P, ctx->topo.blk_row.p, ctx->A32.p, dmask.p, dprobes.p, n_probes,
                              norms, s);
  if (!msg.empty()) { P->err = msg; return EOLC_CUDA_ERROR; }
  double l = 0;
  if (cudaMemcpyAsync(&l, P->dloss.p, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  if (grad_h &&
      cudaMemcpyAsync(grad_h, P->grad.p, sizeof(float) * P->L.total, cudaMemcpyDeviceToHost, s) !=
          cudaSuccess)
    return EOLC_CUDA_ERROR;
  if (cudaStreamSynchronize(s) != cudaSuccess) return EOLC_CUDA_ERROR;
  if (loss) *loss = l;
  return EOLC_OK;
}

eolc_status eolc_lpc_add_system(eolc_lpc *P, eolc_ctx *ctx, const int *fixed_dofs_h, int n_fixed,
                                const float *probes_h, int n_probes) {
  if (!P || !probes_h || n_probes <= 0 || (n_fixed > 0 && !fixed_dofs_h)) return EOLC_BAD_ARG;
  eolc_status st = ctx_mixed_matrix(ctx);
  if (st != EOLC_OK) return st;
  cudaSetDevice(P->device);
  cudaStream_t s = P->stream;
  cudaStreamSynchronize(ctx->stream);
  const int n = ctx->topo.n_nodes, nb = ctx->topo.n_blocks;
  const HostTopology *H = host_topology(ctx);
  if (!H) { P->err = ctx->err; return EOLC_CUDA_ERROR; }
  if (!P->has_train_topo) {
    P->train_topo = *H;
    P->has_train_topo = true;
    if (P->train_blk_row.upload(H->blk_row.data(), nb, s) != cudaSuccess)
      return EOLC_CUDA_ERROR;
  } else if (P->train_topo.n_nodes != n || P->train_topo.n_blocks != nb ||
             P->train_topo.colidx != H->colidx) {
    P->err = "training systems must share one topology";
    return EOLC_BAD_ARG;
  }
  auto mask = pin_mask(n, fixed_dofs_h, n_fixed);
  auto *A = new DevBuf<float>();
  auto *M = new DevBuf<uint8_t>();
  auto *W = new DevBuf<float>();
  if (A->resize(size_t(nb) * 9 + 16) != cudaSuccess ||
      cudaMemcpyAsync(A->p, ctx->A32.p, sizeof(float) * size_t(nb) * 9, cudaMemcpyDeviceToDevice,
                      s) != cudaSuccess ||
      M->upload(mask.data(), mask.size(), s) != cudaSuccess ||
      W->upload(probes_h, size_t(n_probes) * 3 * n, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    delete A; delete M; delete W;
    return EOLC_CUDA_ERROR;
  }
  P->sys_A.push_back(A);
  P->sys_pin.push_back(M);
  P->sys_w.push_back(W);
  P->sys_nprobe.push_back(n_probes);
  P->sys_norms.push_back(probe_norms(n, mask, probes_h, n_probes));
  return EOLC_OK;
}

int eolc_lpc_num_systems(const eolc_lpc *P) { return P ? int(P->sys_A.size()) : 0; }

eolc_status eolc_lpc_blocks(eolc_lpc *P, eolc_ctx *ctx, const int *fixed_dofs_h, int n_fixed,
                            float *G_h) {
  if (!P || !G_h || (n_fixed > 0 && !fixed_dofs_h)) return EOLC_BAD_ARG;
  eolc_status st = ctx_mixed_matrix(ctx);
  if (st != EOLC_OK) return st;
  cudaSetDevice(P->device);
  const int n = ctx->topo.n_nodes, nb = ctx->topo.n_blocks;
  auto mask = pin_mask(n, fixed_dofs_h, n_fixed);
  DevBuf<uint8_t> pin;
  if (pin.upload(mask.data(), mask.size(), P->stream) != cudaSuccess) return EOLC_CUDA_ERROR;
  cudaStreamSynchronize(P->stream);
  const float *Gm = nullptr;
  std::string msg = learned_forward(P, ctx, pin.p, &Gm, ctx->stream);
  if (!msg.empty()) {
    P->err = msg;
    return EOLC_CUDA_ERROR;
  }
  if (cudaMemcpyAsync(G_h, Gm, sizeof(float) * size_t(nb) * 9, cudaMemcpyDeviceToHost,
                      ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return EOLC_CUDA_ERROR;
  return EOLC_OK;
}

eolc_status eolc_lpc_train(eolc_lpc *P, int epochs, float lr, unsigned seed,
                           double *epoch_loss_h) {
  if (!P || epochs <= 0 || !(lr > 0) || P->sys_A.empty()) return EOLC_BAD_ARG;
  cudaSetDevice(P->device);
  cudaStream_t s = P->stream;
  std::string msg = lpc::use_topology(*P, P->train_topo, P->train_blk_row, s);
  if (!msg.empty()) { P->err = msg; return EOLC_BAD_ARG; }
  const int ns = int(P->sys_A.size()), np = P->L.total;
  uint64_t st = 0xD1B54A32D192ED03ull ^ seed;
  std::vector<int> order(ns);
  for (int e = 0; e < epochs; ++e) {
    for (int k = 0; k < ns; ++k) order[k] = k;
    for (int k = ns - 1; k > 0; --k) {  // Fisher-Yates with a 64-bit LCG
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      int j = int((st >> 33) % uint64_t(k + 1));
      std::swap(order[k], order[j]);
    }
    cudaMemsetAsync(P->dloss.p, 0, sizeof(double), s);
    for (int k = 0; k < ns; ++k) {
      int q = order[k];
      cudaMemsetAsync(P->grad.p, 0, sizeof(float) * np, s);
      msg = lpc::loss_grad_system(*P, P->train_blk_row.p, P->sys_A[q]->p, P->sys_pin[q]->p,
                                  P->sys_w[q]->p, P->sys_nprobe[q], P->sys_norms[q], s);
      if (!msg.empty()) { P->err = msg; return EOLC_CUDA_ERROR; }
      P->adam_t += 1;
      const float b1 = 0.9f, b2 = 0.999f;
      float bc1 = 1.f - std::pow(b1, float(P->adam_t)), bc2 = 1.f - std::pow(b2, float(P->adam_t));
      lpc::adam_kernel<<<(np + 255) / 256, 256, 0, s>>>(np, P->params.p, P->grad.p, P->m1.p,
                                                        P->m2.p, lr, b1, b2, 1e-8f, bc1, bc2, 1.f);
    }
    double l = 0;
    if (cudaMemcpyAsync(&l, P->dloss.p, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return EOLC_CUDA_ERROR;
    if (epoch_loss_h) epoch_loss_h[e] = l / ns;
  }
  return EOLC_OK;
}

eolc_status eolc_lpc_clear_systems(eolc_lpc *P) {
  if (!P) return EOLC_BAD_ARG;
  for (auto *p : P->sys_A) delete p;
  for (auto *p : P->sys_pin) delete p;
  for (auto *p : P->sys_w) delete p;
  P->sys_A.clear(); P->sys_pin.clear(); P->sys_w.clear(); P->sys_nprobe.clear();
  P->sys_norms.clear();
  P->has_train_topo = false;
  return EOLC_OK;
}

const char *eolc_lpc_last_error(const eolc_lpc *P) { return P ? P->err.c_str() : "null"; }

}  // extern "C"

// Used by the solver: G = net(MDK) for the context's current FP32 matrix.
namespace eolc {
std::string learned_forward(eolc_lpc *P, eolc_ctx *ctx, const uint8_t *pinned_d,
                            const float **G_out, cudaStream_t s) {
  // the first call on a topology builds the graph (host work and uploads on
  // the network's stream, synchronised); later calls only enqueue on s
  const HostTopology *H = host_topology(ctx);
  if (!H) return ctx->err;
  std::string msg = lpc::use_topology(*P, *H, P->train_blk_row, P->stream, false);
  if (!msg.empty()) return msg;
  msg = lpc::forward_fused(*P, P->G, ctx->topo.blk_row.p, ctx->A32.p, pinned_d, s);
  if (!msg.empty()) return msg;
  *G_out = P->Gv.p;
  return "";
}
}  // namespace eolc
