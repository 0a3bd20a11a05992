// Device build of the topology: the fixed BSR pattern (node pairs sharing a
// triangle or a hinge, columns ascending), each block's element
// contributions in the reference's triplet insertion order (faces ascending,
// then hinges ascending: fillxMI / fillxxMI / fillxB / fillxxB, summed by
// setFromTriplets, Forces.cpp:331-930) and node -> face incidence.  Built on
// every topology change, so per-step refreshes after host remeshing stay on
// the GPU (the reference rebuilds and re-sorts its triplets every step,
// Forces.cpp:925-929).
//
// No global sort: one thread per node builds its own row.
//   topo_check_kernel     index range and degenerate elements (error bits)
//   topo_count_kernel     faces and hinges incident to each node (atomics)
//   scan (3 kernels)      offsets of the incidence lists
//   topo_scatter_kernel   (element << 2 | local vertex) into the lists
//   topo_sort_kernel      each node's lists in element order (the atomics'
//                         order is arbitrary; this makes it deterministic)
//   topo_row_kernel       pass 0: each row's distinct columns (the nodes of
//                         its faces and hinges, by repeated minimum); pass 1: colidx,
//                         blk_row, diag, and each block's contributions in the
//                         reference's insertion order — faces ascending, then
//                         hinges ascending — with the same codes as the host.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <string>

#include "internal.h"

namespace eolc {

namespace {

constexpr int kT = 256;

enum : int {
  kErrRange = 1,
  kErrDegenerateTri = 2,
  kErrDegenerateHinge = 4,
  kErrIsolated = 8
};

__global__ void topo_check_kernel(int N, const int *__restrict__ tri, int n_tri,
                                  const int *__restrict__ hinge, int n_hinge, int *err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int e = 0;
  if (k < n_tri) {
    const int a = tri[3 * k], b = tri[3 * k + 1], c = tri[3 * k + 2];
    if (a < 0 || a >= N || b < 0 || b >= N || c < 0 || c >= N) e |= kErrRange;
    if (a == b || b == c || a == c) e |= kErrDegenerateTri;
  } else if (k < n_tri + n_hinge) {
    const int *v = hinge + 4 * (k - n_tri);
    for (int p = 0; p < 4; ++p) {
      if (v[p] < 0 || v[p] >= N) e |= kErrRange;
      for (int q = p + 1; q < 4; ++q)
        if (v[p] == v[q]) e |= kErrDegenerateHinge;
    }
  }
  if (e) atomicOr(err, e);
}

__global__ void topo_count_kernel(const int *__restrict__ tri, int n_tri,
                                  const int *__restrict__ hinge, int n_hinge, int *fcnt,
                                  int *hcnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_tri) {
    for (int a = 0; a < 3; ++a) atomicAdd(fcnt + tri[3 * k + a], 1);
  } else if (k < n_tri + n_hinge) {
    const int e = k - n_tri;
    for (int a = 0; a < 4; ++a) atomicAdd(hcnt + hinge[4 * e + a], 1);
  }
}

// ---- exclusive scan of n ints into out[0..n] (out[n] = total) -------------
__device__ __forceinline__ int block_scan_incl(int v, int *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    int t = lane < kT / 32 ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    if (lane < kT / 32) sh[lane] = t;
  }
  __syncthreads();
  return v + (w ? sh[w - 1] : 0);
}

__global__ void scan_blocks_kernel(const int *__restrict__ in, int n, int *__restrict__ out,
                                   int *__restrict__ bsum) {
  __shared__ int sh[kT / 32];
  const int k = blockIdx.x * kT + threadIdx.x;
  const int v = k < n ? in[k] : 0;
  const int inc = block_scan_incl(v, sh);
  if (k < n) out[k] = inc - v;
  if (threadIdx.x == kT - 1) bsum[blockIdx.x] = inc;
}

// one CTA: exclusive scan of the block sums in place; bsum[nb] = total
__global__ void scan_sums_kernel(int *bsum, int nb) {
  __shared__ int sh[kT / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += kT) {
    const int k = base + threadIdx.x;
    const int v = k < nb ? bsum[k] : 0;
    const int inc = block_scan_incl(v, sh);
    const int c = carry;
    if (k < nb) bsum[k] = c + inc - v;
    __syncthreads();
    if (threadIdx.x == kT - 1) carry = c + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void scan_add_kernel(int *__restrict__ out, int n, const int *__restrict__ bsum) {
  const int k = blockIdx.x * kT + threadIdx.x;
  if (k < n) out[k] += bsum[blockIdx.x];
  if (k == 0) out[n] = bsum[gridDim.x];
}

__global__ void topo_scatter_kernel(const int *__restrict__ tri, int n_tri,
                                    const int *__restrict__ hinge, int n_hinge, int *fcur,
                                    int *hcur, int *flist, int *hlist) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_tri) {
    for (int a = 0; a < 3; ++a) flist[atomicAdd(fcur + tri[3 * k + a], 1)] = (k << 2) | a;
  } else if (k < n_tri + n_hinge) {
    const int e = k - n_tri;
    for (int a = 0; a < 4; ++a) hlist[atomicAdd(hcur + hinge[4 * e + a], 1)] = (e << 2) | a;
  }
}

__device__ void insertion_sort(int *v, int n) {
  for (int i = 1; i < n; ++i) {
    const int x = v[i];
    int j = i - 1;
    while (j >= 0 && v[j] > x) {
      v[j + 1] = v[j];
      --j;
    }
    v[j + 1] = x;
  }
}

__global__ void topo_sort_kernel(int N, const int *__restrict__ fptr, int *flist,
                                 const int *__restrict__ hptr, int *hlist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  insertion_sort(flist + fptr[i], fptr[i + 1] - fptr[i]);
  insertion_sort(hlist + hptr[i], hptr[i + 1] - hptr[i]);
}

// The smallest node above `last` among the nodes of row i's faces and
// hinges (INT_MAX: none).  Walking it from last = -1 lists the row's distinct
// columns in ascending order without a per-thread buffer.
__device__ __forceinline__ int next_column(int i, int last, const int *__restrict__ tri,
                                           const int *__restrict__ hinge,
                                           const int *__restrict__ fptr,
                                           const int *__restrict__ flist,
                                           const int *__restrict__ hptr,
                                           const int *__restrict__ hlist) {
  int best = INT_MAX;
  for (int q = fptr[i]; q < fptr[i + 1]; ++q) {
    const int t = flist[q] >> 2;
    for (int b = 0; b < 3; ++b) {
      const int c = tri[3 * t + b];
      if (c > last && c < best) best = c;
    }
  }
  for (int q = hptr[i]; q < hptr[i + 1]; ++q) {
    const int e = hlist[q] >> 2;
    for (int b = 0; b < 4; ++b) {
      const int c = hinge[4 * e + b];
      if (c > last && c < best) best = c;
    }
  }
  return best;
}

// pass 0: ncol[i], ncon[i]; pass 1: the row's blocks and contributions.
__global__ void __launch_bounds__(kT)
topo_row_kernel(int N, int pass, const int *__restrict__ tri, const int *__restrict__ hinge,
                const int *__restrict__ fptr, const int *__restrict__ flist,
                const int *__restrict__ hptr, const int *__restrict__ hlist, int *ncol,
                int *ncon, const int *__restrict__ rowptr, const int *__restrict__ cbase,
                int *colidx, int *blk_row, int *diag, int *cptr, int *contrib, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (pass == 0) {
    int u = 0;
    for (int j = next_column(i, -1, tri, hinge, fptr, flist, hptr, hlist); j != INT_MAX;
         j = next_column(i, j, tri, hinge, fptr, flist, hptr, hlist))
      ++u;
    if (u == 0) atomicOr(err, kErrIsolated);
    ncol[i] = u;
    ncon[i] = 3 * (fptr[i + 1] - fptr[i]) + 4 * (hptr[i + 1] - hptr[i]);
    return;
  }
  int pos = cbase[i], blk = rowptr[i], dg = -1;
  for (int j = next_column(i, -1, tri, hinge, fptr, flist, hptr, hlist); j != INT_MAX;
       j = next_column(i, j, tri, hinge, fptr, flist, hptr, hlist), ++blk) {
    colidx[blk] = j;
    blk_row[blk] = i;
    if (j == i) dg = blk;
    cptr[blk] = pos;
    for (int q = fptr[i]; q < fptr[i + 1]; ++q) {
      const int t = flist[q] >> 2, a = flist[q] & 3;
      for (int b = 0; b < 3; ++b)
        if (tri[3 * t + b] == j) contrib[pos++] = contrib_code(t, false, a, b);
    }
    for (int q = hptr[i]; q < hptr[i + 1]; ++q) {
      const int e = hlist[q] >> 2, a = hlist[q] & 3;
      for (int b = 0; b < 4; ++b)
        if (hinge[4 * e + b] == j) contrib[pos++] = contrib_code(e, true, a, b);
    }
  }
  diag[i] = dg;
  if (dg < 0) atomicOr(err, kErrIsolated);
  if (i == N - 1) cptr[rowptr[N]] = pos;
}

int grid(long long n) { return int((n + kT - 1) / kT); }

}  // namespace

struct TopoScratch {
  DevBuf<int> fcnt, hcnt, hptr, hcur, fcur, hlist, ncol, ncon, cbase, bsum, err;
};

void free_topo_scratch(TopoScratch *w) { delete w; }

namespace {

// exclusive scan of n ints (device) into out[0..n]
void scan(const int *in, int n, int *out, DevBuf<int> &bsum, cudaStream_t s) {
  const int nb = grid(n);
  scan_blocks_kernel<<<nb, kT, 0, s>>>(in, n, out, bsum.p);
  scan_sums_kernel<<<1, kT, 0, s>>>(bsum.p, nb);
  scan_add_kernel<<<nb, kT, 0, s>>>(out, n, bsum.p);
}

}  // namespace

std::string build_topology_device(TopoScratch *&w, int N, const int *tri_d, int n_tri,
                                  const int *hinge_d, int n_hinge, DevTopology &T,
                                  cudaStream_t s, long long &launches) {
  if (N <= 0 || n_tri <= 0 || n_hinge < 0) return "bad sizes";
  if (int64_t(n_tri) + n_hinge >= (int64_t(1) << 26)) return "too many elements";
  if (!w) w = new TopoScratch();
  TopoScratch &W = *w;
#define TG(expr)                                                   \
  do {                                                             \
    cudaError_t e_ = (expr);                                       \
    if (e_ != cudaSuccess) return std::string(#expr ": ") + cudaGetErrorString(e_); \
  } while (0)
  const int nb_max = grid(N + 1) + 1;
  TG(W.fcnt.resize(N));
  TG(W.hcnt.resize(N));
  TG(W.fcur.resize(N + 1));
  TG(W.hcur.resize(N + 1));
  TG(W.hptr.resize(N + 1));
  TG(W.ncol.resize(N));
  TG(W.ncon.resize(N));
  TG(W.cbase.resize(N + 1));
  TG(W.bsum.resize(nb_max + 1));
  TG(W.err.resize(1));
  TG(W.hlist.resize(size_t(4) * std::max(1, n_hinge)));
  TG(T.nf_ptr.resize(N + 1));
  TG(T.nf_list.resize(size_t(3) * n_tri));
  TG(T.rowptr.resize(N + 1));
  TG(T.diag.resize(N));
  TG(cudaMemsetAsync(W.fcnt.p, 0, sizeof(int) * N, s));
  TG(cudaMemsetAsync(W.hcnt.p, 0, sizeof(int) * N, s));
  TG(cudaMemsetAsync(W.err.p, 0, sizeof(int), s));
  const int ne = n_tri + n_hinge;
  topo_check_kernel<<<grid(ne), kT, 0, s>>>(N, tri_d, n_tri, hinge_d, n_hinge, W.err.p);
  int err = 0;
  TG(cudaMemcpyAsync(&err, W.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  TG(cudaStreamSynchronize(s));
  launches += 1;
  if (err & kErrRange) return "element index out of range";
  if (err & kErrDegenerateTri) return "degenerate triangle";
  if (err & kErrDegenerateHinge) return "degenerate hinge";
  topo_count_kernel<<<grid(ne), kT, 0, s>>>(tri_d, n_tri, hinge_d, n_hinge, W.fcnt.p, W.hcnt.p);
  scan(W.fcnt.p, N, T.nf_ptr.p, W.bsum, s);
  scan(W.hcnt.p, N, W.hptr.p, W.bsum, s);
  TG(cudaMemcpyAsync(W.fcur.p, T.nf_ptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToDevice, s));
  TG(cudaMemcpyAsync(W.hcur.p, W.hptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToDevice, s));
  topo_scatter_kernel<<<grid(ne), kT, 0, s>>>(tri_d, n_tri, hinge_d, n_hinge, W.fcur.p, W.hcur.p,
                                               T.nf_list.p, W.hlist.p);
  topo_sort_kernel<<<grid(N), kT, 0, s>>>(N, T.nf_ptr.p, T.nf_list.p, W.hptr.p, W.hlist.p);
  topo_row_kernel<<<grid(N), kT, 0, s>>>(N, 0, tri_d, hinge_d, T.nf_ptr.p, T.nf_list.p, W.hptr.p,
                                          W.hlist.p, W.ncol.p, W.ncon.p, nullptr, nullptr,
                                          nullptr, nullptr, nullptr, nullptr, nullptr, W.err.p);
  scan(W.ncol.p, N, T.rowptr.p, W.bsum, s);
  scan(W.ncon.p, N, W.cbase.p, W.bsum, s);
  int tot[2] = {0, 0};
  TG(cudaMemcpyAsync(&tot[0], T.rowptr.p + N, sizeof(int), cudaMemcpyDeviceToHost, s));
  TG(cudaMemcpyAsync(&tot[1], W.cbase.p + N, sizeof(int), cudaMemcpyDeviceToHost, s));
  TG(cudaMemcpyAsync(&err, W.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  TG(cudaStreamSynchronize(s));
  launches += 2 + 3 * 4 + 1;
  if (err & kErrIsolated) return "node without any element";
  const int nblk = tot[0], ncon = tot[1];
  TG(T.colidx.resize(nblk));
  TG(T.blk_row.resize(nblk));
  TG(T.cptr.resize(size_t(nblk) + 1));
  TG(T.contrib.resize(ncon));
  topo_row_kernel<<<grid(N), kT, 0, s>>>(N, 1, tri_d, hinge_d, T.nf_ptr.p, T.nf_list.p, W.hptr.p,
                                          W.hlist.p, W.ncol.p, W.ncon.p, T.rowptr.p, W.cbase.p,
                                          T.colidx.p, T.blk_row.p, T.diag.p, T.cptr.p,
                                          T.contrib.p, W.err.p);
  TG(cudaMemcpyAsync(&err, W.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  TG(cudaStreamSynchronize(s));
  launches += 1;
  if (err & kErrIsolated) return "node without any element";
  T.n_nodes = N;
  T.n_tri = n_tri;
  T.n_hinge = n_hinge;
  T.n_blocks = nblk;
#undef TG
  return "";
}

}  // namespace eolc
