// OBJ frame export from the device state: the two files that
// BrenderManager::exportBrender (BrenderManager.cpp:34-84) opens per frame and
// Cloth::exportBrender (Cloth.cpp:535-590) fills,
//   <dir>/<frame %06d>_Cloth2D.obj   material space: v = (u, 0), vn = +z
//   <dir>/<frame %06d>_Cloth3D.obj   world space: v = x, vn = node normals
// both with vt = u and 1-based "f a/a/a b/b/b c/c/c" faces, byte for byte.
//
// The text is generated on the GPU, one line per thread:
//   obj_normals_kernel  node normals (ArcSim normal<WS>, geometry.cpp:302-316)
//                       in FP64 without contraction, stored as float like the
//                       reference's norBuf (Cloth.cpp:150-165);
//   obj_len_kernel      the length of every line, summed per CTA;
//   obj_scan_kernel     offsets of the CTAs' text (one CTA);
//   obj_write_kernel    each CTA formats its lines into shared memory at the
//                       16-byte phase of its output offset and stores them
//                       with aligned 16-byte stores (bytes at the two ends).
// The host adds the three header lines and writes the files; one
// device-to-host copy carries both files' text.
//
// Positions, texture coordinates and normals go through float as in the
// reference's posBuf/texBuf/norBuf; the 2D file's v line prints the double
// material coordinates.  Its third value is the literal 0 in the reference,
// passed as an int to "%f"; it is written here as 0.000000.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "objfmt.cuh"

using namespace eolc;
using namespace eolc::obj;

namespace {

constexpr int kLineThreads = 256;  // lines per CTA
constexpr int kScanThreads = 1024;

struct ObjArgs {
  int N, F;
  const double *x, *X;
  const int *tri;
  const float *nrm;     // 3N node normals (float)
  long long la;         // lines of the 2D file: 3N + F
  long long lb;         // first line of the 3D file: la rounded up to kLineThreads
  long long lines;      // lb + 3N + F
};

__device__ __forceinline__ char *at(char *o, int n) { return o ? o + n : nullptr; }

// Three "%f" numbers separated by blanks after a prefix, then '\n'.
__device__ __forceinline__ int put_f3(const char *prefix, double a, double b, double c,
                                      int count, char *o, bool &bad) {
  int n = put_str(prefix, o);
  const double v[3] = {a, b, c};
  for (int k = 0; k < count; ++k) {
    if (k) {
      if (o) o[n] = ' ';
      ++n;
    }
    const int m = fmt_f6(v[k], at(o, n));
    if (m < 0) {
      bad = true;
      return n;
    }
    n += m;
  }
  if (o) o[n] = '\n';
  return n + 1;
}

// Line `line` of the concatenated text (nullptr: length only).
__device__ int format_line(const ObjArgs &a, long long line, char *o, bool &bad) {
  int file = 0;
  long long l = line;
  if (line >= a.lb) {
    file = 1;
    l = line - a.lb;
  } else if (line >= a.la) {
    return 0;  // padding between the files
  }
  const long long N = a.N;
  if (l < N) {  // v
    const int i = int(l);
    if (file == 0) return put_f3("v ", a.X[2 * i], a.X[2 * i + 1], 0.0, 3, o, bad);
    return put_f3("v ", double(float(a.x[3 * i])), double(float(a.x[3 * i + 1])),
                  double(float(a.x[3 * i + 2])), 3, o, bad);
  }
  if (l < 2 * N) {  // vt
    const int i = int(l - N);
    return put_f3("vt ", double(float(a.X[2 * i])), double(float(a.X[2 * i + 1])), 0.0, 2, o,
                  bad);
  }
  if (l < 3 * N) {  // vn
    const int i = int(l - 2 * N);
    if (file == 0) return put_str("vn 0.000000 0.000000 1.000000\n", o);
    return put_f3("vn ", double(a.nrm[3 * i]), double(a.nrm[3 * i + 1]),
                  double(a.nrm[3 * i + 2]), 3, o, bad);
  }
  const int f = int(l - 3 * N);  // f a/a/a b/b/b c/c/c
  int n = put_str("f ", o);
  for (int k = 0; k < 3; ++k) {
    const int id = a.tri[3 * f + k] + 1;
    for (int r = 0; r < 3; ++r) {
      n += fmt_i(id, at(o, n));
      if (o) o[n] = r < 2 ? '/' : (k < 2 ? ' ' : '\n');
      ++n;
    }
  }
  return n;
}

// ArcSim normal<WS>(node): n = sum over incident faces of
// cross(e1, e2) * (1 / ((2 |e1|^2) |e2|^2)), e1 = x[v_{j+1}] - x[v],
// e2 = x[v_{j+2}] - x[v]; then n * (1 / |n|), or 0 when |n| = 0.  Faces in
// mesh order, each operation in the reference's order (vectors.hpp:49-54:
// dot accumulates from 0, u / a = u * (1 / a)).  Compiled with -fmad=false.
__global__ void obj_normals_kernel(int N, const double *x, const int *tri, const int *nf_ptr,
                                   const int *nf_list, float *nrm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
  double nx = 0, ny = 0, nz = 0;
  for (int k = nf_ptr[i]; k < nf_ptr[i + 1]; ++k) {
    const int code = nf_list[k];
    const int f = code >> 2, j = code & 3;
    const int a = tri[3 * f + (j + 1) % 3], b = tri[3 * f + (j + 2) % 3];
    const double e1x = x[3 * a] - px, e1y = x[3 * a + 1] - py, e1z = x[3 * a + 2] - pz;
    const double e2x = x[3 * b] - px, e2y = x[3 * b + 1] - py, e2z = x[3 * b + 2] - pz;
    const double cx = e1y * e2z - e1z * e2y;
    const double cy = e1z * e2x - e1x * e2z;
    const double cz = e1x * e2y - e1y * e2x;
    double n1 = 0;
    n1 += e1x * e1x;
    n1 += e1y * e1y;
    n1 += e1z * e1z;
    double n2 = 0;
    n2 += e2x * e2x;
    n2 += e2y * e2y;
    n2 += e2z * e2z;
    const double inv = 1 / (2 * n1 * n2);
    nx = nx + cx * inv;
    ny = ny + cy * inv;
    nz = nz + cz * inv;
  }
  double m2 = 0;
  m2 += nx * nx;
  m2 += ny * ny;
  m2 += nz * nz;
  const double m = sqrt(m2);
  if (m == 0) {
    nx = ny = nz = 0;
  } else {
    const double inv = 1 / m;
    nx = nx * inv;
    ny = ny * inv;
    nz = nz * inv;
  }
  nrm[3 * i] = float(nx);
  nrm[3 * i + 1] = float(ny);
  nrm[3 * i + 2] = float(nz);
}

// Sum of a CTA's per-thread values (kLineThreads threads).
__device__ __forceinline__ int cta_sum(int v, int *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = v;
  __syncthreads();
  int t = 0;
  for (int k = 0; k < kLineThreads / 32; ++k) t += red[k];
  return t;
}

__global__ void __launch_bounds__(kLineThreads) obj_len_kernel(ObjArgs a, int *blk_len,
                                                               int *err) {
  __shared__ int red[kLineThreads / 32];
  const long long line = (long long)blockIdx.x * kLineThreads + threadIdx.x;
  bool bad = false;
  const int len = line < a.lines ? format_line(a, line, nullptr, bad) : 0;
  if (bad) atomicOr(err, 1);
  const int t = cta_sum(len, red);
  if (threadIdx.x == 0) blk_len[blockIdx.x] = t;
}

// Exclusive scan of the CTA lengths; off[nb] = total bytes.
__global__ void __launch_bounds__(kScanThreads) obj_scan_kernel(const int *blk_len, int nb,
                                                                long long *off) {
  __shared__ long long warp_tot[kScanThreads / 32];
  __shared__ long long carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += kScanThreads) {
    const int k = base + threadIdx.x;
    const long long v = k < nb ? blk_len[k] : 0;
    long long inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const long long u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
      long long t = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += u;
      }
      warp_tot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    const long long before = carry + (w ? warp_tot[w - 1] : 0);
    if (k < nb) off[k] = before + inc - v;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry = before + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) off[nb] = carry;
}

__global__ void __launch_bounds__(kLineThreads) obj_write_kernel(ObjArgs a, const long long *off,
                                                                 char *text) {
  __shared__ int red[kLineThreads / 32];
  __shared__ alignas(16) char stage[16 + kLineThreads * kMaxLine];
  const long long line = (long long)blockIdx.x * kLineThreads + threadIdx.x;
  bool bad = false;
  const int len = line < a.lines ? format_line(a, line, nullptr, bad) : 0;
  // exclusive prefix of the lengths within the CTA
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = len;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) red[w] = inc;
  __syncthreads();
  int before = 0, total = 0;
  for (int k = 0; k < kLineThreads / 32; ++k) {
    before += k < w ? red[k] : 0;
    total += red[k];
  }
  const long long g0 = off[blockIdx.x];
  const int phase = int(g0 & 15);
  if (len > 0) format_line(a, line, stage + phase + before + inc - len, bad);
  __syncthreads();
  // global bytes [g0, g0 + total) live at stage[phase + (p - g0)]
  const long long g1 = g0 + total;
  const long long a0 = (g0 + 15) & ~15LL, a1 = g1 & ~15LL;
  if (a0 < a1) {
    const int nv = int((a1 - a0) >> 4);
    const uint4 *src = reinterpret_cast<const uint4 *>(stage + phase + (a0 - g0));
    uint4 *dst = reinterpret_cast<uint4 *>(text + a0);
    for (int k = threadIdx.x; k < nv; k += kLineThreads) dst[k] = src[k];
    const int head = int(a0 - g0), tail = int(g1 - a1);
    if (threadIdx.x < head) text[g0 + threadIdx.x] = stage[phase + threadIdx.x];
    if (threadIdx.x >= 32 && threadIdx.x - 32 < tail)
      text[a1 + threadIdx.x - 32] = stage[phase + (a1 - g0) + threadIdx.x - 32];
  } else {
    for (int k = threadIdx.x; k < total; k += kLineThreads) text[g0 + k] = stage[phase + k];
  }
}

}  // namespace

namespace eolc {

struct ExportWork {
  DevBuf<float> nrm;
  DevBuf<int> blk_len, err;
  DevBuf<long long> off;
  DevBuf<char> text;
  char *host = nullptr;  // pinned copy of the text
  size_t host_cap = 0;
  ~ExportWork() {
    if (host) cudaFreeHost(host);
  }
};

void free_export_work(ExportWork *w) { delete w; }

}  // namespace eolc

namespace {

#define EX_CHECK(expr)                                                  \
  do {                                                                  \
    cudaError_t e_ = (expr);                                            \
    if (e_ != cudaSuccess) {                                            \
      ctx->err = std::string(#expr ": ") + cudaGetErrorString(e_);      \
      return EOLC_CUDA_ERROR;                                           \
    }                                                                   \
  } while (0)

std::string header(int frame, double time, const char *name) {
  char buf[160];
  snprintf(buf, sizeof(buf), "# frame %06d \n# time %f \n# name %s \n", frame, time, name);
  return buf;
}

// Generates both files' text on the device and copies it to the pinned host
// buffer.  len[0], len[1]: body bytes of the 2D and 3D files (no header).
eolc_status generate(eolc_ctx *ctx, size_t len[2]) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!ctx->has_topology) {
    ctx->err = "no topology set";
    return EOLC_NO_TOPOLOGY;
  }
  if (refuse_eol(ctx) != EOLC_OK) return EOLC_BAD_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  if (!ctx->ex_work) ctx->ex_work = new ExportWork();
  ExportWork &W = *ctx->ex_work;
  const DevTopology &T = ctx->topo;
  const int N = T.n_nodes, F = T.n_tri;
  ObjArgs a;
  a.N = N;
  a.F = F;
  a.x = ctx->x.p;
  a.X = ctx->X.p;
  a.tri = T.tri.p;
  a.la = 3LL * N + F;
  a.lb = (a.la + kLineThreads - 1) / kLineThreads * kLineThreads;
  a.lines = a.lb + a.la;
  const long long nbl = (a.lines + kLineThreads - 1) / kLineThreads;
  if (nbl > 0x7fffffffLL) {
    ctx->err = "mesh too large to export";
    return EOLC_BAD_ARG;
  }
  const int nb = int(nbl);
  if (nb == 0) {
    len[0] = len[1] = 0;
    return EOLC_OK;
  }
  EX_CHECK(W.nrm.resize(size_t(3) * (N > 0 ? N : 1)));
  EX_CHECK(W.blk_len.resize(size_t(nb)));
  EX_CHECK(W.off.resize(size_t(nb) + 1));
  EX_CHECK(W.err.resize(1));
  a.nrm = W.nrm.p;
  EX_CHECK(cudaMemsetAsync(W.err.p, 0, sizeof(int), s));
  if (N > 0) {
    obj_normals_kernel<<<(N + 255) / 256, 256, 0, s>>>(N, ctx->x.p, T.tri.p, T.nf_ptr.p,
                                                       T.nf_list.p, W.nrm.p);
    ++ctx->launches;
  }
  obj_len_kernel<<<nb, kLineThreads, 0, s>>>(a, W.blk_len.p, W.err.p);
  obj_scan_kernel<<<1, kScanThreads, 0, s>>>(W.blk_len.p, nb, W.off.p);
  ctx->launches += 2;
  EX_CHECK(cudaGetLastError());
  long long tot[2];
  int bad = 0;
  const long long split_blk = a.lb / kLineThreads;  // first CTA of the 3D file
  EX_CHECK(cudaMemcpyAsync(&tot[0], W.off.p + split_blk, sizeof(long long),
                           cudaMemcpyDeviceToHost, s));
  EX_CHECK(cudaMemcpyAsync(&tot[1], W.off.p + nb, sizeof(long long), cudaMemcpyDeviceToHost, s));
  EX_CHECK(cudaMemcpyAsync(&bad, W.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  EX_CHECK(cudaStreamSynchronize(s));
  if (bad) {
    ctx->err = "a coordinate of magnitude >= 2^63 cannot be written with %f here";
    return EOLC_BAD_ARG;
  }
  const size_t total = size_t(tot[1]);
  if (W.text.n < total + 16) EX_CHECK(W.text.resize(total + 16));
  obj_write_kernel<<<nb, kLineThreads, 0, s>>>(a, W.off.p, W.text.p);
  ++ctx->launches;
  EX_CHECK(cudaGetLastError());
  if (W.host_cap < total + 1) {
    if (W.host) cudaFreeHost(W.host);
    W.host = nullptr;
    W.host_cap = 0;
    EX_CHECK(cudaHostAlloc(&W.host, total + 1, cudaHostAllocDefault));
    W.host_cap = total + 1;
  }
  if (total) EX_CHECK(cudaMemcpyAsync(W.host, W.text.p, total, cudaMemcpyDeviceToHost, s));
  EX_CHECK(cudaStreamSynchronize(s));
  len[0] = size_t(tot[0]);
  len[1] = total - len[0];
  return EOLC_OK;
}

const char *kNames[2] = {"Cloth2D", "Cloth3D"};

}  // namespace

extern "C" eolc_status eolc_export_obj_text(eolc_ctx *ctx, int frame, double time, char *buf,
                                            size_t capacity, size_t len[2]) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!len || (capacity > 0 && !buf)) {
    ctx->err = "bad export arguments";
    return EOLC_BAD_ARG;
  }
  size_t body[2];
  eolc_status st = generate(ctx, body);
  if (st != EOLC_OK) return st;
  const std::string h0 = header(frame, time, kNames[0]), h1 = header(frame, time, kNames[1]);
  len[0] = h0.size() + body[0];
  len[1] = h1.size() + body[1];
  if (!buf) return EOLC_OK;
  if (capacity < len[0] + len[1]) {
    ctx->err = "export buffer too small";
    return EOLC_CAPACITY;
  }
  const char *t = ctx->ex_work->host;
  char *o = buf;
  memcpy(o, h0.data(), h0.size());
  o += h0.size();
  memcpy(o, t, body[0]);
  o += body[0];
  memcpy(o, h1.data(), h1.size());
  o += h1.size();
  memcpy(o, t + body[0], body[1]);
  return EOLC_OK;
}

extern "C" eolc_status eolc_export_obj(eolc_ctx *ctx, const char *dir, int frame,
                                       double time) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!dir) {
    ctx->err = "null export directory";
    return EOLC_BAD_ARG;
  }
  size_t body[2];
  eolc_status st = generate(ctx, body);
  if (st != EOLC_OK) return st;
  const char *t = ctx->ex_work->host;
  const char *part[2] = {t, t + body[0]};
  for (int k = 0; k < 2; ++k) {
    std::string path(dir);
    char name[64];
    snprintf(name, sizeof(name), "/%06d_%s.obj", frame, kNames[k]);
    path += name;
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) {
      ctx->err = "cannot open " + path + ": " + strerror(errno);
      return EOLC_IO_ERROR;
    }
    const std::string h = header(frame, time, kNames[k]);
    const bool ok = fwrite(h.data(), 1, h.size(), fp) == h.size() &&
                    fwrite(part[k], 1, body[k], fp) == body[k];
    const bool closed = fclose(fp) == 0;
    if (!ok || !closed) {
      ctx->err = "write failed: " + path;
      return EOLC_IO_ERROR;
    }
  }
  return EOLC_OK;
}
