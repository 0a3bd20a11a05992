// Box/point - cloth proximity tests (CD2 of Collisions.cpp:55-78 with
// btc::pointTriCollision and btc::boxTriCollision, boxTriCollision.cpp:
// 602-1224), reproducing the reference's contact set bit for bit.
//
// Exactness rules followed here:
//  * every expression is evaluated in FP64 in the reference's order, and this
//    translation unit is compiled with -fmad=false (no contraction); division
//    and square root are IEEE round-to-nearest on the device;
//  * Eigen's Vector3d reductions are ((a0 b0 + a1 b1) + a2 b2) and
//    normalized() divides by sqrt(squaredNorm) (returns the input when it is
//    0);
//  * every acos() of the reference only feeds a comparison with a constant.
//    acos is monotone, so each such test equals a comparison of its argument
//    with a boundary value that the host finds once with the host libm
//    (bisection over the doubles, then checked on a window of neighbours).
//    The device never evaluates acos;
//  * "closest so far" scans with strict < are reproduced by a lexicographic
//    (distance, index) minimum, valid because distances are finite (inputs
//    are checked for NaN/Inf first);
//  * output order: point contacts by point, then per box: vertex-face by
//    cloth vertex, corner-face by corner, edge-edge by (cloth edge in
//    createEdges order, box edge).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "internal.h"

using namespace eolc;

namespace {

constexpr int kCThreads = 256;

// ---------------------------------------------------------------- box data
// Canonical box of boxTriCollision.cpp:285-380: 8 corners + 6 face centres,
// 24 triangles, 12 edges (shared geometry: indices must match the
// reference's to name the same features).
const double kBoxVerts[14][3] = {
    {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1},
    {1, -1, 1},   {1, 1, -1},  {1, 1, 1},   {-1, 0, 0}, {1, 0, 0},
    {0, -1, 0},   {0, 1, 0},   {0, 0, -1},  {0, 0, 1}};
const int kBoxFaces[24][3] = {
    {0, 8, 2},  {1, 8, 0},  {3, 8, 1},  {2, 8, 3},  {4, 10, 0}, {5, 10, 4},
    {1, 10, 5}, {0, 10, 1}, {6, 9, 4},  {7, 9, 6},  {5, 9, 7},  {4, 9, 5},
    {2, 11, 6}, {3, 11, 2}, {7, 11, 3}, {6, 11, 7}, {1, 13, 3}, {5, 13, 1},
    {7, 13, 5}, {3, 13, 7}, {0, 12, 4}, {2, 12, 0}, {6, 12, 2}, {4, 12, 6}};
const int kBoxEdgeVerts[12][4] = {
    {0, 1, 8, 10}, {2, 0, 8, 12}, {1, 3, 8, 13}, {3, 2, 8, 11},
    {0, 4, 10, 12}, {5, 1, 10, 13}, {4, 5, 10, 9}, {6, 2, 11, 12},
    {4, 6, 9, 12}, {3, 7, 11, 13}, {7, 5, 9, 13}, {6, 7, 9, 11}};
const int kBoxVertEdges[8][3] = {{0, 1, 4}, {0, 2, 5}, {1, 3, 7}, {2, 3, 9},
                                 {4, 6, 8}, {5, 6, 10}, {7, 8, 11}, {9, 10, 11}};
const int kBoxEdgeFaces[12][2] = {{1, 7},  {0, 21}, {2, 16},  {3, 13},
                                  {4, 20}, {6, 17}, {5, 11},  {12, 22},
                                  {8, 23}, {14, 19}, {10, 18}, {9, 15}};

struct BoxDev {
  double verts[14][3];
  double faceNors[24][3];
  double vertNors[8][3];
  double edgeN[12][2][3];
  double aabbF[24][6];
  double aabbB[6];
  double par_lo, par_hi;  // acos-parallel test boundaries (global)
  double cn_hi[12];       // angleCN - angleCD > thresh  <=>  y <= cn_hi
  int soft[12];           // box edge with angle < pi/6
};

// ---- host helpers (FP64, -ffp-contract=off for this TU's host code) --------
struct H3 {
  double v[3];
};
H3 h3(double a, double b, double c) { return H3{{a, b, c}}; }
H3 hsub(const H3 &a, const H3 &b) { return h3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
H3 hadd(const H3 &a, const H3 &b) { return h3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
H3 hneg(const H3 &a) { return h3(-a.v[0], -a.v[1], -a.v[2]); }
H3 hscale(double s, const H3 &a) { return h3(s * a.v[0], s * a.v[1], s * a.v[2]); }
H3 hdiv(const H3 &a, double s) { return h3(a.v[0] / s, a.v[1] / s, a.v[2] / s); }
double hdot(const H3 &a, const H3 &b) { return (a.v[0] * b.v[0] + a.v[1] * b.v[1]) + a.v[2] * b.v[2]; }
H3 hcross(const H3 &a, const H3 &b) {
  return h3(a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
            a.v[0] * b.v[1] - a.v[1] * b.v[0]);
}
H3 hnormalized(const H3 &a) {
  double z = hdot(a, a);
  return z > 0.0 ? hdiv(a, std::sqrt(z)) : a;
}

// Order-preserving map of doubles to integers (for bisection over doubles).
int64_t dkey(double d) {
  int64_t i;
  std::memcpy(&i, &d, 8);
  return i >= 0 ? i : int64_t(0x8000000000000000ull) - i;
}
double dval(int64_t k) {
  int64_t i = k >= 0 ? k : int64_t(0x8000000000000000ull) - k;
  double d;
  std::memcpy(&d, &i, 8);
  return d;
}

// Smallest x in [lo, hi] with pred(x) true, for pred false at lo and
// monotone false -> true; returns NaN if pred(hi) is false.
template <typename F>
double first_true(F pred, double lo, double hi) {
  if (!pred(hi)) return NAN;
  if (pred(lo)) return lo;
  int64_t a = dkey(lo), b = dkey(hi);  // pred(a) false, pred(b) true
  while (b - a > 1) {
    int64_t m = a + (b - a) / 2;
    if (pred(dval(m))) b = m; else a = m;
  }
  return dval(b);
}

// Window check that the boundary is a clean monotone transition.
template <typename F>
bool clean_boundary(F pred, double boundary, bool true_above) {
  int64_t k = dkey(boundary);
  for (int d = -2000; d <= 2000; ++d) {
    double x = dval(k + d);
    if (!(x >= -1.0 && x <= 1.0)) continue;
    bool want = true_above ? (d >= 0) : (d <= 0);
    if (pred(x) != want) return false;
  }
  return true;
}

std::string build_box(const eolc_box &bx, BoxDev &B) {
  double S[4][4] = {{0}};
  S[0][0] = 0.5 * bx.dim[0];
  S[1][1] = 0.5 * bx.dim[1];
  S[2][2] = 0.5 * bx.dim[2];
  S[3][3] = 1;
  double E[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += bx.E1[k * 4 + i] * S[k][j];
      E[i][j] = s;
    }
  H3 V[14];
  for (int c = 0; c < 14; ++c) {
    for (int i = 0; i < 3; ++i) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += E[i][k] * (k < 3 ? kBoxVerts[c][k] : 1.0);
      V[c].v[i] = s;
      B.verts[c][i] = s;
    }
  }
  H3 FN[24];
  for (int k = 0; k < 24; ++k) {
    const int *f = kBoxFaces[k];
    H3 dba = hsub(V[f[1]], V[f[0]]), dac = hsub(V[f[0]], V[f[2]]);
    FN[k] = hnormalized(hcross(dba, hneg(dac)));
    for (int i = 0; i < 3; ++i) B.faceNors[k][i] = FN[k].v[i];
    for (int i = 0; i < 3; ++i) {
      double lo = V[f[0]].v[i], hi = V[f[0]].v[i];
      lo = std::min(V[f[1]].v[i], lo); lo = std::min(V[f[2]].v[i], lo);
      hi = std::max(V[f[1]].v[i], hi); hi = std::max(V[f[2]].v[i], hi);
      B.aabbF[k][i] = lo;
      B.aabbF[k][i + 3] = hi;
    }
  }
  for (int i = 0; i < 3; ++i) {
    double lo = V[0].v[i], hi = V[0].v[i];
    for (int c = 1; c < 14; ++c) { lo = std::min(lo, V[c].v[i]); hi = std::max(hi, V[c].v[i]); }
    B.aabbB[i] = lo;
    B.aabbB[i + 3] = hi;
  }
  // angle-weighted vertex normals (createVertNormals, :249-281)
  H3 vn[14];
  double ang[14];
  for (int c = 0; c < 14; ++c) { vn[c] = h3(0, 0, 0); ang[c] = 0; }
  for (int k = 0; k < 24; ++k) {
    const int *f = kBoxFaces[k];
    H3 dba = hsub(V[f[1]], V[f[0]]), dcb = hsub(V[f[2]], V[f[1]]), dac = hsub(V[f[0]], V[f[2]]);
    H3 nor = hnormalized(hcross(dba, hneg(dac)));
    dba = hnormalized(dba); dcb = hnormalized(dcb); dac = hnormalized(dac);
    double a1 = std::acos(hdot(dba, hneg(dac)));
    double a2 = std::acos(hdot(dcb, hneg(dba)));
    double a3 = std::acos(hdot(dac, hneg(dcb)));
    vn[f[0]] = hadd(vn[f[0]], hscale(a1, nor));
    vn[f[1]] = hadd(vn[f[1]], hscale(a2, nor));
    vn[f[2]] = hadd(vn[f[2]], hscale(a3, nor));
    ang[f[0]] += a1; ang[f[1]] += a2; ang[f[2]] += a3;
  }
  for (int c = 0; c < 8; ++c) {
    H3 n = hnormalized(hdiv(vn[c], ang[c]));
    for (int i = 0; i < 3; ++i) B.vertNors[c][i] = n.v[i];
  }
  const double thA = 2.0 * M_PI / 180.0;
  // Parallel tests: skip iff fabs(acos(x)) < thA || fabs(M_PI - acos(x)) < thA.
  auto p1 = [&](double x) { return std::fabs(std::acos(x)) < thA; };
  auto p2 = [&](double x) { return std::fabs(M_PI - std::acos(x)) < thA; };
  B.par_lo = first_true(p1, -1.0, 1.0);
  auto not_p2 = [&](double x) { return !p2(x); };
  double first_false2 = first_true(not_p2, -1.0, 1.0);
  B.par_hi = dval(dkey(first_false2) - 1);
  if (!clean_boundary(p1, B.par_lo, true) || !clean_boundary(p2, B.par_hi, false))
    return "host acos is not monotone near the 2-degree boundaries";
  for (int k = 0; k < 12; ++k) {
    H3 n0 = FN[kBoxEdgeFaces[k][0]], n1 = FN[kBoxEdgeFaces[k][1]];
    for (int i = 0; i < 3; ++i) { B.edgeN[k][0][i] = n0.v[i]; B.edgeN[k][1][i] = n1.v[i]; }
    double angle = std::acos(hdot(n0, n1));
    B.soft[k] = angle < M_PI / 6.0 ? 1 : 0;
    // angleCN - angleCD > thA with angleCD = acos(n1c . n1d): true for
    // y <= cn_hi (decreasing in y).
    double angleCD = std::acos(hdot(n0, n1));
    auto pc = [&](double y) { return std::acos(y) - angleCD > thA; };
    auto not_pc = [&](double y) { return !pc(y); };
    if (std::isnan(angleCD) || !pc(-1.0)) {
      B.cn_hi[k] = -2.0;  // never true on [-1, 1]
    } else {
      double ff = first_true(not_pc, -1.0, 1.0);
      B.cn_hi[k] = std::isnan(ff) ? 1.0 : dval(dkey(ff) - 1);
      if (!clean_boundary(pc, B.cn_hi[k], false))
        return "host acos is not monotone near the wedge boundary";
    }
  }
  return "";
}

// ---------------------------------------------------------------- device
__constant__ int c_box_faces[24][3];
__constant__ int c_box_edge_verts[12][4];
__constant__ int c_box_edge_faces[12][2];
__constant__ int c_box_vert_edges[8][3];
__device__ __forceinline__ int kBoxFacesD(int j, int k) { return c_box_faces[j][k]; }

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 d3(double a, double b, double c) { return D3{a, b, c}; }
__device__ __forceinline__ D3 ldv(const double *p, int i) {
  return d3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator-(D3 a) { return d3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return d3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ D3 operator/(D3 a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double dot(D3 a, D3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double norm(D3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ D3 normalized(D3 a) {
  double z = dot(a, a);
  return z > 0.0 ? a / sqrt(z) : a;
}
// std::min / std::max argument semantics
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ D3 bv(const BoxDev &B, int i) {
  return d3(B.verts[i][0], B.verts[i][1], B.verts[i][2]);
}
__device__ __forceinline__ D3 bfn(const BoxDev &B, int i) {
  return d3(B.faceNors[i][0], B.faceNors[i][1], B.faceNors[i][2]);
}

__device__ __forceinline__ bool check_aabb(const double *a, const double *b) {
  const double t = 1e-3;
  return a[3] + t >= b[0] - t && a[0] - t <= b[3] + t && a[4] + t >= b[1] - t &&
         a[1] - t <= b[4] + t && a[5] + t >= b[2] - t && a[2] - t <= b[5] + t;
}

__device__ __forceinline__ void barycentric(double &alpha, double &beta, D3 a,
                                            D3 b, D3 c, D3 p) {
  D3 v0 = b - a, v1 = c - a, v2 = p - a;
  double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
  double d20 = dot(v2, v0), d21 = dot(v2, v1);
  double denom = d00 * d11 - d01 * d01;
  beta = (d11 * d20 - d01 * d21) / denom;
  double gamma = (d00 * d21 - d01 * d20) / denom;
  alpha = 1.0 - beta - gamma;
}

// intersect_triangle3_inc (raytri.cpp:261-316), same operation order.
__device__ __forceinline__ bool raytri(D3 o, D3 d, D3 v0, D3 v1, D3 v2, double &t) {
  const double EPS = 1e-6;
  D3 e1 = v1 - v0, e2 = v2 - v0;
  D3 pv = d3(d.y * e2.z - d.z * e2.y, d.z * e2.x - d.x * e2.z, d.x * e2.y - d.y * e2.x);
  double det = e1.x * pv.x + e1.y * pv.y + e1.z * pv.z;
  D3 tv = o - v0;
  double inv_det = 1.0 / det;
  D3 qv = d3(tv.y * e1.z - tv.z * e1.y, tv.z * e1.x - tv.x * e1.z, tv.x * e1.y - tv.y * e1.x);
  double u, v;
  if (det > EPS) {
    u = tv.x * pv.x + tv.y * pv.y + tv.z * pv.z;
    if (u < EPS || u > det + -EPS) return false;
    v = d.x * qv.x + d.y * qv.y + d.z * qv.z;
    if (v < EPS || u + v > det + -EPS) return false;
  } else if (det < -EPS) {
    u = tv.x * pv.x + tv.y * pv.y + tv.z * pv.z;
    if (u > -EPS || u < det - -EPS) return false;
    v = d.x * qv.x + d.y * qv.y + d.z * qv.z;
    if (v > -EPS || u + v < det - -EPS) return false;
  } else {
    return false;
  }
  t = (e2.x * qv.x + e2.y * qv.y + e2.z * qv.z) * inv_det;
  return true;
}

// intersect_square (boxTriCollision.cpp:550-600)
__device__ __forceinline__ bool intersect_square(D3 x0, D3 dx, D3 xa, D3 xb, D3 xc,
                                                 double &t) {
  D3 xd = xa + 2.0 * (xc - xa);
  D3 xe = xb + 2.0 * (xc - xb);
  if (raytri(x0, dx, xa, xb, xc, t)) return true;
  if (raytri(x0, dx, xb, xd, xc, t)) return true;
  if (raytri(x0, dx, xd, xe, xc, t)) return true;
  if (raytri(x0, dx, xe, xa, xc, t)) return true;
  t = -1.0;
  return false;
}

__device__ __forceinline__ void put3(double *d, D3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }

__device__ __forceinline__ void blank(eolc_contact &c) {
  double *dp = &c.dist;  // dist and the eight 3-vectors: 25 doubles
  for (int k = 0; k < 25; ++k) dp[k] = 0.0;
  c.count1 = 0; c.count2 = 0;
  c.verts1[0] = c.verts1[1] = c.verts1[2] = 0;
  c.verts2[0] = c.verts2[1] = c.verts2[2] = 0;
  c.tri1 = -1; c.tri2 = -1;
  c.edge1[0] = c.edge1[1] = c.edge1[2] = 0;
  c.n_edge1 = 0;
  c.edge2 = -1;
  c.source = 0;
}

// ---- per-call preparation ----------------------------------------------------
// v2 = x + perturbation, face normals of v2 and of x, non-finite check.
__global__ void perturb_kernel(int n, const double *x, const double *rnd,
                               double thr, double *v2, int *bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  double xi = x[i];
  if (!isfinite(xi)) atomicExch(bad, 1);
  double r = rnd[i] * thr * 1e-3;  // dis(gen)*threshold*1e-3
  v2[i] = xi + r;
}

// createFaceNormals (:233-247) for the perturbed positions and the face
// normals of createEdges (:187-200, unperturbed, (xb-xa) x (xc-xa)).
__global__ void face_normals_kernel(int nf, const int *tri, const double *v2,
                                    const double *x, double *fn2, double *fn0) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nf) return;
  int a = tri[3 * k], b = tri[3 * k + 1], c = tri[3 * k + 2];
  D3 xa = ldv(v2, a), xb = ldv(v2, b), xc = ldv(v2, c);
  D3 dba = xb - xa, dac = xa - xc;
  put3(fn2 + 3 * k, normalized(cross(dba, -dac)));
  D3 ya = ldv(x, a), yb = ldv(x, b), yc = ldv(x, c);
  put3(fn0 + 3 * k, normalized(cross(yb - ya, yc - ya)));
}

// AABB of the perturbed cloth (build_AABB_B): per-CTA partials.
__global__ void aabb_partial_kernel(int n, const double *v2, double *part) {
  __shared__ double s[6][kCThreads];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int c = 0; c < 3; ++c) {
      double v = v2[3 * i + c];
      lo[c] = smin(lo[c], v);
      hi[c] = smax(hi[c], v);
    }
  for (int c = 0; c < 3; ++c) { s[c][threadIdx.x] = lo[c]; s[c + 3][threadIdx.x] = hi[c]; }
  __syncthreads();
  for (int o = kCThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 3; ++c) {
        s[c][threadIdx.x] = smin(s[c][threadIdx.x], s[c][threadIdx.x + o]);
        s[c + 3][threadIdx.x] = smax(s[c + 3][threadIdx.x], s[c + 3][threadIdx.x + o]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void aabb_final_kernel(int nparts, const double *part, double *aabb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double b[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < nparts; ++k)
    for (int c = 0; c < 3; ++c) {
      b[c] = smin(b[c], part[6 * k + c]);
      b[c + 3] = smax(b[c + 3], part[6 * k + c + 3]);
    }
  for (int c = 0; c < 6; ++c) aabb[c] = b[c];
}

// ---- closest-face search for a query point (corner / obstacle point) -----
// Candidate test of the Vertex1-Triangle2 loops (:771-845, :1142-1213).
__device__ __forceinline__ bool vf_candidate(D3 x1, D3 nor1, const int *tri,
                                             const double *v2, const double *fn2,
                                             int j2, double thr, double &dist) {
  int a = tri[3 * j2], b = tri[3 * j2 + 1], c = tri[3 * j2 + 2];
  D3 x2a = ldv(v2, a), x2b = ldv(v2, b), x2c = ldv(v2, c);
  D3 nor2 = ldv(fn2, j2);
  if (dot(nor1, nor2) < 0.0) nor2 = -nor2;
  D3 dx = x1 - x2a;
  double proj = dot(dx, nor2);
  if (proj < 0.0) return false;
  D3 x2 = x1 - proj * nor2;
  dx = x2 - x1;
  dist = norm(dx);
  if (dist > 5.0 * thr) return false;
  double u, v;
  barycentric(u, v, x2a, x2b, x2c, x1);
  double w = 1.0 - u - v;
  if (u < 0.0 || 1.0 < u || v < 0.0 || 1.0 < v || w < 0.0 || 1.0 < w) return false;
  return true;
}

// Lexicographic (dist, j2) minimum per query; one grid-stride pass per
// query, CTA partials then a final pick.
__global__ void vf_argmin_kernel(int nq, const double *qpos, const double *qnor,
                                 const double *aabb2, int nf, const int *tri,
                                 const double *v2, const double *fn2, double thr,
                                 double *part_d, int *part_j) {
  __shared__ double sd[kCThreads];
  __shared__ int sj[kCThreads];
  int qi = blockIdx.y;
  if (qi >= nq) return;
  double best_d = INFINITY;
  int best_j = -1;
  D3 xq = ldv(qpos, qi);
  double pt[6] = {xq.x, xq.y, xq.z, xq.x, xq.y, xq.z};
  // AABB test of the query point against the whole cloth (check_AABB)
  if (check_aabb(pt, aabb2)) {
    D3 x1 = xq, nor1 = ldv(qnor, qi);
    for (int j2 = blockIdx.x * blockDim.x + threadIdx.x; j2 < nf; j2 += gridDim.x * blockDim.x) {
      double d;
      if (vf_candidate(x1, nor1, tri, v2, fn2, j2, thr, d)) {
        if (best_j < 0 || d < best_d) { best_d = d; best_j = j2; }
      }
    }
  }
  sd[threadIdx.x] = best_d;
  sj[threadIdx.x] = best_j;
  __syncthreads();
  for (int o = kCThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      double d2 = sd[threadIdx.x + o];
      int j2 = sj[threadIdx.x + o];
      int j1 = sj[threadIdx.x];
      if (j2 >= 0 && (j1 < 0 || d2 < sd[threadIdx.x] ||
                      (d2 == sd[threadIdx.x] && j2 < j1))) {
        sd[threadIdx.x] = d2;
        sj[threadIdx.x] = j2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part_d[qi * gridDim.x + blockIdx.x] = sd[0];
    part_j[qi * gridDim.x + blockIdx.x] = sj[0];
  }
}

__global__ void vf_pick_kernel(int nq, int nparts, const double *part_d,
                               const int *part_j, int *best) {
  int qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= nq) return;
  double bd = INFINITY;
  int bj = -1;
  for (int k = 0; k < nparts; ++k) {
    int j = part_j[qi * nparts + k];
    double d = part_d[qi * nparts + k];
    if (j >= 0 && (bj < 0 || d < bd || (d == bd && j < bj))) { bd = d; bj = j; }
  }
  best[qi] = bj;
}

// ---- vertex2 - triangle1 (cloth vertex inside box), :675-764 ---------------
__global__ void v2f1_kernel(int nv, int nf, const double *v2, const BoxDev *Bp,
                            double thr, int *best_face) {
  int i2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i2 >= nv) return;
  const BoxDev &B = *Bp;
  D3 x2 = ldv(v2, i2);
  double pt[6] = {x2.x, x2.y, x2.z, x2.x, x2.y, x2.z};
  int best = -1;
  if (check_aabb(pt, B.aabbB)) {
    bool inside = true;
    for (int j1 = 0; j1 < 24; ++j1) {
      D3 x1a = bv(B, kBoxFacesD(j1, 0));
      if (dot(bfn(B, j1), x2 - x1a) > 0.0) { inside = false; break; }
    }
    if (inside) {
      double bd = 0;
      for (int j1 = 0; j1 < 24; ++j1) {
        D3 x1a = bv(B, kBoxFacesD(j1, 0)), x1b = bv(B, kBoxFacesD(j1, 1)),
           x1c = bv(B, kBoxFacesD(j1, 2));
        D3 nor1 = bfn(B, j1);
        D3 dx = x2 - x1a;
        double proj = dot(nor1, dx);
        if (proj > 0.0) continue;
        D3 x1 = x2 - proj * nor1;
        dx = x2 - x1;
        double dist = norm(dx);
        if (dist > 5.0 * thr) continue;
        double u, v;
        barycentric(u, v, x1a, x1b, x1c, x1);
        double w = 1.0 - u - v;
        if (u < 0.0 || 1.0 < u || v < 0.0 || 1.0 < v || w < 0.0 || 1.0 < w) continue;
        if (best < 0 || dist < bd) { best = j1; bd = dist; }
      }
    }
  }
  best_face[i2] = best;
  (void)nf;
}

// ---- edge2 - edge1 (:849-1017) ----------------------------------------------
struct EEOut {
  double dist, u1, u2;
  D3 nor1, nor, x1, x2, tan1;
};

// The full edge-edge test for cloth edge k2 and box edge k1; true when the
// reference pushes a contact.
__device__ bool ee_test(const int4 e2, const double *v2, const double *fn0,
                        const BoxDev &B, int k1, double thr, EEOut *out) {
  D3 x2a = ldv(v2, e2.x), x2b = ldv(v2, e2.y);
  D3 dx2 = x2b - x2a;
  double len2 = norm(dx2);
  D3 n0 = ldv(fn0, e2.z);
  D3 n1 = e2.w >= 0 ? ldv(fn0, e2.w) : d3(0.0, 0.0, 0.0);
  D3 nor2 = normalized(n0 + n1);
  double ab[6] = {smin(x2b.x, x2a.x), smin(x2b.y, x2a.y), smin(x2b.z, x2a.z),
                  smax(x2b.x, x2a.x), smax(x2b.y, x2a.y), smax(x2b.z, x2a.z)};
  if (B.soft[k1]) return false;
  if (!check_aabb(B.aabbF[c_box_edge_faces[k1][0]], ab) &&
      !check_aabb(B.aabbF[c_box_edge_faces[k1][1]], ab))
    return false;
  D3 x1a = bv(B, c_box_edge_verts[k1][0]), x1b = bv(B, c_box_edge_verts[k1][1]);
  D3 dx1 = x1b - x1a;
  double len1 = norm(dx1);
  D3 tan1 = dx1 / len1;
  // fabs(acos(c)) < 2deg || fabs(pi - acos(c)) < 2deg, as boundaries on c
  double c = dot(tan1, nor2);
  if ((c >= B.par_lo && c <= 1.0) || (c <= B.par_hi && c >= -1.0)) return false;
  c = dot(tan1, dx2) / len2;
  if ((c >= B.par_lo && c <= 1.0) || (c <= B.par_hi && c >= -1.0)) return false;
  D3 nor = normalized(cross(dx1, dx2));
  D3 x1c = bv(B, c_box_edge_verts[k1][2]), x1d = bv(B, c_box_edge_verts[k1][3]);
  D3 n1c = d3(B.edgeN[k1][0][0], B.edgeN[k1][0][1], B.edgeN[k1][0][2]);
  D3 n1d = d3(B.edgeN[k1][1][0], B.edgeN[k1][1][1], B.edgeN[k1][1][2]);
  D3 nor1 = normalized(n1c + n1d);
  if (dot(nor, nor1) < 0.0) nor = -nor;
  // angleCN - angleCD > 2deg, as a boundary on n1c . nor
  double y = dot(n1c, nor);
  if (y <= B.cn_hi[k1] && y >= -1.0) return false;
  double u2c, u2d;
  bool i2c = intersect_square(x2a, dx2, x1a, x1b, x1c, u2c);
  bool i2d = intersect_square(x2a, dx2, x1b, x1a, x1d, u2d);
  i2c = i2c && (0.0 <= u2c && u2c <= 1.0);
  i2d = i2d && (0.0 <= u2d && u2d <= 1.0);
  // lineline (:507-526)
  double u1, u2;
  {
    D3 B2B1 = x2b - x2a, A1B1 = x1a - x2a, A2A1 = x1b - x1a;
    D3 AxB = cross(A2A1, B2B1);
    double nA = dot(cross(B2B1, A1B1), AxB);
    double nB = dot(cross(A2A1, A1B1), AxB);
    double d = dot(cross(A2A1, B2B1), AxB);
    u1 = nA / d;
    u2 = nB / d;
  }
  double thresh1 = 1.0 * thr / len1;
  double thresh2 = 1.0 * thr / len2;
  if (u1 < -thresh1 || u1 > 1.0 + thresh1 || u2 < -thresh2 || u2 > 1.0 + thresh2)
    return false;
  D3 x1, x2, dx;
  if (i2c && i2d) {
    x1 = (1.0 - u1) * x1a + u1 * x1b;
    x2 = (1.0 - u2) * x2a + u2 * x2b;
  } else if (i2c || i2d) {
    D3 base = i2c ? x1a : x1b;
    D3 nn = i2c ? n1c : n1d;
    double uu = i2c ? u2c : u2d;
    dx = x2a - base;
    if (dot(dx, nn) < 0.0) u2 = smax(0.0, smin(uu, u2));
    else u2 = smax(uu, smin(1.0, u2));
    x2 = (1.0 - u2) * x2a + u2 * x2b;
    // linepoint (:528-537)
    D3 AP = x2 - x1a, AB = x1b - x1a;
    u1 = dot(AP, AB) / dot(AB, AB);
    x1 = (1.0 - u1) * x1a + u1 * x1b;
  } else {
    return false;
  }
  if (u1 < -thresh1 || u1 > 1.0 + thresh1 || u2 < -thresh2 || u2 > 1.0 + thresh2)
    return false;
  dx = x2 - x1;
  double th = 2.0 * thr;
  if (dot(dx, dx) > th * th) return false;
  if (out) {
    out->dist = norm(dx);
    out->u1 = u1;
    out->u2 = u2;
    out->nor1 = nor1;
    out->nor = nor;
    out->x1 = x1;
    out->x2 = x2;
    out->tan1 = tan1;
  }
  return true;
}

__global__ void ee_mask_kernel(int ne, const int4 *edges, const double *v2,
                               const double *fn0, const BoxDev *Bp, double thr,
                               int *info) {
  int k2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (k2 >= ne) return;
  int4 e = edges[k2];
  int mask = 0;
  for (int k1 = 0; k1 < 12; ++k1)
    if (ee_test(e, v2, fn0, *Bp, k1, thr, nullptr)) mask |= 1 << k1;
  info[k2] = mask;
}

// ---- compaction (exclusive scan of per-item contact counts) ----------------
enum SegKind { kSegPoint = 0, kSegV2F1 = 1, kSegV1F2 = 2, kSegEE = 3 };
struct Seg {
  int kind, start, count, box, qbase;
};
constexpr int kMaxSegs = 64;
struct SegTable {
  int n;
  Seg s[kMaxSegs];
};

__device__ __forceinline__ int seg_of(const SegTable &T, int item) {
  int k = 0;
  while (k + 1 < T.n && item >= T.s[k + 1].start) ++k;
  return k;
}

__device__ __forceinline__ int item_count(const SegTable &T, const int *info, int item) {
  int k = seg_of(T, item);
  int v = info[item];
  return T.s[k].kind == kSegEE ? __popc(v) : (v >= 0 ? 1 : 0);
}

constexpr int kScanItems = 1024;  // items per CTA in the scan

__global__ void scan_reduce_kernel(int L, SegTable T, const int *info, int *bsum) {
  __shared__ int s[kCThreads];
  int base = blockIdx.x * kScanItems;
  int acc = 0;
  for (int k = threadIdx.x; k < kScanItems && base + k < L; k += kCThreads)
    acc += item_count(T, info, base + k);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kCThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = s[0];
}

__global__ void scan_blocks_kernel(int nb, const int *bsum, int *boff, int *total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int run = 0;
  for (int k = 0; k < nb; ++k) { boff[k] = run; run += bsum[k]; }
  *total = run;
}

__global__ void scan_items_kernel(int L, SegTable T, const int *info,
                                  const int *boff, int *off) {
  __shared__ int s[kScanItems];
  int base = blockIdx.x * kScanItems;
  for (int k = threadIdx.x; k < kScanItems; k += kCThreads)
    s[k] = base + k < L ? item_count(T, info, base + k) : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = boff[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k) { int c = s[k]; s[k] = run; run += c; }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kScanItems && base + k < L; k += kCThreads)
    off[base + k] = s[k];
}

// ---- contact writers ----------------------------------------------------------
struct WriteArgs {
  const int *tri;
  const int4 *edges;
  const double *v2, *fn2, *fn0;
  const double *qpos, *qnor;
  const BoxDev *boxes;
  const int *info, *off;
  double thr;
  int nf;
  int capacity;
  eolc_contact *out;
};

__device__ void finish_contact(eolc_contact &c, double thr) {
  double snap = 0.1 * thr;
  for (int i = 0; i < 3; ++i) c.pos1_[i] = c.pos1[i] - snap * c.nor1[i];
}

__global__ void write_kernel(int L, SegTable T, WriteArgs W) {
  int item = blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= L) return;
  int v = W.info[item];
  const Seg &S = T.s[seg_of(T, item)];
  int o = W.off[item];
  int local = item - S.start;
  if (S.kind == kSegPoint || S.kind == kSegV1F2) {
    if (v < 0 || o >= W.capacity) return;
    int qi = S.qbase + local;
    D3 x1 = ldv(W.qpos, qi), nor1 = ldv(W.qnor, qi);
    int j2 = v;
    int a = W.tri[3 * j2], b = W.tri[3 * j2 + 1], cc = W.tri[3 * j2 + 2];
    D3 x2a = ldv(W.v2, a), x2b = ldv(W.v2, b), x2c = ldv(W.v2, cc);
    D3 nor2 = ldv(W.fn2, j2);
    if (dot(nor1, nor2) < 0.0) nor2 = -nor2;
    D3 dx = x1 - x2a;
    double proj = dot(dx, nor2);
    D3 x2 = x1 - proj * nor2;
    dx = x2 - x1;
    double dist = norm(dx);
    double u, vv;
    barycentric(u, vv, x2a, x2b, x2c, x1);
    double w = 1.0 - u - vv;
    eolc_contact c;
    blank(c);
    c.dist = dist;
    put3(c.nor1, nor1); put3(c.nor2, nor2); put3(c.pos1, x1); put3(c.pos2, x2);
    c.count1 = 1; c.count2 = 3;
    c.verts1[0] = local; c.verts1[1] = -1; c.verts1[2] = -1;
    c.verts2[0] = a; c.verts2[1] = b; c.verts2[2] = cc;
    c.weights1[0] = 1.0;
    c.weights2[0] = u; c.weights2[1] = vv; c.weights2[2] = w;
    c.tri2 = j2;
    if (S.kind == kSegV1F2) {
      c.edge1[0] = c_box_vert_edges[local][0];
      c.edge1[1] = c_box_vert_edges[local][1];
      c.edge1[2] = c_box_vert_edges[local][2];
      c.n_edge1 = 3;
    }
    c.source = S.kind == kSegPoint ? 0 : 1 + S.box;
    finish_contact(c, W.thr);
    W.out[o] = c;
  } else if (S.kind == kSegV2F1) {
    if (v < 0 || o >= W.capacity) return;
    const BoxDev &B = W.boxes[S.box];
    int i2 = local, j1 = v;
    D3 x2 = ldv(W.v2, i2);
    D3 x1a = bv(B, c_box_faces[j1][0]), x1b = bv(B, c_box_faces[j1][1]),
       x1c = bv(B, c_box_faces[j1][2]);
    D3 nor1 = bfn(B, j1);
    D3 dx = x2 - x1a;
    double proj = dot(nor1, dx);
    D3 x1 = x2 - proj * nor1;
    dx = x2 - x1;
    double dist = norm(dx);
    double u, vv;
    barycentric(u, vv, x1a, x1b, x1c, x1);
    double w = 1.0 - u - vv;
    // the cloth normal is read at the vertex index (:731)
    D3 nor2 = i2 < W.nf ? ldv(W.fn2, i2) : d3(NAN, NAN, NAN);
    if (dot(nor2, nor1) < 0.0) nor2 = -nor2;
    eolc_contact c;
    blank(c);
    c.dist = dist;
    put3(c.nor1, nor1); put3(c.nor2, nor2); put3(c.pos1, x1); put3(c.pos2, x2);
    c.count1 = 3; c.count2 = 1;
    c.verts1[0] = c_box_faces[j1][0]; c.verts1[1] = c_box_faces[j1][1];
    c.verts1[2] = c_box_faces[j1][2];
    c.verts2[0] = i2; c.verts2[1] = -1; c.verts2[2] = -1;
    c.weights1[0] = u; c.weights1[1] = vv; c.weights1[2] = w;
    c.weights2[0] = 1.0;
    c.tri1 = j1;
    c.source = 1 + S.box;
    finish_contact(c, W.thr);
    W.out[o] = c;
  } else {  // edge-edge
    if (v == 0) return;
    const BoxDev &B = W.boxes[S.box];
    int k2 = local;
    int4 e = W.edges[k2];
    int rank = 0;
    for (int k1 = 0; k1 < 12; ++k1) {
      if (!(v & (1 << k1))) continue;
      int oo = o + rank++;
      if (oo >= W.capacity) continue;
      EEOut r;
      ee_test(e, W.v2, W.fn0, B, k1, W.thr, &r);
      eolc_contact c;
      blank(c);
      c.dist = r.dist;
      put3(c.nor1, r.nor1); put3(c.nor2, r.nor); put3(c.pos1, r.x1); put3(c.pos2, r.x2);
      c.count1 = 2; c.count2 = 2;
      c.verts1[0] = c_box_edge_verts[k1][0]; c.verts1[1] = c_box_edge_verts[k1][1];
      c.verts1[2] = -1;
      c.verts2[0] = e.x; c.verts2[1] = e.y; c.verts2[2] = -1;
      c.weights1[0] = 1.0 - r.u1; c.weights1[1] = r.u1;
      c.weights2[0] = 1.0 - r.u2; c.weights2[1] = r.u2;
      c.edge1[0] = k1; c.n_edge1 = 1;
      c.edge2 = k2;
      put3(c.edge_dir, r.tan1);
      c.source = 1 + S.box;
      finish_contact(c, W.thr);
      W.out[oo] = c;
    }
  }
}

__global__ void copy_best_kernel(int n, const int *best, int *info) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) info[i] = best[i];
}

// createEdges (:141-231), topology part, is built on the device by
// build_edges_device (topology_gpu.cu): per edge (verts(0), verts(1), face0,
// face1 or -1) in the reference's order.

}  // namespace

// ---------------------------------------------------------------------------
namespace eolc {

struct CollideWork {
  int n_nodes = -1, n_tri = -1, n_edges = 0;
  EdgeScratch *es = nullptr;  // scratch of the device edge-list build
  DevBuf<int4> edges;
  DevBuf<double> rnd, x, v2, fn2, fn0, aabb_part, aabb, qpos, qnor, part_d;
  DevBuf<int> part_j, best_q, info, bsum, boff, off, scalars;
  DevBuf<BoxDev> boxes;
  DevBuf<eolc_contact> out;
};

void free_collide_work(CollideWork *w) {
  if (w) free_edge_scratch(w->es);
  delete w;
}

}  // namespace eolc

extern "C" eolc_status eolc_cd2(eolc_ctx *ctx, const double *x_h,
                                const eolc_box *boxes, int n_boxes,
                                const double *points_h, const double *normals_h,
                                int n_points, double threshold,
                                eolc_contact *out_h, int capacity, int *n_out) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!ctx->has_topology) { ctx->err = "no topology set"; return EOLC_NO_TOPOLOGY; }
  if (!x_h || n_boxes < 0 || n_points < 0 || capacity < 0 || !n_out ||
      (n_boxes > 0 && !boxes) || (n_points > 0 && (!points_h || !normals_h)) ||
      (capacity > 0 && !out_h)) {
    ctx->err = "bad collision arguments";
    return EOLC_BAD_ARG;
  }
  if (1 + 3 * n_boxes > kMaxSegs) { ctx->err = "too many boxes"; return EOLC_BAD_ARG; }
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  // the mesh nodes (a topology with EOL nodes adds Eulerian block rows,
  // which CD2 does not see: Collisions.cpp:55-78 packs the mesh nodes)
  const int N = ctx->topo.n_real, F = ctx->topo.n_tri;
  if (!ctx->cd_work) ctx->cd_work = new CollideWork();
  CollideWork &W = *ctx->cd_work;
#define CK(expr)                                                        \
  do {                                                                  \
    cudaError_t e_ = (expr);                                            \
    if (e_ != cudaSuccess) {                                            \
      ctx->err = std::string(#expr ": ") + cudaGetErrorString(e_);      \
      return EOLC_CUDA_ERROR;                                           \
    }                                                                   \
  } while (0)
  static bool tables_set = false;
  if (!tables_set) {
    CK(cudaMemcpyToSymbol(c_box_faces, kBoxFaces, sizeof(kBoxFaces)));
    CK(cudaMemcpyToSymbol(c_box_edge_verts, kBoxEdgeVerts, sizeof(kBoxEdgeVerts)));
    CK(cudaMemcpyToSymbol(c_box_edge_faces, kBoxEdgeFaces, sizeof(kBoxEdgeFaces)));
    CK(cudaMemcpyToSymbol(c_box_vert_edges, kBoxVertEdges, sizeof(kBoxVertEdges)));
    tables_set = true;
  }
  if (W.n_nodes != N || W.n_tri != F) {
    // topology-only parts: cloth edges and the perturbation sequence
    // (std::mt19937 seeded 1, uniform_real_distribution(-1, 1), three draws
    // per vertex, :648-659)
    const std::string emsg = build_edges_device(W.es, ctx->topo.tri.p, F, W.edges, W.n_edges, s,
                                                ctx->launches);
    if (!emsg.empty()) {
      ctx->err = emsg;
      return EOLC_CUDA_ERROR;
    }
    std::vector<double> rnd(size_t(3) * N);
    std::mt19937 gen;
    std::uniform_real_distribution<> dis(-1.0, 1.0);
    gen.seed(1);
    for (size_t k = 0; k < rnd.size(); ++k) rnd[k] = dis(gen);
    CK(W.rnd.upload(rnd.data(), rnd.size(), s));
    CK(cudaStreamSynchronize(s));
    W.n_nodes = N;
    W.n_tri = F;
  }
  const int E = W.n_edges;
  // host box data
  std::vector<BoxDev> hb(std::max(1, n_boxes));
  for (int b = 0; b < n_boxes; ++b) {
    std::string msg = build_box(boxes[b], hb[b]);
    if (!msg.empty()) { ctx->err = msg; return EOLC_BAD_ARG; }
  }
  // queries: obstacle points, then 8 corners per box
  int nq = n_points + 8 * n_boxes;
  std::vector<double> qp(size_t(3) * std::max(1, nq)), qn(size_t(3) * std::max(1, nq));
  for (int i = 0; i < n_points; ++i)
    for (int c = 0; c < 3; ++c) {
      qp[3 * i + c] = points_h[3 * i + c];
      qn[3 * i + c] = normals_h[3 * i + c];
    }
  for (int b = 0; b < n_boxes; ++b)
    for (int i = 0; i < 8; ++i)
      for (int c = 0; c < 3; ++c) {
        qp[3 * (n_points + 8 * b + i) + c] = hb[b].verts[i][c];
        qn[3 * (n_points + 8 * b + i) + c] = hb[b].vertNors[i][c];
      }
  // segments (reference output order)
  SegTable T;
  T.n = 0;
  int L = 0;
  T.s[T.n++] = Seg{kSegPoint, L, n_points, -1, 0};
  L += n_points;
  for (int b = 0; b < n_boxes; ++b) {
    T.s[T.n++] = Seg{kSegV2F1, L, N, b, 0}; L += N;
    T.s[T.n++] = Seg{kSegV1F2, L, 8, b, n_points + 8 * b}; L += 8;
    T.s[T.n++] = Seg{kSegEE, L, E, b, 0}; L += E;
  }
  const int vf_parts = std::max(1, std::min(64, (F + kCThreads - 1) / kCThreads));
  const int n_scan = (std::max(L, 1) + kScanItems - 1) / kScanItems;
  CK(W.x.upload(x_h, size_t(3) * N, s));
  CK(W.v2.resize(size_t(3) * N));
  CK(W.fn2.resize(size_t(3) * F));
  CK(W.fn0.resize(size_t(3) * F));
  CK(W.aabb_part.resize(6 * 64));
  CK(W.aabb.resize(6));
  CK(W.qpos.upload(qp.data(), qp.size(), s));
  CK(W.qnor.upload(qn.data(), qn.size(), s));
  CK(W.part_d.resize(size_t(std::max(1, nq)) * vf_parts));
  CK(W.part_j.resize(size_t(std::max(1, nq)) * vf_parts));
  CK(W.best_q.resize(std::max(1, nq)));
  CK(W.info.resize(std::max(1, L)));
  CK(W.off.resize(std::max(1, L)));
  CK(W.bsum.resize(n_scan));
  CK(W.boff.resize(n_scan));
  CK(W.scalars.resize(2));
  CK(W.boxes.upload(hb.data(), hb.size(), s));
  CK(W.out.resize(std::max(1, capacity)));
  CK(cudaMemsetAsync(W.scalars.p, 0, 2 * sizeof(int), s));
  // perturbation, normals, cloth AABB
  perturb_kernel<<<(3 * N + 255) / 256, 256, 0, s>>>(N, W.x.p, W.rnd.p, threshold,
                                                     W.v2.p, W.scalars.p + 1);
  face_normals_kernel<<<(F + 255) / 256, 256, 0, s>>>(F, ctx->topo.tri.p, W.v2.p, W.x.p,
                                                      W.fn2.p, W.fn0.p);
  int aparts = std::max(1, std::min(64, (N + kCThreads - 1) / kCThreads));
  aabb_partial_kernel<<<aparts, kCThreads, 0, s>>>(N, W.v2.p, W.aabb_part.p);
  aabb_final_kernel<<<1, 32, 0, s>>>(aparts, W.aabb_part.p, W.aabb.p);
  ctx->launches += 4;
  // vertex-face queries (points and box corners) against the cloth faces
  if (nq > 0) {
    dim3 grid(vf_parts, nq);
    vf_argmin_kernel<<<grid, kCThreads, 0, s>>>(nq, W.qpos.p, W.qnor.p, W.aabb.p, F,
                                                ctx->topo.tri.p, W.v2.p, W.fn2.p,
                                                threshold, W.part_d.p, W.part_j.p);
    vf_pick_kernel<<<(nq + 127) / 128, 128, 0, s>>>(nq, vf_parts, W.part_d.p, W.part_j.p,
                                                    W.best_q.p);
    ctx->launches += 2;
  }
  // item info in output order
  if (n_points > 0) {
    copy_best_kernel<<<(n_points + 127) / 128, 128, 0, s>>>(n_points, W.best_q.p, W.info.p);
    ctx->launches += 1;
  }
  for (int b = 0; b < n_boxes; ++b) {
    const Seg &sv = T.s[1 + 3 * b], &sc = T.s[2 + 3 * b], &se = T.s[3 + 3 * b];
    v2f1_kernel<<<(N + 127) / 128, 128, 0, s>>>(N, F, W.v2.p, W.boxes.p + b, threshold,
                                                W.info.p + sv.start);
    copy_best_kernel<<<1, 32, 0, s>>>(8, W.best_q.p + n_points + 8 * b, W.info.p + sc.start);
    ee_mask_kernel<<<(E + 127) / 128, 128, 0, s>>>(E, W.edges.p, W.v2.p, W.fn0.p,
                                                   W.boxes.p + b, threshold,
                                                   W.info.p + se.start);
    ctx->launches += 3;
  }
  if (L > 0) {
    scan_reduce_kernel<<<n_scan, kCThreads, 0, s>>>(L, T, W.info.p, W.bsum.p);
    scan_blocks_kernel<<<1, 32, 0, s>>>(n_scan, W.bsum.p, W.boff.p, W.scalars.p);
    scan_items_kernel<<<n_scan, kCThreads, 0, s>>>(L, T, W.info.p, W.boff.p, W.off.p);
    WriteArgs wa;
    wa.tri = ctx->topo.tri.p;
    wa.edges = W.edges.p;
    wa.v2 = W.v2.p; wa.fn2 = W.fn2.p; wa.fn0 = W.fn0.p;
    wa.qpos = W.qpos.p; wa.qnor = W.qnor.p;
    wa.boxes = W.boxes.p;
    wa.info = W.info.p; wa.off = W.off.p;
    wa.thr = threshold;
    wa.nf = F;
    wa.capacity = capacity;
    wa.out = W.out.p;
    write_kernel<<<(L + 127) / 128, 128, 0, s>>>(L, T, wa);
    ctx->launches += 4;
  }
  CK(cudaGetLastError());
  int sc[2] = {0, 0};
  CK(cudaMemcpyAsync(sc, W.scalars.p, sizeof(sc), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (sc[1]) { ctx->err = "non-finite cloth position"; return EOLC_NONFINITE; }
  *n_out = sc[0];
  int ncopy = std::min(sc[0], capacity);
  if (ncopy > 0) {
    CK(cudaMemcpyAsync(out_h, W.out.p, sizeof(eolc_contact) * ncopy, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
#undef CK
  if (sc[0] > capacity) {
    ctx->err = "contact buffer too small";
    return EOLC_CAPACITY;
  }
  return EOLC_OK;
}

extern "C" eolc_status eolc_edge_list(eolc_ctx *ctx, int *edges_h, int capacity, int *n_edges) {
  if (!ctx) return EOLC_BAD_ARG;
  if (!ctx->has_topology) { ctx->err = "no topology set"; return EOLC_NO_TOPOLOGY; }
  if (!n_edges || capacity < 0 || (capacity > 0 && !edges_h)) {
    ctx->err = "bad edge-list arguments";
    return EOLC_BAD_ARG;
  }
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  if (!ctx->cd_work) ctx->cd_work = new CollideWork();
  CollideWork &W = *ctx->cd_work;
  if (W.n_tri != ctx->topo.n_tri) {
    const std::string msg = build_edges_device(W.es, ctx->topo.tri.p, ctx->topo.n_tri, W.edges,
                                               W.n_edges, s, ctx->launches);
    if (!msg.empty()) { ctx->err = msg; return EOLC_CUDA_ERROR; }
  }
  *n_edges = W.n_edges;
  if (capacity < W.n_edges) { ctx->err = "edge list capacity too small"; return EOLC_CAPACITY; }
  if (W.n_edges > 0) {
    cudaError_t e = cudaMemcpyAsync(edges_h, W.edges.p, sizeof(int4) * W.n_edges,
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return EOLC_CUDA_ERROR; }
  }
  return EOLC_OK;
}
