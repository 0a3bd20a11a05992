// Oracle restatement of CD2 / btc::boxTriCollision / btc::pointTriCollision
// (test infrastructure; see oracle.h).  Control flow, output order and the
// floating-point evaluation order follow src/boxTriCollision.cpp and
// src/Collisions.cpp:55-78 so that the contact set is reproduced exactly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <random>
#include <vector>

#include "oracle.h"
#include "vec3.h"

using orc::V3;
using orc::cross;
using orc::dot;
using orc::norm;
using orc::normalized;

namespace {

// Canonical box (boxTriCollision.cpp:285-380): 8 corners + 6 face centres,
// 24 triangles, 12 edges.  These tables are the box's geometry, which any
// implementation has to share to produce the same indices.
const double kBoxVerts[14][3] = {
    {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1},
    {1, -1, 1},   {1, 1, -1},  {1, 1, 1},   {-1, 0, 0}, {1, 0, 0},
    {0, -1, 0},   {0, 1, 0},   {0, 0, -1},  {0, 0, 1}};
const int kBoxFaces[24][3] = {
    {0, 8, 2},   {1, 8, 0},   {3, 8, 1},   {2, 8, 3},   {4, 10, 0},
    {5, 10, 4},  {1, 10, 5},  {0, 10, 1},  {6, 9, 4},   {7, 9, 6},
    {5, 9, 7},   {4, 9, 5},   {2, 11, 6},  {3, 11, 2},  {7, 11, 3},
    {6, 11, 7},  {1, 13, 3},  {5, 13, 1},  {7, 13, 5},  {3, 13, 7},
    {0, 12, 4},  {2, 12, 0},  {6, 12, 2},  {4, 12, 6}};
const int kBoxEdgeVerts[12][4] = {
    {0, 1, 8, 10}, {2, 0, 8, 12}, {1, 3, 8, 13},  {3, 2, 8, 11},
    {0, 4, 10, 12}, {5, 1, 10, 13}, {4, 5, 10, 9}, {6, 2, 11, 12},
    {4, 6, 9, 12}, {3, 7, 11, 13}, {7, 5, 9, 13}, {6, 7, 9, 11}};
const int kBoxVertEdges[8][3] = {{0, 1, 4}, {0, 2, 5},  {1, 3, 7},
                                 {2, 3, 9}, {4, 6, 8},  {5, 6, 10},
                                 {7, 8, 11}, {9, 10, 11}};
const int kBoxEdgeFaces[12][2] = {{1, 7},   {0, 21},  {2, 16}, {3, 13},
                                  {4, 20},  {6, 17},  {5, 11}, {12, 22},
                                  {8, 23},  {14, 19}, {10, 18}, {9, 15}};

struct Edge {
  int verts[4];
  int faces[2];
  bool internal;
  double angle;
  V3 normals[2];
};

V3 col(const std::vector<double> &m, int i) {
  return orc::mk(m[3 * i], m[3 * i + 1], m[3 * i + 2]);
}

// createFaceNormals (boxTriCollision.cpp:233-247)
std::vector<V3> face_normals(const int *faces, int nf,
                             const std::vector<double> &verts) {
  std::vector<V3> n(nf);
  for (int k = 0; k < nf; ++k) {
    V3 xa = col(verts, faces[3 * k]), xb = col(verts, faces[3 * k + 1]),
       xc = col(verts, faces[3 * k + 2]);
    V3 dba = xb - xa, dac = xa - xc;
    n[k] = normalized(cross(dba, -dac));
  }
  return n;
}

// createEdges (boxTriCollision.cpp:141-231).  The hash kmin + (n+1) kmax is
// evaluated in 32-bit two's-complement arithmetic, as the reference's int
// expression is on its targets.
std::vector<Edge> create_edges(const int *faces, int nf,
                               const std::vector<double> &verts) {
  struct FE { int v[3]; int face; int32_t hash; };
  int n = 3 * nf;
  std::vector<FE> tmp;
  tmp.reserve(n);
  for (int k = 0; k < nf; ++k)
    for (int i = 0; i < 3; ++i) {
      FE fe;
      fe.v[0] = i % 3; fe.v[1] = (i + 1) % 3; fe.v[2] = (i + 2) % 3;
      fe.face = k;
      int a = faces[3 * k + fe.v[0]], b = faces[3 * k + fe.v[1]];
      uint32_t kmin = uint32_t(std::min(a, b) + 1), kmax = uint32_t(std::max(a, b) + 1);
      fe.hash = int32_t(kmin + uint32_t(n + 1) * kmax);
      tmp.push_back(fe);
    }
  std::stable_sort(tmp.begin(), tmp.end(),
                   [](const FE &a, const FE &b) { return a.hash < b.hash; });
  std::vector<Edge> edges;
  int k = 0;
  auto fnormal = [&](int f) {
    V3 xa = col(verts, faces[3 * f]), xb = col(verts, faces[3 * f + 1]),
       xc = col(verts, faces[3 * f + 2]);
    return normalized(cross(xb - xa, xc - xa));
  };
  while (k < n) {
    int f0 = tmp[k].face;
    Edge e;
    e.verts[0] = faces[3 * f0 + tmp[k].v[0]];
    e.verts[1] = faces[3 * f0 + tmp[k].v[1]];
    e.verts[2] = faces[3 * f0 + tmp[k].v[2]];
    V3 n0 = fnormal(f0);
    if (k < n - 1 && tmp[k].hash == tmp[k + 1].hash) {
      int f1 = tmp[k + 1].face;
      V3 n1 = fnormal(f1);
      e.verts[3] = faces[3 * f1 + tmp[k + 1].v[2]];
      e.faces[0] = f0; e.faces[1] = f1;
      e.internal = true;
      e.angle = std::acos(dot(n0, n1));
      e.normals[0] = n0; e.normals[1] = n1;
      k += 2;
    } else {
      e.verts[3] = -1;
      e.faces[0] = f0; e.faces[1] = -1;
      e.internal = false;
      e.angle = 1e9;
      e.normals[0] = n0; e.normals[1] = orc::mk(0, 0, 0);
      k += 1;
    }
    edges.push_back(e);
  }
  return edges;
}

struct Box {
  std::vector<double> verts;  // 3 x 14
  std::vector<V3> faceNors, vertNors;
  std::vector<Edge> edges;
};

// createBox (boxTriCollision.cpp:400-420) with createVertNormals
// (:249-281).  E = E1 * S and verts = E * verts_ are summed in index order.
Box create_box(const eolc_box &bx) {
  double S[4][4] = {{0}};
  S[0][0] = 0.5 * bx.dim[0]; S[1][1] = 0.5 * bx.dim[1];
  S[2][2] = 0.5 * bx.dim[2]; S[3][3] = 1;
  double E[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += bx.E1[k * 4 + i] * S[k][j];
      E[i][j] = s;
    }
  Box b;
  b.verts.assign(3 * 14, 0.0);
  for (int c = 0; c < 14; ++c)
    for (int i = 0; i < 3; ++i) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += E[i][k] * (k < 3 ? kBoxVerts[c][k] : 1.0);
      b.verts[3 * c + i] = s;
    }
  b.faceNors = face_normals(&kBoxFaces[0][0], 24, b.verts);
  // createVertNormals: angle-weighted face normals
  std::vector<V3> vn(14, orc::mk(0, 0, 0));
  std::vector<double> ang(14, 0.0);
  for (int k = 0; k < 24; ++k) {
    const int *f = kBoxFaces[k];
    V3 xa = col(b.verts, f[0]), xb = col(b.verts, f[1]), xc = col(b.verts, f[2]);
    V3 dba = xb - xa, dcb = xc - xb, dac = xa - xc;
    V3 nor = normalized(cross(dba, -dac));
    dba = normalized(dba); dcb = normalized(dcb); dac = normalized(dac);
    double a1 = std::acos(dot(dba, -dac));
    double a2 = std::acos(dot(dcb, -dba));
    double a3 = std::acos(dot(dac, -dcb));
    vn[f[0]] = vn[f[0]] + a1 * nor;
    vn[f[1]] = vn[f[1]] + a2 * nor;
    vn[f[2]] = vn[f[2]] + a3 * nor;
    ang[f[0]] += a1; ang[f[1]] += a2; ang[f[2]] += a3;
  }
  b.vertNors.resize(14);
  for (int k = 0; k < 14; ++k) b.vertNors[k] = normalized(vn[k] / ang[k]);
  for (int k = 0; k < 12; ++k) {
    Edge e;
    for (int i = 0; i < 4; ++i) e.verts[i] = kBoxEdgeVerts[k][i];
    e.faces[0] = kBoxEdgeFaces[k][0];
    e.faces[1] = kBoxEdgeFaces[k][1];
    e.internal = false;
    e.normals[0] = b.faceNors[e.faces[0]];
    e.normals[1] = b.faceNors[e.faces[1]];
    e.angle = std::acos(dot(e.normals[0], e.normals[1]));
    b.edges.push_back(e);
  }
  return b;
}

struct AABB { double v[6]; };

AABB aabb_of(const std::vector<double> &V, int n) {
  AABB a;
  for (int i = 0; i < 3; ++i) { a.v[i] = V[i]; a.v[i + 3] = V[i]; }
  for (int k = 1; k < n; ++k)
    for (int i = 0; i < 3; ++i) {
      a.v[i] = std::min(a.v[i], V[3 * k + i]);
      a.v[i + 3] = std::max(a.v[i + 3], V[3 * k + i]);
    }
  return a;
}

AABB aabb_pt(const V3 &x) { return AABB{{x[0], x[1], x[2], x[0], x[1], x[2]}}; }

// check_AABB (boxTriCollision.cpp:469-485)
bool check_aabb(const AABB &a, const AABB &b) {
  const double t = 1e-3;
  return a.v[3] + t >= b.v[0] - t && a.v[0] - t <= b.v[3] + t &&
         a.v[4] + t >= b.v[1] - t && a.v[1] - t <= b.v[4] + t &&
         a.v[5] + t >= b.v[2] - t && a.v[2] - t <= b.v[5] + t;
}

// barycentric (boxTriCollision.cpp:487-505)
void barycentric(double &alpha, double &beta, const V3 &a, const V3 &b,
                 const V3 &c, const V3 &p) {
  V3 v0 = b - a, v1 = c - a, v2 = p - a;
  double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
  double d20 = dot(v2, v0), d21 = dot(v2, v1);
  double denom = d00 * d11 - d01 * d01;
  beta = (d11 * d20 - d01 * d21) / denom;
  double gamma = (d00 * d21 - d01 * d20) / denom;
  alpha = 1.0 - beta - gamma;
}

// lineline (boxTriCollision.cpp:507-526)
void lineline(double &a, double &b, const V3 &A1, const V3 &A2, const V3 &B1,
              const V3 &B2) {
  V3 B2B1 = B2 - B1, A1B1 = A1 - B1, A2A1 = A2 - A1;
  V3 AxB = cross(A2A1, B2B1);
  double nA = dot(cross(B2B1, A1B1), AxB);
  double nB = dot(cross(A2A1, A1B1), AxB);
  double d = dot(cross(A2A1, B2B1), AxB);
  a = nA / d;
  b = nB / d;
}

// linepoint (boxTriCollision.cpp:528-537)
double linepoint(const V3 &A, const V3 &B, const V3 &P) {
  V3 AP = P - A, AB = B - A;
  return dot(AP, AB) / dot(AB, AB);
}

// intersect_square (boxTriCollision.cpp:550-600)
int intersect_square(const V3 &x0, const V3 &dx, const V3 &xa, const V3 &xb,
                     const V3 &xc, double &t) {
  V3 xd = xa + 2.0 * (xc - xa);
  V3 xe = xb + 2.0 * (xc - xb);
  double tuv[3];
  const V3 *tris[4][3] = {{&xa, &xb, &xc}, {&xb, &xd, &xc}, {&xd, &xe, &xc},
                          {&xe, &xa, &xc}};
  for (auto &tr : tris) {
    if (orc_raytri(x0.v, dx.v, tr[0]->v, tr[1]->v, tr[2]->v, tuv)) {
      t = tuv[0];
      return 1;
    }
  }
  t = -1.0;
  return 0;
}

eolc_contact blank() {
  eolc_contact c{};
  c.tri1 = -1; c.tri2 = -1; c.edge2 = -1;
  return c;
}

void put(double *d, const V3 &v) { d[0] = v[0]; d[1] = v[1]; d[2] = v[2]; }

// Deterministic perturbation of the cloth vertices: std::mt19937 seeded 1
// each call, uniform_real_distribution(-1, 1) scaled by threshold * 1e-3
// (boxTriCollision.cpp:648-659, :1078-1090).
std::vector<double> perturbed(const double *x, int nv, double threshold) {
  std::vector<double> v(x, x + 3 * nv);
  std::mt19937 gen;
  std::uniform_real_distribution<> dis(-1.0, 1.0);
  gen.seed(1);
  for (int i = 0; i < nv; ++i) {
    double r0 = dis(gen) * threshold * 1e-3;
    double r1 = dis(gen) * threshold * 1e-3;
    double r2 = dis(gen) * threshold * 1e-3;
    v[3 * i] += r0; v[3 * i + 1] += r1; v[3 * i + 2] += r2;
  }
  return v;
}

// btc::pointTriCollision with EOL = false (boxTriCollision.cpp:1067-1224).
void point_tri(std::vector<eolc_contact> &out, double threshold,
               const double *pts, const double *nrm, int np, const double *x,
               int nv, const int *faces, int nf) {
  size_t first = out.size();
  std::vector<double> v2 = perturbed(x, nv, threshold);
  std::vector<V3> fn2 = face_normals(faces, nf, v2);
  AABB bb2 = aabb_of(v2, nv);
  for (int i1 = 0; i1 < np; ++i1) {
    V3 x1 = orc::ld(pts + 3 * i1);
    if (!check_aabb(aabb_pt(x1), bb2)) continue;
    bool have = false;
    eolc_contact cmin;
    V3 nor1 = orc::ld(nrm + 3 * i1);
    for (int j2 = 0; j2 < nf; ++j2) {
      const int *f2 = faces + 3 * j2;
      V3 x2a = col(v2, f2[0]), x2b = col(v2, f2[1]), x2c = col(v2, f2[2]);
      V3 nor2 = fn2[j2];
      if (dot(nor1, nor2) < 0.0) nor2 = -nor2;
      V3 dx = x1 - x2a;
      double proj = dot(dx, nor2);
      if (proj < 0.0) continue;
      V3 x2 = x1 - proj * nor2;
      dx = x2 - x1;
      double dist = norm(dx);
      if (dist > 5.0 * threshold) continue;
      double u, v;
      barycentric(u, v, x2a, x2b, x2c, x1);
      double w = 1.0 - u - v;
      if (u < 0.0 || 1.0 < u || v < 0.0 || 1.0 < v || w < 0.0 || 1.0 < w) continue;
      if (have && !(dist < cmin.dist)) continue;
      eolc_contact c = blank();
      c.dist = dist;
      put(c.nor1, nor1); put(c.nor2, nor2); put(c.pos1, x1); put(c.pos2, x2);
      c.count1 = 1; c.count2 = 3;
      c.verts1[0] = i1; c.verts1[1] = -1; c.verts1[2] = -1;
      c.verts2[0] = f2[0]; c.verts2[1] = f2[1]; c.verts2[2] = f2[2];
      c.weights1[0] = 1.0;
      c.weights2[0] = u; c.weights2[1] = v; c.weights2[2] = w;
      c.tri2 = j2;
      cmin = c;
      have = true;
    }
    if (have) out.push_back(cmin);
  }
  double snap = 0.1 * threshold;
  for (size_t k = first; k < out.size(); ++k)
    for (int i = 0; i < 3; ++i)
      out[k].pos1_[i] = out[k].pos1[i] - snap * out[k].nor1[i];
}

// btc::boxTriCollision with EOL = false (boxTriCollision.cpp:602-1063).
void box_tri(std::vector<eolc_contact> &out, double threshold,
             const eolc_box &bx, const double *x, int nv, const int *faces,
             int nf) {
  size_t first = out.size();
  // Edges are built from the unperturbed positions (:602-615).
  std::vector<double> v0(x, x + 3 * nv);
  std::vector<Edge> edges2 = create_edges(faces, nf, v0);
  Box B = create_box(bx);
  std::vector<double> v2 = perturbed(x, nv, threshold);
  std::vector<V3> fn2 = face_normals(faces, nf, v2);
  AABB bb1 = aabb_of(B.verts, 14), bb2 = aabb_of(v2, nv);
  std::vector<AABB> bbF1(24);
  for (int k = 0; k < 24; ++k) {
    V3 xa = col(B.verts, kBoxFaces[k][0]), xb = col(B.verts, kBoxFaces[k][1]),
       xc = col(B.verts, kBoxFaces[k][2]);
    for (int i = 0; i < 3; ++i) {
      double lo = xa[i], hi = xa[i];
      lo = std::min(xb[i], lo); lo = std::min(xc[i], lo);
      hi = std::max(xb[i], hi); hi = std::max(xc[i], hi);
      bbF1[k].v[i] = lo; bbF1[k].v[i + 3] = hi;
    }
  }
  std::vector<AABB> bbE2(edges2.size());
  for (size_t k = 0; k < edges2.size(); ++k) {
    V3 a = col(v2, edges2[k].verts[0]), b = col(v2, edges2[k].verts[1]);
    for (int i = 0; i < 3; ++i) {
      bbE2[k].v[i] = std::min(b[i], a[i]);
      bbE2[k].v[i + 3] = std::max(b[i], a[i]);
    }
  }
  // Vertex2 - Triangle1
  for (int i2 = 0; i2 < nv; ++i2) {
    V3 x2 = col(v2, i2);
    if (!check_aabb(aabb_pt(x2), bb1)) continue;
    bool inside = true;
    for (int j1 = 0; j1 < 24; ++j1) {
      V3 x1a = col(B.verts, kBoxFaces[j1][0]);
      if (dot(B.faceNors[j1], x2 - x1a) > 0.0) { inside = false; break; }
    }
    if (!inside) continue;
    bool have = false;
    eolc_contact cmin;
    for (int j1 = 0; j1 < 24; ++j1) {
      const int *f1 = kBoxFaces[j1];
      V3 x1a = col(B.verts, f1[0]), x1b = col(B.verts, f1[1]),
         x1c = col(B.verts, f1[2]);
      V3 nor1 = B.faceNors[j1];
      V3 dx = x2 - x1a;
      double proj = dot(nor1, dx);
      if (proj > 0.0) continue;
      V3 x1 = x2 - proj * nor1;
      dx = x2 - x1;
      double dist = norm(dx);
      if (dist > 5.0 * threshold) continue;
      double u, v;
      barycentric(u, v, x1a, x1b, x1c, x1);
      double w = 1.0 - u - v;
      if (u < 0.0 || 1.0 < u || v < 0.0 || 1.0 < v || w < 0.0 || 1.0 < w) continue;
      // The cloth "normal" is read from the face-normal array at the
      // vertex index (boxTriCollision.cpp:731).
      V3 nor2 = i2 < nf ? fn2[i2] : orc::mk(NAN, NAN, NAN);
      if (dot(nor2, nor1) < 0.0) nor2 = -nor2;
      if (have && !(dist < cmin.dist)) continue;
      eolc_contact c = blank();
      c.dist = dist;
      put(c.nor1, nor1); put(c.nor2, nor2); put(c.pos1, x1); put(c.pos2, x2);
      c.count1 = 3; c.count2 = 1;
      c.verts1[0] = f1[0]; c.verts1[1] = f1[1]; c.verts1[2] = f1[2];
      c.verts2[0] = i2; c.verts2[1] = -1; c.verts2[2] = -1;
      c.weights1[0] = u; c.weights1[1] = v; c.weights1[2] = w;
      c.weights2[0] = 1.0;
      c.tri1 = j1;
      cmin = c;
      have = true;
    }
    if (have) out.push_back(cmin);
  }
  // Vertex1 - Triangle2 (box corners only)
  for (int i1 = 0; i1 < 8; ++i1) {
    V3 x1 = col(B.verts, i1);
    if (!check_aabb(aabb_pt(x1), bb2)) continue;
    bool have = false;
    eolc_contact cmin;
    V3 nor1 = B.vertNors[i1];
    for (int j2 = 0; j2 < nf; ++j2) {
      const int *f2 = faces + 3 * j2;
      V3 x2a = col(v2, f2[0]), x2b = col(v2, f2[1]), x2c = col(v2, f2[2]);
      V3 nor2 = fn2[j2];
      if (dot(nor1, nor2) < 0.0) nor2 = -nor2;
      V3 dx = x1 - x2a;
      double proj = dot(dx, nor2);
      if (proj < 0.0) continue;
      V3 x2 = x1 - proj * nor2;
      dx = x2 - x1;
      double dist = norm(dx);
      if (dist > 5.0 * threshold) continue;
      double u, v;
      barycentric(u, v, x2a, x2b, x2c, x1);
      double w = 1.0 - u - v;
      if (u < 0.0 || 1.0 < u || v < 0.0 || 1.0 < v || w < 0.0 || 1.0 < w) continue;
      if (have && !(dist < cmin.dist)) continue;
      eolc_contact c = blank();
      c.dist = dist;
      put(c.nor1, nor1); put(c.nor2, nor2); put(c.pos1, x1); put(c.pos2, x2);
      c.count1 = 1; c.count2 = 3;
      c.verts1[0] = i1; c.verts1[1] = -1; c.verts1[2] = -1;
      c.verts2[0] = f2[0]; c.verts2[1] = f2[1]; c.verts2[2] = f2[2];
      c.weights1[0] = 1.0;
      c.weights2[0] = u; c.weights2[1] = v; c.weights2[2] = w;
      c.edge1[0] = kBoxVertEdges[i1][0];
      c.edge1[1] = kBoxVertEdges[i1][1];
      c.edge1[2] = kBoxVertEdges[i1][2];
      c.n_edge1 = 3;
      c.tri2 = j2;
      cmin = c;
      have = true;
    }
    if (have) out.push_back(cmin);
  }
  // Edge2 - Edge1
  const double threshAng = 2.0 * M_PI / 180.0;
  for (size_t k2 = 0; k2 < edges2.size(); ++k2) {
    const Edge &e2 = edges2[k2];
    V3 x2a = col(v2, e2.verts[0]), x2b = col(v2, e2.verts[1]);
    V3 dx2 = x2b - x2a;
    double len2 = norm(dx2);
    V3 nor2 = normalized(e2.normals[0] + e2.normals[1]);
    for (int k1 = 0; k1 < 12; ++k1) {
      const Edge &e1 = B.edges[k1];
      if (e1.angle < M_PI / 6.0) continue;
      if (!check_aabb(bbF1[e1.faces[0]], bbE2[k2]) &&
          !check_aabb(bbF1[e1.faces[1]], bbE2[k2]))
        continue;
      V3 x1a = col(B.verts, e1.verts[0]), x1b = col(B.verts, e1.verts[1]);
      V3 dx1 = x1b - x1a;
      double len1 = norm(dx1);
      V3 tan1 = dx1 / len1;
      double angle = std::acos(dot(tan1, nor2));
      if (std::fabs(angle) < threshAng || std::fabs(M_PI - angle) < threshAng) continue;
      angle = std::acos(dot(tan1, dx2) / len2);
      if (std::fabs(angle) < threshAng || std::fabs(M_PI - angle) < threshAng) continue;
      V3 nor = normalized(cross(dx1, dx2));
      V3 x1c = col(B.verts, e1.verts[2]), x1d = col(B.verts, e1.verts[3]);
      const V3 &n1c = e1.normals[0], &n1d = e1.normals[1];
      V3 nor1 = normalized(n1c + n1d);
      if (dot(nor, nor1) < 0.0) nor = -nor;
      double angleCD = std::acos(dot(n1c, n1d));
      double angleCN = std::acos(dot(n1c, nor));
      if (angleCD < 0.0) { angleCD = -angleCD; angleCN = -angleCN; }
      if (angleCN < -threshAng || angleCN - angleCD > threshAng) continue;
      double u2c, u2d;
      int i2c = intersect_square(x2a, dx2, x1a, x1b, x1c, u2c);
      int i2d = intersect_square(x2a, dx2, x1b, x1a, x1d, u2d);
      i2c = i2c && (0.0 <= u2c && u2c <= 1.0);
      i2d = i2d && (0.0 <= u2d && u2d <= 1.0);
      double u1, u2;
      lineline(u1, u2, x1a, x1b, x2a, x2b);
      double thresh1 = 1.0 * threshold / len1;
      double thresh2 = 1.0 * threshold / len2;
      if (u1 < -thresh1 || u1 > 1.0 + thresh1 || u2 < -thresh2 || u2 > 1.0 + thresh2)
        continue;
      V3 x1, x2, dx;
      if (i2c && i2d) {
        x1 = (1.0 - u1) * x1a + u1 * x1b;
        x2 = (1.0 - u2) * x2a + u2 * x2b;
      } else if (i2c && !i2d) {
        dx = x2a - x1a;
        if (dot(dx, n1c) < 0.0) u2 = std::max(0.0, std::min(u2c, u2));
        else u2 = std::max(u2c, std::min(1.0, u2));
        x2 = (1.0 - u2) * x2a + u2 * x2b;
        u1 = linepoint(x1a, x1b, x2);
        x1 = (1.0 - u1) * x1a + u1 * x1b;
      } else if (!i2c && i2d) {
        dx = x2a - x1b;
        if (dot(dx, n1d) < 0.0) u2 = std::max(0.0, std::min(u2d, u2));
        else u2 = std::max(u2d, std::min(1.0, u2));
        x2 = (1.0 - u2) * x2a + u2 * x2b;
        u1 = linepoint(x1a, x1b, x2);
        x1 = (1.0 - u1) * x1a + u1 * x1b;
      } else {
        continue;
      }
      if (u1 < -thresh1 || u1 > 1.0 + thresh1 || u2 < -thresh2 || u2 > 1.0 + thresh2)
        continue;
      dx = x2 - x1;
      double thresh = 2.0 * threshold;
      if (dot(dx, dx) > thresh * thresh) continue;
      eolc_contact c = blank();
      c.dist = norm(dx);
      put(c.nor1, nor1); put(c.nor2, nor); put(c.pos1, x1); put(c.pos2, x2);
      c.count1 = 2; c.count2 = 2;
      c.verts1[0] = e1.verts[0]; c.verts1[1] = e1.verts[1]; c.verts1[2] = -1;
      c.verts2[0] = e2.verts[0]; c.verts2[1] = e2.verts[1]; c.verts2[2] = -1;
      c.weights1[0] = 1.0 - u1; c.weights1[1] = u1;
      c.weights2[0] = 1.0 - u2; c.weights2[1] = u2;
      c.edge1[0] = k1; c.n_edge1 = 1;
      c.edge2 = int(k2);
      put(c.edge_dir, tan1);
      out.push_back(c);
    }
  }
  // The per-corner de-duplication pass (:1022-1052) never removes anything:
  // the corner loop above already keeps at most one contact per corner and
  // edge contacts have count1 == 2.
  double snap = 0.1 * threshold;
  for (size_t k = first; k < out.size(); ++k)
    for (int i = 0; i < 3; ++i)
      out[k].pos1_[i] = out[k].pos1[i] - snap * out[k].nor1[i];
}

}  // namespace

extern "C" {

int orc_cd2(int n_nodes, const double *x, const int *tri, int n_tri,
            const eolc_box *boxes, int n_boxes, const double *points,
            const double *normals, int n_points, double threshold,
            eolc_contact *out, int cap) {
  std::vector<eolc_contact> cls;
  point_tri(cls, threshold, points, normals, n_points, x, n_nodes, tri, n_tri);
  for (auto &c : cls) c.source = 0;
  for (int b = 0; b < n_boxes; ++b) {
    size_t s = cls.size();
    box_tri(cls, threshold, boxes[b], x, n_nodes, tri, n_tri);
    for (size_t k = s; k < cls.size(); ++k) cls[k].source = 1 + b;
  }
  int n = int(cls.size());
  for (int k = 0; k < n && k < cap; ++k) out[k] = cls[k];
  return n;
}

int orc_create_edges(int n_nodes, const double *x, const int *tri, int n_tri,
                     int *edges6, int cap) {
  std::vector<double> v(x, x + 3 * n_nodes);
  std::vector<Edge> e = create_edges(tri, n_tri, v);
  for (size_t k = 0; k < e.size() && int(k) < cap; ++k) {
    for (int i = 0; i < 4; ++i) edges6[6 * k + i] = e[k].verts[i];
    edges6[6 * k + 4] = e[k].faces[0];
    edges6[6 * k + 5] = e[k].faces[1];
  }
  return int(e.size());
}

}  // extern "C"
