// Oracle meshes (test infrastructure; see oracle.h).
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "oracle.h"

namespace {

// Linear blend (1-s)*a + s*b per component, as the Eigen expressions of
// Cloth::build (Cloth.cpp:63-76).
inline void blend(double s, const double *a, const double *b, double *out,
                  int n) {
  for (int c = 0; c < n; ++c) out[c] = (1 - s) * a[c] + s * b[c];
}

// Node positions of the reference grid (Cloth.cpp:63-76).  corners holds
// p00, p01, p10, p11 as (x, y, z, X, Y).
void grid_nodes(int r0, int r1, const double *corners, double *x, double *X) {
  const double *p00 = corners, *p01 = corners + 5, *p10 = corners + 10,
               *p11 = corners + 15;
  double x00[3] = {p00[0], p00[1], p00[2]}, x01[3] = {p01[0], p01[1], p01[2]};
  double x10[3] = {p10[0], p10[1], p10[2]}, x11[3] = {p11[0], p11[1], p11[2]};
  // Material points are Vector3d with z = 0 in the reference.
  double X00[3] = {p00[3], p00[4], 0}, X01[3] = {p01[3], p01[4], 0};
  double X10[3] = {p10[3], p10[4], 0}, X11[3] = {p11[3], p11[4], 0};
  for (int i = 0; i < r0; ++i) {
    double u = i / (r0 - 1.0);
    double a0[3], a1[3], A0[3], A1[3];
    blend(u, x00, x10, a0, 3);
    blend(u, x01, x11, a1, 3);
    blend(u, X00, X10, A0, 3);
    blend(u, X01, X11, A1, 3);
    for (int j = 0; j < r1; ++j) {
      double v = j / (r1 - 1.0);
      int k = i * r1 + j;
      double xx[3], XX[3];
      blend(v, a0, a1, xx, 3);
      blend(v, A0, A1, XX, 3);
      for (int c = 0; c < 3; ++c) x[3 * k + c] = xx[c];
      X[2 * k + 0] = XX[0];
      X[2 * k + 1] = XX[1];
    }
  }
}

}  // namespace

extern "C" {

void orc_grid2_build(int r0, int r1, const double *corners, double *x,
                     double *X, int *tri) {
  grid_nodes(r0, r1, corners, x, X);
  int t = 0;
  for (int i = 0; i < r0 - 1; ++i) {
    for (int j = 0; j < r1 - 1; ++j) {
      int k0 = i * r1 + j;
      int k1 = k0 + 1, k2 = k0 + r1 + 1, k3 = k0 + r1;
      tri[3 * t + 0] = k0; tri[3 * t + 1] = k1; tri[3 * t + 2] = k2; ++t;
      tri[3 * t + 0] = k0; tri[3 * t + 1] = k2; tri[3 * t + 2] = k3; ++t;
    }
  }
}

void orc_gridc_build(int r0, int r1, const double *corners, double *x,
                     double *X, int *tri) {
  grid_nodes(r0, r1, corners, x, X);
  int nc = r0 * r1;
  // Centre nodes: mean of the quad's four nodes, summed left to right as
  // in Cloth.cpp:84-85.
  for (int i = 0; i < r0 - 1; ++i) {
    for (int j = 0; j < r1 - 1; ++j) {
      int k0 = i * r1 + j;
      int q[4] = {k0, k0 + 1, k0 + r1 + 1, k0 + r1};
      int kc = nc + i * (r1 - 1) + j;
      for (int c = 0; c < 3; ++c) {
        double s = ((x[3 * q[0] + c] + x[3 * q[1] + c]) + x[3 * q[2] + c]) +
                   x[3 * q[3] + c];
        x[3 * kc + c] = s / 4;
      }
      for (int c = 0; c < 2; ++c) {
        double s = ((X[2 * q[0] + c] + X[2 * q[1] + c]) + X[2 * q[2] + c]) +
                   X[2 * q[3] + c];
        X[2 * kc + c] = s / 4;
      }
    }
  }
  // Four faces per quad, vertex order of Cloth.cpp:96-124 (triangulateARC
  // keeps a triangle's input order, io.cpp:244-270).
  int t = 0;
  for (int i = 0; i < r0 - 1; ++i) {
    for (int j = 0; j < r1 - 1; ++j) {
      int k0 = i * r1 + j;
      int kc = nc + i * (r1 - 1) + j;
      int f[4][3] = {{k0, k0 + 1, kc},
                     {k0 + 1, k0 + r1 + 1, kc},
                     {k0 + r1 + 1, k0 + r1, kc},
                     {k0 + r1, k0, kc}};
      for (int a = 0; a < 4; ++a, ++t)
        for (int c = 0; c < 3; ++c) tri[3 * t + c] = f[a][c];
    }
  }
}

// ArcSim adjacency (mesh.cpp:356-378): faces are added in order; each face
// creates its missing edges (v[i], v[NEXT(i)]) in order, then registers
// itself on side 0 of edge (v[NEXT(i)], v[PREV(i)]) when that edge's n[0] is
// v[NEXT(i)], else on side 1.
int orc_hinges(int n_nodes, const int *tri, int n_tri, int *hinge, int cap) {
  (void)n_nodes;
  struct E { int n0, n1, f0, f1; };
  std::vector<E> edges;
  std::unordered_map<uint64_t, int> lookup;
  auto key = [](int a, int b) {
    uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
    return (uint64_t(hi) << 32) | lo;
  };
  edges.reserve(size_t(n_tri) * 3 / 2 + 16);
  for (int f = 0; f < n_tri; ++f) {
    const int *v = tri + 3 * f;
    for (int i = 0; i < 3; ++i) {
      int a = v[i], b = v[(i + 1) % 3];
      auto k = key(a, b);
      if (!lookup.count(k)) {
        lookup[k] = int(edges.size());
        edges.push_back(E{a, b, -1, -1});
      }
    }
    for (int i = 0; i < 3; ++i) {
      int a = v[(i + 1) % 3], b = v[(i + 2) % 3];
      E &e = edges[lookup[key(a, b)]];
      if (e.n0 == a) e.f0 = f; else e.f1 = f;
    }
  }
  int n = 0;
  for (const E &e : edges) {
    if (e.f0 < 0 || e.f1 < 0) continue;
    if (n < cap) {
      // get_other_vert (mesh.hpp:276-280)
      auto other = [&](int f) {
        const int *v = tri + 3 * f;
        if (v[0] != e.n0 && v[0] != e.n1) return v[0];
        if (v[1] != e.n0 && v[1] != e.n1) return v[1];
        return v[2];
      };
      hinge[4 * n + 0] = e.n0;
      hinge[4 * n + 1] = e.n1;
      hinge[4 * n + 2] = other(e.f0);
      hinge[4 * n + 3] = other(e.f1);
    }
    ++n;
  }
  return n;
}

}  // extern "C"
