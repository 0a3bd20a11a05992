// Oracle for the OBJ frame export: the text BrenderManager::exportBrender
// (BrenderManager.cpp:34-84) and Cloth::exportBrender (Cloth.cpp:535-590)
// write for one frame, produced with the C library's snprintf exactly as the
// reference formats it, from node positions x, material coordinates X and
// the triangle list.  Node normals restate ArcSim normal<WS>
// (geometry.cpp:302-316) in FP64 with contraction off.
//
// TEST INFRASTRUCTURE ONLY (what the device export is compared with).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "oracle.h"

namespace {

void append(std::string &s, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
void append(std::string &s, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  int n = vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  s.append(buf, n < int(sizeof(buf)) ? n : int(sizeof(buf)) - 1);
}

// normal<WS>(node) over the node's faces in mesh order (vert->adjf order of a
// mesh built face by face).
void node_normals(int n, const double *x, const int *tri, int n_tri, std::vector<double> &nrm) {
  std::vector<std::vector<std::pair<int, int>>> adj(n);
  for (int f = 0; f < n_tri; ++f)
    for (int j = 0; j < 3; ++j) adj[tri[3 * f + j]].push_back({f, j});
  nrm.assign(size_t(3) * n, 0.0);
  for (int v = 0; v < n; ++v) {
    double s[3] = {0, 0, 0};  // Vec3 n(0)
    for (auto [f, j] : adj[v]) {
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      double e1[3], e2[3];
      for (int c = 0; c < 3; ++c) {
        e1[c] = x[3 * tri[3 * f + j1] + c] - x[3 * v + c];
        e2[c] = x[3 * tri[3 * f + j2] + c] - x[3 * v + c];
      }
      // cross (vectors.hpp:54)
      const double w[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                           e1[0] * e2[1] - e1[1] * e2[0]};
      double a = 0, b = 0;  // norm2 = dot: accumulate from 0 (vectors.hpp:49-50)
      for (int c = 0; c < 3; ++c) a += e1[c] * e1[c];
      for (int c = 0; c < 3; ++c) b += e2[c] * e2[c];
      const double r = 1 / (2 * a * b);  // u / a = u * (1 / a) (vectors.hpp:45)
      for (int c = 0; c < 3; ++c) s[c] = s[c] + w[c] * r;
    }
    double m2 = 0;
    for (int c = 0; c < 3; ++c) m2 += s[c] * s[c];
    const double m = std::sqrt(m2);  // normalize (vectors.hpp:52)
    for (int c = 0; c < 3; ++c) nrm[3 * v + c] = m == 0 ? 0.0 : s[c] * (1 / m);
  }
}

std::string frame_text(int which, int n, const double *x, const double *X, const int *tri,
                       int n_tri, const std::vector<double> &nrm, int frame, double time) {
  const char *name = which == 0 ? "Cloth2D" : "Cloth3D";
  std::string s;
  append(s, "# frame %06d \n", frame);
  append(s, "# time %f \n", time);
  s += std::string("# name ") + name + " \n";
  for (int i = 0; i < n; ++i) {
    if (which == 0)  // mesh.nodes[i]->verts[0]->u (double); the literal 0 as 0.0
      append(s, "v %f %f %f\n", X[2 * i], X[2 * i + 1], 0.0);
    else  // posBuf (float)
      append(s, "v %f %f %f\n", double(float(x[3 * i])), double(float(x[3 * i + 1])),
             double(float(x[3 * i + 2])));
  }
  for (int i = 0; i < n; ++i)  // texBuf (float)
    append(s, "vt %f %f\n", double(float(X[2 * i])), double(float(X[2 * i + 1])));
  for (int i = 0; i < n; ++i) {
    if (which == 0)
      append(s, "vn %f %f %f\n", 0.0, 0.0, 1.0);
    else  // norBuf (float)
      append(s, "vn %f %f %f\n", double(float(nrm[3 * i])), double(float(nrm[3 * i + 1])),
             double(float(nrm[3 * i + 2])));
  }
  for (int f = 0; f < n_tri; ++f) {
    const int a = tri[3 * f] + 1, b = tri[3 * f + 1] + 1, c = tri[3 * f + 2] + 1;
    append(s, "f %i/%i/%i %i/%i/%i %i/%i/%i\n", a, a, a, b, b, b, c, c, c);
  }
  return s;
}

}  // namespace

extern "C" int orc_obj_text(int n_nodes, const double *x, const double *X, const int *tri,
                            int n_tri, int frame, double time, char *buf, long long cap,
                            long long *len) {
  std::vector<double> nrm;
  node_normals(n_nodes, x, tri, n_tri, nrm);
  const std::string a = frame_text(0, n_nodes, x, X, tri, n_tri, nrm, frame, time);
  const std::string b = frame_text(1, n_nodes, x, X, tri, n_tri, nrm, frame, time);
  len[0] = (long long)a.size();
  len[1] = (long long)b.size();
  if (!buf) return 0;
  if (cap < len[0] + len[1]) return 1;
  memcpy(buf, a.data(), a.size());
  memcpy(buf + a.size(), b.data(), b.size());
  return 0;
}

extern "C" void orc_node_normals(int n_nodes, const double *x, const int *tri, int n_tri,
                                 double *out) {
  std::vector<double> nrm;
  node_normals(n_nodes, x, tri, n_tri, nrm);
  memcpy(out, nrm.data(), sizeof(double) * nrm.size());
}
