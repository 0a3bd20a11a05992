// The reference's own collision detection as a C function, for pinning the
// oracle's restatement (oracle/collide.cpp) and the fixtures under
// tests/golden/ (TEST INFRASTRUCTURE ONLY).  Compiled by oracle/build_ref.sh
// together with the reference's src/boxTriCollision.cpp and src/raytri.cpp,
// unmodified, against the minimal Eigen shim in oracle/eigen_shim/ (Eigen
// itself is not vendored with the reference); the output goes to
// oracle/_ref/ only.
//
// ref_cd2 restates CD2 (Collisions.cpp:55-78): the cloth positions and faces
// packed as 3 x n matrices, pointTriCollision first (EOL = false), then
// boxTriCollision per box (EOL = false, every node flagged non-EOL), each
// btc::Collision converted to the library's contact record (source 0 for the
// points, 1 + b for box b; edge1 padded with zeros).
#include <cstring>
#include <memory>
#include <vector>

#include <Eigen/Dense>

#include "../include/eolc.h"
#include "boxTriCollision.h"

namespace {

void to_contact(const btc::Collision &c, int source, eolc_contact &o) {
  std::memset(&o, 0, sizeof(o));
  o.dist = c.dist;
  for (int i = 0; i < 3; ++i) {
    o.nor1[i] = c.nor1(i);
    o.nor2[i] = c.nor2(i);
    o.pos1[i] = c.pos1(i);
    o.pos2[i] = c.pos2(i);
    o.pos1_[i] = c.pos1_(i);
    o.weights1[i] = c.weights1(i);
    o.weights2[i] = c.weights2(i);
    o.edge_dir[i] = c.edgeDir(i);
    o.verts1[i] = c.verts1(i);
    o.verts2[i] = c.verts2(i);
  }
  o.count1 = c.count1;
  o.count2 = c.count2;
  o.tri1 = c.tri1;
  o.tri2 = c.tri2;
  o.n_edge1 = int(c.edge1.size());
  for (int k = 0; k < o.n_edge1 && k < 3; ++k) o.edge1[k] = c.edge1[k];
  o.edge2 = c.edge2;
  o.source = source;
}

}  // namespace

extern "C" int ref_cd2(int n_nodes, const double *x, const int *tri, int n_tri,
                       const eolc_box *boxes, int n_boxes, const double *points,
                       const double *normals, int n_points, double threshold,
                       eolc_contact *out, int cap) {
  using namespace Eigen;
  MatrixXd verts2(3, n_nodes);
  MatrixXi faces2(3, n_tri);
  VectorXi eols(n_nodes);  // all zero: no EOL node
  for (int i = 0; i < n_nodes; ++i)
    for (int c = 0; c < 3; ++c) verts2(c, i) = x[3 * i + c];
  for (int f = 0; f < n_tri; ++f)
    for (int c = 0; c < 3; ++c) faces2(c, f) = tri[3 * f + c];
  MatrixXd pxyz(3, n_points), norms(3, n_points);
  for (int p = 0; p < n_points; ++p)
    for (int c = 0; c < 3; ++c) {
      pxyz(c, p) = points[3 * p + c];
      norms(c, p) = normals[3 * p + c];
    }
  std::vector<std::shared_ptr<btc::Collision> > cls;
  btc::pointTriCollision(cls, threshold, pxyz, norms, verts2, faces2, false);
  std::vector<int> source(cls.size(), 0);
  for (int b = 0; b < n_boxes; ++b) {
    Vector3d dim(boxes[b].dim[0], boxes[b].dim[1], boxes[b].dim[2]);
    Matrix4d E1;
    for (int k = 0; k < 16; ++k) E1(k) = boxes[b].E1[k];  // column-major
    std::vector<std::shared_ptr<btc::Collision> > clst;
    btc::boxTriCollision(clst, threshold, dim, E1, verts2, faces2, eols, false);
    cls.insert(cls.end(), clst.begin(), clst.end());
    source.resize(cls.size(), 1 + b);
  }
  const int n = int(cls.size());
  for (int k = 0; k < n && k < cap; ++k) to_contact(*cls[k], source[k], out[k]);
  return n;
}
