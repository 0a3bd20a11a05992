// Constraints::fill for a mesh with EOL nodes (Constraints.cpp:147-468), on
// the host: the rows the reference hands its QP besides the pins.
//
// Per EOL node, in node order (:146-415):
//   at a box corner or point obstacle (cornerID >= 0): the constraint-table
//     normal nor as an inequality -nor v <= 0 and its orthogonal directions
//     o1 = (0, -nor_z, nor_y), o2 = (o1 x nor)/|o1 x nor| as equalities
//     o v = 0 when the node is locally flat (every adjacent face within 0.5
//     rad of the first) or sits on a point obstacle, else as inequalities
//     -o v <= 0;
//   on a box edge (cdEdges[0]): if locally flat (within 0.1 rad), the node
//     normal as an inequality and -(n x t) v = 0 with t the table's third
//     direction of the edge; else the edge's two face normals as
//     inequalities; then one equality on the node's two Eulerian DOFs: at a
//     boundary node the direction of :379-381 built from the first boundary
//     edge in Node::adje order, inside the mesh the normalised sum of the
//     preserved edges' unit directions, each pointing to its end nearer the
//     material origin (:389-403).
// Then the CD2 contact rows of :422-468 that touch no EOL node.  A node on
// a moving box (Box::v, angular then linear velocity, not zero) gets the
// right-hand sides of :165-172 and :270-277: with xl = E1^-1 [x; 1],
// et = Rigid::integrate(E1, v, h) (Rigid.cpp:79-111) and
// xdot = (et xl - E1 xl) / h, each row's bineq / beq is its direction dotted
// with xdot, signs as the reference writes them (the inequality rows of the
// two orthogonal directions at a bent corner take +o xdot, every other
// inequality -g xdot).  E1 is a rigid frame, so E1^-1 = [R' -R'p].
//
// Geometry follows ArcSim's definitions: face normal normalize((x1 - x0) x
// (x2 - x0)) (mesh.cpp:135-139), node normal normal<WS> (geometry.cpp:
// 302-316) over the node's faces in ascending order (Vert::adjf, filled by
// Mesh::add(Face)), get_angle = acos(clamp(n0^ . n1^, -1, 1)) (geometry.cpp:
// 392-394), is_seam_or_boundary(edge) = fewer than two faces (util.cpp:
// 146-150; a mesh with one vertex per node has no seams).  Zero vectors stay
// zero under normalisation, as with Eigen's normalized().
#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "internal.h"

namespace {

struct V3 {
  double v[3];
};

V3 sub(const V3 &a, const V3 &b) { return {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}}; }
V3 add(const V3 &a, const V3 &b) { return {{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]}}; }
V3 scale(const V3 &a, double s) { return {{a.v[0] * s, a.v[1] * s, a.v[2] * s}}; }
V3 divide(const V3 &a, double s) { return {{a.v[0] / s, a.v[1] / s, a.v[2] / s}}; }
double dot(const V3 &a, const V3 &b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
V3 cross(const V3 &a, const V3 &b) {
  return {{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
           a.v[0] * b.v[1] - a.v[1] * b.v[0]}};
}
V3 normalized(const V3 &a) {
  const double z = dot(a, a);
  return z > 0 ? divide(a, std::sqrt(z)) : a;
}

// Box geometry in the numbering the constraint table's columns use (Box.cpp:
// 25-72): the six face normals +x, -x, +y, -y, +z, -z of the box frame; per
// edge its two faces and the face whose normal runs along it; per corner its
// three edges.
const int kAxisFace[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
const int kEdgeFaces[12][2] = {{1, 3}, {1, 5}, {1, 4}, {1, 2}, {3, 5}, {3, 4},
                               {0, 3}, {2, 5}, {0, 5}, {2, 4}, {0, 4}, {0, 2}};
const int kEdgeAlong[12] = {4, 2, 2, 4, 0, 0, 4, 0, 2, 0, 2, 4};
const int kCornerEdges[8][3] = {{0, 1, 4}, {0, 2, 5}, {1, 3, 7}, {2, 3, 9},
                                {4, 6, 8}, {5, 6, 10}, {7, 8, 11}, {9, 10, 11}};
constexpr int kBoxColumns = 20;  // 8 corners, then 12 edges

// A box's motion over one step, for the moving-obstacle right-hand sides:
// E1, its rigid inverse and et = Rigid::integrate(E1, v, h) = E1 phib, all
// column-major 4x4.
struct BoxMotion {
  bool moving = false;
  double E1[16], E1inv[16], et[16];
};

BoxMotion box_motion(const eolc_box &b, const double *vel, double h) {
  BoxMotion m;
  for (int k = 0; k < 16; ++k) m.E1[k] = b.E1[k];
  if (!vel) return m;
  const V3 w0{{vel[0], vel[1], vel[2]}}, v0{{vel[3], vel[4], vel[5]}};
  m.moving = std::sqrt(dot(w0, w0)) != 0.0 || std::sqrt(dot(v0, v0)) != 0.0;
  if (!m.moving) return m;
  // rigid inverse [R' -R'p]
  for (int k = 0; k < 16; ++k) m.E1inv[k] = 0.0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m.E1inv[4 * c + r] = b.E1[4 * r + c];
  for (int r = 0; r < 3; ++r) {
    double t = 0;
    for (int k = 0; k < 3; ++k) t += b.E1[4 * r + k] * b.E1[12 + k];
    m.E1inv[12 + r] = -t;
  }
  m.E1inv[15] = 1.0;
  // phib of Rigid::integrate: translation h v, or the Rodrigues rotation
  // with the screw's translation when |w| > 1e-10
  double P[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  for (int r = 0; r < 3; ++r) P[12 + r] = h * v0.v[r];
  const double wlen = std::sqrt(dot(w0, w0));
  if (wlen > 1e-10) {
    const V3 w = divide(w0, wlen), v = divide(v0, wlen);
    const double c = std::cos(wlen * h), sn = std::sin(wlen * h), c1 = 1.0 - c;
    const double X = w.v[0], Y = w.v[1], Z = w.v[2];
    const double R[3][3] = {{c + X * X * c1, -Z * sn + X * Y * c1, Y * sn + X * Z * c1},
                            {Z * sn + X * Y * c1, c + Y * Y * c1, -X * sn + Y * Z * c1},
                            {-Y * sn + X * Z * c1, X * sn + Y * Z * c1, c + Z * Z * c1}};
    const V3 cc = cross(w, v);
    V3 d;
    for (int r = 0; r < 3; ++r) {
      const double a0 = (r == 0 ? 1.0 : 0.0) - R[r][0], a1 = (r == 1 ? 1.0 : 0.0) - R[r][1],
                   a2 = (r == 2 ? 1.0 : 0.0) - R[r][2];
      d.v[r] = a0 * cc.v[0] + a1 * cc.v[1] + a2 * cc.v[2];
    }
    const double wv = dot(w, v);
    for (int r = 0; r < 3; ++r) {
      for (int c2 = 0; c2 < 3; ++c2) P[4 * c2 + r] = R[r][c2];
      P[12 + r] = (wv * wlen * h) * w.v[r] + d.v[r];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double t = 0;
      for (int k = 0; k < 4; ++k) t += m.E1[4 * k + r] * P[4 * c + k];
      m.et[4 * c + r] = t;
    }
  return m;
}

// xdot = (et xl - E1 xl) / h with xl = E1^-1 [x; 1].
V3 box_point_velocity(const BoxMotion &m, const V3 &x, double h) {
  double xl[4];
  for (int r = 0; r < 4; ++r)
    xl[r] = m.E1inv[r] * x.v[0] + m.E1inv[4 + r] * x.v[1] + m.E1inv[8 + r] * x.v[2] +
            m.E1inv[12 + r];
  V3 out;
  for (int r = 0; r < 3; ++r) {
    double a = 0, b = 0;
    for (int k = 0; k < 4; ++k) {
      a += m.et[4 * k + r] * xl[k];
      b += m.E1[4 * k + r] * xl[k];
    }
    out.v[r] = (a - b) / h;
  }
  return out;
}

// Constraint table (Constraints::updateTable, :76-105): 9 values per column.
std::vector<double> constraint_table(const eolc_box *boxes, int n_boxes, const double *pn,
                                     int n_points) {
  std::vector<double> T(size_t(9) * (n_points + kBoxColumns * n_boxes), 0.0);
  for (int p = 0; p < n_points; ++p)
    for (int c = 0; c < 3; ++c) T[9 * p + c] = pn[3 * p + c];
  for (int b = 0; b < n_boxes; ++b) {
    V3 fn[6];
    for (int f = 0; f < 6; ++f)
      for (int i = 0; i < 3; ++i) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += boxes[b].E1[4 * k + i] * kAxisFace[f][k];
        fn[f].v[i] = s;
      }
    const int base = n_points + kBoxColumns * b;
    for (int p = 0; p < 8; ++p) {
      V3 cn{{0, 0, 0}};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) cn = add(cn, fn[kEdgeFaces[kCornerEdges[p][i]][j]]);
      cn = normalized(divide(cn, 6.0));
      for (int c = 0; c < 3; ++c) T[9 * (base + p) + c] = cn.v[c];
    }
    for (int e = 0; e < 12; ++e) {
      const V3 *cols[3] = {&fn[kEdgeFaces[e][0]], &fn[kEdgeFaces[e][1]], &fn[kEdgeAlong[e]]};
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) T[9 * (base + 8 + e) + 3 * r + c] = cols[r]->v[c];
    }
  }
  return T;
}

// Rows written into an eolc_rows while they fit; counted regardless.
struct RowSink {
  eolc_rows *R;
  int m = 0, q = 0;
  explicit RowSink(eolc_rows *r) : R(r) {
    if (R->ptr) R->ptr[0] = 0;
  }
  // terms (dof, value); every row has at most 9
  void row(const int *dof, const double *val, int n, double rhs) {
    if (m < R->capacity) {
      for (int t = 0; t < n; ++t) {
        R->col[q] = dof[t];
        R->val[q] = val[t];
        ++q;
      }
      R->rhs[m] = rhs;
      R->ptr[m + 1] = q;
    }
    ++m;
  }
  // a row on the three Lagrangian DOFs of node a
  void node_row(int a, const V3 &g, double rhs = 0.0) {
    const int dof[3] = {3 * a, 3 * a + 1, 3 * a + 2};
    row(dof, g.v, 3, rhs);
  }
};

// Host-only entry point without a context: the reason is in the caller's
// message string only.
eolc_status bad(const char * /*reason*/) { return EOLC_BAD_ARG; }

}  // namespace

extern "C" eolc_status eolc_constraint_rows(const eolc_eol_mesh *mesh, const eolc_box *boxes,
                                            const double *box_velocity_h, int n_boxes,
                                            const double *point_normals_h, int n_points,
                                            const eolc_contact *contacts, int n_contacts,
                                            double h, eolc_rows *eq, eolc_rows *ineq) {
  if (!mesh || !eq || !ineq || n_boxes < 0 || n_points < 0 || n_contacts < 0)
    return bad("null argument");
  if (box_velocity_h && !(h > 0)) return bad("moving boxes need h > 0");
  const eolc_eol_mesh &M = *mesh;
  const int N = M.n_nodes;
  if (N <= 0 || M.n_tri <= 0 || M.n_edges < 0 || M.n_eol < 0 || M.n_eol > N || !M.x || !M.u ||
      !M.tri || (M.n_edges > 0 && !M.edges) ||
      (M.n_eol > 0 && (!M.eol_nodes || !M.corner_id || !M.cd_edge)))
    return bad("bad mesh");
  if ((n_boxes > 0 && !boxes) || (n_points > 0 && !point_normals_h) ||
      (n_contacts > 0 && !contacts))
    return bad("null obstacle");
  for (eolc_rows *R : {eq, ineq})
    if (!R->ptr || R->capacity < 0 || (R->capacity > 0 && (!R->col || !R->val || !R->rhs)))
      return bad("bad row buffers");
  const int n_cols = n_points + kBoxColumns * n_boxes;
  std::vector<int> eol_index(N, -1);
  for (int k = 0; k < M.n_eol; ++k) {
    const int a = M.eol_nodes[k];
    if (a < 0 || a >= N || eol_index[a] >= 0) return bad("bad EOL node list");
    eol_index[a] = k;
    const int c = M.corner_id[k];
    if (c >= n_cols || (c < 0 && (M.cd_edge[k] < 0 || M.cd_edge[k] >= n_cols)))
      return bad("constraint-table column out of range");
  }
  for (int f = 0; f < M.n_tri; ++f) {
    const int *v = M.tri + 3 * f;
    for (int i = 0; i < 3; ++i)
      if (v[i] < 0 || v[i] >= N) return bad("face node out of range");
    if (v[0] == v[1] || v[1] == v[2] || v[0] == v[2]) return bad("face with a repeated node");
  }
  for (int e = 0; e < M.n_edges; ++e) {
    const int a = M.edges[2 * e], b = M.edges[2 * e + 1];
    if (a < 0 || a >= N || b < 0 || b >= N || a == b) return bad("bad edge");
  }
  const std::vector<double> table = constraint_table(boxes, n_boxes, point_normals_h, n_points);
  std::vector<BoxMotion> motion(n_boxes);
  for (int b = 0; b < n_boxes; ++b)
    motion[b] = box_motion(boxes[b], box_velocity_h ? box_velocity_h + 6 * b : nullptr, h);
  // the velocity of node a's point on the box of table column col; false
  // (no right-hand side) for point obstacles and boxes at rest
  auto xdot_of = [&](int col, int a, V3 &xd) {
    if (col < n_points) return false;
    const BoxMotion &m = motion[(col - n_points) / kBoxColumns];
    if (!m.moving) return false;
    xd = box_point_velocity(m, V3{{M.x[3 * a], M.x[3 * a + 1], M.x[3 * a + 2]}}, h);
    return true;
  };
  auto X = [&](int a) { return V3{{M.x[3 * a], M.x[3 * a + 1], M.x[3 * a + 2]}}; };
  auto U = [&](int a) { return V3{{M.u[2 * a], M.u[2 * a + 1], 0.0}}; };
  auto column = [&](int col, int r) {
    const double *t = &table[size_t(9) * col + 3 * r];
    return V3{{t[0], t[1], t[2]}};
  };

  // per EOL node (EoL_index k): its faces (ascending) and its edges
  // (mesh.edges order).  An edge of EOL node k is a boundary edge when fewer
  // than two of k's faces hold its other node.
  std::vector<std::vector<int>> nf(M.n_eol), ne(M.n_eol);
  for (int f = 0; f < M.n_tri; ++f)
    for (int i = 0; i < 3; ++i) {
      const int k = eol_index[M.tri[3 * f + i]];
      if (k >= 0) nf[k].push_back(f);
    }
  for (int e = 0; e < M.n_edges; ++e)
    for (int i = 0; i < 2; ++i) {
      const int k = eol_index[M.edges[2 * e + i]];
      if (k >= 0) ne[k].push_back(e);
    }
  auto boundary_edge = [&](int k, int a, int e) {
    const int b = M.edges[2 * e] == a ? M.edges[2 * e + 1] : M.edges[2 * e];
    int cnt = 0;
    for (const int f : nf[k]) {
      const int *v = M.tri + 3 * f;
      cnt += v[0] == b || v[1] == b || v[2] == b;
    }
    return cnt < 2;
  };
  auto face_normal = [&](int f) {
    const V3 x0 = X(M.tri[3 * f]), x1 = X(M.tri[3 * f + 1]), x2 = X(M.tri[3 * f + 2]);
    return normalized(cross(sub(x1, x0), sub(x2, x0)));
  };
  auto node_normal = [&](int k, int a) {
    V3 n{{0, 0, 0}};
    for (const int f : nf[k]) {
      const int *v = M.tri + 3 * f;
      const int j = v[0] == a ? 0 : v[1] == a ? 1 : 2;
      const V3 e1 = sub(X(v[(j + 1) % 3]), X(a)), e2 = sub(X(v[(j + 2) % 3]), X(a));
      n = add(n, divide(cross(e1, e2), 2 * dot(e1, e1) * dot(e2, e2)));
    }
    return normalized(n);
  };
  auto flat = [&](int k, double limit) {
    if (nf[k].empty()) return true;
    const V3 n0 = normalized(face_normal(nf[k][0]));
    for (size_t q = 1; q < nf[k].size(); ++q) {
      const V3 n1 = normalized(face_normal(nf[k][q]));
      const double c = std::fmin(std::fmax(dot(n0, n1), -1.0), 1.0);
      if (std::acos(c) > limit) return false;
    }
    return true;
  };
  auto unit2 = [](double a, double b) {
    const double z = a * a + b * b;
    return z > 0 ? std::make_pair(a / std::sqrt(z), b / std::sqrt(z)) : std::make_pair(a, b);
  };

  RowSink E(eq), I(ineq);
  for (int a = 0; a < N; ++a) {
    const int k = eol_index[a];
    if (k < 0) continue;
    const int corner = M.corner_id[k];
    if (corner >= 0) {  // :148-262
      const V3 nor = column(corner, 0);
      const V3 o1{{0.0, -nor.v[2], nor.v[1]}};
      const V3 o2 = normalized(normalized(cross(o1, nor)));
      const V3 mnor = scale(nor, -1.0);
      V3 xd;
      const bool mv = xdot_of(corner, a, xd);
      auto rhs = [&](const V3 &g, double sign) { return mv ? sign * dot(g, xd) : 0.0; };
      if (flat(k, 0.5) || corner < n_points) {
        I.node_row(a, mnor, rhs(nor, -1.0));
        E.node_row(a, o1, rhs(o1, 1.0));
        E.node_row(a, o2, rhs(o2, 1.0));
      } else {
        I.node_row(a, mnor, rhs(nor, -1.0));
        I.node_row(a, scale(o1, -1.0), rhs(o1, 1.0));
        I.node_row(a, scale(o2, -1.0), rhs(o2, 1.0));
      }
      continue;
    }
    const int cd = M.cd_edge[k];  // :263-415
    V3 xd;
    const bool mv = xdot_of(cd, a, xd);
    auto rhs = [&](const V3 &g) { return mv ? -dot(g, xd) : 0.0; };
    if (flat(k, 0.1)) {
      const V3 n = node_normal(k, a), fc = cross(n, column(cd, 2));
      I.node_row(a, scale(n, -1.0), rhs(n));
      E.node_row(a, scale(fc, -1.0), rhs(fc));
    } else {
      I.node_row(a, scale(column(cd, 0), -1.0), rhs(column(cd, 0)));
      I.node_row(a, scale(column(cd, 1), -1.0), rhs(column(cd, 1)));
    }
    const int dof[2] = {3 * (N + k), 3 * (N + k) + 1};
    int border = -1;
    for (size_t q = 0; q < ne[k].size() && border < 0; ++q)
      if (boundary_edge(k, a, ne[k][q])) border = ne[k][q];
    double g[2];
    if (border >= 0) {
      const int o = M.edges[2 * border] == a ? M.edges[2 * border + 1] : M.edges[2 * border];
      const auto d = unit2(M.u[2 * a + 1] - M.u[2 * o + 1], -M.u[2 * a] - M.u[2 * o]);
      g[0] = d.first;
      g[1] = d.second;
    } else {
      double t0 = 0, t1 = 0;
      for (const int e : ne[k]) {
        if (!M.preserve || !M.preserve[e]) continue;
        const int n0 = M.edges[2 * e], n1 = M.edges[2 * e + 1];
        const bool far0 = std::sqrt(dot(U(n0), U(n0))) > std::sqrt(dot(U(n1), U(n1)));
        const int from = far0 ? n0 : n1, to = far0 ? n1 : n0;
        const auto d = unit2(M.u[2 * to] - M.u[2 * from], M.u[2 * to + 1] - M.u[2 * from + 1]);
        t0 += d.first;
        t1 += d.second;
      }
      const auto d = unit2(t0, t1);
      g[0] = d.first;
      g[1] = d.second;
    }
    E.row(dof, g, 2, 0.0);
  }
  // CD2 contact rows (:422-468) on nodes without EOL
  for (int c = 0; c < n_contacts; ++c) {
    const eolc_contact &C = contacts[c];
    int nv;
    bool weighted;
    const double *nor;
    if (C.count1 == 3 && C.count2 == 1) {
      nv = 1, nor = C.nor1, weighted = false;
    } else if (C.count1 == 2 && C.count2 == 2) {
      nv = 2, nor = C.nor2, weighted = true;
    } else if (C.count1 == 1 && C.count2 == 3) {
      nv = 3, nor = C.nor2, weighted = true;
    } else {
      continue;
    }
    bool skip = false;
    for (int j = 0; j < nv; ++j) {
      const int a = C.verts2[j];
      if (a < 0 || a >= N) return bad("contact vertex out of range");
      skip = skip || eol_index[a] >= 0;
    }
    if (skip) continue;
    int dof[9];
    double val[9];
    for (int j = 0; j < nv; ++j)
      for (int i = 0; i < 3; ++i) {
        dof[3 * j + i] = 3 * C.verts2[j] + i;
        val[3 * j + i] = weighted ? -nor[i] * C.weights2[j] : -nor[i];
      }
    I.row(dof, val, 3 * nv, 0.0);
  }
  eq->n_rows = E.m;
  ineq->n_rows = I.m;
  return (E.m > eq->capacity || I.m > ineq->capacity) ? EOLC_CAPACITY : EOLC_OK;
}
