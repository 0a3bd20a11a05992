// Device element math for the cloth energies, templated on the arithmetic
// type (double for the FP64 path, float for the mixed-precision path).
//
// Energies (same as the reference's generated routines, in closed form):
//  membrane  ComputeMembrane.cpp:2-320   W = A (mu |S|^2 + lambda/2 tr(S)^2),
//            S = R^T Fm - I, R = P^T Q fixed (co-rotated frame of
//            Forces.cpp:355-368), Fm = sum_v x_v g_v^T;
//            f_v = -R Pk g_v, Pk = A (2 mu S + lambda tr S I);
//            K_vw = A (2 mu (g_v.g_w) R R^T + lambda (R g_v)(R g_w)^T).
//  inertia   ComputeInertial.cpp:2-136   t8 = rho 2A; f_v = t8 g / 6;
//            M_vv = t8/12 I, M_vw = t8/24 I.
//  bending   ComputeBending.cpp:15-738   W = c (1 - u.w), u, w unit normals
//            of (x0,x1,x2) and (x1,x0,x3), c = 3 beta |X1-X0|^2 /
//            cross2(X1-X0, X2-X3); K = d2W/dx2 assembled block by block from
//            the Jacobians dn/dx = [s]x and the Hessian of u.w in (n0, n1).
//
// Edge vectors are formed from FP64 positions before any rounding to the
// arithmetic type, so the FP32 path keeps full FP32 relative precision of
// the element shape even when |x| >> element size.
#pragma once

#include <cuda_runtime.h>

namespace eolc {

template <typename T>
struct v3 {
  T x, y, z;
};

template <typename T>
__device__ __forceinline__ v3<T> mk3(T a, T b, T c) {
  return v3<T>{a, b, c};
}
template <typename T>
__device__ __forceinline__ v3<T> operator+(v3<T> a, v3<T> b) {
  return mk3(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename T>
__device__ __forceinline__ v3<T> operator-(v3<T> a, v3<T> b) {
  return mk3(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <typename T>
__device__ __forceinline__ v3<T> operator-(v3<T> a) {
  return mk3(-a.x, -a.y, -a.z);
}
template <typename T>
__device__ __forceinline__ v3<T> operator*(T s, v3<T> a) {
  return mk3(s * a.x, s * a.y, s * a.z);
}
template <typename T>
__device__ __forceinline__ T dot(v3<T> a, v3<T> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
__device__ __forceinline__ v3<T> cross(v3<T> a, v3<T> b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z,
             a.x * b.y - a.y * b.x);
}
template <typename T>
__device__ __forceinline__ T comp(v3<T> a, int i) {
  return i == 0 ? a.x : (i == 1 ? a.y : a.z);
}

__device__ __forceinline__ float rsqrt_t(float a) { return rsqrtf(a); }
__device__ __forceinline__ double rsqrt_t(double a) { return rsqrt(a); }

// Difference of two FP64 node positions, rounded once to T.
template <typename T>
__device__ __forceinline__ v3<T> dpos(const double *x, int i, int j) {
  return mk3<T>(T(x[3 * i] - x[3 * j]), T(x[3 * i + 1] - x[3 * j + 1]),
                T(x[3 * i + 2] - x[3 * j + 2]));
}

// ---------------------------------------------------------------------------
// Triangle: co-rotated frame, strain, gradients.
template <typename T>
struct Tri {
  T A;          // signed material area
  T g[3][2];    // gradients of the linear shape functions (material space)
  T R[3][2];    // P^T Q
  T S[2][2];    // strain R^T Fm - I
};

// Material-space part of face (a, b, c): signed area and shape-function
// gradients (depend on X only, so they can be computed once per topology).
template <typename T>
struct TriGeo {
  T A;
  T g[3][2];
};
template <typename T>
__device__ __forceinline__ TriGeo<T> make_tri_geo(const double *X, int a, int b, int c) {
  TriGeo<T> q;
  T d00 = T(X[2 * b] - X[2 * a]), d10 = T(X[2 * b + 1] - X[2 * a + 1]);
  T d01 = T(X[2 * c] - X[2 * a]), d11 = T(X[2 * c + 1] - X[2 * a + 1]);
  T t7 = d00 * d11 - d01 * d10;
  q.A = t7 / T(2);
  T it7 = T(1) / t7;
  q.g[1][0] = d11 * it7;
  q.g[1][1] = -d01 * it7;
  q.g[2][0] = -d10 * it7;
  q.g[2][1] = d00 * it7;
  q.g[0][0] = -q.g[1][0] - q.g[2][0];
  q.g[0][1] = -q.g[1][1] - q.g[2][1];
  return q;
}

// The triangle quantities from the edge vectors e0 = x_b - x_a, e1 = x_c -
// x_a and the material-space part.  Follows the frame of faceBasedF
// (Forces.cpp:355-368) and poldec (Forces.cpp:33-52).
template <typename T>
__device__ __forceinline__ Tri<T> make_tri_from(v3<T> e0, v3<T> e1, const TriGeo<T> &geo) {
  Tri<T> q;
  q.A = geo.A;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    q.g[v][0] = geo.g[v][0];
    q.g[v][1] = geo.g[v][1];
  }
  // Fm = e0 gb^T + e1 gc^T (3x2)
  v3<T> F0 = q.g[1][0] * e0 + q.g[2][0] * e1;
  v3<T> F1 = q.g[1][1] * e0 + q.g[2][1] * e1;
  // P rows: px = e0/|e0|, py = (n x px)/|n x px|
  v3<T> n = cross(e0, e1);
  v3<T> px = rsqrt_t(dot(e0, e0)) * e0;
  v3<T> py = cross(n, px);
  py = rsqrt_t(dot(py, py)) * py;
  // Fbar = P Fm, Q = poldec(Fbar)
  T m11 = dot(px, F0), m12 = dot(px, F1), m21 = dot(py, F0), m22 = dot(py, F1);
  T det = m11 * m22 - m12 * m21;
  T sg = det < T(0) ? T(-1) : (det == T(0) ? T(0) : T(1));
  T q00 = m11 + sg * m22, q10 = m21 - sg * m12;
  T q01 = m12 - sg * m21, q11 = m22 + sg * m11;
  T il = rsqrt_t(q00 * q00 + q10 * q10);
  q00 *= il; q10 *= il; q01 *= il; q11 *= il;
  // R = P^T Q
  q.R[0][0] = px.x * q00 + py.x * q10; q.R[0][1] = px.x * q01 + py.x * q11;
  q.R[1][0] = px.y * q00 + py.y * q10; q.R[1][1] = px.y * q01 + py.y * q11;
  q.R[2][0] = px.z * q00 + py.z * q10; q.R[2][1] = px.z * q01 + py.z * q11;
  // S = R^T Fm - I
  v3<T> r0 = mk3(q.R[0][0], q.R[1][0], q.R[2][0]);
  v3<T> r1 = mk3(q.R[0][1], q.R[1][1], q.R[2][1]);
  q.S[0][0] = dot(r0, F0) - T(1);
  q.S[0][1] = dot(r0, F1);
  q.S[1][0] = dot(r1, F0);
  q.S[1][1] = dot(r1, F1) - T(1);
  return q;
}

// Builds the triangle quantities for face (a, b, c) from the node positions.
template <typename T>
__device__ __forceinline__ Tri<T> make_tri(const double *x, const double *X,
                                           int a, int b, int c) {
  return make_tri_from<T>(dpos<T>(x, b, a), dpos<T>(x, c, a), make_tri_geo<T>(X, a, b, c));
}

// Membrane stiffness block K_{la,lb} (3x3, row-major) added into acc with
// weight s.
template <typename T, typename A>
__device__ __forceinline__ void add_membrane_block(const Tri<T> &q, int la,
                                                   int lb, T mu, T lam, T s,
                                                   A *acc) {
  T gg = q.g[la][0] * q.g[lb][0] + q.g[la][1] * q.g[lb][1];
  T Rga[3], Rgb[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    Rga[r] = q.R[r][0] * q.g[la][0] + q.R[r][1] * q.g[la][1];
    Rgb[r] = q.R[r][0] * q.g[lb][0] + q.R[r][1] * q.g[lb][1];
  }
  T c1 = s * q.A * T(2) * mu * gg, c2 = s * q.A * lam;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T RR = q.R[r][0] * q.R[k][0] + q.R[r][1] * q.R[k][1];
      acc[3 * r + k] += A(c1 * RR + c2 * Rga[r] * Rgb[k]);
    }
}

// Membrane force on local vertex la: f = -R Pk g_la.
template <typename T>
__device__ __forceinline__ v3<T> membrane_force(const Tri<T> &q, int la, T mu,
                                                T lam) {
  T tr = q.S[0][0] + q.S[1][1];
  T P00 = q.A * (T(2) * mu * q.S[0][0] + lam * tr);
  T P01 = q.A * (T(2) * mu * q.S[0][1]);
  T P10 = q.A * (T(2) * mu * q.S[1][0]);
  T P11 = q.A * (T(2) * mu * q.S[1][1] + lam * tr);
  T pg0 = P00 * q.g[la][0] + P01 * q.g[la][1];
  T pg1 = P10 * q.g[la][0] + P11 * q.g[la][1];
  return mk3<T>(-(q.R[0][0] * pg0 + q.R[0][1] * pg1),
                -(q.R[1][0] * pg0 + q.R[1][1] * pg1),
                -(q.R[2][0] * pg0 + q.R[2][1] * pg1));
}

// ---------------------------------------------------------------------------
// Hinge
template <typename T>
struct Hinge {
  T c, ir0, ir1, phi;
  v3<T> u, w, pw, pu, a, b;
  v3<T> p, q, qq;  // x1-x0, x2-x0, x3-x1
};

// Material-space part of a hinge: c = 3 beta |X1 - X0|^2 / cross2(X1 - X0,
// X2 - X3) as c_geo beta (X only: once per topology).
template <typename T>
__device__ __forceinline__ T hinge_geo(const double *X, int i0, int i1, int i2, int i3) {
  T dXx = T(X[2 * i1] - X[2 * i0]), dXy = T(X[2 * i1 + 1] - X[2 * i0 + 1]);
  T c2 = dXx * T(X[2 * i2 + 1] - X[2 * i3 + 1]) -
         dXy * T(X[2 * i2] - X[2 * i3]);
  return T(3) * (dXx * dXx + dXy * dXy) / c2;
}

// The hinge quantities from p = x1 - x0, q = x2 - x0, qq = x3 - x1 and c.
template <typename T>
__device__ __forceinline__ Hinge<T> make_hinge_from(v3<T> p, v3<T> q, v3<T> qq, T c) {
  Hinge<T> H;
  H.c = c;
  H.p = p;
  H.q = q;
  H.qq = qq;
  v3<T> n0 = cross(H.p, H.q), n1 = cross(-H.p, H.qq);
  H.ir0 = rsqrt_t(dot(n0, n0));
  H.ir1 = rsqrt_t(dot(n1, n1));
  H.u = H.ir0 * n0;
  H.w = H.ir1 * n1;
  H.phi = dot(H.u, H.w);
  H.pw = H.w - H.phi * H.u;
  H.pu = H.u - H.phi * H.w;
  H.a = H.ir0 * H.pw;
  H.b = H.ir1 * H.pu;
  return H;
}

template <typename T>
__device__ __forceinline__ Hinge<T> make_hinge(const double *x,
                                               const double *X, int i0, int i1,
                                               int i2, int i3, T beta) {
  T dXx = T(X[2 * i1] - X[2 * i0]), dXy = T(X[2 * i1 + 1] - X[2 * i0 + 1]);
  T c2 = dXx * T(X[2 * i2 + 1] - X[2 * i3 + 1]) -
         dXy * T(X[2 * i2] - X[2 * i3]);
  return make_hinge_from<T>(dpos<T>(x, i1, i0), dpos<T>(x, i2, i0), dpos<T>(x, i3, i1),
                            T(3) * beta * (dXx * dXx + dXy * dXy) / c2);
}

// Jacobian vectors: dn0/dx_v = [s0_v]x, dn1/dx_v = [s1_v]x.
template <typename T>
__device__ __forceinline__ v3<T> hinge_s0(const Hinge<T> &H, int v) {
  // n0 = p x q, p = x1 - x0, q = x2 - x0
  return v == 0 ? H.q - H.p : (v == 1 ? -H.q : (v == 2 ? H.p : mk3<T>(0, 0, 0)));
}
template <typename T>
__device__ __forceinline__ v3<T> hinge_s1(const Hinge<T> &H, int v) {
  // n1 = pp x qq, pp = x0 - x1 = -p, qq = x3 - x1
  return v == 0 ? -H.qq : (v == 1 ? H.qq + H.p : (v == 3 ? -H.p : mk3<T>(0, 0, 0)));
}

// acc += s * M with M(i,j) = al * I + sum of outer products, helper:
template <typename T, typename A>
__device__ __forceinline__ void add_outer(A *acc, T s, v3<T> l, v3<T> r) {
  acc[0] += A(s * l.x * r.x); acc[1] += A(s * l.x * r.y); acc[2] += A(s * l.x * r.z);
  acc[3] += A(s * l.y * r.x); acc[4] += A(s * l.y * r.y); acc[5] += A(s * l.y * r.z);
  acc[6] += A(s * l.z * r.x); acc[7] += A(s * l.z * r.y); acc[8] += A(s * l.z * r.z);
}

// Bending stiffness block K_{v,w} = -c * d2(u.w)/dx_v dx_w, times s, into acc.
// Uses [s]x^T (a b^T) [t]x = (a x s)(b x t)^T and
//      [s]x^T [t]x = (s.t) I - t s^T.
template <typename T, typename A>
__device__ __forceinline__ void add_bending_block(const Hinge<T> &H, int v,
                                                  int wv, T s, A *acc) {
  const T k = -s * H.c;  // K = -c * Hessian(phi)
  v3<T> s0v = hinge_s0(H, v), s1v = hinge_s1(H, v);
  v3<T> s0w = hinge_s0(H, wv), s1w = hinge_s1(H, wv);
  T i00 = -H.ir0 * H.ir0, i11 = -H.ir1 * H.ir1, i01 = H.ir0 * H.ir1;
  T phi = H.phi;
  // cross products on each side
  v3<T> u0v = cross(H.u, s0v), w0v = cross(H.w, s0v), pw0v = cross(H.pw, s0v);
  v3<T> u1v = cross(H.u, s1v), w1v = cross(H.w, s1v), pu1v = cross(H.pu, s1v);
  v3<T> u0w = cross(H.u, s0w), w0w = cross(H.w, s0w), pw0w = cross(H.pw, s0w);
  v3<T> u1w = cross(H.u, s1w), w1w = cross(H.w, s1w), pu1w = cross(H.pu, s1w);
  // identity and t s^T parts: T00: i00*phi*(st I - t s^T); T11: i11*phi*(..)
  // T01 / T10: i01*(st I - t s^T)
  T st00 = dot(s0v, s0w), st11 = dot(s1v, s1w), st01 = dot(s0v, s1w),
    st10 = dot(s1v, s0w);
  T diag = k * (i00 * phi * st00 + i11 * phi * st11 + i01 * (st01 + st10));
  acc[0] += A(diag); acc[4] += A(diag); acc[8] += A(diag);
  add_outer(acc, -k * i00 * phi, s0w, s0v);
  add_outer(acc, -k * i11 * phi, s1w, s1v);
  add_outer(acc, -k * i01, s1w, s0v);
  add_outer(acc, -k * i01, s0w, s1v);
  // T00 = i00 [ ... - phi us ut^T + us (pw x t)^T + (pw x s) ut^T ]
  add_outer(acc, -k * i00 * phi, u0v, u0w);
  add_outer(acc, k * i00, u0v, pw0w);
  add_outer(acc, k * i00, pw0v, u0w);
  // T11 with (w, pu)
  add_outer(acc, -k * i11 * phi, w1v, w1w);
  add_outer(acc, k * i11, w1v, pu1w);
  add_outer(acc, k * i11, pu1v, w1w);
  // T01(s0v, s1w) = i01 [ - us ut^T - ws wt^T + phi us wt^T ]
  add_outer(acc, -k * i01, u0v, u1w);
  add_outer(acc, -k * i01, w0v, w1w);
  add_outer(acc, k * i01 * phi, u0v, w1w);
  // T10(s1v, s0w) = i01 [ - us ut^T - ws wt^T + phi ws ut^T ]
  add_outer(acc, -k * i01, u1v, u0w);
  add_outer(acc, -k * i01, w1v, w0w);
  add_outer(acc, k * i01 * phi, w1v, u0w);
  // cross-product curvature terms: k0 [a]x + k1 [b]x
  const int cP0[4] = {-1, 1, 0, 0}, cQ0[4] = {-1, 0, 1, 0};
  const int cP1[4] = {1, -1, 0, 0}, cQ1[4] = {0, -1, 0, 1};
  T k0 = T(cQ0[v] * cP0[wv] - cP0[v] * cQ0[wv]);
  T k1 = T(cQ1[v] * cP1[wv] - cP1[v] * cQ1[wv]);
  v3<T> sk = k0 * H.a + k1 * H.b;
  // [sk]x = [[0,-z,y],[z,0,-x],[-y,x,0]]
  acc[1] += A(k * -sk.z); acc[2] += A(k * sk.y);
  acc[3] += A(k * sk.z);  acc[5] += A(k * -sk.x);
  acc[6] += A(k * -sk.y); acc[7] += A(k * sk.x);
}

}  // namespace eolc

namespace eolc {

// ---------------------------------------------------------------------------
// The bending blocks of one hinge row, grouped for the row-task assembly.
// K_vw = k H_vw with k = -s c and H_vw = Hessian of n0^.n1^ (add_bending_block
// above), written as sums of outer products grouped by their left vector:
//   H_vw = d I + U0v R1w' + PW0v R2w' + W1v R3w' + PU1v R4w' + U1v R5w'
//        + W0v R6w' + s0w T0v' + s1w T1v' + [k0 a + k1 b]x
// with, per vertex x, the Jacobian vectors s0x, s1x, the crosses U0x = u x
// s0x, PW0x = pw x s0x, W0x = w x s0x, U1x = u x s1x, W1x = w x s1x, PU1x =
// pu x s1x, and
//   R1x = i00 (PW0x - phi U0x) + i01 (phi W1x - U1x)   R2x = i00 U0x
//   R3x = i11 (PU1x - phi W1x) + i01 (phi U0x - W0x)   R4x = i11 W1x
//   R5x = -i01 U0x    R6x = -i01 W1x
//   T0x = -i00 phi s0x - i01 s1x    T1x = -i11 phi s1x - i01 s0x
//   d = i00 phi s0v.s0w + i11 phi s1v.s1w + i01 (s0v.s1w + s1v.s0w).
// Eight outer products per block on vectors computed once per vertex (the
// expanded form has sixteen and recomputes the crosses per block); the
// terms are the same, reassociated.
template <typename T>
struct BendLeft {  // what vertex v contributes as the block's row side
  v3<T> s0, s1, U0, PW0, W1, PU1, U1, W0;
};
template <typename T>
struct BendRight {  // what vertex w contributes as the block's column side
  v3<T> s0, s1, R1, R2, R3, R4, R5, R6;
};

template <typename T, int V>
__device__ __forceinline__ BendLeft<T> bend_left(const Hinge<T> &H) {
  BendLeft<T> L;
  L.s0 = hinge_s0(H, V);
  L.s1 = hinge_s1(H, V);
  L.U0 = cross(H.u, L.s0);
  L.PW0 = cross(H.pw, L.s0);
  L.W0 = cross(H.w, L.s0);
  L.U1 = cross(H.u, L.s1);
  L.W1 = cross(H.w, L.s1);
  L.PU1 = cross(H.pu, L.s1);
  return L;
}

template <typename T, int W>
__device__ __forceinline__ BendRight<T> bend_right(const Hinge<T> &H) {
  const T i00 = -H.ir0 * H.ir0, i11 = -H.ir1 * H.ir1, i01 = H.ir0 * H.ir1, phi = H.phi;
  BendRight<T> R;
  R.s0 = hinge_s0(H, W);
  R.s1 = hinge_s1(H, W);
  const v3<T> U0 = cross(H.u, R.s0), PW0 = cross(H.pw, R.s0), W0 = cross(H.w, R.s0);
  const v3<T> U1 = cross(H.u, R.s1), W1 = cross(H.w, R.s1), PU1 = cross(H.pu, R.s1);
  R.R1 = i00 * (PW0 - phi * U0) + i01 * (phi * W1 - U1);
  R.R2 = i00 * U0;
  R.R3 = i11 * (PU1 - phi * W1) + i01 * (phi * U0 - W0);
  R.R4 = i11 * W1;
  R.R5 = -i01 * U0;
  R.R6 = -i01 * W1;
  return R;
}

template <typename T>
__device__ __forceinline__ void outer_add(T *o, v3<T> l, v3<T> r) {
  o[0] += l.x * r.x; o[1] += l.x * r.y; o[2] += l.x * r.z;
  o[3] += l.y * r.x; o[4] += l.y * r.y; o[5] += l.y * r.z;
  o[6] += l.z * r.x; o[7] += l.z * r.y; o[8] += l.z * r.z;
}

// K_vw (3x3, row-major) times s into blk (overwritten).
template <typename T, int V, int W>
__device__ __forceinline__ void bend_block(const Hinge<T> &H, const BendLeft<T> &L,
                                           const BendRight<T> &R, T s, T *blk) {
  const T i00 = -H.ir0 * H.ir0, i11 = -H.ir1 * H.ir1, i01 = H.ir0 * H.ir1, phi = H.phi;
  const v3<T> T0 = (-i00 * phi) * L.s0 - i01 * L.s1;
  const v3<T> T1 = (-i11 * phi) * L.s1 - i01 * L.s0;
  const T d = i00 * phi * dot(L.s0, R.s0) + i11 * phi * dot(L.s1, R.s1) +
              i01 * (dot(L.s0, R.s1) + dot(L.s1, R.s0));
  T h[9] = {d, T(0), T(0), T(0), d, T(0), T(0), T(0), d};
  outer_add(h, L.U0, R.R1);
  outer_add(h, L.PW0, R.R2);
  outer_add(h, L.W1, R.R3);
  outer_add(h, L.PU1, R.R4);
  outer_add(h, L.U1, R.R5);
  outer_add(h, L.W0, R.R6);
  outer_add(h, R.s0, T0);
  outer_add(h, R.s1, T1);
  // curvature terms k0 [a]x + k1 [b]x (the vertex pattern of add_bending_block)
  constexpr int cP0[4] = {-1, 1, 0, 0}, cQ0[4] = {-1, 0, 1, 0};
  constexpr int cP1[4] = {1, -1, 0, 0}, cQ1[4] = {0, -1, 0, 1};
  constexpr int k0 = cQ0[V] * cP0[W] - cP0[V] * cQ0[W];
  constexpr int k1 = cQ1[V] * cP1[W] - cP1[V] * cQ1[W];
  const v3<T> sk = T(k0) * H.a + T(k1) * H.b;
  h[1] -= sk.z; h[2] += sk.y;
  h[3] += sk.z; h[5] -= sk.x;
  h[6] -= sk.y; h[7] += sk.x;
  const T k = -s * H.c;
#pragma unroll
  for (int q = 0; q < 9; ++q) blk[q] = k * h[q];
}

}  // namespace eolc
