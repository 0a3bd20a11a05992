// Oracle element routines (test infrastructure; see oracle.h).
//
// These restate the energies that the reference's Maple-generated routines
// differentiate, in closed form:
//
//  Membrane (ComputeMembrane.cpp:2-320): co-rotated St.Venant-Kirchhoff-type
//    energy with the rotation R = P^T Q held fixed,
//      Fm = sum_v x_v g_v^T,  g_v = rows of inv([Xb-Xa, Xc-Xa]) (ga = -gb-gc)
//      S  = R^T Fm - I,  W = A (mu |S|^2 + lambda/2 tr(S)^2),
//      A  = signed material area, mu = E/(2(1+nu)),
//      lambda = E nu / ((1+nu)(1-2nu)),
//    so f_v = -R Pk g_v with Pk = A (2 mu S + lambda tr(S) I) and the
//    (exactly quadratic) Hessian
//      K_vw = A (2 mu (g_v.g_w) R R^T + lambda (R g_v)(R g_w)^T).
//  Inertial (ComputeInertial.cpp:2-136): t8 = rho * 2A (signed),
//    f_v = t8 g / 6, M_vv = t8/12 I, M_vw = t8/24 I.
//  Bending (ComputeBending.cpp:15-738): hinge energy
//      W = c (1 - n0^.n1^),  c = 3 beta |X1-X0|^2 / cross2(X1-X0, X2-X3),
//    n0 = (x1-x0)x(x2-x0), n1 = (x0-x1)x(x3-x1); f = -dW/dx, K = d2W/dx2
//    (full Hessian, including the terms from the second derivatives of
//    the cross products).
// The closed forms were derived independently of the generated code and
// agree with it to rounding (tests/golden KATs).
#include <cmath>

#include "oracle.h"
#include "vec3.h"

using orc::V3;

namespace {

struct M3 {
  double m[3][3];
};

M3 skew(const V3 &a) {
  M3 s;
  s.m[0][0] = 0;     s.m[0][1] = -a[2]; s.m[0][2] = a[1];
  s.m[1][0] = a[2];  s.m[1][1] = 0;     s.m[1][2] = -a[0];
  s.m[2][0] = -a[1]; s.m[2][1] = a[0];  s.m[2][2] = 0;
  return s;
}

M3 mul(const M3 &A, const M3 &B) {
  M3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += A.m[i][k] * B.m[k][j];
      C.m[i][j] = s;
    }
  return C;
}

M3 transpose(const M3 &A) {
  M3 T;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T.m[i][j] = A.m[j][i];
  return T;
}

// 2x2 polar factor exactly as poldec (Forces.cpp:33-52): Q = M + sign(det M)
// * [[m22, -m21], [-m12, m11]], then Q /= |Q col 0|.  Column-major output.
void poldec(const double F[2][2], double Q[4]) {
  double m11 = F[0][0], m12 = F[0][1], m21 = F[1][0], m22 = F[1][1];
  double det = m11 * m22 - m12 * m21;
  int sign = det < 0 ? -1 : (det == 0 ? 0 : 1);
  double q00 = m11 + sign * m22, q01 = m12 + sign * -m21;
  double q10 = m21 + sign * -m12, q11 = m22 + sign * m11;
  double clen = std::sqrt(q00 * q00 + q10 * q10);
  Q[0] = q00 / clen;
  Q[1] = q10 / clen;
  Q[2] = q01 / clen;
  Q[3] = q11 / clen;
}

}  // namespace

extern "C" {

// Face frame of faceBasedF (Forces.cpp:355-368): P rows are the unit edge
// ab and (n x ab) normalised; Fbar = P Dx inv(DX); Q = poldec(Fbar).
void orc_face_frame(const double *x9, const double *X6, double *P6,
                    double *Q4) {
  V3 xa = orc::ld(x9), xb = orc::ld(x9 + 3), xc = orc::ld(x9 + 6);
  V3 e0 = xb - xa, e1 = xc - xa;
  V3 n = orc::cross(e0, e1);
  V3 px = e0 / orc::norm(e0);
  V3 py = orc::cross(n, px);
  py = py / orc::norm(py);
  double d00 = X6[2] - X6[0], d01 = X6[4] - X6[0];
  double d10 = X6[3] - X6[1], d11 = X6[5] - X6[1];
  double det = d00 * d11 - d10 * d01;
  double i00 = d11 / det, i01 = -d01 / det, i10 = -d10 / det, i11 = d00 / det;
  double Fm[3][2];
  for (int r = 0; r < 3; ++r) {
    Fm[r][0] = e0[r] * i00 + e1[r] * i10;
    Fm[r][1] = e0[r] * i01 + e1[r] * i11;
  }
  double Fb[2][2];
  for (int k = 0; k < 2; ++k) {
    Fb[0][k] = (px[0] * Fm[0][k] + px[1] * Fm[1][k]) + px[2] * Fm[2][k];
    Fb[1][k] = (py[0] * Fm[0][k] + py[1] * Fm[1][k]) + py[2] * Fm[2][k];
  }
  // P (2x3) column-major
  for (int c = 0; c < 3; ++c) {
    P6[2 * c + 0] = px[c];
    P6[2 * c + 1] = py[c];
  }
  poldec(Fb, Q4);
}

void orc_membrane(const double *x9, const double *X6, double e, double nu,
                  const double *P6, const double *Q4, double *W, double *f9,
                  double *K81) {
  double Xax = X6[0], Xay = X6[1], Xbx = X6[2], Xby = X6[3], Xcx = X6[4],
         Xcy = X6[5];
  double t7 = (Xbx - Xax) * (Xcy - Xay) - (Xcx - Xax) * (Xby - Xay);
  double A = t7 / 2;
  double mu = e / (1 + nu) / 2;
  double lam = e * nu / ((1 + nu) * (1 - 2 * nu));
  // g_v: rows of inv([Xb-Xa, Xc-Xa])
  double g[3][2];
  g[1][0] = (Xcy - Xay) / t7;
  g[1][1] = -(Xcx - Xax) / t7;
  g[2][0] = -(Xby - Xay) / t7;
  g[2][1] = (Xbx - Xax) / t7;
  g[0][0] = -g[1][0] - g[2][0];
  g[0][1] = -g[1][1] - g[2][1];
  // R = P^T Q (3x2); P, Q column-major
  double R[3][2];
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 2; ++k)
      R[a][k] = P6[2 * a + 0] * Q4[2 * k + 0] + P6[2 * a + 1] * Q4[2 * k + 1];
  // Fm = sum_v x_v g_v^T (3x2), G = R^T Fm (2x2)
  double Fm[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  for (int v = 0; v < 3; ++v)
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 2; ++k) Fm[r][k] += x9[3 * v + r] * g[v][k];
  double S[2][2];
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 2; ++k)
      S[i][k] = (R[0][i] * Fm[0][k] + R[1][i] * Fm[1][k] + R[2][i] * Fm[2][k]) -
                (i == k ? 1.0 : 0.0);
  double tr = S[0][0] + S[1][1];
  double ss = S[0][0] * S[0][0] + S[0][1] * S[0][1] + S[1][0] * S[1][0] +
              S[1][1] * S[1][1];
  *W = A * (mu * ss + lam / 2 * tr * tr);
  double Pk[2][2];
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 2; ++k)
      Pk[i][k] = A * (2 * mu * S[i][k] + (i == k ? lam * tr : 0.0));
  // Rg_v = R g_v, f_v = -R Pk g_v
  double Rg[3][3];
  for (int v = 0; v < 3; ++v) {
    double pg0 = Pk[0][0] * g[v][0] + Pk[0][1] * g[v][1];
    double pg1 = Pk[1][0] * g[v][0] + Pk[1][1] * g[v][1];
    for (int a = 0; a < 3; ++a) {
      f9[3 * v + a] = -(R[a][0] * pg0 + R[a][1] * pg1);
      Rg[v][a] = R[a][0] * g[v][0] + R[a][1] * g[v][1];
    }
  }
  double RR[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) RR[a][b] = R[a][0] * R[b][0] + R[a][1] * R[b][1];
  for (int v = 0; v < 3; ++v)
    for (int w = 0; w < 3; ++w) {
      double gg = g[v][0] * g[w][0] + g[v][1] * g[w][1];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          K81[(3 * v + a) * 9 + 3 * w + b] =
              A * (2 * mu * gg * RR[a][b] + lam * Rg[v][a] * Rg[w][b]);
    }
}

void orc_inertial(const double *x9, const double *X6, const double *g,
                  double rho, double *W, double *f9, double *M81) {
  double Xax = X6[0], Xay = X6[1], Xbx = X6[2], Xby = X6[3], Xcx = X6[4],
         Xcy = X6[5];
  double t8 = rho * ((Xbx - Xax) * (Xcy - Xay) - (Xcx - Xax) * (Xby - Xay));
  double gx = 0;
  for (int c = 0; c < 3; ++c)
    gx += g[c] * (x9[c] + x9[3 + c] + x9[6 + c]);
  *W = -t8 * gx / 6;
  for (int v = 0; v < 3; ++v)
    for (int c = 0; c < 3; ++c) f9[3 * v + c] = t8 * g[c] / 6;
  for (int i = 0; i < 81; ++i) M81[i] = 0;
  for (int v = 0; v < 3; ++v)
    for (int w = 0; w < 3; ++w)
      for (int c = 0; c < 3; ++c)
        M81[(3 * v + c) * 9 + 3 * w + c] = v == w ? t8 / 12 : t8 / 24;
}

void orc_bending(const double *x12, const double *X8, double beta, double *W,
                 double *f12, double *K144) {
  V3 x0 = orc::ld(x12), x1 = orc::ld(x12 + 3), x2 = orc::ld(x12 + 6),
     x3 = orc::ld(x12 + 9);
  double dXx = X8[2] - X8[0], dXy = X8[3] - X8[1];
  double c2 = dXx * (X8[5] - X8[7]) - dXy * (X8[4] - X8[6]);
  double c = 3 * beta * (dXx * dXx + dXy * dXy) / c2;
  V3 p = x1 - x0, q = x2 - x0, pp = x0 - x1, qq = x3 - x1;
  V3 n0 = orc::cross(p, q), n1 = orc::cross(pp, qq);
  double r0 = orc::norm(n0), r1 = orc::norm(n1);
  V3 u = n0 / r0, w = n1 / r1;
  double phi = orc::dot(u, w);
  *W = c * (1 - phi);
  // a = dphi/dn0 = (w - phi u)/r0, b = dphi/dn1 = (u - phi w)/r1
  V3 a = (w - phi * u) / r0, b = (u - phi * w) / r1;
  // Jacobians dn0/dx_v = [s0_v]x, dn1/dx_v = [s1_v]x
  V3 z = orc::mk(0, 0, 0);
  V3 s0[4] = {q - p, -q, p, z};
  V3 s1[4] = {-qq, qq - pp, z, pp};
  for (int v = 0; v < 4; ++v) {
    V3 gv = orc::cross(a, s0[v]) + orc::cross(b, s1[v]);
    for (int k = 0; k < 3; ++k) f12[3 * v + k] = c * gv[k];
  }
  // Second derivatives of phi w.r.t. (n0, n1)
  M3 H00, H11, H01;
  V3 Pw = w - phi * u;  // P0 w
  V3 Pu = u - phi * w;  // P1 u
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double d = i == j ? 1.0 : 0.0;
      double P0ij = d - u[i] * u[j], P1ij = d - w[i] * w[j];
      H00.m[i][j] = -(phi * P0ij + u[i] * Pw[j] + Pw[i] * u[j]) / (r0 * r0);
      H11.m[i][j] = -(phi * P1ij + w[i] * Pu[j] + Pu[i] * w[j]) / (r1 * r1);
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) {
        double P0ik = (i == k ? 1.0 : 0.0) - u[i] * u[k];
        double P1kj = (k == j ? 1.0 : 0.0) - w[k] * w[j];
        s += P0ik * P1kj;
      }
      H01.m[i][j] = s / (r0 * r1);
    }
  M3 H10 = transpose(H01);
  // Signs of x_v in p, q (part 0) and pp, qq (part 1).
  const double cP0[4] = {-1, 1, 0, 0}, cQ0[4] = {-1, 0, 1, 0};
  const double cP1[4] = {1, -1, 0, 0}, cQ1[4] = {0, -1, 0, 1};
  M3 Sa = skew(a), Sb = skew(b);
  for (int v = 0; v < 4; ++v) {
    M3 J0vT = transpose(skew(s0[v])), J1vT = transpose(skew(s1[v]));
    for (int wv = 0; wv < 4; ++wv) {
      M3 J0w = skew(s0[wv]), J1w = skew(s1[wv]);
      M3 t1 = mul(J0vT, mul(H00, J0w));
      M3 t2 = mul(J1vT, mul(H11, J1w));
      M3 t3 = mul(J0vT, mul(H01, J1w));
      M3 t4 = mul(J1vT, mul(H10, J0w));
      double k0 = cQ0[v] * cP0[wv] - cP0[v] * cQ0[wv];
      double k1 = cQ1[v] * cP1[wv] - cP1[v] * cQ1[wv];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double hphi = t1.m[i][j] + t2.m[i][j] + t3.m[i][j] + t4.m[i][j] +
                        k0 * Sa.m[i][j] + k1 * Sb.m[i][j];
          K144[(3 * v + i) * 12 + 3 * wv + j] = -c * hphi;
        }
    }
  }
}

// intersect_triangle3_inc (raytri.cpp:261-316), same operation order:
// accept when  u >= 1e-6, u <= det - 1e-6, v >= 1e-6, u + v <= det - 1e-6
// for det > 1e-6 (mirrored for det < -1e-6); t, u, v scaled by 1/det.
int orc_raytri(const double *orig, const double *dir, const double *v0,
               const double *v1, const double *v2, double *tuv) {
  const double EPS = 1e-6;
  double e1[3], e2[3], tv[3], pv[3], qv[3];
  for (int i = 0; i < 3; ++i) { e1[i] = v1[i] - v0[i]; e2[i] = v2[i] - v0[i]; }
  pv[0] = dir[1] * e2[2] - dir[2] * e2[1];
  pv[1] = dir[2] * e2[0] - dir[0] * e2[2];
  pv[2] = dir[0] * e2[1] - dir[1] * e2[0];
  double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  for (int i = 0; i < 3; ++i) tv[i] = orig[i] - v0[i];
  double inv_det = 1.0 / det;
  qv[0] = tv[1] * e1[2] - tv[2] * e1[1];
  qv[1] = tv[2] * e1[0] - tv[0] * e1[2];
  qv[2] = tv[0] * e1[1] - tv[1] * e1[0];
  double u, v;
  if (det > EPS) {
    u = tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2];
    if (u < EPS || u > det + -EPS) return 0;
    v = dir[0] * qv[0] + dir[1] * qv[1] + dir[2] * qv[2];
    if (v < EPS || u + v > det + -EPS) return 0;
  } else if (det < -EPS) {
    u = tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2];
    if (u > -EPS || u < det - -EPS) return 0;
    v = dir[0] * qv[0] + dir[1] * qv[1] + dir[2] * qv[2];
    if (v > -EPS || u + v < det - -EPS) return 0;
  } else {
    return 0;
  }
  tuv[0] = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv_det;
  tuv[1] = u * inv_det;
  tuv[2] = v * inv_det;
  return 1;
}

}  // extern "C"
