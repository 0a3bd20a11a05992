// C-linkage shim around the reference's own element and ray-triangle routines.
//
// This file contains no reference code.  It declares the reference functions
// with their published signatures and re-exports them under extern "C" names
// so that ctypes (tests/golden/make_golden.py) can call them.  It is linked
// against the reference sources compiled in place by oracle/build_ref.sh:
//   src/ComputeMembrane.cpp  (ComputeMembrane.h:5-19)
//   src/ComputeBending.cpp   (ComputeBending.h:5-18)
//   src/ComputeInertial.cpp  (ComputeInertial.h:5-17)
//   src/raytri.cpp           (intersect_triangle3_inc, raytri.cpp:261-316)
// The resulting library lives only in oracle/_ref/ and is test infrastructure:
// it generates the committed golden vectors and cross-checks the oracle.

void ComputeMembrane(const double *xa, const double *xb, const double *xc,
                     const double *Xa, const double *Xb, const double *Xc,
                     double e, double nu, const double *P, const double *Q,
                     double *W, double *f, double *K);
void ComputeBending(const double *x0, const double *x1, const double *x2,
                    const double *x3, const double *X0, const double *X1,
                    const double *X2, const double *X3, double beta,
                    double *W, double *f, double *K);
void ComputeInertial(const double *xa, const double *xb, const double *xc,
                     const double *Xa, const double *Xb, const double *Xc,
                     const double *g, double rho, double *W, double *f,
                     double *M);
int intersect_triangle3_inc(const double *orig, const double *dir,
                            const double *vert0, const double *vert1,
                            const double *vert2, double *t, double *u,
                            double *v);

extern "C" {

void ref_membrane(const double *x9, const double *X6, double e, double nu,
                  const double *P6, const double *Q4, double *W, double *f9,
                  double *K81) {
  ComputeMembrane(x9, x9 + 3, x9 + 6, X6, X6 + 2, X6 + 4, e, nu, P6, Q4, W, f9,
                  K81);
}

void ref_bending(const double *x12, const double *X8, double beta, double *W,
                 double *f12, double *K144) {
  ComputeBending(x12, x12 + 3, x12 + 6, x12 + 9, X8, X8 + 2, X8 + 4, X8 + 6,
                 beta, W, f12, K144);
}

void ref_inertial(const double *x9, const double *X6, const double *g,
                  double rho, double *W, double *f9, double *M81) {
  ComputeInertial(x9, x9 + 3, x9 + 6, X6, X6 + 2, X6 + 4, g, rho, W, f9, M81);
}

int ref_raytri(const double *orig, const double *dir, const double *v0,
               const double *v1, const double *v2, double *tuv) {
  return intersect_triangle3_inc(orig, dir, v0, v1, v2, tuv, tuv + 1, tuv + 2);
}
}
