/*
 * femtech_oracle.c -- FP64 CPU restatement of FemTech's explicit-dynamics hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Never linked into the product
 * library.  Every routine names the reference file:line whose algorithm it
 * restates; operation order follows the reference where it is cheap to do so,
 * so that results agree with the reference build (oracle/_ref) to ~1e-14.
 *
 * Parity status: pinned against tests/golden/ (vectors produced by the
 * reference's own sources, see tests/golden/make_golden.py) for element types
 * C3D8/C3D4 and materials 0-5; materials 6 (Ogden) and 7 (anisotropic GOH +
 * 1-term Prony) are new and pinned through reductions to reference laws.
 *
 * Built with -ffp-contract=off so that x86-64 and aarch64 hosts agree bitwise.
 */
#include "femtech_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Gauss point coordinates of the 2x2x2 rule, in the order of
 * src/fem/ShapeFunctions/GaussQuadrature3D.cpp:17-58 (literal value as there). */
#define OR_G 0.577350269189626
static const double kHexGP[8][3] = {
    {-OR_G, -OR_G, OR_G}, {OR_G, -OR_G, OR_G}, {OR_G, OR_G, OR_G}, {-OR_G, OR_G, OR_G},
    {-OR_G, -OR_G, -OR_G}, {OR_G, -OR_G, -OR_G}, {OR_G, OR_G, -OR_G}, {-OR_G, OR_G, -OR_G}};
/* natural-coordinate signs of the C3D8 nodes (ShapeFunction_C3D8.cpp:26-33) */
static const double kHexSign[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

int or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_threads(or_model *m, int n) { m->nthreads = n > 0 ? n : 1; }

/* inverse3x3Matrix, src/math/math.cpp:8-28 (column-major in and out). */
static void or_inv3(const double *mat, double *inv, double *det) {
  double d = mat[0] * (mat[4] * mat[8] - mat[5] * mat[7]) -
             mat[3] * (mat[1] * mat[8] - mat[7] * mat[2]) +
             mat[6] * (mat[1] * mat[5] - mat[4] * mat[2]);
  double id = 1 / d;
  inv[0] = (mat[4] * mat[8] - mat[5] * mat[7]) * id;
  inv[3] = (mat[6] * mat[5] - mat[3] * mat[8]) * id;
  inv[6] = (mat[3] * mat[7] - mat[6] * mat[4]) * id;
  inv[1] = (mat[7] * mat[2] - mat[1] * mat[8]) * id;
  inv[4] = (mat[0] * mat[8] - mat[6] * mat[2]) * id;
  inv[7] = (mat[1] * mat[6] - mat[0] * mat[7]) * id;
  inv[2] = (mat[1] * mat[5] - mat[2] * mat[4]) * id;
  inv[5] = (mat[2] * mat[3] - mat[0] * mat[5]) * id;
  inv[8] = (mat[0] * mat[4] - mat[1] * mat[3]) * id;
  *det = d;
}

/* Column-major 3x3 products with the summation order of a plain
 * triple-loop dgemm: C(i,j) = alpha * sum_l opA(i,l) opB(l,j). */
static void or_gemm(int ta, int tb, double alpha, const double *A, const double *B,
                    double *C) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int l = 0; l < 3; ++l) {
        double a = ta ? A[l + 3 * i] : A[i + 3 * l];
        double b = tb ? B[j + 3 * l] : B[l + 3 * j];
        s += a * b;
      }
      C[i + 3 * j] = alpha * s;
    }
}

/* DeterminateF, src/math/DeterminateF.cpp:38-57. */
static double or_detF(const double *F) {
  double da = F[0], db = F[3], dc = F[6], dd = F[1], de = F[4], df = F[7], dg = F[2],
         dh = F[5], di = F[8];
  return da * (de * di - df * dh) - db * (dd * di - df * dg) + dc * (dd * dh - de * dg);
}

/* InverseF, src/math/InverseF.cpp:38-66: reads F as row-major and writes the
 * row-major inverse, so the column-major result is F^{-1}. */
static void or_invF(const double *F, double detA, double *fInv) {
  double A[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i][j] = F[3 * i + j];
  fInv[0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / detA;
  fInv[1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / detA;
  fInv[2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / detA;
  fInv[3] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / detA;
  fInv[4] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / detA;
  fInv[5] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / detA;
  fInv[6] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / detA;
  fInv[7] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / detA;
  fInv[8] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / detA;
}

/* Voigt [11,22,33,23,13,12] from a column-major 3x3 (upper triangle), the
 * storage order used by every material routine (e.g. HGOIsotropic.cpp:92-105). */
static void or_voigt(const double *S, double *v) {
  v[0] = S[0];
  v[1] = S[4];
  v[2] = S[8];
  v[3] = S[7];
  v[4] = S[6];
  v[5] = S[3];
}

/* CompressibleNeoHookean, src/materials/CompressibleNeoHookean.cpp:15-55. */
static void or_mat_nh(const double *pr, const double *F, double J, double *S6) {
  double mu = pr[1], lambda = pr[2], C[9], Ci[9], Cd;
  or_gemm(1, 0, 1.0, F, F, C);
  or_inv3(C, Ci, &Cd);
  double logJ = lambda * log(J);
  S6[0] = mu * (1.0 - Ci[0]) + logJ * Ci[0];
  S6[1] = mu * (1.0 - Ci[4]) + logJ * Ci[4];
  S6[2] = mu * (1.0 - Ci[8]) + logJ * Ci[8];
  S6[3] = -mu * Ci[7] + logJ * Ci[7];
  S6[4] = -mu * Ci[6] + logJ * Ci[6];
  S6[5] = -mu * Ci[3] + logJ * Ci[3];
}

/* StVenantKirchhoff, src/materials/StVenantKirchhoff.cpp:16-54. */
static void or_mat_svk(const double *pr, const double *F, double *S6) {
  double mu = pr[1], lambda = pr[2], E[9], S[9];
  or_gemm(1, 0, 0.5, F, F, E);
  E[0] -= 0.5;
  E[4] -= 0.5;
  E[8] -= 0.5;
  double tr = E[0] + E[4] + E[8];
  for (int i = 0; i < 9; ++i) S[i] = 2.0 * mu * E[i];
  S[0] += lambda * tr;
  S[4] += lambda * tr;
  S[8] += lambda * tr;
  or_voigt(S, S6);
}

/* LinearElastic, src/materials/LinearElastic.cpp:14-68 (S = F^{-1} P, upper
 * triangle stored even though S is not symmetric). */
static void or_mat_le(const double *pr, const double *F, double J, double *S6) {
  double mu = pr[1], lambda = pr[2], eps[9], P[9], fi[9], S[9];
  double trEps = F[0] + F[4] + F[8] - 3.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) eps[j + 3 * i] = F[j + 3 * i] + F[i + 3 * j];
  eps[0] -= 2.0;
  eps[4] -= 2.0;
  eps[8] -= 2.0;
  for (int i = 0; i < 9; ++i) P[i] = mu * eps[i];
  P[0] += lambda * trEps;
  P[4] += lambda * trEps;
  P[8] += lambda * trEps;
  or_invF(F, J, fi);
  or_gemm(0, 0, 1.0, fi, P, S);
  or_voigt(S, S6);
}

/* Cauchy -> PK2 pull-back S = J F^{-1} sigma F^{-T} (HGOIsotropic.cpp:80-90). */
static void or_pullback(const double *fInv, const double *sigma, double J, double *S) {
  double T[9];
  or_gemm(0, 0, 1.0, fInv, sigma, T);
  or_gemm(0, 1, J, T, fInv, S);
}

/* HGOIsotropic, src/materials/HGOIsotropic.cpp:21-115 (kappa = 1/3). */
static void or_mat_hgo(const double *pr, const double *F, double J, double *S6) {
  double mu = pr[1], lambda = pr[2], k1 = pr[3], k2 = pr[4];
  const double kappa = 1.0 / 3.0;
  double K = lambda + 2.0 * mu / 3.0;
  double hydro = 0.5 * K * (J * J - 1.0) / J;
  double B[9], fi[9], S[9];
  or_gemm(0, 1, 1.0, F, F, B);
  double trB = B[0] + B[4] + B[8];
  double Jm23 = pow(J, -2.0 / 3.0);
  double I1 = Jm23 * trB;
  double Ea = kappa * (I1 - 3.0);
  double fib = 0.0;
  if (Ea > 0.0) fib = 2.0 * k1 * exp(k2 * Ea * Ea) * Ea * kappa;
  double tp = Jm23 * (mu + fib) / J;
  double t3 = trB / 3.0;
  B[0] -= t3;
  B[4] -= t3;
  B[8] -= t3;
  for (int i = 0; i < 9; ++i) B[i] = B[i] * tp;
  B[0] += hydro;
  B[4] += hydro;
  B[8] += hydro;
  or_invF(F, J, fi);
  or_pullback(fi, B, J, S);
  or_voigt(S, S6);
}

/* Deviatoric split + Prony recurrence of HGOIsotropicViscoelastic.cpp:98-159,
 * for nterm terms (g,tau pairs in gt[]).  S (column-major) is updated in place. */
static void or_prony(const double *F, const double *fInv, int nterm, const double *gt,
                     double dt, double *hist27, double *S) {
  double C[9], Sic[9], Sdev[9];
  or_gemm(1, 0, 1.0, F, F, C);
  double SddC = 0.0;
  for (int i = 0; i < 9; ++i) SddC += C[i] * S[i];
  SddC = SddC / 3.0;
  or_gemm(0, 1, SddC, fInv, fInv, Sic);
  for (int i = 0; i < 9; ++i) Sdev[i] = S[i] - Sic[i];
  double *H1 = hist27, *H2 = hist27 + 9, *S0 = hist27 + 18;
  double rt1 = dt / gt[1], c11 = exp(-rt1), c21 = gt[0] * (1 - c11) / rt1;
  if (nterm == 2) {
    double rt2 = dt / gt[3], c12 = exp(-rt2), c22 = gt[2] * (1 - c12) / rt2;
    for (int i = 0; i < 9; ++i) {
      H1[i] = c11 * H1[i] + c21 * (Sdev[i] - S0[i]);
      H2[i] = c12 * H2[i] + c22 * (Sdev[i] - S0[i]);
      S[i] = S[i] + H1[i] + H2[i];
    }
  } else {
    for (int i = 0; i < 9; ++i) {
      H1[i] = c11 * H1[i] + c21 * (Sdev[i] - S0[i]);
      S[i] = S[i] + H1[i];
    }
  }
  for (int i = 0; i < 9; ++i) S0[i] = Sdev[i];
}

/* HGOIsotropicViscoelastic, src/materials/HGOIsotropicViscoelastic.cpp:27-168. */
static void or_mat_hgo_visco(const double *pr, const double *F, double J, double dt,
                             double *hist27, double *S6) {
  double mu = pr[1], lambda = pr[2], k1 = pr[3], k2 = pr[4];
  const double kappa = 1.0 / 3.0;
  double K = lambda + 2.0 * mu / 3.0;
  double hydro = 0.5 * K * (J * J - 1.0) / J;
  double B[9], fi[9], S[9];
  or_gemm(0, 1, 1.0, F, F, B);
  double trB = B[0] + B[4] + B[8];
  double Jm23 = pow(J, -2.0 / 3.0);
  double I1 = Jm23 * trB;
  double Ea = kappa * (I1 - 3.0);
  double fib = 0.0;
  if (Ea > 0.0) fib = 2.0 * k1 * exp(k2 * Ea * Ea) * Ea * kappa;
  double tp = (mu + fib) / J;
  double t3 = trB / 3.0;
  B[0] -= t3;
  B[4] -= t3;
  B[8] -= t3;
  for (int i = 0; i < 9; ++i) B[i] = B[i] * Jm23 * tp;
  B[0] += hydro;
  B[4] += hydro;
  B[8] += hydro;
  or_invF(F, J, fi);
  or_pullback(fi, B, J, S);
  double gt[4] = {pr[5], pr[6], pr[7], pr[8]};
  or_prony(F, fi, 2, gt, dt, hist27, S);
  or_voigt(S, S6);
}

/* Cyclic Jacobi eigen-decomposition of a symmetric 3x3 (column-major), FP64,
 * run to convergence.  Eigenvectors are the columns of V. */
static void or_jacobi3(const double *Ain, double *w, double *V) {
  double A[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i][j] = Ain[i + 3 * j];
  double Q[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    double diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off <= 1e-40 * diag || off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (A[p][q] == 0.0) continue;
        double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) { /* A <- A G */
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) { /* A <- G^T A */
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double qkp = Q[k][p], qkq = Q[k][q];
          Q[k][p] = c * qkp - s * qkq;
          Q[k][q] = s * qkp + c * qkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) {
    w[i] = A[i][i];
    for (int k = 0; k < 3; ++k) V[k + 3 * i] = Q[k][i];
  }
}

/* NEW material 6, 1-term Ogden with the volumetric law of HGOIsotropic.cpp:47:
 * W = (2 mu / alpha^2) sum_i (lbar_i^alpha - 1) + K/2 ((J^2-1)/2 - ln J),
 * props [rho, mu, lambda, alpha], K = lambda + 2 mu / 3.
 * S = sum_i (tau_i / lambda_i^2) N_i N_i^T + J p C^{-1},
 * tau_i = beta_i - mean(beta), beta_i = (2 mu / alpha) lbar_i^alpha. */
static void or_mat_ogden(const double *pr, const double *F, double J, double *S6) {
  double mu = pr[1], lambda = pr[2], alpha = pr[3];
  double K = lambda + 2.0 * mu / 3.0;
  double C[9], Ci[9], Cd, w[3], V[9], S[9];
  or_gemm(1, 0, 1.0, F, F, C);
  or_inv3(C, Ci, &Cd);
  double Jm23 = pow(J, -2.0 / 3.0);
  double Cb[9];
  for (int i = 0; i < 9; ++i) Cb[i] = Jm23 * C[i];
  or_jacobi3(Cb, w, V);
  double beta[3], bm = 0.0;
  for (int i = 0; i < 3; ++i) {
    beta[i] = 2.0 * mu / alpha * pow(w[i], 0.5 * alpha);
    bm += beta[i];
  }
  bm /= 3.0;
  double Jp = 0.5 * K * (J * J - 1.0);
  for (int i = 0; i < 9; ++i) S[i] = Jp * Ci[i];
  for (int k = 0; k < 3; ++k) {
    double f = (beta[k] - bm) * Jm23 / w[k];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) S[i + 3 * j] += f * V[i + 3 * k] * V[j + 3 * k];
  }
  or_voigt(S, S6);
}

/* NEW material 7, anisotropic GOH (one fibre family a0, dispersion kappa) with
 * a 1-term Prony series; generalises HGOIsotropicViscoelastic.cpp:27-168:
 * E = kappa (I1b - 3) + (1 - 3 kappa)(I4b - 1), W_f = k1/(2 k2)(exp(k2 E^2) - 1)
 * for E > 0.  props [rho, mu, lambda, k1, k2, g1, tau1, kappa]. */
static void or_mat_goh_visco(const double *pr, const double *F, double J,
                             const double *a0, double dt, double *hist27, double *S6) {
  double mu = pr[1], lambda = pr[2], k1 = pr[3], k2 = pr[4], kappa = pr[7];
  double K = lambda + 2.0 * mu / 3.0;
  double hydro = 0.5 * K * (J * J - 1.0) / J;
  double B[9], fi[9], S[9], af[3];
  or_gemm(0, 1, 1.0, F, F, B);
  for (int i = 0; i < 3; ++i) af[i] = F[i] * a0[0] + F[i + 3] * a0[1] + F[i + 6] * a0[2];
  double trB = B[0] + B[4] + B[8];
  double aa = af[0] * af[0] + af[1] * af[1] + af[2] * af[2];
  double Jm23 = pow(J, -2.0 / 3.0);
  double I1 = Jm23 * trB, I4 = Jm23 * aa;
  double Ea = kappa * (I1 - 3.0) + (1.0 - 3.0 * kappa) * (I4 - 1.0);
  double dW = 0.0;
  if (Ea > 0.0) dW = k1 * Ea * exp(k2 * Ea * Ea);
  double t1 = (mu + 2.0 * dW * kappa) / J;
  double t4 = 2.0 * dW * (1.0 - 3.0 * kappa) / J;
  double t3 = trB / 3.0, a3 = aa / 3.0;
  double sig[9];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      double db = B[i + 3 * j] - (i == j ? t3 : 0.0);
      double da = af[i] * af[j] - (i == j ? a3 : 0.0);
      sig[i + 3 * j] = Jm23 * (t1 * db + t4 * da) + (i == j ? hydro : 0.0);
    }
  or_invF(F, J, fi);
  or_pullback(fi, sig, J, S);
  double gt[2] = {pr[5], pr[6]};
  or_prony(F, fi, 1, gt, dt, hist27, S);
  or_voigt(S, S6);
}

/* StressUpdate dispatch, src/fem/SolidMechanics/StressUpdate.cpp:7-27 (+6, 7). */
int or_material_stress(int matID, const double *props, const double *F, double J,
                       const double *a0, double dt, double *hist27, double *S6) {
  switch (matID) {
    case 0: /* rigid: pk2 left untouched (zero) */
      for (int i = 0; i < 6; ++i) S6[i] = 0.0;
      return 0;
    case 1: or_mat_nh(props, F, J, S6); return 0;
    case 2: or_mat_svk(props, F, S6); return 0;
    case 3: or_mat_le(props, F, J, S6); return 0;
    case 4: or_mat_hgo(props, F, J, S6); return 0;
    case 5: or_mat_hgo_visco(props, F, J, dt, hist27, S6); return 0;
    case 6: or_mat_ogden(props, F, J, S6); return 0;
    case 7: {
      static const double ez[3] = {1.0, 0.0, 0.0};
      or_mat_goh_visco(props, F, J, a0 ? a0 : ez, dt, hist27, S6);
      return 0;
    }
    default: return -1; /* TerminateFemTech(1) in the reference */
  }
}

/* ShapeFunctions + ShapeFunction_C3D8/C3D4 + AssembleLumpedMass:
 * src/fem/ShapeFunctions/ShapeFunctions.cpp:32-255,
 * src/fem/ShapeFunctions/ShapeFunction_C3D8.cpp:4-128,
 * src/fem/ShapeFunctions/ShapeFunction_C3D4.cpp:6-91,
 * src/fem/Mass/Mass3D.cpp:5-67,127-157. */
int or_setup(or_model *m) {
  int E = m->nelements;
  if (m->nthreads <= 0) m->nthreads = 1;
  m->nGP = (int *)malloc(E * sizeof(int));
  m->nShp = (int *)malloc(E * sizeof(int));
  m->gpPtr = (int *)malloc((E + 1) * sizeof(int));
  m->dsptr = (int *)malloc((E + 1) * sizeof(int));
  m->gptr = (int *)malloc((E + 1) * sizeof(int));
  m->fptr = (int *)malloc((E + 1) * sizeof(int));
  m->pk2ptr = (int *)malloc((E + 1) * sizeof(int));
  m->gpPtr[0] = m->dsptr[0] = m->gptr[0] = m->fptr[0] = m->pk2ptr[0] = 0;
  for (int e = 0; e < E; ++e) {
    int hex = m->etype[e] == OR_C3D8;
    if (!hex && m->etype[e] != OR_C3D4) return -3;
    int nn = m->eptr[e + 1] - m->eptr[e];
    if (nn != (hex ? 8 : 4)) return -3;
    m->nGP[e] = hex ? 8 : 1;
    m->nShp[e] = hex ? 8 : 4;
    m->gpPtr[e + 1] = m->gpPtr[e] + m->nGP[e];
    m->gptr[e + 1] = m->gptr[e] + m->nGP[e] * m->nShp[e];
    m->dsptr[e + 1] = m->dsptr[e] + 3 * m->nGP[e] * m->nShp[e];
    m->fptr[e + 1] = m->fptr[e] + 9 * m->nGP[e];
    m->pk2ptr[e + 1] = m->pk2ptr[e] + 6 * m->nGP[e];
  }
  int nGPt = m->gpPtr[E];
  m->shp = (double *)calloc(m->gptr[E], sizeof(double));
  m->dshp = (double *)calloc(m->dsptr[E], sizeof(double));
  m->detJ = (double *)calloc(nGPt, sizeof(double));
  m->gw = (double *)calloc(nGPt, sizeof(double));
  m->F = (double *)calloc(9 * (size_t)nGPt, sizeof(double));
  m->detF = (double *)calloc(nGPt, sizeof(double));
  m->pk2 = (double *)calloc(6 * (size_t)nGPt, sizeof(double));
  m->hist = (double *)calloc(27 * (size_t)nGPt, sizeof(double));
  m->mass = (double *)calloc(3 * (size_t)m->nNodes, sizeof(double));
  m->fe = (double *)calloc(24 * (size_t)E, sizeof(double));
  m->ce = (double *)calloc(m->nPID > 0 ? m->nPID : 1, sizeof(double));
  for (int i = 0; i < nGPt; ++i) {
    m->F[9 * i] = m->F[9 * i + 4] = m->F[9 * i + 8] = 1.0;
    m->detF[i] = 1.0;
  }
  /* dilatational wave speed, src/timestep/CalculateTimeStep.cpp:12-18 */
  for (int p = 0; p < m->nPID; ++p) {
    const double *pr = m->properties + OR_MAXMATPARAMS * p;
    double mu = pr[1], lambda = pr[2], rho = pr[0];
    double nu = 0.5 * lambda / (lambda + mu);
    m->ce[p] = sqrt(lambda * (1.0 / nu - 1.0) / rho);
  }
  const double *X = m->coordinates;
  for (int e = 0; e < E; ++e) {
    const int *cn = m->connectivity + m->eptr[e];
    int ng = m->nGP[e], ns = m->nShp[e];
    for (int g = 0; g < ng; ++g) {
      double *shp = m->shp + m->gptr[e] + g * ng;
      double *ds = m->dshp + m->dsptr[e] + g * ng * 3;
      double xs[9], Ji[9], det;
      if (m->etype[e] == OR_C3D8) {
        double chi = kHexGP[g][0], eta = kHexGP[g][1], iota = kHexGP[g][2];
        for (int a = 0; a < 8; ++a) {
          double sx = kHexSign[a][0], sy = kHexSign[a][1], sz = kHexSign[a][2];
          shp[a] = ((1 + sx * chi) * (1 + sy * eta) * (1 + sz * iota)) / 8;
          ds[3 * a + 0] = sx * ((1 + sy * eta) * (1 + sz * iota)) / 8;
          ds[3 * a + 1] = sy * ((1 + sx * chi) * (1 + sz * iota)) / 8;
          ds[3 * a + 2] = sz * ((1 + sx * chi) * (1 + sy * eta)) / 8;
        }
        /* Jacobian with the node pairing of ShapeFunction_C3D8.cpp:79-93 */
        for (int j = 0; j < 3; ++j) {
#define XC(k) X[3 * cn[k] + j]
          xs[0 + 3 * j] = (XC(1) - XC(0)) * ds[3 * 1 + 0] + (XC(2) - XC(3)) * ds[3 * 2 + 0] +
                          (XC(5) - XC(4)) * ds[3 * 5 + 0] + (XC(6) - XC(7)) * ds[3 * 6 + 0];
          xs[1 + 3 * j] = (XC(2) - XC(1)) * ds[3 * 2 + 1] + (XC(3) - XC(0)) * ds[3 * 3 + 1] +
                          (XC(6) - XC(5)) * ds[3 * 6 + 1] + (XC(7) - XC(4)) * ds[3 * 7 + 1];
          xs[2 + 3 * j] = (XC(4) - XC(0)) * ds[3 * 4 + 2] + (XC(5) - XC(1)) * ds[3 * 5 + 2] +
                          (XC(6) - XC(2)) * ds[3 * 6 + 2] + (XC(7) - XC(3)) * ds[3 * 7 + 2];
#undef XC
        }
        or_inv3(xs, Ji, &det);
        m->detJ[m->gpPtr[e] + g] = det;
        m->gw[m->gpPtr[e] + g] = 1.0;
      } else {
        shp[0] = 0.25;
        shp[1] = 0.25;
        shp[2] = 0.25;
        shp[3] = 1.0 - 0.25 - 0.25 - 0.25;
        static const double dt4[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
        for (int a = 0; a < 4; ++a)
          for (int k = 0; k < 3; ++k) ds[3 * a + k] = dt4[a][k];
        /* ShapeFunction_C3D4.cpp:59-71 */
        for (int r = 0; r < 3; ++r)
          for (int j = 0; j < 3; ++j) xs[r + 3 * j] = X[3 * cn[r] + j] - X[3 * cn[3] + j];
        or_inv3(xs, Ji, &det);
        m->detJ[m->gpPtr[e] + g] = fabs(det);
        m->gw[m->gpPtr[e] + g] = 1.0 / 6.0;
      }
      for (int a = 0; a < ns; ++a) {
        double *d = ds + 3 * a;
        double c1 = d[0] * Ji[0] + d[1] * Ji[3] + d[2] * Ji[6];
        double c2 = d[0] * Ji[1] + d[1] * Ji[4] + d[2] * Ji[7];
        double c3 = d[0] * Ji[2] + d[1] * Ji[5] + d[2] * Ji[8];
        d[0] = c1;
        d[1] = c2;
        d[2] = c3;
      }
    }
  }
  /* lumped mass: Me = rho sum_gp w detJ N^T N, row-sum, scatter (Mass3D.cpp) */
  for (int e = 0; e < E; ++e) {
    int ng = m->nGP[e], ns = m->nShp[e];
    double Me[8][8];
    for (int a = 0; a < ns; ++a)
      for (int b = 0; b < ns; ++b) Me[a][b] = 0.0;
    for (int g = 0; g < ng; ++g) {
      const double *N = m->shp + m->gptr[e] + g * ng;
      double pf = m->gw[m->gpPtr[e] + g] * m->detJ[m->gpPtr[e] + g];
      for (int a = 0; a < ns; ++a)
        for (int b = 0; b < ns; ++b) Me[a][b] += (N[a] * N[b]) * pf;
    }
    double rho = m->properties[OR_MAXMATPARAMS * m->pid[e]];
    for (int a = 0; a < ns; ++a) {
      double s = Me[a][0] * rho;
      for (int b = 1; b < ns; ++b) s += Me[a][b] * rho;
      int n = m->connectivity[m->eptr[e] + a];
      for (int d = 0; d < 3; ++d) m->mass[3 * n + d] += s;
    }
  }
  return 0;
}

void or_free(or_model *m) {
  free(m->nGP); free(m->nShp); free(m->gpPtr); free(m->dsptr); free(m->gptr);
  free(m->fptr); free(m->pk2ptr); free(m->shp); free(m->dshp); free(m->detJ);
  free(m->gw); free(m->F); free(m->detF); free(m->pk2); free(m->hist);
  free(m->mass); free(m->fe); free(m->ce);
  memset(&m->nGP, 0, sizeof(*m) - offsetof(or_model, nGP));
}

/* One element's internal force: CalculateDeformationGradient.cpp:4-30,
 * DeterminateF, StressUpdate, InternalForceUpdate.cpp:4-28 with
 * StrainDisplacementMatrix.cpp:25-77 (B0^T S by a plain transposed mat-vec). */
static int or_element_force(or_model *m, int e, const double *u, double dt, double *fl) {
  const int *cn = m->connectivity + m->eptr[e];
  int ng = m->nGP[e], ns = m->nShp[e], pidE = m->pid[e];
  int mat = m->materialID[pidE];
  const double *pr = m->properties + OR_MAXMATPARAMS * pidE;
  const double *a0 = m->fiber ? m->fiber + 3 * e : 0;
  for (int k = 0; k < 3 * ns; ++k) fl[k] = 0.0;
  for (int g = 0; g < ng; ++g) {
    const double *ds = m->dshp + m->dsptr[e] + g * ng * 3;
    double *F = m->F + m->fptr[e] + 9 * g;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < ns; ++k) {
          int n = cn[k];
          s = s + (m->coordinates[3 * n + i] + u[3 * n + i]) * ds[k * 3 + j];
        }
        F[i + 3 * j] = s;
      }
    int gi = m->gpPtr[e] + g;
    double J = or_detF(F);
    m->detF[gi] = J;
    double *S6 = m->pk2 + m->pk2ptr[e] + 6 * g;
    if (mat == 0) {
      /* rigid: StressUpdate is a no-op, pk2 keeps its (zero) value */
    } else if (or_material_stress(mat, pr, F, J, a0, dt, m->hist + 27 * (size_t)gi, S6))
      return -1;
    double pf = m->gw[gi] * m->detJ[gi];
    double F11 = F[0], F21 = F[1], F31 = F[2], F12 = F[3], F22 = F[4], F32 = F[5],
           F13 = F[6], F23 = F[7], F33 = F[8];
    for (int k = 0; k < ns; ++k) {
      double x = ds[3 * k], y = ds[3 * k + 1], z = ds[3 * k + 2];
      double Bc[3][6] = {
          {x * F11, y * F12, z * F13, y * F13 + z * F12, x * F13 + z * F11, x * F12 + y * F11},
          {x * F21, y * F22, z * F23, y * F23 + z * F22, x * F23 + z * F21, x * F22 + y * F21},
          {x * F31, y * F32, z * F33, y * F33 + z * F32, x * F33 + z * F31, x * F32 + y * F31}};
      for (int c = 0; c < 3; ++c) {
        double s = 0.0;
        for (int r = 0; r < 6; ++r) s += Bc[c][r] * S6[r];
        fl[3 * k + c] += pf * s;
      }
    }
  }
  return 0;
}

/* GetForce_3D, src/fem/SolidMechanics/GetForce_3D.cpp:5-53: fi = sum of element
 * forces scattered in element order (element forces computed in parallel). */
int or_get_force(or_model *m, const double *u, double dt, double *fi) {
  int E = m->nelements, err = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(m->nthreads) reduction(| : err)
#endif
  for (int e = 0; e < E; ++e) err |= or_element_force(m, e, u, dt, m->fe + 24 * (size_t)e) ? 1 : 0;
  memset(fi, 0, 3 * (size_t)m->nNodes * sizeof(double));
  for (int e = 0; e < E; ++e) {
    const int *cn = m->connectivity + m->eptr[e];
    const double *fl = m->fe + 24 * (size_t)e;
    for (int k = 0; k < m->nShp[e]; ++k)
      for (int l = 0; l < 3; ++l) fi[3 * cn[k] + l] += fl[3 * k + l];
  }
  return err ? -1 : 0;
}

/* helpers of src/math/math.cpp:30-60 */
static double or_tri(const double *s, const double *a, const double *b) {
  return s[2] * (a[0] * b[1] - a[1] * b[0]) + s[0] * (a[1] * b[2] - a[2] * b[1]) -
         s[1] * (a[0] * b[2] - a[2] * b[0]);
}
static double or_ncross(const double *a, const double *b) {
  double z = a[0] * b[1] - a[1] * b[0];
  double x = a[1] * b[2] - a[2] * b[1];
  double y = -a[0] * b[2] + a[2] * b[0];
  return sqrt(x * x + y * y + z * z);
}

/* volumeHexahedron, src/math/Geometry.cpp:3-27 */
static double or_hex_volume(const double *L) {
  double q[6][3];
  for (int i = 0; i < 3; ++i) {
#define P(k) L[3 * (k) + i]
    q[0][i] = P(0) - P(1) + P(2) - P(3) + P(4) - P(5) + P(6) - P(7);
    q[1][i] = P(0) - P(1) - P(2) + P(3) - P(4) + P(5) + P(6) - P(7);
    q[2][i] = -P(0) + P(1) + P(2) - P(3) - P(4) + P(5) + P(6) - P(7);
    q[3][i] = P(0) + P(1) - P(2) - P(3) - P(4) - P(5) + P(6) + P(7);
    q[4][i] = -P(0) - P(1) + P(2) + P(3) - P(4) - P(5) + P(6) + P(7);
    q[5][i] = -P(0) - P(1) - P(2) - P(3) + P(4) + P(5) + P(6) + P(7);
#undef P
  }
  return (or_tri(q[0], q[4], q[3]) + or_tri(q[2], q[0], q[1]) + or_tri(q[1], q[3], q[5])) /
             192.0 +
         or_tri(q[2], q[4], q[5]) / 64.0;
}

/* areaHexahedronFace, src/math/Geometry.cpp:29-64 (the parallelogram test
 * compares signed components against the tolerance, as the reference does). */
static double or_face_area(const double *L, const int *ix) {
  const double *p1 = L + 3 * ix[0], *p2 = L + 3 * ix[1], *p3 = L + 3 * ix[2],
               *p4 = L + 3 * ix[3];
  double tol = 1e-6, cD[3], c1[3], c2[3];
  for (int i = 0; i < 3; ++i) {
    cD[i] = 0.25 * (p1[i] - p2[i] + p3[i] - p4[i]);
    c1[i] = 0.25 * (-p1[i] + p2[i] + p3[i] - p4[i]);
    c2[i] = 0.25 * (-p1[i] - p2[i] + p3[i] + p4[i]);
  }
  if (cD[0] < tol && cD[1] < tol && cD[2] < tol) return 4.0 * or_ncross(c1, c2);
  double t = sqrt(3.0) / 3.0;
  const double q[2] = {-t, t};
  double area = 0.0;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      double v1[3], v2[3];
      for (int k = 0; k < 3; ++k) {
        v1[k] = q[j] * cD[k] + c1[k];
        v2[k] = q[i] * cD[k] + c2[k];
      }
      area += or_ncross(v1, v2);
    }
  return area;
}

/* CalculateCharacteristicLength_C3D8.cpp:3-30 / _C3D4.cpp:5-46 on x = X + u */
static double or_char_length(const or_model *m, int e, const double *u) {
  double L[24];
  const int *cn = m->connectivity + m->eptr[e];
  int nn = m->nShp[e];
  for (int j = 0; j < nn; ++j)
    for (int k = 0; k < 3; ++k) L[3 * j + k] = m->coordinates[3 * cn[j] + k] + u[3 * cn[j] + k];
  if (m->etype[e] == OR_C3D8) {
    static const int ix[24] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 3, 7, 4,
                               1, 2, 6, 5, 0, 1, 5, 4, 3, 2, 6, 7};
    double vol = or_hex_volume(L), amax = 0.0;
    for (int f = 0; f < 6; ++f) {
      double a = or_face_area(L, ix + 4 * f);
      if (a > amax) amax = a;
    }
    return vol / amax;
  }
  static const int ix[16] = {0, 1, 2, 3, 1, 2, 3, 0, 2, 3, 0, 1, 3, 0, 1, 2};
  double amin = 1e6;
  for (int f = 0; f < 4; ++f) {
    const double *x0 = L + 3 * ix[4 * f], *x1 = L + 3 * ix[4 * f + 1],
                 *x2 = L + 3 * ix[4 * f + 2], *x3 = L + 3 * ix[4 * f + 3];
    double v1[3], v2[3], n[3], v3[3];
    for (int i = 0; i < 3; ++i) {
      v1[i] = x2[i] - x1[i];
      v2[i] = x3[i] - x1[i];
    }
    n[0] = v1[1] * v2[2] - v1[2] * v2[1];
    n[1] = -v1[0] * v2[2] + v1[2] * v2[0];
    n[2] = v1[0] * v2[1] - v1[1] * v2[0];
    double cn2 = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int i = 0; i < 3; ++i) n[i] /= cn2;
    for (int i = 0; i < 3; ++i) v3[i] = x0[i] - x1[i];
    double alt = fabs(n[0] * v3[0] + n[1] * v3[1] + n[2] * v3[2]);
    if (alt < amin) amin = alt;
  }
  return amin;
}

/* StableTimeStep, src/timestep/StableTimeStep.cpp:4-40 (the MPI min is the
 * identity on one rank; the FailureTimeStep check is left to the caller). */
double or_stable_time_step(const or_model *m, const double *u, const int *boundary) {
  double dtMin = 1e20;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(m->nthreads) reduction(min : dtMin)
#endif
  for (int e = 0; e < m->nelements; ++e) {
    int active = 0;
    for (int j = m->eptr[e]; j < m->eptr[e + 1]; ++j) {
      int idx = 3 * m->connectivity[j];
      if (!(boundary[idx] & boundary[idx + 1] & boundary[idx + 2])) {
        active = 1;
        break;
      }
    }
    if (!active) continue;
    double d = or_char_length(m, e, u) / m->ce[m->pid[e]];
    if (d < dtMin) dtMin = d;
  }
  return dtMin;
}

/* closed-form half-sine angular history about a fixed axis */
static void or_rot_angle(const double *p, double t, double *theta, double *omega) {
  double a0 = p[6], T = p[7], pi = 3.14159265358979323846;
  if (t <= T) {
    *omega = a0 * T / pi * (1.0 - cos(pi * t / T));
    *theta = a0 * T / pi * (t - T / pi * sin(pi * t / T));
  } else {
    double wT = 2.0 * a0 * T / pi, thT = a0 * T * T / pi;
    *omega = wT;
    *theta = thT + wT * (t - T);
  }
}

/* Driver boundary conditions in the style of examples/ex9/ex9.cpp:187-248:
 * constrained DOFs get the prescribed displacement/velocity and zero
 * acceleration at time t; HOLD DOFs are constrained but left untouched. */
/* interpolateLinear, src/math/math.cpp:99-119: 0 below the table (the
 * reference logs an error), the last value above it, y[0] at x[0], else the
 * segment of the first x[i] >= value. */
double or_interp_linear(int n, const double *x, const double *y, double value) {
  if (value < x[0]) return 0.0;
  if (value > x[n - 1]) return y[n - 1];
  if (value == x[0]) return y[0];
  int index = 0;
  for (int i = 1; i < n; ++i)
    if (value <= x[i]) {
      index = i - 1;
      break;
    }
  return y[index] + (y[index + 1] - y[index]) * (value - x[index]) / (x[index + 1] - x[index]);
}

/* crossProduct / dotProduct3D, src/math/math.cpp:50-60 */
static void or_cross(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = -a[0] * b[2] + a[2] * b[0];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

/* computeDerivatives, examples/ex5/ex5.cpp:976-1020: sampled angular and
 * linear accelerations, the centre-of-mass velocity, and the rate of the
 * rotation generator r from the angular velocity (M. Boyle, "The integration
 * of angular velocity", 2017): rdot = omega / 2 for |r| < 1e-10, else
 * (omega x r + |r| cot|r| omega + (1 - |r| cot|r|) (rhat . omega) rhat) / 2. */
static void or_rigid_deriv(const or_rigid *rb, const double *y, double t, double *yd) {
  for (int k = 0; k < 3; ++k) {
    yd[k] = or_interp_linear(rb->n[k], rb->t[k], rb->v[k], t);
    yd[6 + k] = or_interp_linear(rb->n[3 + k], rb->t[3 + k], rb->v[3 + k], t);
    yd[9 + k] = y[6 + k];
  }
  double r[3] = {y[3], y[4], y[5]};
  double *rdot = yd + 3;
  double rm = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  if (rm < 1e-10) {
    for (int k = 0; k < 3; ++k) rdot[k] = 0.5 * y[k];
  } else {
    double rc = rm / tan(rm), om[3] = {y[0], y[1], y[2]};
    or_cross(om, r, rdot);
    for (int k = 0; k < 3; ++k) r[k] = r[k] / rm;
    double rw = r[0] * om[0] + r[1] * om[1] + r[2] * om[2];
    for (int k = 0; k < 3; ++k) rdot[k] = 0.5 * (rdot[k] + rc * y[k] + (1.0 - rc) * rw * r[k]);
  }
}

/* One step of the explicit Runge-Kutta pair of Dormand and Prince (J. Comput.
 * Appl. Math. 6 (1980) 19-26), fifth-order solution, first stage taken from
 * yd (first same as last) and yd left at f(y(t + h), t + h): what
 * runge_kutta_dopri5<boost::array<double,12>>::do_step(sys, y, yd, t, h) does
 * at ex5.cpp:344 (Boost.Odeint is not part of the reference tree; this is the
 * published tableau).  Sums are formed as y + (h a_i1) k1 + (h a_i2) k2 + ... */
void or_rigid_step(or_rigid *rb, double t, double h) {
  static const double c2 = 1.0 / 5, c3 = 3.0 / 10, c4 = 4.0 / 5, c5 = 8.0 / 9;
  static const double a21 = 1.0 / 5, a31 = 3.0 / 40, a32 = 9.0 / 40, a41 = 44.0 / 45,
                      a42 = -56.0 / 15, a43 = 32.0 / 9, a51 = 19372.0 / 6561,
                      a52 = -25360.0 / 2187, a53 = 64448.0 / 6561, a54 = -212.0 / 729,
                      a61 = 9017.0 / 3168, a62 = -355.0 / 33, a63 = 46732.0 / 5247,
                      a64 = 49.0 / 176, a65 = -5103.0 / 18656;
  static const double b1 = 35.0 / 384, b3 = 500.0 / 1113, b4 = 125.0 / 192,
                      b5 = -2187.0 / 6784, b6 = 11.0 / 84;
  double k2[12], k3[12], k4[12], k5[12], k6[12], x[12];
  const double *y = rb->y, *k1 = rb->yd;
  for (int i = 0; i < 12; ++i) x[i] = y[i] + (h * a21) * k1[i];
  or_rigid_deriv(rb, x, t + h * c2, k2);
  for (int i = 0; i < 12; ++i) x[i] = y[i] + (h * a31) * k1[i] + (h * a32) * k2[i];
  or_rigid_deriv(rb, x, t + h * c3, k3);
  for (int i = 0; i < 12; ++i)
    x[i] = y[i] + (h * a41) * k1[i] + (h * a42) * k2[i] + (h * a43) * k3[i];
  or_rigid_deriv(rb, x, t + h * c4, k4);
  for (int i = 0; i < 12; ++i)
    x[i] = y[i] + (h * a51) * k1[i] + (h * a52) * k2[i] + (h * a53) * k3[i] + (h * a54) * k4[i];
  or_rigid_deriv(rb, x, t + h * c5, k5);
  for (int i = 0; i < 12; ++i)
    x[i] = y[i] + (h * a61) * k1[i] + (h * a62) * k2[i] + (h * a63) * k3[i] +
           (h * a64) * k4[i] + (h * a65) * k5[i];
  or_rigid_deriv(rb, x, t + h, k6);
  for (int i = 0; i < 12; ++i)
    x[i] = y[i] + (h * b1) * k1[i] + (h * b3) * k3[i] + (h * b4) * k4[i] + (h * b5) * k5[i] +
           (h * b6) * k6[i];
  memcpy(rb->y, x, sizeof(x));
  or_rigid_deriv(rb, rb->y, t + h, rb->yd);
}

/* quaternionMultiply, src/math/math.cpp:135-140 */
static void or_qmul(const double *p, const double *q, double *r) {
  r[0] = p[0] * q[0] - p[1] * q[1] - p[2] * q[2] - p[3] * q[3];
  r[1] = p[0] * q[1] + p[1] * q[0] + p[2] * q[3] - p[3] * q[2];
  r[2] = p[0] * q[2] - p[1] * q[3] + p[2] * q[0] + p[3] * q[1];
  r[3] = p[0] * q[3] + p[1] * q[2] - p[2] * q[1] + p[3] * q[0];
}

/* ApplyAccBoundaryConditions for one node, ex5.cpp:345-371: R = exp([0, r])
 * (quaternionExp, math.cpp:122-133), Vp = R V R^-1 (quaternionInverse /
 * quaternionRotate, math.cpp:142-158), then
 *   u = Vp - X + x_cm,  v = omega x Vp + v_cm,
 *   a = 2 omega x v_cm + omega x (omega x Vp) + a_cm + alpha x Vp. */
void or_rigid_point(const or_rigid *rb, const double *X, double *u, double *v, double *a) {
  const double *y = rb->y, *yd = rb->yd;
  double R[4], Ri[4], V[4], RV[4], Vp[4];
  double vm = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
  if (vm == 0) {
    R[0] = 1.0;
    R[1] = R[2] = R[3] = 0.0;
  } else {
    vm = sqrt(vm);
    const double d1 = exp(0.0), d2 = d1 * sin(vm) / vm;
    R[0] = d1 * cos(vm);
    R[1] = d2 * y[3];
    R[2] = d2 * y[4];
    R[3] = d2 * y[5];
  }
  const double nr = R[0] * R[0] + R[1] * R[1] + R[2] * R[2] + R[3] * R[3];
  Ri[0] = R[0] / nr;
  Ri[1] = -R[1] / nr;
  Ri[2] = -R[2] / nr;
  Ri[3] = -R[3] / nr;
  double loc[3];
  for (int j = 0; j < 3; ++j) loc[j] = X[j] - rb->c[j];
  V[0] = 0.0;
  V[1] = loc[0];
  V[2] = loc[1];
  V[3] = loc[2];
  or_qmul(R, V, RV);
  or_qmul(RV, Ri, Vp);
  const double om[3] = {y[0], y[1], y[2]}, al[3] = {yd[0], yd[1], yd[2]},
               vel[3] = {y[6], y[7], y[8]};
  double oR[3], ooR[3], oV[3], aR[3];
  or_cross(om, Vp + 1, oR);
  or_cross(om, oR, ooR);
  or_cross(om, vel, oV);
  or_cross(al, Vp + 1, aR);
  for (int j = 0; j < 3; ++j) {
    u[j] = Vp[j + 1] - loc[j] + y[9 + j];
    v[j] = oR[j] + y[6 + j];
    a[j] = 2.0 * oV[j] + ooR[j] + yd[6 + j] + aR[j];
  }
}

void or_apply_bc(const or_model *m, const int *dof_fn, const or_bc_fn *fns, double t,
                 double *u, double *v, double *a) {
  for (int n = 0; n < m->nNodes; ++n)
    for (int d = 0; d < 3; ++d) {
      int f = dof_fn[3 * n + d];
      if (f < 0) continue;
      const or_bc_fn *b = fns + f;
      int i = 3 * n + d;
      if (b->kind == OR_BCK_RIGID) {
        double ur[3] = {0, 0, 0}, vr[3] = {0, 0, 0}, ar[3] = {0, 0, 0};
        if (m->rigid) or_rigid_point(m->rigid, m->coordinates + 3 * n, ur, vr, ar);
        u[i] = ur[d];
        v[i] = vr[d];
        a[i] = ar[d];
        continue;
      }
      if (b->kind == OR_BCK_FIXED) {
        u[i] = b->p[0];
        v[i] = 0.0;
      } else if (b->kind == OR_BCK_RAMP) {
        u[i] = t * b->p[0];
        v[i] = b->p[0];
      } else if (b->kind == OR_BCK_SINE) {
        u[i] = b->p[0] * sin(b->p[1] * t);
        v[i] = b->p[0] * b->p[1] * cos(b->p[1] * t);
      } else if (b->kind == OR_BCK_ROT) {
        double th, om, r[3], k[3] = {b->p[0], b->p[1], b->p[2]};
        or_rot_angle(b->p, t, &th, &om);
        for (int j = 0; j < 3; ++j) r[j] = m->coordinates[3 * n + j] - b->p[3 + j];
        double c = cos(th), s = sin(th), kr = k[0] * r[0] + k[1] * r[1] + k[2] * r[2];
        double kx[3] = {k[1] * r[2] - k[2] * r[1], k[2] * r[0] - k[0] * r[2],
                        k[0] * r[1] - k[1] * r[0]};
        double Rr[3];
        for (int j = 0; j < 3; ++j) Rr[j] = r[j] * c + kx[j] * s + k[j] * kr * (1.0 - c);
        double w[3] = {om * (k[1] * Rr[2] - k[2] * Rr[1]), om * (k[2] * Rr[0] - k[0] * Rr[2]),
                       om * (k[0] * Rr[1] - k[1] * Rr[0])};
        u[i] = Rr[d] - r[d];
        v[i] = w[d];
      }
      a[i] = 0.0;
    }
}

/* The explicit central-difference loop of examples/ex9/ex9.cpp:79-175
 * (Belytschko Box 6.1): initial dt/force/acceleration, then per step the
 * half-step velocity, displacement update, BCs, GetForce, accelerations,
 * full-step velocity and the next stable dt.  Energy checks and VTU output
 * are left out.  u, v, a hold the initial state on entry and the final state
 * on return.  Every out_every steps u and Time are appended to u_out/t_out. */
/* CalculateStrain.cpp:8-75 (CalculateMaximumPrincipalStrain): the Gauss-point
 * average of the Green-Lagrange strain from the F of the last or_get_force,
 * E = sum_gp (0.5 / nGP) F^T F - 0.5 I (the dgemm of the reference: for column
 * j, row i, s = sum_l F[l,i] F[l,j], E[i,j] = 0.5/nGP s + E[i,j]), then the
 * principal strains from the trigonometric solution of the characteristic
 * equation; ps_max clamped at >= 0, ps_min at <= 0, shear = (max - min) / 2.
 * Any output may be NULL. */
void or_element_strain(const or_model *m, double *Eavg9, double *ps_max, double *ps_min,
                       double *shear_max) {
  const double kPi = 4.0 * atan(1.0);
  for (int elm = 0; elm < m->nelements; ++elm) {
    double E[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int ngp = m->nGP[elm];
    const double pre = 0.5 / (double)ngp;
    for (int gp = 0; gp < ngp; ++gp) {
      const double *F = m->F + m->fptr[elm] + 9 * gp;
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          double s = 0.0;
          for (int l = 0; l < 3; ++l) s += F[l + 3 * i] * F[l + 3 * j];
          E[i + 3 * j] = pre * s + E[i + 3 * j];
        }
    }
    E[0] -= 0.5;
    E[4] -= 0.5;
    E[8] -= 0.5;
    if (Eavg9) memcpy(Eavg9 + 9 * (size_t)elm, E, sizeof(E));
    const double a = E[0], b = E[1], c = E[2], d = E[4], e = E[5], f = E[8];
    const double p1 = b * b + c * c + e * e;
    double e1, e2, e3;
    if (p1 == 0) {
      e1 = a;
      e2 = d;
      e3 = f;
    } else {
      double I1 = a + d + f;
      const double I2 = a * (d + f) + d * f - b * b - c * c - e * e;
      const double I3 = a * d * f + 2.0 * b * c * e - b * b * f - c * c * d - e * e * a;
      const double Q = (3.0 * I2 - I1 * I1) / 9.0;
      const double R = (2.0 * I1 * I1 * I1 - 9.0 * I1 * I2 + 27.0 * I3) / 54.0;
      const double theta = acos(R / sqrt(-Q * Q * Q));
      const double sq = 2.0 * sqrt(-Q);
      I1 = I1 / 3.0;
      e1 = sq * cos(theta / 3.0) + I1;
      e2 = sq * cos((theta + 2.0 * kPi) / 3.0) + I1;
      e3 = sq * cos((theta + 4.0 * kPi) / 3.0) + I1;
    }
    const double mx = fmax(e3, fmax(e2, e1)), mn = fmin(e3, fmin(e2, e1));
    if (shear_max) shear_max[elm] = 0.5 * (mx - mn);
    if (ps_max) ps_max[elm] = mx > 0.0 ? mx : 0.0;
    if (ps_min) ps_min[elm] = mn < 0.0 ? mn : 0.0;
  }
}

static int cmp_double(const void *a, const void *b) {
  const double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

double or_percentile95(const double *data, int n) {
  if (n <= 0) return 0.0;
  double *c = (double *)malloc(n * sizeof(double));
  memcpy(c, data, n * sizeof(double));
  qsort(c, n, sizeof(double), cmp_double);
  int k = (int)(n * 0.95) - 1;
  if (k < 0) k = 0;
  const double v = c[k];
  free(c);
  return v;
}

/* ex5.cpp:1311-1430 on one rank; PS_Old starts at 0 (the driver leaves it
 * uninitialised before the first call) */
void or_injury_step(const or_model *m, or_injury *s, double time, double dt) {
  const int nE = m->nelements;
  double *mx = (double *)malloc(nE * sizeof(double));
  double *mn = (double *)malloc(nE * sizeof(double));
  double *sh = (double *)malloc(nE * sizeof(double));
  or_element_strain(m, NULL, mx, mn, sh);
  for (int j = 0; j < s->n; ++j) {
    const int i = s->ids[j];
    const double cmax = mx[i], cmin = mn[i], cshear = sh[i];
    if (s->max_strain < cmax) {
      s->max_strain = cmax;
      s->max_strain_elem = i;
      s->max_strain_time = time;
    }
    if (s->min_strain > cmin) {
      s->min_strain = cmin;
      s->min_strain_elem = i;
      s->min_strain_time = time;
    }
    if (s->max_shear < cshear) {
      s->max_shear = cshear;
      s->max_shear_elem = i;
      s->max_shear_time = time;
    }
    if (!s->mps15[j] && cmax > 0.15) s->mps15[j] = 1;
    if (!s->mps30[j] && cmax > 0.30) s->mps30[j] = 1;
    const double psr = (cmax - s->ps_old[j]) / dt;
    const double psxsr = cmax * psr;
    if (s->max_psxsr < psxsr) {
      s->max_psxsr = psxsr;
      s->max_psxsr_elem = i;
      s->max_psxsr_time = time;
    }
    if (!s->psr120[j] && psr > 120.0) s->psr120[j] = 1;
    if (!s->psxsr28[j] && psxsr > 28.0) s->psxsr28[j] = 1;
    s->ps_old[j] = cmax;
    s->psxsr[j] = psxsr;
  }
  const double mps95 = or_percentile95(s->ps_old, s->n);
  if (mps95 > s->mps95) {
    s->mps95 = mps95;
    s->mps95_time = time;
    s->mps95_count = 0;
    for (int j = 0; j < s->n; ++j) {
      s->in_mps95[j] = s->ps_old[j] >= mps95;
      s->mps95_count += s->in_mps95[j];
    }
  }
  const double x95 = or_percentile95(s->psxsr, s->n);
  if (x95 > s->mpsxsr95) {
    s->mpsxsr95 = x95;
    s->mpsxsr95_time = time;
    s->mpsxsr95_count = 0;
    for (int j = 0; j < s->n; ++j) {
      s->in_mpsxsr95[j] = s->psxsr[j] >= x95;
      s->mpsxsr95_count += s->in_mpsxsr95[j];
    }
  }
  free(mx);
  free(mn);
  free(sh);
}

int or_explicit_run(or_model *m, const int *dof_fn, const or_bc_fn *fns, int nfn,
                    double t0, double tMax, double reduction, double failure_dt,
                    int max_steps, int out_every, double *u, double *v, double *a,
                    double *u_out, double *t_out, int max_out, int *n_out,
                    int *steps_done, double *time_out, double *dt_out) {
  (void)nfn;
  int nDOF = 3 * m->nNodes, rc = 0;
  int *boundary = (int *)calloc(nDOF, sizeof(int));
  double *fi = (double *)calloc(nDOF, sizeof(double));
  double *vh = (double *)calloc(nDOF, sizeof(double));
  /* energy balance (CheckEnergy.cpp:3-85): previous displacements,
   * accelerations and internal forces; no external forces on this path */
  double *u_prev = NULL, *a_prev = NULL, *fi_prev = NULL;
  double Wint = 0.0, Wext = 0.0;
  if (m->energy) {
    u_prev = (double *)calloc(nDOF, sizeof(double));
    a_prev = (double *)calloc(nDOF, sizeof(double));
    fi_prev = (double *)calloc(nDOF, sizeof(double));
  }
  for (int i = 0; i < nDOF; ++i) boundary[i] = dof_fn[i] != OR_BC_FREE;
  if (m->rigid) { /* ex5.cpp:886-890 */
    memset(m->rigid->y, 0, sizeof(m->rigid->y));
    memset(m->rigid->yd, 0, sizeof(m->rigid->yd));
  }
  double Time = t0;
  *n_out = 0;
  *steps_done = 0;
  or_apply_bc(m, dof_fn, fns, Time, u, v, a);
  double dtmin = or_stable_time_step(m, u, boundary);
  if (dtmin < failure_dt) { rc = -19; goto done; }
  double dt = reduction * dtmin;
  if (or_get_force(m, u, dt, fi)) { rc = -1; goto done; }
  for (int i = 0; i < nDOF; ++i)
    if (!boundary[i]) a[i] = -fi[i] / m->mass[i];
  int step = 0;
  while (Time < tMax && step < max_steps) {
    double t_n = Time, t_np1 = Time + dt;
    Time = t_np1;
    double dt_nphalf = dt, t_nphalf = 0.5 * (t_np1 + t_n);
    for (int i = 0; i < nDOF; ++i)
      vh[i] = boundary[i] ? v[i] : v[i] + (t_nphalf - t_n) * a[i];
    if (m->energy) { /* ex9.cpp:124-129 */
      memcpy(u_prev, u, nDOF * sizeof(double));
      memcpy(a_prev, a, nDOF * sizeof(double));
      memcpy(fi_prev, fi, nDOF * sizeof(double));
    }
    for (int i = 0; i < nDOF; ++i)
      if (!boundary[i]) u[i] = u[i] + dt_nphalf * vh[i];
    if (m->rigid) or_rigid_step(m->rigid, Time - dt, dt); /* ex5.cpp:344 */
    or_apply_bc(m, dof_fn, fns, Time, u, v, a);
    if (or_get_force(m, u, dt, fi)) { rc = -1; break; }
    for (int i = 0; i < nDOF; ++i)
      if (!boundary[i]) a[i] = -fi[i] / m->mass[i];
    for (int i = 0; i < nDOF; ++i)
      if (!boundary[i]) v[i] = vh[i] + (t_np1 - t_nphalf) * a[i];
    if (m->energy && step < m->energy_cap) {
      /* CheckEnergy.cpp:18-55 on one rank: kinetic energy, internal work
       * increment (equ 6.2.14) and the work of the reactions of constrained
       * DOFs (fe = 0) */
      double wke = 0.0, dwi = 0.0, dwe = 0.0;
      for (int i = 0; i < nDOF; ++i) {
        double dd = u[i] - u_prev[i];
        wke += m->mass[i] * v[i] * v[i];
        if (boundary[i]) {
          double reaction = fi_prev[i] + fi[i] + m->mass[i] * (a[i] + a_prev[i]);
          dwe += dd * reaction;
        }
        dwi += dd * (fi_prev[i] + fi[i]);
      }
      Wint += 0.5 * dwi;
      Wext += 0.5 * dwe;
      m->energy[3 * step + 0] = Wint;
      m->energy[3 * step + 1] = Wext;
      m->energy[3 * step + 2] = 0.5 * wke;
    }
    if (m->injury) or_injury_step(m, m->injury, Time, dt_nphalf);  /* ex5.cpp:238-240 */
    ++step;
    if (out_every > 0 && step % out_every == 0 && *n_out < max_out) {
      memcpy(u_out + (size_t)(*n_out) * nDOF, u, nDOF * sizeof(double));
      t_out[*n_out] = Time;
      ++*n_out;
    }
    dtmin = or_stable_time_step(m, u, boundary);
    if (dtmin < failure_dt) { rc = -19; break; }
    dt = reduction * dtmin;
  }
  *steps_done = step;
  *time_out = Time;
  *dt_out = dt;
done:
  free(boundary);
  free(fi);
  free(vh);
  free(u_prev);
  free(a_prev);
  free(fi_prev);
  return rc;
}
