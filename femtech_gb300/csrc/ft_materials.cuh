// ft_materials.cuh -- constitutive laws of the explicit hot path, on the device.
//
// Same laws and material IDs as FemTech's StressUpdate switch
// (src/fem/SolidMechanics/StressUpdate.cpp:7-27) plus two new ones (6 Ogden,
// 7 anisotropic GOH + 1-term Prony).  Every law is written on the displacement
// gradient D = F - I instead of F, with J - 1 taken from the invariants of D
// and log1p/expm1 for ln J and J^{-2/3}: in FP32 the stiff volumetric terms of
// nearly incompressible tissue (bulk/shear ~ 1e4) would otherwise drown in the
// rounding of det(F) - 1.  In exact arithmetic each law equals the reference
// formula cited beside it.
//
// Stress is returned as PK2 in the reference's Voigt order [11,22,33,23,13,12]
// (upper triangle), e.g. CompressibleNeoHookean.cpp:41-55.
#pragma once

#include <cuda_runtime.h>

namespace ftgpu {

template <class R>
struct Sym6 {
  R xx, yy, zz, yz, xz, xy;
};

constexpr int kOgdenSeries = 9;  // terms of the small-strain Ogden series

template <class R>
struct MatP {  // per-part material parameters, precomputed on the host
  R p[9];      // properties[pid*9 + k] converted to R
  R K;         // bulk modulus lambda + 2 mu / 3
  R inv_ce;    // 1 / dilatational wave speed (CalculateTimeStep.cpp:12-18)
  double ce;   // dilatational wave speed in FP64
  int mat;     // material ID
  int pad;
  // Ogden: binomial coefficients binom(alpha/2 - 1, k), k = 1..kOgdenSeries,
  // and the squared Frobenius bound on 2E below which the series is used
  // (0 = always the eigen-decomposition; set on the host from the series'
  // truncation bound for this alpha)
  R ser_a[kOgdenSeries];
  R ser_thr2;
};

template <class R> __device__ __forceinline__ R d_log1p(R x);
template <> __device__ __forceinline__ float d_log1p<float>(float x) { return log1pf(x); }
template <> __device__ __forceinline__ double d_log1p<double>(double x) { return log1p(x); }
template <class R> __device__ __forceinline__ R d_expm1(R x);
template <> __device__ __forceinline__ float d_expm1<float>(float x) { return expm1f(x); }
template <> __device__ __forceinline__ double d_expm1<double>(double x) { return expm1(x); }
template <class R> __device__ __forceinline__ R d_exp(R x);
template <> __device__ __forceinline__ float d_exp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double d_exp<double>(double x) { return exp(x); }
template <class R> __device__ __forceinline__ R d_sqrt(R x);
template <> __device__ __forceinline__ float d_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double d_sqrt<double>(double x) { return sqrt(x); }

// J - 1 = det(I + D) - 1 = tr D + I2(D) + det D  (no cancellation for small D)
template <class R>
__device__ __forceinline__ R jm1_of(const R (&D)[3][3]) {
  R tr = D[0][0] + D[1][1] + D[2][2];
  R i2 = (D[0][0] * D[1][1] - D[0][1] * D[1][0]) + (D[0][0] * D[2][2] - D[0][2] * D[2][0]) +
         (D[1][1] * D[2][2] - D[1][2] * D[2][1]);
  R i3 = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) -
         D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
         D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
  return tr + i2 + i3;
}

// 2E = C - I = D + D^T + D^T D
template <class R>
__device__ __forceinline__ Sym6<R> two_E(const R (&D)[3][3]) {
  Sym6<R> e;
  e.xx = 2 * D[0][0] + (D[0][0] * D[0][0] + D[1][0] * D[1][0] + D[2][0] * D[2][0]);
  e.yy = 2 * D[1][1] + (D[0][1] * D[0][1] + D[1][1] * D[1][1] + D[2][1] * D[2][1]);
  e.zz = 2 * D[2][2] + (D[0][2] * D[0][2] + D[1][2] * D[1][2] + D[2][2] * D[2][2]);
  e.yz = D[1][2] + D[2][1] + (D[0][1] * D[0][2] + D[1][1] * D[1][2] + D[2][1] * D[2][2]);
  e.xz = D[0][2] + D[2][0] + (D[0][0] * D[0][2] + D[1][0] * D[1][2] + D[2][0] * D[2][2]);
  e.xy = D[0][1] + D[1][0] + (D[0][0] * D[0][1] + D[1][0] * D[1][1] + D[2][0] * D[2][1]);
  return e;
}

// 2e = B - I = D + D^T + D D^T
template <class R>
__device__ __forceinline__ Sym6<R> two_e_left(const R (&D)[3][3]) {
  Sym6<R> e;
  e.xx = 2 * D[0][0] + (D[0][0] * D[0][0] + D[0][1] * D[0][1] + D[0][2] * D[0][2]);
  e.yy = 2 * D[1][1] + (D[1][0] * D[1][0] + D[1][1] * D[1][1] + D[1][2] * D[1][2]);
  e.zz = 2 * D[2][2] + (D[2][0] * D[2][0] + D[2][1] * D[2][1] + D[2][2] * D[2][2]);
  e.yz = D[1][2] + D[2][1] + (D[1][0] * D[2][0] + D[1][1] * D[2][1] + D[1][2] * D[2][2]);
  e.xz = D[0][2] + D[2][0] + (D[0][0] * D[2][0] + D[0][1] * D[2][1] + D[0][2] * D[2][2]);
  e.xy = D[0][1] + D[1][0] + (D[0][0] * D[1][0] + D[0][1] * D[1][1] + D[0][2] * D[1][2]);
  return e;
}

// adj(C) for C = I + e (symmetric): C^{-1} = adj(C) / det(C) = adj(C) / J^2
template <class R>
__device__ __forceinline__ Sym6<R> adj_I_plus(const Sym6<R> &e) {
  R cxx = 1 + e.xx, cyy = 1 + e.yy, czz = 1 + e.zz;
  Sym6<R> a;
  a.xx = cyy * czz - e.yz * e.yz;
  a.yy = cxx * czz - e.xz * e.xz;
  a.zz = cxx * cyy - e.xy * e.xy;
  a.yz = e.xz * e.xy - cxx * e.yz;
  a.xz = e.xy * e.yz - cyy * e.xz;
  a.xy = e.xz * e.yz - czz * e.xy;
  return a;
}

// adjugate of F = I + D (general): F^{-1} = adj(F) / J
template <class R>
__device__ __forceinline__ void adj_F(const R (&D)[3][3], R (&A)[3][3]) {
  R f00 = 1 + D[0][0], f11 = 1 + D[1][1], f22 = 1 + D[2][2];
  R f01 = D[0][1], f02 = D[0][2], f10 = D[1][0], f12 = D[1][2], f20 = D[2][0], f21 = D[2][1];
  A[0][0] = f11 * f22 - f12 * f21;
  A[0][1] = f02 * f21 - f01 * f22;
  A[0][2] = f01 * f12 - f02 * f11;
  A[1][0] = f12 * f20 - f10 * f22;
  A[1][1] = f00 * f22 - f02 * f20;
  A[1][2] = f02 * f10 - f00 * f12;
  A[2][0] = f10 * f21 - f11 * f20;
  A[2][1] = f01 * f20 - f00 * f21;
  A[2][2] = f00 * f11 - f01 * f10;
}

// s * M * W * M^T for symmetric W (upper triangle returned)
template <class R>
__device__ __forceinline__ Sym6<R> congruence(const R (&M)[3][3], const Sym6<R> &W, R s) {
  R w[3][3] = {{W.xx, W.xy, W.xz}, {W.xy, W.yy, W.yz}, {W.xz, W.yz, W.zz}};
  R T[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) T[i][j] = M[i][0] * w[0][j] + M[i][1] * w[1][j] + M[i][2] * w[2][j];
  Sym6<R> r;
  r.xx = s * (T[0][0] * M[0][0] + T[0][1] * M[0][1] + T[0][2] * M[0][2]);
  r.yy = s * (T[1][0] * M[1][0] + T[1][1] * M[1][1] + T[1][2] * M[1][2]);
  r.zz = s * (T[2][0] * M[2][0] + T[2][1] * M[2][1] + T[2][2] * M[2][2]);
  r.yz = s * (T[1][0] * M[2][0] + T[1][1] * M[2][1] + T[1][2] * M[2][2]);
  r.xz = s * (T[0][0] * M[2][0] + T[0][1] * M[2][1] + T[0][2] * M[2][2]);
  r.xy = s * (T[0][0] * M[1][0] + T[0][1] * M[1][1] + T[0][2] * M[1][2]);
  return r;
}

template <class R>
__device__ __forceinline__ Sym6<R> sym_scale(const Sym6<R> &a, R s) {
  return Sym6<R>{a.xx * s, a.yy * s, a.zz * s, a.yz * s, a.xz * s, a.xy * s};
}

// ---- 1: compressible Neo-Hookean, CompressibleNeoHookean.cpp:15-55 ----
// S = mu (I - C^-1) + lambda ln J C^-1 = C^-1 (mu 2E + lambda ln J I)
template <class R>
__device__ __forceinline__ Sym6<R> mat_neohookean(const MatP<R> &m, const R (&D)[3][3], R Jm1) {
  R mu = m.p[1], lam = m.p[2];
  Sym6<R> e = two_E(D);
  Sym6<R> a = adj_I_plus(e);
  R J = 1 + Jm1;
  R iJ2 = 1 / (J * J);
  R t = lam * d_log1p(Jm1);
  // T = mu*2E + t I
  R txx = mu * e.xx + t, tyy = mu * e.yy + t, tzz = mu * e.zz + t;
  R tyz = mu * e.yz, txz = mu * e.xz, txy = mu * e.xy;
  Sym6<R> S;
  S.xx = iJ2 * (a.xx * txx + a.xy * txy + a.xz * txz);
  S.yy = iJ2 * (a.xy * txy + a.yy * tyy + a.yz * tyz);
  S.zz = iJ2 * (a.xz * txz + a.yz * tyz + a.zz * tzz);
  S.yz = iJ2 * (a.xy * txz + a.yy * tyz + a.yz * tzz);
  S.xz = iJ2 * (a.xx * txz + a.xy * tyz + a.xz * tzz);
  S.xy = iJ2 * (a.xx * txy + a.xy * tyy + a.xz * tyz);
  return S;
}

// ---- 2: St. Venant-Kirchhoff, StVenantKirchhoff.cpp:16-54 ----
template <class R>
__device__ __forceinline__ Sym6<R> mat_svk(const MatP<R> &m, const R (&D)[3][3]) {
  R mu = m.p[1], lam = m.p[2];
  Sym6<R> e = two_E(D);  // 2E
  R tr = R(0.5) * (e.xx + e.yy + e.zz);
  return Sym6<R>{mu * e.xx + lam * tr, mu * e.yy + lam * tr, mu * e.zz + lam * tr,
                 mu * e.yz, mu * e.xz, mu * e.xy};
}

// ---- 3: linear elastic, LinearElastic.cpp:14-68: S = F^-1 (mu (F + F^T - 2I) + lambda tr eps I),
// stored from the upper triangle of the (non-symmetric) product ----
template <class R>
__device__ __forceinline__ Sym6<R> mat_linear(const MatP<R> &m, const R (&D)[3][3], R Jm1) {
  R mu = m.p[1], lam = m.p[2];
  R tr = D[0][0] + D[1][1] + D[2][2];
  R P[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) P[i][j] = mu * (D[i][j] + D[j][i]) + (i == j ? lam * tr : R(0));
  R A[3][3];
  adj_F(D, A);
  R iJ = 1 / (1 + Jm1);
  Sym6<R> S;
  S.xx = iJ * (A[0][0] * P[0][0] + A[0][1] * P[1][0] + A[0][2] * P[2][0]);
  S.yy = iJ * (A[1][0] * P[0][1] + A[1][1] * P[1][1] + A[1][2] * P[2][1]);
  S.zz = iJ * (A[2][0] * P[0][2] + A[2][1] * P[1][2] + A[2][2] * P[2][2]);
  S.yz = iJ * (A[1][0] * P[0][2] + A[1][1] * P[1][2] + A[1][2] * P[2][2]);
  S.xz = iJ * (A[0][0] * P[0][2] + A[0][1] * P[1][2] + A[0][2] * P[2][2]);
  S.xy = iJ * (A[0][0] * P[0][1] + A[0][1] * P[1][1] + A[0][2] * P[2][1]);
  return S;
}

// Isochoric Cauchy-type tensor of the HGO family pulled back to PK2:
//   S_iso = J F^-1 [ (c1 dev(Bbar) + c4 dev(abar x abar)) / J ] F^-T,
// with Bbar = J^-2/3 B, abar = J^-1/3 F a0.  c4 = 0 drops the fibre term.
template <class R>
__device__ __forceinline__ Sym6<R> hgo_iso_pk2(const R (&D)[3][3], R J, R Jm23,
                                               const Sym6<R> &eB, R c1, R c4, const R (&a)[3]) {
  R t3 = (eB.xx + eB.yy + eB.zz) * R(1.0 / 3.0);  // dev(B) = dev(2e)
  R aa3 = (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) * R(1.0 / 3.0);
  R s = Jm23;
  Sym6<R> W;
  W.xx = s * (c1 * (eB.xx - t3) + c4 * (a[0] * a[0] - aa3));
  W.yy = s * (c1 * (eB.yy - t3) + c4 * (a[1] * a[1] - aa3));
  W.zz = s * (c1 * (eB.zz - t3) + c4 * (a[2] * a[2] - aa3));
  W.yz = s * (c1 * eB.yz + c4 * a[1] * a[2]);
  W.xz = s * (c1 * eB.xz + c4 * a[0] * a[2]);
  W.xy = s * (c1 * eB.xy + c4 * a[0] * a[1]);
  // J F^-1 (W/J) F^-T = adj(F) W adj(F)^T / J^2
  return W;
}

// ---- 4/5/7: HGO family (HGOIsotropic.cpp:21-115, HGOIsotropicViscoelastic.cpp:27-168) ----
// Returns the isochoric PK2 part (which is also the reference's "Sdev") and the
// volumetric part separately so the viscoelastic update can use S_iso.
// J^{-2/3} - 1 from x = J - 1: in FP32 for |x| < 1/32 the binomial series
// of (1 + x)^{-2/3} to degree 7 (truncation below 2^-40 relative), else
// expm1(-2/3 log1p(x)); FP64 always the library functions.
template <class R>
__device__ __forceinline__ R jm23m1_of(R x) {
  if (sizeof(R) == 4 && fabs(x) < R(0.03125)) {
    // binom(-2/3, k): -2/3, 5/9, -40/81, 110/243, -308/729, 2618/6561, -7480/19683
    return x * (R(-2.0 / 3.0) + x * (R(5.0 / 9.0) + x * (R(-40.0 / 81.0) +
                x * (R(110.0 / 243.0) + x * (R(-308.0 / 729.0) + x * (R(2618.0 / 6561.0) +
                x * R(-7480.0 / 19683.0)))))));
  }
  return d_expm1(R(-2.0 / 3.0) * d_log1p(x));
}
template <class R, bool FIBER>
__device__ __forceinline__ void mat_hgo_parts(const MatP<R> &m, const R (&D)[3][3], R Jm1,
                                              const R (&a0)[3], Sym6<R> &Siso, Sym6<R> &Svol) {
  R mu = m.p[1], k1 = m.p[3], k2 = m.p[4];
  R kappa = FIBER ? m.p[7] : R(1.0 / 3.0);
  R J = 1 + Jm1;
  R Jm23m1 = jm23m1_of(Jm1);
  R Jm23 = 1 + Jm23m1;
  Sym6<R> eB = two_e_left(D);
  R I1m3 = 3 * Jm23m1 + Jm23 * (eB.xx + eB.yy + eB.zz);
  R a[3] = {R(0), R(0), R(0)};
  R Ea = kappa * I1m3;
  if (FIBER) {
#pragma unroll
    for (int i = 0; i < 3; ++i) a[i] = a0[i] + D[i][0] * a0[0] + D[i][1] * a0[1] + D[i][2] * a0[2];
    R da0 = a[0] * a0[0] + a[1] * a0[1] + a[2] * a0[2] - 1;  // a0 . D a0
    R Da2 = (a[0] - a0[0]) * (a[0] - a0[0]) + (a[1] - a0[1]) * (a[1] - a0[1]) +
            (a[2] - a0[2]) * (a[2] - a0[2]);
    R q = 2 * da0 + Da2;  // |F a0|^2 - 1
    R I4m1 = Jm23m1 + Jm23 * q;
    Ea += (1 - 3 * kappa) * I4m1;
  }
  R dW = Ea > 0 ? k1 * Ea * d_exp(k2 * Ea * Ea) : R(0);  // dW_f/dE_alpha
  R c1 = mu + 2 * dW * kappa;
  R c4 = FIBER ? 2 * dW * (1 - 3 * kappa) : R(0);
  Sym6<R> W = hgo_iso_pk2(D, J, Jm23, eB, c1, c4, a);
  R A[3][3];
  adj_F(D, A);
  R iJ2 = 1 / (J * J);
  Siso = congruence(A, W, iJ2);
  // S_vol = J p C^-1, p = K (J^2 - 1) / (2 J)  (HGOIsotropic.cpp:47)
  Sym6<R> ce = two_E(D);
  Sym6<R> ac = adj_I_plus(ce);
  R Jp = R(0.5) * m.K * Jm1 * (2 + Jm1);
  Svol = sym_scale(ac, Jp * iJ2);
}

// ---- 6: one-term Ogden (new): W = 2mu/alpha^2 sum(lbar_i^alpha - 1) + K/2((J^2-1)/2 - ln J) ----
// Principal directions by cyclic Jacobi on 2E (fixed sweep count).
template <class R, int SWEEPS>
__device__ __forceinline__ void jacobi_sym3(Sym6<R> A, R (&w)[3], R (&V)[3][3]) {
  R a00 = A.xx, a11 = A.yy, a22 = A.zz, a01 = A.xy, a02 = A.xz, a12 = A.yz;
  R v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const R tiny = sizeof(R) == 4 ? R(1e-37) : R(1e-300);
#pragma unroll
  for (int sw = 0; sw < SWEEPS; ++sw) {
    // rotation (p,q) = (0,1)
    {
      R tau = a11 - a00, apq = a01;
      R sg = tau >= 0 ? R(1) : R(-1);
      R t = 2 * apq * sg / (fabs(tau) + d_sqrt(tau * tau + 4 * apq * apq) + tiny);
      R c = 1 / d_sqrt(1 + t * t), s = t * c;
      a00 -= t * apq;
      a11 += t * apq;
      a01 = 0;
      R r0 = a02, r1 = a12;
      a02 = c * r0 - s * r1;
      a12 = s * r0 + c * r1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        R vp = v[k][0], vq = v[k][1];
        v[k][0] = c * vp - s * vq;
        v[k][1] = s * vp + c * vq;
      }
    }
    // (0,2)
    {
      R tau = a22 - a00, apq = a02;
      R sg = tau >= 0 ? R(1) : R(-1);
      R t = 2 * apq * sg / (fabs(tau) + d_sqrt(tau * tau + 4 * apq * apq) + tiny);
      R c = 1 / d_sqrt(1 + t * t), s = t * c;
      a00 -= t * apq;
      a22 += t * apq;
      a02 = 0;
      R r0 = a01, r1 = a12;
      a01 = c * r0 - s * r1;
      a12 = s * r0 + c * r1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        R vp = v[k][0], vq = v[k][2];
        v[k][0] = c * vp - s * vq;
        v[k][2] = s * vp + c * vq;
      }
    }
    // (1,2)
    {
      R tau = a22 - a11, apq = a12;
      R sg = tau >= 0 ? R(1) : R(-1);
      R t = 2 * apq * sg / (fabs(tau) + d_sqrt(tau * tau + 4 * apq * apq) + tiny);
      R c = 1 / d_sqrt(1 + t * t), s = t * c;
      a11 -= t * apq;
      a22 += t * apq;
      a12 = 0;
      R r0 = a01, r1 = a02;
      a01 = c * r0 - s * r1;
      a02 = s * r0 + c * r1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        R vp = v[k][1], vq = v[k][2];
        v[k][1] = c * vp - s * vq;
        v[k][2] = s * vp + c * vq;
      }
    }
  }
  w[0] = a00;
  w[1] = a11;
  w[2] = a22;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) V[i][j] = v[i][j];
}

// symmetric product of two commuting symmetric matrices (powers of one matrix)
template <class R>
__device__ __forceinline__ Sym6<R> sym_mul(const Sym6<R> &a, const Sym6<R> &b) {
  Sym6<R> r;
  r.xx = a.xx * b.xx + a.xy * b.xy + a.xz * b.xz;
  r.yy = a.xy * b.xy + a.yy * b.yy + a.yz * b.yz;
  r.zz = a.xz * b.xz + a.yz * b.yz + a.zz * b.zz;
  r.yz = a.xy * b.xz + a.yy * b.yz + a.yz * b.zz;
  r.xz = a.xx * b.xz + a.xy * b.yz + a.xz * b.zz;
  r.xy = a.xx * b.xy + a.xy * b.yy + a.xz * b.yz;
  return r;
}

// ln(1 + x) and exp(y) for the small arguments of nearly incompressible
// tissue (|J - 1| << 1): in FP32 the Taylor polynomials to degree 6 and 5
// (truncation below 2^-40 relative for |x|, |y| < 1/32), else the library
// functions; FP64 always the library functions.
template <class R>
__device__ __forceinline__ R log1p_small(R x) {
  if (sizeof(R) == 4 && fabs(x) < R(0.03125))
    return x * (R(1) + x * (R(-0.5) + x * (R(1.0 / 3.0) + x * (R(-0.25) +
                x * (R(0.2) + x * R(-1.0 / 6.0))))));
  return d_log1p(x);
}
template <class R>
__device__ __forceinline__ R exp_small(R y) {
  if (sizeof(R) == 4 && fabs(y) < R(0.03125))
    return R(1) + y * (R(1) + y * (R(0.5) + y * (R(1.0 / 6.0) + y * (R(1.0 / 24.0) +
                y * R(1.0 / 120.0)))));
  return d_exp(y);
}

template <class R>
__device__ __forceinline__ Sym6<R> mat_ogden(const MatP<R> &m, const R (&D)[3][3], R Jm1) {
  R mu = m.p[1], alpha = m.p[3];
  Sym6<R> e = two_E(D);
  R lnJ = log1p_small(Jm1);
  Sym6<R> S;
  const R n2 = e.xx * e.xx + e.yy * e.yy + e.zz * e.zz +
               2 * (e.yz * e.yz + e.xz * e.xz + e.xy * e.xy);
  if (n2 < m.ser_thr2) {
    // Small strain: with M = 2E = C - I the isochoric stress is
    //   S_iso = (2 mu/alpha) J^{-alpha/3} [C^{alpha/2-1} - tr(C^{alpha/2})/3 C^{-1}]
    //         = c [A - Ci - tr(B)/3 (I + Ci)],
    // A = (I+M)^{alpha/2-1} - I, a binomial series in powers of M (exact to
    // FP32 rounding below the host's bound on |M|_F, no eigenvectors, no
    // cancellation of O(1) terms), and B = (I+M)^{alpha/2} - I = A + M + M A
    // (exact: (I+M)^{alpha/2} = (I+M)(I+A)).  By Cayley-Hamilton every power
    // is M^p = a I + b M + c M^2 with
    //   M^{p+1}: (a, b, c) <- (c I3, a - c I2, b + c I1),
    // so the series reduces to scalar coefficients of I, M and M^2, and
    //   tr B = I1 + tr A + tr(M A),  tr M^3 = I1 tr M^2 - I2 I1 + 3 I3.
    // Ci = (I+M)^{-1} - I is exact by Cayley-Hamilton for C = I + M:
    //   C^{-1} = (C^2 - I1(C) C + I2(C) I) / I3(C)
    //   => Ci = (-I3 I - (1 + I1) M + M^2) / (1 + I1 + I2 + I3)
    // (I1..I3: invariants of M; no cancellation).
    const Sym6<R> M2 = sym_mul(e, e);
    const R I1 = e.xx + e.yy + e.zz;
    const R trM2 = M2.xx + M2.yy + M2.zz;
    const R I2 = R(0.5) * (I1 * I1 - trM2);
    const R I3 = e.xx * (e.yy * e.zz - e.yz * e.yz) - e.xy * (e.xy * e.zz - e.yz * e.xz) +
                 e.xz * (e.xy * e.yz - e.yy * e.xz);
    // power 1: (0, 1, 0)
    R pa = 0, pb = 1, pc = 0;
    R Aa = 0, Ab = m.ser_a[0], Ag = 0;  // A  = Aa I + Ab M + Ag M^2
#pragma unroll
    for (int k = 1; k < kOgdenSeries; ++k) {
      const R na = pc * I3, nb = pa - pc * I2, nc = pb + pc * I1;
      pa = na;
      pb = nb;
      pc = nc;
      const R sa = m.ser_a[k];
      Aa += sa * pa;
      Ab += sa * pb;
      Ag += sa * pc;
    }
    const R trM3 = I1 * (trM2 - I2) + R(3) * I3;
    const R trB = I1 + (R(3) * Aa + Ab * I1 + Ag * trM2) + (Aa * I1 + Ab * trM2 + Ag * trM3);
    const R iC3 = R(1) / (1 + I1 + I2 + I3);  // Ci = Ca I + Cb M + Cg M^2
    const R Ca = -I3 * iC3, Cb = -(1 + I1) * iC3, Cg = iC3;
    const R c = 2 * mu / alpha * exp_small(-alpha * R(1.0 / 3.0) * lnJ);
    const R t = trB * R(1.0 / 3.0);
    // the volumetric part J p C^{-1} in the same basis: C^{-1} = I + Ci, and
    // J p = K (J^2 - 1) / 2 (HGOIsotropic.cpp:47 form) -- no second inverse
    const R Jp = R(0.5) * m.K * Jm1 * (2 + Jm1);
    const R ka = c * (Aa - Ca - t * (1 + Ca)) + Jp * (1 + Ca),
            kb = c * (Ab - Cb - t * Cb) + Jp * Cb, kg = c * (Ag - Cg - t * Cg) + Jp * Cg;
    S.xx = ka + kb * e.xx + kg * M2.xx;
    S.yy = ka + kb * e.yy + kg * M2.yy;
    S.zz = ka + kb * e.zz + kg * M2.zz;
    S.yz = kb * e.yz + kg * M2.yz;
    S.xz = kb * e.xz + kg * M2.xz;
    S.xy = kb * e.xy + kg * M2.xy;
    return S;
  } else {
    R w[3], V[3][3];
    jacobi_sym3<R, sizeof(R) == 4 ? 4 : 6>(e, w, V);
    R em[3], mean = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      R y = R(0.5) * alpha * (d_log1p(w[i]) - R(2.0 / 3.0) * lnJ);  // (alpha/2) ln lbar_i^2
      em[i] = d_expm1(y);
      mean += em[i];
    }
    mean *= R(1.0 / 3.0);
    R c = 2 * mu / alpha;
    R f[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) f[i] = c * (em[i] - mean) / (1 + w[i]);
    S.xx = f[0] * V[0][0] * V[0][0] + f[1] * V[0][1] * V[0][1] + f[2] * V[0][2] * V[0][2];
    S.yy = f[0] * V[1][0] * V[1][0] + f[1] * V[1][1] * V[1][1] + f[2] * V[1][2] * V[1][2];
    S.zz = f[0] * V[2][0] * V[2][0] + f[1] * V[2][1] * V[2][1] + f[2] * V[2][2] * V[2][2];
    S.yz = f[0] * V[1][0] * V[2][0] + f[1] * V[1][1] * V[2][1] + f[2] * V[1][2] * V[2][2];
    S.xz = f[0] * V[0][0] * V[2][0] + f[1] * V[0][1] * V[2][1] + f[2] * V[0][2] * V[2][2];
    S.xy = f[0] * V[0][0] * V[1][0] + f[1] * V[0][1] * V[1][1] + f[2] * V[0][2] * V[1][2];
  }
  Sym6<R> ac = adj_I_plus(e);
  R J = 1 + Jm1;
  R Jp = R(0.5) * m.K * Jm1 * (2 + Jm1) / (J * J);
  S.xx += Jp * ac.xx;
  S.yy += Jp * ac.yy;
  S.zz += Jp * ac.zz;
  S.yz += Jp * ac.yz;
  S.xz += Jp * ac.xz;
  S.xy += Jp * ac.xy;
  return S;
}

}  // namespace ftgpu
