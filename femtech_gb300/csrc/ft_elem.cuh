// ft_elem.cuh -- element kernels: internal force, stress update, stable-dt
// contribution and in-block deterministic assembly, one thread block per mesh
// patch.
//
// Reference path replaced (per element, per Gauss point):
//   CalculateDeformationGradient.cpp:4-30, DeterminateF.cpp:38-57,
//   StressUpdate.cpp:7-27 + materials/*, InternalForceUpdate.cpp:4-28 with
//   StrainDisplacementMatrix.cpp:25-77, the element scatter of
//   GetForce_3D.cpp:39-44, and the per-element part of StableTimeStep.cpp:4-40
//   (CalculateTimeStep.cpp:7-21, CalculateCharacteristicLength_C3D8/C3D4).
//
// GB300 layout: a patch is a spatially compact set of <= 256 elements whose
// <= 320 distinct nodes are replicated contiguously ("slots"), so the block
// stages node data with coalesced loads into shared memory, every thread
// computes one element, corner forces land in shared memory and are summed per
// local node in a fixed order (local CSR), and one partial force per slot goes
// back to HBM.  The node kernel adds the (1-8) partials of each node in slot
// order: no floating-point atomics anywhere, so runs are bitwise reproducible.
//
// C3D8 kinematics use the tensor-product structure of the trilinear element:
// the 8 nodal displacement vectors are Hadamard-transformed once, after which
// every column of du/dxi at a Gauss point costs 3 FMAs, and the B0^T S
// contraction is accumulated as 7 moment vectors that one inverse transform
// turns into the 8 nodal forces.  The reference Jacobian's inverse and
// determinant at each Gauss point come from a table written at set-up (FP32
// kernels) or from the same transform of the reference coordinates (FP64).
// Mathematically this is the reference's
//   F = sum_a x_a (x) dN_a/dX,  f_a = sum_gp w detJ B0_a^T S.
#pragma once

#include "ft_common.h"
#include "ft_injury.cuh"

namespace ftgpu {

template <class R> __device__ __forceinline__ R r_inf();
template <> __device__ __forceinline__ float r_inf<float>() { return __int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double r_inf<double>() {
  return __longlong_as_double(0x7ff0000000000000ll);
}

// Hadamard transform of the 8 corner vectors of a C3D8 (node signs of
// ShapeFunction_C3D8.cpp:26-33), scaled by 1/8:
// h = [xi, eta, zeta, xi.eta, xi.zeta, eta.zeta, xi.eta.zeta]
template <class R>
__device__ __forceinline__ void hex_hadamard(const R (&x)[8][3], R (&h)[7][3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    R d0 = x[1][d] - x[0][d], d1 = x[2][d] - x[3][d], d2 = x[5][d] - x[4][d], d3 = x[6][d] - x[7][d];
    R s0 = x[1][d] + x[0][d], s1 = x[2][d] + x[3][d], s2 = x[5][d] + x[4][d], s3 = x[6][d] + x[7][d];
    const R q = R(0.125);
    h[0][d] = q * ((d0 + d1) + (d2 + d3));
    h[3][d] = q * ((d1 - d0) + (d3 - d2));
    h[4][d] = q * ((d2 + d3) - (d0 + d1));
    h[6][d] = q * ((d0 - d1) + (d3 - d2));
    h[1][d] = q * ((s1 - s0) + (s3 - s2));
    h[2][d] = q * ((s2 + s3) - (s0 + s1));
    h[5][d] = q * ((s0 - s1) + (s3 - s2));
  }
}

// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}
// 4- or 8-byte asynchronous global -> shared copy (addresses aligned to n)
template <int NB>
__device__ __forceinline__ void cp_async_small(void *smem_dst, const void *gsrc) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(gsrc), "n"(NB)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <class R> struct Pair;
template <> struct Pair<float> { using T = float2; };
template <> struct Pair<double> { using T = double2; };

// Gauss point g of the 2x2x2 rule in the order of GaussQuadrature3D.cpp:17-58
// (the literal 0.577350269189626 as there): xi > 0 for g in {1,2,5,6},
// eta > 0 for {2,3,6,7}, zeta > 0 for g < 4.
template <class R>
__device__ __forceinline__ void hex_gauss_point(int g, R &xi, R &et, R &ze) {
  const R G = R(0.577350269189626);
  xi = ((g + 1) & 2) ? G : -G;
  et = (g & 2) ? G : -G;
  ze = g < 4 ? G : -G;
}

template <class R>
__device__ __forceinline__ void adj3(const R (&A)[3][3], R (&J)[3][3], R &det) {
  J[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  J[0][1] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
  J[0][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  J[1][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  J[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
  J[1][2] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
  J[2][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  J[2][1] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
  J[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  det = A[0][0] * J[0][0] + A[0][1] * J[1][0] + A[0][2] * J[2][0];
}

// Per-Gauss-point material update on the displacement gradient D = F - I.
// hist points at this element's first history component (stride hs per
// component, gstride per Gauss point).
// Green strain (Voigt, tensor shear) from D
template <class R>
__device__ __forceinline__ void green_strain(const R (&D)[3][3], R (&E)[6]) {
  const Sym6<R> e = two_E(D);
  E[0] = R(0.5) * e.xx;
  E[1] = R(0.5) * e.yy;
  E[2] = R(0.5) * e.zz;
  E[3] = R(0.5) * e.yz;
  E[4] = R(0.5) * e.xz;
  E[5] = R(0.5) * e.xy;
}

// Surrogate input features of one Gauss point as 16 BF16 values (32 bytes).
template <class R>
__device__ __forceinline__ void write_surrogate_features(const R (&D)[3][3], const R (&a0)[3],
                                                         const SurrogateLaw &law, uint16_t *out) {
  R E[6], Slin[6], scale;
  green_strain(D, E);
  float x[kMlpUsedIn];
  surrogate_features(E, a0, law, x, Slin, scale);
  uint32_t w[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float lo = 2 * k < kMlpUsedIn ? x[2 * k] : 0.f;
    const float hi = 2 * k + 1 < kMlpUsedIn ? x[2 * k + 1] : 0.f;
    w[k] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
  }
  reinterpret_cast<uint4 *>(out)[0] = make_uint4(w[0], w[1], w[2], w[3]);
  reinterpret_cast<uint4 *>(out)[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// Material 7 isochoric stress from the surrogate's output sy (inside the trust
// region |E|_F^2 <= trust_e2), else from the plain law; volumetric part exact.
template <class R>
__device__ __forceinline__ void goh_parts_surrogate(const MatP<R> &mp, const R (&D)[3][3], R Jm1,
                                                    const R (&a0)[3], const float *sy,
                                                    const SurrogateLaw &law, Sym6<R> &Si,
                                                    Sym6<R> &Sv) {
  R E[6], Slin[6], scale;
  green_strain(D, E);
  const R e2 = E[0] * E[0] + E[1] * E[1] + E[2] * E[2] +
               R(2) * (E[3] * E[3] + E[4] * E[4] + E[5] * E[5]);
  if (!(e2 <= R(law.trust_e2))) {
    mat_hgo_parts<R, true>(mp, D, Jm1, a0, Si, Sv);
    return;
  }
  float x[kMlpUsedIn];
  surrogate_features(E, a0, law, x, Slin, scale);
  Si = Sym6<R>{Slin[0] + scale * R(sy[0]), Slin[1] + scale * R(sy[1]),
               Slin[2] + scale * R(sy[2]), Slin[3] + scale * R(sy[3]),
               Slin[4] + scale * R(sy[4]), Slin[5] + scale * R(sy[5])};
  const Sym6<R> ce = two_E(D);
  const Sym6<R> ac = adj_I_plus(ce);
  const R J = 1 + Jm1;
  const R Jp = R(0.5) * mp.K * Jm1 * (2 + Jm1) / (J * J);
  Sv = sym_scale(ac, Jp);
}

// hin: the Gauss point's history already loaded into registers (same order
// as hist[c * hs]), or nullptr to read it from hist
template <class R, int MAT>
__device__ __forceinline__ Sym6<R> stress_at(const MatP<R> &mp, const R (&D)[3][3], R Jm1,
                                             const R (&a0)[3], R *hist, long long hs,
                                             const R (&pc)[4], const float *sy,
                                             const SurrogateLaw &law, const R *hin = nullptr) {
  Sym6<R> S;
  if (MAT == 0) {
    S = Sym6<R>{0, 0, 0, 0, 0, 0};
  } else if (MAT == 1) {
    S = mat_neohookean(mp, D, Jm1);
  } else if (MAT == 2) {
    S = mat_svk(mp, D);
  } else if (MAT == 3) {
    S = mat_linear(mp, D, Jm1);
  } else if (MAT == 4) {
    Sym6<R> Si, Sv;
    mat_hgo_parts<R, false>(mp, D, Jm1, a0, Si, Sv);
    S = Sym6<R>{Si.xx + Sv.xx, Si.yy + Sv.yy, Si.zz + Sv.zz, Si.yz + Sv.yz, Si.xz + Sv.xz,
                Si.xy + Sv.xy};
  } else if (MAT == 6) {
    S = mat_ogden(mp, D, Jm1);
  } else {  // 5 / 7: HGO family + Prony series (HGOIsotropicViscoelastic.cpp:98-159)
    Sym6<R> Si, Sv;
    if (MAT == 7 && sy != nullptr)
      goh_parts_surrogate(mp, D, Jm1, a0, sy, law, Si, Sv);
    else
      mat_hgo_parts<R, MAT == 7>(mp, D, Jm1, a0, Si, Sv);
    R sd[6] = {Si.xx, Si.yy, Si.zz, Si.yz, Si.xz, Si.xy};
    R sv[6] = {Sv.xx, Sv.yy, Sv.zz, Sv.yz, Sv.xz, Sv.xy};
    constexpr int NT = MAT == 5 ? 2 : 1;
    R out[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      R s0 = hin ? hin[NT * 6 + c] : hist[(NT * 6 + c) * hs];
      R dS = sd[c] - s0;
      R h1 = pc[0] * (hin ? hin[c] : hist[c * hs]) + pc[1] * dS;
      hist[c * hs] = h1;
      R acc = sd[c] + sv[c] + h1;
      if (NT == 2) {
        R h2 = pc[2] * (hin ? hin[6 + c] : hist[(6 + c) * hs]) + pc[3] * dS;
        hist[(6 + c) * hs] = h2;
        acc += h2;
      }
      hist[(NT * 6 + c) * hs] = sd[c];
      out[c] = acc;
    }
    S = Sym6<R>{out[0], out[1], out[2], out[3], out[4], out[5]};
  }
  return S;
}

// Prony constants c1 = exp(-dt/tau), c2 = g (1 - c1) / (dt/tau) per term
// (HGOIsotropicViscoelastic.cpp:122-131), with 1 - c1 taken as -expm1 so that
// dt << tau keeps its digits in FP32.
template <class R, int MAT>
__device__ __forceinline__ void prony_consts(const MatP<R> &mp, R dt, R (&pc)[4]) {
  pc[0] = pc[1] = pc[2] = pc[3] = 0;
  if (MAT == 5 || MAT == 7) {
    R rt1 = dt / mp.p[6];
    pc[0] = d_exp(-rt1);
    pc[1] = mp.p[5] * (-d_expm1(-rt1)) / rt1;
    if (MAT == 5) {
      R rt2 = dt / mp.p[8];
      pc[2] = d_exp(-rt2);
      pc[3] = mp.p[7] * (-d_expm1(-rt2)) / rt2;
    }
  }
}

template <class R>
__device__ __forceinline__ R norm3(R x, R y, R z) {
  return d_sqrt(x * x + y * y + z * z);
}

// areaHexahedronFace, src/math/Geometry.cpp:29-64 (signed tolerance test kept;
// the 2x2 quadrature uses (q cD + c1) x (q' cD + c2) = c1 x c2 + q cD x c2 + q' c1 x cD).
// (FP64 path; the FP32 C3D8 kernels take face_pair_area_max)
template <class R>
__device__ __forceinline__ R hex_face_area(const R (&xc)[8][3], int i1, int i2, int i3, int i4) {
  R cD[3], c1[3], c2[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    R p1 = xc[i1][k], p2 = xc[i2][k], p3 = xc[i3][k], p4 = xc[i4][k];
    cD[k] = R(0.25) * (p1 - p2 + p3 - p4);
    c1[k] = R(0.25) * (-p1 + p2 + p3 - p4);
    c2[k] = R(0.25) * (-p1 - p2 + p3 + p4);
  }
  R n0x = c1[1] * c2[2] - c1[2] * c2[1], n0y = c1[2] * c2[0] - c1[0] * c2[2],
    n0z = c1[0] * c2[1] - c1[1] * c2[0];
  const R tol = R(1e-6);
  if (cD[0] < tol && cD[1] < tol && cD[2] < tol) return 4 * norm3(n0x, n0y, n0z);
  R n1x = cD[1] * c2[2] - cD[2] * c2[1], n1y = cD[2] * c2[0] - cD[0] * c2[2],
    n1z = cD[0] * c2[1] - cD[1] * c2[0];
  R n2x = c1[1] * cD[2] - c1[2] * cD[1], n2y = c1[2] * cD[0] - c1[0] * cD[2],
    n2z = c1[0] * cD[1] - c1[1] * cD[0];
  const R t = R(0.57735026918962576451);
  R area = 0;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      R qj = j ? t : -t, qi = i ? t : -t;
      area += norm3(n0x + qj * n1x + qi * n2x, n0y + qj * n1y + qi * n2y,
                    n0z + qj * n1z + qi * n2z);
    }
  return area;
}

// FP32 Gauss loop of the C3D8 element with packed FP32 arithmetic: every
// 3x3 product of the kinematics and of B0^T S (du/dxi, D = H A^-T,
// P = S + D S, P A^-1, the moments) carries rows 0 and 1 as one float2
// (fma.rn.f32x2: two independent IEEE fma, half the issued instructions;
// a scalar operand is broadcast at no cost) and row 2 as a scalar.  The
// material law sees the same scalar D as the generic loop.
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }

// hex_hadamard with components x, y of every corner as one float2 and z as a
// scalar (a - b as fma(b, -1, a): one rounding, as the scalar subtraction)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bc2(-1.f), a); }
__device__ __forceinline__ void hex_hadamard_x2(const float2 (&p)[8], const float (&z)[8],
                                                float2 (&hp)[7], float (&hz)[7]) {
  const float2 q = bc2(0.125f);
  {
    const float2 d0 = sub2(p[1], p[0]), d1 = sub2(p[2], p[3]), d2 = sub2(p[5], p[4]),
                 d3 = sub2(p[6], p[7]);
    const float2 s0 = __fadd2_rn(p[1], p[0]), s1 = __fadd2_rn(p[2], p[3]),
                 s2 = __fadd2_rn(p[5], p[4]), s3 = __fadd2_rn(p[6], p[7]);
    hp[0] = __fmul2_rn(q, __fadd2_rn(__fadd2_rn(d0, d1), __fadd2_rn(d2, d3)));
    hp[3] = __fmul2_rn(q, __fadd2_rn(sub2(d1, d0), sub2(d3, d2)));
    hp[4] = __fmul2_rn(q, sub2(__fadd2_rn(d2, d3), __fadd2_rn(d0, d1)));
    hp[6] = __fmul2_rn(q, __fadd2_rn(sub2(d0, d1), sub2(d3, d2)));
    hp[1] = __fmul2_rn(q, __fadd2_rn(sub2(s1, s0), sub2(s3, s2)));
    hp[2] = __fmul2_rn(q, sub2(__fadd2_rn(s2, s3), __fadd2_rn(s0, s1)));
    hp[5] = __fmul2_rn(q, __fadd2_rn(sub2(s0, s1), sub2(s3, s2)));
  }
  {
    const float d0 = z[1] - z[0], d1 = z[2] - z[3], d2 = z[5] - z[4], d3 = z[6] - z[7];
    const float s0 = z[1] + z[0], s1 = z[2] + z[3], s2 = z[5] + z[4], s3 = z[6] + z[7];
    hz[0] = 0.125f * ((d0 + d1) + (d2 + d3));
    hz[3] = 0.125f * ((d1 - d0) + (d3 - d2));
    hz[4] = 0.125f * ((d2 + d3) - (d0 + d1));
    hz[6] = 0.125f * ((d0 - d1) + (d3 - d2));
    hz[1] = 0.125f * ((s1 - s0) + (s3 - s2));
    hz[2] = 0.125f * ((s2 + s3) - (s0 + s1));
    hz[5] = 0.125f * ((s0 - s1) + (s3 - s2));
  }
}

// The areas of two opposite faces at once (areaHexahedronFace,
// Geometry.cpp:29-64), lane x the first face, lane y the second.  In terms of
// the Hadamard coefficients h of the current corner coordinates a face's
// bilinear vectors are c1 = h_a -+ h_b, c2, cD likewise (its two faces
// differ in the sign of the third coordinate), so they form as pairs from
// broadcast scalars.  Area: for a face with all cD components below 1e-6 (the
// reference's signed test) 4 |c1 x c2|, else the 2x2 Gauss rule
// sum |n0 + a n1 + b n2|, a, b = +-1/sqrt 3, from the six dot products of
// n0 = c1 x c2, n1 = cD x c2, n2 = c1 x cD.
__device__ __forceinline__ float face_pair_area_max(const float (&h)[7][3], int a1, int b1,
                                                    int a2, int b2, int aD, int bD) {
  const float2 pm = make_float2(-1.f, 1.f), m1 = bc2(-1.f);
  float2 c1[3], c2[3], cD[3], nc2[3], ncD[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c1[k] = __ffma2_rn(bc2(h[b1][k]), pm, bc2(h[a1][k]));
    c2[k] = __ffma2_rn(bc2(h[b2][k]), pm, bc2(h[a2][k]));
    cD[k] = __ffma2_rn(bc2(h[bD][k]), pm, bc2(h[aD][k]));
    nc2[k] = __fmul2_rn(c2[k], m1);
    ncD[k] = __fmul2_rn(cD[k], m1);
  }
  const float2 n0x = __ffma2_rn(c1[1], c2[2], __fmul2_rn(c1[2], nc2[1])),
               n0y = __ffma2_rn(c1[2], c2[0], __fmul2_rn(c1[0], nc2[2])),
               n0z = __ffma2_rn(c1[0], c2[1], __fmul2_rn(c1[1], nc2[0]));
  const float2 n1x = __ffma2_rn(cD[1], c2[2], __fmul2_rn(cD[2], nc2[1])),
               n1y = __ffma2_rn(cD[2], c2[0], __fmul2_rn(cD[0], nc2[2])),
               n1z = __ffma2_rn(cD[0], c2[1], __fmul2_rn(cD[1], nc2[0]));
  const float2 n2x = __ffma2_rn(c1[1], cD[2], __fmul2_rn(c1[2], ncD[1])),
               n2y = __ffma2_rn(c1[2], cD[0], __fmul2_rn(c1[0], ncD[2])),
               n2z = __ffma2_rn(c1[0], cD[1], __fmul2_rn(c1[1], ncD[0]));
  auto dot = [](float2 ax, float2 ay, float2 az, float2 bx, float2 by, float2 bz) {
    return __ffma2_rn(az, bz, __ffma2_rn(ay, by, __fmul2_rn(ax, bx)));
  };
  const float2 d00 = dot(n0x, n0y, n0z, n0x, n0y, n0z), d11 = dot(n1x, n1y, n1z, n1x, n1y, n1z),
               d22 = dot(n2x, n2y, n2z, n2x, n2y, n2z), d01 = dot(n0x, n0y, n0z, n1x, n1y, n1z),
               d02 = dot(n0x, n0y, n0z, n2x, n2y, n2z), d12 = dot(n1x, n1y, n1z, n2x, n2y, n2z);
  const float t = 0.57735026918962576451f;
  const float2 base = __ffma2_rn(bc2(1.0f / 3.0f), __fadd2_rn(d11, d22), d00);
  const float2 a01 = __fmul2_rn(bc2(2.0f * t), d01), a02 = __fmul2_rn(bc2(2.0f * t), d02),
               a12 = __fmul2_rn(bc2(2.0f / 3.0f), d12);
  const float2 u1 = __fadd2_rn(base, a12), u2 = __ffma2_rn(a12, m1, base);
  const float2 v1 = __fadd2_rn(a01, a02), v2 = __ffma2_rn(a02, m1, a01);
  const float2 pp = __fadd2_rn(u1, v1), mm = __ffma2_rn(v1, m1, u1), pq = __fadd2_rn(u2, v2),
               mq = __ffma2_rn(v2, m1, u2);
  const float tol = 1e-6f;
  const bool par_x = cD[0].x < tol && cD[1].x < tol && cD[2].x < tol;
  const bool par_y = cD[0].y < tol && cD[1].y < tol && cD[2].y < tol;
  const float ax = par_x ? 4.f * sqrtf(d00.x)
                         : (sqrtf(fmaxf(pp.x, 0.f)) + sqrtf(fmaxf(mm.x, 0.f))) +
                               (sqrtf(fmaxf(pq.x, 0.f)) + sqrtf(fmaxf(mq.x, 0.f)));
  const float ay = par_y ? 4.f * sqrtf(d00.y)
                         : (sqrtf(fmaxf(pp.y, 0.f)) + sqrtf(fmaxf(mm.y, 0.f))) +
                               (sqrtf(fmaxf(pq.y, 0.f)) + sqrtf(fmaxf(mq.y, 0.f)));
  return fmaxf(ax, ay);
}

template <int MAT, bool GP>
__device__ __forceinline__ void hex_gauss_loop_x2(const float2 (&hp)[7], const float (&hz)[7],
                                                  const MatP<float> &mp,
                                                  const float (&pc)[4], const float (&a0)[3],
                                                  float *hist, long long hs, long long gs,
                                                  int pass, float &vol, float2 (&mc)[7],
                                                  float (&mz)[7], int &bad,
                                                  const ElemArgs<float> &A, long long gpo,
                                                  const float *gb, int rs) {
  const bool dt_only = pass == kPassDt;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    mc[k] = make_float2(0.f, 0.f);
    mz[k] = 0.f;
  }
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    float xi, et, ze;
    hex_gauss_point(g, xi, et, ze);
    const float ez = et * ze, xz = xi * ze, xe = xi * et;
    // A^{-1} (Q) and det A: values 10g .. 10g+9 as five pairs
    const int o1 = (g & 1) ? rs - 2 : 2;
    const float2 q0 = *reinterpret_cast<const float2 *>(gb),
                 q1 = *reinterpret_cast<const float2 *>(gb + o1),
                 q2 = *reinterpret_cast<const float2 *>(gb + rs),
                 q3 = *reinterpret_cast<const float2 *>(gb + rs + o1),
                 q4 = *reinterpret_cast<const float2 *>(gb + 2 * rs);
    gb += (g & 1) ? 3 * rs - 2 : 2 * rs + 2;
    const float Q[3][3] = {{q0.x, q0.y, q1.x}, {q1.y, q2.x, q2.y}, {q3.x, q3.y, q4.x}};
    const float detA = q4.y;
    // H[d][i] = du_d / dxi_i: column i, rows 0-1 paired, row 2 scalar
    const float2 Hc0 = __ffma2_rn(bc2(ez), hp[6], __ffma2_rn(bc2(ze), hp[4], __ffma2_rn(bc2(et), hp[3], hp[0])));
    const float2 Hc1 = __ffma2_rn(bc2(xz), hp[6], __ffma2_rn(bc2(ze), hp[5], __ffma2_rn(bc2(xi), hp[3], hp[1])));
    const float2 Hc2 = __ffma2_rn(bc2(xe), hp[6], __ffma2_rn(bc2(et), hp[5], __ffma2_rn(bc2(xi), hp[4], hp[2])));
    const float Hz0 = fmaf(ez, hz[6], fmaf(ze, hz[4], fmaf(et, hz[3], hz[0])));
    const float Hz1 = fmaf(xz, hz[6], fmaf(ze, hz[5], fmaf(xi, hz[3], hz[1])));
    const float Hz2 = fmaf(xe, hz[6], fmaf(et, hz[5], fmaf(xi, hz[4], hz[2])));
    // D = H A^{-T} = du/dX, column j
    float2 Dc[3];
    float Dz[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      Dc[j] = __ffma2_rn(bc2(Q[j][2]), Hc2, __ffma2_rn(bc2(Q[j][1]), Hc1, __fmul2_rn(bc2(Q[j][0]), Hc0)));
      Dz[j] = fmaf(Hz2, Q[j][2], fmaf(Hz1, Q[j][1], Hz0 * Q[j][0]));
    }
    const float D[3][3] = {{Dc[0].x, Dc[1].x, Dc[2].x}, {Dc[0].y, Dc[1].y, Dc[2].y},
                           {Dz[0], Dz[1], Dz[2]}};
    const float Jm1 = jm1_of(D);
    vol += (1 + Jm1) * detA;  // det(dx/dxi) = det A det F
    if (dt_only) continue;
    if (!(Jm1 > -1.f) || !(detA != 0)) bad = 1;
    const long long sg = gpo - A.gpbase + g;  // Gauss point within the group
    if (MAT == 7 && pass == kPassSurrogateFeatures) {
      write_surrogate_features(D, a0, A.law, A.surr_x + sg * kMlpIn);
      continue;
    }
    const float *sy = (MAT == 7 && A.surr_y) ? A.surr_y + sg * kMlpOut : nullptr;
    const Sym6<float> S = stress_at<float, MAT>(mp, D, Jm1, a0, hist + g * gs, hs, pc, sy, A.law);
    if (GP) {
      const long long q = gpo + g;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A.gpF[9 * q + i + 3 * j] = double((i == j ? 1.f : 0.f) + D[i][j]);
      A.gpJ[q] = double(1 + Jm1);
      A.gpS[6 * q + 0] = S.xx;
      A.gpS[6 * q + 1] = S.yy;
      A.gpS[6 * q + 2] = S.zz;
      A.gpS[6 * q + 3] = S.yz;
      A.gpS[6 * q + 4] = S.xz;
      A.gpS[6 * q + 5] = S.xy;
    }
    // w det J B0^T S with w = 1: s = det A S, P = s + D s, G = P A^{-1};
    // column j of s, rows 0-1 paired, and row 2
    const float2 sc[3] = {__fmul2_rn(bc2(detA), make_float2(S.xx, S.xy)),
                          __fmul2_rn(bc2(detA), make_float2(S.xy, S.yy)),
                          __fmul2_rn(bc2(detA), make_float2(S.xz, S.yz))};
    const float sz[3] = {sc[2].x, sc[2].y, detA * S.zz};
    float2 Pc[3];
    float Pz[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      // s[k][j] for k = 0, 1, 2: sc[j].x, sc[j].y, sz[j]
      Pc[j] = __ffma2_rn(bc2(sz[j]), Dc[2], __ffma2_rn(bc2(sc[j].y), Dc[1], __ffma2_rn(bc2(sc[j].x), Dc[0], sc[j])));
      Pz[j] = fmaf(Dz[2], sz[j], fmaf(Dz[1], sc[j].y, fmaf(Dz[0], sc[j].x, sz[j])));
    }
    float2 Gc[3];
    float Gz[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      Gc[j] = __ffma2_rn(bc2(Q[2][j]), Pc[2], __ffma2_rn(bc2(Q[1][j]), Pc[1], __fmul2_rn(bc2(Q[0][j]), Pc[0])));
      Gz[j] = fmaf(Pz[2], Q[2][j], fmaf(Pz[1], Q[1][j], Pz[0] * Q[0][j]));
    }
    mc[0] = __fadd2_rn(mc[0], Gc[0]);
    mc[1] = __fadd2_rn(mc[1], Gc[1]);
    mc[2] = __fadd2_rn(mc[2], Gc[2]);
    mc[3] = __ffma2_rn(bc2(et), Gc[0], __ffma2_rn(bc2(xi), Gc[1], mc[3]));
    mc[4] = __ffma2_rn(bc2(ze), Gc[0], __ffma2_rn(bc2(xi), Gc[2], mc[4]));
    mc[5] = __ffma2_rn(bc2(ze), Gc[1], __ffma2_rn(bc2(et), Gc[2], mc[5]));
    mc[6] = __ffma2_rn(bc2(ez), Gc[0], __ffma2_rn(bc2(xz), Gc[1], __ffma2_rn(bc2(xe), Gc[2], mc[6])));
    mz[0] += Gz[0];
    mz[1] += Gz[1];
    mz[2] += Gz[2];
    mz[3] = fmaf(et, Gz[0], fmaf(xi, Gz[1], mz[3]));
    mz[4] = fmaf(ze, Gz[0], fmaf(xi, Gz[2], mz[4]));
    mz[5] = fmaf(ze, Gz[1], fmaf(et, Gz[2], mz[5]));
    mz[6] = fmaf(ez, Gz[0], fmaf(xz, Gz[1], fmaf(xe, Gz[2], mz[6])));
  }
}

// Inverse transform of the moments: f_a = 1/8 sum_k sign_k(a) m_k (one
// force component row; T = float2 for rows 0-1, float for row 2)
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float add2(float a, float b) { return a + b; }
__device__ __forceinline__ float sub2(float a, float b) { return a - b; }
__device__ __forceinline__ float2 neg2(float2 a) { return __fmul2_rn(a, bc2(-1.f)); }
__device__ __forceinline__ float neg2(float a) { return -a; }
__device__ __forceinline__ float2 mul2(float s, float2 a) { return __fmul2_rn(bc2(s), a); }
__device__ __forceinline__ float mul2(float s, float a) { return s * a; }
template <class T>
__device__ __forceinline__ void hex_inverse_transform(const T (&m)[7], T (&f)[8]) {
  const float q = 0.125f;
  const T t1 = add2(m[0], m[6]), t2 = sub2(m[0], m[6]), t3 = add2(m[3], m[4]),
          t4 = sub2(m[3], m[4]);
  const T Pmm = sub2(t1, t3), Ppp = add2(t1, t3), Ppm = add2(t2, t4), Pmp = sub2(t2, t4);
  const T r1 = add2(m[1], m[2]), r2 = sub2(m[1], m[2]);
  const T Qmm = sub2(m[5], r1), Qpp = add2(m[5], r1), Qpm = sub2(r2, m[5]),
          Qmp = sub2(neg2(r2), m[5]);
  f[0] = mul2(q, sub2(Qmm, Pmm));
  f[1] = mul2(q, add2(Qmm, Pmm));
  f[2] = mul2(q, add2(Qpm, Ppm));
  f[3] = mul2(q, sub2(Qpm, Ppm));
  f[4] = mul2(q, sub2(Qmp, Pmp));
  f[5] = mul2(q, add2(Qmp, Pmp));
  f[6] = mul2(q, add2(Qpp, Ppp));
  f[7] = mul2(q, sub2(Qpp, Ppp));
}

// GEO: the Gauss points' A^{-1} and det A come from the setup-time table
// (k_elem_geo; the reference likewise evaluates dN/dX and det J once, at
// initialisation, ShapeFunctions.cpp:197-215) instead of being rebuilt from
// the reference coordinates: `geo` is this element's column of the block's
// shared-memory copy, value k of the 80-value record at geo[(k/4)*rs + k%4].
template <class R, int MAT, bool GP, bool GEO>
__device__ __forceinline__ void hex_element(const R (&x)[8][3], const R (&u)[8][3],
                                            const MatP<R> &mp, const R (&pc)[4],
                                            const R (&a0)[3], R *hist, long long hs,
                                            long long gs, int pass, R (&f)[8][3], R &le,
                                            int &bad, const ElemArgs<R> &A, long long gpo,
                                            const R *geo, int rs) {
  const bool dt_only = pass == kPassDt;
  // characteristic length on the current geometry first (volume / max face
  // area, CalculateCharacteristicLength_C3D8.cpp:6-29) so that the nodal
  // values are dead before the Gauss loop; the 2x2x2 Gauss sum of
  // det(dx/dxi) below is the exact volume of the trilinear hexahedron.
  R vol = 0;
  R m[7][3];
  const R *gb = geo;
  if constexpr (GEO && sizeof(R) == 4) {
    // FP32: corners as (x, y) pairs + z; the current geometry's Hadamard
    // coefficients give the six face areas as three opposite-face pairs
    float2 xp[8], up[8];
    float xz[8], uz[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      up[a] = make_float2(u[a][0], u[a][1]);
      uz[a] = u[a][2];
      xp[a] = __fadd2_rn(make_float2(x[a][0], x[a][1]), up[a]);
      xz[a] = x[a][2] + u[a][2];
    }
    float hcx[7][3];
    {
      float2 hcp[7];
      float hcz[7];
      hex_hadamard_x2(xp, xz, hcp, hcz);
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        hcx[k][0] = hcp[k].x;
        hcx[k][1] = hcp[k].y;
        hcx[k][2] = hcz[k];
      }
    }
    // (0123, 4567): c1 = h0 -+ h4, c2 = h1 -+ h5, cD = h3 -+ h6;
    // (0374, 1265): h1 -+ h3, h2 -+ h4, h5 -+ h6; (0154, 3267): h0 -+ h3, h2 -+ h5, h4 -+ h6
    float amax = face_pair_area_max(hcx, 0, 4, 1, 5, 3, 6);
    amax = fmaxf(amax, face_pair_area_max(hcx, 1, 3, 2, 4, 5, 6));
    amax = fmaxf(amax, face_pair_area_max(hcx, 0, 3, 2, 5, 4, 6));
    float2 hp[7], mc[7];
    float hz[7], mz[7];
    hex_hadamard_x2(up, uz, hp, hz);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      mc[k] = make_float2(0.f, 0.f);
      mz[k] = 0.f;
    }
    hex_gauss_loop_x2<MAT, GP>(hp, hz, mp, pc, a0, hist, hs, gs, pass, vol, mc, mz, bad, A, gpo,
                               gb, rs);
    le = vol / amax;
    if (pass == kPassForce) {
      float2 fp[8];
      float fz[8];
      hex_inverse_transform(mc, fp);
      hex_inverse_transform(mz, fz);
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        f[a][0] = fp[a].x;
        f[a][1] = fp[a].y;
        f[a][2] = fz[a];
      }
    }
    return;
  } else {
  R amax;
  {
    R xc[8][3];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d) xc[a][d] = x[a][d] + u[a][d];
    amax = hex_face_area(xc, 0, 1, 2, 3);
    amax = fmax(amax, hex_face_area(xc, 4, 5, 6, 7));
    amax = fmax(amax, hex_face_area(xc, 0, 3, 7, 4));
    amax = fmax(amax, hex_face_area(xc, 1, 2, 6, 5));
    amax = fmax(amax, hex_face_area(xc, 0, 1, 5, 4));
    amax = fmax(amax, hex_face_area(xc, 3, 2, 6, 7));
  }
  R hx[7][3], hu[7][3];
  if (!GEO) hex_hadamard(x, hx);
  hex_hadamard(u, hu);
#pragma unroll
  for (int i = 0; i < 7; ++i) m[i][0] = m[i][1] = m[i][2] = 0;
  // first pair of the current Gauss point in the geometry rows: value 10 g,
  // at column 0 of a row for even g and column 2 for odd g
  // The loop is not unrolled: one Gauss point's code stays in the
  // instruction cache and its temporaries are the only ones live.
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    R xi, et, ze;
    hex_gauss_point(g, xi, et, ze);
    const R ez = et * ze, xz = xi * ze, xe = xi * et;
    R Q[3][3], detA;  // Q = A^{-1}, A[i][d] = dX_d / dxi_i
    if (GEO) {
      typedef typename Pair<R>::T P2;
      // values 10g .. 10g+9 as five pairs (a pair never straddles a row)
      const int o1 = (g & 1) ? rs - 2 : 2;
      const P2 q0 = *reinterpret_cast<const P2 *>(gb),
               q1 = *reinterpret_cast<const P2 *>(gb + o1),
               q2 = *reinterpret_cast<const P2 *>(gb + rs),
               q3 = *reinterpret_cast<const P2 *>(gb + rs + o1),
               q4 = *reinterpret_cast<const P2 *>(gb + 2 * rs);
      gb += (g & 1) ? 3 * rs - 2 : 2 * rs + 2;
      Q[0][0] = q0.x; Q[0][1] = q0.y; Q[0][2] = q1.x;
      Q[1][0] = q1.y; Q[1][1] = q2.x; Q[1][2] = q2.y;
      Q[2][0] = q3.x; Q[2][1] = q3.y; Q[2][2] = q4.x;
      detA = q4.y;
    } else {
      R Am[3][3], Ad[3][3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Am[0][d] = hx[0][d] + et * hx[3][d] + ze * hx[4][d] + ez * hx[6][d];
        Am[1][d] = hx[1][d] + xi * hx[3][d] + ze * hx[5][d] + xz * hx[6][d];
        Am[2][d] = hx[2][d] + xi * hx[4][d] + et * hx[5][d] + xe * hx[6][d];
      }
      adj3(Am, Ad, detA);
      const R idet = 1 / detA;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Q[i][j] = idet * Ad[i][j];
    }
    R H[3][3];  // H[d][i] = du_d / dxi_i
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      H[d][0] = hu[0][d] + et * hu[3][d] + ze * hu[4][d] + ez * hu[6][d];
      H[d][1] = hu[1][d] + xi * hu[3][d] + ze * hu[5][d] + xz * hu[6][d];
      H[d][2] = hu[2][d] + xi * hu[4][d] + et * hu[5][d] + xe * hu[6][d];
    }
    R D[3][3];  // D = H A^{-T} = du/dX
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        D[i][j] = H[i][0] * Q[j][0] + H[i][1] * Q[j][1] + H[i][2] * Q[j][2];
    const R Jm1 = jm1_of(D);
    // det(dx/dxi) = det A det F
    vol += (1 + Jm1) * detA;
    if (dt_only) continue;
    if (!(Jm1 > R(-1)) || !(detA != 0)) bad = 1;
    const long long sg = gpo - A.gpbase + g;  // Gauss point within the group
    if (MAT == 7 && pass == kPassSurrogateFeatures) {
      write_surrogate_features(D, a0, A.law, A.surr_x + sg * kMlpIn);
      continue;
    }
    const float *sy = (MAT == 7 && A.surr_y) ? A.surr_y + sg * kMlpOut : nullptr;
    Sym6<R> S = stress_at<R, MAT>(mp, D, Jm1, a0, hist + g * gs, hs, pc, sy, A.law);
    if (GP) {
      long long q = gpo + g;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A.gpF[9 * q + i + 3 * j] = double((i == j ? R(1) : R(0)) + D[i][j]);
      A.gpJ[q] = double(1 + Jm1);
      A.gpS[6 * q + 0] = S.xx;
      A.gpS[6 * q + 1] = S.yy;
      A.gpS[6 * q + 2] = S.zz;
      A.gpS[6 * q + 3] = S.yz;
      A.gpS[6 * q + 4] = S.xz;
      A.gpS[6 * q + 5] = S.xy;
    }
    // w detJ B0^T S with w = 1: P = det A F S = det A (S + D S), Gm = P A^{-1}
    const R sxx = detA * S.xx, syy = detA * S.yy, szz = detA * S.zz, syz = detA * S.yz,
            sxz = detA * S.xz, sxy = detA * S.xy;
    const R s[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}};
    R P[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        P[i][j] = s[i][j] + D[i][0] * s[0][j] + D[i][1] * s[1][j] + D[i][2] * s[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      R g0 = P[i][0] * Q[0][0] + P[i][1] * Q[1][0] + P[i][2] * Q[2][0];
      R g1 = P[i][0] * Q[0][1] + P[i][1] * Q[1][1] + P[i][2] * Q[2][1];
      R g2 = P[i][0] * Q[0][2] + P[i][1] * Q[1][2] + P[i][2] * Q[2][2];
      m[0][i] += g0;
      m[1][i] += g1;
      m[2][i] += g2;
      m[3][i] += et * g0 + xi * g1;
      m[4][i] += ze * g0 + xi * g2;
      m[5][i] += ze * g1 + et * g2;
      m[6][i] += ez * g0 + xz * g1 + xe * g2;
    }
  }
  le = vol / amax;
  }
  if (pass == kPassForce) {
    // inverse transform: f_a = 1/8 sum_k sign_k(a) m_k
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const R q = R(0.125);
      R t1 = m[0][i] + m[6][i], t2 = m[0][i] - m[6][i], t3 = m[3][i] + m[4][i],
        t4 = m[3][i] - m[4][i];
      R Pmm = t1 - t3, Ppp = t1 + t3, Ppm = t2 + t4, Pmp = t2 - t4;
      R r1 = m[1][i] + m[2][i], r2 = m[1][i] - m[2][i];
      R Qmm = m[5][i] - r1, Qpp = m[5][i] + r1, Qpm = r2 - m[5][i], Qmp = -r2 - m[5][i];
      f[0][i] = q * (Qmm - Pmm);
      f[1][i] = q * (Qmm + Pmm);
      f[2][i] = q * (Qpm + Ppm);
      f[3][i] = q * (Qpm - Ppm);
      f[4][i] = q * (Qmp - Pmp);
      f[5][i] = q * (Qmp + Pmp);
      f[6][i] = q * (Qpp + Ppp);
      f[7][i] = q * (Qpp - Ppp);
    }
  }
}

// C3D4: one Gauss point at (1/4,1/4,1/4), weight 1/6, |det J|
// (ShapeFunction_C3D4.cpp:59-73, GaussQuadrature3D.cpp:60-69).
template <class R, int MAT, bool GP>
__device__ __forceinline__ void tet_element(const R (&x)[4][3], const R (&u)[4][3],
                                            const MatP<R> &mp, const R (&pc)[4],
                                            const R (&a0)[3], R *hist, long long hs,
                                            int pass, R (&f)[4][3], R &le, int &bad,
                                            const ElemArgs<R> &A, long long gpo, const R *hin) {
  const bool dt_only = pass != kPassForce;
  R Am[3][3], H[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      Am[r][d] = x[r][d] - x[3][d];
      H[d][r] = u[r][d] - u[3][d];
    }
  R Ad[3][3], detA;
  adj3(Am, Ad, detA);
  const R idet = 1 / detA;
  R D[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      D[i][j] = idet * (H[i][0] * Ad[j][0] + H[i][1] * Ad[j][1] + H[i][2] * Ad[j][2]);
  const R Jm1 = jm1_of(D);
  if (!(Jm1 > R(-1)) || !(detA != 0)) bad = 1;
  // (the characteristic length first: the nodal values are dead during the law)
  // min altitude (CalculateCharacteristicLength_C3D4.cpp:5-46): 6V / max |n_face|
  R xc[4][3];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d) xc[a][d] = x[a][d] + u[a][d];
  R six_v = fabs((1 + Jm1) * detA);
  constexpr int fc[4][3] = {{1, 2, 3}, {2, 3, 0}, {3, 0, 1}, {0, 1, 2}};
  R nmax = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int p1 = fc[k][0], p2 = fc[k][1], p3 = fc[k][2];
    R v1x = xc[p2][0] - xc[p1][0], v1y = xc[p2][1] - xc[p1][1], v1z = xc[p2][2] - xc[p1][2];
    R v2x = xc[p3][0] - xc[p1][0], v2y = xc[p3][1] - xc[p1][1], v2z = xc[p3][2] - xc[p1][2];
    R n = norm3(v1y * v2z - v1z * v2y, v1z * v2x - v1x * v2z, v1x * v2y - v1y * v2x);
    nmax = fmax(nmax, n);
  }
  le = six_v / nmax;
  const long long sg = gpo - A.gpbase;  // Gauss point within the group
  if (MAT == 7 && pass == kPassSurrogateFeatures) {
    write_surrogate_features(D, a0, A.law, A.surr_x + sg * kMlpIn);
    return;
  }
  if (!dt_only) {
    const float *sy = (MAT == 7 && A.surr_y) ? A.surr_y + sg * kMlpOut : nullptr;
    Sym6<R> S = stress_at<R, MAT>(mp, D, Jm1, a0, hist, hs, pc, sy, A.law, hin);
    if (GP) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A.gpF[9 * gpo + i + 3 * j] = double((i == j ? R(1) : R(0)) + D[i][j]);
      A.gpJ[gpo] = double(1 + Jm1);
      A.gpS[6 * gpo + 0] = S.xx;
      A.gpS[6 * gpo + 1] = S.yy;
      A.gpS[6 * gpo + 2] = S.zz;
      A.gpS[6 * gpo + 3] = S.yz;
      A.gpS[6 * gpo + 4] = S.xz;
      A.gpS[6 * gpo + 5] = S.xy;
    }
    const R s[3][3] = {{S.xx, S.xy, S.xz}, {S.xy, S.yy, S.yz}, {S.xz, S.yz, S.zz}};
    R P[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        P[i][j] = s[i][j] + D[i][0] * s[0][j] + D[i][1] * s[1][j] + D[i][2] * s[2][j];
    // G = (|det A| / 6) P A^{-1} = sign(det A)/6 * P adj(A)
    const R w = (detA >= 0 ? R(1) : R(-1)) * R(1.0 / 6.0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      R g0 = w * (P[i][0] * Ad[0][0] + P[i][1] * Ad[1][0] + P[i][2] * Ad[2][0]);
      R g1 = w * (P[i][0] * Ad[0][1] + P[i][1] * Ad[1][1] + P[i][2] * Ad[2][1]);
      R g2 = w * (P[i][0] * Ad[0][2] + P[i][1] * Ad[1][2] + P[i][2] * Ad[2][2]);
      f[0][i] = g0;
      f[1][i] = g1;
      f[2][i] = g2;
      f[3][i] = -(g0 + g1 + g2);
    }
  }
}

// Element time step l/c in the element precision R.  FP32: l times the
// FP32 reciprocal wave speed, an FP32 value -- the block minimum is taken in
// FP32 and widened once (exact), so no per-element FP64 work; FP64: l / c as
// CalculateTimeStep.cpp:19.
template <class R>
__device__ __forceinline__ R dt_of(R le, const MatP<R> &mp);
template <>
__device__ __forceinline__ float dt_of<float>(float le, const MatP<float> &mp) {
  return le * mp.inv_ce;
}
template <>
__device__ __forceinline__ double dt_of<double>(double le, const MatP<double> &mp) {
  return le / mp.ce;  // CalculateTimeStep.cpp:19
}

template <class R, int ET>
__device__ __forceinline__ void element_green_strain(const R (&x)[ET == 0 ? 8 : 4][3],
                                                     const R (&u)[ET == 0 ? 8 : 4][3],
                                                     R (&Es)[6]);

// One listed element's injury update (the body of the reference's per-element
// loop, ex5.cpp:1330-1383): principal strains of the averaged Green strain,
// the sticky flags, the principal strain rate against the previous step, and
// the thread's extremes.
template <class R>
__device__ __forceinline__ void injury_element(const ElemArgs<R> &A, int c, const R (&Es)[6],
                                               R dt, R (&v)[4], int (&jj)[4], int (&cc)[4]) {
  R mx, mn, sh;
  principal_strains<R>(Es[0], Es[1], Es[2], Es[3], Es[4], Es[5], mx, mn, sh);
  uint8_t f = A.inj_flags[c];
  if (mx > R(0.15)) f |= kInjMps15;
  if (mx > R(0.30)) f |= kInjMps30;
  const R psr = (mx - A.inj_ps_old[c]) / dt;
  const R psxsr = mx * psr;
  if (psr > R(120)) f |= kInjPsr120;
  if (psxsr > R(28)) f |= kInjPsxsr28;
  A.inj_flags[c] = f;
  A.inj_ps_old[c] = mx;
  A.inj_psxsr[c] = psxsr;
  v[0] = mx;
  v[1] = mn;
  v[2] = sh;
  v[3] = psxsr;
  const int up = A.inj_upos[c];
  jj[0] = jj[1] = jj[2] = jj[3] = up;
  cc[0] = cc[1] = cc[2] = cc[3] = c;
}

// The block's injury extremes into *out: a butterfly per warp, then the warps
// in order by thread 0.  The order (value, then smallest list position) is
// total over listed elements, so the result does not depend on the shape of
// the reduction.  Values are compared in the element precision R (they are R
// values; FP64 compares are slow on this GPU) and widened when written.
// Every thread of the block calls it.
template <int NT, class R>
__device__ __forceinline__ void injury_block_extremes(R (&v)[4], int (&jj)[4], int (&cc)[4],
                                                      InjuryPart *out) {
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R ov = __shfl_xor_sync(0xffffffffu, v[k], o);
      const int oj = __shfl_xor_sync(0xffffffffu, jj[k], o);
      const int oc = __shfl_xor_sync(0xffffffffu, cc[k], o);
      if (inj_better(k, ov, oj, v[k], jj[k])) {
        v[k] = ov;
        jj[k] = oj;
        cc[k] = oc;
      }
    }
  __shared__ R wv[NT / 32][4];
  __shared__ int wj[NT / 32][4], wc[NT / 32][4];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      wv[w][k] = v[k];
      wj[w][k] = jj[k];
      wc[w][k] = cc[k];
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int x = 1; x < (int)(blockDim.x + 31) / 32; ++x)
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (inj_better(k, wv[x][k], wj[x][k], v[k], jj[k])) {
        v[k] = wv[x][k];
        jj[k] = wj[x][k];
        cc[k] = wc[x][k];
      }
  InjuryPart q;
#pragma unroll
  for (int k = 0; k < 4; ++k) {  // no listed element: the reduction's sentinels
    q.v[k] = cc[k] < 0 ? (k == 1 ? 1e300 : -1e300) : double(v[k]);
    q.j[k] = jj[k];
    q.c[k] = cc[k];
  }
  *out = q;
}

template <class R, int ET, int MAT, bool GP, bool INJ>
// C3D8: at most 128 registers per thread (two 256-thread or four 128-thread
// blocks per SM); only the rarely taken eigen-decomposition fallback of the
// Ogden law needs more and spills there.  C3D4 (one Gauss point, latency
// bound): at most 64, for four 256-thread or eight 128-thread blocks per SM
// (head-like mesh: element pass 0.129 ms at 80 registers, 0.118 ms at 64,
// 0.127 ms at 48; the GOH + Prony law spills some of its state at 64).
// INJ: the force pass also updates the brain drivers' per-step injury
// criteria of its listed elements (CalculateInjuryCriterions, ex5.cpp:
// 1311-1430, on the F of this pass) and writes the block's extremes.
__global__ void __launch_bounds__(kElemThreads, ET == 0 ? 2 : 4)
    k_elem(const ElemArgs<R> A, int pass) {
  constexpr int NC = ET == 0 ? 8 : 4;
  constexpr int NGP = ET == 0 ? 8 : 1;
  // one-point elements with a Prony history load it with the other
  // per-element data, before the slot staging
  constexpr int NH = (ET == 1 && (MAT == 5 || MAT == 7)) ? (MAT == 5 ? 18 : 12) : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // staged slots: C3D8 as {x, y, z, pad} records (one vector load per corner),
  // C3D4 as three component arrays (its four scattered corners: 32-bit loads
  // meet fewer bank conflicts; the head's element pass measured 3 % faster)
  constexpr bool PACK = ET == 0;
  Slot4<R> *shX = reinterpret_cast<Slot4<R> *>(smem_raw);
  Slot4<R> *shU = shX + kMaxLocalNodes;
  R *shXs = reinterpret_cast<R *>(smem_raw);
  R *shUs = shXs + 3 * kMaxLocalNodes;
  // [NC*3][blockDim] corner forces; FP32 C3D8: first the elements' reference
  // geometry, [20][blockDim] x 4 values, in the same space (a barrier
  // separates the last geometry read from the first corner-force write)
  R *shF = PACK ? reinterpret_cast<R *>(shU + kMaxLocalNodes) : shUs + 3 * kMaxLocalNodes;
  constexpr bool GEO = ET == 0 && sizeof(R) == 4;
  const int PE = blockDim.x;
  // the local CSR of the in-block assembly: offsets, then entries
  uint16_t *shLp = reinterpret_cast<uint16_t *>(shF + (GEO ? 80 : NC * 3) * PE);
  uint16_t *shLe = shLp + kMaxLocalNodes + 8;
  const int t = threadIdx.x;
  const int p = A.patch_begin + blockIdx.x;
  const int inst = A.patch_inst[p];
  const int e0 = A.patch_elem_off[p], ne = A.patch_elem_off[p + 1] - e0;
  const int s0 = A.patch_node_off[p], ns = A.patch_node_off[p + 1] - s0;
  // per-element loads first: none depends on the staged slots, so their
  // latency overlaps the staging below
  const bool act = t < ne;
  const int e = e0 + (act ? t : 0);
  const long long el = e - A.elem_begin;
  const long long gs = A.nelem, hs = (long long)NGP * A.nelem;
  if (GEO && act) {
    // 20 rows of 16 bytes, coalesced across the block, landing while the
    // per-element loads and the slot staging below are in flight
    const R *src = A.geo + 4 * el;
    R *dst = shF + 4 * t;
#pragma unroll 4
    for (int r = 0; r < 20; ++r) cp_async16(dst + 4 * r * PE, src + 4 * r * gs);
  }
  uint4 cv = make_uint4(0u, 0u, 0u, 0u);
  int pw = 0;
  R a0[3] = {R(1), R(0), R(0)};
  R hin[NH];
#pragma unroll
  for (int k = 0; k < NH; ++k) hin[k] = R(0);
  const int ci = (INJ && act) ? A.inj_cidx[e] : -1;  // listed for the injury criteria
  if (act) {
    if (NC == 8) {
      cv = *reinterpret_cast<const uint4 *>(A.lconn + 8ll * el);
    } else {
      const uint2 v = *reinterpret_cast<const uint2 *>(A.lconn + 4ll * el);
      cv.x = v.x;
      cv.y = v.y;
    }
    pw = A.epid[e];
    if (MAT == 7) {
      a0[0] = A.fib[e];
      a0[1] = A.fib[A.E + e];
      a0[2] = A.fib[2 * A.E + e];
    }
    if (NH > 1 && pass == kPassForce) {
#pragma unroll
      for (int k = 0; k < NH; ++k) hin[k] = A.hist[el + k * hs];
    }
  }
  const Clock *ck = A.clock + A.parity * A.ninst + inst;
  // the slot records go to shared memory by asynchronous copies, in flight
  // together (and with the C3D8 geometry rows) until the one wait below; the
  // padding word of a C3D8 coordinate record is never read
  for (int i = t; i < ns; i += PE) {
    const R *us = A.sU + 4ll * (s0 + i);
    if (PACK) {
#pragma unroll
      for (int h = 0; h < (int)sizeof(Slot4<R>) / 16; ++h)
        cp_async16(reinterpret_cast<char *>(shU + i) + 16 * h, us + h * (16 / sizeof(R)));
      cp_async_small<sizeof(R)>(&shX[i].x, A.sX + s0 + i);
      cp_async_small<sizeof(R)>(&shX[i].y, A.sX + A.S + s0 + i);
      cp_async_small<sizeof(R)>(&shX[i].z, A.sX + 2 * A.S + s0 + i);
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        cp_async_small<sizeof(R)>(shXs + d * kMaxLocalNodes + i, A.sX + d * A.S + s0 + i);
        cp_async_small<sizeof(R)>(shUs + d * kMaxLocalNodes + i, us + d);
      }
    }
  }
  if (ET == 0 && pass == kPassForce) {
    // C3D8: the assembly's local CSR travels with the slots (needed only at
    // the end of the block, but its loads would then be a dependent chain;
    // the latency-bound C3D4 blocks measured faster loading it at the end)
    const int eo = A.patch_ent_off[p], en = A.patch_ent_off[p + 1] - eo;
    if (((eo | en) & 7) == 0) {
      for (int c = t; 8 * c < en; c += PE) cp_async16(shLe + 8 * c, A.lent + eo + 8 * c);
    } else {
      for (int c = t; c < en; c += PE) shLe[c] = A.lent[eo + c];
    }
    for (int i = t; i <= ns; i += PE) shLp[i] = A.lptr[s0 + p + i];
  }
  cp_async_wait_all();  // this thread's slot records (and geometry rows)
  // an instance past its end time: the whole block leaves (uniform per patch)
  if (A.use_clock && ck->done) return;
  const R dt = A.use_clock ? R(ck->dt) : R(A.dt_direct);
  __syncthreads();
  R dte = r_inf<R>();
  int bad = 0;
  // injury extremes of this thread's element: max / min principal strain,
  // max shear, max MPS x rate, with list position and compact index
  R iv[4] = {-r_inf<R>(), r_inf<R>(), -r_inf<R>(), -r_inf<R>()};
  int ij[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff}, ic[4] = {-1, -1, -1, -1};
  R f[NC][3];
  if (act) {
    int lc[NC];
    lc[0] = cv.x & 0xffff; lc[1] = cv.x >> 16; lc[2] = cv.y & 0xffff; lc[3] = cv.y >> 16;
    if (NC == 8) {
      lc[4 % NC] = cv.z & 0xffff; lc[5 % NC] = cv.z >> 16;
      lc[6 % NC] = cv.w & 0xffff; lc[7 % NC] = cv.w >> 16;
    }
    R x[NC][3], u[NC][3];
#pragma unroll
    for (int a = 0; a < NC; ++a) {
      int l = lc[a] < ns ? lc[a] : 0;
      if (lc[a] >= ns) bad |= 2;
      if (PACK) {
        const Slot4<R> xs = shX[l], us = shU[l];
        x[a][0] = xs.x; x[a][1] = xs.y; x[a][2] = xs.z;
        u[a][0] = us.x; u[a][1] = us.y; u[a][2] = us.z;
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          x[a][d] = shXs[d * kMaxLocalNodes + l];
          u[a][d] = shUs[d * kMaxLocalNodes + l];
        }
      }
    }
    R Es[6];  // injury: the element's averaged Green strain (as k_elem_strain)
    if (INJ && ci >= 0) element_green_strain<R, ET>(x, u, Es);
    const bool skip = pw < 0;
    const MatP<R> mp = A.mats[pw & 0x7fffffff];
    R pc[4];
    prony_consts<R, MAT>(mp, dt, pc);
    R *hist = A.hist ? A.hist + el : nullptr;
    R le;
    const long long gpo = A.gpbase + el * NGP;
    if (ET == 0)
      hex_element<R, MAT, GP, GEO>(
          reinterpret_cast<const R(&)[8][3]>(x), reinterpret_cast<const R(&)[8][3]>(u), mp, pc,
          a0, hist, hs, gs, pass, reinterpret_cast<R(&)[8][3]>(f), le, bad, A, gpo, shF + 4 * t,
          4 * PE);
    else
      tet_element<R, MAT, GP>(reinterpret_cast<const R(&)[4][3]>(x),
                              reinterpret_cast<const R(&)[4][3]>(u), mp, pc, a0, hist, hs,
                              pass, reinterpret_cast<R(&)[4][3]>(f), le, bad, A, gpo,
                              NH > 1 ? hin : nullptr);
    if (!GEO && pass == kPassForce) {
#pragma unroll
      for (int a = 0; a < NC; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) shF[(a * 3 + d) * PE + t] = f[a][d];
    }
    if (!skip) dte = dt_of<R>(le, mp);
    if (INJ && ci >= 0) injury_element<R>(A, ci, Es, dt, iv, ij, ic);
  }
  if (GEO && pass == kPassForce) {
    __syncthreads();  // every thread is done with its geometry rows
    if (act) {
#pragma unroll
      for (int a = 0; a < NC; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) shF[(a * 3 + d) * PE + t] = f[a][d];
    }
  }
  if (bad) atomicOr(A.err, (bad & 1 ? kErrInverted : 0) | (bad & 2 ? kErrIndex : 0));
  if (pass == kPassSurrogateFeatures) return;  // features only (uniform per block)
  if (INJ && pass == kPassForce)
    injury_block_extremes<kElemThreads>(iv, ij, ic, reinterpret_cast<InjuryPart *>(A.inj_part) + p);
  // block minimum of the element time steps (in R; widening to FP64 is
  // exact and monotone) -> one FP64 atomicMin per block (positive doubles
  // order like their bit patterns)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dte = fmin(dte, __shfl_xor_sync(0xffffffffu, dte, o));
  __shared__ R wmin[kElemThreads / 32];
  if ((t & 31) == 0) wmin[t >> 5] = dte;
  __syncthreads();
  if (t == 0) {
    R mn = wmin[0];
    for (int w = 1; w < (PE + 31) / 32; ++w) mn = fmin(mn, wmin[w]);
    atomicMin(A.dtmin + A.parity * A.ninst + inst,
              (unsigned long long)__double_as_longlong(double(mn)));
  }
  if (pass != kPassForce) return;
  // in-block assembly: local node i sums its corners in (element, corner) order
  const uint16_t *lp = ET == 0 ? shLp : A.lptr + s0 + p;
  const uint16_t *le = ET == 0 ? shLe : A.lent + A.patch_ent_off[p];
  for (int i = t; i < ns; i += PE) {
    const int b = lp[i], en = lp[i + 1];
    R f0 = 0, f1 = 0, f2 = 0;
    for (int k = b; k < en; ++k) {
      const int ent = le[k];
      const int el = ent / NC, a = ent - el * NC;
      f0 += shF[(a * 3 + 0) * PE + el];
      f1 += shF[(a * 3 + 1) * PE + el];
      f2 += shF[(a * 3 + 2) * PE + el];
    }
    reinterpret_cast<Slot4<R> *>(A.sF)[s0 + i] = Slot4<R>{f0, f1, f2, R(0)};
  }
}

// Setup pass of an FP32 C3D8 group: per Gauss point the inverse Jacobian of
// the reference geometry and its determinant (ShapeFunction_C3D8.cpp:35-120,
// evaluated once as in ShapeFunctions.cpp:197-215), computed in FP64 from the
// slot coordinates.  Per element an 80-value record, value 10 g + k of Gauss
// point g = (Q00 Q01 Q02 Q10 Q11 Q12 Q20 Q21 Q22 det A)[k], stored as 20 rows
// of 4 values: value v at geo[4 (v/4 * nelem + element) + v%4].
template <class R>
__global__ void __launch_bounds__(kElemThreads) k_elem_geo(const ElemArgs<R> A, float *geo) {
  static_assert(sizeof(R) == 4, "the geometry table serves the FP32 element kernels");
  __shared__ double shX[3][kMaxLocalNodes];
  const int p = A.patch_begin + blockIdx.x;
  const int e0 = A.patch_elem_off[p], ne = A.patch_elem_off[p + 1] - e0;
  const int s0 = A.patch_node_off[p], ns = A.patch_node_off[p + 1] - s0;
  for (int i = threadIdx.x; i < ns && i < kMaxLocalNodes; i += blockDim.x)
#pragma unroll
    for (int d = 0; d < 3; ++d) shX[d][i] = double(A.sX[d * A.S + s0 + i]);
  __syncthreads();
  const long long gs = A.nelem;
  int bad = 0;
  for (int t = threadIdx.x; t < ne; t += blockDim.x) {
    const long long el = e0 + t - A.elem_begin;
    double x[8][3];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      int l = A.lconn[8 * el + a];
      if (l >= ns || l >= kMaxLocalNodes) {
        bad |= kErrIndex;
        l = 0;
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) x[a][d] = shX[d][l];
    }
    double hx[7][3];
    hex_hadamard(x, hx);
    for (int g = 0; g < 8; ++g) {
      double xi, et, ze;
      hex_gauss_point(g, xi, et, ze);
      const double ez = et * ze, xz = xi * ze, xe = xi * et;
      double Am[3][3], Ad[3][3], det;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Am[0][d] = hx[0][d] + et * hx[3][d] + ze * hx[4][d] + ez * hx[6][d];
        Am[1][d] = hx[1][d] + xi * hx[3][d] + ze * hx[5][d] + xz * hx[6][d];
        Am[2][d] = hx[2][d] + xi * hx[4][d] + et * hx[5][d] + xe * hx[6][d];
      }
      adj3(Am, Ad, det);
      const double id = 1.0 / det;  // det = 0: non-finite entries, flagged by the force pass
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        const int v = 10 * g + k;
        const double q = k < 9 ? Ad[k / 3][k % 3] * id : det;
        geo[4 * ((v >> 2) * gs + el) + (v & 3)] = float(q);
      }
    }
  }
  if (bad) atomicOr(A.err, bad);
}

// Gauss-point average of the Green strain of one element (see k_elem_strain)
template <class R, int ET>
__device__ __forceinline__ void element_green_strain(const R (&x)[ET == 0 ? 8 : 4][3],
                                                     const R (&u)[ET == 0 ? 8 : 4][3],
                                                     R (&Es)[6]) {
#pragma unroll
  for (int k = 0; k < 6; ++k) Es[k] = R(0);
  if (ET == 0) {
    R hx[7][3], hu[7][3];
    hex_hadamard(reinterpret_cast<const R(&)[8][3]>(x), hx);
    hex_hadamard(reinterpret_cast<const R(&)[8][3]>(u), hu);
    const R G = R(0.577350269189626);
#pragma unroll 1
    for (int g = 0; g < 8; ++g) {  // Gauss points as in hex_element
      const R xi = ((g + 1) & 2) ? G : -G, et = (g & 2) ? G : -G, ze = g < 4 ? G : -G;
      const R ez = et * ze, xz = xi * ze, xe = xi * et;
      R Am[3][3], H[3][3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Am[0][d] = hx[0][d] + et * hx[3][d] + ze * hx[4][d] + ez * hx[6][d];
        Am[1][d] = hx[1][d] + xi * hx[3][d] + ze * hx[5][d] + xz * hx[6][d];
        Am[2][d] = hx[2][d] + xi * hx[4][d] + et * hx[5][d] + xe * hx[6][d];
        H[d][0] = hu[0][d] + et * hu[3][d] + ze * hu[4][d] + ez * hu[6][d];
        H[d][1] = hu[1][d] + xi * hu[3][d] + ze * hu[5][d] + xz * hu[6][d];
        H[d][2] = hu[2][d] + xi * hu[4][d] + et * hu[5][d] + xe * hu[6][d];
      }
      R Ad[3][3], detA;
      adj3(Am, Ad, detA);
      const R idet = 1 / detA;
      R D[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          D[i][j] = idet * (H[i][0] * Ad[j][0] + H[i][1] * Ad[j][1] + H[i][2] * Ad[j][2]);
      R E[6];
      green_strain(D, E);
#pragma unroll
      for (int k = 0; k < 6; ++k) Es[k] += E[k];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) Es[k] *= R(0.125);
  } else {
    R Am[3][3], H[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Am[r][d] = x[r][d] - x[3][d];
        H[d][r] = u[r][d] - u[3][d];
      }
    R Ad[3][3], detA;
    adj3(Am, Ad, detA);
    const R idet = 1 / detA;
    R D[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        D[i][j] = idet * (H[i][0] * Ad[j][0] + H[i][1] * Ad[j][1] + H[i][2] * Ad[j][2]);
    green_strain(D, Es);
  }
}

// Gauss-point average of the Green-Lagrange strain of every element of a group
// (CalculateStrain.cpp:8-33) on the current displacement slots, from the
// displacement gradient D = F - I of each Gauss point:
//   E = (1 / nGP) sum_gp (D + D^T + D^T D) / 2,
// the same quantity as the reference's sum (0.5 / nGP) F^T F - 0.5 I without
// the cancellation of F^T F - I.  Output per element (group order, FP64):
// Voigt xx, yy, zz, yz, xz, xy.
template <class R, int ET>
__global__ void __launch_bounds__(kElemThreads) k_elem_strain(const ElemArgs<R> A, double *Eout) {
  constexpr int NC = ET == 0 ? 8 : 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // staged slots as {x, y, z, pad} records: one vector load per corner
  Slot4<R> *shX = reinterpret_cast<Slot4<R> *>(smem_raw);
  Slot4<R> *shU = shX + kMaxLocalNodes;
  const int PE = blockDim.x;
  const int t = threadIdx.x;
  const int p = A.patch_begin + blockIdx.x;
  const int e0 = A.patch_elem_off[p], ne = A.patch_elem_off[p + 1] - e0;
  const int s0 = A.patch_node_off[p], ns = A.patch_node_off[p + 1] - s0;
  for (int i = t; i < ns; i += PE) {
    shU[i] = reinterpret_cast<const Slot4<R> *>(A.sU)[s0 + i];
    shX[i] = Slot4<R>{A.sX[s0 + i], A.sX[A.S + s0 + i], A.sX[2 * A.S + s0 + i], R(0)};
  }
  __syncthreads();
  if (t >= ne) return;
  const int e = e0 + t;
  const long long el = e - A.elem_begin;
  int lc[NC];
  if (NC == 8) {
    const uint4 v = *reinterpret_cast<const uint4 *>(A.lconn + 8ll * el);
    lc[0] = v.x & 0xffff; lc[1] = v.x >> 16; lc[2] = v.y & 0xffff; lc[3] = v.y >> 16;
    lc[4 % NC] = v.z & 0xffff; lc[5 % NC] = v.z >> 16; lc[6 % NC] = v.w & 0xffff; lc[7 % NC] = v.w >> 16;
  } else {
    const uint2 v = *reinterpret_cast<const uint2 *>(A.lconn + 4ll * el);
    lc[0] = v.x & 0xffff; lc[1] = v.x >> 16; lc[2] = v.y & 0xffff; lc[3] = v.y >> 16;
  }
  R x[NC][3], u[NC][3];
#pragma unroll
  for (int a = 0; a < NC; ++a) {
    const int l = lc[a] < ns ? lc[a] : 0;
    const Slot4<R> xs = shX[l], us = shU[l];
    x[a][0] = xs.x; x[a][1] = xs.y; x[a][2] = xs.z;
    u[a][0] = us.x; u[a][1] = us.y; u[a][2] = us.z;
  }
  R Es[6];
  element_green_strain<R, ET>(x, u, Es);
#pragma unroll
  for (int k = 0; k < 6; ++k) Eout[6 * (long long)e + k] = double(Es[k]);
}

template <class R>
size_t elem_smem_bytes(int ET, int PE) {
  const int NC = ET == 0 ? 8 : 4;
  return sizeof(R) * (6 * (size_t)kMaxLocalNodes + (size_t)NC * 3 * PE);
}

}  // namespace ftgpu
