// ft_mlp.cuh -- the learned constitutive surrogate: shapes, parameter layout and
// the input features / output reconstruction shared by training and in-loop use.
//
// What is learned: the isochoric (deviatoric-response) PK2 stress S_iso(E, a0)
// of the anisotropic GOH law (material 7), i.e. the costly nonlinear part of
// the stress update (exponential fibre term, J^{-2/3}, adjugate products).  The
// volumetric stress and the 1-term Prony recurrence are linear in S_iso and
// stay exact.  The network predicts a residual over a first-order model of the
// law, scaled by |E|^2 (the residual is O(|E|^2)):
//   S_iso = S_lin(E, a0) + s0 out_scale |E|^2 NN(x),  s0 = mu + k1,
//   S_lin = 2 mu dev E + 2 k1 (1-3 kappa) max(Ebar, 0) dev(a0 a0),
//   Ebar  = kappa (I1bar - 3) + (1-3 kappa) (I4bar - 1)   (exact fibre strain),
// so small strains are carried by the exact linear part, and the fibre switch
// (Ebar > 0) is the law's own, which keeps the residual continuous.
// Inputs x: the strain direction E/|E|_F (Voigt 11,22,33,23,13,12, tensor
// shears; |E|_F^2 counts shears twice), |E|_F / 0.2, the fibre a0 and
// Ebar / |E|_F.  Network: 16 (11 used) -> 128 -> 128 -> 128 -> 8 (6 used),
// SiLU, BF16 weights and activations, FP32 accumulation.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ft_materials.cuh"

namespace ftgpu {

constexpr int kMlpIn = 16, kMlpHid = 128, kMlpOut = 8;
constexpr int kMlpUsedIn = 11, kMlpUsedOut = 6;
// flat FP32 parameter vector: W0[128][16] b0 W1[128][128] b1 W2[128][128] b2 W3[8][128] b3
constexpr int kOffW0 = 0;
constexpr int kOffB0 = kOffW0 + kMlpHid * kMlpIn;
constexpr int kOffW1 = kOffB0 + kMlpHid;
constexpr int kOffB1 = kOffW1 + kMlpHid * kMlpHid;
constexpr int kOffW2 = kOffB1 + kMlpHid;
constexpr int kOffB2 = kOffW2 + kMlpHid * kMlpHid;
constexpr int kOffW3 = kOffB2 + kMlpHid;
constexpr int kOffB3 = kOffW3 + kMlpOut * kMlpHid;
constexpr int kMlpParams = kOffB3 + kMlpOut;
constexpr double kStrainScale = 0.2;
constexpr double kE2Floor = 1e-14;

struct SurrogateLaw {  // the GOH parameters the surrogate was trained for
  double mu, k1, k2, kappa;
  double s0;           // output scale mu + k1
  double out_scale;    // extra normalisation of the residual (training std)
  double trust_e2;     // |E|_F^2 above which the plain law is used
};

// Exact GOH fibre strain Ebar for Green strain E (Voigt, tensor shears) and a
// unit fibre a0, without cancellation: with X = 2E, J^2 - 1 = det(I + X) - 1 =
// tr X + I2(X) + det X, jm = J^{-2/3} - 1 = expm1(-log1p(J^2 - 1) / 3),
// I1bar - 3 = jm (3 + tr X) + tr X, I4bar - 1 = jm (1 + a.X.a) + a.X.a.
template <class R>
__device__ __forceinline__ R goh_fibre_strain(const R (&E)[6], const R (&a0)[3], R kappa) {
  const R x0 = 2 * E[0], x1 = 2 * E[1], x2 = 2 * E[2], x3 = 2 * E[3], x4 = 2 * E[4], x5 = 2 * E[5];
  const R tr = x0 + x1 + x2;
  const R i2 = (x0 * x1 - x5 * x5) + (x0 * x2 - x4 * x4) + (x1 * x2 - x3 * x3);
  const R i3 = x0 * (x1 * x2 - x3 * x3) - x5 * (x5 * x2 - x3 * x4) + x4 * (x5 * x3 - x1 * x4);
  const R jm = d_expm1(R(-1.0 / 3.0) * d_log1p(tr + i2 + i3));
  const R aXa = a0[0] * a0[0] * x0 + a0[1] * a0[1] * x1 + a0[2] * a0[2] * x2 +
                R(2) * (a0[1] * a0[2] * x3 + a0[0] * a0[2] * x4 + a0[0] * a0[1] * x5);
  const R i1m3 = jm * (R(3) + tr) + tr;
  const R i4m1 = jm * (R(1) + aXa) + aXa;
  return kappa * i1m3 + (R(1) - R(3) * kappa) * i4m1;
}

// features and linear part from the Green strain (symmetric, Voigt order) and a0
template <class R>
__device__ inline void surrogate_features(const R (&E)[6], const R (&a0)[3],
                                          const SurrogateLaw &law, float (&x)[kMlpUsedIn],
                                          R (&Slin)[6], R &scale) {
  const R tr3 = (E[0] + E[1] + E[2]) / R(3);
  const R c4 = R(1) - R(3) * R(law.kappa);
  const R Eb = goh_fibre_strain(E, a0, R(law.kappa));
  const R f = Eb > R(0) ? R(2) * R(law.k1) * c4 * Eb : R(0);
  const R mu2 = R(2) * R(law.mu);
  const R third = R(1) / R(3);
  Slin[0] = mu2 * (E[0] - tr3) + f * (a0[0] * a0[0] - third);
  Slin[1] = mu2 * (E[1] - tr3) + f * (a0[1] * a0[1] - third);
  Slin[2] = mu2 * (E[2] - tr3) + f * (a0[2] * a0[2] - third);
  Slin[3] = mu2 * E[3] + f * a0[1] * a0[2];
  Slin[4] = mu2 * E[4] + f * a0[0] * a0[2];
  Slin[5] = mu2 * E[5] + f * a0[0] * a0[1];
  R e2 = E[0] * E[0] + E[1] * E[1] + E[2] * E[2] + R(2) * (E[3] * E[3] + E[4] * E[4] + E[5] * E[5]);
  if (e2 < R(kE2Floor)) e2 = R(kE2Floor);
  scale = R(law.s0) * R(law.out_scale) * e2;
  const R en = d_sqrt(e2), inv = R(1) / en;
  for (int k = 0; k < 6; ++k) x[k] = float(E[k] * inv);
  x[6] = float(en / R(kStrainScale));
  x[7] = float(a0[0]);
  x[8] = float(a0[1]);
  x[9] = float(a0[2]);
  x[10] = float(Eb * inv);
}

}  // namespace ftgpu

struct ftgpu_surrogate;
namespace ftgpu {
// host side, implemented in ft_mlp.cu: fused tensor-core inference of n
// feature rows (BF16 bits [n][16]) into outputs [n][8] on stream st (a device
// wait that gives up or-s kErrWait into *err); the trained law
int surrogate_infer(ftgpu_surrogate *s, const uint16_t *X, long long n, float *Y,
                    cudaStream_t st, int *err);
SurrogateLaw surrogate_law(const ftgpu_surrogate *s);
int surrogate_device(const ftgpu_surrogate *s);
}  // namespace ftgpu
