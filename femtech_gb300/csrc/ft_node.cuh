// ft_node.cuh -- nodal kernels: deterministic force gather fused with the
// central-difference update, boundary conditions and the clock advance.
//
// Reference path replaced, per step (examples/ex9/ex9.cpp:107-175):
//   f_net = fe - fi (GetForce_3D.cpp:49-51), a = f_net / m for free DOFs
//   (CalculateAcclerations.cpp:7-11), v = v_half + (t_{n+1} - t_half) a,
//   then -- once the stable dt of the new geometry is known -- the next
//   step's v_half = v + (t_half' - t_{n+1}) a, u += dt v_half and the driver's
//   ApplyBoundaryConditions at the new time, and Time/dt bookkeeping.
// Nodal state is FP64 SoA [3][N]; the per-slot partial forces are summed in
// slot order, so the result does not depend on scheduling.
#pragma once

#include "ft_common.h"

namespace ftgpu {

__device__ __forceinline__ void rot_angle(const double *p, double t, double &th, double &om) {
  const double a0 = p[6], T = p[7], pi = 3.14159265358979323846;
  if (t <= T) {
    om = a0 * T / pi * (1.0 - cos(pi * t / T));
    th = a0 * T / pi * (t - T / pi * sin(pi * t / T));
  } else {
    const double wT = 2.0 * a0 * T / pi, thT = a0 * T * T / pi;
    om = wT;
    th = thT + wT * (t - T);
  }
}

// cos / sin of the rotation angle and the angular velocity of a rigid-rotation
// function at time t (the only transcendental work of the rotation).
__device__ __forceinline__ void rot_trig(const BcFn &b, double t, double &c, double &s,
                                         double &om) {
  double th;
  rot_angle(b.p, t, th, om);
  c = cos(th);
  s = sin(th);
}

// Displacement and velocity of node n under a rigid rotation (Rodrigues).
__device__ __forceinline__ void rot_apply(const BcFn &b, double c, double s, double om,
                                          const double *X, long long N, long long n,
                                          double (&ur)[3], double (&vr)[3]) {
  const double k0 = b.p[0], k1 = b.p[1], k2 = b.p[2];
  const double r0 = X[n] - b.p[3], r1 = X[N + n] - b.p[4], r2 = X[2 * N + n] - b.p[5];
  const double kr = k0 * r0 + k1 * r1 + k2 * r2;
  const double R0 = r0 * c + (k1 * r2 - k2 * r1) * s + k0 * kr * (1.0 - c);
  const double R1 = r1 * c + (k2 * r0 - k0 * r2) * s + k1 * kr * (1.0 - c);
  const double R2 = r2 * c + (k0 * r1 - k1 * r0) * s + k2 * kr * (1.0 - c);
  ur[0] = R0 - r0;
  ur[1] = R1 - r1;
  ur[2] = R2 - r2;
  vr[0] = om * (k1 * R2 - k2 * R1);
  vr[1] = om * (k2 * R0 - k0 * R2);
  vr[2] = om * (k0 * R1 - k1 * R0);
}

// Prescribed displacement / velocity of DOF d of node n at time t.  Only the
// rigid rotation reads the node's reference position (SoA X, stride N).
__device__ __forceinline__ void bc_value(const BcFn &b, int d, double t, const double *X,
                                         long long N, long long n, double &u, double &v) {
  switch (b.kind) {
    case kBckFixed: u = b.p[0]; v = 0.0; break;
    case kBckRamp: u = t * b.p[0]; v = b.p[0]; break;
    case kBckSine: u = b.p[0] * sin(b.p[1] * t); v = b.p[0] * b.p[1] * cos(b.p[1] * t); break;
    default: {  // rigid rotation about a fixed axis
      double th, om;
      rot_angle(b.p, t, th, om);
      const double k0 = b.p[0], k1 = b.p[1], k2 = b.p[2];
      const double r0 = X[n] - b.p[3], r1 = X[N + n] - b.p[4], r2 = X[2 * N + n] - b.p[5];
      const double c = cos(th), s = sin(th), kr = k0 * r0 + k1 * r1 + k2 * r2;
      const double R0 = r0 * c + (k1 * r2 - k2 * r1) * s + k0 * kr * (1.0 - c);
      const double R1 = r1 * c + (k2 * r0 - k0 * r2) * s + k1 * kr * (1.0 - c);
      const double R2 = r2 * c + (k0 * r1 - k1 * r0) * s + k2 * kr * (1.0 - c);
      const double w0 = om * (k1 * R2 - k2 * R1), w1 = om * (k2 * R0 - k0 * R2),
                   w2 = om * (k0 * R1 - k1 * R0);
      u = d == 0 ? R0 - r0 : (d == 1 ? R1 - r1 : R2 - r2);
      v = d == 0 ? w0 : (d == 1 ? w1 : w2);
    }
  }
}

// ---- rigid body driven by sampled accelerations (ex5.cpp:339-392) ----

// interpolateLinear (src/math/math.cpp:99-119) of the table (x, y) of n
// points: 0 below the table, the last value above it, y[0] at x[0], else the
// segment of the first x[i] >= value (i >= 1), evaluated with the segment
// slopes g precomputed on the host (the reference divides per lookup; the
// results differ in the last bit).  The search starts at i = cur + 1: every
// x[1..cur] lies below every value looked up from now on (times only grow),
// so the segment is the reference's.  seg = the segment found, -1 for the
// three end cases.
__device__ __forceinline__ double rb_interp(const double *x, const double *y, const double *g,
                                            int n, int cur, double value, int &seg) {
  seg = -1;
  if (value < x[0]) return 0.0;
  if (value > x[n - 1]) return y[n - 1];
  if (value == x[0]) return y[0];
  int i = cur + 1 < 1 ? 1 : cur + 1;
  while (i < n - 1 && !(value <= x[i])) ++i;
  seg = i - 1;
  return fma(g[seg], value - x[seg], y[seg]);
}

// |r| cot|r| = 1 - s P(s) and (1 - |r| cot|r|) / |r|^2 = P(s), s = |r|^2, from
// the Maclaurin series x cot x = 1 - sum_{n>=1} 2^{2n} |B_{2n}| x^{2n} / (2n)!
// (B: Bernoulli numbers), twelve terms: for s < 1/4 the first omitted term is
// below 1e-19.  Estrin's scheme (four dependent steps instead of Horner's
// eleven: the step is a latency-bound FP64 chain), no division.
__device__ __forceinline__ double xcotx_p(double s) {
  const double s2 = s * s, s4 = s2 * s2, s8 = s4 * s4;
  const double p0 = fma(1.0 / 45.0, s, 1.0 / 3.0);
  const double p1 = fma(1.0 / 4725.0, s, 2.0 / 945.0);
  const double p2 = fma(1382.0 / 638512875.0, s, 2.0 / 93555.0);
  const double p3 = fma(3617.0 / 162820783125.0, s, 4.0 / 18243225.0);
  const double p4 = fma(349222.0 / 1531329465290625.0, s, 87734.0 / 38979295480125.0);
  const double p5 = fma(472728182.0 / 201919571963756521875.0, s, 310732.0 / 13447856940643125.0);
  const double q0 = fma(p1, s2, p0), q1 = fma(p3, s2, p2), q2 = fma(p5, s2, p4);
  return fma(q2, s8, fma(q1, s4, q0));
}

// Rate of the rotation generator (ex5.cpp:1001-1018; M. Boyle, "The
// integration of angular velocity", 2017): component c of
// (omega x r + |r| cot|r| omega + (1 - |r| cot|r|) (rhat . omega) rhat) / 2,
// omega / 2 for |r| < 1e-10.  Every lane evaluates the same branch.
__device__ __forceinline__ double rb_rdot(int c, double w0, double w1, double w2, double r0,
                                          double r1, double r2) {
  const double wc = c == 0 ? w0 : (c == 1 ? w1 : w2);
  const double s = r0 * r0 + r1 * r1 + r2 * r2;
  if (s < 1e-20) return 0.5 * wc;
  double rc, g;
  if (s < 0.25) {
    g = xcotx_p(s);
    rc = fma(-s, g, 1.0);
  } else {
    const double rm = sqrt(s);
    rc = rm / tan(rm);
    g = (1.0 - rc) / s;
  }
  const double cr = c == 0 ? w1 * r2 - w2 * r1 : (c == 1 ? -w0 * r2 + w2 * r0 : w0 * r1 - w1 * r0);
  const double rcmp = c == 0 ? r0 : (c == 1 ? r1 : r2);
  const double rw = r0 * w0 + r1 * w1 + r2 * w2;
  return 0.5 * (cr + rc * wc + g * rw * rcmp);
}

// Component j (lane j < 12) of computeDerivatives (ex5.cpp:976-1020) at the
// stage state held one component per lane, with the accelerations al[3],
// ac[3] sampled at the stage time.  All 32 lanes take part in the shuffles.
__device__ __forceinline__ double rb_deriv_lane(int j, double xj, const double *acc) {
  const unsigned full = 0xffffffffu;
  const double w0 = __shfl_sync(full, xj, 0), w1 = __shfl_sync(full, xj, 1),
               w2 = __shfl_sync(full, xj, 2), r0 = __shfl_sync(full, xj, 3),
               r1 = __shfl_sync(full, xj, 4), r2 = __shfl_sync(full, xj, 5);
  const double vel = __shfl_sync(full, xj, j >= 9 && j < 12 ? j - 3 : 0);
  if (j < 3) return acc[j];
  if (j < 6) return rb_rdot(j - 3, w0, w1, w2, r0, r1, r2);
  if (j < 9) return acc[j - 3];
  return vel;
}

// One integrator step of instance i's rigid body from t over h, by one warp:
// the explicit Runge-Kutta pair of Dormand and Prince (J. Comput. Appl. Math.
// 6 (1980) 19-26), fifth-order solution, first stage from the stored
// derivative and the derivative at t + h stored for the next step -- what
// boost::numeric::odeint::runge_kutta_dopri5::do_step(sys, y, yd, t, h) does
// at ex5.cpp:344.  FP64 issue is slow on this GPU and one instance's step is
// a chain of dependent operations, so it is spread over the warp: lanes 0-29
// look up the six channels at the five new stage times (the accelerations
// depend on time only), then lane j < 12 carries state component j through
// the stages, and lanes 0-11 write the node maps of the new state
// (ex5.cpp:345-371 as matrices).
__device__ void rigid_advance(const NodeArgs &A, int i, double t, double h,
                              double (*sacc)[6]) {
  const RigidBody &rb = A.rb[i];
  if (!rb.on) return;
  RigidState *st = A.rbstate + i;
  const int lane = threadIdx.x & 31;
  {
    const int k = lane / 5, s = lane - 5 * (lane / 5);
    int seg = -1;
    if (lane < 30) {
      const double cs = s == 0 ? 1.0 / 5 : (s == 1 ? 3.0 / 10 : (s == 2 ? 4.0 / 5 : 8.0 / 9));
      const double tv = s == 4 ? t + h : t + h * cs;
      const int n = rb.cnt[k];
      const double *x = A.rbtab + rb.off[k];
      sacc[s][k] = rb_interp(x, x + n, x + 2 * n, n, st->cur[k], tv, seg);
    }
    __syncwarp();
    if (lane < 30 && s == 0 && seg >= 0) st->cur[k] = seg;  // stage 2: the earliest time
    __syncwarp();
  }
  constexpr double a21 = 1.0 / 5, a31 = 3.0 / 40, a32 = 9.0 / 40, a41 = 44.0 / 45,
                   a42 = -56.0 / 15, a43 = 32.0 / 9, a51 = 19372.0 / 6561,
                   a52 = -25360.0 / 2187, a53 = 64448.0 / 6561, a54 = -212.0 / 729,
                   a61 = 9017.0 / 3168, a62 = -355.0 / 33, a63 = 46732.0 / 5247,
                   a64 = 49.0 / 176, a65 = -5103.0 / 18656;
  constexpr double b1 = 35.0 / 384, b3 = 500.0 / 1113, b4 = 125.0 / 192,
                   b5 = -2187.0 / 6784, b6 = 11.0 / 84;
  const int j = lane < 12 ? lane : 0;
  const double y = st->y[j], k1 = st->yd[j];
  double x = y + (h * a21) * k1;
  const double k2 = rb_deriv_lane(j, x, sacc[0]);
  x = y + (h * a31) * k1 + (h * a32) * k2;
  const double k3 = rb_deriv_lane(j, x, sacc[1]);
  x = y + (h * a41) * k1 + (h * a42) * k2 + (h * a43) * k3;
  const double k4 = rb_deriv_lane(j, x, sacc[2]);
  x = y + (h * a51) * k1 + (h * a52) * k2 + (h * a53) * k3 + (h * a54) * k4;
  const double k5 = rb_deriv_lane(j, x, sacc[3]);
  x = y + (h * a61) * k1 + (h * a62) * k2 + (h * a63) * k3 + (h * a64) * k4 + (h * a65) * k5;
  const double k6 = rb_deriv_lane(j, x, sacc[4]);
  const double yn = y + (h * b1) * k1 + (h * b3) * k3 + (h * b4) * k4 + (h * b5) * k5 +
                    (h * b6) * k6;
  const double ydn = rb_deriv_lane(j, yn, sacc[4]);
  if (lane < 12) {
    st->y[j] = yn;
    st->yd[j] = ydn;
  }
  // the new state on every lane
  const unsigned full = 0xffffffffu;
  double Y[12], L[3];
#pragma unroll
  for (int c = 0; c < 12; ++c) Y[c] = __shfl_sync(full, yn, c);
#pragma unroll
  for (int c = 0; c < 3; ++c) L[c] = __shfl_sync(full, ydn, c);
  const double acm = __shfl_sync(full, ydn, lane >= 9 && lane < 12 ? lane - 3 : 6);
  // R = exp([0, r]) (quaternionExp, math.cpp:122-133): cos|r| and sin|r| / |r|
  // by their Maclaurin series for |r| < 1/2 (nine terms each, the first
  // omitted one below 1e-18), the library functions beyond; V -> R V R^-1 as
  // the matrix of q / |q| (|q|^2 = 1 to rounding, so 1 / |q|^2 = 2 - |q|^2)
  const double s = Y[3] * Y[3] + Y[4] * Y[4] + Y[5] * Y[5];
  double qw = 1.0, d2 = 1.0;
  if (s != 0.0) {
    if (s < 0.25) {
      double cw = 1.0 / 20922789888000.0, sw = 1.0 / 355687428096000.0;
      cw = fma(cw, -s, 1.0 / 87178291200.0);
      sw = fma(sw, -s, 1.0 / 1307674368000.0);
      cw = fma(cw, -s, 1.0 / 479001600.0);
      sw = fma(sw, -s, 1.0 / 6227020800.0);
      cw = fma(cw, -s, 1.0 / 3628800.0);
      sw = fma(sw, -s, 1.0 / 39916800.0);
      cw = fma(cw, -s, 1.0 / 40320.0);
      sw = fma(sw, -s, 1.0 / 362880.0);
      cw = fma(cw, -s, 1.0 / 720.0);
      sw = fma(sw, -s, 1.0 / 5040.0);
      cw = fma(cw, -s, 1.0 / 24.0);
      sw = fma(sw, -s, 1.0 / 120.0);
      cw = fma(cw, -s, 1.0 / 2.0);
      sw = fma(sw, -s, 1.0 / 6.0);
      qw = fma(cw, -s, 1.0);
      d2 = fma(sw, -s, 1.0);
    } else {
      const double vm = sqrt(s);
      double sn;
      sincos(vm, &sn, &qw);
      d2 = sn / vm;
    }
  }
  const double qx = d2 * Y[3], qy = d2 * Y[4], qz = d2 * Y[5];
  const double nq = qw * qw + qx * qx + qy * qy + qz * qz;
  const double s2 = 2.0 * (2.0 - nq);
  double M[9], R[9];
  M[0] = -s2 * (qy * qy + qz * qz);
  M[1] = s2 * (qx * qy - qw * qz);
  M[2] = s2 * (qx * qz + qw * qy);
  M[3] = s2 * (qx * qy + qw * qz);
  M[4] = -s2 * (qx * qx + qz * qz);
  M[5] = s2 * (qy * qz - qw * qx);
  M[6] = s2 * (qx * qz - qw * qy);
  M[7] = s2 * (qy * qz + qw * qx);
  M[8] = -s2 * (qx * qx + qy * qy);
#pragma unroll
  for (int c = 0; c < 9; ++c) R[c] = M[c] + ((c & 3) == 0 ? 1.0 : 0.0);
  RigidStep *S = A.rbstep + i;
  const double w0 = Y[0], w1 = Y[1], w2 = Y[2];
  if (lane < 9) {  // entry (r, c) of Mm, [omega]x R and ([omega]x^2 + [alpha]x) R
    const int r = lane / 3, c = lane - 3 * (lane / 3);
    const double W[9] = {0.0, -w2, w1, w2, 0.0, -w0, -w1, w0, 0.0};
    const double Al[9] = {0.0, -L[2], L[1], L[2], 0.0, -L[0], -L[1], L[0], 0.0};
    double WW[3];  // row r of [omega]x^2 + [alpha]x
#pragma unroll
    for (int k = 0; k < 3; ++k)
      WW[k] = W[3 * r] * W[k] + W[3 * r + 1] * W[3 + k] + W[3 * r + 2] * W[6 + k] + Al[3 * r + k];
    S->Mm[lane] = M[lane];
    S->WM[lane] = W[3 * r] * R[c] + W[3 * r + 1] * R[3 + c] + W[3 * r + 2] * R[6 + c];
    S->AM[lane] = WW[0] * R[c] + WW[1] * R[3 + c] + WW[2] * R[6 + c];
  } else if (lane < 12) {  // component c of x_cm, v_cm and 2 omega x v_cm + a_cm
    const int c = lane - 9;
    const double v0 = Y[6], v1 = Y[7], v2 = Y[8];
    const double ov = c == 0 ? w1 * v2 - w2 * v1 : (c == 1 ? -w0 * v2 + w2 * v0 : w0 * v1 - w1 * v0);
    S->disp[c] = Y[9 + c];
    S->vel[c] = Y[6 + c];
    S->ca[c] = 2.0 * ov + acm;
  }
}

// Displacement, velocity and acceleration of node n under its instance's
// rigid-body motion (ex5.cpp:361-370 through the maps of RigidStep).
__device__ __forceinline__ void rigid_node(const RigidStep *S, const double *X, long long N,
                                           long long n, double (&u)[3], double (&v)[3],
                                           double (&a)[3]) {
  const double x0 = X[n] - S->c[0], x1 = X[N + n] - S->c[1], x2 = X[2 * N + n] - S->c[2];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    u[r] = S->Mm[3 * r] * x0 + S->Mm[3 * r + 1] * x1 + S->Mm[3 * r + 2] * x2 + S->disp[r];
    v[r] = S->WM[3 * r] * x0 + S->WM[3 * r + 1] * x1 + S->WM[3 * r + 2] * x2 + S->vel[r];
    a[r] = S->AM[3 * r] * x0 + S->AM[3 * r + 1] * x1 + S->AM[3 * r + 2] * x2 + S->ca[r];
  }
}

// Time bookkeeping of one step, as the driver does it on the host
// (ex9.cpp:107-113,172): t_{n+1} = t_n + dt, t_half = (t_{n+1} + t_n) / 2, the
// next dt = ExplicitTimeStepReduction * StableTimeStep(), and the stop tests.
__device__ __forceinline__ StepScalars step_scalars(const Clock &ck, const InstParams &ip,
                                                    unsigned long long dtbits, int mode) {
  StepScalars s;
  const double t_n = ck.time, dt = ck.dt;
  s.t_np1 = t_n + dt;
  const double t_half = 0.5 * (s.t_np1 + t_n);
  const double raw = __longlong_as_double((long long)dtbits);
  s.ndt = ip.reduction * raw;
  int done = 0;
  if (!(s.t_np1 < ip.tmax)) done |= 1;
  if (ck.step + 1 >= ip.step_limit) done |= 2;
  if (raw < ip.failure_dt) done |= 4;
  s.done = done;
  s.advance = (mode == kNodeFused) && !done;
  s.t_np2 = s.t_np1 + s.ndt;
  const double t_half2 = 0.5 * (s.t_np2 + s.t_np1);
  s.c1 = s.t_np1 - t_half;
  s.c2 = t_half2 - s.t_np1;
  s.c12 = t_half2 - t_half;
  s.c1f = float(s.c1);
  s.c12f = float(s.c12);
  return s;
}

// FP32 <-> FP64 conversions of the mixed nodal update by integer bit
// arithmetic.  This GPU converts between FP32 and FP64 on its FP64 pipe (two
// lanes per SM and cycle); a handful of integer operations give the same
// bits for every normal number, and the rare others (zero, subnormal,
// overflow, inf, NaN) take the hardware conversion.
// float -> double: exact (rebias the exponent by 1023 - 127 = 896, widen the
// mantissa).
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned ex = b & 0x7f800000u;
  if (ex == 0u || ex == 0x7f800000u) return (double)f;
  const unsigned hi = (b & 0x80000000u) | (((b >> 3) & 0x0fffffffu) + (896u << 20));
  return __hiloint2double((int)hi, (int)(b << 29));
}
// double -> float, round to nearest even: the top 9 bits of (hi:lo) << 3 hold
// the low exponent bits, the next 23 the kept mantissa; the 29 bits shifted
// out decide the rounding (a carry into the exponent is the correct result,
// up to infinity at the top of the range); the exponent is rebiased modulo
// 512, exact for results in the normal FP32 range.
__device__ __forceinline__ float d2f_bits(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned e11 = (hi >> 20) & 0x7ffu;
  if (e11 <= 896u || e11 >= 1151u) return __double2float_rn(d);
  unsigned t = __funnelshift_l(lo, hi, 3);
  const unsigned rem = lo << 3;
  t += (rem > 0x80000000u || (rem == 0x80000000u && (t & 1u))) ? 1u : 0u;
  return __uint_as_float(((t - (384u << 23)) & 0x7fffffffu) | (hi & 0x80000000u));
}

template <class R>
__global__ void __launch_bounds__(512, 2) k_node(const NodeArgs A) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= A.N) return;
  const int inst = A.node_inst ? A.node_inst[n] : 0;
  const InstParams &ip = A.inst[inst];
  const bool leader = (n == ip.node_begin);
  const Slot4<R> *sF = reinterpret_cast<const Slot4<R> *>(A.sF);
  Slot4<R> *sU = reinterpret_cast<Slot4<R> *>(A.sU);
  const int sb = A.slot_off[n], se = A.slot_off[n + 1];
  const long long N = A.N;

  if (A.mode == kNodeScatterU) {  // replicate u into the patch slots
    const Slot4<R> r{R(A.u[n]), R(A.u[N + n]), R(A.u[2 * N + n]), R(0)};
    for (int k = sb; k < se; ++k) sU[A.slots[k]] = r;
    return;
  }
  if (A.mode == kNodeGather) {  // assembled internal force fi = sum of partials
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int k = sb; k < se; ++k) {
      const Slot4<R> q = sF[A.slots[k]];
      f0 += double(q.x);
      f1 += double(q.y);
      f2 += double(q.z);
    }
    A.fi_out[n] = f0;
    A.fi_out[N + n] = f1;
    A.fi_out[2 * N + n] = f2;
    return;
  }

  const Clock ck = A.clock[A.parity * A.ninst + inst];
  if (A.mode == kNodeBegin) {
    // first half of a step: v_half, u update, BCs at t_{n+1} (ex9.cpp:109-138)
    if (ck.done) return;
    const double t_n = ck.time, dt = ck.dt, t_np1 = t_n + dt, t_half = 0.5 * (t_np1 + t_n);
    double un[3];
    // rigid-body DOFs: the motion at t_{n+1} (k_rigid_begin advanced it)
    double ru[3] = {0.0, 0.0, 0.0}, rv[3] = {0.0, 0.0, 0.0}, ra[3] = {0.0, 0.0, 0.0};
    if (A.rbstep) {
      bool rig = false;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int fn = A.nbc[d * N + n];
        if (fn >= 0 && A.fns[fn].kind == kBckRigid) rig = true;
      }
      if (rig) rigid_node(A.rbstep + inst, A.X, N, n, ru, rv, ra);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int fn = A.nbc[d * N + n];
      const double uold = A.u[d * N + n];
      double u = uold;
      if (fn == kBcFree) {
        const double vh = A.v[d * N + n] + (t_half - t_n) * A.a[d * N + n];
        u = u + dt * vh;
        A.vh[d * N + n] = vh;
        A.u[d * N + n] = u;
      } else if (fn >= 0 && A.fns[fn].kind == kBckRigid) {
        // v_half of a constrained DOF is unused: it keeps a_n + a_{n+1}, the
        // inertia term of the DOF's reaction in the energy balance
        const double aold = A.a[d * N + n];
        u = ru[d];
        A.u[d * N + n] = u;
        A.v[d * N + n] = rv[d];
        A.a[d * N + n] = ra[d];
        A.vh[d * N + n] = aold + ra[d];
      } else if (fn >= 0) {
        double vb;
        bc_value(A.fns[fn], d, t_np1, A.X, N, n, u, vb);
        A.u[d * N + n] = u;
        A.v[d * N + n] = vb;
        A.a[d * N + n] = 0.0;
      }
      if (A.du) reinterpret_cast<R *>(A.du)[d * N + n] = R(u - uold);  // energy: this step's du
      un[d] = u;
    }
    const Slot4<R> r{R(un[0]), R(un[1]), R(un[2]), R(0)};
    for (int k = sb; k < se; ++k) sU[A.slots[k]] = r;
    return;
  }
  if (A.mode == kNodeInit) {
    // accelerations after the pre-loop GetForce (ex9.cpp:90-93): the partials
    // summed in slot order, in R (the energy balance's f_prev, as
    // k_node_step sums them) and in FP64
    R fr[3] = {0, 0, 0};
    double fd[3] = {0.0, 0.0, 0.0};
    for (int k = sb; k < se; ++k) {
      const Slot4<R> q = sF[A.slots[k]];
      fr[0] += q.x;
      fr[1] += q.y;
      fr[2] += q.z;
      fd[0] += double(q.x);
      fd[1] += double(q.y);
      fd[2] += double(q.z);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (A.fprev) reinterpret_cast<R *>(A.fprev)[d * N + n] = fr[d];
      if (A.nbc[d * N + n] != kBcFree) continue;
      const double f = fd[d];
      A.a[d * N + n] = A.fp64 ? -f / A.mass[n] : -f * A.minv[n];
    }
    if (leader) A.dtmin[A.parity * A.ninst + inst] = kDtHugeBits;
    return;
  }

}

// Step scalars of every instance for one end-of-step launch: the new dt from
// the dt minimum, the time levels, the velocity coefficients, the done flags
// and the trigonometry of the rigid-rotation functions at the new time.  One
// thread per instance, launched between the element pass and k_node_step, so
// that the FP64 divisions and sin/cos run once per instance and step rather
// than once per node block (FP64 issue is slow on this GPU).
// With the node-pass split, thread i also evaluates boundary function i once
// for the step when its value is the same for every node (fixed, ramp, sine)
// and one instance owns it (BcFn::pad): u and v at that instance's t_{n+2},
// the values node_step's bc_value would compute per DOF.
__global__ void k_step_scalars(const NodeArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (A.fnval && i < A.nfns) {
    const BcFn &b = A.fns[i];
    if (b.kind <= kBckSine && b.pad >= 0) {
      const int o = b.pad;
      const Clock co = A.clock[A.parity * A.ninst + o];
      const StepScalars so =
          step_scalars(co, A.inst[o], A.dtmin[A.parity * A.ninst + o], A.mode);
      if (so.advance && !co.done) {
        double u, v;
        bc_value(b, 0, so.t_np2, A.X, A.N, 0, u, v);
        A.fnval[i] = make_double2(u, v);
      }
    }
  }
  if (i >= A.ninst) return;
  const Clock ck = A.clock[A.parity * A.ninst + i];
  const StepScalars sc = step_scalars(ck, A.inst[i], A.dtmin[A.parity * A.ninst + i], A.mode);
  A.stepsc[i] = sc;
  // the instance's clock for the next step and its fresh dt-minimum slot
  // (the other parity: nothing reads them before the next element pass).
  // The first node's thread of k_node_step writes the same values.
  Clock nx = ck;
  if (!ck.done) {
    nx.time = sc.t_np1;
    nx.dt = sc.ndt;
    nx.step = ck.step + 1;
    nx.done = sc.done;
    nx.err = (sc.done & 4) ? kErrDt : 0;
  }
  A.clock[(A.parity ^ 1) * A.ninst + i] = nx;
  A.dtmin[(A.parity ^ 1) * A.ninst + i] = kDtHugeBits;
  if (sc.advance && !ck.done)
    for (int k = 0; k < A.nrot; ++k) {
      double *r = A.rottrig + 3 * ((long long)i * kMaxRotFns + k);
      rot_trig(A.fns[A.rot_ids[k]], sc.t_np2, r[0], r[1], r[2]);
    }
}

// The driven nodes' motion at t_{n+2} for the next step, after
// k_step_scalars, one warp per instance: the rigid body's integrator step
// (ex5.cpp:344 with Time = t_{n+2}, dt = the new dt) and the trigonometry of
// the rigid-rotation functions (lane k: function k).  It runs on a second
// stream beside k_node_step over the nodes without such DOFs: the integrator
// and sin/cos are latency-bound FP64 chains, the free-node update is
// bandwidth-bound, and only the driven nodes (k_node_step over their list,
// after this kernel) need the result.
__global__ void __launch_bounds__(32) k_driven_step(const NodeArgs A) {
  __shared__ double sacc[5][6];
  const int i = blockIdx.x;
  const Clock ck = A.clock[A.parity * A.ninst + i];
  const StepScalars sc = A.stepsc[i];
  if (!sc.advance || ck.done) return;
  const int k = threadIdx.x;
  if (k < A.nrot) {
    double *r = A.rottrig + 3 * ((long long)i * kMaxRotFns + k);
    rot_trig(A.fns[A.rot_ids[k]], sc.t_np2, r[0], r[1], r[2]);
  }
  if (A.rb) rigid_advance(A, i, sc.t_np2 - sc.ndt, sc.ndt, sacc);
}

// Before a kNodeBegin launch: advance each running instance's rigid body to
// t_{n+1} = t_n + dt (ex5.cpp:344 with Time = t_{n+1}).  One warp per instance.
__global__ void __launch_bounds__(32) k_rigid_begin(const NodeArgs A) {
  __shared__ double sacc[5][6];
  const int i = blockIdx.x;
  const Clock ck = A.clock[A.parity * A.ninst + i];
  if (ck.done) return;
  const double t_np1 = ck.time + ck.dt;
  rigid_advance(A, i, t_np1 - ck.dt, ck.dt, sacc);
}

// The constrained DOFs of node n in k_node_step: their kinetic-energy and
// reaction-work terms (EN) and, when the step advances, the boundary
// functions at t_{n+2} (a rigid rotation or the instance's rigid body
// evaluated once for the node's three DOFs).  Out of line: only boundary
// nodes take it, and the free-node path keeps its registers.  The reaction
// is fi_prev + fi + m (a + a_prev) (CheckEnergy.cpp:39-42); a + a_prev is
// kept in v_half for a rigid-body DOF and is 0 for the other constrained
// DOFs (a = 0 there).
template <class R, bool EN>
__device__ __forceinline__ void node_step_bc_body(const NodeArgs &A, long long n, int inst,
                                                  const StepScalars &sc, const int *nbc,
                                                  const double *fsum, const R *du_,
                                                  const R *fp_, const double *vb_,
                                                  const double *vh0, double mass, double *un,
                                                  R &eke, R &ewe) {
  const long long N = A.N;
  const bool advance = sc.advance;
  double ur[3] = {0.0, 0.0, 0.0}, vr[3] = {0.0, 0.0, 0.0}, ar[3] = {0.0, 0.0, 0.0};
  bool rigd[3] = {false, false, false}, rig = false;
  int rot_fn = -1;
  for (int d = 0; d < 3; ++d) {
    const int fn = nbc[d];
    if (fn < 0) continue;
    const int kind = A.fns[fn].kind;
    rigd[d] = kind == kBckRigid && A.rbstep;
    rig = rig || rigd[d];
    if (kind == kBckRot && rot_fn < 0) rot_fn = fn;
  }
  double aold[3] = {0.0, 0.0, 0.0};
  if (advance && rig) {  // rigid body at t_{n+2} (k_driven_step advanced it)
    for (int d = 0; d < 3; ++d)
      if (rigd[d]) aold[d] = A.a[d * N + n];
    rigid_node(A.rbstep + inst, A.X, N, n, ur, vr, ar);
  }
  if (advance && rot_fn >= 0) {
    const BcFn &b = A.fns[rot_fn];
    double c, s, om;
    if (b.pad >= 0 && b.pad < A.nrot) {
      const double *r = A.rottrig + 3 * ((long long)inst * kMaxRotFns + b.pad);
      c = r[0];
      s = r[1];
      om = r[2];
    } else {
      rot_trig(b, sc.t_np2, c, s, om);
    }
    rot_apply(b, c, s, om, A.X, N, n, ur, vr);
  }
  for (int d = 0; d < 3; ++d) {
    const int fn = nbc[d];
    if (fn == kBcFree) continue;
    if (EN) {
      const R fi = R(fsum[d]);
      const R vb = R(vb_[d]);
      eke += R(mass) * vb * vb;
      ewe += rigd[d] ? du_[d] * (fp_[d] + fi + R(mass * vh0[d])) : du_[d] * (fp_[d] + fi);
    }
    if (fn >= 0 && advance) {
      double u, vb, ab = 0.0;
      if (rigd[d]) {
        u = ur[d];
        vb = vr[d];
        ab = ar[d];
        A.vh[d * N + n] = aold[d] + ab;
      } else if (fn == rot_fn) {
        u = ur[d];
        vb = vr[d];
      } else {
        bc_value(A.fns[fn], d, sc.t_np2, A.X, N, n, u, vb);
      }
      A.u[d * N + n] = u;
      A.v[d * N + n] = vb;
      A.a[d * N + n] = ab;
      un[d] = u;
    }
  }
}

// Out-of-line copy for the all-node launch, whose free-node path keeps its
// registers; the driven-node launch inlines the body.
template <class R, bool EN>
__device__ __noinline__ void node_step_bc(const NodeArgs &A, long long n, int inst,
                                          const StepScalars &sc, const int *nbc,
                                          const double *fsum, const R *du_, const R *fp_,
                                          const double *vb_, const double *vh0, double mass,
                                          double *un, R &eke, R &ewe) {
  node_step_bc_body<R, EN>(A, n, inst, sc, nbc, fsum, du_, fp_, vb_, vh0, mass, un, eke, ewe);
}

// End of step n (mode kNodeFused also starts step n+1; kNodeFinish stops
// there), with the step scalars k_step_scalars left for the node's instance.
// At most 64 registers: the kernel waits on memory, so resident warps matter.
// One node of k_node_step.  EN: also this node's share of the energy balance
// (CheckEnergy.cpp:18-55 with fe = 0): kinetic energy m v_{n+1}^2, internal
// work du (f_prev + f) and, for constrained DOFs, the work of the reaction
// (node_step_bc).  The terms are formed in the element precision R (FP32 in
// mixed mode, where du and f are FP32 already: FP64 issue is slow on this
// GPU), FP64 in FP64 mode.
template <class R, bool EN, bool BCI = false>
__device__ __forceinline__ void node_step(const NodeArgs &A, long long n, R &eke, R &ewi,
                                          R &ewe) {
  const long long N = A.N;
  const Slot4<R> *sF = reinterpret_cast<const Slot4<R> *>(A.sF);
  Slot4<R> *sU = reinterpret_cast<Slot4<R> *>(A.sU);
  const int inst = A.node_inst ? A.node_inst[n] : 0;
  // the node's slots: one 16-byte record, so that the partial-force loads
  // wait on one round trip instead of two (offsets, then slot ids)
  const int4 sr = A.slot4[n];
  int4 sr2 = make_int4(-1, -1, -1, -1);
  if (A.slot4b) sr2 = A.slot4b[n];
  const int ss[8] = {sr.x, sr.y, sr.z, sr.w, sr2.x, sr2.y, sr2.z, sr2.w};
  const bool csr = sr.x == kSlotCsr;
  int nbc[3];
  double u0[3], vh0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    nbc[d] = A.nbc[d * N + n];
    u0[d] = A.u[d * N + n];
    vh0[d] = A.vh[d * N + n];
  }
  const bool anybc = nbc[0] != kBcFree || nbc[1] != kBcFree || nbc[2] != kBcFree;
  if (anybc && A.skip_driven) {  // handled by the driven-node branch of the step
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (nbc[d] >= 0 && (A.fns[nbc[d]].kind == kBckRigid || A.fns[nbc[d]].kind == kBckRot))
        return;
  }
  // 1/m (mixed mode, FP32; FP64 mode divides by m as the reference does)
  const float minv = sizeof(R) == 8 ? 0.f : A.minv[n];
  // energy inputs of all three DOFs, issued with the other loads and before
  // any store of this node (the stores could alias them and serialise loads)
  R *du = reinterpret_cast<R *>(A.du), *fp = reinterpret_cast<R *>(A.fprev);
  R du_[3] = {0, 0, 0}, fp_[3] = {0, 0, 0};
  double vb_[3] = {0.0, 0.0, 0.0};
  const double mass = EN ? A.mass[n] : 0.0;
  if (EN) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      du_[d] = du[d * N + n];
      fp_[d] = fp[d * N + n];
      if (nbc[d] != kBcFree) vb_[d] = A.v[d * N + n];  // constrained DOF: v(t_{n+1})
    }
  }

  // sum of the patch partials in slot order (in the element precision)
  R fs0 = 0, fs1 = 0, fs2 = 0;
  if (!csr) {
    Slot4<R> q[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (ss[j] >= 0) q[j] = sF[ss[j]];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (ss[j] >= 0) {
        fs0 += q[j].x;
        fs1 += q[j].y;
        fs2 += q[j].z;
      }
    if (A.slot4b) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (ss[4 + j] >= 0) q[j] = sF[ss[4 + j]];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (ss[4 + j] >= 0) {
          fs0 += q[j].x;
          fs1 += q[j].y;
          fs2 += q[j].z;
        }
    }
  } else {
    for (int k = A.slot_off[n]; k < A.slot_off[n + 1]; ++k) {
      const Slot4<R> q = sF[A.slots[k]];
      fs0 += q.x;
      fs1 += q.y;
      fs2 += q.z;
    }
  }
  const InstParams &ip = A.inst[inst];
  const bool leader = (n == ip.node_begin);
  const Clock ck = A.clock[A.parity * A.ninst + inst];
  // kNodeFused / kNodeFinish: end of step n (+ start of step n+1 when fused)
  Clock *nxt = A.clock + (A.parity ^ 1) * A.ninst + inst;
  if (ck.done) {
    // keep both clock slots and the next dt-min slot valid for the next run
    if (leader) {
      *nxt = ck;
      A.dtmin[(A.parity ^ 1) * A.ninst + inst] = kDtHugeBits;
    }
    return;
  }
  const StepScalars sc = A.stepsc[inst];
  const bool advance = sc.advance;
  constexpr bool kF64 = sizeof(R) == 8;
  const double fsum[3] = {double(fs0), double(fs1), double(fs2)};
  const R fsr[3] = {fs0, fs1, fs2};
  // mixed mode: a = f / m and the velocity increments c a in FP32 (f is an
  // FP32 sum), accumulated into the FP64 state -- one FP64 add per DOF
  // instead of a multiply and a fused multiply-add: FP64 issue is slow on
  // this GPU
  const float c1f = sc.c1f, c12f = sc.c12f;
  double un[3] = {u0[0], u0[1], u0[2]};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int fn = nbc[d];
    if (EN) {
      const R fi = fsr[d];  // a sum in the element precision
      if (fn == kBcFree) {
        R v1;
        if (kF64) {
          v1 = R(vh0[d] + sc.c1 * (-fsum[d] / A.mass[n]));
        } else {
          v1 = R(vh0[d]) + R(c1f) * (-fi * R(minv));
        }
        eke += R(mass) * v1 * v1;
      }
      ewi += du_[d] * (fp_[d] + fi);
      fp[d * N + n] = fi;
    }
    if (fn == kBcFree) {
      const double vh = vh0[d];
      if (kF64) {
        const double acc = -fsum[d] / A.mass[n];
        if (advance) {  // the two half-step updates of ex9.cpp:147-152 and :116-123
          const double vel = vh + sc.c1 * acc;
          const double vh2 = vel + sc.c2 * acc;
          un[d] = u0[d] + sc.ndt * vh2;
          A.vh[d * N + n] = vh2;
          A.u[d * N + n] = un[d];
        } else {
          A.v[d * N + n] = vh + sc.c1 * acc;
          A.a[d * N + n] = acc;
        }
      } else {
        const float acc = -float(fsr[d]) * minv;
        if (advance) {  // one update with the combined coefficient t_half' - t_half
          const double vh2 = vh + double(c12f * acc);
          un[d] = u0[d] + sc.ndt * vh2;
          A.vh[d * N + n] = vh2;
          A.u[d * N + n] = un[d];
        } else {
          A.v[d * N + n] = vh + double(c1f * acc);
          A.a[d * N + n] = double(acc);
        }
      }
    }
  }
  if (anybc) {
    if (BCI)
      node_step_bc_body<R, EN>(A, n, inst, sc, nbc, fsum, du_, fp_, vb_, vh0, mass, un, eke, ewe);
    else
      node_step_bc<R, EN>(A, n, inst, sc, nbc, fsum, du_, fp_, vb_, vh0, mass, un, eke, ewe);
  }
  if (EN && advance) {
#pragma unroll
    for (int d = 0; d < 3; ++d) du[d * N + n] = R(un[d] - u0[d]);
  }
  if (advance) {
    const Slot4<R> r{R(un[0]), R(un[1]), R(un[2]), R(0)};
    if (!csr) {
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (ss[j] >= 0) sU[ss[j]] = r;
    } else {
      for (int k = A.slot_off[n]; k < A.slot_off[n + 1]; ++k) sU[A.slots[k]] = r;
    }
  }
  if (leader) {
    Clock c;
    c.time = sc.t_np1;
    c.dt = sc.ndt;
    c.step = ck.step + 1;
    c.done = sc.done;
    c.err = (sc.done & 4) ? kErrDt : 0;
    *nxt = c;
    A.dtmin[(A.parity ^ 1) * A.ninst + inst] = kDtHugeBits;
  }
}

// The mixed-precision step of every node that is not in the rest list, one
// thread per node: gather the partials (slot records, or the node's slot list
// when it has more), a = f / m in FP32, then for a free DOF either v_half' =
// v_half + c12 a and u' = u + dt v_half' in FP64, or -- the step that ends a
// run -- v = v_half + c1 a and a; a DOF under a cached boundary function
// takes its u and v at t_{n+2} from fnval (a = 0), a held DOF keeps u; u'
// goes back into the node's slots.  The operations and their order are
// node_step's, so the bits are too; the FP32 <-> FP64 conversions are integer
// arithmetic, and no per-node transcendental or clock work is on this path.
__global__ void __launch_bounds__(512, 2) k_node_free(const NodeArgs A) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= A.N) return;
  const long long N = A.N;
  // every load of the node up front (a rest node's are wasted, the others'
  // latencies overlap): kind, slot records, state, 1/m
  const int kind = __ldg(A.nkind + n);
  const int4 sr = __ldg(A.slot4 + n);
  int4 sr2 = make_int4(-1, -1, -1, -1);
  if (A.slot4b) sr2 = __ldg(A.slot4b + n);
  const int inst = A.node_inst ? __ldg(A.node_inst + n) : 0;
  double u0[3], vh0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    u0[d] = A.u[d * N + n];  // (read and written here: plain loads)
    vh0[d] = A.vh[d * N + n];
  }
  const float minv = __ldg(A.minv + n);
  if (kind & kNodeRest) return;
  int fn[3] = {kBcFree, kBcFree, kBcFree};
  if (kind & kNodeBcCached) {
#pragma unroll
    for (int d = 0; d < 3; ++d) fn[d] = __ldg(A.nbc + d * N + n);
  }
  const Slot4<float> *sF = reinterpret_cast<const Slot4<float> *>(A.sF);
  const bool csr = sr.x == kSlotCsr;
  const int s4[4] = {sr.x, sr.y, sr.z, sr.w};
  const int s8[4] = {sr2.x, sr2.y, sr2.z, sr2.w};
  float fs0 = 0.f, fs1 = 0.f, fs2 = 0.f;
  if (!csr) {
    Slot4<float> q[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (s4[j] >= 0) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(sF + s4[j]));
        q[j] = Slot4<float>{v.x, v.y, v.z, v.w};
      }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (s4[j] >= 0) {
        fs0 += q[j].x;
        fs1 += q[j].y;
        fs2 += q[j].z;
      }
    if (A.slot4b) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s8[j] >= 0) q[j] = sF[s8[j]];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s8[j] >= 0) {
          fs0 += q[j].x;
          fs1 += q[j].y;
          fs2 += q[j].z;
        }
    }
  } else {
    for (int k = A.slot_off[n]; k < A.slot_off[n + 1]; ++k) {
      const Slot4<float> q = sF[A.slots[k]];
      fs0 += q.x;
      fs1 += q.y;
      fs2 += q.z;
    }
  }
  if (A.clock[A.parity * A.ninst + inst].done) return;  // past its end: nothing moves
  const StepScalars &sc = A.stepsc[inst];
  const float fs[3] = {fs0, fs1, fs2};
  if (!sc.advance) {  // the run ends with this step: v and a of the free DOFs
    const float c1f = sc.c1f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (fn[d] != kBcFree) continue;
      const float acc = -fs[d] * minv;
      A.v[d * N + n] = vh0[d] + f2d_bits(c1f * acc);
      A.a[d * N + n] = f2d_bits(acc);
    }
    return;
  }
  const float c12f = sc.c12f;
  const double ndt = sc.ndt;
  float r[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double un = u0[d];
    if (fn[d] == kBcFree) {
      const float acc = -fs[d] * minv;
      const double vh2 = vh0[d] + f2d_bits(c12f * acc);
      un = u0[d] + ndt * vh2;
      A.vh[d * N + n] = vh2;
      A.u[d * N + n] = un;
    } else if (fn[d] >= 0) {  // boundary function: u, v at t_{n+2}, a = 0
      const double2 bv = A.fnval[fn[d]];
      un = bv.x;
      A.u[d * N + n] = bv.x;
      A.v[d * N + n] = bv.y;
      A.a[d * N + n] = 0.0;
    }
    r[d] = d2f_bits(un);
  }
  Slot4<float> *sU = reinterpret_cast<Slot4<float> *>(A.sU);
  const Slot4<float> w{r[0], r[1], r[2], 0.f};
  if (!csr) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (s4[j] >= 0) sU[s4[j]] = w;
    if (A.slot4b) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s8[j] >= 0) sU[s8[j]] = w;
    }
  } else {
    for (int k = A.slot_off[n]; k < A.slot_off[n + 1]; ++k) sU[A.slots[k]] = w;
  }
}

// LIST: over A.node_list (the driven nodes of the rigid-body branch, whose
// boundary path is inlined), else over every node.  At most 64 registers
// (two 512-thread blocks per SM) also with the energy terms: their spills
// cost less than half the resident warps (block node pass with the energy
// balance 0.51 ms at 128 registers, 0.445 ms at 64).
template <class R, bool EN, bool LIST = false>
__global__ void __launch_bounds__(512, LIST ? 1 : 2) k_node_step(const NodeArgs A) {
  long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool on = n < A.N;
  if (LIST) {
    on = n < A.nlist;
    n = on ? A.node_list[n] : 0;
  }
  R eke = 0, ewi = 0, ewe = 0;
  if (!EN) {
    if (on) node_step<R, false, LIST>(A, n, eke, ewi, ewe);
    return;
  }
  if (on) node_step<R, true, LIST>(A, n, eke, ewi, ewe);
  // block partials in a fixed order: warp butterfly in R, then the warps in
  // order in FP64
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    eke += __shfl_xor_sync(0xffffffffu, eke, o);
    ewi += __shfl_xor_sync(0xffffffffu, ewi, o);
    ewe += __shfl_xor_sync(0xffffffffu, ewe, o);
  }
  __shared__ double part[16][3];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    part[w][0] = double(eke);
    part[w][1] = double(ewi);
    part[w][2] = double(ewe);
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x + 31) / 32; ++k) s += part[k][threadIdx.x];
    A.epart[3 * (A.epart_off + blockIdx.x) + threadIdx.x] = s;
  }
}

// The energy balance of the step just finished from the block partials of
// k_node_step (one block, fixed summation order): the reference's CheckEnergy
// after the velocity update (ex9.cpp:154-156).  Skipped for a step that did
// not run (the instance was already done).
__global__ void __launch_bounds__(1024) k_energy_reduce(const NodeArgs A, int nblocks) {
  __shared__ double red[3][1024];
  double s[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] += A.epart[3 * (long long)b + k];
#pragma unroll
  for (int k = 0; k < 3; ++k) red[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  if (A.clock[A.parity * A.ninst].done) return;
  EnergyState e = *A.energy;
  const double wke = 0.5 * red[0][0];
  e.Wint += 0.5 * red[1][0];
  e.Wext += 0.5 * red[2][0];
  e.WKE = wke;
  e.total = fabs(wke + e.Wint - e.Wext);
  const double mx = fmax(fabs(e.Wint), fmax(fabs(e.Wext), fabs(wke)));
  if (e.total > 0.01 * mx) ++e.violations;
  if (mx > 0.0) e.max_ratio = fmax(e.max_ratio, e.total / mx);
  ++e.steps;
  *A.energy = e;
}

// Pre-loop clock: dt = reduction * StableTimeStep() at t0 (ex9.cpp:87).
__global__ void k_clock_init(Clock *clock, unsigned long long *dtmin, const InstParams *ip,
                             int ninst, double t0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ninst) return;
  const double raw = __longlong_as_double((long long)dtmin[i]);
  Clock c;
  c.time = t0;
  c.dt = ip[i].reduction * raw;
  c.step = 0;
  c.done = 0;
  if (raw < ip[i].failure_dt) c.done |= 4;
  if (!(t0 < ip[i].tmax)) c.done |= 1;
  c.err = (c.done & 4) ? kErrDt : 0;
  clock[i] = c;
  clock[ninst + i] = c;
  dtmin[i] = kDtHugeBits;
  dtmin[ninst + i] = kDtHugeBits;
}

// Apply the boundary functions at time t (pre-loop BC call, ex9.cpp:84).
// (and, R: the node's displacement replicated into its patch slots, as
// k_node's ScatterU mode does, in the element precision)
template <class R>
__global__ void k_apply_bc(const NodeArgs A, double t) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= A.N) return;
  const long long N = A.N;
  const int inst = A.node_inst ? A.node_inst[n] : 0;
  double un[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int fn = A.nbc[d * N + n];
    un[d] = A.u[d * N + n];
    if (fn < 0) continue;
    double u, v, a = 0.0;
    if (A.fns[fn].kind == kBckRigid) {  // the rigid body's current state
      double ru[3], rv[3], ra[3];
      rigid_node(A.rbstep + inst, A.X, N, n, ru, rv, ra);
      u = ru[d];
      v = rv[d];
      a = ra[d];
    } else {
      bc_value(A.fns[fn], d, t, A.X, N, n, u, v);
    }
    A.u[d * N + n] = u;
    A.v[d * N + n] = v;
    A.a[d * N + n] = a;
    un[d] = u;
  }
  const Slot4<R> r{R(un[0]), R(un[1]), R(un[2]), R(0)};
  Slot4<R> *sU = reinterpret_cast<Slot4<R> *>(A.sU);
  for (int k = A.slot_off[n]; k < A.slot_off[n + 1]; ++k) sU[A.slots[k]] = r;
}

}  // namespace ftgpu
