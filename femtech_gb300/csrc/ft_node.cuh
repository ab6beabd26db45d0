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
  return s;
}

template <class R>
__global__ void __launch_bounds__(512) k_node(const NodeArgs A) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= A.N) return;
  const int inst = A.node_inst ? A.node_inst[n] : 0;
  const InstParams &ip = A.inst[inst];
  const bool leader = (n == ip.node_begin);
  const R *sF = reinterpret_cast<const R *>(A.sF);
  R *sU = reinterpret_cast<R *>(A.sU);
  const int sb = A.slot_off[n], se = A.slot_off[n + 1];
  const long long N = A.N, S = A.S;

  if (A.mode == kNodeScatterU) {  // replicate u into the patch slots
    for (int k = sb; k < se; ++k) {
      const int s = A.slots[k];
#pragma unroll
      for (int d = 0; d < 3; ++d) sU[d * S + s] = R(A.u[d * N + n]);
    }
    return;
  }
  if (A.mode == kNodeGather) {  // assembled internal force fi = sum of partials
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double f = 0.0;
      for (int k = sb; k < se; ++k) f += double(sF[d * S + A.slots[k]]);
      A.fi_out[d * N + n] = f;
    }
    return;
  }

  const Clock ck = A.clock[A.parity * A.ninst + inst];
  if (A.mode == kNodeBegin) {
    // first half of a step: v_half, u update, BCs at t_{n+1} (ex9.cpp:109-138)
    if (ck.done) return;
    const double t_n = ck.time, dt = ck.dt, t_np1 = t_n + dt, t_half = 0.5 * (t_np1 + t_n);
    double un[3];
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
    for (int k = sb; k < se; ++k) {
      const int s = A.slots[k];
#pragma unroll
      for (int d = 0; d < 3; ++d) sU[d * S + s] = R(un[d]);
    }
    return;
  }
  if (A.mode == kNodeInit) {
    // accelerations after the pre-loop GetForce (ex9.cpp:90-93)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (A.fprev) {  // energy balance: f of the pre-loop state, summed as k_node_step does
        R fr = 0;
        for (int k = sb; k < se; ++k) fr += sF[d * S + A.slots[k]];
        reinterpret_cast<R *>(A.fprev)[d * N + n] = fr;
      }
      if (A.nbc[d * N + n] != kBcFree) continue;
      double f = 0.0;
      for (int k = sb; k < se; ++k) f += double(sF[d * S + A.slots[k]]);
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
__global__ void k_step_scalars(const NodeArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ninst) return;
  const Clock ck = A.clock[A.parity * A.ninst + i];
  const StepScalars sc = step_scalars(ck, A.inst[i], A.dtmin[A.parity * A.ninst + i], A.mode);
  A.stepsc[i] = sc;
  if (sc.advance && !ck.done)
    for (int k = 0; k < A.nrot; ++k) {
      double *r = A.rottrig + 3 * ((long long)i * kMaxRotFns + k);
      rot_trig(A.fns[A.rot_ids[k]], sc.t_np2, r[0], r[1], r[2]);
    }
}

// End of step n (mode kNodeFused also starts step n+1; kNodeFinish stops
// there), with the step scalars k_step_scalars left for the node's instance.
// At most 64 registers: the kernel waits on memory, so resident warps matter.
// One node of k_node_step.  EN: also this node's share of the energy balance
// (CheckEnergy.cpp:18-55 with fe = 0): kinetic energy m v_{n+1}^2, internal
// work du (f_prev + f) and, for constrained DOFs, the work of the reaction
// du (f_prev + f + m (a + a_prev)) with a = a_prev = 0 on constrained DOFs.
// The terms are formed in the element precision R (FP32 in mixed mode, where
// du and f are FP32 already: FP64 issue is slow on this GPU), FP64 in FP64
// mode.
template <class R, bool EN>
__device__ __forceinline__ void node_step(const NodeArgs &A, long long n, R &eke, R &ewi,
                                          R &ewe) {
  const long long N = A.N, S = A.S;
  const R *sF = reinterpret_cast<const R *>(A.sF);
  R *sU = reinterpret_cast<R *>(A.sU);
  const int inst = A.node_inst ? A.node_inst[n] : 0;
  const int sb = A.slot_off[n], se = A.slot_off[n + 1];
  int nbc[3];
  double u0[3], vh0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    nbc[d] = A.nbc[d * N + n];
    u0[d] = A.u[d * N + n];
    vh0[d] = A.vh[d * N + n];
  }
  // 1/m (mixed mode; FP64 mode divides by m as the reference does)
  const double minv = sizeof(R) == 8 ? 0.0 : A.minv[n];
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
  for (int k = sb; k < se; ++k) {
    const int s = A.slots[k];
    fs0 += sF[s];
    fs1 += sF[S + s];
    fs2 += sF[2 * S + s];
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
  double un[3];
  // a rigid rotation drives all its DOFs at once: evaluate it once per node
  double ur[3] = {0.0, 0.0, 0.0}, vr[3] = {0.0, 0.0, 0.0};
  int rot_fn = -1;
  if (advance) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int fn = nbc[d];
      if (fn >= 0 && rot_fn < 0 && A.fns[fn].kind == kBckRot) rot_fn = fn;
    }
    if (rot_fn >= 0) {
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
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int fn = nbc[d];
    double u = u0[d];
    if (EN) {
      const R fi = R(fsum[d]);  // exact: a sum in the element precision
      const R w = du_[d] * (fp_[d] + fi);
      if (fn == kBcFree) {
        R v1;
        if (kF64) {
          v1 = R(vh0[d] + sc.c1 * (-fsum[d] / A.mass[n]));
        } else {
          v1 = R(vh0[d]) + R(sc.c1) * (-fi * R(minv));
        }
        eke += R(mass) * v1 * v1;
      } else {
        const R vb = R(vb_[d]);
        eke += R(mass) * vb * vb;
        ewe += w;
      }
      ewi += w;
      fp[d * N + n] = fi;
    }
    if (fn == kBcFree) {
      const double acc = kF64 ? -fsum[d] / A.mass[n] : -fsum[d] * minv;
      const double vh = vh0[d];
      if (advance) {
        double vh2;
        if (kF64) {  // the two half-step updates of ex9.cpp:147-152 and :116-123
          const double vel = vh + sc.c1 * acc;
          vh2 = vel + sc.c2 * acc;
        } else {  // one update with the combined coefficient t_half' - t_half
          vh2 = vh + sc.c12 * acc;
        }
        u = u + sc.ndt * vh2;
        A.vh[d * N + n] = vh2;
        A.u[d * N + n] = u;
      } else {
        A.v[d * N + n] = vh + sc.c1 * acc;
        A.a[d * N + n] = acc;
      }
    } else if (fn >= 0 && advance) {
      double vb;
      if (fn == rot_fn) {
        u = ur[d];
        vb = vr[d];
      } else {
        bc_value(A.fns[fn], d, sc.t_np2, A.X, N, n, u, vb);
      }
      A.u[d * N + n] = u;
      A.v[d * N + n] = vb;
      A.a[d * N + n] = 0.0;
    }
    un[d] = u;
  }
  if (EN && advance) {
#pragma unroll
    for (int d = 0; d < 3; ++d) du[d * N + n] = R(un[d] - u0[d]);
  }
  if (advance) {
    const R r0 = R(un[0]), r1 = R(un[1]), r2 = R(un[2]);
    for (int k = sb; k < se; ++k) {
      const int s = A.slots[k];
      sU[s] = r0;
      sU[S + s] = r1;
      sU[2 * S + s] = r2;
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

template <class R, bool EN>
__global__ void __launch_bounds__(512, EN ? 1 : 2) k_node_step(const NodeArgs A) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  R eke = 0, ewi = 0, ewe = 0;
  if (!EN) {
    if (n < A.N) node_step<R, false>(A, n, eke, ewi, ewe);
    return;
  }
  if (n < A.N) node_step<R, true>(A, n, eke, ewi, ewe);
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
    A.epart[3 * (long long)blockIdx.x + threadIdx.x] = s;
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
__global__ void k_apply_bc(const NodeArgs A, double t) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= A.N) return;
  const long long N = A.N;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int fn = A.nbc[d * N + n];
    if (fn < 0) continue;
    double u, v;
    bc_value(A.fns[fn], d, t, A.X, N, n, u, v);
    A.u[d * N + n] = u;
    A.v[d * N + n] = v;
    A.a[d * N + n] = 0.0;
  }
}

}  // namespace ftgpu
