// ft_common.h -- device data structures shared by the kernels and the host
// orchestration of the explicit hot path.
#pragma once

#include <cstdint>

#include "ft_materials.cuh"
#include "ft_mlp.cuh"

namespace ftgpu {

constexpr int kMaxPatchElems = 256;   // elements per patch (thread block) upper bound
constexpr int kMaxLocalNodes = 320;   // local nodes per patch (shared memory bound)
constexpr int kElemThreads = 256;     // upper bound of threads per element block

// Shared memory of an element block's staged local CSR (the in-block
// assembly's offsets and corner entries, 16-bit): kMaxLocalNodes + 1 offsets
// padded to 8, then NC entries per element.
__host__ __device__ constexpr size_t elem_csr_smem_bytes(int NC, int PE) {
  return 2 * ((size_t)kMaxLocalNodes + 8) + 2 * (size_t)NC * PE;
}

// Per-instance clock, double-buffered by step parity.  Between steps it holds
// the state the reference keeps in the globals Time and dt (ex9.cpp:9).
struct Clock {
  double time;     // t_n
  double dt;       // dt_n (the next step's increment)
  long long step;  // steps completed
  int done;        // bit0 tMax reached, bit1 step limit, bit2 error
  int err;
};

struct InstParams {
  double tmax;
  double reduction;   // ExplicitTimeStepReduction
  double failure_dt;  // FailureTimeStep
  long long step_limit;
  int node_begin;     // first node: its thread advances the clock
  int pad;
};

struct BcFn {
  int kind;
  int pad;
  double p[8];
};

// Start value of the stable-dt minimum: the reference's "huge" = 1e20
// (include/GlobalVariables.h:15, StableTimeStep.cpp:6), as FP64 bits.
constexpr unsigned long long kDtHugeBits = 0x4415af1d78b58c40ull;

// Rigid-rotation functions whose trigonometry the nodal step caches per block
// (BcFn::pad holds a function's cache slot, -1 if none).
constexpr int kMaxRotFns = 8;

enum { kBcFree = -1, kBcHold = -2 };

// One patch slot of the partial-force and displacement-replica arrays: x, y,
// z and a pad, so that the node kernels' gathers and scatters (slots of a
// node are spread over patches) move one 16-byte (FP32) or 32-byte (FP64)
// record per slot instead of three scattered words.
template <class R>
struct alignas(4 * sizeof(R)) Slot4 {
  R x, y, z, w;
};
enum { kBckFixed = 0, kBckRamp = 1, kBckSine = 2, kBckRot = 3, kBckRigid = 4 };
enum { kNodeBcCached = 1, kNodeRest = 2 };
enum { kErrInverted = 1, kErrDt = 2, kErrIndex = 4, kErrWait = 8 };

constexpr int kSlotCsr = -2;  // NodeArgs::slot4 marker: more slots than the records hold

template <class Real>
struct ElemArgs {
  // patches
  const int *patch_elem_off;  // [P+1] (element index in group order)
  const int *patch_node_off;  // [P+1] (slot index)
  const int *patch_inst;      // [P]
  const int *patch_ent_off;   // [P+1] into lent
  const uint16_t *lptr;       // per patch: n_local+1 offsets (block at patch_node_off[p]+p)
  const uint16_t *lent;       // local CSR entries: e_local * NC + corner
  // elements (group order)
  const uint16_t *lconn;      // this group's [nelem*NC] local node of each corner
  const int *epid;            // [E] part | (skip-dt << 31)
  const Real *fib;            // [3][E] unit fibre (material 7) or null
  // slots
  const Real *sX;             // [3][S] reference coordinates (patch-relative in mixed mode)
  const Real *sU;             // [S] Slot4: displacement replicas
  Real *sF;                   // [S] Slot4: patch-partial internal forces
  // material state
  Real *hist;                 // [ncomp][NGP][nelem] of this group
  // FP32 C3D8 groups: the reference geometry, written once at set-up -- per
  // element 80 values (Gauss point g: A^{-1} row major, then det A, at
  // 10 g .. 10 g + 9) in 20 rows of 4, value v at [4 (v/4 * nelem + e) + v%4]
  // (null for C3D4 groups and in FP64 mode)
  const Real *geo;
  const MatP<Real> *mats;
  // clock
  Clock *clock;               // [2][ninst]
  unsigned long long *dtmin;  // [2][ninst] (FP64 bit patterns)
  int *err;
  // optional Gauss-point outputs, [gpbase + e*NGP + g]
  double *gpF;
  double *gpJ;
  double *gpS;
  long long S, E;             // SoA strides
  int ninst, parity;
  int patch_begin, npatch, elem_begin, nelem;
  int use_clock;              // 1: dt and done flags from the clock; 0: dt_direct
  double dt_direct;
  long long gpbase;
  // learned surrogate of the material-7 isochoric stress (null when off):
  // pass 2 writes BF16 features [gp][16], the force pass reads outputs [gp][8]
  uint16_t *surr_x;
  const float *surr_y;
  SurrogateLaw law;
  // per-step injury criteria fused into the force pass (launch mode 2):
  // listed elements in group order and their state (null otherwise)
  const int *inj_cidx;        // [E] compact index or -1
  const int *inj_upos;        // [listed] position in the caller's list
  uint8_t *inj_flags;         // [listed]
  Real *inj_ps_old, *inj_psxsr;
  void *inj_part;             // [patches] InjuryPart block extremes
};

enum { kPassForce = 0, kPassDt = 1, kPassSurrogateFeatures = 2 };

// Energy balance of the explicit loop (CheckEnergy.cpp:3-85): cumulative
// internal and external work, kinetic energy of the last step, the balance
// |WKE + Wint - Wext| and its worst ratio to max(|Wint|, |Wext|, |WKE|), and
// the steps whose balance exceeded 1 % of that maximum (the reference's
// "Energy Violation" warning).
struct EnergyState {
  double Wint, Wext, WKE, total, max_ratio;
  long long steps, violations;
};

// Rigid body of an instance driven by sampled accelerations (the brain
// drivers' ApplyAccBoundaryConditions, examples/ex5/ex5.cpp:339-392):
// channels 0-2 angular acceleration x, y, z, 3-5 linear acceleration x, y, z,
// each a table of cnt[k] times, cnt[k] values and cnt[k] segment slopes
// (the last unused) at off[k] of the table array.
struct RigidBody {
  int off[6], cnt[6];
  int on, pad;
};

// Integrator state (ex5.cpp:100-105): y = [omega, r, v_cm, x_cm] (r: rotation
// generator, R = exp(r) as a quaternion), yd = dy/dt at the last step's end
// (first same as last), cur[k] = a table index at or below every later
// lookup of channel k.
struct RigidState {
  double y[12], yd[12];
  int cur[6];
  int pad[2];
};

// The motion of every driven node at the current time, as three affine maps
// of the position relative to the centre c (X' = X - c):
//   u = Mm X' + disp,  v = WM X' + vel,  a = AM X' + ca,
// Mm = R - I, WM = [omega]x R, AM = ([omega]x^2 + [alpha]x) R,
// ca = 2 omega x v_cm + a_cm.
struct RigidStep {
  double Mm[9], WM[9], AM[9];
  double disp[3], vel[3], ca[3], c[3];
};

// Per-instance scalars of one end-of-step launch (k_step_scalars)
struct StepScalars {
  double t_np1, t_np2, ndt;
  double c1;   // t_{n+1} - t_half         (full-step velocity)
  double c2;   // t_half' - t_{n+1}        (next half-step velocity)
  double c12;  // t_half' - t_half         (both at once)
  float c1f, c12f;  // c1 and c12 rounded to FP32 (the mixed update's increments)
  int done;
  bool advance;
};

struct NodeArgs {
  const int *slot_off;        // [N+1]
  const int *slots;           // node -> slots
  // [N] the node's first four slots in CSR order (-1: none), or x = kSlotCsr
  // for a node with more slots than the records hold (read through slot_off /
  // slots); slot4b, when set (meshes where many nodes have more than four
  // slots, e.g. tetrahedra), slots five to eight
  const int4 *slot4;
  const int4 *slot4b;
  const int *node_inst;       // [N] or null (one instance)
  const int16_t *nbc;         // [3N] per-DOF function (-1 free, -2 hold, >= 0 fn)
  // mixed-precision split of the node pass (null: no split): per node
  // kNodeBcCached (its constrained DOFs follow node-independent functions,
  // values in fnval, or hold) and kNodeRest (left to k_node_step over the
  // rest list: a node without slots, a rigid-rotation or rigid-body DOF)
  const uint8_t *nkind;
  double2 *fnval;             // [nfns] u, v at t_{n+2} of a cached function
  int nfns;
  const BcFn *fns;
  const double *X;            // [3][N] FP64 reference coordinates
  double *u, *v, *a, *vh;     // [3][N]
  const double *mass;         // [N] lumped mass (FP64)
  const float *minv;          // [N] 1 / mass (mixed mode)
  const void *sF;             // [S] Slot4<Real> partial forces
  void *sU;                   // [S] Slot4<Real> displacement replicas
  Clock *clock;
  unsigned long long *dtmin;
  const InstParams *inst;
  int *err;
  double *fi_out;             // optional [3][N] assembled internal force
  long long N, S;
  int ninst, parity;
  int mode;                   // kNodeBegin / kNodeFused / kNodeFinish / kNodeInit
  int fp64;                   // slot arrays are double
  int nrot;                   // rigid-rotation functions with a cache slot
  int rot_ids[kMaxRotFns];    // their indices in fns
  StepScalars *stepsc;        // [ninst] written by k_step_scalars
  double *rottrig;            // [ninst][kMaxRotFns][3] cos, sin, omega at t_{n+2}
  // energy balance (single instance; null when off)
  void *du;                   // [3][N] u_{n+1} - u_n of the step being finished (Real)
  void *fprev;                // [3][N] internal force of the previous step (Real)
  double *epart;              // [node blocks][3] partial sums: kinetic, internal, external
  EnergyState *energy;
  // rigid bodies driven by sampled accelerations (null when none)
  const RigidBody *rb;        // [ninst]
  const double *rbtab;        // tables of every instance
  RigidState *rbstate;        // [ninst]
  RigidStep *rbstep;          // [ninst]
  // k_node_step over a subset: node_list (nlist entries) or every node but
  // the driven ones -- a rigid-body or rigid-rotation DOF (skip_driven); its
  // energy partials start at block epart_off
  const int *node_list;
  long long nlist;
  int skip_driven;
  long long epart_off;
};

enum { kNodeBegin = 0, kNodeFused = 1, kNodeFinish = 2, kNodeInit = 3, kNodeGather = 4,
       kNodeScatterU = 5 };

}  // namespace ftgpu
