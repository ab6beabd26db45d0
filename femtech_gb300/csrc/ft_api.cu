// ft_api.cu -- the C ABI of include/ftgpu.h: device memory, one-time setup,
// symbol-compatible primitives and the graph-captured explicit loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ft_common.h"
#include "ft_injury.cuh"
#include "ft_launch.h"
#include "ft_node.cuh"
#include "ft_patches.h"
#include "ftgpu.h"

namespace ftgpu {

static thread_local std::string g_last_error;

static int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

// shared with the surrogate translation unit
int record_error(int code, const char *msg) { return fail(code, msg); }

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(FTGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)
#define CKI(expr)                                                                         \
  do {                                                                                    \
    int r_ = (expr);                                                                      \
    if (r_ != 0)                                                                          \
      return r_ > 0 ? fail(FTGPU_ERR_CUDA, std::string(#expr) + ": " +                    \
                                               cudaGetErrorString((cudaError_t)r_))       \
                    : r_;                                                                 \
  } while (0)

// Owning device buffer.
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  int alloc(size_t b) {
    release();
    if (b == 0) b = 16;
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(FTGPU_ERR_ALLOC, "cudaMalloc of " + std::to_string(b) + " bytes failed");
    }
    bytes = b;
    return 0;
  }
  template <class T>
  int upload(const T *h, size_t n) {
    int r = alloc(n * sizeof(T));
    if (r) return r;
    if (n && cudaMemcpy(p, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(FTGPU_ERR_CUDA, "upload failed");
    return 0;
  }
  template <class T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};

// Mass of one element's corners: m_a = rho * sum_gp w detJ N_a
// (Mass3D.cpp:5-67 row-sum lumping with sum_b N_b = 1), FP64.
template <int ET>
__global__ void k_mass(const int *patch_elem_off, const int *patch_node_off,
                       const int *patch_ent_off, const uint16_t *lptr, const uint16_t *lent,
                       const uint16_t *lconn, const int *epid, const int *slot_node,
                       const double *X, long long N, const MatP<double> *mats, int patch_begin,
                       int elem_begin, double *sM) {
  constexpr int NC = ET == 0 ? 8 : 4;
  __shared__ double shM[NC][kMaxPatchElems];
  const int p = patch_begin + blockIdx.x;
  const int e0 = patch_elem_off[p], ne = patch_elem_off[p + 1] - e0;
  const int s0 = patch_node_off[p], ns = patch_node_off[p + 1] - s0;
  const int t = threadIdx.x;
  if (t < ne) {
    const int e = e0 + t;
    double x[NC][3];
    for (int a = 0; a < NC; ++a) {
      const int n = slot_node[s0 + lconn[NC * (long long)(e - elem_begin) + a]];
      for (int d = 0; d < 3; ++d) x[a][d] = X[d * N + n];
    }
    const double rho = mats[epid[e] & 0x7fffffff].p[0];
    double m[NC];
    for (int a = 0; a < NC; ++a) m[a] = 0.0;
    if (ET == 0) {
      const int sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
      const int sg[8][3] = {{-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1},
                            {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}};
      const double G = 0.577350269189626;
      for (int g = 0; g < 8; ++g) {
        const double xi = sg[g][0] * G, et = sg[g][1] * G, ze = sg[g][2] * G;
        double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double N[8];
        for (int a = 0; a < 8; ++a) {
          const double sx = sgn[a][0], sy = sgn[a][1], sz = sgn[a][2];
          N[a] = (1 + sx * xi) * (1 + sy * et) * (1 + sz * ze) / 8;
          const double dx = sx * (1 + sy * et) * (1 + sz * ze) / 8;
          const double dy = sy * (1 + sx * xi) * (1 + sz * ze) / 8;
          const double dz = sz * (1 + sx * xi) * (1 + sy * et) / 8;
          for (int d = 0; d < 3; ++d) {
            A[0][d] += dx * x[a][d];
            A[1][d] += dy * x[a][d];
            A[2][d] += dz * x[a][d];
          }
        }
        const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                           A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                           A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
        for (int a = 0; a < 8; ++a) m[a] += det * N[a];
      }
    } else {
      double A[3][3];
      for (int r = 0; r < 3; ++r)
        for (int d = 0; d < 3; ++d) A[r][d] = x[r][d] - x[3][d];
      const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                         A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                         A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
      for (int a = 0; a < 4; ++a) m[a] = fabs(det) / 6.0 * 0.25;
    }
    for (int a = 0; a < NC; ++a) shM[a][t] = rho * m[a];
  }
  __syncthreads();
  const uint16_t *lp = lptr + s0 + p;
  const uint16_t *le = lent + patch_ent_off[p];
  for (int i = t; i < ns; i += blockDim.x) {
    double s = 0.0;
    for (int k = lp[i]; k < lp[i + 1]; ++k) {
      const int ent = le[k];
      s += shM[ent % NC][ent / NC];
    }
    sM[s0 + i] = s;
  }
}

__global__ void k_gather_mass(const int *slot_off, const int *slots, const double *sM,
                              long long N, double *mass) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double s = 0.0;
  for (int k = slot_off[n]; k < slot_off[n + 1]; ++k) s += sM[slots[k]];
  mass[n] = s;
}

__global__ void k_fill_u64(unsigned long long *p, unsigned long long v, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// ------------------------------------------------------------------------
struct EngineBase {
  virtual ~EngineBase() = default;
};

}  // namespace ftgpu

using namespace ftgpu;

struct ftgpu_model {
  int device = 0;
  int precision = FTGPU_MIXED;
  cudaStream_t stream = nullptr;
  // host inputs (reference layout)
  int nNodes = 0, nE = 0, nPID = 0;
  std::vector<double> X;
  std::vector<int> eptr, conn, etype, pid, materialID;
  std::vector<double> props, fiber;
  std::vector<int> dof_fn;
  std::vector<BcFn> fns;
  int ninst = 1;
  std::vector<int> node_off;
  std::vector<InstParams> inst;
  bool inst_set = false;
  int patch_elems = 0;
  int node_threads = 128;  // nodal block (4M block: 0.834 ms/step against 0.839 at 256)
  bool setup_done = false, init_done = false;
  PatchSet ps;
  // per group: material 0 (rigid, zero stress) with every node of every
  // element fully constrained -- zero force and no stable-dt contribution,
  // so the loop's force and dt passes skip it (its force slots stay zero)
  std::vector<char> group_idle;
  std::vector<int> gp_off;  // reference Gauss-point offset of each element
  long long ngp_total = 0;
  long long S = 0;
  std::vector<double> mass_host;
  std::vector<double> t0_state;  // pending initial state
  double t0 = 0.0;
  // device buffers
  DBuf patch_elem_off, patch_node_off, patch_inst, patch_ent_off, lptr, lent, lconn, epid, fib;
  DBuf sX, sU, sF, mats;
  std::vector<std::unique_ptr<DBuf>> hist;
  std::vector<std::unique_ptr<DBuf>> geo;  // per C3D8 group: Gauss-point A^{-1}, det A
  DBuf clock, dtmin, err, instp;
  DBuf stepsc, rottrig;  // per-instance step scalars / rotation trigonometry
  DBuf stage;            // AoS staging of host <-> device state copies (u, v, a)
  cudaStream_t cstream[3] = {};   // copy streams of the three state arrays
  cudaEvent_t cev[3] = {};
  // injury criteria of the brain drivers (single instance only)
  bool injury_on = false;
  int inj_n = 0;
  std::vector<int> inj_upos;  // compact index -> position in the caller's list
  std::vector<int> inj_group_n;  // listed elements per group (groups with none are skipped)
  DBuf inj_cidx, inj_upos_d, inj_eref, inj_ps_old, inj_psxsr, inj_flags, inj_part, inj_part2,
      inj_done, inj_state, inj_hist;
  // energy balance of the explicit loop (CheckEnergy), single instance only
  bool energy_on = false;
  DBuf du, fprev, epart, estate;
  // rigid bodies driven by sampled accelerations, per instance
  struct RigidHost {
    bool on = false;
    std::vector<double> tab[6];  // times then values of each channel
    double c[3] = {0.0, 0.0, 0.0};
  };
  std::vector<RigidHost> rigid;
  bool rigid_on = false;
  DBuf rb, rbtab, rbstate, rbstep;
  DBuf rig_list;                // driven nodes: a rigid-body or rigid-rotation DOF
  std::vector<int> rig_host;
  // from the boundary table (upload_bc): nodes with a rigid-body or
  // rigid-rotation DOF, and the nodes with a rigid-body DOF
  std::vector<int> drv_nodes, rigid_nodes;
  long long rig_nodes = 0;
  cudaStream_t stream2 = nullptr;  // the driven-node branch of a step
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // models with several element groups: every second group's pass runs on
  // gstream beside the others (disjoint patches and slots; the dt minimum
  // and the error word are atomics), so a small group's partial last wave
  // fills with the next group's blocks
  cudaStream_t gstream = nullptr;
  cudaEvent_t ev_gfork = nullptr, ev_gjoin = nullptr;
  DBuf slot_off, slots, slot4, slot4b, node_inst, nbc, fnsbuf;
  // mixed-precision node pass split: k_node_free over every node not marked
  // kNodeRest in nkind, k_node_step over rest_list (the marked ones)
  std::vector<int> slot4_host;
  int node_split = 1;         // ftgpu_set_node_split
  std::vector<int> fn_owner;  // instance owning each boundary function, -1 none / shared
  DBuf nkind, fnval, rest_list;
  long long rest_n = 0;
  DBuf dX, u, v, a, vh, mass, minv, fi;
  DBuf gpF, gpJ, gpS;
  // graph of one chunk of steps (plain, and with timing events): the first
  // chunk of a run opens with the half-step of ex9.cpp:109-138 from (u, v,
  // a); the chunks after it continue from the half-step state the previous
  // one left (cont_exec)
  cudaGraphExec_t chunk_exec = nullptr, cont_exec = nullptr;
  int chunk_steps = 0;
  // shorter graphs of 2, 4, ..., 14 steps (index steps / 2) for the end of a
  // run, so that a run of any length launches no steps past its limit: with
  // the opening half-step (a run shorter than a chunk) and without it
  cudaGraphExec_t tail_exec[8] = {}, tailc_exec[8] = {};
  cudaGraphExec_t prof_exec = nullptr;
  int prof_steps = 0;
  std::vector<cudaEvent_t> prof_ev;
  Clock *h_clock = nullptr;  // pinned
  int *h_err = nullptr;
  // learned surrogate for material-7 groups
  ftgpu_surrogate *surr = nullptr;
  SurrogateLaw surr_law{};
  DBuf surr_x, surr_y;                // [gp][16] BF16, [gp][8] FP32
  std::vector<long long> surr_base;   // per group: first Gauss point in the buffers
  ~ftgpu_model() {
    if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
    if (cont_exec) cudaGraphExecDestroy(cont_exec);
    for (cudaGraphExec_t &e : tail_exec)
      if (e) cudaGraphExecDestroy(e);
    for (cudaGraphExec_t &e : tailc_exec)
      if (e) cudaGraphExecDestroy(e);
    if (prof_exec) cudaGraphExecDestroy(prof_exec);
    for (cudaEvent_t e : prof_ev) cudaEventDestroy(e);
    if (h_clock) cudaFreeHost(h_clock);
    if (h_err) cudaFreeHost(h_err);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (stream2) cudaStreamDestroy(stream2);
    if (ev_gfork) cudaEventDestroy(ev_gfork);
    if (ev_gjoin) cudaEventDestroy(ev_gjoin);
    if (gstream) cudaStreamDestroy(gstream);
    for (int k = 0; k < 3; ++k) {
      if (cev[k]) cudaEventDestroy(cev[k]);
      if (cstream[k]) cudaStreamDestroy(cstream[k]);
    }
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

bool is_fp64(const ftgpu_model *m) { return m->precision == FTGPU_FP64; }

// Captured graphs bake in buffer pointers and BC tables: drop them whenever those change.
void drop_graphs(ftgpu_model *m) {
  if (m->chunk_exec) cudaGraphExecDestroy(m->chunk_exec);
  if (m->cont_exec) cudaGraphExecDestroy(m->cont_exec);
  for (cudaGraphExec_t &e : m->tail_exec) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
  }
  for (cudaGraphExec_t &e : m->tailc_exec) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
  }
  if (m->prof_exec) cudaGraphExecDestroy(m->prof_exec);
  m->chunk_exec = m->cont_exec = m->prof_exec = nullptr;
  m->chunk_steps = m->prof_steps = 0;
}

int max_patch(const ftgpu_model *m) {
  int pe = m->patch_elems > 0 ? m->patch_elems : 128;
  if (is_fp64(m)) pe = std::min(pe, 128);
  return std::max(32, std::min(pe, kMaxPatchElems));
}

template <class R>
ElemArgs<R> elem_args(ftgpu_model *m, const PatchGroup &g, int gi) {
  ElemArgs<R> A;
  memset(&A, 0, sizeof(A));
  A.patch_elem_off = m->patch_elem_off.as<int>();
  A.patch_node_off = m->patch_node_off.as<int>();
  A.patch_inst = m->patch_inst.as<int>();
  A.patch_ent_off = m->patch_ent_off.as<int>();
  A.lptr = m->lptr.as<uint16_t>();
  A.lent = m->lent.as<uint16_t>();
  A.lconn = m->lconn.as<uint16_t>() + m->ps.group_lconn_off[gi];
  A.epid = m->epid.as<int>();
  A.fib = m->fib.as<R>();
  A.sX = m->sX.as<R>();
  A.sU = m->sU.as<R>();
  A.sF = m->sF.as<R>();
  A.hist = m->hist[gi] ? m->hist[gi]->as<R>() : nullptr;
  A.geo = gi < (int)m->geo.size() && m->geo[gi] ? m->geo[gi]->as<R>() : nullptr;
  A.mats = m->mats.as<MatP<R>>();
  A.clock = m->clock.as<Clock>();
  A.dtmin = m->dtmin.as<unsigned long long>();
  A.err = m->err.as<int>();
  A.gpF = m->gpF.as<double>();
  A.gpJ = m->gpJ.as<double>();
  A.gpS = m->gpS.as<double>();
  A.S = m->S;
  A.E = m->nE;
  A.ninst = m->ninst;
  A.parity = 0;
  A.patch_begin = g.patch_begin;
  A.npatch = g.npatch;
  A.elem_begin = g.elem_begin;
  A.nelem = g.nelem;
  A.use_clock = 1;
  A.dt_direct = 0.0;
  long long gpb = 0;
  for (int k = 0; k < gi; ++k) gpb += (long long)m->ps.groups[k].nelem * (m->ps.groups[k].etype == 0 ? 8 : 1);
  A.gpbase = gpb;
  A.surr_x = nullptr;
  A.surr_y = nullptr;
  A.law = m->surr_law;
  return A;
}

NodeArgs node_args(ftgpu_model *m, int mode, int parity) {
  NodeArgs A;
  memset(&A, 0, sizeof(A));
  A.slot_off = m->slot_off.as<int>();
  A.slots = m->slots.as<int>();
  A.slot4 = m->slot4.as<int4>();
  A.slot4b = m->slot4b.p ? m->slot4b.as<int4>() : nullptr;
  A.node_inst = m->ninst > 1 ? m->node_inst.as<int>() : nullptr;
  A.nbc = m->nbc.as<int16_t>();
  A.nkind = m->nkind.p ? m->nkind.as<uint8_t>() : nullptr;
  A.fnval = m->nkind.p ? m->fnval.as<double2>() : nullptr;
  A.nfns = (int)m->fns.size();
  A.fns = m->fnsbuf.as<BcFn>();
  A.X = m->dX.as<double>();
  A.u = m->u.as<double>();
  A.v = m->v.as<double>();
  A.a = m->a.as<double>();
  A.vh = m->vh.as<double>();
  A.mass = m->mass.as<double>();
  A.minv = m->minv.as<float>();
  A.sF = m->sF.p;
  A.sU = m->sU.p;
  A.clock = m->clock.as<Clock>();
  A.dtmin = m->dtmin.as<unsigned long long>();
  A.inst = m->instp.as<InstParams>();
  A.err = m->err.as<int>();
  A.fi_out = m->fi.as<double>();
  A.N = m->nNodes;
  A.S = m->S;
  A.ninst = m->ninst;
  A.parity = parity;
  A.mode = mode;
  A.fp64 = is_fp64(m) ? 1 : 0;
  A.nrot = 0;
  for (size_t i = 0; i < m->fns.size() && A.nrot < kMaxRotFns; ++i)
    if (m->fns[i].kind == kBckRot) A.rot_ids[A.nrot++] = (int)i;
  A.stepsc = m->stepsc.as<StepScalars>();
  A.rottrig = m->rottrig.as<double>();
  if (m->rigid_on) {
    A.rb = m->rb.as<RigidBody>();
    A.rbtab = m->rbtab.as<double>();
    A.rbstate = m->rbstate.as<RigidState>();
    A.rbstep = m->rbstep.as<RigidStep>();
  }
  if (m->energy_on) {
    A.du = m->du.p;
    A.fprev = m->fprev.p;
    A.epart = m->epart.as<double>();
    A.energy = m->estate.as<EnergyState>();
  }
  return A;
}

template <class R, bool EN>
void node_step_launch(long long nb, int th, cudaStream_t st, const NodeArgs &A) {
  if (A.node_list)
    k_node_step<R, EN, true><<<(unsigned)nb, th, 0, st>>>(A);
  else
    k_node_step<R, EN, false><<<(unsigned)nb, th, 0, st>>>(A);
}

int launch_node(ftgpu_model *m, int mode, int parity) {
  NodeArgs A = node_args(m, mode, parity);
  const int th = m->node_threads;
  long long nb = (m->nNodes + th - 1) / th;
  const bool step = mode == kNodeFused || mode == kNodeFinish;
  const bool en = step && m->energy_on;
  const bool f64 = is_fp64(m);
  auto node_step = [&](long long blocks, cudaStream_t st, const NodeArgs &B) {
    if (f64)
      en ? node_step_launch<double, true>(blocks, th, st, B)
         : node_step_launch<double, false>(blocks, th, st, B);
    else
      en ? node_step_launch<float, true>(blocks, th, st, B)
         : node_step_launch<float, false>(blocks, th, st, B);
  };
  const bool fork = step && m->rig_nodes > 0 && m->stream2;
  if (step) {  // (with the fork, the rotation trigonometry moves to k_driven_step)
    NodeArgs S = A;
    if (fork) S.nrot = 0;
    const long long nth = std::max<long long>(m->ninst, A.nkind ? (long long)m->fns.size() : 0);
    k_step_scalars<<<(unsigned)((nth + 127) / 128), 128, 0, m->stream>>>(S);
  }
  if (fork) {
    // fork: the driven nodes' motion (rigid bodies' integrator, rotation
    // trigonometry) and then those nodes on the second stream, every other
    // node on the first; join before what follows
    const long long nbr = (m->rig_nodes + th - 1) / th;
    NodeArgs B = A;
    B.node_list = m->rig_list.as<int>();
    B.nlist = m->rig_nodes;
    B.epart_off = nb;
    A.skip_driven = 1;
    CK(cudaEventRecord(m->ev_fork, m->stream));
    CK(cudaStreamWaitEvent(m->stream2, m->ev_fork, 0));
    k_driven_step<<<(unsigned)m->ninst, 32, 0, m->stream2>>>(B);
    node_step(nbr, m->stream2, B);
    if (!f64 && !en && A.nkind) {  // every other node: the split, as below
      k_node_free<<<(unsigned)nb, th, 0, m->stream>>>(A);
      if (m->rest_n > 0) {
        NodeArgs C = A;
        C.node_list = m->rest_list.as<int>();
        C.nlist = m->rest_n;
        node_step((m->rest_n + th - 1) / th, m->stream, C);
      }
    } else {
      node_step(nb, m->stream, A);
    }
    CK(cudaEventRecord(m->ev_join, m->stream2));
    CK(cudaStreamWaitEvent(m->stream, m->ev_join, 0));
    nb += nbr;
  } else if (step) {
    if (m->rigid_on) {  // records without driven nodes: the state still advances
      NodeArgs S = A;
      S.nrot = 0;
      k_driven_step<<<(unsigned)m->ninst, 32, 0, m->stream>>>(S);
    }
    if (!f64 && !en && A.nkind) {
      // free nodes on their lean kernel, the rest through k_node_step's list
      k_node_free<<<(unsigned)nb, th, 0, m->stream>>>(A);
      if (m->rest_n > 0) {
        NodeArgs B = A;
        B.node_list = m->rest_list.as<int>();
        B.nlist = m->rest_n;
        node_step((m->rest_n + th - 1) / th, m->stream, B);
      }
    } else {
      node_step(nb, m->stream, A);
    }
  } else {
    if (mode == kNodeBegin && m->rigid_on)
      k_rigid_begin<<<(unsigned)m->ninst, 32, 0, m->stream>>>(A);
    if (f64)
      k_node<double><<<(unsigned)nb, th, 0, m->stream>>>(A);
    else
      k_node<float><<<(unsigned)nb, th, 0, m->stream>>>(A);
  }
  if (en) k_energy_reduce<<<1, 1024, 0, m->stream>>>(A, (int)nb);
  return (int)cudaGetLastError();
}

template <class R>
int launch_groups_t(ftgpu_model *m, int parity, int use_clock, double dt_direct, int gp,
                    int dt_only) {
  const int PE = max_patch(m);
  auto active = [&](size_t gi) {
    return m->ps.groups[gi].npatch > 0 &&
           !(gp != kLaunchGaussPoints && gi < m->group_idle.size() && m->group_idle[gi]);
  };
  int nact = 0;
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi) nact += active(gi) ? 1 : 0;
  const bool split = nact > 1 && m->gstream;
  if (split) {
    CK(cudaEventRecord(m->ev_gfork, m->stream));
    CK(cudaStreamWaitEvent(m->gstream, m->ev_gfork, 0));
  }
  int k = 0;  // active groups so far
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi) {
    const PatchGroup &g = m->ps.groups[gi];
    if (!active(gi)) continue;
    cudaStream_t st = split && (k++ & 1) ? m->gstream : m->stream;
    ElemArgs<R> A = elem_args<R>(m, g, (int)gi);
    A.parity = parity;
    // the injury criteria ride on the force pass of groups with listed elements
    int mode = gp;
    if (gp == kLaunchInjury) {
      if (dt_only == kPassForce && m->injury_on && m->inj_group_n[gi] > 0) {
        A.inj_cidx = m->inj_cidx.as<int>();
        A.inj_upos = m->inj_upos_d.as<int>();
        A.inj_flags = m->inj_flags.as<uint8_t>();
        A.inj_ps_old = m->inj_ps_old.as<R>();
        A.inj_psxsr = m->inj_psxsr.as<R>();
        A.inj_part = m->inj_part.p;
      } else {
        mode = kLaunchPlain;
      }
    }
    A.use_clock = use_clock;
    A.dt_direct = dt_direct;
    const size_t smem = elem_smem_bytes_host<R>(g.etype, PE);
    if (m->surr && g.mat == 7 && dt_only == kPassForce && sizeof(R) == 4) {
      // surrogate: features of every Gauss point, one fused MLP pass, then
      // the force pass reading the network outputs
      const long long base = m->surr_base[gi];
      const long long ngp = (long long)g.nelem * (g.etype == 0 ? 8 : 1);
      A.surr_x = m->surr_x.as<uint16_t>() + base * kMlpIn;
      int r = launch_elem<R>(g.etype, g.mat, 0, g.npatch, PE, smem, st, A,
                             kPassSurrogateFeatures);
      if (r) return r;
      r = surrogate_infer(m->surr, A.surr_x, ngp, m->surr_y.as<float>() + base * kMlpOut,
                          st, m->err.as<int>());
      if (r) return r;
      A.surr_x = nullptr;
      A.surr_y = m->surr_y.as<float>() + base * kMlpOut;
    }
    int r = launch_elem<R>(g.etype, g.mat, mode, g.npatch, PE, smem, st, A, dt_only);
    if (r) return r;
  }
  if (split) {
    CK(cudaEventRecord(m->ev_gjoin, m->gstream));
    CK(cudaStreamWaitEvent(m->stream, m->ev_gjoin, 0));
  }
  return 0;
}

int launch_groups(ftgpu_model *m, int parity, int use_clock, double dt_direct, int gp,
                  int dt_only) {
  return is_fp64(m) ? launch_groups_t<double>(m, parity, use_clock, dt_direct, gp, dt_only)
                    : launch_groups_t<float>(m, parity, use_clock, dt_direct, gp, dt_only);
}

int fill_dtmin(ftgpu_model *m) {
  k_fill_u64<<<(2 * m->ninst + 255) / 256, 256, 0, m->stream>>>(
      m->dtmin.as<unsigned long long>(), kDtHugeBits, 2 * m->ninst);
  return (int)cudaGetLastError();
}

// Host arrays are AoS [node*3 + d] (the reference's layout), device state is
// SoA [3][N]: the transpose runs on the device through a staging buffer, and
// the host copy is one contiguous cudaMemcpyAsync straight from / into the
// caller's array (full link bandwidth when the caller's memory is pinned).
__global__ void k_aos_to_soa(const double *aos, double *soa, long long N) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) soa[k * N + n] = aos[3 * n + k];
}
__global__ void k_soa_to_aos(const double *soa, double *aos, long long N) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) aos[3 * n + k] = soa[k * N + n];
}

int ensure_stage(ftgpu_model *m) {
  const size_t b = 3 * (size_t)m->nNodes * sizeof(double);
  if (m->stage.bytes >= b) return 0;
  return m->stage.alloc(b);
}

// Staging for the three state arrays at once, with a copy stream each.
int ensure_stage3(ftgpu_model *m) {
  const size_t b = 9 * (size_t)m->nNodes * sizeof(double);
  if (m->stage.bytes < b) CKI(m->stage.alloc(b));
  for (int k = 0; k < 3; ++k) {
    if (!m->cstream[k]) CK(cudaStreamCreateWithFlags(&m->cstream[k], cudaStreamNonBlocking));
    if (!m->cev[k]) CK(cudaEventCreateWithFlags(&m->cev[k], cudaEventDisableTiming));
  }
  return 0;
}

// u, v, a between AoS host arrays and the SoA device state in one call: each
// array has its own staging third and copy stream, so the three host <->
// device copies run side by side and overlap the transposes (which run on
// the model's stream).  (Kernels reading or writing page-locked host arrays
// in place through their mapping measured slower: 1.8 / 5.4 ms against
// 1.5 / 1.6 ms for the 4M-node block's three arrays.)  Null host arrays:
// zero (upload) / not read (download).
int upload_state3(ftgpu_model *m, const double *const h[3], DBuf *const d[3]) {
  const long long N = m->nNodes;
  CKI(ensure_stage3(m));
  CK(cudaEventRecord(m->cev[0], m->stream));  // the state is free to overwrite
  for (int k = 0; k < 3; ++k) {
    if (!h[k]) continue;
    double *st = m->stage.as<double>() + 3 * N * k;
    CK(cudaStreamWaitEvent(m->cstream[k], m->cev[0], 0));
    CK(cudaMemcpyAsync(st, h[k], 3 * N * sizeof(double), cudaMemcpyHostToDevice, m->cstream[k]));
  }
  for (int k = 0; k < 3; ++k) {
    if (!h[k]) {
      CK(cudaMemsetAsync(d[k]->p, 0, 3 * N * sizeof(double), m->stream));
      continue;
    }
    CK(cudaEventRecord(m->cev[k], m->cstream[k]));
    CK(cudaStreamWaitEvent(m->stream, m->cev[k], 0));
    k_aos_to_soa<<<(unsigned)((N + 255) / 256), 256, 0, m->stream>>>(
        m->stage.as<double>() + 3 * N * k, d[k]->as<double>(), N);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(m->stream));
  return 0;
}

int download_state3(ftgpu_model *m, DBuf *const d[3], double *const h[3]) {
  const long long N = m->nNodes;
  CKI(ensure_stage3(m));
  bool staged[3] = {false, false, false};
  for (int k = 0; k < 3; ++k) {
    if (!h[k]) continue;
    k_soa_to_aos<<<(unsigned)((N + 255) / 256), 256, 0, m->stream>>>(
        d[k]->as<double>(), m->stage.as<double>() + 3 * N * k, N);
    CK(cudaGetLastError());
    CK(cudaEventRecord(m->cev[k], m->stream));
    CK(cudaStreamWaitEvent(m->cstream[k], m->cev[k], 0));
    CK(cudaMemcpyAsync(h[k], m->stage.as<double>() + 3 * N * k, 3 * N * sizeof(double),
                       cudaMemcpyDeviceToHost, m->cstream[k]));
    staged[k] = true;
  }
  CK(cudaStreamSynchronize(m->stream));
  for (int k = 0; k < 3; ++k)
    if (staged[k]) CK(cudaStreamSynchronize(m->cstream[k]));
  return 0;
}

// AoS [3N] host -> SoA [3][N] device (h == NULL: zero)
int upload_aos(ftgpu_model *m, const double *h, DBuf &d) {
  const long long N = m->nNodes;
  if (!h) {
    CK(cudaMemsetAsync(d.p, 0, 3 * N * sizeof(double), m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return 0;
  }
  CKI(ensure_stage(m));
  CK(cudaMemcpyAsync(m->stage.p, h, 3 * N * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  k_aos_to_soa<<<(unsigned)((N + 255) / 256), 256, 0, m->stream>>>(m->stage.as<double>(),
                                                                    d.as<double>(), N);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(m->stream));
  return 0;
}

int download_aos(ftgpu_model *m, const DBuf &d, double *h) {
  if (!h) return 0;
  const long long N = m->nNodes;
  CKI(ensure_stage(m));
  k_soa_to_aos<<<(unsigned)((N + 255) / 256), 256, 0, m->stream>>>(d.as<double>(),
                                                                    m->stage.as<double>(), N);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h, m->stage.p, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  return 0;
}

// Reference layout and principal strains of the averaged Green strain of
// each element (CalculateStrain.cpp:38-74, FP64): out per element = Eavg
// column-major 3x3, max principal strain clamped >= 0, min clamped <= 0,
// max shear (max - min) / 2 of the unclamped extremes.
__global__ void k_principal_strain(const double *E6, long long nE, double *out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nE) return;
  const double xx = E6[6 * i], yy = E6[6 * i + 1], zz = E6[6 * i + 2];
  const double yz = E6[6 * i + 3], xz = E6[6 * i + 4], xy = E6[6 * i + 5];
  double *o = out + 12 * i;
  o[0] = xx; o[1] = xy; o[2] = xz;
  o[3] = xy; o[4] = yy; o[5] = yz;
  o[6] = xz; o[7] = yz; o[8] = zz;
  const double a = xx, b = xy, c = xz, d = yy, e = yz, f = zz;
  const double p1 = b * b + c * c + e * e;
  double e1, e2, e3;
  if (p1 == 0) {
    e1 = a;
    e2 = d;
    e3 = f;
  } else {  // trigonometric roots of x^3 - I1 x^2 + I2 x - I3 (as the reference)
    double I1 = a + d + f;
    const double I2 = a * (d + f) + d * f - b * b - c * c - e * e;
    const double I3 = a * d * f + 2.0 * b * c * e - b * b * f - c * c * d - e * e * a;
    const double Q = (3.0 * I2 - I1 * I1) / 9.0;
    const double R = (2.0 * I1 * I1 * I1 - 9.0 * I1 * I2 + 27.0 * I3) / 54.0;
    const double theta = acos(R / sqrt(-Q * Q * Q));
    const double sq = 2.0 * sqrt(-Q);
    const double kPi = 3.141592653589793;
    I1 = I1 / 3.0;
    e1 = sq * cos(theta / 3.0) + I1;
    e2 = sq * cos((theta + 2.0 * kPi) / 3.0) + I1;
    e3 = sq * cos((theta + 4.0 * kPi) / 3.0) + I1;
  }
  const double mx = fmax(e3, fmax(e2, e1)), mn = fmin(e3, fmin(e2, e1));
  o[9] = mx > 0.0 ? mx : 0.0;
  o[10] = mn < 0.0 ? mn : 0.0;
  o[11] = 0.5 * (mx - mn);
}

template <class R>
int strain_groups_t(ftgpu_model *m, double *E6) {
  const int PE = max_patch(m);
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi) {
    const PatchGroup &g = m->ps.groups[gi];
    const ElemArgs<R> A = elem_args<R>(m, g, (int)gi);
    const size_t smem = strain_smem_bytes_host<R>();
    const int r = launch_strain<R>(g.etype, g.npatch, PE, smem, m->stream, A, E6);
    if (r) return fail(FTGPU_ERR_CUDA, std::string("element strain pass: ") +
                                           cudaGetErrorString((cudaError_t)r));
  }
  return 0;
}

int check_err(ftgpu_model *m) {
  CK(cudaMemcpyAsync(m->h_err, m->err.p, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  int e = *m->h_err;
  if (e & kErrInverted) return fail(FTGPU_ERR_INVERTED, "non-positive or non-finite Jacobian");
  if (e & kErrIndex) return fail(FTGPU_ERR_INPUT, "local node index out of range");
  if (e & kErrWait) return fail(FTGPU_ERR_CUDA, "tensor-core inference gave up waiting");
  return 0;
}

// Per-element part word: part | (1 << 31) when every node of the element has
// all three DOFs constrained (skipped by StableTimeStep.cpp:13-19).
int upload_epid(ftgpu_model *m, bool zero_idle) {
  std::vector<int> w(m->nE);
  for (int ge = 0; ge < m->nE; ++ge) {
    const int e = m->ps.elem_order[ge];
    bool active = false;
    for (int k = m->eptr[e]; k < m->eptr[e + 1]; ++k) {
      const int n = m->conn[k];
      bool all = true;
      for (int d = 0; d < 3; ++d)
        if (m->dof_fn.empty() || m->dof_fn[3 * n + d] == FTGPU_BC_FREE) all = false;
      if (!all) {
        active = true;
        break;
      }
    }
    w[ge] = m->pid[e] | (active ? 0 : (int)0x80000000u);
  }
  m->group_idle.assign(m->ps.groups.size(), 0);
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi) {
    const PatchGroup &g = m->ps.groups[gi];
    if (g.mat != 0 || g.npatch == 0) continue;
    bool idle = true;
    for (int ge = g.elem_begin; ge < g.elem_begin + g.nelem && idle; ++ge)
      idle = (w[ge] & (int)0x80000000u) != 0;
    m->group_idle[gi] = idle ? 1 : 0;
    if (idle && zero_idle) {  // its slots may hold forces of an earlier BC table
      const size_t rb = is_fp64(m) ? sizeof(Slot4<double>) : sizeof(Slot4<float>);
      const long long s0 = m->ps.patch_node_off[g.patch_begin];
      const long long s1 = m->ps.patch_node_off[g.patch_begin + g.npatch];
      CK(cudaMemsetAsync((char *)m->sF.p + s0 * rb, 0, (s1 - s0) * rb, m->stream));
    }
  }
  return m->epid.upload(w.data(), w.size());
}

// The instance of every node (empty node_off: one instance).
static int instance_of(const ftgpu_model *m, long long n) {
  if (m->node_off.size() < 2) return 0;
  return (int)(std::upper_bound(m->node_off.begin(), m->node_off.end(), (int)n) -
               m->node_off.begin()) - 1;
}

// The split of the mixed-precision node pass: k_node_free takes every node
// whose constrained DOFs (if any) follow a fixed / ramp / sine function owned
// by one instance (its value at the new time is evaluated once per step by
// k_step_scalars, which also advances the instances' clocks) or hold; a node
// without slots and a node with a rigid-rotation or rigid-body DOF go to
// k_node_step over rest_list.
int upload_split(ftgpu_model *m) {
  const long long N = m->nNodes;
  m->nkind.release();
  m->rest_list.release();
  m->rest_n = 0;
  if (is_fp64(m) || !m->node_split || (long long)m->slot4_host.size() != 4 * N) return 0;
  std::vector<uint8_t> kind(N, 0);
  if (!m->dof_fn.empty())
    for (long long n = 0; n < N; ++n)
      for (int d = 0; d < 3; ++d) {
        const int f = m->dof_fn[3 * n + d];
        if (f == FTGPU_BC_FREE) continue;
        kind[n] |= kNodeBcCached;
        if (f >= 0 && (m->fns[f].kind > kBckSine || m->fn_owner[f] < 0)) kind[n] |= kNodeRest;
      }
  // the rest list leaves out the driven nodes: the driven-node branch of
  // the step (a second stream) updates them
  std::vector<char> drv(N, 0);
  for (const int n : m->drv_nodes) drv[n] = 1;
  std::vector<int> list;
  for (long long n = 0; n < N; ++n) {
    if (m->slot4_host[4 * n] == -1) kind[n] |= kNodeRest;  // no slots
    if ((kind[n] & kNodeRest) && !drv[n]) list.push_back((int)n);
  }
  CKI(m->nkind.upload(kind.data(), kind.size()));
  CKI(m->fnval.alloc(std::max<size_t>(m->fns.size(), 1) * sizeof(double2)));
  m->rest_n = (long long)list.size();
  if (!list.empty()) CKI(m->rest_list.upload(list.data(), list.size()));
  return 0;
}

int upload_bc(ftgpu_model *m) {
  const long long N = m->nNodes;
  std::vector<int16_t> nb(3 * N, (int16_t)FTGPU_BC_FREE);
  if (!m->dof_fn.empty())
    for (long long n = 0; n < N; ++n)
      for (int d = 0; d < 3; ++d) nb[d * N + n] = (int16_t)m->dof_fn[3 * n + d];
  int r = m->nbc.upload(nb.data(), nb.size());
  if (r) return r;
  // driven nodes (a rigid-body or rigid-rotation DOF), once per table
  m->drv_nodes.clear();
  m->rigid_nodes.clear();
  if (!m->dof_fn.empty())
    for (long long n = 0; n < N; ++n) {
      bool drv = false, rgd = false;
      for (int d = 0; d < 3; ++d) {
        const int f = m->dof_fn[3 * n + d];
        if (f < 0) continue;
        drv |= m->fns[f].kind == kBckRigid || m->fns[f].kind == kBckRot;
        rgd |= m->fns[f].kind == kBckRigid;
      }
      if (drv) m->drv_nodes.push_back((int)n);
      if (rgd) m->rigid_nodes.push_back((int)n);
    }
  // the instance that owns each function (-1: unused or shared by several)
  m->fn_owner.assign(m->fns.size(), -2);
  if (!m->dof_fn.empty())
    for (long long i = 0; i < 3 * N; ++i) {
      const int fi = m->dof_fn[i];
      if (fi < 0) continue;
      const int o = instance_of(m, i / 3);
      int &w = m->fn_owner[fi];
      w = (w == -2 || w == o) ? o : -1;
    }
  for (int &w : m->fn_owner) w = w < 0 ? -1 : w;
  // pad: a rigid rotation's trigonometry cache slot; a fixed / ramp / sine
  // function's owning instance (its values are evaluated once per step)
  std::vector<BcFn> f = m->fns;
  int slot = 0;
  for (size_t i = 0; i < f.size(); ++i) {
    BcFn &b = f[i];
    if (b.kind == kBckRot)
      b.pad = slot < kMaxRotFns ? slot++ : -1;
    else
      b.pad = b.kind <= kBckSine ? m->fn_owner[i] : -1;
  }
  if (f.empty()) {
    f.resize(1);
    f[0].pad = -1;
  }
  r = m->fnsbuf.upload(f.data(), f.size());
  if (r) return r;
  return upload_split(m);
}

template <class R>
int upload_materials(ftgpu_model *m) {
  std::vector<MatP<R>> t(m->nPID);
  for (int p = 0; p < m->nPID; ++p) {
    const double *pr = &m->props[FTGPU_MAXMATPARAMS * p];
    MatP<R> q;
    memset(&q, 0, sizeof(q));
    for (int k = 0; k < 9; ++k) q.p[k] = R(pr[k]);
    const double mu = pr[1], lambda = pr[2], rho = pr[0];
    q.K = R(lambda + 2.0 * mu / 3.0);
    // CalculateTimeStep.cpp:16-18
    const double nu = 0.5 * lambda / (lambda + mu);
    const double ce = std::sqrt(lambda * (1.0 / nu - 1.0) / rho);
    q.ce = ce;
    q.inv_ce = R(1.0 / ce);
    q.mat = m->materialID[p];
    if (q.mat == 6) {
      // binomial coefficients of (1+x)^(alpha/2-1), powers 1..n
      const double a = pr[3];
      double ba = 1.0;
      for (int k = 0; k < kOgdenSeries; ++k) {
        ba *= (a / 2.0 - 1.0 - k) / (k + 1.0);
        q.ser_a[k] = R(ba);
      }
      // FP32 path: the series while |2E|_F < r, r the largest radius (at most
      // 0.3) whose truncation bound sum_{k > n} |b_a,k| (3 + 2 r) r^k stays
      // below 1e-7 r (FP32 rounding of the leading term; the 1 + 2 (1 + r)
      // weighs A itself and tr B = tr(A + M + M A)); FP64 mode keeps the
      // eigen path
      auto tail = [&](double r) {
        double ca = ba, rk = std::pow(r, kOgdenSeries), t = 0.0;
        for (int k = kOgdenSeries; k < kOgdenSeries + 400; ++k) {
          ca *= (a / 2.0 - 1.0 - k) / (k + 1.0);
          rk *= r;
          t += std::fabs(ca) * (3.0 + 2.0 * r) * rk;
        }
        return t;
      };
      double lo = 0.0, hi = 0.3;
      if (tail(hi) <= 1e-7 * hi) {
        lo = hi;
      } else {
        for (int it = 0; it < 60; ++it) {
          const double mid = 0.5 * (lo + hi);
          (tail(mid) <= 1e-7 * mid ? lo : hi) = mid;
        }
      }
      q.ser_thr2 = sizeof(R) == 4 ? R(lo * lo) : R(0);
    }
    t[p] = q;
  }
  return m->mats.upload(t.data(), t.size());
}

int prepare_graphs(ftgpu_model *m);

template <class R>
int setup_t(ftgpu_model *m) {
  const long long N = m->nNodes;
  const int E = m->nE;
  // element material / instance for grouping
  std::vector<int> emat(E), einst(E, 0), ninst_of(N, 0);
  if (m->ninst > 1)
    for (int i = 0; i < m->ninst; ++i)
      for (int n = m->node_off[i]; n < m->node_off[i + 1]; ++n) ninst_of[n] = i;
  for (int e = 0; e < E; ++e) {
    if (m->pid[e] < 0 || m->pid[e] >= m->nPID) return fail(FTGPU_ERR_INPUT, "pid out of range");
    const int mt = m->materialID[m->pid[e]];
    if (mt < 0 || mt > 7) return fail(FTGPU_ERR_MATERIAL, "unknown material ID");
    emat[e] = mt;
    einst[e] = ninst_of[m->conn[m->eptr[e]]];
    for (int k = m->eptr[e]; k < m->eptr[e + 1]; ++k)
      if (ninst_of[m->conn[k]] != einst[e]) return fail(FTGPU_ERR_INPUT, "element spans instances");
  }
  const int PE = max_patch(m);
  int rc = build_patches((int)N, E, m->X.data(), m->eptr.data(), m->conn.data(), m->etype.data(),
                         emat.data(), einst.data(), PE, kMaxLocalNodes, m->ps);
  if (rc) return fail(FTGPU_ERR_INPUT, "invalid mesh (element type / node count / node index)");
  PatchSet &ps = m->ps;
  const int P = (int)ps.patch_inst.size();
  m->S = (long long)ps.slot_node.size();
  const long long S = m->S;
  CKI(m->patch_elem_off.upload(ps.patch_elem_off.data(), P + 1));
  CKI(m->patch_node_off.upload(ps.patch_node_off.data(), P + 1));
  CKI(m->patch_inst.upload(ps.patch_inst.data(), P));
  CKI(m->patch_ent_off.upload(ps.patch_ent_off.data(), P + 1));
  CKI(m->lptr.upload(ps.lptr.data(), ps.lptr.size()));
  CKI(m->lent.upload(ps.lent.data(), ps.lent.size()));
  CKI(m->lconn.upload(ps.lconn.data(), ps.lconn.size()));
  CKI(m->slot_off.upload(ps.node_slot_off.data(), N + 1));
  CKI(m->slots.upload(ps.node_slots.data(), ps.node_slots.size()));
  {
    // slot records: four slots per node, eight (a second record array) when
    // more than 5 % of the nodes have more than four (tetrahedral meshes)
    long long over4 = 0;
    for (long long n = 0; n < N; ++n) over4 += ps.node_slot_off[n + 1] - ps.node_slot_off[n] > 4;
    const int W = over4 * 20 > N ? 8 : 4;
    std::vector<int> rec(4 * (size_t)N, -1), rec2(W == 8 ? 4 * (size_t)N : 0, -1);
    for (long long n = 0; n < N; ++n) {
      const int b = ps.node_slot_off[n], e = ps.node_slot_off[n + 1];
      if (e - b > W) {
        rec[4 * n] = kSlotCsr;
        continue;
      }
      for (int k = b; k < e; ++k) {
        const int j = k - b;
        (j < 4 ? rec[4 * n + j] : rec2[4 * n + j - 4]) = ps.node_slots[k];
      }
    }
    CKI(m->slot4.upload(rec.data(), rec.size()));
    m->slot4_host = std::move(rec);
    m->slot4b.release();
    if (W == 8) CKI(m->slot4b.upload(rec2.data(), rec2.size()));
  }
  CKI(upload_epid(m, false));  // the force slots are allocated zeroed below
  CKI(upload_materials<R>(m));
  if (m->ps.groups.size() > 1 && !m->gstream) {  // element groups side by side
    CK(cudaStreamCreateWithFlags(&m->gstream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&m->ev_gfork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&m->ev_gjoin, cudaEventDisableTiming));
  }
  // reference coordinates per slot: absolute in FP64 mode, relative to the
  // patch's first node in mixed mode (keeps FP32 digits for element geometry)
  {
    std::vector<R> sx(3 * S);
    for (int p = 0; p < P; ++p) {
      const int s0 = ps.patch_node_off[p], s1 = ps.patch_node_off[p + 1];
      double anc[3] = {0, 0, 0};
      if (!is_fp64(m))
        for (int d = 0; d < 3; ++d) anc[d] = m->X[3 * ps.slot_node[s0] + d];
      for (int s = s0; s < s1; ++s)
        for (int d = 0; d < 3; ++d) sx[d * S + s] = R(m->X[3 * ps.slot_node[s] + d] - anc[d]);
    }
    CKI(m->sX.upload(sx.data(), sx.size()));
  }
  CKI(m->sU.alloc(S * sizeof(Slot4<R>)));
  CK(cudaMemset(m->sU.p, 0, S * sizeof(Slot4<R>)));
  CKI(m->sF.alloc(S * sizeof(Slot4<R>)));
  CK(cudaMemset(m->sF.p, 0, S * sizeof(Slot4<R>)));
  // fibres (material 7), group order, SoA
  bool any7 = false;
  for (auto &g : ps.groups) any7 |= g.mat == 7;
  if (any7) {
    std::vector<R> fb(3 * (size_t)E, R(0));
    for (int ge = 0; ge < E; ++ge) {
      const int e = ps.elem_order[ge];
      double a0[3] = {1, 0, 0};
      if (!m->fiber.empty()) {
        for (int d = 0; d < 3; ++d) a0[d] = m->fiber[3 * e + d];
        double nrm = std::sqrt(a0[0] * a0[0] + a0[1] * a0[1] + a0[2] * a0[2]);
        if (nrm > 0)
          for (int d = 0; d < 3; ++d) a0[d] /= nrm;
      }
      for (int d = 0; d < 3; ++d) fb[d * (size_t)E + ge] = R(a0[d]);
    }
    CKI(m->fib.upload(fb.data(), fb.size()));
  }
  // viscoelastic history per group: [ncomp][NGP][nelem], zero
  m->hist.clear();
  for (auto &g : ps.groups) {
    int nc = g.mat == 5 ? 18 : (g.mat == 7 ? 12 : 0);
    if (nc == 0) {
      m->hist.emplace_back(nullptr);
      continue;
    }
    const size_t n = (size_t)nc * (g.etype == 0 ? 8 : 1) * g.nelem;
    auto b = std::make_unique<DBuf>();
    CKI(b->alloc(n * sizeof(R)));
    CK(cudaMemset(b->p, 0, n * sizeof(R)));
    m->hist.push_back(std::move(b));
  }
  // reference Gauss-point offsets (gpPtr of ShapeFunctions.cpp:64-165)
  m->gp_off.assign(E + 1, 0);
  for (int e = 0; e < E; ++e) m->gp_off[e + 1] = m->gp_off[e] + (m->etype[e] == 0 ? 8 : 1);
  m->ngp_total = m->gp_off[E];
  // nodal state
  {
    std::vector<double> xs(3 * N);
    for (long long n = 0; n < N; ++n)
      for (int d = 0; d < 3; ++d) xs[d * N + n] = m->X[3 * n + d];
    CKI(m->dX.upload(xs.data(), xs.size()));
  }
  for (DBuf *b : {&m->u, &m->v, &m->a, &m->vh, &m->fi}) {
    CKI(b->alloc(3 * N * sizeof(double)));
    CK(cudaMemset(b->p, 0, 3 * N * sizeof(double)));
  }
  CKI(upload_bc(m));
  // instances
  if (!m->inst_set) {
    m->ninst = 1;
    m->node_off = {0, (int)N};
    m->inst.assign(1, InstParams{1e300, 0.9, 0.0, 0, 0, 0});
  }
  if (m->ninst > 1) {
    std::vector<int> ni(N);
    for (int i = 0; i < m->ninst; ++i)
      for (int n = m->node_off[i]; n < m->node_off[i + 1]; ++n) ni[n] = i;
    CKI(m->node_inst.upload(ni.data(), N));
  }
  for (int i = 0; i < m->ninst; ++i) m->inst[i].node_begin = m->node_off[i];
  CKI(m->instp.upload(m->inst.data(), m->ninst));
  CKI(upload_bc(m));  // function owners and the node-pass split need the instances
  std::vector<Clock> ck(2 * m->ninst);
  for (auto &c : ck) c = Clock{0.0, 0.0, 0, 0, 0};
  CKI(m->clock.upload(ck.data(), ck.size()));
  CKI(m->dtmin.alloc(2 * m->ninst * sizeof(unsigned long long)));
  CKI(m->stepsc.alloc(m->ninst * sizeof(StepScalars)));
  CKI(m->rottrig.alloc((size_t)m->ninst * kMaxRotFns * 3 * sizeof(double)));
  CKI(m->err.alloc(sizeof(int)));
  CK(cudaMemset(m->err.p, 0, sizeof(int)));
  // FP32: reference geometry of every C3D8 Gauss point, once (the element
  // passes read it instead of rebuilding A^{-1} from the slot coordinates)
  m->geo.clear();
  if constexpr (sizeof(R) == 4) {
    for (size_t gi = 0; gi < ps.groups.size(); ++gi) {
      const PatchGroup &g = ps.groups[gi];
      if (g.etype != 0 || g.nelem == 0) {
        m->geo.emplace_back(nullptr);
        continue;
      }
      auto b = std::make_unique<DBuf>();
      CKI(b->alloc((size_t)80 * g.nelem * sizeof(float)));
      m->geo.push_back(std::move(b));
      const ElemArgs<float> A = elem_args<float>(m, g, (int)gi);
      CK((cudaError_t)launch_geo_f32(g.npatch, m->stream, A, m->geo.back()->as<float>()));
    }
  }
  CKI(fill_dtmin(m));
  // lumped mass on the device (FP64), replaces AssembleLumpedMass()
  {
    DBuf sM, snode, mpd;
    CKI(sM.alloc(S * sizeof(double)));
    CKI(snode.upload(ps.slot_node.data(), ps.slot_node.size()));
    std::vector<MatP<double>> md(m->nPID);
    for (int p = 0; p < m->nPID; ++p) {
      memset(&md[p], 0, sizeof(md[p]));
      for (int k = 0; k < 9; ++k) md[p].p[k] = m->props[9 * p + k];
    }
    CKI(mpd.upload(md.data(), md.size()));
    for (size_t gi = 0; gi < ps.groups.size(); ++gi) {
      const PatchGroup &g = ps.groups[gi];
      const uint16_t *lc = m->lconn.as<uint16_t>() + ps.group_lconn_off[gi];
      if (g.npatch == 0) continue;
      if (g.etype == 0)
        k_mass<0><<<g.npatch, PE, 0, m->stream>>>(
            m->patch_elem_off.as<int>(), m->patch_node_off.as<int>(), m->patch_ent_off.as<int>(),
            m->lptr.as<uint16_t>(), m->lent.as<uint16_t>(), lc, m->epid.as<int>(),
            snode.as<int>(), m->dX.as<double>(), N, mpd.as<MatP<double>>(), g.patch_begin,
            g.elem_begin, sM.as<double>());
      else
        k_mass<1><<<g.npatch, PE, 0, m->stream>>>(
            m->patch_elem_off.as<int>(), m->patch_node_off.as<int>(), m->patch_ent_off.as<int>(),
            m->lptr.as<uint16_t>(), m->lent.as<uint16_t>(), lc, m->epid.as<int>(),
            snode.as<int>(), m->dX.as<double>(), N, mpd.as<MatP<double>>(), g.patch_begin,
            g.elem_begin, sM.as<double>());
      CK(cudaGetLastError());
    }
    CKI(m->mass.alloc(N * sizeof(double)));
    k_gather_mass<<<(unsigned)((N + 255) / 256), 256, 0, m->stream>>>(
        m->slot_off.as<int>(), m->slots.as<int>(), sM.as<double>(), N, m->mass.as<double>());
    CK(cudaGetLastError());
    m->mass_host.resize(N);
    CK(cudaMemcpyAsync(m->mass_host.data(), m->mass.p, N * sizeof(double), cudaMemcpyDeviceToHost,
                       m->stream));
    CK(cudaStreamSynchronize(m->stream));
    std::vector<float> mi(N);
    for (long long n = 0; n < N; ++n) mi[n] = (float)(1.0 / m->mass_host[n]);
    CKI(m->minv.upload(mi.data(), N));
  }
  if (m->h_clock) cudaFreeHost(m->h_clock);
  m->h_clock = nullptr;
  CK(cudaMallocHost((void **)&m->h_clock, sizeof(Clock) * std::max(2 * m->ninst, 2)));
  if (!m->h_err) CK(cudaMallocHost((void **)&m->h_err, sizeof(int)));
  m->setup_done = true;
  m->init_done = false;
  drop_graphs(m);
  return prepare_graphs(m);
}

int ensure_gp(ftgpu_model *m) {
  const size_t n = (size_t)m->ngp_total;
  if (m->gpJ.bytes >= n * sizeof(double)) return 0;
  CKI(m->gpF.alloc(9 * n * sizeof(double)));
  CKI(m->gpJ.alloc(n * sizeof(double)));
  CKI(m->gpS.alloc(6 * n * sizeof(double)));
  return 0;
}

// One chunk: BEGIN, K x (element groups, node), the last node pass FINISH.
// With prof, event-record nodes bracket every element pass and node pass
// (events 2k / 2k+1 / 2k+2 around step k).
constexpr int kInjHistWords = 2 * 8 * kRadixBins + 2;  // histograms + two counters

template <class R>
InjuryArgs<R> injury_args(ftgpu_model *m, int parity) {
  InjuryArgs<R> A;
  A.cidx = m->inj_cidx.as<int>();
  A.upos = m->inj_upos_d.as<int>();
  A.eref = m->inj_eref.as<int>();
  A.ps_old = m->inj_ps_old.as<R>();
  A.psxsr = m->inj_psxsr.as<R>();
  A.flags = m->inj_flags.as<uint8_t>();
  A.part = m->inj_part.as<InjuryPart>();
  A.part2 = m->inj_part2.as<InjuryPart>();
  A.done_blocks = m->inj_done.as<unsigned>();
  A.state = m->inj_state.as<InjuryState>();
  A.clock = m->clock.as<Clock>();
  A.hist = m->inj_hist.as<unsigned>();
  A.count = A.hist + 2 * 8 * kRadixBins;
  A.n = m->inj_n;
  A.parity = parity;
  int np = 0;
  for (auto &g : m->ps.groups) np += g.npatch;
  A.npart = np;
  return A;
}

// One step of the injury criteria after the element pass (whose force
// launches of groups with listed elements updated the per-element criteria
// and left each block's extremes, launch mode kLaunchInjury): the step's
// extremes (which also clears the histograms), the radix passes of both
// selections, the element lists and the running maxima.  Partials of patches
// without listed elements keep their sentinel values.
template <class R>
int launch_injury_t(ftgpu_model *m, int parity) {
  const InjuryArgs<R> J = injury_args<R>(m, parity);
  k_injury_reduce<R><<<(J.npart + kInjReduceSpan - 1) / kInjReduceSpan, 256, 0, m->stream>>>(J);
  const int hb = std::min((m->inj_n + kInjThreads - 1) / kInjThreads, 512);
  for (int pass = 0; pass < (int)sizeof(R); ++pass)
    k_radix_hist<R><<<dim3(hb, 2), kInjThreads, 0, m->stream>>>(J, pass);
  k_radix_list<R><<<hb, kInjThreads, 0, m->stream>>>(J);
  k_radix_final<R><<<1, kRadixBins, 0, m->stream>>>(J);
  CK(cudaGetLastError());
  return 0;
}

int launch_injury(ftgpu_model *m, int parity) {
  return is_fp64(m) ? launch_injury_t<double>(m, parity) : launch_injury_t<float>(m, parity);
}

// Steps per chunk graph (even: the clock slots alternate with the step
// parity, so a graph of an even number of steps fits any starting step).
constexpr int kChunkSteps = 16;

// A graph of K steps.  open: it starts with the half-step from (u, v, a)
// (kNodeBegin); otherwise it continues from the half-step state that the
// previous graph of the run left.  The steps are all fused (full step, then
// the next half-step): the step that reaches the run's step limit, tmax or a
// failed dt finishes instead (v and a at t_{n+1}, the state a run ends in),
// so a run is a sequence of graphs without a finish / restart at their
// seams.  prof: the timing graph (events around every pass), which opens
// and finishes every chunk.
int capture_chunk(ftgpu_model *m, int K, bool prof, bool open = true) {
  // a tail graph (even K from 2 to 14) is captured once and kept in its slot
  const bool tail = !prof && K < kChunkSteps;
  if (tail && (K < 2 || (K & 1))) return fail(FTGPU_ERR_INPUT, "tail graph of an odd step count");
  if (prof) open = true;
  int tail_steps = K;  // the slot of a tail graph fixes its step count
  cudaGraphExec_t &exec = tail ? (open ? m->tail_exec[K / 2] : m->tailc_exec[K / 2])
                               : prof ? m->prof_exec : open ? m->chunk_exec : m->cont_exec;
  // (the opening and continuing full chunks are both kChunkSteps long)
  int &steps = tail ? tail_steps : prof ? m->prof_steps : m->chunk_steps;
  if (exec && steps == K) return 0;
  if (exec) cudaGraphExecDestroy(exec);
  exec = nullptr;
  if (prof) {
    for (cudaEvent_t e : m->prof_ev) cudaEventDestroy(e);
    m->prof_ev.assign(2 * K + 1, nullptr);
    for (auto &e : m->prof_ev) CK(cudaEventCreate(&e));
  }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  int r = open ? launch_node(m, kNodeBegin, 0) : 0;
  for (int k = 0; k < K && !r; ++k) {
    if (prof) r = (int)cudaEventRecordWithFlags(m->prof_ev[2 * k], m->stream, cudaEventRecordExternal);
    if (!r) r = launch_groups(m, k & 1, 1, 0.0, m->injury_on ? kLaunchInjury : kLaunchPlain, 0);
    if (prof && !r)
      r = (int)cudaEventRecordWithFlags(m->prof_ev[2 * k + 1], m->stream, cudaEventRecordExternal);
    if (!r && m->injury_on) r = launch_injury(m, k & 1);
    if (!r) r = launch_node(m, prof && k == K - 1 ? kNodeFinish : kNodeFused, k & 1);
  }
  if (prof && !r) r = (int)cudaEventRecordWithFlags(m->prof_ev[2 * K], m->stream, cudaEventRecordExternal);
  cudaError_t ce = cudaStreamEndCapture(m->stream, &g);
  if (r) return fail(FTGPU_ERR_CUDA, std::string("capture launch: ") + cudaGetErrorString((cudaError_t)r));
  if (ce != cudaSuccess) return fail(FTGPU_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return fail(FTGPU_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ce));
  steps = K;
  return 0;
}

// Capture the loop's graphs (the 16-step chunk and the 2..14-step tails) at
// set-up, so that the first run of a model does not pay for capture and
// instantiation.  A later change of what a step launches (boundary
// conditions, energy, injury criteria, surrogate, driven nodes) drops them
// and the next run captures again.
int prepare_graphs(ftgpu_model *m) {
  for (bool open : {true, false}) {
    CKI(capture_chunk(m, kChunkSteps, false, open));
    for (int K = 2; K < kChunkSteps; K += 2) CKI(capture_chunk(m, K, false, open));
  }
  return 0;
}

// The host side of the explicit loop: launch chunk graphs until every
// instance is done (tMax, step limit) or an error shows up.
int run_impl(ftgpu_model *m, int max_steps, int *steps_done, bool prof, double *elem_ms,
             double *node_ms, double *device_ms) {
  if (!m || !m->init_done) return fail(FTGPU_ERR_STATE, "run before init_explicit");
  if (steps_done) *steps_done = 0;
  if (elem_ms) *elem_ms = 0.0;
  if (node_ms) *node_ms = 0.0;
  if (device_ms) *device_ms = 0.0;
  if (max_steps <= 0) return FTGPU_OK;
  CK(cudaSetDevice(m->device));
  const int ni = m->ninst;
  CK(cudaMemcpyAsync(m->h_clock, m->clock.p, sizeof(Clock) * ni, cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  const long long start0 = m->h_clock[0].step;
  for (int i = 0; i < ni; ++i) {
    m->h_clock[i].done &= ~2;  // a new run lifts the previous step limit
    m->inst[i].step_limit = m->h_clock[i].step + max_steps;
  }
  CK(cudaMemcpyAsync(m->clock.p, m->h_clock, sizeof(Clock) * ni, cudaMemcpyHostToDevice, m->stream));
  CK(cudaMemcpyAsync(m->instp.p, m->inst.data(), ni * sizeof(InstParams), cudaMemcpyHostToDevice,
                     m->stream));
  const int K = kChunkSteps;
  CKI(capture_chunk(m, K, prof, true));
  if (!prof) CKI(capture_chunk(m, K, false, false));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (device_ms) {
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, m->stream));
  }
  // every launch advances each running instance by its steps (or ends it)
  const long long max_chunks = (max_steps + 1) / 2 + 2;
  int rc = FTGPU_OK;
  long long prev = start0;
  long long left = max_steps;  // most steps any running instance still has
  for (long long c = 0; c < max_chunks; ++c) {
    // the run's first graph opens with the half-step, the others continue
    const bool open = c == 0;
    cudaGraphExec_t g = prof ? m->prof_exec : open ? m->chunk_exec : m->cont_exec;
    if (!prof && left < K) {
      // the end of the run: the shortest even graph that covers it
      const int Kt = (int)std::max<long long>(2, (left + 1) & ~1ll);
      if (Kt < K) {
        CKI(capture_chunk(m, Kt, false, open));
        g = open ? m->tail_exec[Kt / 2] : m->tailc_exec[Kt / 2];
      }
    }
    CK(cudaGraphLaunch(g, m->stream));
    CK(cudaMemcpyAsync(m->h_clock, m->clock.p, sizeof(Clock) * ni, cudaMemcpyDeviceToHost,
                       m->stream));
    CK(cudaMemcpyAsync(m->h_err, m->err.p, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (prof) {
      const long long taken = m->h_clock[0].step - prev;
      for (long long k = 0; k < std::min<long long>(taken, K); ++k) {
        float a = 0.f, b = 0.f;
        CK(cudaEventElapsedTime(&a, m->prof_ev[2 * k], m->prof_ev[2 * k + 1]));
        CK(cudaEventElapsedTime(&b, m->prof_ev[2 * k + 1], m->prof_ev[2 * k + 2]));
        if (elem_ms) *elem_ms += a;
        if (node_ms) *node_ms += b;
      }
    }
    prev = m->h_clock[0].step;
    left = 0;
    for (int i = 0; i < ni; ++i)
      if (!m->h_clock[i].done)
        left = std::max<long long>(left, m->inst[i].step_limit - m->h_clock[i].step);
    if (*m->h_err & kErrInverted) {
      rc = fail(FTGPU_ERR_INVERTED, "non-positive or non-finite Jacobian");
      break;
    }
    if (*m->h_err & kErrWait) {
      rc = fail(FTGPU_ERR_CUDA, "tensor-core inference gave up waiting");
      break;
    }
    bool all = true, dterr = false;
    for (int i = 0; i < ni; ++i) {
      all &= m->h_clock[i].done != 0;
      dterr |= (m->h_clock[i].done & 4) != 0;
    }
    if (dterr) {
      rc = fail(FTGPU_ERR_DT, "time step below FailureTimeStep");
      break;
    }
    if (all) break;
  }
  if (device_ms) {
    CK(cudaEventRecord(e1, m->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    *device_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (steps_done) *steps_done = (int)(m->h_clock[0].step - start0);
  return rc;
}

}  // namespace

// ------------------------------------------------------------------------
extern "C" {

const char *ftgpu_status_string(int s) {
  switch (s) {
    case FTGPU_OK: return "ok";
    case FTGPU_ERR_MATERIAL: return "unknown material";
    case FTGPU_ERR_INPUT: return "bad input";
    case FTGPU_ERR_ALLOC: return "device allocation failed";
    case FTGPU_ERR_DT: return "time step below FailureTimeStep";
    case FTGPU_ERR_INVERTED: return "inverted or non-finite element";
    case FTGPU_ERR_CUDA: return "CUDA error";
    case FTGPU_ERR_STATE: return "call out of order";
    case FTGPU_ERR_NODEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char *ftgpu_last_error(void) { return g_last_error.c_str(); }

int ftgpu_create(ftgpu_model **out, int device, int precision) {
  if (!out) return fail(FTGPU_ERR_INPUT, "null output pointer");
  *out = nullptr;
  if (precision != FTGPU_FP64 && precision != FTGPU_MIXED) return fail(FTGPU_ERR_INPUT, "precision");
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd <= device || device < 0) {
    cudaGetLastError();
    return fail(FTGPU_ERR_NODEVICE, "no CUDA device available");
  }
  CK(cudaSetDevice(device));
  auto m = std::make_unique<ftgpu_model>();
  m->device = device;
  m->precision = precision;
  CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  *out = m.release();
  return FTGPU_OK;
}

int ftgpu_destroy(ftgpu_model *m) {
  if (!m) return FTGPU_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  delete m;
  return FTGPU_OK;
}

int ftgpu_set_mesh(ftgpu_model *m, int nNodes, int nelements, const double *coordinates,
                   const int *eptr, const int *connectivity, const int *etype, const int *pid) {
  if (!m || nNodes <= 0 || nelements <= 0 || !coordinates || !eptr || !connectivity || !etype ||
      !pid)
    return fail(FTGPU_ERR_INPUT, "set_mesh: bad arguments");
  m->nNodes = nNodes;
  m->nE = nelements;
  m->X.assign(coordinates, coordinates + 3 * (size_t)nNodes);
  m->eptr.assign(eptr, eptr + nelements + 1);
  const int nc = eptr[nelements];
  if (nc <= 0) return fail(FTGPU_ERR_INPUT, "set_mesh: empty connectivity");
  m->conn.assign(connectivity, connectivity + nc);
  m->etype.assign(etype, etype + nelements);
  m->pid.assign(pid, pid + nelements);
  for (int e = 0; e < nelements; ++e) {
    if (etype[e] != FTGPU_C3D8 && etype[e] != FTGPU_C3D4)
      return fail(FTGPU_ERR_INPUT, "set_mesh: element type must be C3D8 or C3D4");
    if (eptr[e + 1] - eptr[e] != (etype[e] == FTGPU_C3D8 ? 8 : 4))
      return fail(FTGPU_ERR_INPUT, "set_mesh: node count does not match element type");
  }
  for (int k = 0; k < nc; ++k)
    if (connectivity[k] < 0 || connectivity[k] >= nNodes)
      return fail(FTGPU_ERR_INPUT, "set_mesh: node index out of range");
  m->setup_done = m->init_done = false;
  return FTGPU_OK;
}

int ftgpu_set_materials(ftgpu_model *m, int nPID, const int *materialID, const double *props) {
  if (!m || nPID <= 0 || !materialID || !props) return fail(FTGPU_ERR_INPUT, "set_materials");
  for (int p = 0; p < nPID; ++p)
    if (materialID[p] < 0 || materialID[p] > 7)
      return fail(FTGPU_ERR_MATERIAL, "unknown material ID (StressUpdate.cpp:25)");
  m->nPID = nPID;
  m->materialID.assign(materialID, materialID + nPID);
  m->props.assign(props, props + FTGPU_MAXMATPARAMS * (size_t)nPID);
  if (m->setup_done) {
    int r = is_fp64(m) ? upload_materials<double>(m) : upload_materials<float>(m);
    if (r) return r;
    drop_graphs(m);
  }
  return FTGPU_OK;
}

int ftgpu_set_fibers(ftgpu_model *m, const double *fiber) {
  if (!m || !fiber || m->nE <= 0) return fail(FTGPU_ERR_INPUT, "set_fibers");
  m->fiber.assign(fiber, fiber + 3 * (size_t)m->nE);
  m->setup_done = false;
  return FTGPU_OK;
}

int ftgpu_set_bc(ftgpu_model *m, const int *dof_fn, int nfn, const ftgpu_bc_fn *fns) {
  if (!m || m->nNodes <= 0 || !dof_fn || nfn < 0) return fail(FTGPU_ERR_INPUT, "set_bc");
  m->dof_fn.assign(dof_fn, dof_fn + 3 * (size_t)m->nNodes);
  for (int v : m->dof_fn)
    if (v < FTGPU_BC_HOLD || v >= nfn) return fail(FTGPU_ERR_INPUT, "set_bc: function index");
  m->fns.resize(nfn);
  for (int i = 0; i < nfn; ++i) {
    m->fns[i].kind = fns[i].kind;
    m->fns[i].pad = 0;
    for (int k = 0; k < 8; ++k) m->fns[i].p[k] = fns[i].p[k];
    if (fns[i].kind < 0 || fns[i].kind > 4) return fail(FTGPU_ERR_INPUT, "set_bc: kind");
  }
  if (m->setup_done) {
    CKI(upload_bc(m));
    CKI(upload_epid(m, true));
    drop_graphs(m);
  }
  return FTGPU_OK;
}

int ftgpu_set_instances(ftgpu_model *m, int ninst, const int *node_offset, const double *tmax,
                        const double *reduction, const double *failure_dt) {
  if (!m || ninst <= 0 || !node_offset || node_offset[0] != 0 || node_offset[ninst] != m->nNodes)
    return fail(FTGPU_ERR_INPUT, "set_instances");
  m->ninst = ninst;
  m->node_off.assign(node_offset, node_offset + ninst + 1);
  m->inst.resize(ninst);
  for (int i = 0; i < ninst; ++i) {
    if (node_offset[i + 1] <= node_offset[i]) return fail(FTGPU_ERR_INPUT, "empty instance");
    m->inst[i] = InstParams{tmax ? tmax[i] : 1e300, reduction ? reduction[i] : 0.9,
                            failure_dt ? failure_dt[i] : 0.0, 0, node_offset[i], 0};
  }
  m->inst_set = true;
  m->setup_done = false;
  return FTGPU_OK;
}

int ftgpu_set_patch_size(ftgpu_model *m, int pe) {
  if (!m || pe < 0 || pe > kMaxPatchElems) return fail(FTGPU_ERR_INPUT, "set_patch_size");
  m->patch_elems = pe;
  m->setup_done = false;
  return FTGPU_OK;
}

int ftgpu_set_surrogate(ftgpu_model *m, ftgpu_surrogate *s, double trust_e2) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "set_surrogate before setup");
  if (s && is_fp64(m)) return fail(FTGPU_ERR_STATE, "the surrogate runs in mixed precision only");
  drop_graphs(m);
  m->surr = s;
  if (!s) return FTGPU_OK;
  if (surrogate_device(s) != m->device) return fail(FTGPU_ERR_INPUT, "surrogate on another device");
  m->surr_law = surrogate_law(s);
  m->surr_law.trust_e2 = trust_e2;
  m->surr_base.assign(m->ps.groups.size(), 0);
  long long n = 0;
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi) {
    const PatchGroup &g = m->ps.groups[gi];
    m->surr_base[gi] = n;
    if (g.mat == 7) n += (long long)g.nelem * (g.etype == 0 ? 8 : 1);
  }
  if (n == 0) return FTGPU_OK;
  CKI(m->surr_x.alloc(n * kMlpIn * sizeof(uint16_t)));
  CKI(m->surr_y.alloc(n * kMlpOut * sizeof(float)));
  return FTGPU_OK;
}

int ftgpu_set_node_threads(ftgpu_model *m, int threads) {
  if (!m) return fail(FTGPU_ERR_INPUT, "set_node_threads");
  if (threads == 0) threads = 128;
  if (threads < 64 || threads > 512 || threads % 32) return fail(FTGPU_ERR_INPUT, "node threads");
  m->node_threads = threads;
  drop_graphs(m);
  return FTGPU_OK;
}

int ftgpu_set_node_split(ftgpu_model *m, int on) {
  if (!m || (on != 0 && on != 1)) return fail(FTGPU_ERR_INPUT, "set_node_split");
  if (m->node_split == on) return FTGPU_OK;
  m->node_split = on;
  if (m->setup_done) {
    CK(cudaSetDevice(m->device));
    CKI(upload_split(m));
    drop_graphs(m);
  }
  return FTGPU_OK;
}

int ftgpu_setup(ftgpu_model *m) {
  if (!m || m->nNodes <= 0 || m->nPID <= 0) return fail(FTGPU_ERR_STATE, "setup before mesh/materials");
  CK(cudaSetDevice(m->device));
  return is_fp64(m) ? setup_t<double>(m) : setup_t<float>(m);
}

int ftgpu_get_mass(ftgpu_model *m, double *mass) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "get_mass before setup");
  for (int n = 0; n < m->nNodes; ++n)
    for (int d = 0; d < 3; ++d) mass[3 * n + d] = m->mass_host[n];
  return FTGPU_OK;
}

int ftgpu_num_gauss_points(ftgpu_model *m) {
  if (!m || !m->setup_done) return 0;
  return (int)m->ngp_total;
}

int ftgpu_get_force(ftgpu_model *m, const double *u, double dt, double *fi, double *f_net) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "get_force before setup");
  CK(cudaSetDevice(m->device));
  CKI(upload_aos(m, u, m->u));
  CKI(launch_node(m, kNodeScatterU, 0));
  CKI(ensure_gp(m));
  CKI(fill_dtmin(m));
  CKI(launch_groups(m, 0, 0, dt, 1, 0));
  CKI(launch_node(m, kNodeGather, 0));
  CKI(check_err(m));
  std::vector<double> h(3 * (size_t)m->nNodes);
  CKI(download_aos(m, m->fi, h.data()));
  if (fi) memcpy(fi, h.data(), h.size() * sizeof(double));
  if (f_net)
    for (size_t i = 0; i < h.size(); ++i) f_net[i] = -h[i];
  return FTGPU_OK;
}

int ftgpu_stable_time_step(ftgpu_model *m, const double *u, double *dt_min) {
  if (!m || !m->setup_done || !dt_min) return fail(FTGPU_ERR_STATE, "stable_time_step before setup");
  CK(cudaSetDevice(m->device));
  CKI(upload_aos(m, u, m->u));
  CKI(launch_node(m, kNodeScatterU, 0));
  CKI(fill_dtmin(m));
  CKI(launch_groups(m, 0, 0, 0.0, 0, 1));
  std::vector<unsigned long long> h(2 * m->ninst);
  CK(cudaMemcpyAsync(h.data(), m->dtmin.p, h.size() * 8, cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  double mn = 1e20;  // "huge" of GlobalVariables.h:15
  for (int i = 0; i < m->ninst; ++i) {
    double v;
    memcpy(&v, &h[i], 8);
    mn = std::min(mn, v);
  }
  *dt_min = mn;
  CKI(fill_dtmin(m));
  return check_err(m);
}

int ftgpu_get_gauss_points(ftgpu_model *m, double *F, double *detF, double *pk2) {
  if (!m || !m->setup_done || m->gpJ.bytes == 0) return fail(FTGPU_ERR_STATE, "no recorded Gauss points");
  const size_t n = (size_t)m->ngp_total;
  std::vector<double> f(9 * n), j(n), s(6 * n);
  CK(cudaMemcpy(f.data(), m->gpF.p, f.size() * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(j.data(), m->gpJ.p, j.size() * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(s.data(), m->gpS.p, s.size() * 8, cudaMemcpyDeviceToHost));
  // group order -> reference element order
  long long q = 0;
  for (const PatchGroup &g : m->ps.groups) {
    const int ng = g.etype == 0 ? 8 : 1;
    for (int k = 0; k < g.nelem; ++k) {
      const int e = m->ps.elem_order[g.elem_begin + k];
      for (int gp = 0; gp < ng; ++gp, ++q) {
        const long long r = m->gp_off[e] + gp;
        if (F) memcpy(F + 9 * r, &f[9 * q], 9 * sizeof(double));
        if (detF) detF[r] = j[q];
        if (pk2) memcpy(pk2 + 6 * r, &s[6 * q], 6 * sizeof(double));
      }
    }
  }
  return FTGPU_OK;
}

int ftgpu_set_state(ftgpu_model *m, const double *u, const double *v, const double *a,
                    double time) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "set_state before setup");
  CK(cudaSetDevice(m->device));
  const double *const hs[3] = {u, v, a};
  DBuf *const ds[3] = {&m->u, &m->v, &m->a};
  CKI(upload_state3(m, hs, ds));
  m->t0 = time;
  m->init_done = false;
  return FTGPU_OK;
}

// Driven nodes and rigid bodies at the start of the loop: the list of
// nodes with rigid-body or rigid-rotation DOFs; every rigid-body DOF must belong
// to an instance with acceleration records; state zero (ex5.cpp:886-890),
// table cursors at 0 and the node maps of the zero state (u = v = a = 0).
int reset_rigid(ftgpu_model *m) {
  if (m->rigid_on && (int)m->rigid.size() != m->ninst)
    return fail(FTGPU_ERR_STATE, "the instance layout changed after set_rigid_body: set the "
                                 "acceleration records again");
  const std::vector<int> &rig = m->drv_nodes;  // driven nodes (from upload_bc)
  for (const int node : m->rigid_nodes) {
    int inst = 0;
    if (m->inst_set)
      inst = (int)(std::upper_bound(m->node_off.begin(), m->node_off.end(), node) -
                   m->node_off.begin()) - 1;
    if (!m->rigid_on || inst >= (int)m->rigid.size() || !m->rigid[inst].on)
      return fail(FTGPU_ERR_INPUT, "rigid-body DOF in an instance without acceleration records");
  }
  if (rig != m->rig_host) {  // a new driven-node list: the captured branch changes
    drop_graphs(m);
    m->rig_host = rig;
    m->rig_nodes = (long long)rig.size();
    if (!rig.empty()) CKI(m->rig_list.upload(rig.data(), rig.size()));
  }
  if (!rig.empty() && !m->stream2) {
    CK(cudaStreamCreateWithFlags(&m->stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&m->ev_join, cudaEventDisableTiming));
  }
  if (!m->rigid_on) return 0;
  std::vector<RigidState> st(m->ninst);
  std::vector<RigidStep> sp(m->ninst);
  for (int i = 0; i < m->ninst; ++i) {
    memset(&st[i], 0, sizeof(RigidState));
    memset(&sp[i], 0, sizeof(RigidStep));
    for (int j = 0; j < 3; ++j) sp[i].c[j] = m->rigid[i].c[j];
  }
  CK(cudaMemcpyAsync(m->rbstate.p, st.data(), st.size() * sizeof(RigidState),
                     cudaMemcpyHostToDevice, m->stream));
  CK(cudaMemcpyAsync(m->rbstep.p, sp.data(), sp.size() * sizeof(RigidStep),
                     cudaMemcpyHostToDevice, m->stream));
  CK(cudaStreamSynchronize(m->stream));  // the host vectors go out of scope
  return 0;
}

int ftgpu_init_explicit(ftgpu_model *m, double reduction, double failure_dt, double tmax) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "init_explicit before setup");
  CK(cudaSetDevice(m->device));
  if (!m->inst_set) {
    m->inst[0].tmax = tmax;
    m->inst[0].reduction = reduction;
    m->inst[0].failure_dt = failure_dt;
  }
  for (int i = 0; i < m->ninst; ++i) m->inst[i].step_limit = 0x7fffffffffffffffll;
  CK(cudaMemcpyAsync(m->instp.p, m->inst.data(), m->ninst * sizeof(InstParams),
                     cudaMemcpyHostToDevice, m->stream));
  CK(cudaMemsetAsync(m->err.p, 0, sizeof(int), m->stream));
  CKI(reset_rigid(m));
  NodeArgs A = node_args(m, kNodeBegin, 0);
  // the boundary values at t0, and u into the slots in the same pass
  if (is_fp64(m))
    k_apply_bc<double><<<(unsigned)((m->nNodes + 255) / 256), 256, 0, m->stream>>>(A, m->t0);
  else
    k_apply_bc<float><<<(unsigned)((m->nNodes + 255) / 256), 256, 0, m->stream>>>(A, m->t0);
  CK(cudaGetLastError());
  CKI(fill_dtmin(m));
  // The initial force needs the initial dt only where a Prony series
  // integrates over it (materials 5, 7): there a dt pass runs first and the
  // force pass reads the clock; otherwise the force pass itself gives the dt
  // minimum (it always contributes the elements' l/c), then the clock starts.
  bool prony = false;
  for (const PatchGroup &g : m->ps.groups) prony |= g.npatch > 0 && (g.mat == 5 || g.mat == 7);
  if (prony) {
    CKI(launch_groups(m, 0, 0, 0.0, 0, 1));
    k_clock_init<<<(m->ninst + 127) / 128, 128, 0, m->stream>>>(
        m->clock.as<Clock>(), m->dtmin.as<unsigned long long>(), m->instp.as<InstParams>(),
        m->ninst, m->t0);
    CK(cudaGetLastError());
    CKI(launch_groups(m, 0, 1, 0.0, 0, 0));
  } else {
    CKI(launch_groups(m, 0, 0, 0.0, 0, 0));
    k_clock_init<<<(m->ninst + 127) / 128, 128, 0, m->stream>>>(
        m->clock.as<Clock>(), m->dtmin.as<unsigned long long>(), m->instp.as<InstParams>(),
        m->ninst, m->t0);
    CK(cudaGetLastError());
  }
  if (m->injury_on) {  // the injury state starts from zero with the loop
    const size_t rb = is_fp64(m) ? sizeof(double) : sizeof(float);
    CK(cudaMemsetAsync(m->inj_ps_old.p, 0, m->inj_n * rb, m->stream));
    CK(cudaMemsetAsync(m->inj_psxsr.p, 0, m->inj_n * rb, m->stream));
    CK(cudaMemsetAsync(m->inj_flags.p, 0, m->inj_n, m->stream));
    CK(cudaMemsetAsync(m->inj_state.p, 0, sizeof(InjuryState), m->stream));
  }
  if (m->energy_on) {  // CheckEnergy's works start from zero with the loop
    CK(cudaMemsetAsync(m->du.p, 0, m->du.bytes, m->stream));
    CK(cudaMemsetAsync(m->estate.p, 0, sizeof(EnergyState), m->stream));
  }
  CKI(launch_node(m, kNodeInit, 0));
  // the clocks and the error word with one wait
  CK(cudaMemcpyAsync(m->h_clock, m->clock.p, sizeof(Clock) * m->ninst, cudaMemcpyDeviceToHost,
                     m->stream));
  CKI(check_err(m));
  for (int i = 0; i < m->ninst; ++i)
    if (m->h_clock[i].done & 4) return fail(FTGPU_ERR_DT, "initial dt below FailureTimeStep");
  m->init_done = true;
  return FTGPU_OK;
}

int ftgpu_run(ftgpu_model *m, int max_steps, int *steps_done) {
  return run_impl(m, max_steps, steps_done, false, nullptr, nullptr, nullptr);
}

int ftgpu_run_timed(ftgpu_model *m, int max_steps, int *steps_done, double *device_ms) {
  return run_impl(m, max_steps, steps_done, false, nullptr, nullptr, device_ms);
}

int ftgpu_run_profiled(ftgpu_model *m, int max_steps, int *steps_done, double *elem_ms,
                       double *node_ms) {
  return run_impl(m, max_steps, steps_done, true, elem_ms, node_ms, nullptr);
}

int ftgpu_layout_info(ftgpu_model *m, long long *npatch, long long *nslots, int *ngroups) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "layout_info before setup");
  if (npatch) *npatch = (long long)m->ps.patch_inst.size();
  if (nslots) *nslots = m->S;
  if (ngroups) *ngroups = (int)m->ps.groups.size();
  return FTGPU_OK;
}

int ftgpu_get_state(ftgpu_model *m, double *u, double *v, double *a, double *time, double *dt,
                    long long *step) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "get_state before setup");
  CK(cudaSetDevice(m->device));
  DBuf *const ds[3] = {&m->u, &m->v, &m->a};
  double *const hs[3] = {u, v, a};
  CKI(download_state3(m, ds, hs));
  Clock c;
  CK(cudaMemcpy(&c, m->clock.p, sizeof(Clock), cudaMemcpyDeviceToHost));
  if (time) *time = c.time;
  if (dt) *dt = c.dt;
  if (step) *step = c.step;
  return FTGPU_OK;
}

int ftgpu_get_instance_clock(ftgpu_model *m, double *time, double *dt, long long *step, int *done) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "get_instance_clock before setup");
  std::vector<Clock> c(m->ninst);
  CK(cudaMemcpy(c.data(), m->clock.p, sizeof(Clock) * m->ninst, cudaMemcpyDeviceToHost));
  for (int i = 0; i < m->ninst; ++i) {
    if (time) time[i] = c[i].time;
    if (dt) dt[i] = c[i].dt;
    if (step) step[i] = c[i].step;
    if (done) done[i] = c[i].done;
  }
  return FTGPU_OK;
}

int ftgpu_launches_per_step(ftgpu_model *m) {
  if (!m || !m->setup_done) return 0;
  int g = 0;
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi)
    g += m->ps.groups[gi].npatch > 0 && !(gi < m->group_idle.size() && m->group_idle[gi]);
  // element groups, k_step_scalars, k_node_step; a surrogate adds the
  // feature pass and the inference kernel of each material-7 group
  if (m->surr)
    for (auto &x : m->ps.groups) g += 2 * (x.npatch > 0 && x.mat == 7);
  int inj = 0;
  if (m->injury_on)  // (element work rides on the force pass) reduce, radix passes, list, final
    inj = 1 + (is_fp64(m) ? 8 : 4) + 2;
  // mixed precision without the energy balance: the node pass is
  // k_node_free plus k_node_step over the rest list (when it has nodes)
  const int split = (m->nkind.p && !m->energy_on && m->rest_n > 0) ? 1 : 0;
  // driven nodes: k_driven_step and k_node_step over their list (second
  // stream); acceleration records without driven nodes: k_driven_step alone
  const int drv = m->rig_nodes > 0 ? 2 : (m->rigid_on ? 1 : 0);
  return g + 2 + split + drv + (m->energy_on ? 1 : 0) + inj;  // + k_energy_reduce
}

int ftgpu_element_strain(ftgpu_model *m, double *Eavg, double *ps_max, double *ps_min,
                         double *shear_max) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "element_strain before setup");
  CK(cudaSetDevice(m->device));
  const long long nE = m->nE;
  DBuf e6, out;
  CKI(e6.alloc(6 * (size_t)nE * sizeof(double)));
  CKI(out.alloc(12 * (size_t)nE * sizeof(double)));
  CKI(launch_node(m, kNodeScatterU, 0));
  CKI(is_fp64(m) ? strain_groups_t<double>(m, e6.as<double>())
                 : strain_groups_t<float>(m, e6.as<double>()));
  k_principal_strain<<<(unsigned)((nE + 255) / 256), 256, 0, m->stream>>>(e6.as<double>(), nE,
                                                                          out.as<double>());
  CK(cudaGetLastError());
  std::vector<double> h(12 * (size_t)nE);
  CK(cudaMemcpyAsync(h.data(), out.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                     m->stream));
  CK(cudaStreamSynchronize(m->stream));
  // group order -> reference element order
  for (long long q = 0; q < nE; ++q) {
    const int e = m->ps.elem_order[q];
    const double *r = &h[12 * q];
    if (Eavg) memcpy(Eavg + 9 * (size_t)e, r, 9 * sizeof(double));
    if (ps_max) ps_max[e] = r[9];
    if (ps_min) ps_min[e] = r[10];
    if (shear_max) shear_max[e] = r[11];
  }
  return FTGPU_OK;
}

int ftgpu_write_vtu(ftgpu_model *m, const char *dir, const char *name, int step, int ncell,
                    const int *const *cell_data, const char *const *cell_names) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "write_vtu before setup");
  const size_t n3 = 3 * (size_t)m->nNodes;
  std::vector<double> u(n3), a(n3), E(9 * (size_t)m->nE);
  CKI(ftgpu_get_state(m, u.data(), nullptr, a.data(), nullptr, nullptr, nullptr));
  CKI(ftgpu_element_strain(m, E.data(), nullptr, nullptr, nullptr));
  std::vector<int> bnd(n3, 0);
  for (size_t i = 0; i < m->dof_fn.size() && i < n3; ++i) bnd[i] = m->dof_fn[i] != FTGPU_BC_FREE;
  const int r = ftgpu_write_vtu_arrays(dir, name, step, m->nNodes, m->nE, m->X.data(),
                                       m->eptr.data(), m->conn.data(), m->etype.data(),
                                       m->pid.data(), u.data(), a.data(), bnd.data(), E.data(),
                                       ncell, cell_data, cell_names);
  if (r) return fail(r, "write_vtu: cannot write the output files");
  return FTGPU_OK;
}

static_assert(sizeof(ftgpu_injury) == sizeof(InjuryState), "injury record layout");

int ftgpu_set_injury(ftgpu_model *m, int n, const int *element_ids) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "set_injury before setup");
  CK(cudaSetDevice(m->device));
  CK(cudaStreamSynchronize(m->stream));
  drop_graphs(m);
  m->init_done = false;  // the loop must start again from init_explicit
  if (n <= 0) {
    m->injury_on = false;
    m->inj_n = 0;
    return FTGPU_OK;
  }
  if (!element_ids) return fail(FTGPU_ERR_INPUT, "set_injury: no element list");
  if (m->ninst != 1)
    return fail(FTGPU_ERR_INPUT, "injury criteria are kept for single-instance models");
  const int E = m->nE;
  std::vector<int> pos(E, -1);  // reference id -> position in the list
  for (int j = 0; j < n; ++j) {
    if (element_ids[j] < 0 || element_ids[j] >= E)
      return fail(FTGPU_ERR_INPUT, "set_injury: element id out of range");
    if (pos[element_ids[j]] >= 0) return fail(FTGPU_ERR_INPUT, "set_injury: repeated element");
    pos[element_ids[j]] = j;
  }
  // listed elements in group order ("compact" index)
  std::vector<int> cidx(E, -1), eref;
  m->inj_upos.clear();
  for (int ge = 0; ge < E; ++ge) {
    const int e = m->ps.elem_order[ge];
    if (pos[e] < 0) continue;
    cidx[ge] = (int)eref.size();
    eref.push_back(e);
    m->inj_upos.push_back(pos[e]);
  }
  const size_t rb = is_fp64(m) ? sizeof(double) : sizeof(float);
  int np = 0;
  for (auto &g : m->ps.groups) np += g.npatch;
  CKI(m->inj_cidx.upload(cidx.data(), E));
  CKI(m->inj_upos_d.upload(m->inj_upos.data(), n));
  CKI(m->inj_eref.upload(eref.data(), n));
  CKI(m->inj_ps_old.alloc(n * rb));
  CKI(m->inj_psxsr.alloc(n * rb));
  CKI(m->inj_flags.alloc(n));
  CKI(m->inj_part.alloc(np * sizeof(InjuryPart)));
  CKI(m->inj_part2.alloc(((np + kInjReduceSpan - 1) / kInjReduceSpan) * sizeof(InjuryPart)));
  CKI(m->inj_done.alloc(sizeof(unsigned)));
  CK(cudaMemset(m->inj_done.p, 0, sizeof(unsigned)));
  {  // sentinel partials (no element) for the patches of groups never launched
    std::vector<InjuryPart> sp(np);
    for (auto &q : sp)
      for (int k = 0; k < 4; ++k) {
        q.v[k] = k == 1 ? 1e300 : -1e300;
        q.j[k] = 0x7fffffff;
        q.c[k] = -1;
      }
    CK(cudaMemcpy(m->inj_part.p, sp.data(), np * sizeof(InjuryPart), cudaMemcpyHostToDevice));
  }
  m->inj_group_n.assign(m->ps.groups.size(), 0);
  for (size_t gi = 0; gi < m->ps.groups.size(); ++gi) {
    const PatchGroup &g = m->ps.groups[gi];
    for (int k = 0; k < g.nelem; ++k) m->inj_group_n[gi] += cidx[g.elem_begin + k] >= 0;
  }
  CKI(m->inj_state.alloc(sizeof(InjuryState)));
  CKI(m->inj_hist.alloc(kInjHistWords * sizeof(unsigned)));
  CK(cudaMemset(m->inj_ps_old.p, 0, n * rb));
  CK(cudaMemset(m->inj_psxsr.p, 0, n * rb));
  CK(cudaMemset(m->inj_flags.p, 0, n));
  CK(cudaMemset(m->inj_state.p, 0, sizeof(InjuryState)));
  m->inj_n = n;
  m->injury_on = true;
  return FTGPU_OK;
}

int ftgpu_get_injury(ftgpu_model *m, ftgpu_injury *out, int *flags, double *ps) {
  if (!m || !m->injury_on) return fail(FTGPU_ERR_STATE, "injury criteria are off");
  CK(cudaSetDevice(m->device));
  CK(cudaStreamSynchronize(m->stream));
  if (out) CK(cudaMemcpy(out, m->inj_state.p, sizeof(ftgpu_injury), cudaMemcpyDeviceToHost));
  const int n = m->inj_n;  // device arrays are in group order: back to the caller's
  if (flags) {
    std::vector<uint8_t> f(n);
    CK(cudaMemcpy(f.data(), m->inj_flags.p, n, cudaMemcpyDeviceToHost));
    for (int c = 0; c < n; ++c) flags[m->inj_upos[c]] = f[c];
  }
  if (ps) {
    std::vector<double> v(n);
    if (is_fp64(m)) {
      CK(cudaMemcpy(v.data(), m->inj_ps_old.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> w(n);
      CK(cudaMemcpy(w.data(), m->inj_ps_old.p, n * sizeof(float), cudaMemcpyDeviceToHost));
      for (int c = 0; c < n; ++c) v[c] = w[c];
    }
    for (int c = 0; c < n; ++c) ps[m->inj_upos[c]] = v[c];
  }
  return FTGPU_OK;
}

int ftgpu_set_energy(ftgpu_model *m, int enable) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "set_energy before setup");
  if (enable && m->ninst != 1)
    return fail(FTGPU_ERR_INPUT, "energy balance is kept for single-instance models");
  CK(cudaSetDevice(m->device));
  CK(cudaStreamSynchronize(m->stream));
  if (enable && !m->energy_on) {
    // du and f_prev in the element precision (FP32 in mixed mode)
    const size_t n3b = 3 * (size_t)m->nNodes * (is_fp64(m) ? sizeof(double) : sizeof(float));
    // smallest node block: 64; the rigid-body branch adds at most as many
    const size_t maxblocks = 2 * (((size_t)m->nNodes + 63) / 64);
    CKI(m->du.alloc(n3b));
    CKI(m->fprev.alloc(n3b));
    CKI(m->epart.alloc(3 * maxblocks * sizeof(double)));
    CKI(m->estate.alloc(sizeof(EnergyState)));
    CK(cudaMemset(m->du.p, 0, n3b));
    CK(cudaMemset(m->fprev.p, 0, n3b));
    CK(cudaMemset(m->estate.p, 0, sizeof(EnergyState)));
  }
  m->energy_on = enable != 0;
  drop_graphs(m);
  m->init_done = false;  // the loop must start again from init_explicit
  return FTGPU_OK;
}

int ftgpu_set_rigid_body(ftgpu_model *m, int inst, const int *npts, const double *const *times,
                         const double *const *values, const double *centre) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "set_rigid_body before setup");
  if (inst < 0 || inst >= m->ninst) return fail(FTGPU_ERR_INPUT, "set_rigid_body: instance");
  CK(cudaSetDevice(m->device));
  CK(cudaStreamSynchronize(m->stream));
  if ((int)m->rigid.size() != m->ninst) m->rigid.assign(m->ninst, ftgpu_model::RigidHost());
  ftgpu_model::RigidHost r;
  if (npts) {
    if (!times || !values) return fail(FTGPU_ERR_INPUT, "set_rigid_body: tables");
    for (int k = 0; k < 6; ++k) {
      const int n = npts[k];
      if (n < 1 || !times[k] || !values[k])
        return fail(FTGPU_ERR_INPUT, "set_rigid_body: every channel needs >= 1 sample");
      for (int j = 0; j < n; ++j) {
        if (!std::isfinite(times[k][j]) || !std::isfinite(values[k][j]))
          return fail(FTGPU_ERR_INPUT, "set_rigid_body: non-finite sample");
        if (j > 0 && times[k][j] < times[k][j - 1])
          return fail(FTGPU_ERR_INPUT, "set_rigid_body: sample times must not decrease");
      }
      r.tab[k].assign(times[k], times[k] + n);
      r.tab[k].insert(r.tab[k].end(), values[k], values[k] + n);
    }
    if (centre)
      for (int j = 0; j < 3; ++j) r.c[j] = centre[j];
    r.on = true;
  }
  m->rigid[inst] = r;
  m->rigid_on = false;
  for (auto &x : m->rigid) m->rigid_on = m->rigid_on || x.on;
  if (m->rigid_on) {
    std::vector<RigidBody> rb(m->ninst);
    std::vector<double> tab;
    for (int i = 0; i < m->ninst; ++i) {
      memset(&rb[i], 0, sizeof(RigidBody));
      rb[i].on = m->rigid[i].on ? 1 : 0;
      for (int k = 0; k < 6 && rb[i].on; ++k) {
        const std::vector<double> &t = m->rigid[i].tab[k];
        const int n = (int)t.size() / 2;
        rb[i].off[k] = (int)tab.size();
        rb[i].cnt[k] = n;
        tab.insert(tab.end(), t.begin(), t.end());
        for (int j = 0; j < n; ++j)  // segment slopes (a zero-length segment is never used)
          tab.push_back(j + 1 < n && t[j + 1] > t[j] ? (t[n + j + 1] - t[n + j]) / (t[j + 1] - t[j])
                                                     : 0.0);
      }
    }
    if (tab.empty()) tab.push_back(0.0);
    CKI(m->rb.upload(rb.data(), rb.size()));
    CKI(m->rbtab.upload(tab.data(), tab.size()));
    CKI(m->rbstate.alloc(m->ninst * sizeof(RigidState)));
    CKI(m->rbstep.alloc(m->ninst * sizeof(RigidStep)));
  }
  drop_graphs(m);
  m->init_done = false;  // the loop must start again from init_explicit
  return FTGPU_OK;
}

int ftgpu_get_rigid_body(ftgpu_model *m, int inst, double *y, double *yd) {
  if (!m || !m->rigid_on) return fail(FTGPU_ERR_STATE, "no rigid body");
  if (inst < 0 || inst >= m->ninst || !m->rigid[inst].on)
    return fail(FTGPU_ERR_INPUT, "get_rigid_body: instance without acceleration records");
  CK(cudaSetDevice(m->device));
  RigidState st;
  CK(cudaMemcpyAsync(&st, m->rbstate.as<RigidState>() + inst, sizeof(st), cudaMemcpyDeviceToHost,
                     m->stream));
  CK(cudaStreamSynchronize(m->stream));
  for (int j = 0; j < 12; ++j) {
    if (y) y[j] = st.y[j];
    if (yd) yd[j] = st.yd[j];
  }
  return FTGPU_OK;
}

int ftgpu_get_energy(ftgpu_model *m, double *internal_work, double *external_work,
                     double *kinetic_energy, double *max_violation, long long *violations) {
  if (!m || !m->energy_on) return fail(FTGPU_ERR_STATE, "energy balance is off");
  CK(cudaSetDevice(m->device));
  EnergyState e;
  CK(cudaMemcpyAsync(&e, m->estate.p, sizeof(e), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  if (internal_work) *internal_work = e.Wint;
  if (external_work) *external_work = e.Wext;
  if (kinetic_energy) *kinetic_energy = e.WKE;
  if (max_violation) *max_violation = e.max_ratio;
  if (violations) *violations = e.violations;
  return FTGPU_OK;
}

int ftgpu_check(ftgpu_model *m) {
  if (!m || !m->setup_done) return fail(FTGPU_ERR_STATE, "check before setup");
  CK(cudaSetDevice(m->device));
  return check_err(m);
}

}  // extern "C"
