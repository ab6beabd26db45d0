/*
 * refshim.cpp -- glue that lets FemTech's own hot-path sources (compiled
 * unmodified from the reference tree by oracle/Makefile) run as a single-rank
 * library, plus an extern "C" driver API used to produce golden vectors.
 *
 * TEST INFRASTRUCTURE ONLY: the output (oracle/_ref/libfemtech_ref.so) is a
 * checker; it is never linked into the product.
 *
 * What is project-written here (the reference's own versions need MPI,
 * ParMETIS, BLAS or the mesh readers):
 *   - one-rank MPI bodies (collectives are copies),
 *   - plain triple-loop dgemm_/dgemv_ (include/blas.h:14-26 signatures),
 *   - definitions of the globals normally defined by the readers
 *     (src/io/input/ReadInputFile.cpp:6-19, ReadMaterials.cpp:5-6), by
 *     InitFinalizeFemTech.cpp:9-11 and by PartitionMesh.cpp (halo pattern,
 *     empty on one rank) and by the example drivers (ex9.cpp:9-17),
 *   - StressUpdate: forwards material IDs 0-5 to the reference routines (as
 *     src/fem/SolidMechanics/StressUpdate.cpp:7-27 does) and 6/7 to the FP64
 *     restatements of the new laws in oracle/femtech_oracle.c,
 *   - a driver loop in the shape of examples/ex9/ex9.cpp:79-175.
 */
#include "FemTech.h"
#include "blas.h"

#include <algorithm>
#include <vector>
#include <stdarg.h>
#include <sys/stat.h>
#include <unistd.h>
#include <stdexcept>
#include <string>

extern "C" {
#include "femtech_oracle.h"
}

/* ---------------- one-rank MPI ---------------- */
static size_t dtsize(MPI_Datatype t) { return (size_t)t; }
int MPI_Init(int *, char ***) { return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
int MPI_Abort(MPI_Comm, int code) { throw std::runtime_error("MPI_Abort " + std::to_string(code)); }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, n * dtsize(t));
  return 0;
}
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, n * dtsize(t));
  return 0;
}
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, n * dtsize(t));
  return 0;
}
int MPI_Gatherv(const void *s, int n, MPI_Datatype t, void *r, const int *, const int *displs,
                MPI_Datatype, int, MPI_Comm) {
  memcpy((char *)r + displs[0] * dtsize(t), s, n * dtsize(t));
  return 0;
}
int MPI_Scatterv(const void *s, const int *counts, const int *displs, MPI_Datatype t, void *r,
                 int, MPI_Datatype, int, MPI_Comm) {
  memcpy(r, (const char *)s + displs[0] * dtsize(t), counts[0] * dtsize(t));
  return 0;
}
int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }

/* ---------------- plain BLAS (column-major) ---------------- */
extern "C" void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha, double *a,
                       int *lda, double *b, int *ldb, double *beta, double *c, int *ldc) {
  bool tA = (*ta == 'T' || *ta == 't'), tB = (*tb == 'T' || *tb == 't');
  for (int j = 0; j < *n; ++j)
    for (int i = 0; i < *m; ++i) {
      double s = 0.0;
      for (int l = 0; l < *k; ++l) {
        double x = tA ? a[l + *lda * i] : a[i + *lda * l];
        double y = tB ? b[j + *ldb * l] : b[l + *ldb * j];
        s += x * y;
      }
      double *cij = c + i + *ldc * j;
      *cij = (*beta == 0.0) ? *alpha * s : *alpha * s + *beta * *cij;
    }
}
extern "C" void dgemv_(char *tr, int *m, int *n, double *alpha, double *a, int *lda, double *x,
                       int *incx, double *beta, double *y, int *incy) {
  bool t = (*tr == 'T' || *tr == 't');
  int ny = t ? *n : *m, nx = t ? *m : *n;
  for (int j = 0; j < ny; ++j) {
    double s = 0.0;
    for (int i = 0; i < nx; ++i) {
      double aij = t ? a[i + *lda * j] : a[j + *lda * i];
      s += aij * x[i * *incx];
    }
    double *yj = y + j * *incy;
    *yj = (*beta == 0.0) ? *alpha * s : *alpha * s + *beta * *yj;
  }
}
extern "C" void dgesv_(int *, int *, double *, int *, int *, double *, int *, int *info) { *info = -1; }
extern "C" void dgetrf_(int *, int *, double *, int *, int *, int *info) { *info = -1; }
extern "C" void dgetrs_(char *, int *, int *, double *, int *, int *, double *, int *, int *info) { *info = -1; }

/* ---------------- logging: errors and warnings to stderr ---------------- */
/* CheckEnergy (src/fem/SolidMechanics/CheckEnergy.cpp:60-63) keeps its
 * running works in function statics and only logs them; while an energy
 * buffer is set, the logged values (the first double argument) are taken
 * from the log calls, and its violation warnings are not printed. */
static double *g_energy = nullptr;
static int g_energy_cap = 0;
static double g_wint = 0.0, g_wext = 0.0, g_wke = 0.0;
static void vlog(enum logLevel level, const char *fmt, va_list ap) {
  if (g_energy) {
    if (strncmp(fmt, "Internal Work", 13) == 0) { g_wint = va_arg(ap, double); return; }
    if (strncmp(fmt, "External Work", 13) == 0) { g_wext = va_arg(ap, double); return; }
    if (strncmp(fmt, "Kinetic Energy", 14) == 0) { g_wke = va_arg(ap, double); return; }
    if (strncmp(fmt, "Total Energy", 12) == 0 || strncmp(fmt, "Energy Violation", 16) == 0)
      return;
  }
  if (level > WARNING) return;
  vfprintf(stderr, fmt, ap);
  fputc('\n', stderr);
}
#define LOGFN(name)                                   \
  void name(enum logLevel level, const char *fmt, ...) { \
    va_list ap;                                       \
    va_start(ap, fmt);                                \
    vlog(level, fmt, ap);                             \
    va_end(ap);                                       \
  }
LOGFN(fileLog)
LOGFN(fileLogMaster)
LOGFN(fileLogSingle)
void fileLogMatrix(enum logLevel, const double *, const int, const int, const char *, ...) {}
void fileLogMatrixRM(enum logLevel, const double *, const int, const int, const char *, ...) {}
void fileLogMatrixSingle(enum logLevel, const double *, const int, const int, const char *, ...) {}
void fileLogMatrixRMSingle(enum logLevel, const double *, const int, const int, const char *, ...) {}
void fileLogArray(enum logLevel, const double *, const int, const char *, ...) {}
void fileLogArrayMaster(enum logLevel, const double *, const int, const char *, ...) {}
void fileLogArraySingle(enum logLevel, const double *, const int, const char *, ...) {}
void fileLogArrayInt(enum logLevel, const int *, const int, const char *, ...) {}
void fileLogArrayIntMaster(enum logLevel, const int *, const int, const char *, ...) {}
void fileLogArrayIntSingle(enum logLevel, const int *, const int, const char *, ...) {}

struct RefTerminate {
  int code;
};
void TerminateFemTech(int errorCode) { throw RefTerminate{errorCode}; }
void FreeArrays() {}

/* ---------------- globals defined outside the compiled files ----------------
 * (the mesh globals come with src/io/input/ReadInputFile.cpp:5-20) */
double *mass, *stiffness, *rhs; /* src/fem/Assembly.cpp:3-4 */
int *materialID;
double *properties;
int world_rank = 0, world_size = 1;
std::string uid = "oracle";
int *globalNodeID;
int sendProcessCount = 0;
int *sendProcessID, *sendNeighbourCount, *sendNeighbourCountCum, *sendNodeIndex;
double *sendNodeDisplacement, *recvNodeDisplacement;
double Time, dt;
double ExplicitTimeStepReduction = 0.8;
double FailureTimeStep = 0.0;
bool ImplicitStatic = false, ImplicitDynamic = false, ExplicitDynamic = true;

/* history and fibre arrays of the new materials 6/7 */
static double *g_hist = nullptr;
static double *g_fiber = nullptr;

/* StressUpdate: material switch of src/fem/SolidMechanics/StressUpdate.cpp:7-27 */
void StressUpdate(int e, int gp) {
  int mat = materialID[pid[e]];
  switch (mat) {
    case 0: break;
    case 1: CompressibleNeoHookean(e, gp); break;
    case 2: StVenantKirchhoff(e, gp); break;
    case 3: LinearElastic(e, gp); break;
    case 4: HGOIsotropic(e, gp); break;
    case 5: HGOIsotropicViscoelastic(e, gp); break;
    case 6:
    case 7: {
      int gi = gpPtr[e] + gp;
      or_material_stress(mat, &properties[MAXMATPARAMS * pid[e]], &F[fptr[e] + 9 * gp],
                         detF[detFptr[e] + gp], g_fiber ? g_fiber + 3 * e : nullptr, dt,
                         g_hist + 27 * (size_t)gi, &pk2[pk2ptr[e] + 6 * gp]);
      break;
    }
    default: TerminateFemTech(1);
  }
}

/* compare / unique of src/io/PartitionMesh.cpp:450-466 (that file needs
 * ParMETIS and is not built): ascending int order; in-place removal of
 * adjacent duplicates, returning the new length */
int compare(const void *a, const void *b) { return (*(int *)a - *(int *)b); }
int unique(int *arr, int n) {
  if (n <= 0) return 0;
  int j = 0;
  for (int i = 0; i < n; ++i)
    if (i == 0 || arr[i] != arr[j - 1]) arr[j++] = arr[i];
  return j;
}

/* ---------------- extern "C" driver API ---------------- */
extern "C" {

/* ReadInputFile (the reference's ReadAbaqus / ReadLsDyna on one rank), then
 * the single-rank node renumbering of updateConnectivityGlobalToLocal
 * (PartitionMesh.cpp:485-535, restated: local node j = the j-th smallest node
 * ID, coordinates of its first occurrence).  Sizes into sz[0..4] = nNodes,
 * nelements, ndim, nPIDglobal, connectivity length; the arrays are read with
 * ref_mesh_arrays. */
static std::vector<int> g_gid;
int ref_read_mesh(const char *path, int *sz) {
  try {
    nallelements = 0;
    nelements = 0;
    nNodes = 0;
    ndim = 0;
    ReadInputFile(path);
  } catch (RefTerminate &t) {
    return -t.code;
  }
  const int total = eptr[nelements];
  std::vector<int> sorted(connectivity, connectivity + total);
  std::sort(sorted.begin(), sorted.end());
  sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
  const int nU = (int)sorted.size();
  double *nc = (double *)malloc(sizeof(double) * ndim * (nU > 0 ? nU : 1));
  for (int j = 0; j < nU; ++j)
    for (int i = 0; i < total; ++i)
      if (connectivity[i] == sorted[j]) {
        memcpy(nc + ndim * j, coordinates + ndim * i, ndim * sizeof(double));
        break;
      }
  for (int i = 0; i < total; ++i)
    connectivity[i] = (int)(std::lower_bound(sorted.begin(), sorted.end(), connectivity[i]) -
                            sorted.begin());
  free(coordinates);
  coordinates = nc;
  nNodes = nU;
  g_gid.assign(sorted.begin(), sorted.end());
  for (int &g : g_gid) g += 1;
  sz[0] = nNodes;
  sz[1] = nelements;
  sz[2] = ndim;
  sz[3] = nPIDglobal;
  sz[4] = total;
  return 0;
}

/* WriteVTU + WritePVD (src/io/output/WriteVTU.cpp, WritePVD.cpp) of the mesh
 * of the last ref_setup with the given state, in directory dir (results/vtu
 * is created first: the reference expects it); stepTimes has step + 1
 * entries.  u is copied (the writer flushes tiny displacements in place). */
int ref_write_vtu(const char *dir, const char *name, int step, const double *u, const double *a,
                  const int *bnd, const double *E, int ncell, int **cell_data,
                  const char **cell_names, const double *stepTimes) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return -1;
  if (chdir(dir)) return -2;
  mkdir("results", 0755);
  mkdir("results/vtu", 0755);
  memcpy(displacements, u, sizeof(double) * nDOF);
  memcpy(accelerations, a, sizeof(double) * nDOF);
  memcpy(boundary, bnd, sizeof(int) * nDOF);
  memcpy(Eavg, E, sizeof(double) * 9 * nelements);
  free(stepTime);
  stepTime = (double *)malloc(sizeof(double) * (step + 1));
  memcpy(stepTime, stepTimes, sizeof(double) * (step + 1));
  WriteVTU(name, step, cell_data, ncell, cell_names);
  WritePVD(name, step);
  return chdir(cwd) ? -3 : 0;
}

/* the arrays of the last ref_read_mesh; etype: 0 "C3D8", 1 "C3D4", 2 "T3D2",
 * -1 other */
void ref_mesh_arrays(double *coords, int *ep, int *conn, int *etype, int *pidOut, int *eid,
                     int *gid) {
  memcpy(coords, coordinates, sizeof(double) * ndim * nNodes);
  memcpy(ep, eptr, sizeof(int) * (nelements + 1));
  memcpy(conn, connectivity, sizeof(int) * eptr[nelements]);
  memcpy(pidOut, pid, sizeof(int) * nelements);
  memcpy(eid, global_eid, sizeof(int) * nelements);
  memcpy(gid, g_gid.data(), sizeof(int) * nNodes);
  for (int e = 0; e < nelements; ++e) {
    const char *t = ElementType[e];
    etype[e] = strcmp(t, "C3D8") == 0 ? 0 : (strcmp(t, "C3D4") == 0 ? 1 : (strcmp(t, "T3D2") == 0 ? 2 : -1));
  }
}

int ref_setup(int nN, int nE, const double *coords, const int *ep, const int *conn,
              const int *etype, const int *pidIn, int nP, const int *matID, const double *props,
              const double *fiber) {
  try {
    ndim = 3;
    nNodes = nN;
    nelements = nallelements = nE;
    nDOF = 3 * nN;
    nPID = nPIDglobal = nP;
    coordinates = (double *)malloc(sizeof(double) * 3 * nN);
    memcpy(coordinates, coords, sizeof(double) * 3 * nN);
    eptr = (int *)malloc(sizeof(int) * (nE + 1));
    memcpy(eptr, ep, sizeof(int) * (nE + 1));
    connectivity = (int *)malloc(sizeof(int) * ep[nE]);
    memcpy(connectivity, conn, sizeof(int) * ep[nE]);
    pid = (int *)malloc(sizeof(int) * nE);
    memcpy(pid, pidIn, sizeof(int) * nE);
    global_eid = (int *)malloc(sizeof(int) * nE);
    ElementType = (char **)malloc(sizeof(char *) * nE);
    static char hex[] = "C3D8", tet[] = "C3D4";
    for (int e = 0; e < nE; ++e) {
      global_eid[e] = e;
      ElementType[e] = etype[e] == 0 ? hex : tet;
    }
    materialID = (int *)malloc(sizeof(int) * nP);
    memcpy(materialID, matID, sizeof(int) * nP);
    properties = (double *)malloc(sizeof(double) * MAXMATPARAMS * nP);
    memcpy(properties, props, sizeof(double) * MAXMATPARAMS * nP);
    sendProcessCount = 0;
    sendNeighbourCountCum = (int *)calloc(1, sizeof(int));
    ExplicitDynamic = true;
    AllocateArrays();
    if (energyFile) {
      fclose(energyFile);
      energyFile = nullptr;
      remove(("energy_" + uid + ".dat").c_str());
    }
    ShapeFunctions();
    AssembleLumpedMass();
    free(g_hist);
    g_hist = (double *)calloc(27 * (size_t)gpPtr[nE], sizeof(double));
    free(g_fiber);
    g_fiber = nullptr;
    if (fiber) {
      g_fiber = (double *)malloc(sizeof(double) * 3 * nE);
      memcpy(g_fiber, fiber, sizeof(double) * 3 * nE);
    }
    Time = 0.0;
    dt = 0.0;
    return 0;
  } catch (RefTerminate &t) {
    return -t.code;
  }
}

int ref_get_mass(double *m) {
  memcpy(m, mass, sizeof(double) * nDOF);
  return 0;
}

int ref_num_gp(void) { return gpPtr[nelements]; }

int ref_get_gp(double *Fout, double *detFout, double *pk2out) {
  int ng = gpPtr[nelements];
  if (Fout) memcpy(Fout, F, sizeof(double) * 9 * ng);
  if (detFout) memcpy(detFout, detF, sizeof(double) * ng);
  if (pk2out) memcpy(pk2out, pk2, sizeof(double) * 6 * ng);
  return 0;
}

int ref_get_shape(double *dshpOut, double *detJOut) {
  if (dshpOut) memcpy(dshpOut, dshp, sizeof(double) * dsptr[nelements]);
  if (detJOut) memcpy(detJOut, detJacobian, sizeof(double) * gpPtr[nelements]);
  return 0;
}

/* GetForce() on the given displacements with the given global dt. */
int ref_get_force(const double *u, double dtIn, double *fiOut, double *fnetOut) {
  try {
    memcpy(displacements, u, sizeof(double) * nDOF);
    dt = dtIn;
    GetForce();
    if (fiOut) memcpy(fiOut, fi, sizeof(double) * nDOF);
    if (fnetOut) memcpy(fnetOut, f_net, sizeof(double) * nDOF);
    return 0;
  } catch (RefTerminate &t) {
    return -t.code;
  }
}

double ref_stable_time_step(const double *u, const int *bnd) {
  try {
    memcpy(displacements, u, sizeof(double) * nDOF);
    memcpy(boundary, bnd, sizeof(int) * nDOF);
    FailureTimeStep = 0.0;
    return StableTimeStep();
  } catch (RefTerminate &t) {
    return -(double)t.code;
  }
}

/* The explicit loop of examples/ex9/ex9.cpp:79-175 with driver-side
 * boundary conditions given as per-DOF function indices (see or_apply_bc). */
/* CalculateMaximumPrincipalStrain (CalculateStrain.cpp:8-75) of every element
 * on the F of the last ref_get_force: Eavg (9 per element, the reference's
 * Eavg layout), the clamped max / min principal strains and the max shear. */
int ref_element_strain(double *Eavg9, double *ps_max, double *ps_min, double *shear_max) {
  try {
    for (int elm = 0; elm < nelements; ++elm) {
      double mx, mn, sh;
      CalculateMaximumPrincipalStrain(elm, &mx, &mn, &sh);
      if (Eavg9) memcpy(Eavg9 + 9 * (size_t)elm, Eavg + 9 * (size_t)elm, 9 * sizeof(double));
      if (ps_max) ps_max[elm] = mx;
      if (ps_min) ps_min[elm] = mn;
      if (shear_max) shear_max[elm] = sh;
    }
    return 0;
  } catch (RefTerminate &t) {
    return -t.code;
  }
}

/* The reference's 95th percentiles (math.cpp:160-196 and 198-325) of n values
 * (one rank). */
int ref_percentile95(double *data, int n, double *brute, double *parallel) {
  try {
    *brute = compute95thPercentileValueBruteForce(data, n);
    *parallel = compute95thPercentileValue(data, n);
    return 0;
  } catch (RefTerminate &t) {
    return -t.code;
  }
}

/* interpolateLinear (math.cpp:99-119) */
double ref_interp_linear(int n, double *x, double *y, double value) {
  return interpolateLinear(n, x, y, value);
}

/* The per-node body of ApplyAccBoundaryConditions (examples/ex5/ex5.cpp:
 * 345-371) on the reference's own quaternion and vector helpers (math.cpp):
 * the driver itself needs Boost.Odeint, which the reference tree does not
 * carry, so its loop body is restated here over the reference's functions.
 * y, yd: the integrator state yInt / ydotInt; X: the node position. */
void ref_rigid_point(const double *y, const double *yd, const double *X, double *u, double *v,
                     double *a) {
  double r[4], R[4], Rinv[4], V[4], Vp[4];
  double omegaR[3], omega[3], omegaOmegaR[3], omegaVel[3], vel[3];
  double alpha[3], alphaR[3], locV[3];
  r[0] = 0.0;
  r[1] = y[3];
  r[2] = y[4];
  r[3] = y[5];
  quaternionExp(r, R);
  quaternionInverse(R, Rinv);
  for (int j = 0; j < 3; ++j) {
    omega[j] = y[j];
    alpha[j] = yd[j];
    vel[j] = y[6 + j];
    locV[j] = X[j];
  }
  V[0] = 0.0;
  V[1] = locV[0];
  V[2] = locV[1];
  V[3] = locV[2];
  quaternionRotate(V, R, Rinv, Vp);
  crossProduct(omega, &(Vp[1]), omegaR);
  crossProduct(omega, omegaR, omegaOmegaR);
  crossProduct(omega, vel, omegaVel);
  crossProduct(alpha, &(Vp[1]), alphaR);
  for (int j = 0; j < 3; ++j) {
    u[j] = Vp[j + 1] - locV[j] + y[9 + j];
    v[j] = omegaR[j] + y[6 + j];
    a[j] = 2.0 * omegaVel[j] + omegaOmegaR[j] + yd[6 + j] + alphaR[j];
  }
}

/* Energy output of the next ref_explicit_run: per step the cumulative internal
 * and external work and the kinetic energy that the reference's own
 * CheckEnergy() logs (ex9.cpp:154-156 calls it after every step).  Its works
 * accumulate in statics over the life of the process, so one energy run per
 * process gives works from zero. */
void ref_set_energy_out(double *buf, int cap) {
  g_energy = buf;
  g_energy_cap = cap;
}

int ref_explicit_run(const int *dof_fn, const or_bc_fn *fns, int nfn, double t0, double tMax,
                     double reduction, int max_steps, int out_every, double *uInOut,
                     double *vInOut, double *aInOut, double *u_out, double *t_out, int max_out,
                     int *n_out, int *steps_done, double *time_out, double *dt_out) {
  (void)nfn;
  try {
    or_model bcm;
    memset(&bcm, 0, sizeof(bcm));
    bcm.nNodes = nNodes;
    bcm.coordinates = coordinates;
    memcpy(displacements, uInOut, sizeof(double) * nDOF);
    memcpy(velocities, vInOut, sizeof(double) * nDOF);
    memcpy(accelerations, aInOut, sizeof(double) * nDOF);
    for (int i = 0; i < nDOF; ++i) boundary[i] = dof_fn[i] != OR_BC_FREE;
    ExplicitTimeStepReduction = reduction;
    FailureTimeStep = 0.0;
    Time = t0;
    *n_out = 0;
    or_apply_bc(&bcm, dof_fn, fns, Time, displacements, velocities, accelerations);
    dt = ExplicitTimeStepReduction * StableTimeStep();
    GetForce();
    CalculateAccelerations();
    int step = 0;
    while (Time < tMax && step < max_steps) {
      double t_n = Time;
      double t_np1 = Time + dt;
      Time = t_np1;
      double dt_nphalf = dt;
      double t_nphalf = 0.5 * (t_np1 + t_n);
      for (int i = 0; i < nDOF; i++) {
        if (boundary[i])
          velocities_half[i] = velocities[i];
        else
          velocities_half[i] = velocities[i] + (t_nphalf - t_n) * accelerations[i];
      }
      if (g_energy) {  // ex9.cpp:124-129
        memcpy(displacements_prev, displacements, nDOF * sizeof(double));
        memcpy(accelerations_prev, accelerations, nDOF * sizeof(double));
        memcpy(fi_prev, fi, nDOF * sizeof(double));
        memcpy(fe_prev, fe, nDOF * sizeof(double));
      }
      for (int i = 0; i < nDOF; i++)
        if (!boundary[i]) displacements[i] = displacements[i] + dt_nphalf * velocities_half[i];
      or_apply_bc(&bcm, dof_fn, fns, Time, displacements, velocities, accelerations);
      GetForce();
      CalculateAccelerations();
      for (int i = 0; i < nDOF; i++)
        if (!boundary[i]) velocities[i] = velocities_half[i] + (t_np1 - t_nphalf) * accelerations[i];
      if (g_energy && step < g_energy_cap) {
        CheckEnergy(Time, 1);  // writeFlag != 0: log only (ex9.cpp:154-156)
        g_energy[3 * step + 0] = g_wint;
        g_energy[3 * step + 1] = g_wext;
        g_energy[3 * step + 2] = g_wke;
      }
      ++step;
      if (out_every > 0 && step % out_every == 0 && *n_out < max_out) {
        memcpy(u_out + (size_t)(*n_out) * nDOF, displacements, sizeof(double) * nDOF);
        t_out[*n_out] = Time;
        ++*n_out;
      }
      dt = ExplicitTimeStepReduction * StableTimeStep();
    }
    *steps_done = step;
    *time_out = Time;
    *dt_out = dt;
    memcpy(uInOut, displacements, sizeof(double) * nDOF);
    memcpy(vInOut, velocities, sizeof(double) * nDOF);
    memcpy(aInOut, accelerations, sizeof(double) * nDOF);
    return 0;
  } catch (RefTerminate &t) {
    return -t.code;
  }
}

}  // extern "C"
