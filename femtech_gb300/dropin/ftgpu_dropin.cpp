// ftgpu_dropin.cpp -- FemTech's hot-path functions on the GB300 engine.
//
// Link this file (and libftgpu.so) into a FemTech build in place of
//   src/fem/SolidMechanics/GetForce.cpp, GetForce_3D.cpp,
//   src/fem/SolidMechanics/CalculateAcclerations.cpp,
//   src/timestep/StableTimeStep.cpp and src/fem/Mass/Mass3D.cpp (AssembleLumpedMass),
// and the example drivers run unchanged: the functions below have the
// reference's names, take no arguments and read/write the reference's globals
// (include/GlobalVariables.h), exactly like the functions they replace.
// Call FemTechGPU_Attach(precision) once after ReadInputFile/ReadMaterials/
// PartitionMesh (or let the first call attach in FP64 mode).
//
// Errors are reported the reference's way: TerminateFemTech(code) with the
// reference's codes (1 material, 3 input, 12 allocation, 19 time step).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ftgpu.h"

// ---- reference globals (declared in include/GlobalVariables.h) ----
extern int nelements;
extern int nNodes;
extern int ndim;
extern int nDOF;
extern int nPIDglobal;
extern double *coordinates;
extern int *connectivity;
extern int *eptr;
extern int *pid;
extern char **ElementType;
extern int *materialID;
extern double *properties;
extern double *mass;
extern double *displacements;
extern double *accelerations;
extern int *boundary;
extern double *fe;
extern double *fi;
extern double *f_net;
extern double dt;
extern double FailureTimeStep;
void TerminateFemTech(int errorCode);

extern "C" int FemTechGPU_Attach(int precision);

namespace {

ftgpu_model *g_model = nullptr;
std::vector<int> g_boundary;  // boundary[] as last given to the engine

int code_of(int status) {
  switch (status) {
    case FTGPU_ERR_MATERIAL: return 1;
    case FTGPU_ERR_ALLOC: return 12;
    case FTGPU_ERR_DT: return 19;
    default: return 3;
  }
}

void check(int status, const char *what) {
  if (status == FTGPU_OK) return;
  fprintf(stderr, "ftgpu: %s failed: %s (%s)\n", what, ftgpu_status_string(status),
          ftgpu_last_error());
  TerminateFemTech(code_of(status));
}

// boundary[] flags become HOLD constraints (the drivers set the values themselves)
void sync_boundary() {
  if (!boundary) return;
  if ((int)g_boundary.size() == nDOF && memcmp(g_boundary.data(), boundary, nDOF * sizeof(int)) == 0)
    return;
  g_boundary.assign(boundary, boundary + nDOF);
  std::vector<int> dof_fn(nDOF);
  for (int i = 0; i < nDOF; ++i) dof_fn[i] = boundary[i] ? FTGPU_BC_HOLD : FTGPU_BC_FREE;
  check(ftgpu_set_bc(g_model, dof_fn.data(), 0, nullptr), "set_bc");
}

void ensure_attached() {
  if (!g_model) check(FemTechGPU_Attach(FTGPU_FP64), "attach");
}

}  // namespace

// Attach the engine to the mesh and materials in the reference globals.
extern "C" int FemTechGPU_Attach(int precision) {
  if (ndim != 3) return FTGPU_ERR_INPUT;
  if (g_model) ftgpu_destroy(g_model);
  g_model = nullptr;
  int rc = ftgpu_create(&g_model, 0, precision);
  if (rc) return rc;
  std::vector<int> etype(nelements);
  for (int e = 0; e < nelements; ++e) {
    if (strcmp(ElementType[e], "C3D8") == 0)
      etype[e] = FTGPU_C3D8;
    else if (strcmp(ElementType[e], "C3D4") == 0)
      etype[e] = FTGPU_C3D4;
    else
      return FTGPU_ERR_INPUT;  // truss elements stay on the CPU path
  }
  rc = ftgpu_set_mesh(g_model, nNodes, nelements, coordinates, eptr, connectivity, etype.data(), pid);
  if (rc) return rc;
  rc = ftgpu_set_materials(g_model, nPIDglobal, materialID, properties);
  if (rc) return rc;
  g_boundary.clear();
  rc = ftgpu_setup(g_model);
  if (rc) return rc;
  if (boundary) sync_boundary();
  return FTGPU_OK;
}

extern "C" void FemTechGPU_Detach(void) {
  if (g_model) ftgpu_destroy(g_model);
  g_model = nullptr;
  g_boundary.clear();
}

// AssembleLumpedMass (src/fem/Mass/Mass3D.cpp:127-157): allocates and fills mass[nDOF].
void AssembleLumpedMass(void) {
  ensure_attached();
  mass = (double *)calloc(nDOF, sizeof(double));
  if (!mass) TerminateFemTech(12);
  check(ftgpu_get_mass(g_model, mass), "get_mass");
}

// GetForce (src/fem/SolidMechanics/GetForce.cpp:12-25, GetForce_3D.cpp:5-53):
// fi = internal force on the current displacements, f_net = fe - fi.  The
// viscoelastic history lives on the device and advances once per call with
// the global dt, as in the reference.
void GetForce() {
  ensure_attached();
  sync_boundary();
  check(ftgpu_get_force(g_model, displacements, dt, fi, nullptr), "get_force");
  for (int i = 0; i < nDOF; ++i) f_net[i] = fe[i] - fi[i];
}

// CalculateAccelerations (src/fem/SolidMechanics/CalculateAcclerations.cpp:4-13).
void CalculateAccelerations() {
  for (int i = 0; i < nDOF; ++i)
    if (!boundary[i]) accelerations[i] = f_net[i] / mass[i];
}

// StableTimeStep (src/timestep/StableTimeStep.cpp:4-40).
double StableTimeStep() {
  ensure_attached();
  sync_boundary();
  double dtMin = 0.0;
  check(ftgpu_stable_time_step(g_model, displacements, &dtMin), "stable_time_step");
  if (dtMin < FailureTimeStep) {
    fprintf(stderr, "Timestep too small, dt = %15.9e\n", dtMin);
    TerminateFemTech(19);
  }
  return dtMin;
}
