// A FemTech-style driver in the shape of examples/ex9/ex9.cpp, linked against
// femtech_gb300/dropin/ftgpu_dropin.cpp: the globals and the loop are the
// driver's, GetForce / CalculateAccelerations / StableTimeStep /
// AssembleLumpedMass come from the GPU drop-in.  One C3D8 (examples/ex9/
// 1-elt-cube.k), Neo-Hookean rho 1040, mu = lambda = 100 (examples/ex9/
// materials.dat), ramped tension dMax 7 mm over tMax 1 s, dt factor 0.8.
// Writes every step's displacements (24 doubles) to argv[1].
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

// ---- the reference globals this driver owns (include/GlobalVariables.h) ----
int nelements, nNodes, ndim, nDOF, nPIDglobal;
double *coordinates;
int *connectivity, *eptr, *pid;
char **ElementType;
int *materialID;
double *properties;
double *mass, *displacements, *velocities, *velocities_half, *accelerations;
int *boundary;
double *fe, *fi, *f_net;
double Time, dt;
double ExplicitTimeStepReduction = 0.8;
double FailureTimeStep = 1e-11;

void TerminateFemTech(int code) {
  fprintf(stderr, "TerminateFemTech(%d)\n", code);
  exit(100 + code);
}

void GetForce();
void CalculateAccelerations();
double StableTimeStep();
void AssembleLumpedMass();
extern "C" int FemTechGPU_Attach(int precision);

static void ApplyBoundaryConditions(double dMax, double tMax) {  // ex9.cpp:187-248
  const double tol = 1e-5;
  const double applied = Time * (dMax / tMax);
  for (int i = 0; i < nNodes; i++) {
    for (int d = 0; d < 3; ++d) {
      const int index = 3 * i + d;
      if (fabs(coordinates[index]) < tol) {
        boundary[index] = 1;
        displacements[index] = 0.0;
        velocities[index] = 0.0;
        accelerations[index] = 0.0;
      }
    }
    const int index = 3 * i + 1;
    if (fabs(coordinates[index] - 0.005) < tol) {
      boundary[index] = 1;
      displacements[index] = applied;
      velocities[index] = dMax / tMax;
      accelerations[index] = 0.0;
    }
  }
}

int main(int argc, char **argv) {
  static double X[24] = {0, 0, 0, 0.005, 0, 0, 0, 0.005, 0, 0.005, 0.005, 0,
                         0, 0, 0.005, 0.005, 0, 0.005, 0, 0.005, 0.005, 0.005, 0.005, 0.005};
  static int conn[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  static int ep[2] = {0, 8}, pd[1] = {0}, mid[1] = {1};
  static double props[9] = {1040.0, 100.0, 100.0, 0, 0, 0, 0, 0, 0};
  static char c3d8[] = "C3D8";
  static char *et[1] = {c3d8};
  nelements = 1; nNodes = 8; ndim = 3; nDOF = 24; nPIDglobal = 1;
  coordinates = X; connectivity = conn; eptr = ep; pid = pd; ElementType = et;
  materialID = mid; properties = props;
  displacements = (double *)calloc(nDOF, sizeof(double));
  velocities = (double *)calloc(nDOF, sizeof(double));
  velocities_half = (double *)calloc(nDOF, sizeof(double));
  accelerations = (double *)calloc(nDOF, sizeof(double));
  boundary = (int *)calloc(nDOF, sizeof(int));
  fe = (double *)calloc(nDOF, sizeof(double));
  fi = (double *)calloc(nDOF, sizeof(double));
  f_net = (double *)calloc(nDOF, sizeof(double));
  FILE *out = fopen(argv[1], "wb");
  if (FemTechGPU_Attach(0) != 0) TerminateFemTech(3);
  const double tMax = 1.0, dMax = 0.007;
  Time = 0.0;
  AssembleLumpedMass();
  ApplyBoundaryConditions(dMax, tMax);
  dt = ExplicitTimeStepReduction * StableTimeStep();
  GetForce();
  CalculateAccelerations();
  int steps = 0;
  while (Time < tMax) {  // ex9.cpp:107-175
    double t_n = Time, t_np1 = Time + dt;
    Time = t_np1;
    double dt_nphalf = dt, t_nphalf = 0.5 * (t_np1 + t_n);
    for (int i = 0; i < nDOF; i++)
      velocities_half[i] =
          boundary[i] ? velocities[i] : velocities[i] + (t_nphalf - t_n) * accelerations[i];
    for (int i = 0; i < nDOF; i++)
      if (!boundary[i]) displacements[i] += dt_nphalf * velocities_half[i];
    ApplyBoundaryConditions(dMax, tMax);
    GetForce();
    CalculateAccelerations();
    for (int i = 0; i < nDOF; i++)
      if (!boundary[i]) velocities[i] = velocities_half[i] + (t_np1 - t_nphalf) * accelerations[i];
    fwrite(displacements, sizeof(double), nDOF, out);
    ++steps;
    dt = ExplicitTimeStepReduction * StableTimeStep();
  }
  fclose(out);
  printf("steps %d time %.17g\n", steps, Time);
  return 0;
}
