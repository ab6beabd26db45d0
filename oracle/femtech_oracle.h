/*
 * femtech_oracle.h -- FP64 CPU restatement of FemTech's explicit-dynamics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA path is compared
 * against; it is never linked into, imported by or called from the product
 * library (femtech_gb300/).  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py use it.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the reference's own
 * sources (compiled unmodified by oracle/Makefile into oracle/_ref/), and the
 * CPU test-suite checks this restatement against them.  The Ogden (6) and
 * anisotropic GOH + Prony (7) laws have no reference implementation; they are
 * pinned through special cases that reduce to reference laws (Ogden alpha=2 ==
 * HGOIsotropic with k1=0, GOH kappa=1/3 == HGOIsotropicViscoelastic with
 * g2=0) plus energy finite-difference checks.
 *
 * Layout follows the reference (include/GlobalVariables.h): AoS nodal arrays
 * [node*3+dim], CSR connectivity (eptr), per-part properties[pid*9+k].
 */
#ifndef FEMTECH_ORACLE_H
#define FEMTECH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAXMATPARAMS 9
#define OR_C3D8 0
#define OR_C3D4 1

/* boundary-condition function kinds (per constrained DOF) */
#define OR_BC_FREE (-1)
#define OR_BC_HOLD (-2)
#define OR_BCK_FIXED 0 /* u = p0, v = 0                                     */
#define OR_BCK_RAMP 1  /* u = p0 * t, v = p0  (examples/ex9/ex9.cpp:227-244) */
#define OR_BCK_SINE 2  /* u = p0 * sin(p1 t), v = p0 p1 cos(p1 t)           */
#define OR_BCK_ROT 3   /* rigid rotation: axis p0..2, centre p3..5,
                          half-sine angular acceleration peak p6 over p7 s  */
#define OR_BCK_RIGID 4 /* rigid-body motion of or_model.rigid (u, v and a)  */

typedef struct or_bc_fn {
  int kind;
  int pad;
  double p[8];
} or_bc_fn;

/* Per-step injury criteria of the brain drivers (examples/ex5/ex5.cpp:
 * 1311-1430, CalculateInjuryCriterions) for the elements ids[0..n): running
 * extremes of the principal strains (value, element, time), sticky flags
 * MPS > 0.15 / 0.30, principal strain rate > 120 /s, MPS x rate > 28 /s, and
 * the largest 95th percentiles of MPS and of MPS x rate with the elements at
 * or above them.  The caller owns every array (n entries each). */
typedef struct or_injury {
  int n;
  const int *ids;
  double *ps_old, *psxsr;
  int *mps15, *mps30, *psr120, *psxsr28, *in_mps95, *in_mpsxsr95;
  double max_strain, max_strain_time, min_strain, min_strain_time;
  double max_shear, max_shear_time, max_psxsr, max_psxsr_time;
  int max_strain_elem, min_strain_elem, max_shear_elem, max_psxsr_elem;
  double mps95, mps95_time, mpsxsr95, mpsxsr95_time;
  int mps95_count, mpsxsr95_count;
} or_injury;

/* Rigid-body motion driven by sampled accelerations, as the brain drivers
 * apply it to the nodes of material-0 parts (examples/ex5/ex5.cpp:339-392,
 * ApplyAccBoundaryConditions).  Channels 0-2: angular acceleration about x,
 * y, z; 3-5: linear acceleration along x, y, z; each a table of n[k]
 * (time, value) pairs with non-decreasing times.  The integrator state of
 * ex5.cpp:100-105: y = [omega(3), r(3), v_cm(3), x_cm(3)] with r the rotation
 * generator (R = exp of the pure quaternion r), yd = dy/dt at the last step's
 * end time (zero at the start, ex5.cpp:886-890).  Positions rotate about
 * centre c (the reference rotates about the origin of the shifted mesh). */
typedef struct or_rigid {
  int n[6];
  const double *t[6], *v[6];
  double c[3];
  double y[12], yd[12];
} or_rigid;

typedef struct or_model {
  /* inputs, reference layout; owned by the caller */
  int nNodes, nelements, nPID;
  const double *coordinates; /* 3*nNodes                              */
  const int *eptr;           /* nelements+1                           */
  const int *connectivity;   /* eptr[nelements]                       */
  const int *etype;          /* OR_C3D8 / OR_C3D4 per element         */
  const int *pid;            /* part id per element                   */
  const int *materialID;     /* per part                              */
  const double *properties;  /* 9 per part                            */
  const double *fiber;       /* 3 per element (material 7) or NULL    */
  /* derived (owned by the oracle) */
  int *nGP, *nShp, *gpPtr, *dsptr, *gptr, *fptr, *pk2ptr;
  double *shp, *dshp, *detJ, *gw;
  double *F, *detF, *pk2;
  double *hist; /* 27 doubles per Gauss point: H1[9], H2[9], S0n[9] */
  double *mass; /* 3*nNodes                                          */
  double *fe;   /* scratch: 24 doubles per element                   */
  double *ce;   /* dilatational wave speed per part                  */
  int nthreads;
  /* optional output of or_explicit_run: per step the cumulative internal
   * work, external work and the kinetic energy of CheckEnergy
   * (src/fem/SolidMechanics/CheckEnergy.cpp:3-85); NULL = not computed */
  double *energy;
  int energy_cap; /* steps the energy buffer holds (3 doubles each)    */
  /* optional: injury criteria updated after every step of
   * or_explicit_run (NULL = not computed) */
  or_injury *injury;
  /* optional: the rigid body of OR_BCK_RIGID functions (NULL = none);
   * or_explicit_run zeroes its state and advances it by one step per step */
  or_rigid *rigid;
} or_model;

int or_setup(or_model *m);
void or_free(or_model *m);
int or_get_force(or_model *m, const double *u, double dt, double *fi);
double or_stable_time_step(const or_model *m, const double *u, const int *boundary);
int or_material_stress(int matID, const double *props, const double *F, double J,
                       const double *a0, double dt, double *hist27, double *S6);
int or_explicit_run(or_model *m, const int *dof_fn, const or_bc_fn *fns, int nfn,
                    double t0, double tMax, double reduction, double failure_dt,
                    int max_steps, int out_every, double *u, double *v, double *a,
                    double *u_out, double *t_out, int max_out, int *n_out,
                    int *steps_done, double *time_out, double *dt_out);
void or_element_strain(const or_model *m, double *Eavg9, double *ps_max, double *ps_min,
                       double *shear_max);
/* 95th percentile as compute95thPercentileValueBruteForce (math.cpp:160-196):
 * the element of rank (int)(0.95 n) - 1 of the values (rank clamped at 0) */
double or_percentile95(const double *data, int n);
/* one call of CalculateInjuryCriterions on the F of the last or_get_force */
void or_injury_step(const or_model *m, or_injury *s, double time, double dt);
void or_apply_bc(const or_model *m, const int *dof_fn, const or_bc_fn *fns,
                 double t, double *u, double *v, double *a);
/* interpolateLinear (src/math/math.cpp:99-119) */
double or_interp_linear(int n, const double *x, const double *y, double value);
/* one integrator step of ex5.cpp:344 from t over h (Dormand-Prince 5(4)) */
void or_rigid_step(or_rigid *rb, double t, double h);
/* displacement, velocity and acceleration of a point at reference position
 * X under the current state (ex5.cpp:345-371) */
void or_rigid_point(const or_rigid *rb, const double *X, double *u, double *v, double *a);
void or_set_threads(or_model *m, int n);
int or_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
