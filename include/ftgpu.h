/*
 * ftgpu.h -- C ABI of the GB300 (sm_103a) explicit-dynamics engine.
 *
 * The engine replaces FemTech's per-step hot path: the internal force of every
 * element (GetForce / GetForce_3D with CalculateDeformationGradient,
 * DeterminateF, StressUpdate, InternalForceUpdate), the nodal assembly, the
 * accelerations, the central-difference velocity/displacement update of the
 * example drivers and the stable-time-step reduction.  Arrays cross the ABI in
 * the reference's own layout (include/GlobalVariables.h): AoS nodal arrays
 * indexed [node*3+dim], CSR connectivity eptr/connectivity, per-part
 * materialID[] and properties[pid*MAXMATPARAMS+k] as filled by ReadMaterials().
 *
 * Plain C types only.  Every call returns FTGPU_OK (0) or a negative status;
 * the library never aborts the process (the reference calls
 * TerminateFemTech(code) -> MPI_Abort; callers map the negative codes back).
 * One model is driven from one host thread (the reference is non-reentrant
 * too: its scratch arrays mat1..mat4, B and fintGQ are globals).
 */
#ifndef FTGPU_H
#define FTGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mirroring TerminateFemTech's codes where one exists) ---- */
#define FTGPU_OK 0
#define FTGPU_ERR_MATERIAL (-1)    /* unknown material ID: StressUpdate.cpp:25-26 (code 1)   */
#define FTGPU_ERR_INPUT (-3)       /* bad mesh / argument: TerminateFemTech(3)               */
#define FTGPU_ERR_ALLOC (-12)      /* device allocation failed: AllocateArrays.cpp (code 12) */
#define FTGPU_ERR_DT (-19)         /* dt below FailureTimeStep: StableTimeStep.cpp:35-38     */
#define FTGPU_ERR_INVERTED (-20)   /* J <= 0 or non-finite at a Gauss point                  */
#define FTGPU_ERR_CUDA (-30)       /* CUDA runtime error                                     */
#define FTGPU_ERR_STATE (-31)      /* call out of order (e.g. step before setup)             */
#define FTGPU_ERR_NODEVICE (-32)   /* no CUDA device / extension not usable                  */

/* ---- precision modes ---- */
#define FTGPU_FP64 0  /* element kinematics, stress and nodal state in FP64       */
#define FTGPU_MIXED 1 /* FP32 element kinematics/stress, FP64 nodal state and dt   */

/* ---- element types (ElementType strings "C3D8"/"C3D4" of the reference) ---- */
#define FTGPU_C3D8 0
#define FTGPU_C3D4 1
#define FTGPU_T3D2 2 /* truss: read by ftgpu_read_mesh, not taken by ftgpu_set_mesh */

/* ---- material IDs (StressUpdate.cpp:7-27, plus two new laws) ----
 * 0 rigid, 1 compressible Neo-Hookean [rho,mu,lambda], 2 St.Venant-Kirchhoff
 * [rho,mu,lambda], 3 linear elastic [rho,mu,lambda], 4 HGO isotropic
 * [rho,mu,lambda,k1,k2], 5 HGO isotropic + 2-term Prony
 * [rho,mu,lambda,k1,k2,g1,t1,g2,t2], 6 one-term Ogden [rho,mu,lambda,alpha],
 * 7 anisotropic GOH (fibre per element, dispersion kappa) + 1-term Prony
 * [rho,mu,lambda,k1,k2,g1,t1,kappa]. */
#define FTGPU_MAXMATPARAMS 9

/* ---- boundary-condition functions (driver-side BCs of examples/exN) ----
 * Each DOF is FTGPU_BC_FREE, FTGPU_BC_HOLD (constrained, values untouched: the
 * reference's boundary[] flag alone) or the index of a function below.
 * A constrained DOF gets u(t), v(t) and a = 0 after every displacement update,
 * as ApplyBoundaryConditions does in examples/ex9/ex9.cpp:187-248. */
#define FTGPU_BC_FREE (-1)
#define FTGPU_BC_HOLD (-2)
#define FTGPU_BCK_FIXED 0 /* u = p0, v = 0                                         */
#define FTGPU_BCK_RAMP 1  /* u = p0 * t, v = p0                                    */
#define FTGPU_BCK_SINE 2  /* u = p0 sin(p1 t), v = p0 p1 cos(p1 t)                 */
#define FTGPU_BCK_ROT 3   /* rigid rotation about unit axis p0..2 through p3..5 with
                             angular acceleration p6 sin(pi t / p7) for t <= p7     */
#define FTGPU_BCK_RIGID 4 /* rigid-body motion of the node's instance from its
                             acceleration records (ftgpu_set_rigid_body): u, v
                             and a of the node as ApplyAccBoundaryConditions
                             sets them (examples/ex5/ex5.cpp:339-392)            */

typedef struct ftgpu_bc_fn {
  int kind;
  int pad;
  double p[8];
} ftgpu_bc_fn;

typedef struct ftgpu_model ftgpu_model;

/* Create / destroy a model on a CUDA device.  precision: FTGPU_FP64 / MIXED. */
int ftgpu_create(ftgpu_model **out, int device, int precision);
int ftgpu_destroy(ftgpu_model *m);
const char *ftgpu_status_string(int status);
const char *ftgpu_last_error(void);

/* ---- mesh input (host only, no device needed) ----
 * Reads an Abaqus .inp or LS-DYNA .k file (by extension) into the arrays a
 * single-rank FemTech run holds after ReadInputFile + PartitionMesh
 * (ReadInputFile.cpp:26-77, ReadAbaqus.cpp:26-246, ReadLsDyna.cpp:48-319,
 * PartitionMesh.cpp:485-535): nodes used by elements, numbered by ascending
 * node ID (global_node_id, 1-based); elements in file order with their IDs;
 * pid = element set index in order of first appearance (.inp) or part ID - 1
 * (.k); nPID distinct parts, nPIDglobal = largest pid + 1.  etype: FTGPU_C3D8,
 * FTGPU_C3D4, FTGPU_T3D2 or -1 (other Abaqus types; LS-DYNA node counts
 * classified as the reference does).  missing_nodes: used nodes that no node
 * line defined (their coordinates are 0, as in the reference). */
typedef struct ftgpu_mesh {
  int nNodes, nelements, ndim, nPID, nPIDglobal;
  long long missing_nodes;
  double *coordinates; /* ndim * nNodes */
  int *eptr;           /* nelements + 1 */
  int *connectivity;   /* eptr[nelements], local node indices */
  int *etype, *pid, *global_eid; /* nelements */
  int *global_node_id; /* nNodes */
} ftgpu_mesh;
int ftgpu_read_mesh(const char *path, ftgpu_mesh **out);
void ftgpu_free_mesh(ftgpu_mesh *mesh);
const char *ftgpu_read_mesh_error(void);

/* ---- output steps: the reference's ASCII VTU files (WriteVTU.cpp:3-263,
 * WritePVD.cpp:6-36, one rank) ----
 * ftgpu_write_vtu writes <dir>/results/vtu/<name>.vtu.<step>.0000 and
 * <dir>/results/<name>.<step>.pvtu from the model's current state: deformed
 * points, connectivity / offsets / VTK types, Displacements, Accelerations,
 * Boundary (constrained DOFs), PartID, AvgStrain (CalculateStrain's Eavg,
 * computed on the device), ProcID and ncell extra Int32 cell arrays (the
 * brain drivers' injury outputs).  Text and layout are the reference's;
 * displacements below 1e-20 in magnitude are written as 0 as the reference
 * writes them (it also flushes them in its state; the device state is left
 * as it is).  dir NULL or "" = the working directory.  ftgpu_write_pvd writes
 * <dir>/<name without extension>.pvd listing steps 0..step with their times.
 * ftgpu_write_vtu_arrays is the same writer on host arrays (reference layout,
 * boundary as 0/1 per DOF, Eavg 9 per element); it needs no device. */
int ftgpu_write_vtu(ftgpu_model *m, const char *dir, const char *name, int step, int ncell,
                    const int *const *cell_data, const char *const *cell_names);
int ftgpu_write_vtu_arrays(const char *dir, const char *name, int step, int nNodes,
                           int nelements, const double *coordinates, const int *eptr,
                           const int *connectivity, const int *etype, const int *pid,
                           const double *u, const double *a, const int *boundary,
                           const double *Eavg, int ncell, const int *const *cell_data,
                           const char *const *cell_names);
int ftgpu_write_pvd(const char *dir, const char *name, int step, const double *step_time);

/* Mesh in the reference's arrays (ReadInputFile + PartitionMesh leave these in
 * coordinates, eptr, connectivity, ElementType, pid: GlobalVariables.h:34-48).
 * etype[e] is FTGPU_C3D8 or FTGPU_C3D4.  Arrays are copied. */
int ftgpu_set_mesh(ftgpu_model *m, int nNodes, int nelements, const double *coordinates,
                   const int *eptr, const int *connectivity, const int *etype, const int *pid);

/* Materials as ReadMaterials() leaves them (ReadMaterials.cpp:8-138):
 * materialID[nPID], properties[nPID*FTGPU_MAXMATPARAMS]. */
int ftgpu_set_materials(ftgpu_model *m, int nPID, const int *materialID,
                        const double *properties);

/* Unit fibre direction per element (3*nelements), used by material 7. */
int ftgpu_set_fibers(ftgpu_model *m, const double *fiber);

/* Boundary conditions: dof_fn[3*nNodes] (FREE, HOLD or function index) and the
 * function table.  Replaces the boundary[] array plus the driver's
 * ApplyBoundaryConditions() (ex9.cpp:187-248). */
int ftgpu_set_bc(ftgpu_model *m, const int *dof_fn, int nfn, const ftgpu_bc_fn *fns);

/* Several independent instances in one model (batched ensemble).  Nodes of
 * instance i are [node_offset[i], node_offset[i+1]); no element may span two
 * instances.  Per-instance end time, dt reduction factor and failure dt.
 * Without this call the model is one instance. */
int ftgpu_set_instances(ftgpu_model *m, int ninst, const int *node_offset, const double *tmax,
                        const double *reduction, const double *failure_dt);

/* Patch size (elements per thread block) used when setup() builds its
 * element patches: 0 = default.  Exposed for the autotuner. */
int ftgpu_set_patch_size(ftgpu_model *m, int elements_per_patch);

/* Threads per block of the nodal kernels (64..512, multiple of 32; 0 =
 * default 128).  Exposed for the autotuner. */
int ftgpu_set_node_threads(ftgpu_model *m, int threads);

/* Mixed precision: the nodal pass as a lean kernel over the free and
 * function-driven nodes plus the general kernel over the rest (1, the
 * default), or the general kernel over every node (0).  Same results either
 * way.  Exposed for the autotuner; no counterpart in the reference. */
int ftgpu_set_node_split(ftgpu_model *m, int on);

/* One-time setup on the device: element patches, reference shape-function
 * data and the lumped mass.  Replaces ShapeFunctions() (ShapeFunctions.cpp:32)
 * and AssembleLumpedMass() (Mass3D.cpp:127). */
int ftgpu_setup(ftgpu_model *m);

/* Lumped mass per DOF, as AssembleLumpedMass() leaves mass[nDOF]. */
int ftgpu_get_mass(ftgpu_model *m, double *mass);

/* ---- symbol-compatible primitives (one call = one reference function) ---- */

/* GetForce() (GetForce.cpp:12-25 -> GetForce_3D.cpp:5-53) on displacements
 * u[nDOF] with the global dt used by the viscoelastic update: writes
 * fi[nDOF] (internal force) and, if non-NULL, f_net = -fi.  Viscoelastic
 * history advances exactly as one reference GetForce() call does. */
int ftgpu_get_force(ftgpu_model *m, const double *u, double dt, double *fi, double *f_net);

/* StableTimeStep() (StableTimeStep.cpp:4-40) on displacements u[nDOF]:
 * min over elements (elements whose nodes are all fully constrained are
 * skipped) of characteristic length / dilatational wave speed. */
int ftgpu_stable_time_step(ftgpu_model *m, const double *u, double *dt_min);

/* Per-Gauss-point F (column-major 9), detF and PK2 (Voigt 11,22,33,23,13,12)
 * of the last ftgpu_get_force call, in the reference's element order and
 * Gauss-point order (fptr/detFptr/pk2ptr layout of ShapeFunctions.cpp). */
int ftgpu_get_gauss_points(ftgpu_model *m, double *F, double *detF, double *pk2);

/* Number of Gauss points (8 per C3D8, 1 per C3D4). */
int ftgpu_num_gauss_points(ftgpu_model *m);

/* ---- device-resident explicit loop (fast mode) ---- */

/* Initial state (AoS [nDOF], any may be NULL = zero) and start time. */
int ftgpu_set_state(ftgpu_model *m, const double *u, const double *v, const double *a,
                    double time);

/* The pre-loop sequence of examples/ex9/ex9.cpp:81-93: apply BCs at t0,
 * dt = reduction * StableTimeStep(), GetForce(), CalculateAccelerations().
 * reduction / failure_dt / tmax apply to every instance not configured by
 * ftgpu_set_instances. */
int ftgpu_init_explicit(ftgpu_model *m, double reduction, double failure_dt, double tmax);

/* Advance every instance by up to max_steps central-difference steps
 * (ex9.cpp:107-175) or until Time >= tMax; the loop runs on the device as
 * CUDA graphs of 16 steps and, at the end of the run, one of 2-14 steps.
 * *steps_done = steps taken by instance 0. */
int ftgpu_run(ftgpu_model *m, int max_steps, int *steps_done);

/* ftgpu_run with CUDA events recorded on the model's stream around the whole
 * run: *device_ms is the device time of the steps taken. */
int ftgpu_run_timed(ftgpu_model *m, int max_steps, int *steps_done, double *device_ms);

/* ftgpu_run with an event before and after every element pass and nodal pass
 * of every step: *elem_ms / *node_ms are the summed device times of the
 * element kernels (all groups) and of the nodal kernel. */
int ftgpu_run_profiled(ftgpu_model *m, int max_steps, int *steps_done, double *elem_ms,
                       double *node_ms);

/* Measured FP32 FMA throughput of `device` (TFLOP/s, FMA = 2 flops): 16
 * independent FMA chains per thread on every SM, best of five launches timed
 * with CUDA events.  The denominator of the element pass's FP32 fraction
 * (no counterpart in the reference, which has no GPU code). */
int ftgpu_fp32_fma_peak(int device, double *tflops, double *ms_best);

/* Number of element patches (thread blocks of one element pass) and of node
 * slots (patch-local node replicas): the sizes the traffic model uses. */
int ftgpu_layout_info(ftgpu_model *m, long long *npatch, long long *nslots, int *ngroups);

/* State after the last completed step, AoS [nDOF] (any pointer may be NULL),
 * plus the instance-0 time, next dt and step count. */
int ftgpu_get_state(ftgpu_model *m, double *u, double *v, double *a, double *time, double *dt,
                    long long *step);

/* Per-instance time / next dt / steps / done flag (arrays of ninst). */
int ftgpu_get_instance_clock(ftgpu_model *m, double *time, double *dt, long long *step,
                             int *done);

/* Number of kernel launches one step issues (element groups + nodal update). */
int ftgpu_launches_per_step(ftgpu_model *m);

/* Synchronise and return the device error word (0 = none). */
int ftgpu_check(ftgpu_model *m);

/* ---- element strain (output steps) ----
 * CalculateStrain() + CalculateMaximumPrincipalStrain()
 * (src/elements/ElementCalculations/CalculateStrain.cpp:8-97) on the model's
 * current displacements: per element the Gauss-point average of the
 * Green-Lagrange strain Eavg[9*e .. 9*e+8] (column-major 3x3, the layout of
 * the reference's Eavg global that WriteVTU writes), the largest principal
 * strain clamped at >= 0, the smallest clamped at <= 0 and the largest shear
 * strain (max - min) / 2, in the reference's element order.  Any output may
 * be NULL. */
int ftgpu_element_strain(ftgpu_model *m, double *Eavg, double *ps_max, double *ps_min,
                         double *shear_max);

/* ---- per-step injury criteria (brain drivers) ----
 * CalculateInjuryCriterions (examples/ex5/ex5.cpp:1311-1430), called after
 * every step of the brain drivers, for the elements element_ids[0..n)
 * (elementIDInjury of ex5.cpp:1248-1280): principal strains of each listed
 * element (CalculateMaximumPrincipalStrain), running extremes with element and
 * time, sticky flags, and the largest 95th percentiles of the maximum
 * principal strain (MPS95) and of MPS x its rate, with the elements at or above
 * them when each maximum was set.  PS_Old starts at 0.  Kept on the device
 * inside the loop; set after ftgpu_setup, before ftgpu_init_explicit (it
 * resets the loop); n = 0 turns it off.  Single-instance models only. */
typedef struct ftgpu_injury {
  double max_strain, max_strain_time, min_strain, min_strain_time;
  double max_shear, max_shear_time, max_psxsr, max_psxsr_time;
  int max_strain_elem, min_strain_elem, max_shear_elem, max_psxsr_elem;
  double mps95, mps95_time, mpsxsr95, mpsxsr95_time;
  int mps95_count, mpsxsr95_count;
  long long steps;
} ftgpu_injury;
#define FTGPU_INJ_MPS15 1    /* MPS > 0.15 at some step (CSDM-15)   */
#define FTGPU_INJ_MPS30 2    /* MPS > 0.30 (CSDM-30)                 */
#define FTGPU_INJ_PSR120 4   /* MPS rate > 120 /s                    */
#define FTGPU_INJ_PSXSR28 8  /* MPS x rate > 28 /s                   */
#define FTGPU_INJ_MPS95 16   /* in the MPS95 element list            */
#define FTGPU_INJ_PSXSR95 32 /* in the MPS x rate 95 element list    */
int ftgpu_set_injury(ftgpu_model *m, int n, const int *element_ids);
/* the record, per listed element the flag bits above and the last MPS;
 * any output may be NULL */
int ftgpu_get_injury(ftgpu_model *m, ftgpu_injury *out, int *flags, double *mps);

/* ---- energy balance of the explicit loop ----
 * CheckEnergy() (src/fem/SolidMechanics/CheckEnergy.cpp:3-85), which every
 * example driver calls after each step (examples/ex9/ex9.cpp:154-156): per
 * step the kinetic energy 1/2 sum m v^2, the internal work increment
 * 1/2 sum du (f_prev + f) and the work of the reactions of constrained DOFs
 * (no external forces on this path), accumulated from the start of the loop.
 * Fused into the nodal step (one extra launch per step for the fixed-order
 * reduction).  ftgpu_set_energy after ftgpu_setup, before
 * ftgpu_init_explicit (it resets the loop); single-instance models only. */
int ftgpu_set_energy(ftgpu_model *m, int enable);
/* cumulative internal and external work, the last step's kinetic energy, the
 * largest |WKE + Wint - Wext| / max(|Wint|, |Wext|, |WKE|) seen and the number
 * of steps where it exceeded 1 % (the reference's "Energy Violation" warning) */
int ftgpu_get_energy(ftgpu_model *m, double *internal_work, double *external_work,
                     double *kinetic_energy, double *max_violation, long long *violations);

/* ---- rigid-body motion from sampled accelerations (the brain drivers' skull
 * boundary condition: InitBoundaryCondition's tables, ex5.cpp:574-720, the
 * odeint Dormand-Prince 5(4) integrator state, ex5.cpp:100-105 and 886-890,
 * computeDerivatives, ex5.cpp:976-1020, and ApplyAccBoundaryConditions,
 * ex5.cpp:339-392, which this replaces) ----
 * Channels 0-2: angular acceleration about x, y, z (rad/s^2); 3-5: linear
 * acceleration along x, y, z (m/s^2); channel k has npts[k] >= 1 samples
 * times[k][j] (s, non-decreasing), values[k][j], read as interpolateLinear
 * (math.cpp:99-119) does.  Positions rotate about centre (NULL = the origin,
 * where ex5 has moved the sensor point by TransformMesh).  Every DOF of the
 * instance whose function has kind FTGPU_BCK_RIGID follows the motion.  Each
 * step integrates the 12-state ODE once from Time - dt over dt, starting from
 * zero state and zero derivative at ftgpu_init_explicit.  After ftgpu_setup,
 * before ftgpu_init_explicit; npts = NULL removes the instance's records. */
int ftgpu_set_rigid_body(ftgpu_model *m, int inst, const int *npts, const double *const *times,
                         const double *const *values, const double *centre);
/* integrator state of an instance: y = [omega(3), r(3), v_cm(3), x_cm(3)]
 * (the reference's yInt) and yd = its derivative at the current time
 * (ydotInt); either may be NULL */
int ftgpu_get_rigid_body(ftgpu_model *m, int inst, double *y, double *yd);

/* ---- learned constitutive surrogate for material 7 (no counterpart in the
 * reference; it replaces the isochoric part of HGOIsotropicViscoelastic's
 * stress, HGOIsotropicViscoelastic.cpp:53-97, generalised to fibres) ----
 * An MLP 16(11 used)->128->128->128->8(6 used), SiLU, BF16 weights and
 * activations, FP32 accumulation, trained on the GPU on samples of the plain
 * law.  It predicts S_iso = S_lin + s0 out_scale |E|^2 NN(x) (S_lin: the
 * law's first-order model with its exact fibre switch; x: strain direction and
 * magnitude, fibre, fibre strain); the volumetric stress and the Prony
 * recurrence stay exact.  properties: the 9 material-7 parameters. */
typedef struct ftgpu_surrogate ftgpu_surrogate;
int ftgpu_surrogate_create(ftgpu_surrogate **out, int device, const double *properties,
                           unsigned long long seed);
int ftgpu_surrogate_destroy(ftgpu_surrogate *s);
/* nsamples states: random rotation, principal stretches in [lo, hi], random
 * fibre; targets normalised to unit RMS (the RMS becomes the output scale).
 * The sampled box should cover the trust region: |E_ii| <= sqrt(trust_e2). */
int ftgpu_surrogate_generate(ftgpu_surrogate *s, long long nsamples, unsigned long long seed,
                             double stretch_lo, double stretch_hi);
/* Adam (cosine-decayed lr) over the generated samples; *final_loss = last batch MSE */
int ftgpu_surrogate_train(ftgpu_surrogate *s, int epochs, int batch, double lr,
                          double *final_loss);
/* raw network outputs y[n][8] for features x[n][16] (host arrays) */
int ftgpu_surrogate_forward(ftgpu_surrogate *s, long long n, const float *x, float *y);
/* the same through the fused inference kernel used in the loop (tcgen05 MMAs,
 * FP32 accumulators in tensor memory) */
int ftgpu_surrogate_infer(ftgpu_surrogate *s, long long n, const float *x, float *y);
/* the same through a warp-level mma.sync kernel (a cross-check of the above) */
int ftgpu_surrogate_infer_mma(ftgpu_surrogate *s, long long n, const float *x, float *y);
/* Training GEMMs (forward, dX and dW of ftgpu_surrogate_train / _forward /
 * _gradient) on the tcgen05 tensor cores with TMEM accumulators
 * (tensor_cores = 1, the default) or on a warp-level mma.sync kernel (0, kept
 * as a cross-check).  No counterpart in the reference (no learned parts). */
int ftgpu_surrogate_gemm_path(ftgpu_surrogate *s, int tensor_cores);
/* MSE loss and its gradient w.r.t. the FP32 parameter vector for one batch */
int ftgpu_surrogate_gradient(ftgpu_surrogate *s, long long n, const float *x, const float *t,
                             float *grad, double *loss);
/* FP32 parameter vector out (get) and/or in (set); layout W0 b0 W1 b1 W2 b2 W3 b3 */
int ftgpu_surrogate_params(ftgpu_surrogate *s, float *get, const float *set);
/* the first n generated samples: features x[n][16], targets t[n][8] */
int ftgpu_surrogate_samples(ftgpu_surrogate *s, long long n, float *x, float *t);
int ftgpu_surrogate_num_params(void);
/* the RMS of the generated targets (1 before generation): network outputs are
 * in units of s0 * out_scale * |E|_F^2 */
int ftgpu_surrogate_output_scale(ftgpu_surrogate *s, double *out_scale);
/* predicted isochoric PK2 S[n][6] (Voigt 11 22 33 23 13 12) for Green strains
 * E[n][6] (same order, tensor shears) and unit fibres a0[n][3], through the
 * element kernel's features and the fused inference kernel */
int ftgpu_surrogate_predict(ftgpu_surrogate *s, long long n, const double *E, const double *a0,
                            double *S);
/* Use the surrogate for every material-7 element of the model (mixed
 * precision; after ftgpu_setup).  Gauss points with |E|_F^2 > trust_e2 fall
 * back to the plain law.  s = NULL detaches it. */
int ftgpu_set_surrogate(ftgpu_model *m, ftgpu_surrogate *s, double trust_e2);

/* ---- allocation-free internal force (no counterpart in the reference) ----
 * For callers that cannot let a library allocate device memory (they own all
 * of it, e.g. through their own pool, or run under a fixed budget): the C3D8
 * internal force fi of one material on caller-owned DEVICE arrays in the
 * reference layout -- coordinates[3*nNodes], connectivity[8*nelements],
 * u[3*nNodes], and the node -> element-corner map node_elem_ptr[nNodes+1] /
 * node_elem_ent[8*nelements] (entries e*8+corner in [0, 8*nelements),
 * summed in the given order; an entry outside that range returns
 * FTGPU_ERR_INPUT) -- written to fi[3*nNodes] (device).  properties: 9 host
 * doubles.  Materials 0, 1, 2, 3, 4 and 6 in FP64; 5 and 7 (they carry
 * viscoelastic history between calls) return FTGPU_ERR_INPUT, any other ID
 * FTGPU_ERR_MATERIAL.  No cudaMalloc/cudaFree: the corner-force scratch is a
 * static device array holding FTGPU_NOALLOC_MAX_ELEMENTS elements; larger
 * meshes are rejected with FTGPU_ERR_INPUT.  The first call on a device
 * looks up that array's address, which stays valid for the life of the
 * device's primary context.  The call reads its error word back and waits
 * for its stream, so it cannot be captured into a CUDA graph.  All calls
 * share the array, so calls that overlap on the GPU race. */
#define FTGPU_NOALLOC_MAX_ELEMENTS 32768
int ftgpu_hex8_force_noalloc(int nNodes, int nelements, const double *coordinates,
                             const int *connectivity, const int *node_elem_ptr,
                             const int *node_elem_ent, const double *u, int materialID,
                             const double *properties, double *fi, void *stream);

#ifdef __cplusplus
}
#endif
#endif
