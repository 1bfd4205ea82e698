/*
 * lbmpsm.h -- C ABI of the GB300 lattice-Boltzmann partially-saturated-cell
 * (PSM) library (liblbmpsm_gb300.so).
 *
 * The library replaces the LBM library behind the LAMMPS commands
 * `fix lbm-psm`, `fix lbm-psm-bc` and `fix lbm-psm-vti` of
 * timnajuch/LAMMPS-LBM-PSM.  The LAMMPS host keeps time integration,
 * neighbour lists, ghost atoms, reverse communication and the lubrication
 * pair style; each entry point below replaces one call site of the reference
 * (cited per function, paths relative to the reference repository).
 *
 * Conventions
 *   - Plain C types only; arrays of 3-vectors are row-major n x 3 (the
 *     layout of LAMMPS' contiguous double** atom arrays, pass x[0]).
 *   - Every function returns LBMPSM_OK (0) or a negative LBMPSM_ERR_* code;
 *     lbmpsm_last_error() gives the message.  Where the reference calls
 *     error->all() the library returns an error instead; nothing exits or
 *     throws across the ABI.
 *   - One handle = one lattice resident on one GPU, one CUDA stream.  Calls
 *     on a handle must come from one thread at a time.  Host-pointer calls
 *     are synchronous; *_device calls are asynchronous on the handle's stream.
 *   - Node layouts exchanged with the host follow the reference lattice
 *     (src/LBM_PSM_lattice.h:88-90): node (i*ny + j)*nz + k over the local
 *     array including the one-node halo, populations f[node*q + iq].
 */
#ifndef LBMPSM_H
#define LBMPSM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBMPSM_ABI_VERSION 1

/* status codes */
#define LBMPSM_OK 0
#define LBMPSM_ERR_ARG (-1)      /* "Illegal fix lbm-psm command" and bad arguments */
#define LBMPSM_ERR_MACH (-2)     /* Ma > 0.3 (src/fix_LBM_PSM.cpp:122-125) */
#define LBMPSM_ERR_GRID (-3)     /* domain / dx not integral (src/fix_LBM_PSM.cpp:135-140) */
#define LBMPSM_ERR_NOMEM (-4)    /* device or pinned host allocation failed */
#define LBMPSM_ERR_CUDA (-5)     /* a CUDA runtime call failed */
#define LBMPSM_ERR_STATE (-6)    /* call not valid in the handle's current state */
#define LBMPSM_ERR_CAPACITY (-7) /* more particle images than the handle was sized for, or a
                                   lbmpsm_export_fields_static request beyond
                                   LBMPSM_EXPORT_STATIC_MAX_BYTES */
#define LBMPSM_ERR_NUMERIC (-8)  /* non-finite populations or mass drift detected */
#define LBMPSM_ERR_TIMEOUT (-9)  /* a bounded device-side wait gave up */

/* population storage of the lattice */
#define LBMPSM_STORAGE_FP64 0 /* plain FP64, the reference arithmetic */
#define LBMPSM_STORAGE_FP32 1 /* FP32 deviations f_i - w_i*rho0, FP32 collision */
#define LBMPSM_STORAGE_FP16 2 /* FP16 scaled deviations, FP32 collision */
#define LBMPSM_STORAGE_BF16 3 /* BF16 deviations, FP32 collision */

/* `fix lbm-psm-bc` keywords (src/fix_LBM_PSM_BC.cpp:21-39) */
#define LBMPSM_BC_NONE 0
#define LBMPSM_BC_SHEAR 1
#define LBMPSM_BC_XFLOW 2
#define LBMPSM_BC_CHANNEL 3
#define LBMPSM_BC_CHANNEL_VELIN_PRESSOUT 4
#define LBMPSM_BC_CLOSEDBOX 5

/* PSM weighting B_n of the solid operator */
#define LBMPSM_WEIGHT_REFERENCE 0 /* B_n = eps_n, renormalised when sum > 1 (reference) */
#define LBMPSM_WEIGHT_NOBLE_TORCZYNSKI 1 /* B_n = eps_n(tau-1/2)/((1-eps_n)+(tau-1/2)) */

/* Launch shape of the FP32/FP16 collide kernel (no reference counterpart).
 * AUTO: at the start of the second step (the first step's map has filled the
 * particle table) the library times every candidate -- the row pipeline with
 * 3, 2, 4 or 5 shared-memory stages -- for a few even/odd step pairs on a
 * scratch copy of the populations and keeps the fastest (a few milliseconds,
 * one temporary population-sized allocation; skipped, and retried on the next
 * step, while the stream is being captured; the default shape is kept if the
 * allocation fails).  The candidates give bit-identical results.  DEFAULT:
 * the 3-stage pipeline, untimed.  The environment variable LBMPSM_PIPE_STAGES
 * (2..5 stages, or 0 = the direct kernel, which rows longer than 256 nodes
 * use anyway) overrides both. */
#define LBMPSM_TUNE_AUTO 0
#define LBMPSM_TUNE_DEFAULT 1

typedef struct lbmpsm_handle lbmpsm_handle;

/* Arguments of `fix lbm-psm` (src/fix_LBM_PSM.cpp:15-83) plus the LAMMPS
 * domain that fix_LBM_PSM::init() reads (src/fix_LBM_PSM.cpp:104-177). */
typedef struct {
  int dimension;   /* domain->dimension: 2 or 3 */
  double boxlo[3]; /* domain->boxlo */
  double prd[3];   /* domain->xprd, yprd, zprd */
  int periodic[3]; /* domain->xperiodic, yperiodic, zperiodic */
  int nevery;      /* every */
  int Nlc;         /* Nlc */
  double lc, rho, nu, Re;
  double tau;      /* tau (the fix's default is 0.7) */
  double Fext[3];  /* Fext fx fy fz (physical volume force) */
} lbmpsm_fix_params;

/* Options that have no counterpart in the reference (defaults: all zero). */
typedef struct {
  int storage;       /* LBMPSM_STORAGE_* */
  int device;        /* CUDA device ordinal */
  int max_images;    /* particle images per step the handle is sized for (0: 4096, grows
                        on host-pointer calls) */
  double max_radius; /* largest particle radius, physical units (0: derived per call on
                        host-pointer calls; required for *_device calls) */
  int psm_weighting; /* LBMPSM_WEIGHT_* */
  int collide_tuning; /* LBMPSM_TUNE_*: how the FP32/FP16 collide kernel's launch shape is chosen */
} lbmpsm_options;

/* Derived quantities of fix_LBM_PSM::init and UnitConversion
 * (src/LBM_PSM_unitConversion.cpp:15-38). */
typedef struct {
  int dimension, q;
  int nx, ny, nz;        /* global node counts as fix init computes them (nz = 0 in 2-D) */
  int local[3];          /* reference local array incl. halo: nx+2, ny+2, nz+2 (1 in 2-D) */
  int storage_dims[3];   /* device array extents (periodic axes carry no halo) */
  double dx, Uc, u_lb, tc, dt_d;
  double forceFactor, torqueFactor, volumeForceFactor;
  double dt_dem;         /* the DEM timestep fix init writes to update->dt */
  double Ma;
  double F_lbm[3];       /* lattice-unit body force */
  int64_t steps;         /* LBM steps done on this handle */
  size_t device_bytes;   /* device memory held by the handle */
  int collide_stages;    /* FP32/FP16 collide launch shape: pipeline stages, 0 = direct kernel
                            (-1 for FP64 storage) */
  int collide_blocks;    /* its grid (persistent blocks; 0 for the direct kernel) */
  float collide_tune_ms[4]; /* autotuner: ms per even+odd step pair of the shapes with 3, 2,
                            4 and 5 stages (-1: not timed or not fitting) */
} lbmpsm_info;

/* Replaces fix_LBM_PSM::init (src/fix_LBM_PSM.cpp:104-177): unit conversion,
 * Mach and grid checks, lattice allocation and initialisation to
 * equilibrium at rho = 1, u = 0.  opts may be NULL. */
int lbmpsm_create(const lbmpsm_fix_params* params, const lbmpsm_options* opts,
                  lbmpsm_handle** out);
/* Replaces ~fix_LBM_PSM (src/fix_LBM_PSM.cpp:86-93). */
void lbmpsm_destroy(lbmpsm_handle* h);
/* Text of the last error on this handle (or of the last failed create when
 * h is NULL).  Never NULL. */
const char* lbmpsm_last_error(const lbmpsm_handle* h);
int lbmpsm_get_info(const lbmpsm_handle* h, lbmpsm_info* info);

/* Replaces the keyword parsing of fix_LBM_PSM_BC (src/fix_LBM_PSM_BC.cpp:16-39)
 * and fix_LBM_PSM_BC::init (:145-148). */
int lbmpsm_set_bc(lbmpsm_handle* h, int bc_type);

/* One LBM coupling step for n particle images (locals then ghosts, LAMMPS
 * order), replacing the LBM branch of fix_LBM_PSM::post_force
 * (src/fix_LBM_PSM.cpp:197-229): setParticlesOnLattice
 * (src/LBM_PSM_exchangeParticleData.cpp:24-112), the halo exchange
 * (src/LBM_PSM_MPICOMM.h:79-147), macroCollideStream
 * (src/LBM_PSM_BGK_dynamics.cpp:81-109) and calculateHydrodynamicInteractions
 * per image (src/LBM_PSM_exchangeParticleData.cpp:172-244).
 * Inputs: tag[n], x/v/omega[n*3], radius[n] (physical units, host memory).
 * Outputs per image, physical units, before ghost bookkeeping: fh[n*3],
 * th[n*3], stresslet[n*6].  The caller applies f += fh (locals), f = fh
 * (ghosts), v_tally and reverse_comm exactly as the reference fix does. */
int lbmpsm_step(lbmpsm_handle* h, int n, const int* tag, const double* x, const double* v,
                const double* omega, const double* radius, double* fh, double* th,
                double* stresslet);
/* Same, with all arrays in device memory; asynchronous on the handle's
 * stream.  Requires opts.max_radius >= every radius.  The step reads the
 * image arrays in place (and keeps copies for lbmpsm_run_fixed); the outputs
 * (each may be NULL) are written by the step's own reduction, and the handle
 * keeps a copy as well (lbmpsm_read_forces).  The arrays may differ from
 * call to call. */
int lbmpsm_step_device(lbmpsm_handle* h, int n, const int* tag, const double* x,
                       const double* v, const double* omega, const double* radius, double* fh,
                       double* th, double* stresslet);
/* Zou-He boundaries of the selected `fix lbm-psm-bc` keyword on the
 * post-stream populations: replaces fix_LBM_PSM_BC::post_force
 * (src/fix_LBM_PSM_BC.cpp:151-402) and ZouHeBC (src/LBM_PSM_zou_he_BC.cpp:25-398).
 * Asynchronous on the handle's stream. */
int lbmpsm_apply_bc(lbmpsm_handle* h);

/* Macro fields.  The reference keeps rho and u arrays that macroCollideStream
 * refreshes every step (src/LBM_PSM_BGK_dynamics.cpp:48-77); here they are
 * written only by steps that follow a request, so that ordinary steps move
 * only populations.  WriteVTI::pre_force reads them one step later, so the
 * `fix lbm-psm-vti` caller requests them one LBM step before each write. */
int lbmpsm_request_macro(lbmpsm_handle* h);
/* Replaces the field read of WriteVTI::execute_write_vti
 * (src/fix_LBM_PSM_writeVTI.h:146-169): interior nodes, z outermost, x
 * innermost; solid = min(eps1+eps2, 1)*B0, rho*rho0, u*u0 (u_z = 0 in 2-D).
 * as_double selects double (1) or float (0) output arrays; any pointer may
 * be NULL.  Before the first requested step rho = 1 and u = 0, as after
 * initialise_dynamics. */
int lbmpsm_export_fields(lbmpsm_handle* h, int as_double, double B0, double rho0, double u0,
                         void* solid, void* rho, void* u);

/* Post-stream populations in the reference layout (local array with halo,
 * f[node*q+iq], FP64).  Replaces LBMPSMLattice::getVector_f_curr /
 * setVector_f_curr (src/LBM_PSM_lattice.cpp:250-252) as used by
 * `fix lbm-psm-restart` (src/fix_LBM_PSM_writeReadRestart.cpp:62,75).
 * Halo planes of periodic axes are returned as copies of the periodic twin
 * and ignored on input. */
int lbmpsm_get_populations(lbmpsm_handle* h, double* f);
int lbmpsm_set_populations(lbmpsm_handle* h, const double* f);
/* Particle table per node in the reference layout: ids[2N], eps[2N],
 * us[6N] (LBMPSMLattice::getParticleDataOnLatticeNode,
 * src/LBM_PSM_lattice.cpp:255).  Halo nodes of periodic axes read as empty.
 * FP64 storage keeps eps and us in FP64 (the reference's values bit for bit);
 * FP32 / FP16 storage keeps only their FP32 roundings, returned widened. */
int lbmpsm_get_particle_table(lbmpsm_handle* h, int* ids, double* eps, double* us);

/* Global FP64 check (no reference counterpart): total mass and momentum of
 * the stored nodes, and a status word that is non-zero if any population is
 * not finite.  Returns LBMPSM_ERR_NUMERIC in that case. */
int lbmpsm_check(lbmpsm_handle* h, double* mass, double* momentum3);

/* Block until all work queued on the handle's stream is done. */
int lbmpsm_synchronize(lbmpsm_handle* h);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their
 * own device work after *_device calls. */
void* lbmpsm_stream(lbmpsm_handle* h);
/* 1 when lbmpsm_step works on the caller's host arrays in place: the device
 * reads pageable host memory through the host's page tables (NVLink-C2C on
 * Grace), so the step's image preparation reads the images and its reduction
 * writes fh, th and stresslet with no staging copies; 0 when the images are
 * staged through pinned memory and copied (devices without that access, or
 * the environment variable LBMPSM_HOST_STAGING=1 at lbmpsm_create); -1 for
 * a NULL handle.  Both give the same results bit for bit.  Single-box
 * handles only: lbmpsm_step_batch always stages. */
int lbmpsm_host_direct(const lbmpsm_handle* h);

/* Run nsteps coupling steps with the particle images already on the device
 * (as last passed to lbmpsm_step or lbmpsm_step_device), fixed in place,
 * each step followed by the boundary condition when one is set.  The step
 * sequence is captured once into a CUDA graph and replayed.  The forces of
 * each step land in the handle's own buffers (read with lbmpsm_read_forces). */
int lbmpsm_run_fixed(lbmpsm_handle* h, int nsteps);
/* Copy the per-image outputs of the last step to host memory. */
int lbmpsm_read_forces(lbmpsm_handle* h, int n, double* fh, double* th, double* stresslet);

/* Batched ensemble: nbox independent lattices ("boxes") that share the
 * lattice geometry (dimension, domain lengths, periodicity, lattice spacing)
 * but each have their own fix parameters (tau, rho, nu, Re, Fext, boxlo),
 * held in one allocation and advanced by one set of kernels per step (the
 * boxes are stacked along z on the device, each wrapping within itself).
 * One such box per LAMMPS run is what `fix lbm-psm` describes
 * (src/fix_LBM_PSM.cpp:104-177); the ensemble has no counterpart in the
 * reference.  Boundary conditions are not available for nbox > 1.
 * params points to nbox structures.  A handle from lbmpsm_create is an
 * ensemble of one box. */
int lbmpsm_create_batch(int nbox, const lbmpsm_fix_params* params, const lbmpsm_options* opts,
                        lbmpsm_handle** out);
/* lbmpsm_step for an ensemble: box[i] is the box of image i, and its
 * position is in that box's own frame.  Outputs per image as lbmpsm_step. */
int lbmpsm_step_batch(lbmpsm_handle* h, int n, const int* box, const int* tag, const double* x,
                      const double* v, const double* omega, const double* radius, double* fh,
                      double* th, double* stresslet);
/* The box that lbmpsm_get/set_populations, lbmpsm_export_fields and
 * lbmpsm_get_particle_table address (default 0). */
int lbmpsm_select_box(lbmpsm_handle* h, int box);

/* Allocation-free variant of lbmpsm_export_fields; no counterpart in the
 * reference.  For callers that cannot allocate device memory while a run is
 * under way: a host program whose pool allocator already holds nearly all of
 * HBM, or one whose other streams on the GPU must not be stalled by the
 * device-wide wait of cudaFree.  Same arguments and output as
 * lbmpsm_export_fields, staged through one fixed device array of
 * LBMPSM_EXPORT_STATIC_MAX_BYTES that every GPU loading the library holds
 * until exit; the requested fields must fit in it (float output: 4 bytes per
 * node per component, double 8; solid and rho one component, u three),
 * otherwise the call returns LBMPSM_ERR_CAPACITY and allocates nothing.  The
 * first call on each device looks up the array's device address; make it
 * before any stream capture begins.  Calls share the array; the library
 * serialises them with a process-wide lock held until each call's copies
 * have finished.  Synchronous, like lbmpsm_export_fields. */
#define LBMPSM_EXPORT_STATIC_MAX_BYTES (64u * 1024u * 1024u)
int lbmpsm_export_fields_static(lbmpsm_handle* h, int as_double, double B0, double rho0,
                                double u0, void* solid, void* rho, void* u);

/* Groups of lattices stepped together (no reference counterpart).  Boxes of
 * one geometry share an ensemble handle (lbmpsm_create_batch); boxes of other
 * sizes need their own handles.  A group advances several handles as one:
 * lbmpsm_group_run_fixed runs nsteps steps of every member exactly as
 * lbmpsm_run_fixed would (each with the images it holds from its last step,
 * each with its boundary condition), with one step of all members captured
 * once per A-A parity into a single CUDA graph whose branches run
 * concurrently, so that every step is one graph launch.  Members must be on
 * one device and at the same step parity; a member with a macro-field store
 * pending is rejected (LBMPSM_ERR_STATE).  The group's work is ordered after
 * the members' earlier work and before their later work.  Destroy the group
 * before its members. */
typedef struct lbmpsm_group lbmpsm_group;
int lbmpsm_group_create(lbmpsm_handle* const* handles, int count, lbmpsm_group** out);
/* When every member is 3-D and periodic on every axis, the members share
 * storage precision and PSM weighting, either all or none have a body force,
 * there are at most 16 members and (FP32/FP16/BF16 storage) no x-row is longer
 * than 96 nodes, the collide of all members is ONE persistent launch per
 * step: its blocks walk tiles of one to several x-rows of every member (small
 * boxes pack several rows per tile) and run each member's own node collision,
 * so the results equal the members' own steps bit for bit.  The maps, faces
 * and reductions of the members run as concurrent graph branches before and
 * after it.  Otherwise each member keeps its own collide launch.  The
 * environment variable LBMPSM_GROUP_FUSE=0 keeps the per-member launches. */
int lbmpsm_group_run_fixed(lbmpsm_group* g, int nsteps);
/* Collide launches per step of the group's current graphs: 1 when fused,
 * the member count otherwise, -1 before the first run. */
int lbmpsm_group_collide_launches(const lbmpsm_group* g);
/* The group's tuner: the first lbmpsm_group_run_fixed call with at least 8
 * steps, on members that qualify for one collide launch, runs two steps of
 * each plan untimed (capturing their graphs) and two timed, then keeps the
 * faster plan for the rest of the group's life (both give the same results
 * bit for bit).  ms[0] = per-member launches, ms[1] = one launch, in ms per
 * step (-1: not timed).  LBMPSM_GROUP_FUSE=0 / =1 fixes the plan instead. */
int lbmpsm_group_tune_ms(const lbmpsm_group* g, float* ms);
void* lbmpsm_group_stream(lbmpsm_group* g); /* the cudaStream_t the group's graphs run on */
const char* lbmpsm_group_last_error(const lbmpsm_group* g);
void lbmpsm_group_destroy(lbmpsm_group* g);

/* Sensitivities of the time-averaged drag (the reference has
 * no adjoint; the forward step is lbmpsm_step's).  Both calls run nsteps
 * ordinary coupling steps with one fixed set of particle images -- exactly
 * the launches of nsteps lbmpsm_step calls with these arrays, so the lattice
 * ends where those calls leave it -- and differentiate
 *
 *   J = 1/M * sum_{t=t0..t1} sum_images  direction . F_image(t),  M = t1-t0+1,
 *
 * F_image the hydrodynamic force lbmpsm_step returns at step t (steps
 * numbered 1..nsteps from the call).  Parameters: tau (the relaxation time,
 * with the unit factors of lbmpsm_get_info held fixed), Fext (as in
 * lbmpsm_fix_params) and the image centres.  The solid fraction of a node is
 * a sub-cell count (calcSolidFraction), piecewise constant in the centre;
 * its centre derivative is taken as the central difference of that count at
 * +-centre_step (physical units), the quantity a central finite difference of
 * J with that step sees to first order.  Ghost images carry their own rows:
 * sum them into their owner like forces.
 *
 * Needs FP64 storage, one box, every axis periodic and no boundary
 * condition; a node in the surface shells of more than two particles, or of
 * two images of one particle, is rejected (LBMPSM_ERR_ARG).  Both calls
 * allocate their scratch on entry and free it on return.
 *
 * lbmpsm_adjoint_drag: reverse sweep.  The state before every
 * checkpoint_every-th step is kept in HBM; the reverse pass recomputes each
 * segment from its checkpoint.  Device memory: (nsteps/checkpoint_every +
 * checkpoint_every + 1) population arrays (FP64, Q per node).  Outputs (any
 * may be NULL except dJ_dx when n > 0): J; dJ/dtau; dJ/dFext[3]; dJ/dx[3n]
 * per image row; the total drag along direction of every step [nsteps].
 *
 * lbmpsm_tangent_drag: forward-mode sweep along (dtau, dFext[3], dx[3n]);
 * dFext and dx may be NULL (zero).  Outputs J and dJ = grad J . direction. */
int lbmpsm_adjoint_drag(lbmpsm_handle* h, int n, const int* tag, const double* x,
                        const double* v, const double* omega, const double* radius, int nsteps,
                        int t0, int t1, const double* direction, int checkpoint_every,
                        double centre_step, double* J, double* dJ_dtau, double* dJ_dFext,
                        double* dJ_dx, double* drag_per_step);
int lbmpsm_tangent_drag(lbmpsm_handle* h, int n, const int* tag, const double* x,
                        const double* v, const double* omega, const double* radius, int nsteps,
                        int t0, int t1, const double* direction, double centre_step,
                        double dtau, const double* dFext, const double* dx, double* J,
                        double* dJ);

#ifdef __cplusplus
}
#endif
#endif
