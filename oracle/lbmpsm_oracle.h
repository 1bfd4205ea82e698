/*
 * lbmpsm_oracle.h -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * C interface shared by the two CPU oracles of the LBM-PSM hot path:
 *   - liblbmpsm_oracle.so : a plain-C restatement of the reference algorithm
 *                           (oracle/lbmpsm_oracle.c), built on any host;
 *   - _ref/libref_oracle.so: the reference's own unmodified LBM_PSM_*.cpp
 *                           sources compiled against stub LAMMPS/MPI headers
 *                           (oracle/ref/), built only where the reference
 *                           sources are present.
 * Both export exactly these symbols so that tests can run the same case
 * through either and compare them bit for bit.
 *
 * Only tests/, the smoke check and bench.py's CPU-baseline leg may load
 * these libraries; the product path never does.
 *
 * Units/arguments follow `fix lbm-psm` (src/fix_LBM_PSM.cpp:15-83) and the
 * LAMMPS domain it reads in init() (src/fix_LBM_PSM.cpp:104-177).  Layouts
 * follow the reference lattice (src/LBM_PSM_lattice.h:88-90): node index
 * (i*ny + j)*nz + k over the local array INCLUDING the one-node halo, and
 * populations as f[node*q + iq].
 */
#ifndef LBMPSM_ORACLE_H
#define LBMPSM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

typedef struct {
  int dimension;        /* 2 or 3 (domain->dimension) */
  double boxlo[3];      /* domain->boxlo */
  double prd[3];        /* domain->xprd/yprd/zprd */
  int periodic[3];      /* domain->x/y/zperiodic */
  /* fix lbm-psm keywords */
  int nevery;
  int Nlc;
  double lc, rho, nu, Re, tau;
  double Fext[3];
  /* fix lbm-psm-bc keyword: 0 none, 1 shear, 2 xFlow, 3 channel,
   * 4 channel-velIn-pressOut, 5 closedBox (src/fix_LBM_PSM_BC.cpp:21-39) */
  int bc_type;
} orc_params;

typedef struct {
  int nx, ny, nz;       /* local array size INCLUDING halo (nz = 1 in 2-D) */
  int q;
  double dx, Uc, u_lb, tc, dt_d;
  double forceFactor, torqueFactor, volumeForceFactor;
  double dt_dem;        /* update->dt set by fix init */
  double Ma;
  double F_lbm[3];
} orc_info;

/* Error codes returned where the reference calls error->all(). */
#define ORC_OK 0
#define ORC_ERR_ARG (-1)
#define ORC_ERR_MACH (-2)
#define ORC_ERR_GRID (-3)
#define ORC_ERR_NOMEM (-4)

int orc_create(const orc_params* p, orc_sim** out);
void orc_destroy(orc_sim* s);
int orc_get_info(const orc_sim* s, orc_info* info);
/* Worker threads for the collide-stream and force loops (restatement only;
 * the reference build ignores it).  Results do not depend on it. */
void orc_set_threads(orc_sim* s, int nthreads);

/* One LBM coupling step as fix_LBM_PSM::post_force performs it on a
 * single rank (src/fix_LBM_PSM.cpp:197-264) for n particle images
 * (locals then ghosts, LAMMPS order):
 *   setParticlesOnLattice -> halo exchange -> macroCollideStream ->
 *   calculateHydrodynamicInteractions per image.
 * Outputs are per image, before any ghost bookkeeping: fh[3n], th[3n],
 * stresslet[6n].  x, v, omega are row-major n x 3. */
int orc_step(orc_sim* s, int n, const int* tag, const double* x, const double* v,
             const double* omega, const double* radius, double* fh, double* th,
             double* stresslet);
/* The sub-steps of orc_step, for finer-grained comparisons. */
int orc_map(orc_sim* s, int n, const int* tag, const double* x, const double* v,
            const double* omega, const double* radius);
int orc_collide_stream(orc_sim* s); /* halo exchange + macroCollideStream */
int orc_reduce(orc_sim* s, int n, const int* tag, const double* x, const double* radius,
               double* fh, double* th, double* stresslet);
/* fix_LBM_PSM_BC::post_force (src/fix_LBM_PSM_BC.cpp:151-402) */
int orc_apply_bc(orc_sim* s);

/* State read-back (reference layouts, halo included). */
int orc_get_f(const orc_sim* s, double* f);            /* nx*ny*nz*q */
int orc_set_f(orc_sim* s, const double* f);
int orc_get_macro(const orc_sim* s, double* rho, double* u); /* N, 3N */
/* pData: ids[2N], eps[2N], us[6N], F[6N] (per node, slot-major inside) */
int orc_get_pdata(const orc_sim* s, int* ids, double* eps, double* us, double* F);
/* Field read of execute_write_vti (src/fix_LBM_PSM_writeVTI.h:146-169):
 * interior nodes, z outermost, x innermost; solid = min(eps1+eps2, 1)*B0,
 * rho*rho0, u*u0.  Returns the number of points written. */
int orc_export_fields(const orc_sim* s, double B0, double rho0, double u0, double* solid,
                      double* rho, double* u);

/* The file output of `fix lbm-psm-vti` on one process (vti_oracle.c, in the
 * restatement library only): execute_write_vti<T>
 * (src/fix_LBM_PSM_writeVTI.h:82-253) writing the piece and the master file
 * for double fields solid, rho (one per interior node) and u (three). */
int orc_write_vti(const char* folder, const char* name, int timestep, int binary, int use_double,
                  int dimension, const int* local, const double* origin, double dx,
                  const double* solid, const double* rho, const double* u);

/* ---- LAMMPS single-rank emulation (not part of the reference sources) ----
 * Ghost images as CommBrick::borders() creates them on one process with
 * periodic axes: per dimension x,y,z, first the atoms with
 * coord <= lo+cutghost are imaged at +prd, then the atoms with
 * coord >= hi-cutghost at -prd; both swaps of a dimension scan the same
 * range (locals plus ghosts of earlier dimensions).  Non-periodic axes and
 * z in 2-D make no ghosts.
 * On input the first nlocal rows of every array hold the owned atoms; the
 * arrays must have room for max_images rows.  Returns the total number of
 * images (nlocal + nghost), or -1 if max_images is too small.  owner[i] is
 * the index of the image that image i was copied from (i for locals);
 * swap[i] is the swap that created it (-1 for locals). */
int orc_make_ghosts(int dimension, const double* boxlo, const double* prd, const int* periodic,
                    double cutghost, int nlocal, int max_images, int* tag, double* x, double* v,
                    double* omega, double* radius, int* owner, int* swap);
/* comm->reverse_comm() on one rank: walk the swaps in reverse order and add
 * each ghost's row into the image it was copied from.  vals is n x width. */
void orc_reverse_comm(int n, int nlocal, const int* owner, const int* swap, int width,
                      double* vals);

#ifdef __cplusplus
}
#endif
#endif
