/*
 * lbmpsm_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C restatement of the reference LBM-PSM hot path
 * (timnajuch/LAMMPS-LBM-PSM, src/LBM_PSM_*.cpp and the two fixes that drive
 * it), kept in the reference's own data layout: FP64 array-of-structures
 * populations with a one-node halo, push streaming into a ping-pong buffer,
 * and the per-node two-slot particle table.  Every floating-point
 * expression keeps the reference's operand order so that, built with
 * -ffp-contract=off, the results are bit-identical to the reference compiled
 * from its own sources (checked by tests/test_oracle_pin.py against
 * oracle/_ref/libref_oracle.so and the committed golden fixtures).
 *
 * It is the checker of the CUDA path and the timed CPU baseline of
 * bench.py; the product library never links or calls it.
 */
#include "lbmpsm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int id[2];
  double eps[2];
  double us[6];
  double F[6];
} orc_pdata;

typedef struct {
  double nu_lb, dx, dx_d, Uc, u_lb, dt_d, tc;
  double forceFactor, torqueFactor, volumeForceFactor;
} orc_units;

struct orc_sim {
  int dim, q;
  int nx, ny, nz; /* local sizes with halo */
  int periodic[3];
  double origin[3];
  double prd[3];
  double rho_phys;
  int nevery;
  orc_units un;
  double tau, omega;
  double F_lbm[3];
  double F_mag2;
  double invCsPow2, invCsPow4;
  double w[19];
  int ex[19], ey[19], ez[19];
  double* f_curr;
  double* f_next;
  double* rho;
  double* u;
  orc_pdata* pd;
  int bc_type;
  int nthreads;
};

/* Velocity sets: src/LBM_PSM_lattice.h:186-209. */
static const int D2Q9_ex[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int D2Q9_ey[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int D3Q19_ex[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
static const int D3Q19_ey[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
static const int D3Q19_ez[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};

static inline long nidx(const orc_sim* s, int i, int j, int k) {
  return ((long)i * s->ny + j) * s->nz + k;
}

/* UnitConversion::UnitConversion (src/LBM_PSM_unitConversion.cpp:15-38). */
static void units_init(orc_units* u, double rhof, double nu, double lc, double Re, int N,
                       double tau) {
  double Uc_d = 1.0, Lc_d = 1.0;
  double csPow2 = 1.0 / 3.0;
  u->nu_lb = (tau - 0.5) * csPow2;
  u->dx = lc / (double)(N - 1);
  u->dx_d = Lc_d / (double)(N - 1);
  u->Uc = Re * nu / lc;
  u->u_lb = Re * u->nu_lb / (double)(N - 1);
  u->dt_d = u->dx_d * u->u_lb / Uc_d;
  u->tc = lc / u->Uc;
  u->forceFactor = rhof * pow(lc, 4) / pow(u->tc, 2) * pow(u->dx_d, 4) / pow(u->dt_d, 2);
  u->torqueFactor = rhof * pow(lc, 5) / pow(u->tc, 2) * pow(u->dx_d, 5) / pow(u->dt_d, 2);
  u->volumeForceFactor = rhof * lc / pow(u->tc, 2) * u->dx_d / pow(u->dt_d, 2);
}

/* LBMPSMDynamics::feq, node overload (src/LBM_PSM_dynamics.h:43-59). */
static inline double feq_node(const orc_sim* s, int iq, double rho, const double* u) {
  const double ex_i = s->ex[iq], ey_i = s->ey[iq], ez_i = s->ez[iq];
  const double w_i = s->w[iq];
  const double ux = u[0], uy = u[1], uz = u[2];
  double eiq_dot_u = ex_i * ux + ey_i * uy + ez_i * uz;
  return rho * w_i *
         (1.0 + eiq_dot_u * s->invCsPow2 + eiq_dot_u * eiq_dot_u * 0.5 * s->invCsPow4 -
          0.5 * (ux * ux + uy * uy + uz * uz) * s->invCsPow2);
}

/* LBMPSMDynamics::feq, std::array overload (src/LBM_PSM_dynamics.h:72-85). */
static inline double feq_arr(const orc_sim* s, int iq, double rho, const double* u) {
  const double ex_i = s->ex[iq], ey_i = s->ey[iq], ez_i = s->ez[iq];
  const double eiq_dot_u = ex_i * u[0] + ey_i * u[1] + ez_i * u[2];
  const double u_dot_u = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  return rho * s->w[iq] *
         (1.0 + eiq_dot_u * s->invCsPow2 + 0.5 * eiq_dot_u * eiq_dot_u * s->invCsPow4 -
          0.5 * u_dot_u * s->invCsPow2);
}

/* LBMPSMDynamics::F_iq, node overload (src/LBM_PSM_dynamics.h:102-116). */
static inline double F_iq(const orc_sim* s, int iq, const double* u, const double* F) {
  double ex_i = s->ex[iq], ey_i = s->ey[iq], ez_i = s->ez[iq];
  double w_i = s->w[iq];
  double ux = u[0], uy = u[1], uz = u[2];
  return w_i * (((ex_i - ux) * F[0] + (ey_i - uy) * F[1] + (ez_i - uz) * F[2]) * s->invCsPow2 +
                ((ex_i * ux + ey_i * uy + ez_i * uz) * s->invCsPow4 *
                 (ex_i * F[0] + ey_i * F[1] + ez_i * F[2])));
}

/* fix_LBM_PSM::init (src/fix_LBM_PSM.cpp:104-177) with the lattice
 * construction it triggers: LBMPSMLattice ctor (src/LBM_PSM_lattice.cpp:16-118),
 * initialise_domain (:142-186), LBMPSMDynamics ctor
 * (src/LBM_PSM_dynamics.cpp:15-34), initialise_dynamics
 * (src/LBM_PSM_BGK_dynamics.cpp:22-44).  One rank, no decomposition. */
int orc_create(const orc_params* p, orc_sim** out) {
  *out = NULL;
  if (!p || (p->dimension != 2 && p->dimension != 3)) return ORC_ERR_ARG;
  if (p->nevery <= 0 || p->Nlc <= 0 || p->lc <= 0.0 || p->rho <= 0.0 || p->nu <= 0.0 ||
      p->Re <= 0.0 || p->tau <= 0.5)
    return ORC_ERR_ARG;
  if (p->bc_type < 0 || p->bc_type > 5) return ORC_ERR_ARG;
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  if (!s) return ORC_ERR_NOMEM;
  s->dim = p->dimension;
  s->nevery = p->nevery;
  s->rho_phys = p->rho;
  s->bc_type = p->bc_type;
  s->nthreads = 1;
  for (int d = 0; d < 3; ++d) {
    s->periodic[d] = p->periodic[d];
    s->prd[d] = p->prd[d];
  }
  units_init(&s->un, p->rho, p->nu, p->lc, p->Re, p->Nlc, p->tau);

  double Ma = s->un.u_lb / (1.0 / sqrt(3.0));
  if (Ma > 0.3) {
    free(s);
    return ORC_ERR_MACH;
  }
  double SMALL = 1e-15;
  double dx = s->un.dx;
  if (pow(((double)((int)(p->prd[0] / dx + 0.5)) - p->prd[0] / dx), 2.0) > SMALL ||
      pow(((double)((int)(p->prd[1] / dx + 0.5)) - p->prd[1] / dx), 2.0) > SMALL ||
      pow(((double)((int)(p->prd[2] / dx + 0.5)) - p->prd[2] / dx), 2.0) > SMALL) {
    free(s);
    return ORC_ERR_GRID;
  }
  int gnx = p->prd[0] / dx + 1.5;
  if (p->periodic[0]) gnx -= 1;
  int gny = p->prd[1] / dx + 1.5;
  if (p->periodic[1]) gny -= 1;
  int gnz = 0;
  if (p->dimension == 3) {
    gnz = p->prd[2] / dx + 1.5;
    if (p->periodic[2]) gnz -= 1;
  }
  s->origin[0] = p->boxlo[0];
  s->origin[1] = p->boxlo[1];
  s->origin[2] = p->boxlo[2];
  if (p->dimension == 2) s->origin[2] = 0.0;
  /* UnitConversion::get_volume_force_lb (src/LBM_PSM_unitConversion.cpp:81-88) */
  for (int d = 0; d < 3; ++d) s->F_lbm[d] = p->Fext[d] / s->un.volumeForceFactor;

  s->tau = p->tau;
  s->omega = 1.0 / p->tau;
  /* lattice sizes on one rank: n + 2*envelopeWidth; nz = 1 in 2-D */
  s->nx = gnx + 2;
  s->ny = gny + 2;
  s->nz = (p->dimension == 3) ? gnz + 2 : 1;
  {
    double csPow2 = 1.0 / 3.0;
    double csPow4 = csPow2 * csPow2;
    s->invCsPow2 = 1.0 / csPow2;
    s->invCsPow4 = 1.0 / csPow4;
  }
  if (p->dimension == 2) {
    s->q = 9;
    for (int i = 0; i < 9; ++i) {
      s->ex[i] = D2Q9_ex[i];
      s->ey[i] = D2Q9_ey[i];
      s->ez[i] = 0;
    }
    s->w[0] = 4.0 / 9.0;
    for (int i = 1; i < 5; ++i) s->w[i] = 1.0 / 9.0;
    for (int i = 5; i < 9; ++i) s->w[i] = 1.0 / 36.0;
  } else {
    s->q = 19;
    for (int i = 0; i < 19; ++i) {
      s->ex[i] = D3Q19_ex[i];
      s->ey[i] = D3Q19_ey[i];
      s->ez[i] = D3Q19_ez[i];
    }
    s->w[0] = 1.0 / 3.0;
    for (int i = 1; i < 7; ++i) s->w[i] = 1.0 / 18.0;
    for (int i = 7; i < 19; ++i) s->w[i] = 1.0 / 36.0;
  }
  long N = (long)s->nx * s->ny * s->nz;
  s->f_curr = (double*)malloc(sizeof(double) * N * s->q);
  s->f_next = (double*)malloc(sizeof(double) * N * s->q);
  s->rho = (double*)calloc(N, sizeof(double));
  s->u = (double*)calloc(3 * N, sizeof(double));
  s->pd = (orc_pdata*)calloc(N, sizeof(orc_pdata));
  if (!s->f_curr || !s->f_next || !s->rho || !s->u || !s->pd) {
    orc_destroy(s);
    return ORC_ERR_NOMEM;
  }
  /* initialise_dynamics(1, 0, 0, 0): rho = 1, u = 0, f = feq everywhere. */
  for (long n = 0; n < N; ++n) {
    s->rho[n] = 1.0;
    s->u[3 * n] = s->u[3 * n + 1] = s->u[3 * n + 2] = 0.0;
    for (int iq = 0; iq < s->q; ++iq) {
      double v = feq_node(s, iq, s->rho[n], &s->u[3 * n]);
      s->f_curr[n * s->q + iq] = v;
      s->f_next[n * s->q + iq] = v;
    }
  }
  s->F_mag2 = s->F_lbm[0] * s->F_lbm[0] + s->F_lbm[1] * s->F_lbm[1] + s->F_lbm[2] * s->F_lbm[2];
  *out = s;
  return ORC_OK;
}

void orc_destroy(orc_sim* s) {
  if (!s) return;
  free(s->f_curr);
  free(s->f_next);
  free(s->rho);
  free(s->u);
  free(s->pd);
  free(s);
}

void orc_set_threads(orc_sim* s, int nthreads) {
  if (s) s->nthreads = nthreads > 0 ? nthreads : 1;
}

int orc_get_info(const orc_sim* s, orc_info* info) {
  if (!s || !info) return ORC_ERR_ARG;
  info->nx = s->nx;
  info->ny = s->ny;
  info->nz = s->nz;
  info->q = s->q;
  info->dx = s->un.dx;
  info->Uc = s->un.Uc;
  info->u_lb = s->un.u_lb;
  info->tc = s->un.tc;
  info->dt_d = s->un.dt_d;
  info->forceFactor = s->un.forceFactor;
  info->torqueFactor = s->un.torqueFactor;
  info->volumeForceFactor = s->un.volumeForceFactor;
  /* update->dt = get_phys_time(1)/nevery (src/fix_LBM_PSM.cpp:120) */
  info->dt_dem = (1.0 * s->un.dt_d * s->un.tc) / ((double)s->nevery);
  info->Ma = s->un.u_lb / (1.0 / sqrt(3.0));
  for (int d = 0; d < 3; ++d) info->F_lbm[d] = s->F_lbm[d];
  return ORC_OK;
}

/* LBMPSMLattice::setParticleOnLattice (src/LBM_PSM_lattice.cpp:257-299). */
static void set_particle(orc_pdata* pd, int pID, const double* uP, double eps) {
  int slot = -1;
  if (pd->id[0] == pID)
    slot = 0;
  else if (pd->id[1] == pID)
    slot = 1;
  else if (pID != pd->id[0] && pID != pd->id[1] && pd->id[0] == 0)
    slot = 0;
  else if (pID != pd->id[0] && pID != pd->id[1] && pd->id[1] == 0)
    slot = 1;
  if (slot < 0) return; /* a third particle on the node is dropped */
  pd->id[slot] = pID;
  pd->eps[slot] = eps;
  pd->us[3 * slot + 0] = uP[0];
  pd->us[3 * slot + 1] = uP[1];
  pd->us[3 * slot + 2] = uP[2];
  pd->F[3 * slot + 0] = 0.0;
  pd->F[3 * slot + 1] = 0.0;
  pd->F[3 * slot + 2] = 0.0;
}

/* LBMPSMLattice::setToZero (src/LBM_PSM_lattice.cpp:302-324). */
static void set_to_zero(orc_pdata* pd, int pID) {
  int slot = -1;
  if (pd->id[0] == pID)
    slot = 0;
  else if (pd->id[1] == pID)
    slot = 1;
  if (slot < 0) return;
  pd->id[slot] = 0;
  pd->eps[slot] = 0.0;
  for (int c = 0; c < 3; ++c) {
    pd->us[3 * slot + c] = 0.0;
    pd->F[3 * slot + c] = 0.0;
  }
}

/* ExchangeParticleData::calcSolidFraction
 * (src/LBM_PSM_exchangeParticleData.cpp:116-169). */
static double calc_solid_fraction(int dim, int i, int j, int k, double xP, double yP, double zP,
                                  double rP_LB) {
  const int slicesPerDim = 10;
  double sliceWidth = 1.0 / ((double)slicesPerDim);
  double fraction = 1.0 / ((double)(slicesPerDim * slicesPerDim));
  double dx_sq[10], dy_sq[10], dz_sq[10];
  if (dim == 3) fraction = 1.0 / ((double)(slicesPerDim * slicesPerDim * slicesPerDim));
  double sqrt2half = sqrt(2.1) / 2.0;
  if (dim == 3) sqrt2half = sqrt(3.1) / 2.0;
  double dx = (double)i - xP;
  double dy = (double)j - yP;
  double dz = (double)k - zP;
  double dist = dx * dx + dy * dy + dz * dz;
  double rP = rP_LB + sqrt2half;
  if (dist > rP * rP) return 0.0;
  double rM = rP_LB - sqrt2half;
  if (dist < rM * rM) return 1.0;
  double rSq = rP_LB * rP_LB;
  for (int m = 0; m < slicesPerDim; ++m) {
    double delta = -0.5 + ((double)m + 0.5) * sliceWidth;
    double dx_i = dx + delta;
    dx_sq[m] = dx_i * dx_i;
    double dy_i = dy + delta;
    dy_sq[m] = dy_i * dy_i;
    double dz_i = dz + delta;
    dz_sq[m] = dz_i * dz_i;
  }
  int n = 0;
  if (dim == 2) {
    for (int a = 0; a < slicesPerDim; ++a)
      for (int b = 0; b < slicesPerDim; ++b)
        if (dx_sq[a] + dy_sq[b] < rSq) ++n;
  } else {
    for (int a = 0; a < slicesPerDim; ++a)
      for (int b = 0; b < slicesPerDim; ++b)
        for (int c = 0; c < slicesPerDim; ++c)
          if (dx_sq[a] + dy_sq[b] + dz_sq[c] < rSq) ++n;
  }
  return fraction * ((double)n);
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Lattice-local particle centre on one rank:
 * x_lb_global - (nxTotal - pc*2*ew - 1) with nxTotal = pc = 0
 * (src/LBM_PSM_exchangeParticleData.cpp:31-37). */
static inline void local_centre(const orc_sim* s, const double* xp, double* xl) {
  for (int d = 0; d < 3; ++d) {
    double g = (xp[d] - s->origin[d]) / s->un.dx;
    xl[d] = g - ((0 - ((double)0 * 2.0 * (double)1)) - 1);
  }
}

/* ExchangeParticleData::setParticlesOnLattice
 * (src/LBM_PSM_exchangeParticleData.cpp:24-112). */
int orc_map(orc_sim* s, int n, const int* tag, const double* x, const double* v,
            const double* omega, const double* radius) {
  if (!s || n < 0) return ORC_ERR_ARG;
  const int ny = s->ny, nz = s->nz;
  for (int ip = 0; ip < n; ++ip) {
    double xl[3];
    local_centre(s, &x[3 * ip], xl);
    double r_lb = radius[ip] / s->un.dx;
    int zone[3][2] = {{(int)(xl[0] - r_lb) - 2, (int)(xl[0] + r_lb) + 2},
                      {(int)(xl[1] - r_lb) - 2, (int)(xl[1] + r_lb) + 2},
                      {(int)(xl[2] - r_lb) - 2, (int)(xl[2] + r_lb) + 2}};
    for (int b = 0; b < 2; ++b) {
      zone[0][b] = clampi(zone[0][b], 0, s->nx);
      zone[1][b] = clampi(zone[1][b], 0, s->ny);
      zone[2][b] = clampi(zone[2][b], 0, s->nz);
      if (zone[2][b] < b) zone[2][b] = b; /* 2-D: keep one z layer */
    }
    const double uTrans[3] = {v[3 * ip + 0] / s->un.Uc * s->un.u_lb,
                              v[3 * ip + 1] / s->un.Uc * s->un.u_lb,
                              v[3 * ip + 2] / s->un.Uc * s->un.u_lb};
    const double omegaLB[3] = {omega[3 * ip + 0] * s->un.tc * s->un.dt_d,
                               omega[3 * ip + 1] * s->un.tc * s->un.dt_d,
                               omega[3 * ip + 2] * s->un.tc * s->un.dt_d};
    const int t = tag[ip];
    for (int i = zone[0][0]; i < zone[0][1]; ++i) {
      for (int j = zone[1][0]; j < zone[1][1]; ++j) {
        for (int k = zone[2][0]; k < zone[2][1]; ++k) {
          long ind = ((long)i * ny + j) * nz + k;
          double sf = calc_solid_fraction(s->dim, i, j, k, xl[0], xl[1], xl[2], r_lb);
          int id_old = 0;
          double sf_old = 0.0;
          orc_pdata* pn = &s->pd[ind];
          if (t == pn->id[0]) {
            id_old = pn->id[0];
            sf_old = pn->eps[0];
          } else if (t == pn->id[1]) {
            id_old = pn->id[1];
            sf_old = pn->eps[1];
          }
          int decFlag = (sf > 0.00001) + 2 * (sf_old > 0.00001);
          double dx = (double)i - xl[0];
          double dy = (double)j - xl[1];
          double dz = (double)k - xl[2];
          double uNode[3];
          uNode[0] = uTrans[0] + omegaLB[1] * dz - omegaLB[2] * dy;
          uNode[1] = uTrans[1] + omegaLB[2] * dx - omegaLB[0] * dz;
          uNode[2] = uTrans[2] + omegaLB[0] * dy - omegaLB[1] * dx;
          switch (decFlag) {
            case 0:
              set_to_zero(pn, t);
              break;
            case 1:
              set_particle(pn, t, uNode, sf);
              break;
            case 2:
              if (id_old == t) set_to_zero(pn, t);
              break;
            case 3:
              if (sf > sf_old || id_old == t) set_particle(pn, t, uNode, sf);
              break;
          }
        }
      }
    }
  }
  return ORC_OK;
}

/* LBMPSMMPI::sendRecvData on one rank (src/LBM_PSM_MPICOMM.h:79-147):
 * for a periodic axis the halo plane 0 receives plane n-2 and plane n-1
 * receives plane 1 (whole planes, all populations); a non-periodic axis is
 * left alone. */
static void halo_exchange(orc_sim* s, int axis) {
  const int q = s->q;
  int n = axis == 0 ? s->nx : (axis == 1 ? s->ny : s->nz);
  int dst[2] = {0, n - 1};
  int src[2] = {n - 2, 1};
  for (int e = 0; e < 2; ++e) {
    for (int a = 0; a < (axis == 0 ? 1 : s->nx); ++a) {
      for (int b = 0; b < (axis == 1 ? 1 : s->ny); ++b) {
        for (int c = 0; c < (axis == 2 ? 1 : s->nz); ++c) {
          int si = axis == 0 ? src[e] : a, sj = axis == 1 ? src[e] : b,
              sk = axis == 2 ? src[e] : c;
          int di = axis == 0 ? dst[e] : a, dj = axis == 1 ? dst[e] : b,
              dk = axis == 2 ? dst[e] : c;
          memcpy(&s->f_curr[nidx(s, di, dj, dk) * q], &s->f_curr[nidx(s, si, sj, sk) * q],
                 sizeof(double) * q);
        }
      }
    }
  }
}

/* LBMPSMBGKDynamics::compute_macro_values (src/LBM_PSM_BGK_dynamics.cpp:48-77). */
static inline void compute_macro(orc_sim* s, long n) {
  double rho_tmp = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
  const double* f = &s->f_curr[n * s->q];
  for (int iq = 0; iq < s->q; ++iq) {
    double fi = f[iq];
    rho_tmp += fi;
    jx += fi * s->ex[iq];
    jy += fi * s->ey[iq];
    jz += fi * s->ez[iq];
  }
  s->rho[n] = rho_tmp;
  jx += s->F_lbm[0] * 0.5;
  jy += s->F_lbm[1] * 0.5;
  jz += s->F_lbm[2] * 0.5;
  s->u[3 * n + 0] = jx / rho_tmp;
  s->u[3 * n + 1] = jy / rho_tmp;
  s->u[3 * n + 2] = jz / rho_tmp;
}

/* LBMPSMBGKDynamics::collisionAndStream (src/LBM_PSM_BGK_dynamics.h:40-114),
 * with add_Fhyd (src/LBM_PSM_lattice.cpp:355-363).  The f0 write of the
 * reference is dead (never read) and omitted. */
static inline void collide_stream_q(orc_sim* s, long n, int iq, long target) {
  const long ind_iq = n * s->q + iq;
  double rho = s->rho[n];
  double fi = s->f_curr[ind_iq];
  double fi_eq = feq_node(s, iq, rho, &s->u[3 * n]);
  orc_pdata* nd = &s->pd[n];
  int pID1 = nd->id[0], pID2 = nd->id[1];
  double F_lbm_iq = 0.0;
  if (s->F_mag2 > 0.0) F_lbm_iq = (1.0 - 0.5 * s->omega) * F_iq(s, iq, &s->u[3 * n], s->F_lbm);
  if (pID1 <= 0 && pID2 <= 0) {
    s->f_next[target * s->q + iq] = fi + (fi_eq - fi) * s->omega + F_lbm_iq;
    return;
  }
  double B1 = 0.0, B2 = 0.0, solid_coll1 = 0.0, solid_coll2 = 0.0;
  double oneMinusOmega = 1.0 - s->omega;
  if (pID1 > 0) {
    B1 = nd->eps[0];
    double uS[3] = {nd->us[0], nd->us[1], nd->us[2]};
    double f0_solid1 = feq_arr(s, iq, rho, uS);
    solid_coll1 = f0_solid1 - fi + oneMinusOmega * (fi - fi_eq);
  }
  if (pID2 > 0) {
    B2 = nd->eps[1];
    double uS[3] = {nd->us[3], nd->us[4], nd->us[5]};
    double f0_solid2 = feq_arr(s, iq, rho, uS);
    solid_coll2 = f0_solid2 - fi + oneMinusOmega * (fi - fi_eq);
  }
  double Btot = B1 + B2;
  if (Btot > 1.0) {
    B1 = B1 / Btot;
    B2 = B2 / Btot;
    Btot = 1.0;
  }
  s->f_next[target * s->q + iq] = fi + (1.0 - Btot) * (fi_eq - fi) * s->omega +
                                  B1 * solid_coll1 + B2 * solid_coll2 + F_lbm_iq;
  const double e[3] = {s->ex[iq], s->ey[iq], s->ez[iq]};
  if (pID1 > 0) {
    int slot = nd->id[0] == pID1 ? 0 : (nd->id[1] == pID1 ? 1 : -1);
    if (slot >= 0)
      for (int d = 0; d < 3; ++d) nd->F[3 * slot + d] += -B1 * solid_coll1 * e[d];
  }
  if (pID2 > 0) {
    int slot = nd->id[0] == pID2 ? 0 : (nd->id[1] == pID2 ? 1 : -1);
    if (slot >= 0)
      for (int d = 0; d < 3; ++d) nd->F[3 * slot + d] += -B2 * solid_coll2 * e[d];
  }
}

/* fix_LBM_PSM::post_force halo exchange (src/fix_LBM_PSM.cpp:206-213) and
 * LBMPSMBGKDynamics::macroCollideStream (src/LBM_PSM_BGK_dynamics.cpp:81-109). */
int orc_collide_stream(orc_sim* s) {
  if (!s) return ORC_ERR_ARG;
  for (int axis = 0; axis < (s->dim == 2 ? 2 : 3); ++axis)
    if (s->periodic[axis]) halo_exchange(s, axis);
  const int nx = s->nx, ny = s->ny, nz = s->nz;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(s->nthreads)
#endif
  for (int i = 0; i < nx; ++i) {
    for (int j = 0; j < ny; ++j) {
      for (int k = 0; k < nz; ++k) {
        long n = nidx(s, i, j, k);
        compute_macro(s, n);
        for (int iq = 0; iq < s->q; ++iq) {
          int is = i + s->ex[iq];
          if (is < 0 || is > nx - 1) continue;
          int js = j + s->ey[iq];
          if (js < 0 || js > ny - 1) continue;
          int ks = k + s->ez[iq];
          if (ks < 0 || ks > nz - 1) continue;
          collide_stream_q(s, n, iq, nidx(s, is, js, ks));
        }
      }
    }
  }
  double* t = s->f_curr;
  s->f_curr = s->f_next;
  s->f_next = t;
  return ORC_OK;
}

/* ExchangeParticleData::calculateHydrodynamicInteractions
 * (src/LBM_PSM_exchangeParticleData.cpp:172-244) for one image. */
static void reduce_one(const orc_sim* s, int t, const double* xp, double rp, double* fH,
                       double* tH, double* S) {
  const int ew = 1;
  double xl[3];
  local_centre(s, xp, xl);
  double r_lb = rp / s->un.dx;
  int zone[3][2] = {{(int)(xl[0] - r_lb) - 2, (int)(xl[0] + r_lb) + 2},
                    {(int)(xl[1] - r_lb) - 2, (int)(xl[1] + r_lb) + 2},
                    {(int)(xl[2] - r_lb) - 2, (int)(xl[2] + r_lb) + 2}};
  for (int b = 0; b < 2; ++b) {
    zone[0][b] = clampi(zone[0][b], ew, s->nx - ew);
    zone[1][b] = clampi(zone[1][b], ew, s->ny - ew);
    /* fmax(fmin(fmax(z, ew), nz-ew), b): in 2-D nz-ew = 0 wins over ew */
    int zz = zone[2][b] < ew ? ew : zone[2][b];
    zz = zz > s->nz - ew ? s->nz - ew : zz;
    zone[2][b] = zz < b ? b : zz;
  }
  const double ff = s->un.forceFactor, tf = s->un.torqueFactor;
  for (int i = zone[0][0]; i < zone[0][1]; ++i) {
    for (int j = zone[1][0]; j < zone[1][1]; ++j) {
      for (int k = zone[2][0]; k < zone[2][1]; ++k) {
        const orc_pdata* pn = &s->pd[nidx(s, i, j, k)];
        double Fh[3];
        if (t == pn->id[0]) {
          Fh[0] = pn->F[0];
          Fh[1] = pn->F[1];
          Fh[2] = pn->F[2];
        } else if (t == pn->id[1]) {
          Fh[0] = pn->F[3];
          Fh[1] = pn->F[4];
          Fh[2] = pn->F[5];
        } else {
          continue;
        }
        fH[0] += Fh[0] * ff;
        fH[1] += Fh[1] * ff;
        fH[2] += Fh[2] * ff;
        double dx = (double)i - xl[0];
        double dy = (double)j - xl[1];
        double dz = (double)k - xl[2];
        tH[0] += (dy * Fh[2] - dz * Fh[1]) * tf;
        tH[1] += (dz * Fh[0] - dx * Fh[2]) * tf;
        tH[2] += (dx * Fh[1] - dy * Fh[0]) * tf;
        S[0] -= 0.5 * (dx * Fh[0] + dx * Fh[0]) * tf;
        S[1] -= 0.5 * (dy * Fh[1] + dy * Fh[1]) * tf;
        S[2] -= 0.5 * (dz * Fh[2] + dz * Fh[2]) * tf;
        S[3] -= 0.5 * (dy * Fh[0] + dx * Fh[1]) * tf;
        S[4] -= 0.5 * (dz * Fh[0] + dx * Fh[2]) * tf;
        S[5] -= 0.5 * (dz * Fh[1] + dy * Fh[2]) * tf;
      }
    }
  }
}

/* The per-image loop of fix_LBM_PSM::post_force (src/fix_LBM_PSM.cpp:223-259):
 * each image's F/T/stresslet starts at zero. */
int orc_reduce(orc_sim* s, int n, const int* tag, const double* x, const double* radius,
               double* fh, double* th, double* stresslet) {
  if (!s || n < 0) return ORC_ERR_ARG;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(s->nthreads)
#endif
  for (int ip = 0; ip < n; ++ip) {
    double F[3] = {0.0, 0.0, 0.0}, T[3] = {0.0, 0.0, 0.0};
    double S[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    reduce_one(s, tag[ip], &x[3 * ip], radius[ip], F, T, S);
    for (int d = 0; d < 3; ++d) {
      fh[3 * ip + d] = F[d];
      th[3 * ip + d] = T[d];
    }
    for (int d = 0; d < 6; ++d) stresslet[6 * ip + d] = S[d];
  }
  return ORC_OK;
}

int orc_step(orc_sim* s, int n, const int* tag, const double* x, const double* v,
             const double* omega, const double* radius, double* fh, double* th,
             double* stresslet) {
  int rc = orc_map(s, n, tag, x, v, omega, radius);
  if (rc) return rc;
  rc = orc_collide_stream(s);
  if (rc) return rc;
  return orc_reduce(s, n, tag, x, radius, fh, th, stresslet);
}

/* ---------------- Zou-He faces (src/LBM_PSM_zou_he_BC.cpp) ---------------- */
#define F_(k) f[k]

/* setZouHeVelBC2D_xn (:25-40) */
static void zh2_vel_xn(double* f, double ux) {
  double rho = 1.0 / (1.0 - ux) * (F_(0) + F_(2) + F_(4) + 2.0 * (F_(3) + F_(6) + F_(7)));
  F_(5) = F_(7) + 0.5 * (F_(4) - F_(2)) + rho * ux * (1.0 / 6.0);
  F_(8) = F_(6) + 0.5 * (F_(2) - F_(4)) + rho * ux * (1.0 / 6.0);
  F_(1) = F_(3) + (2.0 / 3.0) * rho * ux;
}
/* setZouHeVelBC2D_xp (:43-58) */
static void zh2_vel_xp(double* f, double ux) {
  double rho = 1.0 / (1.0 - ux) * (F_(0) + F_(2) + F_(4) + 2.0 * (F_(1) + F_(5) + F_(8)));
  F_(7) = F_(5) + 0.5 * (F_(2) - F_(4)) - rho * ux * (1.0 / 6.0);
  F_(6) = F_(8) + 0.5 * (F_(4) - F_(2)) - rho * ux * (1.0 / 6.0);
  F_(3) = F_(1) - (2.0 / 3.0) * rho * ux;
}
/* setZouHeDensBC2D_xp (:61-76) */
static void zh2_dens_xp(double* f, double rho_bc) {
  double ux = -1.0 + 1.0 / rho_bc * (F_(0) + F_(2) + F_(4) + 2.0 * (F_(1) + F_(5) + F_(8)));
  F_(6) = F_(8) + 0.5 * (F_(4) - F_(2)) - rho_bc * ux * (1.0 / 6.0);
  F_(7) = F_(5) + 0.5 * (F_(2) - F_(4)) - rho_bc * ux * (1.0 / 6.0);
  F_(3) = F_(1) - (2.0 / 3.0) * rho_bc * ux;
}
/* setZouHeVelBC2D_yn (:79-94) */
static void zh2_vel_yn(double* f, double ux) {
  double rho = F_(0) + F_(3) + F_(1) + 2.0 * (F_(8) + F_(4) + F_(7));
  F_(6) = F_(8) + 0.5 * (F_(1) - F_(3)) - rho * ux * 0.5;
  F_(5) = F_(7) + 0.5 * (F_(3) - F_(1)) + rho * ux * 0.5;
  F_(2) = F_(4);
}
/* setZouHeVelBC2D_yp (:97-112) */
static void zh2_vel_yp(double* f, double ux) {
  double rho = F_(0) + F_(3) + F_(1) + 2.0 * (F_(6) + F_(2) + F_(5));
  F_(7) = F_(5) + 0.5 * (F_(1) - F_(3)) - rho * ux * 0.5;
  F_(8) = F_(6) + 0.5 * (F_(3) - F_(1)) + rho * ux * 0.5;
  F_(4) = F_(2);
}

/* setZouHeVelBC3D_xn (:153-185) */
static void zh3_vel_xn(double* f, double ux, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double rho = 1.0 / (1.0 - ux) *
               (F_(0) + F_(3) + F_(4) + F_(5) + F_(6) + F_(11) + F_(17) + F_(18) + F_(12) +
                2.0 * (F_(2) + F_(14) + F_(8) + F_(16) + F_(10)));
  double Nyx = 0.5 * (F_(3) + F_(11) + F_(17) - (F_(4) + F_(18) + F_(12))) - o3 * rho * uy;
  double Nzx = 0.5 * (F_(5) + F_(18) + F_(11) - (F_(6) + F_(17) + F_(12))) - o3 * rho * uz;
  F_(1) = F_(2) + o3 * rho * ux;
  F_(13) = F_(14) + rho * o6 * (ux - uy) + Nyx;
  F_(7) = F_(8) + rho * o6 * (ux + uy) - Nyx;
  F_(9) = F_(10) + rho * o6 * (ux + uz) - Nzx;
  F_(15) = F_(16) + rho * o6 * (ux - uz) + Nzx;
}
/* setZouHeVelBC3D_xp (:189-221) */
static void zh3_vel_xp(double* f, double ux, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double rho = 1.0 / (1.0 + ux) *
               (F_(0) + F_(3) + F_(4) + F_(5) + F_(6) + F_(11) + F_(17) + F_(18) + F_(12) +
                2.0 * (F_(1) + F_(7) + F_(13) + F_(9) + F_(15)));
  double Nyx = 0.5 * (F_(3) + F_(11) + F_(17) - (F_(4) + F_(18) + F_(12))) - o3 * rho * uy;
  double Nzx = 0.5 * (F_(5) + F_(18) + F_(11) - (F_(6) + F_(17) + F_(12))) - o3 * rho * uz;
  F_(2) = F_(1) - o3 * rho * ux;
  F_(14) = F_(13) + rho * o6 * (-ux + uy) - Nyx;
  F_(8) = F_(7) + rho * o6 * (-ux - uy) + Nyx;
  F_(10) = F_(9) + rho * o6 * (-ux - uz) + Nzx;
  F_(16) = F_(15) + rho * o6 * (-ux + uz) - Nzx;
}
/* setZouHeDensBC3D_xp (:225-257) */
static void zh3_dens_xp(double* f, double rho_bc, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double ux = -1.0 + 1.0 / rho_bc *
                         (F_(0) + F_(3) + F_(4) + F_(5) + F_(6) + F_(11) + F_(17) + F_(18) +
                          F_(12) + 2.0 * (F_(1) + F_(7) + F_(13) + F_(9) + F_(15)));
  double Nyx = 0.5 * (F_(3) + F_(11) + F_(17) - (F_(4) + F_(18) + F_(12))) - o3 * rho_bc * uy;
  double Nzx = 0.5 * (F_(5) + F_(18) + F_(11) - (F_(6) + F_(17) + F_(12))) - o3 * rho_bc * uz;
  F_(2) = F_(1) - o3 * rho_bc * ux;
  F_(14) = F_(13) + rho_bc * o6 * (-ux + uy) - Nyx;
  F_(8) = F_(7) + rho_bc * o6 * (-ux - uy) + Nyx;
  F_(10) = F_(9) + rho_bc * o6 * (-ux - uz) + Nzx;
  F_(16) = F_(15) + rho_bc * o6 * (-ux + uz) - Nzx;
}
/* setZouHeVelBC3D_yn (:261-293) */
static void zh3_vel_yn(double* f, double ux, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double rho = 1.0 / (1.0 - uy) *
               (F_(0) + F_(1) + F_(2) + F_(5) + F_(6) + F_(9) + F_(15) + F_(16) + F_(10) +
                2.0 * (F_(4) + F_(13) + F_(8) + F_(18) + F_(12)));
  double Nxy = 0.5 * (F_(1) + F_(9) + F_(15) - (F_(2) + F_(16) + F_(10))) - o3 * rho * ux;
  double Nzy = 0.5 * (F_(5) + F_(9) + F_(16) - (F_(6) + F_(15) + F_(10))) - o3 * rho * uz;
  F_(3) = F_(4) + o3 * rho * uy;
  F_(7) = F_(8) + rho * o6 * (uy + ux) - Nxy;
  F_(14) = F_(13) + rho * o6 * (uy - ux) + Nxy;
  F_(11) = F_(12) + rho * o6 * (uy + uz) - Nzy;
  F_(17) = F_(18) + rho * o6 * (uy - uz) + Nzy;
}
/* setZouHeVelBC3D_yp (:296-328) */
static void zh3_vel_yp(double* f, double ux, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double rho = 1.0 / (1.0 + uy) *
               (F_(0) + F_(1) + F_(2) + F_(5) + F_(6) + F_(9) + F_(15) + F_(16) + F_(10) +
                2.0 * (F_(3) + F_(7) + F_(14) + F_(11) + F_(17)));
  double Nxy = 0.5 * (F_(1) + F_(9) + F_(15) - (F_(2) + F_(16) + F_(10))) - o3 * rho * ux;
  double Nzy = 0.5 * (F_(5) + F_(9) + F_(16) - (F_(6) + F_(15) + F_(10))) - o3 * rho * uz;
  F_(4) = F_(3) - o3 * rho * uy;
  F_(8) = F_(7) + rho * o6 * (-uy - ux) + Nxy;
  F_(13) = F_(14) + rho * o6 * (-uy + ux) - Nxy;
  F_(12) = F_(11) + rho * o6 * (-uy - uz) + Nzy;
  F_(18) = F_(17) + rho * o6 * (-uy + uz) - Nzy;
}
/* setZouHeVelBC3D_zn (:331-363) */
static void zh3_vel_zn(double* f, double ux, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double rho = 1.0 / (1.0 - uz) *
               (F_(0) + F_(1) + F_(2) + F_(3) + F_(4) + F_(7) + F_(13) + F_(14) + F_(8) +
                2.0 * (F_(6) + F_(15) + F_(10) + F_(17) + F_(12)));
  double Nxz = 0.5 * (F_(1) + F_(7) + F_(13) - (F_(2) + F_(14) + F_(8))) - o3 * rho * ux;
  double Nyz = 0.5 * (F_(3) + F_(7) + F_(14) - (F_(4) + F_(13) + F_(8))) - o3 * rho * uy;
  F_(5) = F_(6) + o3 * rho * uz;
  F_(9) = F_(10) + rho * o6 * (uz + ux) - Nxz;
  F_(16) = F_(15) + rho * o6 * (uz - ux) + Nxz;
  F_(11) = F_(12) + rho * o6 * (uz + uy) - Nyz;
  F_(18) = F_(17) + rho * o6 * (uz - uy) + Nyz;
}
/* setZouHeVelBC3D_zp (:366-398) */
static void zh3_vel_zp(double* f, double ux, double uy, double uz) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0;
  double rho = 1.0 / (1.0 + uz) *
               (F_(0) + F_(1) + F_(2) + F_(3) + F_(4) + F_(7) + F_(14) + F_(8) + F_(13) +
                2.0 * (F_(5) + F_(9) + F_(16) + F_(11) + F_(18)));
  double Nxz = 0.5 * (F_(1) + F_(7) + F_(13) - (F_(2) + F_(14) + F_(8))) - o3 * rho * ux;
  double Nyz = 0.5 * (F_(3) + F_(7) + F_(14) - (F_(4) + F_(13) + F_(8))) - o3 * rho * uy;
  F_(6) = F_(5) - o3 * rho * uz;
  F_(15) = F_(16) + rho * o6 * (-uz + ux) - Nxz;
  F_(10) = F_(9) + rho * o6 * (-uz - ux) + Nxz;
  F_(17) = F_(18) + rho * o6 * (-uz + uy) - Nyz;
  F_(12) = F_(11) + rho * o6 * (-uz - uy) + Nyz;
}
#undef F_

enum { FACE_VEL2_XN, FACE_VEL2_XP, FACE_DENS2_XP, FACE_VEL2_YN, FACE_VEL2_YP,
       FACE_VEL3_XN, FACE_VEL3_XP, FACE_DENS3_XP, FACE_VEL3_YN, FACE_VEL3_YP,
       FACE_VEL3_ZN, FACE_VEL3_ZP };

/* One ZouHeBC face call over an inclusive index range of the face plane. */
static void apply_face(orc_sim* s, int kind, int plane, int a0, int a1, int b0, int b1,
                       double p0) {
  const int q = s->q;
  for (int a = a0; a <= a1; ++a) {
    for (int b = b0; b <= b1; ++b) {
      int i, j, k;
      switch (kind) {
        case FACE_VEL2_XN: case FACE_VEL2_XP: case FACE_DENS2_XP:
          i = plane; j = a; k = 0; break;
        case FACE_VEL2_YN: case FACE_VEL2_YP:
          i = a; j = plane; k = 0; break;
        case FACE_VEL3_XN: case FACE_VEL3_XP: case FACE_DENS3_XP:
          i = plane; j = a; k = b; break;
        case FACE_VEL3_YN: case FACE_VEL3_YP:
          i = a; j = plane; k = b; break;
        default:
          i = a; j = b; k = plane; break;
      }
      double* f = &s->f_curr[nidx(s, i, j, k) * q];
      switch (kind) {
        case FACE_VEL2_XN: zh2_vel_xn(f, p0); break;
        case FACE_VEL2_XP: zh2_vel_xp(f, p0); break;
        case FACE_DENS2_XP: zh2_dens_xp(f, p0); break;
        case FACE_VEL2_YN: zh2_vel_yn(f, p0); break;
        case FACE_VEL2_YP: zh2_vel_yp(f, p0); break;
        case FACE_VEL3_XN: zh3_vel_xn(f, p0, 0.0, 0.0); break;
        case FACE_VEL3_XP: zh3_vel_xp(f, p0, 0.0, 0.0); break;
        case FACE_DENS3_XP: zh3_dens_xp(f, p0, 0.0, 0.0); break;
        case FACE_VEL3_YN: zh3_vel_yn(f, p0, 0.0, 0.0); break;
        case FACE_VEL3_YP: zh3_vel_yp(f, p0, 0.0, 0.0); break;
        case FACE_VEL3_ZN: zh3_vel_zn(f, p0, 0.0, 0.0); break;
        case FACE_VEL3_ZP: zh3_vel_zp(f, p0, 0.0, 0.0); break;
      }
    }
  }
}

/* fix_LBM_PSM_BC::post_force on one rank (src/fix_LBM_PSM_BC.cpp:151-402). */
int orc_apply_bc(orc_sim* s) {
  if (!s) return ORC_ERR_ARG;
  const int ew = 1;
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double u = s->un.u_lb, rho_out = 1.0;
  if (s->dim == 2) {
    switch (s->bc_type) {
      case 1:
        apply_face(s, FACE_VEL2_YN, ew, ew, nx - 1 - ew, 0, 0, -u);
        apply_face(s, FACE_VEL2_YP, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, u);
        break;
      case 2:
        apply_face(s, FACE_VEL2_XN, ew, ew, ny - 1 - ew, 0, 0, u);
        apply_face(s, FACE_DENS2_XP, nx - 1 - ew, ew, ny - 1 - ew, 0, 0, rho_out);
        apply_face(s, FACE_VEL2_YN, ew, 1 + ew, nx - 2 - ew, 0, 0, u);
        apply_face(s, FACE_VEL2_YP, ny - 1 - ew, 1 + ew, nx - 2 - ew, 0, 0, u);
        break;
      case 3:
        apply_face(s, FACE_VEL2_YN, ew, ew, nx - 1 - ew, 0, 0, 0.0);
        apply_face(s, FACE_VEL2_YP, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, 0.0);
        break;
      case 4:
        apply_face(s, FACE_VEL2_XN, ew, ew, ny - 1 - ew, 0, 0, u);
        apply_face(s, FACE_DENS2_XP, nx - 1 - ew, ew, ny - 1 - ew, 0, 0, rho_out);
        apply_face(s, FACE_VEL2_YN, ew, ew, nx - 1 - ew, 0, 0, 0.0);
        apply_face(s, FACE_VEL2_YP, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, 0.0);
        break;
      case 5:
        apply_face(s, FACE_VEL2_XN, ew, ew, ny - 1 - ew, 0, 0, 0.0);
        apply_face(s, FACE_VEL2_XP, nx - 1 - ew, ew, ny - 1 - ew, 0, 0, 0.0);
        apply_face(s, FACE_VEL2_YN, ew, ew, nx - 1 - ew, 0, 0, 0.0);
        apply_face(s, FACE_VEL2_YP, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, 0.0);
        break;
      default:
        break;
    }
  } else {
    switch (s->bc_type) {
      case 1:
        apply_face(s, FACE_VEL3_YN, ew, ew, nx - 1 - ew, ew, nz - 1 - ew, -u);
        apply_face(s, FACE_VEL3_YP, ny - 1 - ew, ew, nx - 1 - ew, ew, nz - 1 - ew, u);
        break;
      case 2:
        apply_face(s, FACE_VEL3_XN, ew, ew, ny - 1 - ew, ew, nz - 1 - ew, u);
        apply_face(s, FACE_DENS3_XP, nx - 1 - ew, ew, ny - 1 - ew, ew, nz - 1 - ew, rho_out);
        apply_face(s, FACE_VEL3_YN, ew, ew, nx - 1 - ew, ew, nz - 1 - ew, u);
        apply_face(s, FACE_VEL3_YP, ny - 1 - ew, ew, nx - 1 - ew, ew, nz - 1 - ew, u);
        apply_face(s, FACE_VEL3_ZN, ew, ew, nx - 1 - ew, ew, ny - 1 - ew, u);
        apply_face(s, FACE_VEL3_ZP, nz - 1 - ew, ew, nx - 1 - ew, ew, ny - 1 - ew, u);
        break;
      case 3:
        apply_face(s, FACE_VEL3_YN, ew, ew, nx - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_YP, ny - 1 - ew, ew, nx - 1 - ew, ew, nz - 1 - ew, 0.0);
        break;
      case 4:
        apply_face(s, FACE_VEL3_XN, ew, ew, ny - 1 - ew, ew, nz - 1 - ew, u);
        apply_face(s, FACE_DENS3_XP, nx - 1 - ew, ew, ny - 1 - ew, ew, nz - 1 - ew, rho_out);
        apply_face(s, FACE_VEL3_YN, ew, ew, nx - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_YP, ny - 1 - ew, ew, nx - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_ZN, ew, ew, nx - 1 - ew, ew, ny - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_ZP, nz - 1 - ew, ew, nx - 1 - ew, ew, ny - 1 - ew, 0.0);
        break;
      case 5:
        apply_face(s, FACE_VEL3_XN, ew, ew, ny - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_XP, nx - 1 - ew, ew, ny - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_YN, ew, ew, nx - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_YP, ny - 1 - ew, ew, nx - 1 - ew, ew, nz - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_ZN, ew, ew, nx - 1 - ew, ew, ny - 1 - ew, 0.0);
        apply_face(s, FACE_VEL3_ZP, nz - 1 - ew, ew, nx - 1 - ew, ew, ny - 1 - ew, 0.0);
        break;
      default:
        break;
    }
  }
  return ORC_OK;
}

/* ---------------- read-back ---------------- */
int orc_get_f(const orc_sim* s, double* f) {
  if (!s || !f) return ORC_ERR_ARG;
  memcpy(f, s->f_curr, sizeof(double) * (size_t)s->nx * s->ny * s->nz * s->q);
  return ORC_OK;
}

int orc_set_f(orc_sim* s, const double* f) {
  if (!s || !f) return ORC_ERR_ARG;
  memcpy(s->f_curr, f, sizeof(double) * (size_t)s->nx * s->ny * s->nz * s->q);
  return ORC_OK;
}

int orc_get_macro(const orc_sim* s, double* rho, double* u) {
  if (!s) return ORC_ERR_ARG;
  long N = (long)s->nx * s->ny * s->nz;
  if (rho) memcpy(rho, s->rho, sizeof(double) * N);
  if (u) memcpy(u, s->u, sizeof(double) * 3 * N);
  return ORC_OK;
}

int orc_get_pdata(const orc_sim* s, int* ids, double* eps, double* us, double* F) {
  if (!s) return ORC_ERR_ARG;
  long N = (long)s->nx * s->ny * s->nz;
  for (long n = 0; n < N; ++n) {
    const orc_pdata* p = &s->pd[n];
    for (int b = 0; b < 2; ++b) {
      if (ids) ids[2 * n + b] = p->id[b];
      if (eps) eps[2 * n + b] = p->eps[b];
    }
    for (int c = 0; c < 6; ++c) {
      if (us) us[6 * n + c] = p->us[c];
      if (F) F[6 * n + c] = p->F[c];
    }
  }
  return ORC_OK;
}

/* execute_write_vti field read on one rank (src/fix_LBM_PSM_writeVTI.h:146-169). */
int orc_export_fields(const orc_sim* s, double B0, double rho0, double u0, double* solid,
                      double* rho, double* u) {
  if (!s) return ORC_ERR_ARG;
  const int env = 1;
  int kStart = s->dim == 3 ? env : 0;
  int zEnd = s->dim == 3 ? s->nz - env : 1;
  int id = 0;
  for (int k = kStart; k < zEnd; k++)
    for (int j = env; j < s->ny - env; j++)
      for (int i = env; i < s->nx - env; i++) {
        long idx = nidx(s, i, j, k);
        double Bv = s->pd[idx].eps[0] + s->pd[idx].eps[1];
        if (solid) solid[id] = (Bv > 1.0 ? 1.0 : Bv) * B0;
        if (rho) rho[id] = s->rho[idx] * rho0;
        if (u) {
          u[3 * id + 0] = s->u[3 * idx + 0] * u0;
          u[3 * id + 1] = s->u[3 * idx + 1] * u0;
          u[3 * id + 2] = s->dim == 3 ? s->u[3 * idx + 2] * u0 : 0.0;
        }
        id++;
      }
  return id;
}
