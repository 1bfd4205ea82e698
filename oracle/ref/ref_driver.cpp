/*
 * ref_driver.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * Drives the reference's own, unmodified LBM library classes
 * (src/LBM_PSM_*.cpp of timnajuch/LAMMPS-LBM-PSM, compiled in place by
 * oracle/Makefile against the stub headers in oracle/ref/stubs) through the
 * orc_* interface of oracle/lbmpsm_oracle.h.  The fix classes of the
 * reference need LAMMPS, which is not available, so the few lines of
 * fix_LBM_PSM::init/post_force and fix_LBM_PSM_BC::post_force that call the
 * library are restated here for one rank.
 */
#include <cmath>
#include <cstring>
#include <vector>

#include "LBM_PSM_BGK_dynamics.h"
#include "LBM_PSM_MPICOMM.h"
#include "LBM_PSM_exchangeParticleData.h"
#include "LBM_PSM_unitConversion.h"
#include "LBM_PSM_zou_he_BC.h"
#include "lbmpsm_oracle.h"

struct orc_sim {
  orc_params p;
  UnitConversion* uc = nullptr;
  LBMPSMBGKDynamics* dyn = nullptr;
  ExchangeParticleData* exch = nullptr;
  LBMPSMMPI* comm = nullptr;
  ZouHeBC* zh = nullptr;
  std::vector<double> F_lbm;
  double tc = 0.0;
};

namespace {
std::vector<double*> rows(const double* a, int n) {
  std::vector<double*> r((size_t)n + 1);
  for (int i = 0; i < n; ++i) r[i] = const_cast<double*>(a + 3 * (size_t)i);
  return r;
}
}  // namespace

extern "C" {

/* fix_LBM_PSM ctor argument checks (src/fix_LBM_PSM.cpp:15-83) and init()
 * (src/fix_LBM_PSM.cpp:104-177) on one rank. */
int orc_create(const orc_params* p, orc_sim** out) {
  *out = nullptr;
  if (!p || (p->dimension != 2 && p->dimension != 3)) return ORC_ERR_ARG;
  if (p->nevery <= 0 || p->Nlc <= 0 || p->lc <= 0.0 || p->rho <= 0.0 || p->nu <= 0.0 ||
      p->Re <= 0.0 || p->tau <= 0.5)
    return ORC_ERR_ARG;
  if (p->bc_type < 0 || p->bc_type > 5) return ORC_ERR_ARG;
  orc_sim* s = new orc_sim();
  s->p = *p;
  int decomposition[3] = {1, 1, 1};
  int procCoordinates[3] = {0, 0, 0};
  int procNeigh[6] = {0, 0, 0, 0, 0, 0};
  s->comm = new LBMPSMMPI(MPI_COMM_WORLD, decomposition, procNeigh, procCoordinates, p->dimension);
  s->uc = new UnitConversion(p->rho, p->nu, p->lc, p->Re, p->Nlc, p->tau, p->dimension);
  double Ma = s->uc->get_u_lb() / (1.0 / sqrt(3.0));
  if (Ma > 0.3) {
    orc_destroy(s);
    return ORC_ERR_MACH;
  }
  double SMALL = 1e-15;
  double dx = s->uc->get_dx();
  if (pow(((double)((int)(p->prd[0] / dx + 0.5)) - p->prd[0] / dx), 2.0) > SMALL ||
      pow(((double)((int)(p->prd[1] / dx + 0.5)) - p->prd[1] / dx), 2.0) > SMALL ||
      pow(((double)((int)(p->prd[2] / dx + 0.5)) - p->prd[2] / dx), 2.0) > SMALL) {
    orc_destroy(s);
    return ORC_ERR_GRID;
  }
  int nx = p->prd[0] / dx + 1.5;
  if (p->periodic[0]) nx -= 1;
  int ny = p->prd[1] / dx + 1.5;
  if (p->periodic[1]) ny -= 1;
  int nz = 0;
  if (p->dimension == 3) {
    nz = p->prd[2] / dx + 1.5;
    if (p->periodic[2]) nz -= 1;
  }
  vector<double> boxLength{p->prd[0], p->prd[1], p->prd[2]};
  vector<double> origin{p->boxlo[0], p->boxlo[1], p->boxlo[2]};
  if (p->dimension == 2) origin[2] = 0.0;
  s->F_lbm = s->uc->get_volume_force_lb(vector<double>{p->Fext[0], p->Fext[1], p->Fext[2]});
  s->dyn = new LBMPSMBGKDynamics(p->tau, nx, ny, nz, s->F_lbm, decomposition, procCoordinates,
                                 origin, boxLength, p->dimension);
  s->dyn->initialise_domain(dx, dx, dx);
  s->dyn->initialise_dynamics(1.0, 0.0, 0.0, 0.0);
  s->exch = new ExchangeParticleData(p->dimension, origin);
  s->zh = new ZouHeBC(s->dyn);
  s->tc = p->lc / (p->Re * p->nu / p->lc);
  *out = s;
  return ORC_OK;
}

void orc_destroy(orc_sim* s) {
  if (!s) return;
  delete s->zh;
  delete s->exch;
  delete s->dyn;
  delete s->uc;
  delete s->comm;
  delete s;
}

void orc_set_threads(orc_sim*, int) {}

int orc_get_info(const orc_sim* s, orc_info* info) {
  if (!s || !info) return ORC_ERR_ARG;
  info->nx = s->dyn->get_nx();
  info->ny = s->dyn->get_ny();
  info->nz = s->dyn->get_nz();
  info->q = s->dyn->get_q();
  info->dx = s->uc->get_dx();
  info->Uc = s->uc->get_Uc();
  info->u_lb = s->uc->get_u_lb();
  info->tc = s->tc;
  info->dt_d = s->uc->get_dt_d();
  info->forceFactor = s->uc->get_forceFactor();
  info->torqueFactor = s->uc->get_torqueFactor();
  info->volumeForceFactor = 0.0;
  info->dt_dem = s->uc->get_phys_time(1.0) / ((double)s->p.nevery);
  info->Ma = s->uc->get_u_lb() / (1.0 / sqrt(3.0));
  for (int d = 0; d < 3; ++d) info->F_lbm[d] = s->F_lbm[d];
  return ORC_OK;
}

int orc_map(orc_sim* s, int n, const int* tag, const double* x, const double* v,
            const double* omega, const double* radius) {
  if (!s || n < 0) return ORC_ERR_ARG;
  auto xr = rows(x, n), vr = rows(v, n), wr = rows(omega, n);
  s->exch->setParticlesOnLattice(s->dyn, s->uc, n, const_cast<int*>(tag), xr.data(), vr.data(),
                                 wr.data(), const_cast<double*>(radius));
  return ORC_OK;
}

/* Halo exchange and collide-stream as fix_LBM_PSM::post_force calls them
 * (src/fix_LBM_PSM.cpp:206-215). */
int orc_collide_stream(orc_sim* s) {
  if (!s) return ORC_ERR_ARG;
  LBMPSMBGKDynamics* d = s->dyn;
  if (s->p.dimension == 2) {
    s->comm->sendRecvData<double>(d->getVector_f_curr(), 0, d->get_nx(), d->get_ny(), 1,
                                  d->get_envelopeWidth(), s->p.periodic[0]);
    s->comm->sendRecvData<double>(d->getVector_f_curr(), 1, d->get_nx(), d->get_ny(), 1,
                                  d->get_envelopeWidth(), s->p.periodic[1]);
  } else {
    for (int axis = 0; axis < 3; ++axis)
      s->comm->sendRecvData<double>(d->getVector_f_curr(), axis, d->get_nx(), d->get_ny(),
                                    d->get_nz(), d->get_envelopeWidth(), s->p.periodic[axis]);
  }
  d->macroCollideStream();
  return ORC_OK;
}

int orc_reduce(orc_sim* s, int n, const int* tag, const double* x, const double* radius,
               double* fh, double* th, double* stresslet) {
  if (!s || n < 0) return ORC_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    double F[3] = {0.0, 0.0, 0.0}, T[3] = {0.0, 0.0, 0.0}, S[6] = {0, 0, 0, 0, 0, 0};
    s->exch->calculateHydrodynamicInteractions(s->dyn, s->uc, tag[i], const_cast<double*>(x + 3 * (size_t)i),
                                               radius[i], F, T, S);
    for (int c = 0; c < 3; ++c) {
      fh[3 * i + c] = F[c];
      th[3 * i + c] = T[c];
    }
    for (int c = 0; c < 6; ++c) stresslet[6 * i + c] = S[c];
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

/* fix_LBM_PSM_BC::post_force on one rank (src/fix_LBM_PSM_BC.cpp:151-402). */
int orc_apply_bc(orc_sim* s) {
  if (!s) return ORC_ERR_ARG;
  const int ew = s->dyn->get_envelopeWidth();
  const int nx = s->dyn->get_nx(), ny = s->dyn->get_ny(), nz = s->dyn->get_nz();
  const double u = s->uc->get_u_lb(), rho_out = 1.0;
  ZouHeBC* z = s->zh;
  if (s->p.dimension == 2) {
    switch (s->p.bc_type) {
      case 1:
        z->setZouHeVelBC2D_yn(0 + ew, ew, nx - 1 - ew, -u);
        z->setZouHeVelBC2D_yp(ny - 1 - ew, ew, nx - 1 - ew, u);
        break;
      case 2:
        z->setZouHeVelBC2D_xn(ew, ew, ny - 1 - ew, u);
        z->setZouHeDensBC2D_xp(nx - 1 - ew, ew, ny - 1 - ew, rho_out);
        z->setZouHeVelBC2D_yn(0 + ew, 1 + ew, nx - 2 - ew, u);
        z->setZouHeVelBC2D_yp(ny - 1 - ew, 1 + ew, nx - 2 - ew, u);
        break;
      case 3:
        z->setZouHeVelBC2D_yn(0 + ew, ew, nx - 1 - ew, 0.0);
        z->setZouHeVelBC2D_yp(ny - 1 - ew, ew, nx - 1 - ew, 0.0);
        break;
      case 4:
        z->setZouHeVelBC2D_xn(ew, ew, ny - 1 - ew, u);
        z->setZouHeDensBC2D_xp(nx - 1 - ew, ew, ny - 1 - ew, rho_out);
        z->setZouHeVelBC2D_yn(0 + ew, ew, nx - 1 - ew, 0.0);
        z->setZouHeVelBC2D_yp(ny - 1 - ew, ew, nx - 1 - ew, 0.0);
        break;
      case 5:
        z->setZouHeVelBC2D_xn(ew, ew, ny - 1 - ew, 0.0);
        z->setZouHeVelBC2D_xp(nx - 1 - ew, ew, ny - 1 - ew, 0.0);
        z->setZouHeVelBC2D_yn(0 + ew, ew, nx - 1 - ew, 0.0);
        z->setZouHeVelBC2D_yp(ny - 1 - ew, ew, nx - 1 - ew, 0.0);
        break;
      default:
        break;
    }
  } else {
    const int X0 = ew, X1 = nx - 1 - ew, Y0 = ew, Y1 = ny - 1 - ew, Z0 = ew, Z1 = nz - 1 - ew;
    switch (s->p.bc_type) {
      case 1:
        z->setZouHeVelBC3D_yn(0 + ew, X0, X1, Z0, Z1, -u, 0.0, 0.0);
        z->setZouHeVelBC3D_yp(ny - 1 - ew, X0, X1, Z0, Z1, u, 0.0, 0.0);
        break;
      case 2:
        z->setZouHeVelBC3D_xn(0 + ew, Y0, Y1, Z0, Z1, u, 0.0, 0.0);
        z->setZouHeDensBC3D_xp(nx - 1 - ew, Y0, Y1, Z0, Z1, rho_out, 0.0, 0.0);
        z->setZouHeVelBC3D_yn(0 + ew, X0, X1, Z0, Z1, u, 0.0, 0.0);
        z->setZouHeVelBC3D_yp(ny - 1 - ew, X0, X1, Z0, Z1, u, 0.0, 0.0);
        z->setZouHeVelBC3D_zn(0 + ew, X0, X1, Y0, Y1, u, 0.0, 0.0);
        z->setZouHeVelBC3D_zp(nz - 1 - ew, X0, X1, Y0, Y1, u, 0.0, 0.0);
        break;
      case 3:
        z->setZouHeVelBC3D_yn(0 + ew, X0, X1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_yp(ny - 1 - ew, X0, X1, Z0, Z1, 0.0, 0.0, 0.0);
        break;
      case 4:
        z->setZouHeVelBC3D_xn(0 + ew, Y0, Y1, Z0, Z1, u, 0.0, 0.0);
        z->setZouHeDensBC3D_xp(nx - 1 - ew, Y0, Y1, Z0, Z1, rho_out, 0.0, 0.0);
        z->setZouHeVelBC3D_yn(0 + ew, X0, X1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_yp(ny - 1 - ew, X0, X1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_zn(0 + ew, X0, X1, Y0, Y1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_zp(nz - 1 - ew, X0, X1, Y0, Y1, 0.0, 0.0, 0.0);
        break;
      case 5:
        z->setZouHeVelBC3D_xn(0 + ew, Y0, Y1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_xp(nx - 1 - ew, Y0, Y1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_yn(0 + ew, X0, X1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_yp(ny - 1 - ew, X0, X1, Z0, Z1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_zn(0 + ew, X0, X1, Y0, Y1, 0.0, 0.0, 0.0);
        z->setZouHeVelBC3D_zp(nz - 1 - ew, X0, X1, Y0, Y1, 0.0, 0.0, 0.0);
        break;
      default:
        break;
    }
  }
  return ORC_OK;
}

int orc_get_f(const orc_sim* s, double* f) {
  if (!s || !f) return ORC_ERR_ARG;
  const vector<double>& fc = s->dyn->getVector_f_curr();
  std::memcpy(f, fc.data(), sizeof(double) * fc.size());
  return ORC_OK;
}

int orc_set_f(orc_sim* s, const double* f) {
  if (!s || !f) return ORC_ERR_ARG;
  vector<double> copy(f, f + s->dyn->getVector_f_curr().size());
  s->dyn->setVector_f_curr(copy);
  return ORC_OK;
}

int orc_get_macro(const orc_sim* s, double* rho, double* u) {
  if (!s) return ORC_ERR_ARG;
  const vector<double>& r = s->dyn->get_rho_reference();
  const vector<double>& uu = s->dyn->get_u_reference();
  if (rho) std::memcpy(rho, r.data(), sizeof(double) * r.size());
  if (u) std::memcpy(u, uu.data(), sizeof(double) * uu.size());
  return ORC_OK;
}

int orc_get_pdata(const orc_sim* s, int* ids, double* eps, double* us, double* F) {
  if (!s) return ORC_ERR_ARG;
  long N = (long)s->dyn->get_nx() * s->dyn->get_ny() * s->dyn->get_nz();
  for (long n = 0; n < N; ++n) {
    ParticleDataOnLattice pd = s->dyn->getParticleDataOnLatticeNode((int)n);
    for (int b = 0; b < 2; ++b) {
      if (ids) ids[2 * n + b] = pd.particleID[b];
      if (eps) eps[2 * n + b] = pd.solidFraction[b];
    }
    for (int c = 0; c < 6; ++c) {
      if (us) us[6 * n + c] = pd.particleVelocity[c];
      if (F) F[6 * n + c] = pd.hydrodynamicForce[c];
    }
  }
  return ORC_OK;
}

/* The field read of WriteVTI::execute_write_vti on one rank
 * (src/fix_LBM_PSM_writeVTI.h:146-169). */
int orc_export_fields(const orc_sim* s, double B0, double rho0, double u0, double* solid,
                      double* rho, double* u) {
  if (!s) return ORC_ERR_ARG;
  const int env = 1;
  const int dim = s->p.dimension;
  const int nxL = s->dyn->get_nx(), nyL = s->dyn->get_ny(), nzL = dim == 3 ? s->dyn->get_nz() : 1;
  const vector<double>& r = s->dyn->get_rho_reference();
  const vector<double>& uu = s->dyn->get_u_reference();
  int kStart = dim == 3 ? env : 0;
  int zEnd = dim == 3 ? nzL - env : 1;
  int id = 0;
  for (int k = kStart; k < zEnd; k++)
    for (int j = env; j < nyL - env; j++)
      for (int i = env; i < nxL - env; i++) {
        int idx = i * nyL * nzL + j * nzL + k;
        ParticleDataOnLattice pD = s->dyn->getParticleDataOnLatticeNode(idx);
        double Bv = (pD.solidFraction[0] + pD.solidFraction[1]);
        if (solid) solid[id] = (Bv > 1.0 ? 1.0 : Bv) * B0;
        if (rho) rho[id] = r[idx] * rho0;
        if (u) {
          u[3 * id + 0] = uu[3 * idx + 0] * u0;
          u[3 * id + 1] = uu[3 * idx + 1] * u0;
          u[3 * id + 2] = dim == 3 ? uu[3 * idx + 2] * u0 : 0.0;
        }
        id++;
      }
  return id;
}

}  // extern "C"
