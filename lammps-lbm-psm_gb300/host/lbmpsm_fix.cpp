// lbmpsm_fix.cpp -- the fix classes of lbmpsm_fix.h.
#include "lbmpsm_fix.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>

namespace lbmpsm_host {

namespace {

// utils::numeric / utils::inumeric of LAMMPS: the whole word must parse
double numeric(const std::string& s) {
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(s.c_str(), &end);
  if (s.empty() || end != s.c_str() + s.size() || errno == ERANGE)
    throw LammpsError("Expected floating point parameter instead of '" + s + "' in input script");
  return v;
}

long inumeric(const std::string& s) {
  char* end = nullptr;
  errno = 0;
  const long v = std::strtol(s.c_str(), &end, 10);
  if (s.empty() || end != s.c_str() + s.size() || errno == ERANGE)
    throw LammpsError("Expected integer parameter instead of '" + s + "' in input script");
  return v;
}

// std::ostream's default formatting of a double (6 significant digits)
std::string fmt(double v) {
  char b[64];
  std::snprintf(b, sizeof b, "%g", v);
  return b;
}

[[noreturn]] void lib_error(lbmpsm_handle* h) {
  const char* m = lbmpsm_last_error(h);
  throw LammpsError(m && *m ? m : "lbm-psm: device call failed");
}

}  // namespace

// ------------------------------------------------------------------ atoms
Atoms ghost_images(const Domain& d, double cutghost, const Atoms& owned) {
  Atoms a;
  const int nloc = owned.nlocal;
  a.nlocal = nloc;
  a.tag.assign(owned.tag.begin(), owned.tag.begin() + nloc);
  a.x.assign(owned.x.begin(), owned.x.begin() + 3 * nloc);
  a.v.assign(owned.v.begin(), owned.v.begin() + 3 * nloc);
  a.omega.assign(owned.omega.begin(), owned.omega.begin() + 3 * nloc);
  a.radius.assign(owned.radius.begin(), owned.radius.begin() + nloc);
  a.owner.resize(nloc);
  a.swap.assign(nloc, -1);
  for (int i = 0; i < nloc; ++i) a.owner[i] = i;
  int iswap = 0;
  for (int dim = 0; dim < d.dimension; ++dim) {
    if (!d.periodic[dim]) continue;
    const int present = a.size();  // both swaps of this dimension scan these
    const double lo = d.boxlo[dim], hi = d.boxhi[dim], prd = d.prd(dim);
    for (int ineed = 0; ineed < 2; ++ineed) {
      std::vector<int> sel;
      for (int i = 0; i < present; ++i) {
        const double c = a.x[3 * i + dim];
        if (ineed == 0 ? c <= lo + cutghost : c >= hi - cutghost) sel.push_back(i);
      }
      const double shift = ineed == 0 ? prd : -prd;
      for (int i : sel) {
        a.tag.push_back(a.tag[i]);
        for (int c = 0; c < 3; ++c) {
          a.x.push_back(c == dim ? a.x[3 * i + c] + shift : a.x[3 * i + c]);
          a.v.push_back(a.v[3 * i + c]);
          a.omega.push_back(a.omega[3 * i + c]);
        }
        a.radius.push_back(a.radius[i]);
        a.owner.push_back(i);
        a.swap.push_back(iswap);
      }
      ++iswap;
    }
  }
  a.f.assign(3 * (size_t)a.size(), 0.0);
  a.torque.assign(3 * (size_t)a.size(), 0.0);
  return a;
}

void reverse_comm(std::vector<double>& rows3, const Atoms& a) {
  const int n = a.size();
  if (n == a.nlocal) return;
  int maxswap = -1;
  for (int g = a.nlocal; g < n; ++g) maxswap = std::max(maxswap, a.swap[g]);
  for (int sw = maxswap; sw >= 0; --sw)
    for (int g = 0; g < n; ++g)
      if (a.swap[g] == sw)
        for (int c = 0; c < 3; ++c) rows3[3 * (size_t)a.owner[g] + c] += rows3[3 * (size_t)g + c];
}

// ------------------------------------------------------------------ lbm-psm
FixLbmPsm::FixLbmPsm(const std::vector<std::string>& args, int storage, int device,
                     double max_radius)
    : storage_(storage), device_(device), max_radius_(max_radius) {
  const int narg = (int)args.size();
  if (narg < 15) throw LammpsError("Illegal fix lbm-psm command");
  prm_.tau = 0.7;
  prm_.nevery = 1;
  int iarg = 3;
  auto need = [&](int k) {
    if (iarg + k > narg) throw LammpsError("Illegal fix lbm-psm command");
  };
  while (iarg < narg) {
    const std::string& kw = args[iarg];
    if (kw == "every") {
      need(2);
      nevery = (int)inumeric(args[iarg + 1]);
      if (nevery <= 0) throw LammpsError("Illegal fix lbm-psm command");
      prm_.nevery = nevery;
      iarg += 2;
    } else if (kw == "Nlc") {
      need(2);
      prm_.Nlc = (int)inumeric(args[iarg + 1]);
      if (prm_.Nlc <= 0) throw LammpsError("Illegal fix lbm-psm command");
      have_[0] = true;
      iarg += 2;
    } else if (kw == "lc" || kw == "rho" || kw == "nu" || kw == "Re") {
      need(2);
      const double v = numeric(args[iarg + 1]);
      if (v <= 0.0) throw LammpsError("Illegal fix lbm-psm command");
      if (kw == "lc") prm_.lc = v, have_[1] = true;
      if (kw == "rho") prm_.rho = v, have_[2] = true;
      if (kw == "nu") prm_.nu = v, have_[3] = true;
      if (kw == "Re") prm_.Re = v, have_[4] = true;
      iarg += 2;
    } else if (kw == "tau") {
      need(2);
      prm_.tau = numeric(args[iarg + 1]);
      if (prm_.tau <= 0.5) throw LammpsError("Illegal fix lbm-psm command");
      iarg += 2;
    } else if (kw == "Fext") {
      need(4);
      for (int c = 0; c < 3; ++c) prm_.Fext[c] = numeric(args[iarg + 1 + c]);
      iarg += 4;
    } else {
      throw LammpsError("Illegal fix lbm-psm command");
    }
  }
  rho_ = prm_.rho;
}

FixLbmPsm::~FixLbmPsm() { lbmpsm_destroy(h_); }

double FixLbmPsm::init(const Domain& d) {
  for (bool k : have_)
    if (!k) throw LammpsError("Illegal fix lbm-psm command");
  if (h_) {  // init() runs again on every run: no leak
    lbmpsm_destroy(h_);
    h_ = nullptr;
  }
  prm_.dimension = d.dimension;
  for (int c = 0; c < 3; ++c) {
    prm_.boxlo[c] = d.boxlo[c];
    prm_.prd[c] = d.prd(c);
    prm_.periodic[c] = d.periodic[c];
    origin[c] = (c < 2 || d.dimension == 3) ? d.boxlo[c] : 0.0;
  }
  lbmpsm_options o{};
  o.storage = storage_;
  o.device = device_;
  o.max_radius = max_radius_;
  if (lbmpsm_create(&prm_, &o, &h_) != LBMPSM_OK) lib_error(nullptr);
  lbmpsm_get_info(h_, &info_);
  hydro.clear();
  return info_.dt_dem;
}

void FixLbmPsm::post_force(long ntimestep, Atoms& a) {
  const int n = a.size(), nl = a.nlocal;
  if (ntimestep % nevery) {
    // re-apply the stored force and torque of the owned atoms
    const int rows = std::min(nl, (int)(hydro.size() / 6));
    for (int i = 0; i < rows; ++i)
      for (int c = 0; c < 3; ++c) {
        a.f[3 * i + c] += hydro[6 * i + c];
        a.torque[3 * i + c] += hydro[6 * i + 3 + c];
      }
    return;
  }
  std::vector<double> fh(3 * (size_t)n), th(3 * (size_t)n), S(6 * (size_t)n);
  if (lbmpsm_step(h_, n, a.tag.data(), a.x.data(), a.v.data(), a.omega.data(), a.radius.data(),
                  fh.data(), th.data(), S.data()) != LBMPSM_OK)
    lib_error(h_);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      const size_t k = 3 * (size_t)i + c;
      if (i < nl) {
        a.f[k] += fh[k];
        a.torque[k] += th[k];
      } else {
        a.f[k] = fh[k];
        a.torque[k] = th[k];
      }
    }
  hydro.resize(6 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      hydro[6 * (size_t)i + c] = fh[3 * (size_t)i + c];
      hydro[6 * (size_t)i + 3 + c] = th[3 * (size_t)i + c];
    }
  for (int k = 0; k < 6; ++k) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += S[6 * (size_t)i + k];
    virial[k] = s;  // v_tally(i, stresslet) summed over the images
  }
  reverse_comm(a.f, a);
  reverse_comm(a.torque, a);
}

// ------------------------------------------------------------------ lbm-psm-bc
FixLbmPsmBC::FixLbmPsmBC(const std::vector<std::string>& args, FixLbmPsm& fix) : fix_(fix) {
  if (args.size() < 4) throw LammpsError("Illegal fix lbm-psm-bc command");
  const std::string& k = args[3];
  if (k == "shear")
    type_ = LBMPSM_BC_SHEAR;
  else if (k == "xFlow")
    type_ = LBMPSM_BC_XFLOW;
  else if (k == "channel")
    type_ = LBMPSM_BC_CHANNEL;
  else if (k == "channel-velIn-pressOut")
    type_ = LBMPSM_BC_CHANNEL_VELIN_PRESSOUT;
  else if (k == "closedBox")
    type_ = LBMPSM_BC_CLOSEDBOX;
  else
    throw LammpsError("Illegal fix lbm-psm-bc command");
}

void FixLbmPsmBC::init() {
  if (lbmpsm_set_bc(fix_.lattice(), type_) != LBMPSM_OK) lib_error(fix_.lattice());
}

void FixLbmPsmBC::post_force(long ntimestep) {
  if (ntimestep % fix_.nevery) return;
  if (lbmpsm_apply_bc(fix_.lattice()) != LBMPSM_OK) lib_error(fix_.lattice());
}

// ------------------------------------------------------------------ lbm-psm-vti
FixLbmPsmVTI::FixLbmPsmVTI(const std::vector<std::string>& args, FixLbmPsm& fix,
                           std::string folder)
    : fix_(fix), folder_(std::move(folder)) {
  const int narg = (int)args.size();
  if (narg < 5) throw LammpsError("Illegal fix lbm-psm-vti command");
  int iarg = 3;
  while (iarg < narg) {
    const std::string& kw = args[iarg];
    if (iarg + 2 > narg) throw LammpsError("Illegal fix lbm-psm-vti command");
    if (kw == "every") {
      nevery_ = (int)inumeric(args[iarg + 1]);
      if (nevery_ <= 0) throw LammpsError("Illegal fix lbm-psm-vti command");
    } else if (kw == "binary" || kw == "useDouble") {
      const long v = inumeric(args[iarg + 1]);
      if (v < 0 || v > 1) throw LammpsError("Illegal fix lbm-psm-vti command");
      (kw == "binary" ? binary_ : useDouble_) = v == 1;
    } else {
      throw LammpsError("Illegal fix lbm-psm-vti command");
    }
    iarg += 2;
  }
  if (nevery_ == 0) throw LammpsError("Illegal fix lbm-psm-vti command");
}

void FixLbmPsmVTI::init() {
  std::filesystem::remove_all(folder_);
  std::filesystem::create_directories(folder_);
  write(0, 0.0);
}

void FixLbmPsmVTI::before_lbm_step(long ntimestep) {
  for (long t = ntimestep + 1; t < ntimestep + 1 + fix_.nevery; ++t)
    if (t % nevery_ == 0) {
      lbmpsm_request_macro(fix_.lattice());
      break;
    }
}

void FixLbmPsmVTI::pre_force(long ntimestep) {
  if (ntimestep % nevery_) return;
  write(ntimestep, fix_.info().Uc / fix_.info().u_lb);
}

// one-process form of WriteVTI::execute_write_vti's file output
// (src/fix_LBM_PSM_writeVTI.h:171-253)
std::string FixLbmPsmVTI::write(long timestep, double u0) {
  lbmpsm_handle* h = fix_.lattice();
  lbmpsm_info in{};
  lbmpsm_get_info(h, &in);
  const int dim = in.dimension;
  const long nx_i = in.local[0] - 2, ny_i = in.local[1] - 2, nz_i = dim == 3 ? in.local[2] - 2 : 1;
  const size_t nP = (size_t)nx_i * ny_i * nz_i;
  const size_t es = useDouble_ ? 8 : 4;
  std::vector<unsigned char> solid(es * nP), rho(es * nP), u(3 * es * nP);
  if (lbmpsm_export_fields(h, useDouble_ ? 1 : 0, 1.0, fix_.get_rho(), u0, solid.data(),
                           rho.data(), u.data()) != LBMPSM_OK)
    lib_error(h);
  return write_vti_files(folder_, fileName_, timestep, dim, in.local, fix_.origin, in.dx, binary_,
                         useDouble_, solid.data(), rho.data(), u.data());
}

std::string write_vti_files(const std::string& folder, const std::string& file_name, long timestep,
                            int dim, const int local[3], const double origin[3], double dx,
                            bool binary, bool use_double, const void* solid_p, const void* rho_p,
                            const void* u_p) {
  const long nx_i = local[0] - 2, ny_i = local[1] - 2, nz_i = dim == 3 ? local[2] - 2 : 1;
  const size_t nP = (size_t)nx_i * ny_i * nz_i;
  const size_t es = use_double ? 8 : 4;
  const unsigned char* solid = static_cast<const unsigned char*>(solid_p);
  const unsigned char* rho = static_cast<const unsigned char*>(rho_p);
  const unsigned char* u = static_cast<const unsigned char*>(u_p);
  // coordinate of local node (1,1,1): origin + i*dx - dx (src/LBM_PSM_lattice.cpp:162-164)
  const double* o = origin;
  const double ox = o[0] + 1 * dx - dx * 1;
  const double oy = o[1] + 1 * dx - dx * 1;
  const double oz = dim == 3 ? o[2] + 1 * dx - dx * 1 : 0.0;
  const std::string type = use_double ? "Float64" : "Float32";
  char stamp[32];
  std::snprintf(stamp, sizeof stamp, "%08ld", timestep);
  const std::string base = file_name + "." + stamp;
  const std::string vname = folder + "/" + base + "_rank0.vti";
  const std::string ext = "0 " + std::to_string(nx_i - 1) + " 0 " + std::to_string(ny_i - 1) +
                          " 0 " + std::to_string(nz_i - 1);
  const std::string org = fmt(ox) + " " + fmt(oy) + " " + fmt(oz);
  const std::string spacing = fmt(dx) + " " + fmt(dx) + " " + fmt(dx);
  if (binary) {
    const uint32_t b_sz = (uint32_t)(nP * es), u_sz = (uint32_t)(3 * nP * es);
    std::ofstream f(vname, std::ios::binary);
    f << "<?xml version=\"1.0\"?>\n<VTKFile type=\"ImageData\" version=\"1.0\" "
         "byte_order=\"LittleEndian\" header_type=\"UInt32\">\n"
      << " <ImageData WholeExtent=\"" << ext << "\" Origin=\"" << org << "\" Spacing=\""
      << spacing << "\">\n"
      << "  <Piece Extent=\"" << ext << "\">\n"
      << "   <PointData>\n"
      << "    <DataArray type=\"" << type << "\" Name=\"SolidFraction\" format=\"appended\" offset=\"0\"/>\n"
      << "    <DataArray type=\"" << type << "\" Name=\"Density\" format=\"appended\" offset=\""
      << (4 + (size_t)b_sz) << "\"/>\n"
      << "    <DataArray type=\"" << type
      << "\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"appended\" offset=\""
      << 2 * (4 + (size_t)b_sz) << "\"/>\n"
      << "   </PointData>\n  </Piece>\n </ImageData>\n <AppendedData encoding=\"raw\">_";
    auto put = [&](uint32_t sz, const unsigned char* d) {
      f.write(reinterpret_cast<const char*>(&sz), sizeof sz);
      f.write(reinterpret_cast<const char*>(d), (std::streamsize)sz);
    };
    put(b_sz, solid);
    put(b_sz, rho);
    put(u_sz, u);
    f << "\n </AppendedData>\n</VTKFile>";
  } else {
    std::ofstream f(vname);
    f << "<?xml version=\"1.0\"?>\n<VTKFile type=\"ImageData\" version=\"0.1\">\n"
      << " <ImageData WholeExtent=\"" << ext << "\" Origin=\"" << org << "\" Spacing=\""
      << spacing << "\">\n"
      << "  <Piece Extent=\"" << ext << "\">\n   <PointData>\n";
    auto value = [&](const unsigned char* d, size_t i) {
      if (use_double) {
        double x;
        std::memcpy(&x, d + 8 * i, 8);
        return x;
      }
      float x;
      std::memcpy(&x, d + 4 * i, 4);
      return (double)x;
    };
    struct Arr {
      const char* name;
      int comp;
      const unsigned char* d;
    };
    const Arr arrs[3] = {{"SolidFraction", 1, solid}, {"Density", 1, rho}, {"Velocity", 3, u}};
    for (const Arr& ar : arrs) {
      f << "    <DataArray type=\"" << type << "\" Name=\"" << ar.name
        << "\" NumberOfComponents=\"" << ar.comp << "\" format=\"ascii\">\n";
      const size_t cnt = nP * (size_t)ar.comp;
      for (size_t i = 0; i < cnt; ++i) f << fmt(value(ar.d, i)) << (i % 10 == 9 ? "\n" : " ");
      f << "\n    </DataArray>\n";
    }
    f << "   </PointData>\n  </Piece>\n </ImageData>\n</VTKFile>";
  }
  std::ofstream p(folder + "/" + base + ".pvti");
  p << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PImageData\" version=\"0.1\">\n"
    << " <PImageData WholeExtent=\"" << ext << "\" Origin=\"" << org << "\" Spacing=\""
    << spacing << "\">\n"
    << "  <PPointData>\n"
    << "   <PDataArray type=\"" << type << "\" Name=\"SolidFraction\"/>\n"
    << "   <PDataArray type=\"" << type << "\" Name=\"Density\"/>\n"
    << "   <PDataArray type=\"" << type << "\" Name=\"Velocity\" NumberOfComponents=\"3\"/>\n"
    << "  </PPointData>\n"
    << "  <Piece Extent=\"" << ext << "\" Source=\"" << base << "_rank0.vti\"/>\n"
    << " </PImageData>\n</VTKFile>";
  return vname;
}

// ------------------------------------------------------------------ restart
std::string restart_file_name(int rank) {
  return "LBM-PSM-restartFile-processor-" + std::to_string(rank) + ".bin";
}

void write_restart(const std::string& path, const std::vector<double>& f) {
  if (f.size() >= (size_t)1 << 32)
    throw LammpsError("lbm-psm-restart: local array too large for the 32-bit size field");
  std::ofstream o(path, std::ios::binary);
  const uint32_t n = (uint32_t)f.size();
  o.write(reinterpret_cast<const char*>(&n), sizeof n);
  o.write(reinterpret_cast<const char*>(f.data()), (std::streamsize)(8 * f.size()));
  if (!o) throw LammpsError("lbm-psm-restart: cannot write " + path);
}

std::vector<double> read_restart(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  uint32_t n = 0;
  if (!in.read(reinterpret_cast<char*>(&n), sizeof n))
    throw LammpsError("lbm-psm-restart: cannot read " + path);
  std::vector<double> f(n);
  if (!in.read(reinterpret_cast<char*>(f.data()), (std::streamsize)(8 * (size_t)n)))
    throw LammpsError("lbm-psm-restart: " + path + " holds fewer than " + std::to_string(n) +
                      " values");
  return f;
}

FixLbmPsmRestart::FixLbmPsmRestart(const std::vector<std::string>& args, FixLbmPsm& fix,
                                   int rank, std::string folder)
    : fix_(fix) {
  const int narg = (int)args.size();
  if (narg < 9) throw LammpsError("Illegal fix lbm-psm-restart command");
  path_ = (std::filesystem::path(folder) / restart_file_name(rank)).string();
  int iarg = 3;
  while (iarg < narg) {
    const std::string& kw = args[iarg];
    if (kw != "every" && kw != "write" && kw != "read")
      throw LammpsError("Illegal fix lbm-psm-restart command");
    if (iarg + 2 > narg) throw LammpsError("Illegal fix lbm-psm-restart command");
    long v;
    try {
      v = inumeric(args[iarg + 1]);
    } catch (const LammpsError&) {
      throw LammpsError("Illegal fix lbm-psm-restart command");
    }
    if (kw == "every") {
      if (v <= 0) throw LammpsError("Illegal fix lbm-psm-restart command");
      nevery_ = (int)v;
    } else {
      if (v < 0 || v > 1) throw LammpsError("Illegal fix lbm-psm-restart command");
      (kw == "write" ? iWrite_ : iRead_) = (int)v;
    }
    iarg += 2;
  }
}

void FixLbmPsmRestart::init() {
  if (iRead_ != 1) return;
  const lbmpsm_info& in = fix_.info();
  const size_t want = (size_t)in.local[0] * in.local[1] * in.local[2] * in.q;
  std::vector<double> f = read_restart(path_);
  if (f.size() != want)
    throw LammpsError("lbm-psm-restart: " + path_ + " holds " + std::to_string(f.size()) +
                      " values, the lattice needs " + std::to_string(want));
  if (lbmpsm_set_populations(fix_.lattice(), f.data()) != LBMPSM_OK) lib_error(fix_.lattice());
}

void FixLbmPsmRestart::pre_force(long ntimestep) {
  if (ntimestep % nevery_) return;
  if (iWrite_ != 1) return;
  const lbmpsm_info& in = fix_.info();
  std::vector<double> f((size_t)in.local[0] * in.local[1] * in.local[2] * in.q);
  if (lbmpsm_get_populations(fix_.lattice(), f.data()) != LBMPSM_OK) lib_error(fix_.lattice());
  write_restart(path_, f);
}

}  // namespace lbmpsm_host
