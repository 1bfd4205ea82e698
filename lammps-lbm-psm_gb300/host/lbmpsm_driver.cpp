// lbmpsm_driver -- a standalone host driver running the LAMMPS call sequence
// of the lbm-psm fixes (lbmpsm_fix.h) from a small input deck, with a minimal
// DEM stepper in place of LAMMPS' integrators.
//
//   lbmpsm_driver DECK            run the deck
//   lbmpsm_driver --check DECK    parse the deck and construct the fixes only
//                                 (argument errors are reported, no GPU used)
//
// Deck lines (# starts a comment):
//   dimension 2|3
//   boundary p|f p|f p|f
//   box xlo xhi ylo yhi zlo zhi
//   atoms FILE          one atom per line: tag x y z vx vy vz wx wy wz radius density
//   cutghost C          ghost cut-off (communicate cutoff of the LAMMPS run)
//   storage fp64|fp32|fp16|bf16
//   fix ID group STYLE args...   STYLE = lbm-psm | lbm-psm-bc | lbm-psm-vti | lbm-psm-restart
//   dem none|nve        none: atoms held in place; nve: explicit update with the
//                       hydrodynamic force and torque (sphere mass and inertia from
//                       density), periodic wrap
//   output FILE         per timestep: "step N", then per owned atom: tag F[3] T[3]
//                       (the coupling steps' forces and, on the timesteps between
//                       them, the stored forces the fix re-applies)
//   run N
//
// Per timestep, in LAMMPS' order: ghost images of the owned atoms, pre_force
// (vti, restart), post_force (lbm-psm, then lbm-psm-bc), then the DEM update.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>

#include "lbmpsm_fix.h"

using namespace lbmpsm_host;

namespace {

struct Deck {
  Domain dom;
  std::string atoms_file, output_file, dem = "none";
  double cutghost = 0.0;
  int storage = LBMPSM_STORAGE_FP64;
  long nrun = 0;
  std::vector<std::vector<std::string>> fixes;
};

std::vector<std::string> words(const std::string& line) {
  std::istringstream in(line.substr(0, line.find('#')));
  std::vector<std::string> w;
  std::string s;
  while (in >> s) w.push_back(s);
  return w;
}

Deck read_deck(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw LammpsError("Cannot open input script " + path);
  Deck d;
  std::string line;
  while (std::getline(in, line)) {
    const auto w = words(line);
    if (w.empty()) continue;
    const std::string& c = w[0];
    auto need = [&](size_t k) {
      if (w.size() < k) throw LammpsError("Illegal " + c + " command");
    };
    if (c == "dimension") {
      need(2);
      d.dom.dimension = std::stoi(w[1]);
    } else if (c == "boundary") {
      need(4);
      for (int k = 0; k < 3; ++k) d.dom.periodic[k] = w[1 + k] == "p" ? 1 : 0;
    } else if (c == "box") {
      need(7);
      for (int k = 0; k < 3; ++k) {
        d.dom.boxlo[k] = std::stod(w[1 + 2 * k]);
        d.dom.boxhi[k] = std::stod(w[2 + 2 * k]);
      }
    } else if (c == "atoms") {
      need(2);
      d.atoms_file = w[1];
    } else if (c == "cutghost") {
      need(2);
      d.cutghost = std::stod(w[1]);
    } else if (c == "storage") {
      need(2);
      d.storage = w[1] == "fp32"   ? LBMPSM_STORAGE_FP32
                  : w[1] == "fp16" ? LBMPSM_STORAGE_FP16
                  : w[1] == "bf16" ? LBMPSM_STORAGE_BF16
                                   : LBMPSM_STORAGE_FP64;
    } else if (c == "fix") {
      need(4);
      d.fixes.emplace_back(w.begin() + 1, w.end());  // ID group style args...
    } else if (c == "dem") {
      need(2);
      d.dem = w[1];
    } else if (c == "output") {
      need(2);
      d.output_file = w[1];
    } else if (c == "run") {
      need(2);
      d.nrun = std::stol(w[1]);
    } else {
      throw LammpsError("Unknown command: " + line);
    }
  }
  return d;
}

// owned atoms and their densities
Atoms read_atoms(const std::string& path, std::vector<double>& density) {
  std::ifstream in(path);
  if (!in) throw LammpsError("Cannot open atom file " + path);
  Atoms a;
  std::string line;
  while (std::getline(in, line)) {
    const auto w = words(line);
    if (w.empty()) continue;
    if (w.size() != 12) throw LammpsError("Atom line needs 12 values: " + line);
    a.tag.push_back(std::stoi(w[0]));
    for (int k = 0; k < 3; ++k) a.x.push_back(std::stod(w[1 + k]));
    for (int k = 0; k < 3; ++k) a.v.push_back(std::stod(w[4 + k]));
    for (int k = 0; k < 3; ++k) a.omega.push_back(std::stod(w[7 + k]));
    a.radius.push_back(std::stod(w[10]));
    density.push_back(std::stod(w[11]));
  }
  a.nlocal = a.size();
  return a;
}

struct Fixes {
  std::unique_ptr<FixLbmPsm> lbm;
  std::unique_ptr<FixLbmPsmBC> bc;
  std::unique_ptr<FixLbmPsmVTI> vti;
  std::unique_ptr<FixLbmPsmRestart> restart;
};

// the fixes in definition order; the sibling fixes find the lbm-psm fix the
// way the reference's do (the first one defined)
Fixes make_fixes(const Deck& d) {
  Fixes f;
  for (const auto& w : d.fixes) {
    std::vector<std::string> args = w;  // ID group style args...
    const std::string& style = args[2];
    if (style == "lbm-psm") {
      f.lbm = std::make_unique<FixLbmPsm>(args, d.storage);
    } else if (style == "lbm-psm-bc" || style == "lbm-psm-vti" || style == "lbm-psm-restart") {
      if (!f.lbm) throw LammpsError("Fix " + style + " requires fix lbm-psm");
      if (style == "lbm-psm-bc") f.bc = std::make_unique<FixLbmPsmBC>(args, *f.lbm);
      if (style == "lbm-psm-vti") f.vti = std::make_unique<FixLbmPsmVTI>(args, *f.lbm);
      if (style == "lbm-psm-restart") f.restart = std::make_unique<FixLbmPsmRestart>(args, *f.lbm);
    } else {
      throw LammpsError("Unrecognized fix style '" + style + "'");
    }
  }
  if (!f.lbm) throw LammpsError("The deck defines no fix lbm-psm");
  return f;
}

// explicit update of the owned atoms with their total force and torque
void dem_nve(const Domain& dom, double dt, const std::vector<double>& density, Atoms& own,
             const Atoms& step) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < own.nlocal; ++i) {
    const double r = own.radius[i];
    const double m = dom.dimension == 3 ? density[i] * 4.0 / 3.0 * pi * r * r * r
                                        : density[i] * pi * r * r;
    const double I = (dom.dimension == 3 ? 0.4 : 0.5) * m * r * r;
    for (int c = 0; c < 3; ++c) {
      own.v[3 * i + c] += dt * step.f[3 * i + c] / m;
      own.omega[3 * i + c] += dt * step.torque[3 * i + c] / I;
      double x = own.x[3 * i + c] + dt * own.v[3 * i + c];
      if (c < dom.dimension && dom.periodic[c]) {
        const double lo = dom.boxlo[c], L = dom.prd(c);
        x = lo + std::fmod(std::fmod(x - lo, L) + L, L);
      }
      own.x[3 * i + c] = x;
    }
  }
}

int run(const std::string& path, bool check_only) {
  const Deck d = read_deck(path);
  Fixes f = make_fixes(d);
  if (check_only) {
    std::printf("deck ok: %zu fixes\n", d.fixes.size());
    return 0;
  }
  std::vector<double> density;
  Atoms own = read_atoms(d.atoms_file, density);
  const double dt = f.lbm->init(d.dom);
  if (f.bc) f.bc->init();
  if (f.restart) f.restart->init();
  if (f.vti) f.vti->init();
  FILE* out = d.output_file.empty() ? nullptr : std::fopen(d.output_file.c_str(), "w");
  for (long t = 0; t < d.nrun; ++t) {
    Atoms a = ghost_images(d.dom, d.cutghost, own);
    if (f.vti) f.vti->pre_force(t);
    if (f.restart) f.restart->pre_force(t);
    if (f.vti) f.vti->before_lbm_step(t);
    f.lbm->post_force(t, a);
    if (f.bc) f.bc->post_force(t);
    if (out) {
      std::fprintf(out, "step %ld\n", t);
      for (int i = 0; i < a.nlocal; ++i) {
        std::fprintf(out, "%d", a.tag[i]);
        for (int c = 0; c < 3; ++c) std::fprintf(out, " %.17g", a.f[3 * i + c]);
        for (int c = 0; c < 3; ++c) std::fprintf(out, " %.17g", a.torque[3 * i + c]);
        std::fprintf(out, "\n");
      }
    }
    if (d.dem == "nve") dem_nve(d.dom, dt, density, own, a);
  }
  if (out) std::fclose(out);
  std::printf("ran %ld steps, dt %.17g\n", d.nrun, dt);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const bool check = argc == 3 && std::string(argv[1]) == "--check";
  if (argc != 2 && !check) {
    std::fprintf(stderr, "usage: lbmpsm_driver [--check] DECK\n");
    return 2;
  }
  try {
    return run(argv[check ? 2 : 1], check);
  } catch (const LammpsError& e) {
    std::fprintf(stderr, "ERROR: %s\n", e.what());
    return 1;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ERROR: %s\n", e.what());
    return 1;
  }
}
