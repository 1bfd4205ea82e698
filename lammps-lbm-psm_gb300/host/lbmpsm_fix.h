// lbmpsm_fix.h -- C++ host side of the LAMMPS drop-in over the C ABI
// (include/lbmpsm.h): the reference's fix classes with their argument
// syntax, error messages and per-step bookkeeping, and the lattice work done
// by the GPU library.
//
// The reference fixes (src/fix_LBM_PSM.{h,cpp}, src/fix_LBM_PSM_BC.{h,cpp},
// src/fix_LBM_PSM_writeVTI.{h,cpp}, src/fix_LBM_PSM_writeReadRestart.{h,cpp})
// are LAMMPS Fix subclasses; LAMMPS owns the atoms, the ghost images and the
// reverse communication.  Without a LAMMPS tree these classes run over a
// minimal stand-in for that state (Domain, Atoms) with LAMMPS' one-process
// ghost generation and reverse communication restated, so that a standalone
// driver runs the call sequence a LAMMPS build would.  In a LAMMPS build the
// same member functions become the fixes' init / post_force / pre_force, the
// stand-ins become atom->x / v / omega / radius / f / torque, and
// LammpsError becomes error->all.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "lbmpsm.h"

namespace lbmpsm_host {

// error->all(FLERR, msg) of the reference
class LammpsError : public std::runtime_error {
 public:
  explicit LammpsError(const std::string& m) : std::runtime_error(m) {}
};

// domain->dimension, boxlo, boxhi, x/y/zperiodic
struct Domain {
  int dimension = 3;
  double boxlo[3] = {0.0, 0.0, 0.0};
  double boxhi[3] = {1.0, 1.0, 1.0};
  int periodic[3] = {1, 1, 1};
  double prd(int d) const { return boxhi[d] - boxlo[d]; }
};

// Owned atoms (nlocal) followed by ghost images, in LAMMPS order; vectors of
// triples are row-major n x 3.
struct Atoms {
  int nlocal = 0;
  std::vector<int> tag;
  std::vector<double> x, v, omega, radius;
  std::vector<double> f, torque;
  std::vector<int> owner;  // image -> the image it was copied from (itself for owned atoms)
  std::vector<int> swap;   // swap that created a ghost (-1 for owned atoms)
  int size() const { return (int)tag.size(); }
};

// CommBrick::borders() on one process: per periodic dimension, every atom
// present so far with coord <= lo + cutghost is imaged at +prd, then every
// atom with coord >= hi - cutghost at -prd (both swaps scan the same atoms).
Atoms ghost_images(const Domain& d, double cutghost, const Atoms& owned);
// CommBrick::reverse_comm() on one process: swaps in reverse order, each
// ghost's row (3 values) added into the image it was copied from.
void reverse_comm(std::vector<double>& rows3, const Atoms& a);

// fix ID group lbm-psm every N Nlc N lc L rho R nu NU Re RE [tau T] [Fext fx fy fz]
// (src/fix_LBM_PSM.cpp:15-83 arguments, :104-177 init, :181-266 post_force).
class FixLbmPsm {
 public:
  explicit FixLbmPsm(const std::vector<std::string>& args,
                     int storage = LBMPSM_STORAGE_FP64, int device = 0, double max_radius = 0.0);
  ~FixLbmPsm();
  FixLbmPsm(const FixLbmPsm&) = delete;
  FixLbmPsm& operator=(const FixLbmPsm&) = delete;

  // builds the lattice (again on every run, without leaking the previous
  // one) and returns the DEM timestep the reference writes to update->dt
  double init(const Domain& d);
  // an LBM coupling step every nevery timesteps: locals get +=, ghosts get =,
  // then ghosts are reverse-summed into their owners; on other steps the
  // stored hydrodynamic force / torque of the locals is added again
  void post_force(long ntimestep, Atoms& a);

  double get_rho() const { return rho_; }
  lbmpsm_handle* lattice() const { return h_; }
  const lbmpsm_info& info() const { return info_; }
  int nevery = 1;
  std::vector<double> hydro;  // n x 6: F, T of the last LBM step per image
  double virial[6] = {0, 0, 0, 0, 0, 0};  // stresslet summed over the images
  double origin[3] = {0, 0, 0};            // lattice origin (z = 0 in 2-D)

 private:
  lbmpsm_fix_params prm_{};
  bool have_[5] = {false, false, false, false, false};  // Nlc lc rho nu Re given
  double rho_ = 0.0;
  int storage_, device_;
  double max_radius_;
  lbmpsm_handle* h_ = nullptr;
  lbmpsm_info info_{};
};

// fix ID group lbm-psm-bc KEYWORD (src/fix_LBM_PSM_BC.cpp:16-39, 145-402)
class FixLbmPsmBC {
 public:
  FixLbmPsmBC(const std::vector<std::string>& args, FixLbmPsm& fix);
  void init();
  void post_force(long ntimestep);
  int type() const { return type_; }

 private:
  FixLbmPsm& fix_;
  int type_ = LBMPSM_BC_NONE;
};

// fix ID group lbm-psm-vti every N [binary 0|1] [useDouble 0|1]
// (src/fix_LBM_PSM_writeVTI.cpp:15-114, src/fix_LBM_PSM_writeVTI.h:82-253),
// one process: per output step one .vti piece and the .pvti master file.
class FixLbmPsmVTI {
 public:
  FixLbmPsmVTI(const std::vector<std::string>& args, FixLbmPsm& fix,
               std::string folder = "flow_field_output_data");
  void init();
  // the reference reads the macroscopic fields of the previous LBM step in
  // pre_force; the library stores them only on request, so this asks for
  // them before the LBM step whose fields the next written step reads
  void before_lbm_step(long ntimestep);
  void pre_force(long ntimestep);
  std::string write(long timestep, double u0);

 private:
  FixLbmPsm& fix_;
  std::string folder_, fileName_ = "flow_field";
  bool binary_ = true, useDouble_ = false;
  int nevery_ = 0;
};

// fix ID group lbm-psm-restart every N write 0|1 read 0|1
// (src/fix_LBM_PSM_writeReadRestart.cpp:15-103)
class FixLbmPsmRestart {
 public:
  FixLbmPsmRestart(const std::vector<std::string>& args, FixLbmPsm& fix, int rank = 0,
                   std::string folder = ".");
  void init();
  void pre_force(long ntimestep);

 private:
  FixLbmPsm& fix_;
  int nevery_ = 1, iWrite_ = 0, iRead_ = 0;
  std::string path_;
};

// The files of one `fix lbm-psm-vti` output step on one process
// (src/fix_LBM_PSM_writeVTI.h:171-253): the .vti piece of the interior
// nodes and the .pvti master file, for fields as lbmpsm_export_fields
// returns them (float or double as use_double; solid and rho one value per
// node, u three).  local: the local array sizes with the halo; origin: the
// domain's boxlo.  Returns the piece's path.
std::string write_vti_files(const std::string& folder, const std::string& file_name, long timestep,
                            int dimension, const int local[3], const double origin[3], double dx,
                            bool binary, bool use_double, const void* solid, const void* rho,
                            const void* u);

// the restart file of one rank: a uint32 count, then that many doubles
std::string restart_file_name(int rank);
void write_restart(const std::string& path, const std::vector<double>& f);
std::vector<double> read_restart(const std::string& path);

}  // namespace lbmpsm_host
