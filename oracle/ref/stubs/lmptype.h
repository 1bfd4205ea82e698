/* Stub of LAMMPS lmptype.h: only the integer types the reference's LBM
 * library uses (TEST INFRASTRUCTURE ONLY, for building the oracle). */
#ifndef ORACLE_STUB_LMPTYPE_H
#define ORACLE_STUB_LMPTYPE_H
#include <cstdint>
namespace LAMMPS_NS {
typedef int tagint;
typedef int64_t bigint;
}  // namespace LAMMPS_NS
#endif
