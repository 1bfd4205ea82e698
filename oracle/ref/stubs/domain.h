/* Stub of LAMMPS domain.h (TEST INFRASTRUCTURE ONLY): included by the
 * reference's LBM library, nothing from it is used. */
#ifndef ORACLE_STUB_DOMAIN_H
#define ORACLE_STUB_DOMAIN_H
#endif
