/* Stub of LAMMPS atom.h (TEST INFRASTRUCTURE ONLY): the reference's LBM
 * library includes it but uses nothing from it. */
#ifndef ORACLE_STUB_ATOM_H
#define ORACLE_STUB_ATOM_H
#endif
