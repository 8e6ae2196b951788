/*
 * CPU oracle for the bonded forces -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of HyMD's f2py Fortran kernels, used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the checker.
 * Nothing in the hymd_gb300 product path loads this library.
 *
 *   orc_bonds_f32 / orc_angles_f32 / orc_dihedrals_f32 : cbf / caf / cdf
 *       (hymd/compute_bond_forces.f90, hymd/compute_angle_forces.f90,
 *        hymd/compute_dihedral_forces.f90, hymd/dipole_reconstruction.f90)
 *   orc_bonds_f64 / orc_angles_f64 / orc_dihedrals_f64 : cbf_d / caf_d / cdf_d
 *       (the __double.f90 variants, which differ only in storage precision)
 *
 * Build: oracle/Makefile (gcc -O2 -shared -fPIC), output oracle/libbonded_oracle.so.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define RT float
#define SFX _f32
#include "bonded_oracle_impl.h"
#undef RT
#undef SFX

#define RT double
#define SFX _f64
#include "bonded_oracle_impl.h"
#undef RT
#undef SFX
