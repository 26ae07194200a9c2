/*
 * ff_oracle.h -- CPU FP64 cutoff Lennard-Jones + reaction-field forces (the CutoffPeriodic form
 * of OpenMM's NonbondedForce), O(N^2) minimum image. TEST INFRASTRUCTURE ONLY.
 */
#ifndef RBX_FF_ORACLE_H
#define RBX_FF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* num_systems independent cubic boxes; system s holds atoms [atom_offsets[s], atom_offsets[s+1])
 * with edge box[s] and cutoff cutoff[s] (< box/2). pos[3*natoms]; per-atom charge (e), sigma
 * (nm), epsilon (kJ/mol), body id (pairs with equal positive id excluded). Writes force
 * [3*natoms] (kJ/mol/nm) and energy[num_systems] (kJ/mol). */
void orc_lj_rf(int num_systems, const int* atom_offsets, const double* box, const double* cutoff, double eps_solvent,
               const double* pos, const double* charge, const double* sigma, const double* epsilon, const int* body,
               double* force, double* energy, int nthreads);

/* Forces on the selected atoms only (force[3*num_selected]) of one box holding atoms [a0, a1):
 * spot checks of systems too large for the all-pairs loop over every atom. */
void orc_lj_rf_atoms(int a0, int a1, double L, double rc, double eps_solvent, const double* pos, const double* charge,
                     const double* sigma, const double* epsilon, const int* body, int num_selected,
                     const int* selected, double* force);

#ifdef __cplusplus
}
#endif
#endif
