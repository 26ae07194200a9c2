/*
 * rbx_oracle.h -- CPU restatement (FP64, plain C) of the OpenMM rigid-body plugin's integrator.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path: tests/, the smoke
 * check and bench.py's CPU arm may load it; the product (openmm_rigidbody_plugin_gb300) never
 * links, loads or falls back to it.
 *
 * Two flavours, selected per system with `robust`:
 *   robust = 0  restates the reference's CPU code path step by step (Smith/Kopp eigensolver,
 *               signed-component orthonormal(), no pcm reset, elliptic exact rotation only);
 *               pinned against the reference itself through tests/golden/.
 *   robust = 1  the project's robust FP64 oracle: cyclic-Jacobi eigensolver, |component|
 *               orthonormal(), pcm reset, singleton bodies become free atoms, and closed-form free
 *               rotation for spherical, symmetric and linear tops, where the reference divides
 *               by zero (reference defects D1-D5).
 */
#ifndef RBX_ORACLE_H
#define RBX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_system orc_system;

/* Body record layout returned by orc_get_body (36 doubles), same order as the reference harness:
 * N, dof, loc, mass, I[3], invI[3], rcm[3], pcm[3], q[4], pi[4], force[3], torque[4], twoKt, twoKr */
#define ORC_BODY_RECORD 36

const char* orc_last_error(void);

/* RigidBodySystem::initialize (openmmapi/src/RigidBodySystem.cpp:55-114) for a system without
 * virtual sites or constraints. */
orc_system* orc_create(int natoms, const double* masses, const int* body_indices, int mode, int robust);
void orc_destroy(orc_system* s);

/* RigidBodySystem::update(geometry=true, velocities=true) (RigidBodySystem.cpp:120-142). */
int orc_setup(orc_system* s, const double* R, const double* V, const double* F);

/* RigidBodySystem::integratePart1 / integratePart2 (RigidBodySystem.cpp:170-204).  Arrays are
 * [natoms*3] in the user's atom order. */
void orc_part1(orc_system* s, double dt, const double* F, double* V, double* R);
void orc_part2(orc_system* s, double dt, const double* R, const double* F, double* V);

/* RigidBodySystem::computeKineticEnergies (RigidBodySystem.cpp:210-220): out[0]=KE_t, out[1]=KE_r */
void orc_kinetic(orc_system* s, const double* V, double* out);

/* Refined ("shadow") energies, the reference's COMPMOD path (RigidBodyIntegrator::
 * setComputeRefinedEnergies, openmmapi/src/RigidBodyIntegrator.cpp:34-38; kernels in
 * platforms/cuda/src/kernels/rigidbodyintegrator.cu:238-243, :285-292, :318-321, :380-384,
 * :433-469). mode 0 = off, 1 = on, 2 = on with the reference's free-atom weights (which give
 * 4/3 of the kinetic energy for uniform motion). While on, part1/part2 accumulate the stencils;
 * orc_refined gives [KE_t, KE_r, U_refinement] after a part2, F = that part2's force array. */
void orc_set_refined(orc_system* s, int mode);
void orc_refined(orc_system* s, const double* V, const double* F, double dt, double* out);

int orc_num_dof(const orc_system* s);
int orc_num_bodies(const orc_system* s);
int orc_num_free(const orc_system* s);
int orc_num_body_atoms(const orc_system* s);
int orc_atom_index(const orc_system* s, int i);        /* free atoms first, then body atoms */
void orc_get_body(const orc_system* s, int i, double* out);
void orc_get_body_fixed(const orc_system* s, double* out); /* [num_body_atoms*3] */

/* Replace the state of body i: rcm[3], pcm[3], q[4], pi[4] (geometry unchanged). */
void orc_set_body_state(orc_system* s, int i, const double* rcm, const double* pcm,
                        const double* q, const double* pi);
/* Replace the geometry of body i: I[3], body-frame positions d[N*3] (dof recomputed from I[2]). */
void orc_set_body_geometry(orc_system* s, int i, const double* I, const double* d);

/* nsteps of Part1 + Part2 with a fixed force array (integrator-only timing), body and free-atom
 * loops split over nthreads POSIX threads. Returns wall seconds. */
double orc_run_fixed_force(orc_system* s, double dt, const double* F, double* V, double* R,
                           int nsteps, int nthreads);

/* Single-body primitives, exposed for unit tests. q, pi updated in place. */
void orc_exact_rotation(const double* I, const double* invI, double* q, double* pi,
                        double dt, int robust);
void orc_nosquish_rotation(const double* invI, int dof, double* q, double* pi, double dt, int n);
void orc_jacobi_sncndn(double u, double m, double* sn, double* cn, double* dn);
double orc_carlson_rc(double x, double y);
double orc_carlson_rf(double x, double y, double z);
double orc_carlson_rj(double x, double y, double z, double p);
/* Symmetric 3x3 eigen-decomposition: values descending in w, eigenvectors as ROWS of A.
 * robust=0: Smith/Kopp as in openmmapi/src/eigenDecomposition.cpp; robust=1: cyclic Jacobi. */
void orc_eigen(const double* M, double* w, double* A, int robust);

#ifdef __cplusplus
}
#endif
#endif
