/*
 * ff_oracle.c -- CPU (FP64, plain C) cutoff Lennard-Jones + reaction-field forces.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA force kernels (csrc/rbx_forces.cu). The
 * product never links or loads it.
 *
 * The functional form is that of OpenMM's NonbondedForce with the CutoffPeriodic method, as the
 * OpenMM user guide documents it (OpenMM itself is not part of the reference plugin and is not
 * installed here, so parity with OpenMM is unpinned; the form is restated from the documented
 * equations):
 *   E_coul = K q_i q_j (1/r + k_rf r^2 - c_rf),  k_rf = (eps_s - 1) / ((2 eps_s + 1) rc^3),
 *                                                 c_rf = 1/rc + k_rf rc^2,
 *   E_lj   = 4 eps_ij ((sigma_ij/r)^12 - (sigma_ij/r)^6)   (no switching, no shift),
 *   sigma_ij = (sigma_i + sigma_j)/2, eps_ij = sqrt(eps_i eps_j)   (Lorentz-Berthelot),
 * for r < rc under the minimum-image convention of a cubic box, K = 138.935456 kJ nm/(mol e^2).
 * Pairs of atoms of the same rigid body are excluded altogether, as the plugin's ForceField
 * helper removes intra-body nonbonded interactions (python/forcefield.py:131-138).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>

#include "ff_oracle.h"

#define ONE_4PI_EPS0 138.935456

typedef struct {
    const double *pos, *charge, *sigma, *epsilon;
    const int* body;
    int a0, a1;
    double L, rc, krf, crf;
} ff_box;

/* Force on atom i and its half share of the pair energies (each pair is seen from both ends). */
static void atom_force(const ff_box* b, int i, double* f, double* e_half) {
    const double rc2 = b->rc * b->rc;
    double fx = 0, fy = 0, fz = 0, e = 0;
    for (int j = b->a0; j < b->a1; j++) {
        if (j == i) continue;
        if (b->body[i] > 0 && b->body[i] == b->body[j]) continue;
        double d[3];
        for (int c = 0; c < 3; c++) {
            double x = b->pos[3 * i + c] - b->pos[3 * j + c];
            x -= b->L * nearbyint(x / b->L);
            d[c] = x;
        }
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 >= rc2) continue;
        const double r = sqrt(r2), inv_r2 = 1.0 / r2;
        const double qq = ONE_4PI_EPS0 * b->charge[i] * b->charge[j];
        const double sig = 0.5 * (b->sigma[i] + b->sigma[j]);
        const double eps = sqrt(b->epsilon[i] * b->epsilon[j]);
        const double s2 = sig * sig * inv_r2, s6 = s2 * s2 * s2;
        /* -dE/dr / r */
        double g = qq * (1.0 / (r2 * r) - 2.0 * b->krf) + 4.0 * eps * (12.0 * s6 * s6 - 6.0 * s6) * inv_r2;
        fx += g * d[0];
        fy += g * d[1];
        fz += g * d[2];
        e += qq * (1.0 / r + b->krf * r2 - b->crf) + 4.0 * eps * (s6 * s6 - s6);
    }
    f[0] = fx;
    f[1] = fy;
    f[2] = fz;
    *e_half = 0.5 * e;
}

static ff_box make_box(int s, const int* atom_offsets, const double* box, const double* cutoff, double eps_solvent,
                       const double* pos, const double* charge, const double* sigma, const double* epsilon,
                       const int* body) {
    ff_box b;
    b.pos = pos;
    b.charge = charge;
    b.sigma = sigma;
    b.epsilon = epsilon;
    b.body = body;
    b.a0 = atom_offsets[s];
    b.a1 = atom_offsets[s + 1];
    b.L = box[s];
    b.rc = cutoff[s];
    b.krf = (eps_solvent - 1.0) / ((2.0 * eps_solvent + 1.0) * b.rc * b.rc * b.rc);
    b.crf = 1.0 / b.rc + b.krf * b.rc * b.rc;
    return b;
}

typedef struct {
    int num_systems;
    const int* atom_offsets;
    const double *box, *cutoff, *pos, *charge, *sigma, *epsilon;
    const int* body;
    double eps_solvent;
    double *force, *energy;
    int tid, nthreads;
} ff_job;

static void* ff_worker(void* arg) {
    ff_job* J = (ff_job*)arg;
    for (int s = 0; s < J->num_systems; s++) {
        ff_box b = make_box(s, J->atom_offsets, J->box, J->cutoff, J->eps_solvent, J->pos, J->charge, J->sigma,
                            J->epsilon, J->body);
        for (int i = b.a0 + J->tid; i < b.a1; i += J->nthreads) {
            double e;
            atom_force(&b, i, J->force + 3 * (size_t)i, &e);
            J->energy[i] = e; /* per-atom share; summed per system in a fixed order below */
        }
    }
    return NULL;
}

void orc_lj_rf(int num_systems, const int* atom_offsets, const double* box, const double* cutoff, double eps_solvent,
               const double* pos, const double* charge, const double* sigma, const double* epsilon, const int* body,
               double* force, double* energy, int nthreads) {
    const int natoms = atom_offsets[num_systems];
    double* e_atom = (double*)malloc(sizeof(double) * (size_t)(natoms > 0 ? natoms : 1));
    if (nthreads < 1) nthreads = 1;
    ff_job* jobs = (ff_job*)malloc(sizeof(ff_job) * (size_t)nthreads);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        ff_job J = {num_systems, atom_offsets, box, cutoff, pos, charge, sigma, epsilon, body, eps_solvent,
                    force, e_atom, t, nthreads};
        jobs[t] = J;
        if (t > 0) pthread_create(&th[t], NULL, ff_worker, &jobs[t]);
    }
    ff_worker(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    for (int s = 0; s < num_systems; s++) {
        double e = 0.0;
        for (int i = atom_offsets[s]; i < atom_offsets[s + 1]; i++) e += e_atom[i];
        energy[s] = e;
    }
    free(th);
    free(jobs);
    free(e_atom);
}

void orc_lj_rf_atoms(int a0, int a1, double L, double rc, double eps_solvent, const double* pos, const double* charge,
                     const double* sigma, const double* epsilon, const int* body, int num_selected,
                     const int* selected, double* force) {
    int offsets[2] = {a0, a1};
    ff_box b = make_box(0, offsets, &L, &rc, eps_solvent, pos, charge, sigma, epsilon, body);
    for (int k = 0; k < num_selected; k++) {
        double e;
        atom_force(&b, selected[k], force + 3 * (size_t)k, &e);
    }
}
