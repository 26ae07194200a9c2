// C entry points around the reference plugin's own CPU integrator (RigidBodySystem), compiled
// from the reference sources by oracle/Makefile into oracle/_ref/librefrb.so.
//
// Test infrastructure only: this library is the checker that pins the oracle restatement
// (oracle/rbx_oracle.c) and generates the golden fixtures under tests/golden/. It drives exactly
// the calls the Reference platform makes in one step (platforms/reference/src/
// ReferenceRigidBodyKernels.cpp:82-108) minus constraints, virtual sites and the force call:
//   RigidBodySystem::initialize  (openmmapi/src/RigidBodySystem.cpp:55-114)
//   RigidBodySystem::update      (openmmapi/src/RigidBodySystem.cpp:120-142)
//   RigidBodySystem::integratePart1/2 (openmmapi/src/RigidBodySystem.cpp:170-204)
//   RigidBodySystem::computeKineticEnergies (openmmapi/src/RigidBodySystem.cpp:210-220)
#include "RigidBodySystem.h"
#include "openmm/System.h"
#include "openmm/internal/ContextImpl.h"
#include <cstring>
#include <exception>
#include <string>
#include <vector>

using namespace OpenMM;
using namespace RigidBodyPlugin;

namespace {
thread_local std::string g_err;

struct RefHandle {
    System system;
    ContextImpl* ctx = nullptr;
    RigidBodySystem bodies;
    std::vector<int> bodyIndices;
    int mode = 0;
    std::vector<Vec3> R, V, F;
    ~RefHandle() { delete ctx; }
};

void toVec(const double* a, int n, std::vector<Vec3>& out) {
    out.resize(n);
    for (int i = 0; i < n; i++) out[i] = Vec3(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
}
void fromVec(const std::vector<Vec3>& v, double* a) {
    for (size_t i = 0; i < v.size(); i++) { a[3 * i] = v[i][0]; a[3 * i + 1] = v[i][1]; a[3 * i + 2] = v[i][2]; }
}
}  // namespace

extern "C" {

const char* refrb_last_error() { return g_err.c_str(); }

void* refrb_create(int natoms, const double* masses, const int* bodyIndices, int mode) {
    try {
        RefHandle* h = new RefHandle();
        for (int i = 0; i < natoms; i++) h->system.addParticle(masses[i]);
        h->ctx = new ContextImpl(h->system);
        h->bodyIndices.assign(bodyIndices, bodyIndices + natoms);
        h->mode = mode;
        return h;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void refrb_destroy(void* p) { delete static_cast<RefHandle*>(p); }

// Context creation plus setPositions: initialize, then update(geometry, velocities).
int refrb_set_state(void* p, const double* R, const double* V, const double* F) {
    RefHandle* h = static_cast<RefHandle*>(p);
    try {
        int n = h->system.getNumParticles();
        toVec(R, n, h->ctx->positions);
        toVec(V, n, h->ctx->velocities);
        toVec(F, n, h->ctx->forces);
        h->bodies.initialize(*h->ctx, h->bodyIndices, h->mode);
        h->bodies.update(*h->ctx, true, true);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

void refrb_part1(void* p, double dt, const double* F, double* V, double* R) {
    RefHandle* h = static_cast<RefHandle*>(p);
    int n = h->system.getNumParticles();
    toVec(F, n, h->F); toVec(V, n, h->V); toVec(R, n, h->R);
    h->bodies.integratePart1(dt, h->F, h->V, h->R);
    fromVec(h->V, V); fromVec(h->R, R);
}

void refrb_part2(void* p, double dt, const double* R, const double* F, double* V) {
    RefHandle* h = static_cast<RefHandle*>(p);
    int n = h->system.getNumParticles();
    toVec(F, n, h->F); toVec(V, n, h->V); toVec(R, n, h->R);
    h->bodies.integratePart2(dt, h->R, h->F, h->V);
    fromVec(h->V, V);
}

void refrb_kinetic(void* p, const double* V, double* out2) {
    RefHandle* h = static_cast<RefHandle*>(p);
    std::vector<Vec3> v;
    toVec(V, h->system.getNumParticles(), v);
    h->bodies.computeKineticEnergies(v);
    out2[0] = h->bodies.getTranslationalEnergy();
    out2[1] = h->bodies.getRotationalEnergy();
}

int refrb_num_dof(void* p) { return static_cast<RefHandle*>(p)->bodies.getNumDOF(); }
int refrb_num_bodies(void* p) { return static_cast<RefHandle*>(p)->bodies.getNumBodies(); }
int refrb_num_free(void* p) { return static_cast<RefHandle*>(p)->bodies.getNumFree(); }
int refrb_num_body_atoms(void* p) { return static_cast<RefHandle*>(p)->bodies.getNumBodyAtoms(); }
int refrb_atom_index(void* p, int i) { return static_cast<RefHandle*>(p)->bodies.getAtomIndex(i); }

// Body record: N, dof, loc, mass, I[3], invI[3], rcm[3], pcm[3], q[4], pi[4], force[3], torque[4],
// twoKt, twoKr  (36 doubles).
void refrb_get_body(void* p, int i, double* out) {
    RigidBody b = static_cast<RefHandle*>(p)->bodies.getRigidBody(i);
    int k = 0;
    out[k++] = b.N; out[k++] = b.dof; out[k++] = b.loc; out[k++] = b.mass;
    for (int j = 0; j < 3; j++) out[k++] = b.I[j];
    for (int j = 0; j < 3; j++) out[k++] = b.invI[j];
    for (int j = 0; j < 3; j++) out[k++] = b.rcm[j];
    for (int j = 0; j < 3; j++) out[k++] = b.pcm[j];
    for (int j = 0; j < 4; j++) out[k++] = b.q[j];
    for (int j = 0; j < 4; j++) out[k++] = b.pi[j];
    for (int j = 0; j < 3; j++) out[k++] = b.force[j];
    for (int j = 0; j < 4; j++) out[k++] = b.torque[j];
    out[k++] = b.twoKt; out[k++] = b.twoKr;
}

void refrb_get_body_fixed(void* p, double* out) {
    RefHandle* h = static_cast<RefHandle*>(p);
    int n = h->bodies.getNumBodyAtoms();
    for (int i = 0; i < n; i++) {
        Vec3 x = h->bodies.getBodyFixedPosition(i);
        out[3 * i] = x[0]; out[3 * i + 1] = x[1]; out[3 * i + 2] = x[2];
    }
}

}  // extern "C"
