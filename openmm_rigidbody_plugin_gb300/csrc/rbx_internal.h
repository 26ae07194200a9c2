// rbx_internal.h -- device-side system description shared by the host code (rbx_host.cpp,
// rbx_batch.cpp) and the CUDA kernels (rbx_step.cuh, rbx_kernels.cu, rbx_refined.cu, rbx_forces.cu,
// rbx_setup.cu).
//
// HBM layout (one integrator):
//   body state   14 components r.xyz, v.xyz, q.wxyz, pi.wxyz per body (112 B/body):
//                  double precision: FP64 SoA, 14 rows of nb_pad
//                  single/mixed:     float-float SoA, 14 rows of hi parts then 14 rows of lo
//   constants    double: invm [nb] + invI FP64 SoA 3 x nb_pad                   (32 B/body)
//                single/mixed: FP32 SoA 11 x nb_pad: invm, invI.xyz, I0-I1, I1-I2, I0-I2, then
//                the low parts of invm and invI.xyz (float-float)                  (44 B/body)
//   atom0        int [nb+1]: first body atom of each body (library order)       (4 B/body)
//   cls          uint8 [nb]: rotation class (rbx::RotClass)                      (1 B/body)
//   d            body-frame atom positions, SoA 3 x nba_pad, float (single/mixed) or double
//   atom_loc     int [nba]: device slot of each body atom (library order)
//   free_loc     int [nf]:  device slot of each free atom
//   tile_body0   int [n_body_tiles+1]: bodies of tile t are [tile_body0[t], tile_body0[t+1])
//   ref_start    refined energies only: what part1 and fused steps record for part2 to close
//                the stencils. Bodies: kRefBodyRows rows of nb_pad: F h/m [3], then, single/mixed,
//                q(t+h) - q(t) [4] and the body angular momentum L(t-h/2) of the backward virtual
//                rotation [3], or, double, the quaternion stencil 0.5 [q(t-h) - q(t)] + 2.5
//                [q(t+h) - q(t)] [4]; then free atoms: 3 rows of nf_pad (F h/m). float (single,
//                mixed) or double (double precision).
//   ref_out      refined energies only, float, written by part2. Bodies: 3 rows of nb_pad (KE_t
//                correction, KE_r correction, |F|^2/m + tau.I^-1.tau); then free atoms: 2 rows of
//                nf_pad (KE_t correction, |F|^2/m).
#pragma once

#include <vector_types.h>

#include <cstddef>
#include <cstdint>
#include <vector>

struct rbx_integrator;  // include/rbx.h

namespace rbx {

enum Precision : int { PREC_SINGLE = 0, PREC_MIXED = 1, PREC_DOUBLE = 2 };
enum StepKind : int { STEP_PART1 = 0, STEP_PART2 = 1, STEP_FUSED = 2 };

// Double precision: one 256-thread CTA per tile of at most 256 bodies / 512 body atoms.
constexpr int kThreads = 256;
constexpr int kTileBodies = 256;
constexpr int kTileAtomsD = 512;
// Single/mixed precision: one CTA of NT threads per tile of at most NT bodies / 4 NT body atoms,
// 768 threads per SM: NT = 256 (3 CTAs per SM, the default) or 128 (6 per SM, bodies of at most
// kWarpBody atoms), chosen per integrator (rbx_set_tile_threads). Results do not depend on it.
constexpr int kThreadsF = 256;
constexpr int kThreadsFNarrow = 128;
constexpr int kTileAtomsF = 4 * kThreadsF;
constexpr int kWarpBody = 32;       // bodies of more atoms are summed by a whole warp
constexpr int kBconstRows = 11;     // rows of the FP32 body-constant table (single/mixed)
constexpr int kRefBodyRows = 10;    // rows of ref_start per body

// Tile limits of a precision at a step-kernel block size (nt: single/mixed only).
inline int tile_atoms(int prec, int nt = kThreadsF) { return prec == PREC_DOUBLE ? kTileAtomsD : 4 * nt; }
inline int tile_bodies(int prec, int nt = kThreadsF) { return prec == PREC_DOUBLE ? kTileBodies : nt; }
// Free atoms per free-atom tile: one per thread of the step kernel.
inline int free_per_tile(int prec, int nt = kThreadsF) { return prec == PREC_DOUBLE ? kThreads : nt; }

struct DevSys {
    int nb, nf, nba, nb_pad, nba_pad, nf_pad;
    int n_body_tiles, n_free_tiles;
    int tile_threads;  // single/mixed: the step kernel's block size (kThreadsF or kThreadsFNarrow)
    int large;         // 1: a body has more than kWarpBody atoms (the step kernels' LARGE form)
    int rot_n;  // NO-SQUISH substeps; 0 = exact rotation
    void* state;           // double* (double precision) or float* (float-float, single/mixed)
    const double* invm;    // double precision only
    const double* invI;    // double precision only
    const float* bconst;   // single/mixed only: kBconstRows rows of nb_pad
    const int* atom0;
    const uint8_t* cls;
    const void* d;
    const int* atom_loc;
    const int* free_loc;
    const int* tile_body0;
    void* ref_start;  // null unless refined energies are on (then the step kernels fill it)
    float* ref_out;
    // Failure detector of the step kernels: a body (library order) or free atom whose new state
    // is not finite gets its flag byte set and status[0] incremented. Null: not monitored.
    unsigned int* status;
    uint8_t* body_bad;  // [nb_pad]
    uint8_t* free_bad;  // [nf_pad]
};

struct DevBuf {
    void* posq;
    void* corr;
    void* velm;
    const long long* force;
    int stride;
};

// Cutoff LJ + reaction-field force field over many independent cubic boxes (rbx_forces.cu).
// Interacting atoms (non-zero charge or LJ epsilon) are listed system by system and, within a
// system, body by body: the interacting atoms of one rigid body (or one free atom) form a group,
// a contiguous range of the list. Neighbour lists pair groups, not atoms: a rigid group's atoms stay
// within its radius of its centroid whatever it rotates, so only centroid motion ages a list.
// Cells (of groups, by centroid) of all systems are numbered consecutively.
struct FFSys {
    int a0, a1;   // device slots of the system's atoms
    int i0, i1;   // its interacting atoms, as a range of the interacting-atom list
    int g0, g1;   // its groups
    int c0, nc;   // first cell and cells per box edge of the list build (1: one cell, all pairs)
    float L, invL, rc2, krf, crf;
    float rl;          // cutoff + skin: groups are listed when their centroids lie within rl + both radii
    float half_skin2;  // (skin/2)^2: a centroid moved this far since the build invalidates the lists
    int pair_image;    // 1: cutoff + two radii may reach half the box; the force pass takes the
                       // minimum image per pair (else one shift per listed group)
};
struct FFDev {
    int S, n_int, n_groups, n_cells;
    const FFSys* sys;     // [S]
    const int* iatom;     // [n_int] device slot of each interacting atom
    const int* isys;      // [n_int] its system
    const float4* param;  // [n_int] sqrt(K) q, sigma/2, sqrt(epsilon), body id (int bits; 0 = free)
    const int* grp_k0;    // [n_groups] first interacting atom of each group
    const int* grp_n;     // [n_groups] its atoms
    const int2* grp_kn;   // [n_groups] (grp_k0, grp_n) together: one load per listed group
    const int* gsys;      // [n_groups] its system
    const int* kgrp;      // [n_int] group of each interacting atom
    float4* gcen;         // [n_groups] centroid (wrapped into the box) and radius, every evaluation
    float4* gref;         // [n_groups] centroid at the last build
    float4* gq;           // [n_groups] cell order: centroid and radius (list builds)
    int* cell_of;         // [n_groups]
    int* cell_count;      // [n_cells], zero between evaluations
    int* cell_start;      // [n_cells + 1] (entry c0 + nc^3 of each system ends it)
    int* cell_cursor;     // [n_cells]
    int* cell_list;       // [n_groups] group indices in cell order (of the last list build)
    float4* cpos;         // [n_int] x, y, z (wrapped into the box), sqrt(K) q (or the atom's type)
    double* e_group;      // [n_groups] half pair-energy sums of each group (energy evaluations)
    // Neighbour lists of groups, rebuilt per system when one of its centroids has moved more than
    // half the skin since the last build, and for every system at the last evaluation of every
    // step call and at the first evaluation after a state is set
    unsigned char* rebuild;  // [S] 1: rebuild this system's lists before the next force pass
    unsigned int* rebuilds;  // [S] list builds of each system so far (a statistic)
    unsigned int* nbr;       // entries: listed group - g0 of the system; entry e of group g at
                             // g*cap + e
    int* ncnt;               // [n_groups] entries per group
    int cap;                 // entries per group allocated
    // Atom types (ntypes > 0): the distinct (sqrt(K) q, sigma/2, sqrt(epsilon)) of the interacting
    // atoms; cpos .w then holds the atom's type (int bits) instead of its charge, so that the force
    // pass reads one 16-byte record per neighbour, and takes each pair's (K q_i q_j, C12, C6) from
    // a table of type pairs
    const float4* types;     // [ntypes * ntypes] the type-pair table
    const int* atype;        // [n_int] type of each interacting atom
    int ntypes;
    double* energy;       // [S] potential energy per system (kJ/mol)
    float fcap;           // > 0: each atom's force is scaled down to at most this magnitude
    unsigned int* sys_status;  // [S] bit 0: a force of the system is non-finite or beyond the
                               // fixed-point range (never during a capped relaxation); bit 1: a list
                               // outgrew its capacity
    int cell_threads;     // block size of the cell list-build kernel: 64, 128 (default) or 256
    // work lists of the list builds (set with the state): every cell of the multi-cell boxes with
    // its system, and every 64-group chunk (first group) of the single-cell boxes
    int n_mc, n_sc;
    const int* mc_cell;
    const int* mc_sys;
    const int* sc_sys;
    const int* sc_g0;
    // groups of the force passes (set at creation, put in spatial order with the state), by size:
    // at most 4, at most 8 and more than 8 interacting atoms (force_pass_of)
    int n_pass[3];
    const int* pass_groups[3];
};
// The force pass runs in three launches by group size: at most 4 interacting atoms (waters, free
// atoms), at most 8 (tetrahedral bodies) and more (rings, larger bodies, in chunks of 12).
constexpr int kForcePasses = 3;
inline int force_pass_of(int atoms) { return atoms <= 4 ? 0 : atoms <= 8 ? 1 : 2; }
// Interacting atoms of one system: the force pass streams (atom << 5 | lane) words.
constexpr int kMaxSystemAtoms = 1 << 26;
int launch_forces(const FFDev& D, int prec, const DevBuf& B, bool energy, void* stream);
// Fixed-point forces of slots [0, natoms) -> user-order doubles out[3*natoms] (kJ/mol/nm).
int launch_forces_to_user(const long long* force, int stride, int natoms, double* out, void* stream);

struct KEScratch {
    double* partial;      // 2 * n_blocks
    unsigned int* count;  // 1
    double* out;          // 2
};

// Launchers (rbx_kernels.cu). Return the number of kernels enqueued, or -1 on a launch error.
// launch_step runs the refined-energy variants of the step kernels when s.ref_start is set.
int launch_step(int prec, int kind, const DevSys& s, const DevBuf& b, double dt, void* stream);
// rbx_refined.cu: the refined-energy step kernels and the fixed-order FP64 sum of ref_out into
// out[3] = [sum of KE_t corrections, sum of KE_r corrections, sum of |F|^2/m + tau.I^-1.tau].
int launch_step_refined(int prec, int kind, const DevSys& s, const DevBuf& b, double dt, void* stream);
struct RefScratch {
    double* partial;      // 3 * n_blocks
    unsigned int* count;  // 1
    double* out;          // 3
};
int refined_blocks(const DevSys& s);
int launch_refined_sum(const DevSys& s, const RefScratch& k, int n_blocks, void* stream);
int launch_kinetic(int prec, const DevSys& s, const DevBuf& b, const KEScratch& k, int n_blocks, void* stream);
// Free atoms under constraints: the unconstrained displacement into OpenMM's posDelta, and the move
// by the corrected displacement (mid-step velocity = displacement / dt).
int launch_free_delta(int prec, const DevSys& s, const DevBuf& b, void* pos_delta, double dt, void* stream);
int launch_free_apply_delta(int prec, const DevSys& s, const DevBuf& b, const void* pos_delta, double dt, void* stream);
int launch_forces_from_host(int prec, const double* f_dev_user, const int* location, int natoms, long long* force,
                            int stride, void* stream);
int launch_load_positions(int prec, const double* x_dev_user, const double* v_dev_user, const double* masses,
                          const int* location, int natoms, const DevBuf& b, void* stream);
int launch_store_positions(int prec, const DevBuf& b, const int* location, int natoms, double* x_dev_user,
                           double* v_dev_user, void* stream);
int kinetic_blocks(const DevSys& s);

// Record an error message for rbx_last_error() and return `code` (defined in rbx_host.cpp).
int set_error(int code, const char* fmt, ...);

// Device-side body setup (rbx_setup.cu): principal moments I (3 rows of nb_pad), degrees of
// freedom per body, their sum (atomically added) and a status word (bit 0: non-finite state).
struct SetupOut {
    double* I;
    int* dof;
    int* ndof;
    unsigned int* status;
};
int launch_setup_bodies(int prec, const DevSys& s, const DevBuf& b, const double* bmass, const SetupOut& out,
                        void* stream);

// Re-planning the library order on the device (rbx_plan.cu). launch_plan_order checks that the
// new slots are distinct (status != 0 otherwise; non-negative slots below nslots are the caller's
// check) and sorts bodies by the lowest slot of their atoms and free atoms by slot.
struct PlanOrder {
    int nb, nf, natoms, nslots;  // nslots = largest slot + 1
    const int* ref_first;        // [nb+1] reference order
    const int* ref_atoms;        // [nba]
    const int* loc;              // [natoms] new slots
    const int* free_old;         // [nf] free atoms (user indices) in any order
    unsigned int* seen;          // scratch [(nslots + 31) / 32]
    int* status;                 // [1]
    int *mark_body, *mark_free;  // scratch [nslots] each
    int* scan;                   // scratch [nslots]
    int* aux;                    // scratch [scan_aux_len(max(nslots, nb + 1))]
    int* lib_body_new;           // [nb] out: library position -> reference body
    int* free_new;               // [nf] out: free atoms in slot order
};
// launch_plan_maps derives, for the new order, where every body, body atom and free atom comes
// from in the current arrays (idx_*), and the new first-atom, slot and inverse maps.
struct PlanMaps {
    int nb, nf;
    const int* ref_first;
    const int* ref_atoms;
    const int* loc;
    const int* lib_body_new;
    const int* lib_pos_old;      // [nb] reference body -> current library position
    const int* atom0_old;        // [nb+1]
    const int* free_new;
    const int* free_index_old;   // [natoms] free atom (user index) -> current free position
    int* lib_pos_new;            // [nb]
    int* atom0_new;              // [nb+1]
    int* idx_body;               // [nb]  new library position -> current library position
    int* idx_atom;               // [nba] new body-atom index -> current body-atom index
    int* atom_loc_new;           // [nba]
    int* idx_free;               // [nf]  new free position -> current free position
    int* free_loc_new;           // [nf]
    int* free_index_new;         // [natoms]
    int* aux;                    // scan scratch
};
size_t scan_aux_len(int n);
int device_exclusive_scan(int* data, int n, int* aux, void* stream);
int launch_plan_order(const PlanOrder& P, void* stream);
int launch_plan_maps(const PlanMaps& M, void* stream);
// dst[r * ld + i] = src[r * ld + idx[i]] for rows r < rows, i < n; elements of 1, 4 or 8 bytes.
int launch_gather_rows(void* dst, const void* src, int rows, size_t ld, int n, const int* idx, int elem_bytes,
                       void* stream);

// Internal views of an integrator for the batched driver (defined in rbx_host.cpp).
DevSys device_system(const rbx_integrator* h);
// Device bytes the integrator holds (every allocation it made, as requested from cudaMalloc).
size_t device_bytes(const rbx_integrator* h);
// The failure detector's counter (synchronises `stream`) and, when it is non-zero, the flag bytes of
// every body (library order, [nb]) and free atom (library order, [nf]); all zero otherwise.
int failure_flags(rbx_integrator* h, void* stream, std::vector<uint8_t>& body_bad, std::vector<uint8_t>& free_bad,
                  unsigned int* count);
// Host copies of the body geometry, fetched from the device after a device-side setup (all of
// it, or only the degrees of freedom per body).
int ensure_host_geometry(rbx_integrator* h);
int sync_host_dof(rbx_integrator* h);
// For systems whose atoms occupy consecutive device-slot ranges [slot_offsets[s],
// slot_offsets[s+1]): the library-order ranges of their bodies (body0[S+1]) and free atoms
// (free0[S+1]), and their degrees of freedom (dof[S]).
int system_ranges(rbx_integrator* h, const std::vector<int>& slot_offsets, std::vector<int>& body0,
                  std::vector<int>& free0, std::vector<int>& dof);
// Body-atom positions rebuilt from the stored body state (the step kernels' arithmetic).
int launch_sync_positions(int prec, const DevSys& s, const DevBuf& b, void* stream);
// Scale the body COM velocities and quaternion momenta and the free atoms' velocities.
int launch_scale_momenta(int prec, const DevSys& s, const DevBuf& b, double factor, void* stream);
// [KE_t, KE_r] of each system (out[2*S]), FP64, fixed order, one block per system.
int launch_kinetic_systems(int prec, const DevSys& s, const DevBuf& b, const int* body0, const int* free0,
                           int num_systems, double* out, void* stream);

}  // namespace rbx
