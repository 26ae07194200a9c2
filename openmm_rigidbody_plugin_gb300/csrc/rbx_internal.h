// rbx_internal.h -- device-side system description shared by the host code (rbx_host.cpp) and
// the CUDA kernels (rbx_kernels.cu).
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
#pragma once

#include <cstdint>

namespace rbx {

enum Precision : int { PREC_SINGLE = 0, PREC_MIXED = 1, PREC_DOUBLE = 2 };
enum StepKind : int { STEP_PART1 = 0, STEP_PART2 = 1, STEP_FUSED = 2 };

// Double precision: one 256-thread CTA per tile of at most 256 bodies / 512 body atoms.
constexpr int kThreads = 256;
constexpr int kTileBodies = 256;
constexpr int kTileAtomsD = 512;
// Single/mixed precision: one 256-thread CTA per tile of at most 256 bodies / 1024 body atoms.
constexpr int kThreadsF = 256;
constexpr int kTileBodiesF = 256;
constexpr int kTileAtomsF = 1024;
constexpr int kBconstRows = 11;     // rows of the FP32 body-constant table (single/mixed)

inline int tile_atoms(int prec) { return prec == PREC_DOUBLE ? kTileAtomsD : kTileAtomsF; }
inline int tile_bodies(int prec) { return prec == PREC_DOUBLE ? kTileBodies : kTileBodiesF; }
// Free atoms per free-atom tile: one per thread of the precision's step kernel.
inline int free_per_tile(int prec) { return prec == PREC_DOUBLE ? kThreads : kThreadsF; }

struct DevSys {
    int nb, nf, nba, nb_pad, nba_pad;
    int n_body_tiles, n_free_tiles;
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
};

struct DevBuf {
    void* posq;
    void* corr;
    void* velm;
    const long long* force;
    int stride;
};

struct KEScratch {
    double* partial;      // 2 * n_blocks
    unsigned int* count;  // 1
    double* out;          // 2
};

// Launchers (rbx_kernels.cu). Return the number of kernels enqueued, or -1 on a launch error.
int launch_step(int prec, int kind, const DevSys& s, const DevBuf& b, double dt, void* stream);
int launch_kinetic(int prec, const DevSys& s, const DevBuf& b, const KEScratch& k, int n_blocks, void* stream);
int launch_forces_from_host(int prec, const double* f_dev_user, const int* location, int natoms, long long* force,
                            int stride, void* stream);
int launch_load_positions(int prec, const double* x_dev_user, const double* v_dev_user, const double* masses,
                          const int* location, int natoms, const DevBuf& b, void* stream);
int launch_store_positions(int prec, const DevBuf& b, const int* location, int natoms, double* x_dev_user,
                           double* v_dev_user, void* stream);
int kinetic_blocks(const DevSys& s);
size_t step_smem_bytes(int prec);

// Record an error message for rbx_last_error() and return `code` (defined in rbx_host.cpp).
int set_error(int code, const char* fmt, ...);

}  // namespace rbx
