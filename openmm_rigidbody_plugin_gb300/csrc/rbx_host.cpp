// rbx_host.cpp -- host side of librbx: the C ABI declared in include/rbx.h.
//
// Holds the rigid-body system description (the role of RigidBodySystem,
// openmmapi/src/RigidBodySystem.cpp), builds body geometry and momenta from atom positions and
// velocities (RigidBody::buildGeometry/buildDynamics, openmmapi/src/RigidBody.cpp:65-142) with a
// robust eigensolver, plans the tiles of the step kernels and owns every device allocation.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/rbx.h"
#include "rbx_devarray.h"
#include "rbx_internal.h"
#include "rbx_math.cuh"
#include "rbx_setup.cuh"

using namespace rbx;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CUDA_TRY(call)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(RBX_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

int rbx::set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

struct rbx_integrator {
    int natoms = 0, nb = 0, nf = 0, nba = 0, ndof = 0, mode = 0, prec = PREC_MIXED, device = 0;
    int max_location = 0;  // largest device slot in use; every buffer stride must exceed it
    int ncons = 0;         // constraints between free atoms (each removes one degree of freedom)
    int nb_pad = 0, nba_pad = 0, nf_pad = 0, n_body_tiles = 0, n_free_tiles = 0;
    int tile_threads = kThreadsF;  // single/mixed step-kernel block size (rbx_set_tile_threads)
    int max_body_atoms = 0;
    bool have_state = false;
    int last_launches = 0;
    std::vector<double> masses;
    std::vector<int> location;          // user atom -> device slot
    std::vector<int> free_atoms;        // user index of each free atom, in device-slot order
    // Bodies in the reference's order (ascending body index, RigidBodySystem.cpp:28-49); every
    // host copy of per-body data is kept in this order.
    std::vector<int> ref_first;         // [nb+1] first body atom of each body
    std::vector<int> ref_atoms;         // [nba] user index of each body atom
    std::vector<double> I;              // [nb*3] principal moments
    std::vector<double> dfix;           // [nba*3] body-frame positions, ref_atoms order
    std::vector<double> invm, invI;     // [nb], [nb*3]
    std::vector<uint8_t> cls;           // [nb]
    std::vector<int> dof;               // [nb]
    // Atoms whose body index is used once: free atoms here, one-atom bodies in the reference
    // (RigidBodySystem.cpp:37-47), which counts 5 or 6 degrees of freedom for each; single_dof is
    // that count at the last state upload (rbx_get_num_dof_reference).
    std::vector<int> singletons;
    int single_dof = 0;
    DevArray<int> d_single_loc;
    DevArray<double> d_single_x;
    // Library order, the order of every device array: bodies by the lowest device slot of their
    // atoms, so that a tile's atoms occupy a narrow slot range. Re-planned when slots change.
    std::vector<int> lib_body;          // [nb] library position -> reference body
    std::vector<int> lib_pos;           // [nb] reference body -> library position
    std::vector<int> body_first;        // [nb+1] first body atom (library order)
    std::vector<int> body_atoms;        // [nba] user index of each body atom (library order)
    std::vector<int> tile_body0;        // [n_body_tiles+1]
    // After a re-plan on the device only lib_body and tile_body0 are current on the host; location,
    // free_atoms, lib_pos, body_first and body_atoms are rebuilt on demand (ensure_host_plan).
    bool host_plan_valid = true;
    // device copies of the plan: reference-order body atoms (fixed) and the current inverse maps
    DevArray<int> d_ref_first, d_ref_atoms, d_lib_pos, d_free_atoms, d_free_index;
    // scratch of the device re-plan (allocated at its first use)
    DevArray<int> r_loc, r_marks, r_scan, r_aux, r_status, r_lib_body, r_free, r_idx;
    DevArray<unsigned int> r_seen;
    int r_nslots = 0;

    DevArray<double> d_state, d_invm, d_invI;  // d_state holds FP64 rows or float-float rows
    DevArray<float> d_bconst;                   // single/mixed: 11 rows (see kBconstRows)
    DevArray<int> d_atom0, d_atom_loc, d_free_loc, d_tiles;
    DevArray<double> d_bmass, d_I;  // body-atom masses (library order); moments of the device setup
    DevArray<int> d_dof, d_setup_counts;
    bool host_geom_valid = true;    // host copies of the geometry match the device (false after a device setup)
    DevArray<uint8_t> d_cls;
    // failure detector of the step kernels (DevSys::status): counter and flag bytes
    DevArray<unsigned int> d_status;
    DevArray<uint8_t> d_body_bad, d_free_bad;
    DevArray<unsigned char> d_fixed;  // float or double SoA
    DevArray<double> d_ke_partial, d_ke_out;
    DevArray<unsigned int> d_ke_count;
    double* h_ke = nullptr;  // pinned [8]: kinetic energies [0, 2), refined sums [2, 5)

    // refined energies (rbx_set_compute_refined_energies): stencil sums and per-unit terms
    bool refined = false;
    int ref_phase = 0;  // 0: no stencil, 1: started by part1 or a fused step, 2: closed by part2
    double ref_dt = 0.0;
    DevArray<unsigned char> d_ref_start;
    DevArray<float> d_ref_out;
    DevArray<double> d_ref_partial, d_ref_res;
    DevArray<unsigned int> d_ref_count;

    // owned OpenMM-layout context (host-buffer API)
    int stride = 0;
    DevArray<unsigned char> c_posq, c_corr, c_velm;
    DevArray<long long> c_force;
    DevArray<double> c_x, c_v, c_f, c_m;
    // pipelined host-buffer steps: double-buffered staging, copy streams and their events
    DevArray<double> p_f[2], p_x[2], p_v[2];
    cudaStream_t p_in = nullptr, p_out = nullptr;
    cudaEvent_t p_in_done[2] = {nullptr, nullptr}, p_compute_done[2] = {nullptr, nullptr};
    cudaEvent_t p_out_done[2] = {nullptr, nullptr};
    long p_calls = 0;
    DevArray<int> c_loc;

    DevSys sys() const {
        DevSys s;
        s.nb = nb; s.nf = nf; s.nba = nba; s.nb_pad = nb_pad; s.nba_pad = nba_pad; s.nf_pad = nf_pad;
        s.n_body_tiles = n_body_tiles; s.n_free_tiles = n_free_tiles; s.rot_n = mode;
        s.tile_threads = tile_threads;
        s.large = max_body_atoms > kWarpBody ? 1 : 0;
        s.state = d_state.p; s.invm = d_invm.p; s.invI = d_invI.p; s.bconst = d_bconst.p;
        s.atom0 = d_atom0.p; s.cls = d_cls.p;
        s.d = d_fixed.p; s.atom_loc = d_atom_loc.p; s.free_loc = d_free_loc.p; s.tile_body0 = d_tiles.p;
        s.ref_start = refined ? (void*)d_ref_start.p : nullptr;
        s.ref_out = refined ? d_ref_out.p : nullptr;
        s.status = d_status.p; s.body_bad = d_body_bad.p; s.free_bad = d_free_bad.p;
        return s;
    }
    ~rbx_integrator() {
        if (h_ke) cudaFreeHost(h_ke);
        for (int s = 0; s < 2; s++) {
            if (p_in_done[s]) cudaEventDestroy(p_in_done[s]);
            if (p_compute_done[s]) cudaEventDestroy(p_compute_done[s]);
            if (p_out_done[s]) cudaEventDestroy(p_out_done[s]);
        }
        if (p_in) cudaStreamDestroy(p_in);
        if (p_out) cudaStreamDestroy(p_out);
    }
};

rbx::DevSys rbx::device_system(const rbx_integrator* h) { return h->sys(); }

size_t rbx::device_bytes(const rbx_integrator* h) {
    size_t n = h->d_single_loc.bytes() + h->d_single_x.bytes() + h->d_ref_first.bytes() + h->d_ref_atoms.bytes() +
               h->d_lib_pos.bytes() + h->d_free_atoms.bytes() + h->d_free_index.bytes() + h->r_loc.bytes() +
               h->r_marks.bytes() + h->r_scan.bytes() + h->r_aux.bytes() + h->r_status.bytes() + h->r_lib_body.bytes() +
               h->r_free.bytes() + h->r_idx.bytes() + h->r_seen.bytes() + h->d_state.bytes() + h->d_invm.bytes() +
               h->d_invI.bytes() + h->d_bconst.bytes() + h->d_atom0.bytes() + h->d_atom_loc.bytes() +
               h->d_free_loc.bytes() + h->d_tiles.bytes() + h->d_bmass.bytes() + h->d_I.bytes() + h->d_dof.bytes() +
               h->d_setup_counts.bytes() + h->d_cls.bytes() + h->d_status.bytes() + h->d_body_bad.bytes() +
               h->d_free_bad.bytes() + h->d_fixed.bytes() + h->d_ke_partial.bytes() + h->d_ke_out.bytes() +
               h->d_ke_count.bytes() + h->d_ref_start.bytes() + h->d_ref_out.bytes() + h->d_ref_partial.bytes() +
               h->d_ref_res.bytes() + h->d_ref_count.bytes() + h->c_posq.bytes() + h->c_corr.bytes() +
               h->c_velm.bytes() + h->c_force.bytes() + h->c_x.bytes() + h->c_v.bytes() + h->c_f.bytes() +
               h->c_m.bytes() + h->c_loc.bytes();
    for (int s = 0; s < 2; s++) n += h->p_f[s].bytes() + h->p_x[s].bytes() + h->p_v[s].bytes();
    return n;
}

int rbx::failure_flags(rbx_integrator* h, void* stream, std::vector<uint8_t>& body_bad, std::vector<uint8_t>& free_bad,
                       unsigned int* count) {
    CUDA_TRY(cudaSetDevice(h->device));
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(h->h_ke + 7, h->d_status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    unsigned int c = 0;
    std::memcpy(&c, h->h_ke + 7, sizeof c);
    *count = c;
    body_bad.assign(h->nb, 0);
    free_bad.assign(h->nf, 0);
    if (!c) return RBX_OK;
    if (h->nb) CUDA_TRY(cudaMemcpy(body_bad.data(), h->d_body_bad.p, h->nb, cudaMemcpyDeviceToHost));
    if (h->nf) CUDA_TRY(cudaMemcpy(free_bad.data(), h->d_free_bad.p, h->nf, cudaMemcpyDeviceToHost));
    return RBX_OK;
}

namespace {
// Host copies of the plan after a re-plan on the device: slots and free-atom order from the device,
// the body order's inverse and atom lists rebuilt from lib_body.
int ensure_host_plan(rbx_integrator* h) {
    if (h->host_plan_valid) return RBX_OK;
    CUDA_TRY(cudaSetDevice(h->device));
    CUDA_TRY(cudaMemcpy(h->location.data(), h->c_loc.p, sizeof(int) * (size_t)h->natoms, cudaMemcpyDeviceToHost));
    if (h->nf)
        CUDA_TRY(cudaMemcpy(h->free_atoms.data(), h->d_free_atoms.p, sizeof(int) * (size_t)h->nf, cudaMemcpyDeviceToHost));
    h->lib_pos.resize(h->nb);
    h->body_first.assign(1, 0);
    h->body_atoms.clear();
    h->body_atoms.reserve(h->nba);
    for (int L = 0; L < h->nb; L++) {
        const int b = h->lib_body[L];
        h->lib_pos[b] = L;
        for (int a = h->ref_first[b]; a < h->ref_first[b + 1]; a++) h->body_atoms.push_back(h->ref_atoms[a]);
        h->body_first.push_back((int)h->body_atoms.size());
    }
    h->host_plan_valid = true;
    return RBX_OK;
}
}  // namespace

int rbx::sync_host_dof(rbx_integrator* h) {
    if (h->host_geom_valid || !h->have_state || h->nb == 0) return RBX_OK;
    std::vector<int> dof(h->nb);
    CUDA_TRY(cudaMemcpy(dof.data(), h->d_dof.p, dof.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int L = 0; L < h->nb; L++) h->dof[h->lib_body[L]] = dof[L];
    return RBX_OK;
}

int rbx::ensure_host_geometry(rbx_integrator* h) {
    if (h->host_geom_valid || !h->have_state) return RBX_OK;
    if (int rc = ensure_host_plan(h)) return rc;
    const int nb = h->nb, nbp = h->nb_pad, nbap = h->nba_pad;
    std::vector<double> I((size_t)3 * nbp);
    std::vector<int> dof(std::max(nb, 1));
    std::vector<uint8_t> cls(std::max(nb, 1));
    CUDA_TRY(cudaMemcpy(I.data(), h->d_I.p, I.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(dof.data(), h->d_dof.p, dof.size() * sizeof(int), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(cls.data(), h->d_cls.p, cls.size(), cudaMemcpyDeviceToHost));
    std::vector<double> invm(std::max(nb, 1)), invI((size_t)3 * nbp), d((size_t)3 * nbap);
    if (h->prec == PREC_DOUBLE) {
        CUDA_TRY(cudaMemcpy(invm.data(), h->d_invm.p, invm.size() * sizeof(double), cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(invI.data(), h->d_invI.p, invI.size() * sizeof(double), cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(d.data(), h->d_fixed.p, d.size() * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> bc((size_t)kBconstRows * nbp), df((size_t)3 * nbap);
        CUDA_TRY(cudaMemcpy(bc.data(), h->d_bconst.p, bc.size() * sizeof(float), cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(df.data(), h->d_fixed.p, df.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int L = 0; L < nb; L++) {
            invm[L] = (double)bc[L] + (double)bc[L + (size_t)7 * nbp];
            for (int k = 0; k < 3; k++)
                invI[L + (size_t)k * nbp] = (double)bc[L + (size_t)(1 + k) * nbp] + (double)bc[L + (size_t)(8 + k) * nbp];
        }
        for (size_t i = 0; i < df.size(); i++) d[i] = df[i];
    }
    for (int L = 0; L < nb; L++) {
        const int b = h->lib_body[L];
        for (int k = 0; k < 3; k++) {
            h->I[3 * b + k] = I[L + (size_t)k * nbp];
            h->invI[3 * b + k] = invI[L + (size_t)k * nbp];
        }
        h->invm[b] = invm[L];
        h->cls[b] = cls[L];
        h->dof[b] = dof[L];
        for (int j = 0; j < h->ref_first[b + 1] - h->ref_first[b]; j++)
            for (int c = 0; c < 3; c++)
                h->dfix[3 * (size_t)(h->ref_first[b] + j) + c] = d[h->body_first[L] + j + (size_t)c * nbap];
    }
    h->host_geom_valid = true;
    return RBX_OK;
}

int rbx::system_ranges(rbx_integrator* h, const std::vector<int>& slot_offsets, std::vector<int>& body0,
                        std::vector<int>& free0, std::vector<int>& dof) {
    if (int rc = ensure_host_plan(h)) return rc;
    const int S = (int)slot_offsets.size() - 1;
    body0.assign(S + 1, h->nb);
    free0.assign(S + 1, h->nf);
    dof.assign(S, 0);
    // library order: bodies by their lowest slot, free atoms by slot (both ascending)
    int s = 0;
    for (int L = 0; L < h->nb; L++) {
        int lo = INT32_MAX;
        for (int k = h->body_first[L]; k < h->body_first[L + 1]; k++) lo = std::min(lo, h->location[h->body_atoms[k]]);
        while (s < S && lo >= slot_offsets[s + 1]) body0[++s] = L;
        if (s < S) dof[s] += h->dof[h->lib_body[L]];
    }
    for (int t = s + 1; t <= S; t++) body0[t] = h->nb;
    body0[0] = 0;
    s = 0;
    for (int j = 0; j < h->nf; j++) {
        const int slot = h->location[h->free_atoms[j]];
        while (s < S && slot >= slot_offsets[s + 1]) free0[++s] = j;
        if (s < S) dof[s] += 3;
    }
    for (int t = s + 1; t <= S; t++) free0[t] = h->nf;
    free0[0] = 0;
    return RBX_OK;
}

namespace {

// The atoms of one body in the user's host arrays (the accessor of build_body, rbx_setup.cuh).
struct HostAtoms {
    int n;
    const int* atoms;
    const double* masses;
    const double* R;
    const double* V;
    double* dfix;
    double mass(int j) const { return masses[atoms[j]]; }
    V3<double> pos(int j) const {
        const int i = atoms[j];
        return v3<double>(R[3 * i], R[3 * i + 1], R[3 * i + 2]);
    }
    V3<double> vel(int j) const {
        const int i = atoms[j];
        return v3<double>(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
    }
    void set_d(int j, V3<double> d) {
        dfix[3 * j] = d.x;
        dfix[3 * j + 1] = d.y;
        dfix[3 * j + 2] = d.z;
    }
};

template <class T> int upload(DevArray<T>& a, const std::vector<T>& h) {
    if (a.alloc(h.size()) != cudaSuccess) return fail(RBX_ERR_CUDA, "cudaMalloc of %zu bytes failed", h.size() * sizeof(T));
    if (!h.empty()) CUDA_TRY(cudaMemcpy(a.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return RBX_OK;
}

// Library order and tiles. Bodies are ordered by the lowest device slot of their atoms (stable,
// ties by body index) and free atoms by their slot, so that consecutive threads of a tile touch
// neighbouring slots of the force, position and velocity buffers. A tile is a run of
// consecutive bodies under the per-CTA body and atom limits (rbx_create has rejected any body
// larger than one tile).
// Greedy packing of the library order into tiles of at most TB bodies and TA body atoms.
void pack_tiles(rbx_integrator* h) {
    const int TA = tile_atoms(h->prec, h->tile_threads), TB = tile_bodies(h->prec, h->tile_threads), nb = h->nb;
    h->tile_body0.assign(1, 0);
    for (int L = 0; L < nb;) {
        int atoms = 0, cnt = 0;
        while (L < nb && cnt < TB) {
            const int b = h->lib_body[L];
            const int n = h->ref_first[b + 1] - h->ref_first[b];
            if (atoms + n > TA) break;
            atoms += n;
            cnt++;
            L++;
        }
        h->tile_body0.push_back(L);
    }
    h->n_body_tiles = (int)h->tile_body0.size() - 1;
    const int fpt = free_per_tile(h->prec, h->tile_threads);
    h->n_free_tiles = (h->nf + fpt - 1) / fpt;
}

void plan_order(rbx_integrator* h) {
    const int nb = h->nb;
    std::vector<int> key(nb);
    for (int b = 0; b < nb; b++) {
        int k = h->location[h->ref_atoms[h->ref_first[b]]];
        for (int a = h->ref_first[b] + 1; a < h->ref_first[b + 1]; a++) k = std::min(k, h->location[h->ref_atoms[a]]);
        key[b] = k;
    }
    h->lib_body.resize(nb);
    for (int b = 0; b < nb; b++) h->lib_body[b] = b;
    std::stable_sort(h->lib_body.begin(), h->lib_body.end(), [&](int a, int b) { return key[a] < key[b]; });
    h->lib_pos.resize(nb);
    h->body_first.assign(1, 0);
    h->body_atoms.clear();
    for (int L = 0; L < nb; L++) {
        const int b = h->lib_body[L];
        h->lib_pos[b] = L;
        for (int a = h->ref_first[b]; a < h->ref_first[b + 1]; a++) h->body_atoms.push_back(h->ref_atoms[a]);
        h->body_first.push_back((int)h->body_atoms.size());
    }
    std::stable_sort(h->free_atoms.begin(), h->free_atoms.end(),
                     [&](int a, int b) { return h->location[a] < h->location[b]; });
    pack_tiles(h);
}

// Device copies of the library order: first atom of each body, tiles and device slots, and the
// maps a re-plan on the device starts from.
int upload_layout(rbx_integrator* h) {
    if (int rc = ensure_host_plan(h)) return rc;
    std::vector<int> atom_loc(h->nba), free_loc(h->nf);
    for (int k = 0; k < h->nba; k++) atom_loc[k] = h->location[h->body_atoms[k]];
    for (int j = 0; j < h->nf; j++) free_loc[j] = h->location[h->free_atoms[j]];
    std::vector<double> bmass(h->nba);
    for (int k = 0; k < h->nba; k++) bmass[k] = h->masses[h->body_atoms[k]];
    int rc = upload(h->d_atom0, h->body_first);
    if (!rc) rc = upload(h->d_bmass, bmass);
    if (!rc) rc = upload(h->d_tiles, h->tile_body0);
    if (!rc) rc = upload(h->d_atom_loc, atom_loc);
    if (!rc) rc = upload(h->d_free_loc, free_loc);
    if (!rc) rc = upload(h->c_loc, h->location);
    if (!rc) rc = upload(h->d_ref_first, h->ref_first);
    if (!rc) rc = upload(h->d_ref_atoms, h->ref_atoms);
    if (!rc) rc = upload(h->d_lib_pos, h->lib_pos);
    if (!rc) rc = upload(h->d_free_atoms, h->free_atoms);
    std::vector<int> free_index(h->natoms, -1);
    for (int j = 0; j < h->nf; j++) free_index[h->free_atoms[j]] = j;
    if (!rc) rc = upload(h->d_free_index, free_index);
    return rc;
}

// Device copies of the body constants in the library order: 1/m and 1/I (FP64 for double;
// float-float for single and mixed, with the moment gaps formed in FP64 so that they keep their
// relative accuracy for nearly degenerate tops), rotation classes and body-frame positions.
int upload_bodies(rbx_integrator* h) {
    if (int rc = ensure_host_plan(h)) return rc;
    const int nb = h->nb, nbp = h->nb_pad, nbap = h->nba_pad;
    if (h->prec == PREC_DOUBLE) {
        std::vector<double> invm(std::max(nb, 1), 0.0), invI((size_t)3 * nbp, 0.0);
        for (int L = 0; L < nb; L++) {
            const int b = h->lib_body[L];
            invm[L] = h->invm[b];
            for (int k = 0; k < 3; k++) invI[L + (size_t)k * nbp] = h->invI[3 * b + k];
        }
        CUDA_TRY(cudaMemcpy(h->d_invm.p, invm.data(), invm.size() * sizeof(double), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_invI.p, invI.data(), invI.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> bconst((size_t)kBconstRows * nbp, 0.0f);
        for (int L = 0; L < nb; L++) {
            const int b = h->lib_body[L];
            const double* I = &h->I[3 * b];
            const double cst[7] = {h->invm[b], h->invI[3 * b], h->invI[3 * b + 1], h->invI[3 * b + 2],
                                   I[0] - I[1], I[1] - I[2], I[0] - I[2]};
            for (int k = 0; k < 7; k++) bconst[L + (size_t)k * nbp] = (float)cst[k];
            for (int k = 0; k < 4; k++) bconst[L + (size_t)(7 + k) * nbp] = (float)(cst[k] - (double)(float)cst[k]);
        }
        CUDA_TRY(cudaMemcpy(h->d_bconst.p, bconst.data(), bconst.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    std::vector<uint8_t> cls(std::max(nb, 1), 0);
    for (int L = 0; L < nb; L++) cls[L] = h->cls[h->lib_body[L]];
    CUDA_TRY(cudaMemcpy(h->d_cls.p, cls.data(), cls.size(), cudaMemcpyHostToDevice));
    std::vector<double> d((size_t)3 * nbap, 0.0);
    for (int L = 0; L < nb; L++) {
        const int b = h->lib_body[L];
        for (int j = 0; j < h->ref_first[b + 1] - h->ref_first[b]; j++)
            for (int c = 0; c < 3; c++) d[h->body_first[L] + j + (size_t)c * nbap] = h->dfix[3 * (size_t)(h->ref_first[b] + j) + c];
    }
    if (h->prec == PREC_DOUBLE) {
        CUDA_TRY(cudaMemcpy(h->d_fixed.p, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(d.begin(), d.end());
        CUDA_TRY(cudaMemcpy(h->d_fixed.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    return RBX_OK;
}

int check(const rbx_integrator* h) {
    if (!h) return fail(RBX_ERR_INVALID_ARGUMENT, "null integrator handle");
    return RBX_OK;
}

int check_ready(const rbx_integrator* h, const rbx_buffers* buf) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body state: call rbx_upload_state first");
    if (!buf || !buf->posq || !buf->velm || !buf->force) return fail(RBX_ERR_INVALID_ARGUMENT, "null device buffer");
    if (h->prec == PREC_MIXED && !buf->posq_correction)
        return fail(RBX_ERR_INVALID_ARGUMENT, "mixed precision needs posq_correction");
    if (buf->stride < h->natoms) return fail(RBX_ERR_INVALID_ARGUMENT, "stride %d < number of atoms %d", buf->stride, h->natoms);
    if (3LL * buf->stride > INT_MAX)  // force rows are indexed slot + 2 x stride in 32 bits
        return fail(RBX_ERR_UNSUPPORTED, "stride %d exceeds the 32-bit device indexing of this build", buf->stride);
    if (h->max_location >= buf->stride)
        return fail(RBX_ERR_INVALID_ARGUMENT, "device slot %d outside buffers of stride %d", h->max_location, buf->stride);
    return RBX_OK;
}

DevBuf devbuf(const rbx_buffers* b) {
    DevBuf d;
    d.posq = b->posq; d.corr = b->posq_correction; d.velm = b->velm; d.force = b->force; d.stride = b->stride;
    return d;
}

int run_step(rbx_integrator* h, int kind, void* stream, const rbx_buffers* buf, double dt) {
    int rc = check_ready(h, buf);
    if (rc) return rc;
    if (!(dt == dt) || dt == 0.0) return fail(RBX_ERR_INVALID_ARGUMENT, "step size must be finite and non-zero");
    CUDA_TRY(cudaSetDevice(h->device));
    int n = launch_step(h->prec, kind, h->sys(), devbuf(buf), dt, stream);
    if (n < 0) return fail(RBX_ERR_CUDA, "step kernel launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    h->last_launches = n;
    if (h->refined) {
        // part1 and fused steps start the refined-energy stencils; part2 closes them if the last
        // start used the same step size
        if (kind == STEP_PART2) h->ref_phase = h->ref_phase == 1 && h->ref_dt == dt ? 2 : 0;
        else h->ref_phase = 1;
        h->ref_dt = dt;
    }
    return RBX_OK;
}

// Re-plan the library order for new device slots, on the device (rbx_plan.cu): sort bodies by
// the lowest slot of their atoms and free atoms by slot, pack tiles on the host, then move every
// per-body, per-body-atom and per-free-atom array to the new order with raw gathers, so the state
// moves bit for bit. Host copies of the plan are rebuilt only on demand.
// Device allocations replaced during a re-plan, freed once the stream has finished with them.
struct Retired {
    cudaStream_t st = nullptr;
    std::vector<void*> ptrs;
    template <class A> void take(A& a) {
        if (a.p) ptrs.push_back(a.p);
        a.p = nullptr;
        a.n = 0;
    }
    ~Retired() {
        if (ptrs.empty()) return;
        cudaStreamSynchronize(st);
        for (void* p : ptrs) cudaFree(p);
    }
};

int replan_device(rbx_integrator* h, const int* location, int nslots) {
    const int n = h->natoms, nb = h->nb, nf = h->nf, nba = h->nba;
    cudaStream_t st = nullptr;
    Retired old;
    old.st = st;
    if (h->r_nslots < nslots) {
        const size_t aux = scan_aux_len(std::max(nslots, nb + 1));
        if (h->r_marks.alloc((size_t)2 * nslots) != cudaSuccess || h->r_scan.alloc(nslots) != cudaSuccess ||
            h->r_seen.alloc((size_t)(nslots + 31) / 32) != cudaSuccess || h->r_aux.alloc(aux) != cudaSuccess)
            return fail(RBX_ERR_CUDA, "cudaMalloc of the re-plan scratch failed");
        h->r_nslots = nslots;
    }
    if (!h->r_loc.p && (h->r_loc.alloc(n) != cudaSuccess || h->r_status.alloc(1) != cudaSuccess ||
                        h->r_lib_body.alloc(std::max(nb, 1)) != cudaSuccess ||
                        h->r_free.alloc(std::max(nf, 1)) != cudaSuccess ||
                        h->r_idx.alloc((size_t)nb + nba + nf + 1) != cudaSuccess))
        return fail(RBX_ERR_CUDA, "cudaMalloc of the re-plan scratch failed");
    CUDA_TRY(cudaMemcpyAsync(h->r_loc.p, location, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
    PlanOrder P;
    P.nb = nb; P.nf = nf; P.natoms = n; P.nslots = nslots;
    P.ref_first = h->d_ref_first.p; P.ref_atoms = h->d_ref_atoms.p; P.loc = h->r_loc.p; P.free_old = h->d_free_atoms.p;
    P.seen = h->r_seen.p; P.status = h->r_status.p; P.mark_body = h->r_marks.p; P.mark_free = h->r_marks.p + nslots;
    P.scan = h->r_scan.p; P.aux = h->r_aux.p; P.lib_body_new = h->r_lib_body.p; P.free_new = h->r_free.p;
    if (launch_plan_order(P, st)) return fail(RBX_ERR_CUDA, "re-plan kernels failed: %s", cudaGetErrorString(cudaGetLastError()));
    std::vector<int> lib_body(nb);
    int status = 0;
    if (nb) CUDA_TRY(cudaMemcpyAsync(lib_body.data(), h->r_lib_body.p, sizeof(int) * (size_t)nb, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&status, h->r_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (status) return fail(RBX_ERR_INVALID_ARGUMENT, "a device slot is assigned to two atoms");

    // new maps, then every array gathered into a fresh allocation and swapped in
    DevArray<int> lib_pos, atom0, atom_loc, free_loc, free_index;
    if (lib_pos.alloc(std::max(nb, 1)) != cudaSuccess || atom0.alloc(nb + 1) != cudaSuccess ||
        atom_loc.alloc(std::max(nba, 1)) != cudaSuccess || free_loc.alloc(std::max(nf, 1)) != cudaSuccess ||
        free_index.alloc(n) != cudaSuccess)
        return fail(RBX_ERR_CUDA, "cudaMalloc of the new plan failed");
    CUDA_TRY(cudaMemcpyAsync(free_index.p, h->d_free_index.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    int* idx_body = h->r_idx.p;
    int* idx_atom = idx_body + nb;
    int* idx_free = idx_atom + nba;
    PlanMaps M;
    M.nb = nb; M.nf = nf;
    M.ref_first = h->d_ref_first.p; M.ref_atoms = h->d_ref_atoms.p; M.loc = h->r_loc.p;
    M.lib_body_new = h->r_lib_body.p; M.lib_pos_old = h->d_lib_pos.p; M.atom0_old = h->d_atom0.p;
    M.free_new = h->r_free.p; M.free_index_old = h->d_free_index.p;
    M.lib_pos_new = lib_pos.p; M.atom0_new = atom0.p; M.idx_body = idx_body; M.idx_atom = idx_atom;
    M.atom_loc_new = atom_loc.p; M.idx_free = idx_free; M.free_loc_new = free_loc.p; M.free_index_new = free_index.p;
    M.aux = h->r_aux.p;
    if (launch_plan_maps(M, st)) return fail(RBX_ERR_CUDA, "re-plan map kernels failed: %s", cudaGetErrorString(cudaGetLastError()));

    const size_t nbp = h->nb_pad, nbap = h->nba_pad, nfp = h->nf_pad;
    const int es = h->prec == PREC_DOUBLE ? 8 : 4;
    // Every array is gathered into a new allocation first; the swaps are applied only when all
    // gathers are enqueued, so a failure leaves the integrator in its previous plan. The stream is
    // drained before any allocation touched by a gather is freed.
    std::vector<std::function<void()>> commit;
    struct Drain {
        cudaStream_t st;
        ~Drain() { cudaStreamSynchronize(st); }
    } drain{st};
    auto regather = [&](auto& arr, int rows, size_t ld, int count, const int* idx, int ebytes) -> int {
        if (!arr.p || count == 0) return RBX_OK;
        auto tmp = std::make_shared<std::remove_reference_t<decltype(arr)>>();
        if (tmp->alloc(arr.n) != cudaSuccess) return fail(RBX_ERR_CUDA, "cudaMalloc during the re-plan failed");
        if (launch_gather_rows(tmp->p, arr.p, rows, ld, count, idx, ebytes, st))
            return fail(RBX_ERR_CUDA, "re-plan gather failed: %s", cudaGetErrorString(cudaGetLastError()));
        commit.push_back([&arr, tmp, &old]() {
            arr.swap(*tmp);
            old.take(*tmp);
        });
        return RBX_OK;
    };
    int rc = regather(h->d_state, h->prec == PREC_DOUBLE ? 14 : 28, nbp, nb, idx_body, es);
    if (!rc && h->prec == PREC_DOUBLE) rc = regather(h->d_invm, 1, nbp, nb, idx_body, 8);
    if (!rc && h->prec == PREC_DOUBLE) rc = regather(h->d_invI, 3, nbp, nb, idx_body, 8);
    if (!rc && h->prec != PREC_DOUBLE) rc = regather(h->d_bconst, kBconstRows, nbp, nb, idx_body, 4);
    if (!rc) rc = regather(h->d_cls, 1, nbp, nb, idx_body, 1);
    if (!rc) rc = regather(h->d_I, 3, nbp, nb, idx_body, 8);
    if (!rc) rc = regather(h->d_dof, 1, nbp, nb, idx_body, 4);
    if (!rc) rc = regather(h->d_fixed, 3, nbap, nba, idx_atom, es);
    if (!rc) rc = regather(h->d_bmass, 1, nbap, nba, idx_atom, 8);
    if (!rc) rc = regather(h->d_body_bad, 1, nbp, nb, idx_body, 1);
    if (!rc) rc = regather(h->d_free_bad, 1, nfp, nf, idx_free, 1);
    if (!rc && h->d_ref_start.p) {
        // body rows then free-atom rows of one allocation each: gather both parts into a new one
        auto s2 = std::make_shared<DevArray<unsigned char>>();
        auto o2 = std::make_shared<DevArray<float>>();
        if (s2->alloc(h->d_ref_start.n) != cudaSuccess || o2->alloc(h->d_ref_out.n) != cudaSuccess)
            return fail(RBX_ERR_CUDA, "cudaMalloc during the re-plan failed");
        unsigned char* fs_old = h->d_ref_start.p + kRefBodyRows * nbp * es;
        unsigned char* fs_new = s2->p + kRefBodyRows * nbp * es;
        if (launch_gather_rows(s2->p, h->d_ref_start.p, kRefBodyRows, nbp, nb, idx_body, es, st) ||
            launch_gather_rows(fs_new, fs_old, 3, nfp, nf, idx_free, es, st) ||
            launch_gather_rows(o2->p, h->d_ref_out.p, 3, nbp, nb, idx_body, 4, st) ||
            launch_gather_rows(o2->p + 3 * nbp, h->d_ref_out.p + 3 * nbp, 2, nfp, nf, idx_free, 4, st))
            return fail(RBX_ERR_CUDA, "re-plan gather failed: %s", cudaGetErrorString(cudaGetLastError()));
        commit.push_back([h, s2, o2, &old]() {
            h->d_ref_start.swap(*s2);
            h->d_ref_out.swap(*o2);
            old.take(*s2);
            old.take(*o2);
        });
    }
    if (rc) return rc;
    for (auto& f : commit) f();
    // the plan itself
    h->lib_body.swap(lib_body);
    pack_tiles(h);
    CUDA_TRY(cudaStreamSynchronize(st));  // gathers done before the old arrays are freed below
    h->d_atom0.swap(atom0);
    h->d_atom_loc.swap(atom_loc);
    h->d_free_loc.swap(free_loc);
    h->d_lib_pos.swap(lib_pos);
    h->d_free_index.swap(free_index);
    h->d_free_atoms.swap(h->r_free);
    h->c_loc.swap(h->r_loc);
    if ((rc = upload(h->d_tiles, h->tile_body0))) return rc;
    h->max_location = nslots - 1;
    h->host_plan_valid = false;
    return RBX_OK;
}

}  // namespace

// Reset the failure detector (a new state replaces the flagged one). Asynchronous on `stream`.
static int clear_failures(rbx_integrator* h, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st));
    CUDA_TRY(cudaMemsetAsync(h->d_body_bad.p, 0, h->d_body_bad.n, st));
    CUDA_TRY(cudaMemsetAsync(h->d_free_bad.p, 0, h->d_free_bad.n, st));
    return RBX_OK;
}

// Degrees of freedom the reference gives a one-atom body at positions x (RigidBody.cpp:65-107):
// its centre of mass is (0 + x m) * (1/m) (Vec3 division multiplies by the reciprocal), and
// collinear() takes the displacement x - rcm as the axis. A zero displacement gives a NaN axis,
// the test fails and the body counts 6; a rounding residue passes it, and the body counts 5.
static int reference_singleton_dof(const double* x, double m) {
    const double r = 1.0 / m;
    bool zero = true;
    for (int k = 0; k < 3; k++) zero = zero && (x[k] - (0.0 + x[k] * m) * r == 0.0);
    return zero ? 6 : 5;
}

extern "C" {

const char* rbx_last_error(void) { return g_err.c_str(); }
int rbx_version(void) { return 100; }

int rbx_create(rbx_integrator** out, int num_atoms, const int* body_indices, const double* masses, int rotation_mode,
               int precision, int device) {
    if (!out) return fail(RBX_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (num_atoms <= 0 || !body_indices || !masses) return fail(RBX_ERR_INVALID_ARGUMENT, "need num_atoms > 0, body indices and masses");
    if (rotation_mode < 0) return fail(RBX_ERR_INVALID_ARGUMENT, "Rotation mode cannot be negative");
    if (precision < PREC_SINGLE || precision > PREC_DOUBLE) return fail(RBX_ERR_INVALID_ARGUMENT, "unknown precision %d", precision);
    rbx_integrator* h = new (std::nothrow) rbx_integrator();
    if (!h) return fail(RBX_ERR_INVALID_ARGUMENT, "out of host memory");
    h->natoms = num_atoms;
    h->mode = rotation_mode;
    h->prec = precision;
    h->device = device;
    h->masses.assign(masses, masses + num_atoms);
    h->location.resize(num_atoms);
    for (int i = 0; i < num_atoms; i++) h->location[i] = i;
    h->max_location = num_atoms - 1;

    // Compact positive ids in ascending order (cleanBodyIndices, RigidBodySystem.cpp:28-49);
    // an id used by one atom only makes that atom free.
    int maxid = 0;
    for (int i = 0; i < num_atoms; i++) maxid = std::max(maxid, body_indices[i]);
    std::vector<int> count((size_t)maxid + 1, 0);
    for (int i = 0; i < num_atoms; i++)
        if (body_indices[i] > 0) count[body_indices[i]]++;
    std::vector<int> compact((size_t)maxid + 1, -1);
    int nb = 0;
    for (int id = 1; id <= maxid; id++)
        if (count[id] > 1) compact[id] = nb++;
    std::vector<std::vector<int>> members(nb);
    for (int i = 0; i < num_atoms; i++) {
        int id = body_indices[i];
        bool in_body = id > 0 && compact[id] >= 0;
        if (!(masses[i] > 0.0)) {
            if (in_body) { delete h; return fail(RBX_ERR_INVALID_ARGUMENT, "atom %d of a rigid body has no mass", i); }
            if (masses[i] < 0.0) { delete h; return fail(RBX_ERR_INVALID_ARGUMENT, "atom %d has negative mass", i); }
            continue;  // massless free atoms are not integrated
        }
        if (in_body) members[compact[id]].push_back(i);
        else h->free_atoms.push_back(i);
        if (id > 0 && count[id] == 1) h->singletons.push_back(i);
    }
    h->nb = nb;
    h->nf = (int)h->free_atoms.size();
    h->ref_first.assign(1, 0);
    for (int b = 0; b < nb; b++) {
        if ((int)members[b].size() > tile_atoms(precision)) {
            delete h;
            return fail(RBX_ERR_UNSUPPORTED, "a rigid body of %d atoms exceeds the %d-atom tile of this build",
                        (int)members[b].size(), tile_atoms(precision));
        }
        for (int i : members[b]) h->ref_atoms.push_back(i);
        h->ref_first.push_back((int)h->ref_atoms.size());
        h->max_body_atoms = std::max(h->max_body_atoms, (int)members[b].size());
    }
    h->nba = (int)h->ref_atoms.size();
    plan_order(h);
    h->nb_pad = ((std::max(nb, 1) + 31) / 32) * 32;
    h->nba_pad = ((std::max(h->nba, 1) + 31) / 32) * 32;
    h->nf_pad = ((std::max(h->nf, 1) + 31) / 32) * 32;
    // Device indices are 32-bit: the largest are row 27 of the float-float body state
    // (28 x nb_pad) and row 2 of the body-frame coordinates and of the free-atom rows.
    if (28LL * h->nb_pad > INT_MAX || 3LL * h->nba_pad > INT_MAX || 3LL * h->nf_pad > INT_MAX) {
        const int nba = h->nba, nf = h->nf;
        delete h;
        return fail(RBX_ERR_UNSUPPORTED, "%d bodies, %d body atoms and %d free atoms exceed the 32-bit device indexing of this build",
                    nb, nba, nf);
    }
    h->I.assign((size_t)nb * 3, 0.0);
    h->dfix.assign((size_t)h->nba * 3, 0.0);
    h->invm.assign(nb, 0.0);
    h->invI.assign((size_t)nb * 3, 0.0);
    h->cls.assign(nb, 0);
    h->dof.assign(nb, 6);

    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete h; return fail(RBX_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e)); }
    int rc = upload_layout(h);
    if (!rc && h->d_state.alloc((size_t)14 * h->nb_pad) != cudaSuccess) rc = fail(RBX_ERR_CUDA, "cudaMalloc body state");
    if (precision == PREC_DOUBLE) {
        if (!rc && h->d_invm.alloc(std::max(nb, 1)) != cudaSuccess) rc = fail(RBX_ERR_CUDA, "cudaMalloc invm");
        if (!rc && h->d_invI.alloc((size_t)3 * h->nb_pad) != cudaSuccess) rc = fail(RBX_ERR_CUDA, "cudaMalloc invI");
    } else if (!rc && h->d_bconst.alloc((size_t)kBconstRows * h->nb_pad) != cudaSuccess) {
        rc = fail(RBX_ERR_CUDA, "cudaMalloc body constants");
    }
    if (!rc && h->d_cls.alloc(std::max(nb, 1)) != cudaSuccess) rc = fail(RBX_ERR_CUDA, "cudaMalloc cls");
    const size_t dsz = precision == PREC_DOUBLE ? sizeof(double) : sizeof(float);
    if (!rc && h->d_fixed.alloc((size_t)3 * h->nba_pad * dsz) != cudaSuccess) rc = fail(RBX_ERR_CUDA, "cudaMalloc body-frame positions");
    if (!rc) {
        DevSys s = h->sys();
        int kb = kinetic_blocks(s);
        if (h->d_ke_partial.alloc((size_t)2 * kb) != cudaSuccess || h->d_ke_out.alloc(2) != cudaSuccess ||
            h->d_ke_count.alloc(1) != cudaSuccess)
            rc = fail(RBX_ERR_CUDA, "cudaMalloc kinetic-energy scratch");
        else if (cudaMemset(h->d_ke_count.p, 0, sizeof(unsigned int)) != cudaSuccess ||
                 cudaMallocHost((void**)&h->h_ke, 8 * sizeof(double)) != cudaSuccess)
            rc = fail(RBX_ERR_CUDA, "kinetic-energy scratch initialisation failed");
    }
    if (!rc && h->d_state.p) rc = cudaMemset(h->d_state.p, 0, sizeof(double) * 14 * h->nb_pad) == cudaSuccess ? 0 : fail(RBX_ERR_CUDA, "cudaMemset");
    if (!rc && (h->d_status.alloc(1) != cudaSuccess || h->d_body_bad.alloc(h->nb_pad) != cudaSuccess ||
                h->d_free_bad.alloc(h->nf_pad) != cudaSuccess))
        rc = fail(RBX_ERR_CUDA, "cudaMalloc of the failure flags");
    if (!rc) rc = clear_failures(h, nullptr);
    if (rc) { delete h; return rc; }
    *out = h;
    return RBX_OK;
}

int rbx_destroy(rbx_integrator* h) {
    if (!h) return RBX_OK;
    cudaSetDevice(h->device);
    delete h;
    return RBX_OK;
}

int rbx_set_atom_locations(rbx_integrator* h, const int* location) {
    int rc = check(h);
    if (rc) return rc;
    if (!location) return fail(RBX_ERR_INVALID_ARGUMENT, "null location array");
    int lo = INT32_MAX, hi = -1;
    for (int i = 0; i < h->natoms; i++) {
        lo = std::min(lo, location[i]);
        hi = std::max(hi, location[i]);
    }
    if (lo < 0) {
        const int i = (int)(std::find_if(location, location + h->natoms, [](int s) { return s < 0; }) - location);
        return fail(RBX_ERR_INVALID_ARGUMENT, "negative location for atom %d", i);
    }
    CUDA_TRY(cudaSetDevice(h->device));
    return replan_device(h, location, hi + 1);
}

// Body state rows (14 per body, library order) -> device layout of the integrator's precision:
// FP64 rows for double, float-float rows (14 hi rows then 14 lo rows) for single and mixed.
static int put_state(rbx_integrator* h, const std::vector<double>& rows /* 14 x nb_pad */) {
    const size_t n = rows.size();
    if (h->prec == PREC_DOUBLE) {
        CUDA_TRY(cudaMemcpy(h->d_state.p, rows.data(), n * sizeof(double), cudaMemcpyHostToDevice));
        return RBX_OK;
    }
    std::vector<float> f(2 * n);
    for (size_t i = 0; i < n; i++) {
        float hi = (float)rows[i];
        f[i] = hi;
        f[n + i] = (float)(rows[i] - (double)hi);
    }
    CUDA_TRY(cudaMemcpy(h->d_state.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    return RBX_OK;
}

static int get_state(rbx_integrator* h, std::vector<double>& rows) {
    const size_t n = (size_t)14 * h->nb_pad;
    rows.assign(n, 0.0);
    if (h->prec == PREC_DOUBLE) {
        CUDA_TRY(cudaMemcpy(rows.data(), h->d_state.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        return RBX_OK;
    }
    std::vector<float> f(2 * n);
    CUDA_TRY(cudaMemcpy(f.data(), h->d_state.p, f.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) rows[i] = (double)f[i] + (double)f[n + i];
    return RBX_OK;
}

int rbx_upload_state(rbx_integrator* h, const double* positions, const double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if (!positions || !velocities) return fail(RBX_ERR_INVALID_ARGUMENT, "null positions or velocities");
    if ((rc = ensure_host_plan(h))) return rc;
    const int nb = h->nb, nbp = h->nb_pad;
    std::vector<double> state((size_t)14 * nbp, 0.0);
    int ndof = 3 * h->nf;  // three per free atom (RigidBodySystem.cpp:130 counts one: defect D8)
    for (int b = 0; b < nb; b++) {
        const int f = h->ref_first[b], N = h->ref_first[b + 1] - f;
        BodySetup s;
        HostAtoms at{N, &h->ref_atoms[f], h->masses.data(), positions, velocities, &h->dfix[3 * (size_t)f]};
        build_body(at, s);
        for (int k = 0; k < 3; k++) { h->I[3 * b + k] = s.I[k]; h->invI[3 * b + k] = s.invI[k]; }
        h->invm[b] = s.invm;
        h->cls[b] = s.cls;
        h->dof[b] = s.dof;
        ndof += s.dof;
        double row[14] = {s.r.x, s.r.y, s.r.z, s.v.x, s.v.y, s.v.z, s.q.w, s.q.x, s.q.y, s.q.z, s.pi.w, s.pi.x, s.pi.y, s.pi.z};
        for (int k = 0; k < 14; k++) {
            if (!std::isfinite(row[k])) return fail(RBX_ERR_NUMERIC, "non-finite rigid-body state for body %d", b);
            state[h->lib_pos[b] + (size_t)k * nbp] = row[k];
        }
    }
    h->ndof = ndof;
    if ((rc = clear_failures(h, nullptr))) return rc;
    h->single_dof = 0;
    for (int i : h->singletons) h->single_dof += reference_singleton_dof(positions + 3 * (size_t)i, h->masses[i]);
    CUDA_TRY(cudaSetDevice(h->device));
    if ((rc = put_state(h, state))) return rc;
    if ((rc = upload_bodies(h))) return rc;
    h->have_state = true;
    h->host_geom_valid = true;
    h->ref_phase = 0;
    return RBX_OK;
}

int rbx_upload_state_device(rbx_integrator* h, void* stream, const rbx_buffers* buf) {
    int rc = check(h);
    if (rc) return rc;
    if (!buf || !buf->posq || !buf->velm) return fail(RBX_ERR_INVALID_ARGUMENT, "null device buffer");
    if (h->prec == PREC_MIXED && !buf->posq_correction)
        return fail(RBX_ERR_INVALID_ARGUMENT, "mixed precision needs posq_correction");
    if (buf->stride < h->natoms || h->max_location >= buf->stride)
        return fail(RBX_ERR_INVALID_ARGUMENT, "device slots outside buffers of stride %d", buf->stride);
    if (3LL * buf->stride > INT_MAX)
        return fail(RBX_ERR_UNSUPPORTED, "stride %d exceeds the 32-bit device indexing of this build", buf->stride);
    CUDA_TRY(cudaSetDevice(h->device));
    if (!h->d_I.p && (h->d_I.alloc((size_t)3 * h->nb_pad) != cudaSuccess || h->d_dof.alloc(std::max(h->nb, 1)) != cudaSuccess ||
                      h->d_setup_counts.alloc(2) != cudaSuccess))
        return fail(RBX_ERR_CUDA, "cudaMalloc of setup arrays failed");
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = clear_failures(h, stream))) return rc;
    CUDA_TRY(cudaMemsetAsync(h->d_setup_counts.p, 0, 2 * sizeof(int), st));
    SetupOut o{h->d_I.p, h->d_dof.p, h->d_setup_counts.p, (unsigned int*)(h->d_setup_counts.p + 1)};
    if (launch_setup_bodies(h->prec, h->sys(), devbuf(buf), h->d_bmass.p, o, stream) < 0)
        return fail(RBX_ERR_CUDA, "body setup kernel failed: %s", cudaGetErrorString(cudaGetLastError()));
    int counts[2] = {0, 0};
    CUDA_TRY(cudaMemcpyAsync(counts, h->d_setup_counts.p, sizeof counts, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (counts[1]) return fail(RBX_ERR_NUMERIC, "non-finite rigid-body state from the device setup");
    int single_dof = 0;
    if (!h->singletons.empty()) {  // the positions of the one-atom bodies of the reference
        const int ns = (int)h->singletons.size();
        if ((rc = ensure_host_plan(h))) return rc;
        std::vector<int> loc(ns);
        for (int k = 0; k < ns; k++) loc[k] = h->location[h->singletons[k]];
        if (!h->d_single_loc.p && (h->d_single_loc.alloc(ns) != cudaSuccess || h->d_single_x.alloc((size_t)3 * ns) != cudaSuccess))
            return fail(RBX_ERR_CUDA, "cudaMalloc of the one-atom body arrays failed");
        CUDA_TRY(cudaMemcpyAsync(h->d_single_loc.p, loc.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
        if (launch_store_positions(h->prec, devbuf(buf), h->d_single_loc.p, ns, h->d_single_x.p, nullptr, stream) < 0)
            return fail(RBX_ERR_CUDA, "position gather failed: %s", cudaGetErrorString(cudaGetLastError()));
        std::vector<double> x((size_t)3 * ns);
        CUDA_TRY(cudaMemcpyAsync(x.data(), h->d_single_x.p, x.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        for (int k = 0; k < ns; k++) single_dof += reference_singleton_dof(&x[3 * (size_t)k], h->masses[h->singletons[k]]);
    }
    h->single_dof = single_dof;
    h->ndof = 3 * h->nf + counts[0];
    h->have_state = true;
    h->host_geom_valid = false;
    h->ref_phase = 0;
    h->last_launches = 1;
    return RBX_OK;
}

int rbx_get_num_dof(const rbx_integrator* h, int* out) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "degrees of freedom are known after rbx_upload_state");
    *out = h->ndof - h->ncons;  // numDOF = free - constraints + body dof (RigidBodySystem.cpp:130)
    return RBX_OK;
}

int rbx_set_tile_threads(rbx_integrator* h, int threads) {
    int rc = check(h);
    if (rc) return rc;
    if (threads != kThreadsF && threads != kThreadsFNarrow)
        return fail(RBX_ERR_INVALID_ARGUMENT, "tile threads must be %d or %d, not %d", kThreadsF, kThreadsFNarrow, threads);
    if (h->prec == PREC_DOUBLE && threads != kThreadsF)
        return fail(RBX_ERR_UNSUPPORTED, "double precision has one tile shape (%d threads)", kThreadsF);
    if (threads == kThreadsFNarrow && h->max_body_atoms > kWarpBody)
        return fail(RBX_ERR_UNSUPPORTED, "the %d-thread tile takes bodies of at most %d atoms, not %d", threads,
                    kWarpBody, h->max_body_atoms);
    if (threads == h->tile_threads) return RBX_OK;
    CUDA_TRY(cudaSetDevice(h->device));
    CUDA_TRY(cudaDeviceSynchronize());  // no step in flight reads the old tiles
    const int old = h->tile_threads;
    h->tile_threads = threads;
    pack_tiles(h);
    if ((rc = upload(h->d_tiles, h->tile_body0))) {
        h->tile_threads = old;
        pack_tiles(h);
        return rc;
    }
    return RBX_OK;
}

int rbx_get_tile_threads(const rbx_integrator* h, int* out) {
    int rc = check(h);
    if (rc) return rc;
    *out = h->prec == PREC_DOUBLE ? kThreads : h->tile_threads;
    return RBX_OK;
}

int rbx_check_state(rbx_integrator* h, void* stream, int* bad_bodies, int* bad_free) {
    int rc = check(h);
    if (rc) return rc;
    std::vector<uint8_t> bb, fb;
    unsigned int count = 0;
    if ((rc = rbx::failure_flags(h, stream, bb, fb, &count))) return rc;
    int nbad_b = 0, nbad_f = 0, first_b = -1, first_f = -1;
    if (count) {
        if ((rc = ensure_host_plan(h))) return rc;
        for (int L = 0; L < h->nb; L++)
            if (bb[L]) {
                nbad_b++;
                const int rb = h->lib_body[L];
                if (first_b < 0 || rb < first_b) first_b = rb;
            }
        for (int j = 0; j < h->nf; j++)
            if (fb[j]) {
                nbad_f++;
                const int a = h->free_atoms[j];
                if (first_f < 0 || a < first_f) first_f = a;
            }
    }
    if (bad_bodies) *bad_bodies = nbad_b;
    if (bad_free) *bad_free = nbad_f;
    if (!count) return RBX_OK;
    return fail(RBX_ERR_NUMERIC, "non-finite state after a step: %d bodies (first: body %d in ascending body-index "
                "order) and %d free atoms (first: atom %d)", nbad_b, first_b, nbad_f, first_f);
}

int rbx_get_num_dof_reference(const rbx_integrator* h, int* out) {
    int rc = check(h);
    if (rc) return rc;
    if (!out) return fail(RBX_ERR_INVALID_ARGUMENT, "null output pointer");
    if (!h->have_state) return fail(RBX_ERR_STATE, "degrees of freedom are known after rbx_upload_state");
    // numDOF = numFree - numConstraints + sum of body dof (RigidBodySystem.cpp:130): one per free
    // atom, and the atoms of unique indices as one-atom bodies
    const int nsingle = (int)h->singletons.size();
    const int body_dof = h->ndof - 3 * h->nf;
    *out = (h->nf - nsingle) - h->ncons + body_dof + h->single_dof;
    return RBX_OK;
}

int rbx_set_constraints(rbx_integrator* h, int num_constraints, const int* atom_pairs) {
    int rc = check(h);
    if (rc) return rc;
    if (num_constraints < 0 || (num_constraints > 0 && !atom_pairs))
        return fail(RBX_ERR_INVALID_ARGUMENT, "need a non-negative count and the atom pairs");
    std::vector<char> in_body(h->natoms, 0);
    for (int a : h->ref_atoms) in_body[a] = 1;
    for (int k = 0; k < 2 * num_constraints; k++) {
        const int a = atom_pairs[k];
        if (a < 0 || a >= h->natoms) return fail(RBX_ERR_INVALID_ARGUMENT, "constraint %d: atom %d out of range", k / 2, a);
        if (in_body[a]) return fail(RBX_ERR_INVALID_ARGUMENT, "Constraints involving rigid-body atoms are not allowed");
    }
    h->ncons = num_constraints;
    return RBX_OK;
}

int rbx_free_atoms_delta(rbx_integrator* h, void* stream, const rbx_buffers* buf, void* pos_delta, double dt) {
    int rc = check_ready(h, buf);
    if (rc) return rc;
    if (!pos_delta) return fail(RBX_ERR_INVALID_ARGUMENT, "null posDelta buffer");
    if (!(dt == dt) || dt == 0.0) return fail(RBX_ERR_INVALID_ARGUMENT, "step size must be finite and non-zero");
    CUDA_TRY(cudaSetDevice(h->device));
    const int n = launch_free_delta(h->prec, h->sys(), devbuf(buf), pos_delta, dt, stream);
    if (n < 0) return fail(RBX_ERR_CUDA, "free-atom delta kernel failed: %s", cudaGetErrorString(cudaGetLastError()));
    h->last_launches = n;
    return RBX_OK;
}

int rbx_integrate_part1_delta(rbx_integrator* h, void* stream, const rbx_buffers* buf, const void* pos_delta,
                              double dt) {
    int rc = check_ready(h, buf);
    if (rc) return rc;
    if (!pos_delta) return fail(RBX_ERR_INVALID_ARGUMENT, "null posDelta buffer");
    if (!(dt == dt) || dt == 0.0) return fail(RBX_ERR_INVALID_ARGUMENT, "step size must be finite and non-zero");
    if (h->refined)
        return fail(RBX_ERR_UNSUPPORTED, "refined energies are not available with constrained free atoms in this build");
    CUDA_TRY(cudaSetDevice(h->device));
    DevSys s = h->sys();
    s.n_free_tiles = 0;  // the step kernel moves the bodies only
    const int n1 = launch_step(h->prec, STEP_PART1, s, devbuf(buf), dt, stream);
    const int n2 = n1 < 0 ? -1 : launch_free_apply_delta(h->prec, h->sys(), devbuf(buf), pos_delta, dt, stream);
    if (n1 < 0 || n2 < 0) return fail(RBX_ERR_CUDA, "constrained part1 failed: %s", cudaGetErrorString(cudaGetLastError()));
    h->last_launches = n1 + n2;
    return RBX_OK;
}
int rbx_get_num_bodies(const rbx_integrator* h, int* out) { int rc = check(h); if (!rc) *out = h->nb; return rc; }
int rbx_get_num_free(const rbx_integrator* h, int* out) { int rc = check(h); if (!rc) *out = h->nf; return rc; }
int rbx_get_rotation_mode(const rbx_integrator* h, int* out) { int rc = check(h); if (!rc) *out = h->mode; return rc; }

int rbx_integrate_part1(rbx_integrator* h, void* stream, const rbx_buffers* buf, double dt) {
    return run_step(h, STEP_PART1, stream, buf, dt);
}
int rbx_integrate_part2(rbx_integrator* h, void* stream, const rbx_buffers* buf, double dt) {
    return run_step(h, STEP_PART2, stream, buf, dt);
}
int rbx_integrate_fused(rbx_integrator* h, void* stream, const rbx_buffers* buf, double dt) {
    return run_step(h, STEP_FUSED, stream, buf, dt);
}

int rbx_kinetic_energies(rbx_integrator* h, void* stream, const rbx_buffers* buf, double* out2) {
    int rc = check_ready(h, buf);
    if (rc) return rc;
    if (!out2) return fail(RBX_ERR_INVALID_ARGUMENT, "null output");
    CUDA_TRY(cudaSetDevice(h->device));
    DevSys s = h->sys();
    KEScratch k{h->d_ke_partial.p, h->d_ke_count.p, h->d_ke_out.p};
    if (launch_kinetic(h->prec, s, devbuf(buf), k, kinetic_blocks(s), stream) < 0)
        return fail(RBX_ERR_CUDA, "kinetic-energy launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    CUDA_TRY(cudaMemcpyAsync(h->h_ke, h->d_ke_out.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    out2[0] = h->h_ke[0];
    out2[1] = h->h_ke[1];
    h->last_launches = 1;
    return RBX_OK;
}

int rbx_set_compute_refined_energies(rbx_integrator* h, int compute) {
    int rc = check(h);
    if (rc) return rc;
    h->refined = compute != 0;
    h->ref_phase = 0;
    if (!h->refined || h->d_ref_start.p) return RBX_OK;
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t es = h->prec == PREC_DOUBLE ? sizeof(double) : sizeof(float);
    const size_t start = (kRefBodyRows * (size_t)h->nb_pad + 3 * (size_t)h->nf_pad) * es;
    const size_t terms = 3 * (size_t)h->nb_pad + 2 * (size_t)h->nf_pad;
    const int blocks = refined_blocks(h->sys());
    if (h->d_ref_start.alloc(start) != cudaSuccess || h->d_ref_out.alloc(terms) != cudaSuccess ||
        h->d_ref_partial.alloc((size_t)3 * blocks) != cudaSuccess || h->d_ref_res.alloc(3) != cudaSuccess ||
        h->d_ref_count.alloc(1) != cudaSuccess) {
        h->refined = false;
        return fail(RBX_ERR_CUDA, "cudaMalloc of the refined-energy arrays failed");
    }
    CUDA_TRY(cudaMemset(h->d_ref_start.p, 0, start));
    CUDA_TRY(cudaMemset(h->d_ref_out.p, 0, terms * sizeof(float)));
    CUDA_TRY(cudaMemset(h->d_ref_count.p, 0, sizeof(unsigned int)));
    return RBX_OK;
}

int rbx_get_compute_refined_energies(const rbx_integrator* h, int* out) {
    int rc = check(h);
    if (!rc) *out = h->refined ? 1 : 0;
    return rc;
}

// Plain kinetic energies and, with refined energies on, the sums of the refined terms written by
// the last part2: h_ke[0, 2) and h_ke[2, 5).
static int refined_sums(rbx_integrator* h, void* stream, const rbx_buffers* buf) {
    int rc = check_ready(h, buf);
    if (rc) return rc;
    if (h->refined && h->ref_phase != 2)
        return fail(RBX_ERR_STATE, "refined energies need a completed step (part1 or fused, then part2 with the same "
                                   "step size) since the last state change");
    CUDA_TRY(cudaSetDevice(h->device));
    DevSys s = h->sys();
    cudaStream_t st = (cudaStream_t)stream;
    KEScratch k{h->d_ke_partial.p, h->d_ke_count.p, h->d_ke_out.p};
    if (launch_kinetic(h->prec, s, devbuf(buf), k, kinetic_blocks(s), stream) < 0)
        return fail(RBX_ERR_CUDA, "kinetic-energy launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    CUDA_TRY(cudaMemcpyAsync(h->h_ke, h->d_ke_out.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    h->last_launches = 1;
    if (h->refined) {
        RefScratch r{h->d_ref_partial.p, h->d_ref_count.p, h->d_ref_res.p};
        if (launch_refined_sum(s, r, refined_blocks(s), stream) < 0)
            return fail(RBX_ERR_CUDA, "refined-energy sum failed: %s", cudaGetErrorString(cudaGetLastError()));
        CUDA_TRY(cudaMemcpyAsync(h->h_ke + 2, h->d_ref_res.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        h->last_launches = 2;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return RBX_OK;
}

int rbx_refined_kinetic_energies(rbx_integrator* h, void* stream, const rbx_buffers* buf, double* out2) {
    if (!out2) return fail(RBX_ERR_INVALID_ARGUMENT, "null output");
    int rc = refined_sums(h, stream, buf);
    if (rc) return rc;
    out2[0] = h->h_ke[0] + (h->refined ? h->h_ke[2] : 0.0);
    out2[1] = h->h_ke[1] + (h->refined ? h->h_ke[3] : 0.0);
    return RBX_OK;
}

int rbx_potential_energy_refinement(rbx_integrator* h, void* stream, const rbx_buffers* buf, double* out1) {
    if (!out1) return fail(RBX_ERR_INVALID_ARGUMENT, "null output");
    int rc = check(h);
    if (rc) return rc;
    if (!h->refined) {
        *out1 = 0.0;
        return RBX_OK;
    }
    if ((rc = refined_sums(h, stream, buf))) return rc;
    *out1 = -h->h_ke[4] * h->ref_dt * h->ref_dt / 24.0;
    return RBX_OK;
}

int rbx_get_body_state(rbx_integrator* h, double* state) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body state");
    if ((rc = ensure_host_plan(h))) return rc;
    std::vector<double> s;
    CUDA_TRY(cudaSetDevice(h->device));
    if ((rc = get_state(h, s))) return rc;
    for (int b = 0; b < h->nb; b++)
        for (int k = 0; k < 14; k++) state[14 * (size_t)b + k] = s[h->lib_pos[b] + (size_t)k * h->nb_pad];
    return RBX_OK;
}

int rbx_set_body_state(rbx_integrator* h, const double* state) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body geometry: call rbx_upload_state first");
    if ((rc = ensure_host_plan(h))) return rc;
    std::vector<double> s((size_t)14 * h->nb_pad, 0.0);
    for (int b = 0; b < h->nb; b++)
        for (int k = 0; k < 14; k++) s[h->lib_pos[b] + (size_t)k * h->nb_pad] = state[14 * (size_t)b + k];
    CUDA_TRY(cudaSetDevice(h->device));
    h->ref_phase = 0;
    if ((rc = clear_failures(h, nullptr))) return rc;
    return put_state(h, s);
}

// Raw rows: the body state's device words, 112 bytes per body in every precision (14 doubles, or
// 14 high then 14 low floats of the float-float state), bodies in ascending body index.
int rbx_get_body_state_raw(rbx_integrator* h, void* rows) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body state");
    if (!rows && h->nb) return fail(RBX_ERR_INVALID_ARGUMENT, "null output");
    if ((rc = ensure_host_plan(h))) return rc;
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t nbp = (size_t)h->nb_pad;
    if (h->prec == PREC_DOUBLE) {
        std::vector<double> d(14 * nbp);
        CUDA_TRY(cudaMemcpy(d.data(), h->d_state.p, d.size() * sizeof(double), cudaMemcpyDeviceToHost));
        double* out = (double*)rows;
        for (int b = 0; b < h->nb; b++)
            for (int k = 0; k < 14; k++) out[14 * (size_t)b + k] = d[h->lib_pos[b] + k * nbp];
    } else {
        std::vector<float> f(28 * nbp);
        CUDA_TRY(cudaMemcpy(f.data(), h->d_state.p, f.size() * sizeof(float), cudaMemcpyDeviceToHost));
        float* out = (float*)rows;
        for (int b = 0; b < h->nb; b++)
            for (int k = 0; k < 28; k++) out[28 * (size_t)b + k] = f[h->lib_pos[b] + k * nbp];
    }
    return RBX_OK;
}

int rbx_set_body_state_raw(rbx_integrator* h, const void* rows) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body geometry: call rbx_upload_state first");
    if (!rows && h->nb) return fail(RBX_ERR_INVALID_ARGUMENT, "null state");
    if ((rc = ensure_host_plan(h))) return rc;
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t nbp = (size_t)h->nb_pad;
    if (h->prec == PREC_DOUBLE) {
        std::vector<double> d(14 * nbp, 0.0);
        const double* in = (const double*)rows;
        for (int b = 0; b < h->nb; b++)
            for (int k = 0; k < 14; k++) d[h->lib_pos[b] + k * nbp] = in[14 * (size_t)b + k];
        CUDA_TRY(cudaMemcpy(h->d_state.p, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(28 * nbp, 0.0f);
        const float* in = (const float*)rows;
        for (int b = 0; b < h->nb; b++)
            for (int k = 0; k < 28; k++) f[h->lib_pos[b] + k * nbp] = in[28 * (size_t)b + k];
        CUDA_TRY(cudaMemcpy(h->d_state.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    h->ref_phase = 0;
    return clear_failures(h, nullptr);
}

int rbx_get_body_geometry(rbx_integrator* h, double* moments, double* body_fixed) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body geometry");
    if ((rc = ensure_host_geometry(h))) return rc;
    if (moments) std::memcpy(moments, h->I.data(), h->I.size() * sizeof(double));
    if (body_fixed) std::memcpy(body_fixed, h->dfix.data(), h->dfix.size() * sizeof(double));
    return RBX_OK;
}

int rbx_get_body_atoms(rbx_integrator* h, int* first_atom, int* atoms) {
    int rc = check(h);
    if (rc) return rc;
    if (first_atom) std::memcpy(first_atom, h->ref_first.data(), h->ref_first.size() * sizeof(int));
    if (atoms) std::memcpy(atoms, h->ref_atoms.data(), h->ref_atoms.size() * sizeof(int));
    return RBX_OK;
}

// ----------------------------------------------------------------------------------------------
// Owned context buffers and the host-buffer step
// ----------------------------------------------------------------------------------------------
static int ensure_context(rbx_integrator* h) {
    if (h->c_posq.p) {
        if (h->max_location >= h->stride)
            return fail(RBX_ERR_INVALID_ARGUMENT, "device slot %d outside the owned buffers (stride %d)", h->max_location, h->stride);
        return RBX_OK;
    }
    CUDA_TRY(cudaSetDevice(h->device));
    const long long stride = ((std::max<long long>(h->natoms, h->max_location + 1LL) + 31) / 32) * 32;
    if (3 * stride > INT_MAX)
        return fail(RBX_ERR_UNSUPPORTED, "%d atoms exceed the 32-bit device indexing of this build", h->natoms);
    h->stride = (int)stride;
    const size_t p4 = h->prec == PREC_DOUBLE ? 32 : 16, v4 = h->prec == PREC_SINGLE ? 16 : 32;
    if (h->c_posq.alloc(p4 * h->stride) != cudaSuccess || h->c_velm.alloc(v4 * h->stride) != cudaSuccess ||
        h->c_force.alloc((size_t)3 * h->stride) != cudaSuccess || h->c_x.alloc((size_t)3 * h->natoms) != cudaSuccess ||
        h->c_v.alloc((size_t)3 * h->natoms) != cudaSuccess || h->c_f.alloc((size_t)3 * h->natoms) != cudaSuccess ||
        h->c_m.alloc(h->natoms) != cudaSuccess)
        return fail(RBX_ERR_CUDA, "cudaMalloc of context buffers failed");
    if (h->prec == PREC_MIXED && h->c_corr.alloc(16 * (size_t)h->stride) != cudaSuccess)
        return fail(RBX_ERR_CUDA, "cudaMalloc of position corrections failed");
    CUDA_TRY(cudaMemset(h->c_posq.p, 0, p4 * h->stride));
    CUDA_TRY(cudaMemset(h->c_velm.p, 0, v4 * h->stride));
    CUDA_TRY(cudaMemset(h->c_force.p, 0, sizeof(long long) * 3 * h->stride));
    if (h->c_corr.p) CUDA_TRY(cudaMemset(h->c_corr.p, 0, 16 * (size_t)h->stride));
    CUDA_TRY(cudaMemcpy(h->c_m.p, h->masses.data(), sizeof(double) * h->natoms, cudaMemcpyHostToDevice));
    return RBX_OK;
}

int rbx_context_buffers(rbx_integrator* h, rbx_buffers* out) {
    int rc = check(h);
    if (rc) return rc;
    if ((rc = ensure_context(h))) return rc;
    out->posq = h->c_posq.p;
    out->posq_correction = h->c_corr.p;
    out->velm = h->c_velm.p;
    out->force = h->c_force.p;
    out->stride = h->stride;
    return RBX_OK;
}

int rbx_context_set_state(rbx_integrator* h, void* stream, const double* positions, const double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if ((rc = ensure_context(h))) return rc;
    if ((rc = rbx_upload_state(h, positions, velocities))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(h->c_x.p, positions, sizeof(double) * 3 * h->natoms, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(h->c_v.p, velocities, sizeof(double) * 3 * h->natoms, cudaMemcpyHostToDevice, st));
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    if (launch_load_positions(h->prec, h->c_x.p, h->c_v.p, h->c_m.p, h->c_loc.p, h->natoms, devbuf(&b), stream) < 0)
        return fail(RBX_ERR_CUDA, "position upload kernel failed");
    CUDA_TRY(cudaStreamSynchronize(st));
    return RBX_OK;
}

int rbx_context_get_range(rbx_integrator* h, void* stream, int first_atom, int count, double* positions,
                          double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if (first_atom < 0 || count < 0 || first_atom + count > h->natoms)
        return fail(RBX_ERR_INVALID_ARGUMENT, "atom range [%d, %d) outside [0, %d)", first_atom, first_atom + count, h->natoms);
    if ((rc = ensure_context(h))) return rc;
    if (count == 0) return RBX_OK;
    cudaStream_t st = (cudaStream_t)stream;
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    double* x = h->c_x.p + 3 * (size_t)first_atom;
    double* v = h->c_v.p + 3 * (size_t)first_atom;
    if (launch_store_positions(h->prec, devbuf(&b), h->c_loc.p + first_atom, count, x, velocities ? v : nullptr,
                               stream) < 0)
        return fail(RBX_ERR_CUDA, "position download kernel failed");
    if (positions) CUDA_TRY(cudaMemcpyAsync(positions, x, sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, st));
    if (velocities) CUDA_TRY(cudaMemcpyAsync(velocities, v, sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return RBX_OK;
}

int rbx_context_load(rbx_integrator* h, void* stream, const double* positions, const double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if (!positions || !velocities) return fail(RBX_ERR_INVALID_ARGUMENT, "null positions or velocities");
    if ((rc = ensure_context(h))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(h->c_x.p, positions, sizeof(double) * 3 * h->natoms, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(h->c_v.p, velocities, sizeof(double) * 3 * h->natoms, cudaMemcpyHostToDevice, st));
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    if (launch_load_positions(h->prec, h->c_x.p, h->c_v.p, h->c_m.p, h->c_loc.p, h->natoms, devbuf(&b), stream) < 0)
        return fail(RBX_ERR_CUDA, "position upload kernel failed");
    CUDA_TRY(cudaStreamSynchronize(st));
    h->ref_phase = 0;
    return RBX_OK;
}

int rbx_context_sync_bodies(rbx_integrator* h, void* stream) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->have_state) return fail(RBX_ERR_STATE, "no rigid-body state");
    if ((rc = ensure_context(h))) return rc;
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    if (launch_sync_positions(h->prec, h->sys(), devbuf(&b), stream) < 0)
        return fail(RBX_ERR_CUDA, "position rebuild kernel failed");
    h->last_launches = 1;
    return RBX_OK;
}

int rbx_context_set_forces(rbx_integrator* h, void* stream, const double* forces) {
    int rc = check(h);
    if (rc) return rc;
    if ((rc = ensure_context(h))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(h->c_f.p, forces, sizeof(double) * 3 * h->natoms, cudaMemcpyHostToDevice, st));
    if (launch_forces_from_host(h->prec, h->c_f.p, h->c_loc.p, h->natoms, h->c_force.p, h->stride, stream) < 0)
        return fail(RBX_ERR_CUDA, "force conversion kernel failed");
    return RBX_OK;
}

int rbx_context_get_state(rbx_integrator* h, void* stream, double* positions, double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if ((rc = ensure_context(h))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    if (launch_store_positions(h->prec, devbuf(&b), h->c_loc.p, h->natoms, h->c_x.p, velocities ? h->c_v.p : nullptr,
                               stream) < 0)
        return fail(RBX_ERR_CUDA, "position download kernel failed");
    if (positions) CUDA_TRY(cudaMemcpyAsync(positions, h->c_x.p, sizeof(double) * 3 * h->natoms, cudaMemcpyDeviceToHost, st));
    if (velocities) CUDA_TRY(cudaMemcpyAsync(velocities, h->c_v.p, sizeof(double) * 3 * h->natoms, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return RBX_OK;
}

int rbx_step_host(rbx_integrator* h, void* stream, int nsteps, double dt, const double* forces, double* positions,
                  double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if (nsteps < 1) return fail(RBX_ERR_INVALID_ARGUMENT, "nsteps must be >= 1");
    if (!forces) return fail(RBX_ERR_INVALID_ARGUMENT, "null forces");
    if ((rc = rbx_context_set_forces(h, stream, forces))) return rc;
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    int launches = 1;
    if ((rc = rbx_integrate_part1(h, stream, &b, dt))) return rc;
    for (int n = 1; n < nsteps; n++) {
        if ((rc = rbx_integrate_fused(h, stream, &b, dt))) return rc;
        launches++;
    }
    if ((rc = rbx_integrate_part2(h, stream, &b, dt))) return rc;
    launches += 2;  // part2 + force conversion
    if ((rc = rbx_context_get_state(h, stream, positions, velocities))) return rc;
    h->last_launches = launches + 1;
    return RBX_OK;
}

// Pipelined host-buffer steps. Call i uses staging slot i % 2: its forces go up on the input
// stream once call i-2 has finished reading that slot, its kernels run on `stream` once the
// upload has landed (and once call i-2's results have left the output slot), and its positions
// and velocities go down on the output stream once the kernels are done. Consecutive calls so
// overlap one call's upload and another's download with a third's kernels.
int rbx_step_host_async(rbx_integrator* h, void* stream, int nsteps, double dt, const double* forces,
                        double* positions, double* velocities) {
    int rc = check(h);
    if (rc) return rc;
    if (nsteps < 1) return fail(RBX_ERR_INVALID_ARGUMENT, "nsteps must be >= 1");
    if (!forces || !positions || !velocities) return fail(RBX_ERR_INVALID_ARGUMENT, "null host array");
    if ((rc = ensure_context(h))) return rc;
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t n3 = (size_t)3 * h->natoms;
    if (!h->p_out) {
        // First use: staging buffers, events and copy streams. Each piece is made only if it is
        // missing, so a call after a failure here completes the setup without leaking; p_out is
        // created last and marks it complete.
        for (int s = 0; s < 2; s++) {
            if ((!h->p_f[s].p && h->p_f[s].alloc(n3) != cudaSuccess) || (!h->p_x[s].p && h->p_x[s].alloc(n3) != cudaSuccess) ||
                (!h->p_v[s].p && h->p_v[s].alloc(n3) != cudaSuccess))
                return fail(RBX_ERR_CUDA, "cudaMalloc of pipeline staging failed");
            if (!h->p_in_done[s]) CUDA_TRY(cudaEventCreateWithFlags(&h->p_in_done[s], cudaEventDisableTiming));
            if (!h->p_compute_done[s]) CUDA_TRY(cudaEventCreateWithFlags(&h->p_compute_done[s], cudaEventDisableTiming));
            if (!h->p_out_done[s]) CUDA_TRY(cudaEventCreateWithFlags(&h->p_out_done[s], cudaEventDisableTiming));
            CUDA_TRY(cudaEventRecord(h->p_compute_done[s], (cudaStream_t)stream));
            CUDA_TRY(cudaEventRecord(h->p_out_done[s], (cudaStream_t)stream));
        }
        if (!h->p_in) CUDA_TRY(cudaStreamCreateWithFlags(&h->p_in, cudaStreamNonBlocking));
        CUDA_TRY(cudaStreamCreateWithFlags(&h->p_out, cudaStreamNonBlocking));
    }
    const int s = (int)(h->p_calls & 1);
    cudaStream_t st = (cudaStream_t)stream;
    // upload
    CUDA_TRY(cudaStreamWaitEvent(h->p_in, h->p_compute_done[s], 0));
    CUDA_TRY(cudaMemcpyAsync(h->p_f[s].p, forces, sizeof(double) * n3, cudaMemcpyHostToDevice, h->p_in));
    CUDA_TRY(cudaEventRecord(h->p_in_done[s], h->p_in));
    // kernels
    CUDA_TRY(cudaStreamWaitEvent(st, h->p_in_done[s], 0));
    if (launch_forces_from_host(h->prec, h->p_f[s].p, h->c_loc.p, h->natoms, h->c_force.p, h->stride, stream) < 0)
        return fail(RBX_ERR_CUDA, "force conversion kernel failed");
    rbx_buffers b;
    rbx_context_buffers(h, &b);
    int launches = 1;
    if ((rc = rbx_integrate_part1(h, stream, &b, dt))) return rc;
    for (int n = 1; n < nsteps; n++) {
        if ((rc = rbx_integrate_fused(h, stream, &b, dt))) return rc;
        launches++;
    }
    if ((rc = rbx_integrate_part2(h, stream, &b, dt))) return rc;
    launches += 2;
    CUDA_TRY(cudaStreamWaitEvent(st, h->p_out_done[s], 0));
    if (launch_store_positions(h->prec, devbuf(&b), h->c_loc.p, h->natoms, h->p_x[s].p, h->p_v[s].p, stream) < 0)
        return fail(RBX_ERR_CUDA, "position download kernel failed");
    CUDA_TRY(cudaEventRecord(h->p_compute_done[s], st));
    // download
    CUDA_TRY(cudaStreamWaitEvent(h->p_out, h->p_compute_done[s], 0));
    CUDA_TRY(cudaMemcpyAsync(positions, h->p_x[s].p, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->p_out));
    CUDA_TRY(cudaMemcpyAsync(velocities, h->p_v[s].p, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->p_out));
    CUDA_TRY(cudaEventRecord(h->p_out_done[s], h->p_out));
    h->p_calls++;
    h->last_launches = launches + 1;
    return RBX_OK;
}

int rbx_step_host_wait(rbx_integrator* h) {
    int rc = check(h);
    if (rc) return rc;
    if (!h->p_out) return RBX_OK;
    CUDA_TRY(cudaSetDevice(h->device));
    CUDA_TRY(cudaStreamSynchronize(h->p_out));
    for (int s = 0; s < 2; s++) CUDA_TRY(cudaEventSynchronize(h->p_out_done[s]));
    return RBX_OK;
}

int rbx_last_launch_count(const rbx_integrator* h) { return h ? h->last_launches : 0; }

}  // extern "C"
