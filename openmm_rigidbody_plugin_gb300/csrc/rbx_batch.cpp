// rbx_batch.cpp -- batched systems: one integrator over the atoms of many independent periodic
// systems, forces from the library's cell-list LJ + reaction-field kernels, and runs of steps
// replayed from a captured CUDA graph. The C ABI is declared in include/rbx.h.
//
// Every system keeps a contiguous range of device slots, so the integrator's library order (bodies
// by lowest slot) keeps each system's bodies and free atoms contiguous as well, which the
// per-system kinetic-energy reduction relies on.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <new>
#include <thread>
#include <vector>

#include "../../include/rbx.h"
#include "rbx_devarray.h"
#include "rbx_internal.h"

using namespace rbx;

namespace {

constexpr double kOne4PiEps0 = 138.935456;  // kJ nm / (mol e^2)
constexpr double kSkin = 0.06;              // nm: neighbour-list skin (of group centroids)
constexpr int kMaxTypes = 32;               // atom types of the type-pair table (FFDev::types)

#define BATCH_TRY(call)                                                                             \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return set_error(RBX_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

float int_bits(int v) {
    float f;
    std::memcpy(&f, &v, sizeof f);
    return f;
}

// body(s) for every system s, the systems split into contiguous ranges of about equal group counts
// over the host's cores. Each call writes only its own system's outputs, so the results do not
// depend on the split; a thread that cannot be started leaves its range to the calling thread.
template <class F> void for_each_system(const std::vector<FFSys>& sys, F&& body) {
    const int S = (int)sys.size();
    const long long groups = S ? (long long)sys[S - 1].g1 - sys[0].g0 : 0;
    const int nt = (int)std::min<long long>({(long long)std::max(1u, std::thread::hardware_concurrency()), 32LL,
                                             std::max(1LL, groups / 20000)});
    std::vector<int> lo(nt + 1, S);
    lo[0] = 0;
    for (int t = 1, s = 0; t < nt; t++) {
        while (s < S && (long long)(sys[s].g0 - sys[0].g0) * nt < groups * t) s++;
        lo[t] = s;
    }
    auto run = [&](int t) {
        for (int s = lo[t]; s < lo[t + 1]; s++) body(s);
    };
    std::vector<std::thread> pool;
    std::vector<int> inline_ranges;
    for (int t = 1; t < nt; t++) {
        try {
            pool.emplace_back(run, t);
        } catch (...) {
            inline_ranges.push_back(t);
        }
    }
    run(0);
    for (int t : inline_ranges) run(t);
    for (std::thread& th : pool) th.join();
}

template <class T> int upload_vec(DevArray<T>& a, const std::vector<T>& h) {
    if (a.alloc(h.size()) != cudaSuccess) return set_error(RBX_ERR_CUDA, "cudaMalloc of %zu bytes failed", h.size() * sizeof(T));
    if (!h.empty()) BATCH_TRY(cudaMemcpy(a.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return RBX_OK;
}

}  // namespace

struct rbx_batch {
    rbx_integrator* integ = nullptr;
    int S = 0, natoms = 0, prec = PREC_MIXED, device = 0;
    std::vector<int> offsets;
    // force field
    DevArray<FFSys> d_sys;
    DevArray<int> d_iatom, d_isys, d_cell_of, d_cell_count, d_cell_start, d_cell_cursor, d_cell_list;
    DevArray<int> d_grp_k0, d_grp_n, d_gsys, d_kgrp;
    DevArray<int2> d_grp_kn;
    DevArray<int> d_mc_cell, d_mc_sys, d_sc_sys, d_sc_g0;
    DevArray<int> d_pass_groups[kForcePasses];  // FFDev::pass_groups
    DevArray<float4> d_param, d_cpos, d_gcen, d_gref, d_gq, d_types;
    DevArray<unsigned char> d_rebuild;  // FFDev::rebuild
    DevArray<unsigned int> d_nbr;       // neighbour lists of groups (FFDev::nbr)
    DevArray<int> d_ncnt, d_atype;
    DevArray<unsigned int> d_rebuilds;  // list builds per system (FFDev::rebuilds)
    // host copies for the set-up with a state: systems, cells allocated per system, group layout
    std::vector<FFSys> sys_h;
    std::vector<int> cells_alloc, iatom_h, grp_k0_h, grp_n_h;
    std::vector<double> box_h;
    DevArray<double> d_e_group, d_energy;
    FFDev ff{};
    // per-system reductions
    DevArray<int> d_body0, d_free0;
    std::vector<int> body0_h, free0_h;  // host copies: library-order body / free-atom ranges per system
    DevArray<unsigned int> d_sys_status;  // [S] force-kernel failures (FFDev::sys_status)
    DevArray<double> d_ke, d_user;
    std::vector<int> dof;
    double* h_out = nullptr;  // pinned [3*S]
    int last_launches = 0;
    bool u_valid = false;  // d_energy holds the potential energy of the current positions
    // the force buffer holds the forces of the current positions, formed (with their energy) from
    // lists built at those positions: a step call then starts without a force evaluation
    bool f_valid = false;
    // captured runs of (forces, fused step)
    // optional event timing of the force and integrator launch groups (direct launches only)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_marks;  // (start event, end event) per group
    std::vector<int> ev_kind;                   // 0 = forces, 1 = integrator
    int ev_used = 0;
    int graph_k = 0;
    int graph_launches = 0;  // kernels in one replay of the graph
    double graph_dt = 0.0;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;

    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    cudaEvent_t event() {
        if (ev_used == (int)ev_pool.size()) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            ev_pool.push_back(e);
        }
        return ev_pool[ev_used++];
    }
    ~rbx_batch() {
        for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
        drop_graph();
        if (cap_stream) cudaStreamDestroy(cap_stream);
        if (h_out) cudaFreeHost(h_out);
        if (integ) rbx_destroy(integ);
    }
};

namespace {

int check(const rbx_batch* b) { return b ? RBX_OK : set_error(RBX_ERR_INVALID_ARGUMENT, "null batch handle"); }

// Neighbour-list geometry for a state (host positions, user order): each group's radius about its
// centroid (constant for a rigid body), and from the largest radius of each system its list cells
// (at least cutoff + skin + two radii per edge), the build work lists and the list capacity.
int setup_lists(rbx_batch* b, const double* x) {
    const int S = b->S;
    std::vector<FFSys> sys = b->sys_h;
    std::vector<int> mc_cell, mc_sys, sc_sys, sc_g0;
    std::vector<uint32_t> zkey(b->grp_n_h.size());  // spatial order of each system's groups (see below)
    std::vector<double> rho(S, 0.0);                // largest atom distance from a group centroid
    // per system (in parallel): centroids, their Z-order codes and the largest radius
    for_each_system(sys, [&](int s) {
        const FFSys& f = sys[s];
        const double L = b->box_h[s];
        auto img = [L](double d) { return d - L * std::nearbyint(d / L); };
        double rho_max = 0.0;
        for (int g = f.g0; g < f.g1; g++) {
            const int k0 = b->grp_k0_h[g], n = b->grp_n_h[g];
            const double* x0 = x + 3 * (size_t)b->iatom_h[k0];
            double c[3] = {0.0, 0.0, 0.0};
            for (int a = 1; a < n; a++)
                for (int d = 0; d < 3; d++) c[d] += img(x[3 * (size_t)b->iatom_h[k0 + a] + d] - x0[d]);
            for (int d = 0; d < 3; d++) c[d] = x0[d] + c[d] / n;
            // Z-order (Morton) code of the centroid on a 1024^3 grid of the box
            uint32_t z = 0;
            for (int d = 0; d < 3; d++) {
                double u = c[d] / L;
                u -= std::floor(u);
                const uint32_t q = std::min<uint32_t>(1023, (uint32_t)(u * 1024.0));
                for (int bit = 0; bit < 10; bit++) z |= ((q >> bit) & 1u) << (3 * bit + d);
            }
            zkey[g] = z;
            for (int a = 0; a < n; a++) {
                double r2 = 0.0;
                for (int d = 0; d < 3; d++) {
                    const double v = img(x[3 * (size_t)b->iatom_h[k0 + a] + d] - c[d]);
                    r2 += v * v;
                }
                rho_max = std::max(rho_max, std::sqrt(r2));
            }
        }
        rho[s] = rho_max;
    });
    double cap_need = 1.0;
    for (int s = 0; s < S; s++) {
        FFSys& f = sys[s];
        const double L = b->box_h[s], rho_max = rho[s];
        // the device forms the radii in FP32: a margin of 1e-3 nm keeps its ones within the cells
        const double edge = (double)f.rl + 2.0 * rho_max + 1e-3;
        f.pair_image = std::sqrt((double)f.rc2) + 2.0 * rho_max + 1e-3 >= 0.5 * L ? 1 : 0;
        int nc = (int)std::floor(L / edge);
        if (nc > b->cells_alloc[s]) nc = b->cells_alloc[s];
        if (nc < 3) nc = 1;
        f.nc = nc;
        if (nc > 1) {
            for (int c = 0; c < nc * nc * nc; c++) {
                mc_cell.push_back(f.c0 + c);
                mc_sys.push_back(s);
            }
        } else {
            for (int g = f.g0; g < f.g1; g += 64) {
                sc_sys.push_back(s);
                sc_g0.push_back(g);
            }
        }
        const int G = f.g1 - f.g0;
        const double reach = (double)f.rl + 2.0 * rho_max;
        const double expect = 4.18879 * reach * reach * reach * (double)G / (L * L * L);
        cap_need = std::max(cap_need, std::min((double)std::max(G - 1, 1), 1.35 * expect + 32.0));
    }
    const int cap = std::max(32, ((int)std::ceil(cap_need) + 31) / 32 * 32);
    const size_t entries = (size_t)std::max(b->ff.n_groups, 1) * (size_t)cap;
    if (b->d_nbr.n < entries && b->d_nbr.alloc(entries) != cudaSuccess)
        return set_error(RBX_ERR_CUDA, "cudaMalloc of the neighbour lists failed (%d entries per group)", cap);
    // The force pass takes its groups in this order: system by system, each system's groups in
    // Z-order of their centroids (ties by index), so that the warps resident on an SM at once work
    // on neighbouring groups and find much of each other's neighbours in L1. The order schedules
    // work only: every group's forces are formed alike whichever warp forms them. Each system's
    // share of a pass is filled and sorted in place, the systems in parallel.
    {
        std::vector<int> pass[kForcePasses];
        std::vector<size_t> at((size_t)kForcePasses * (S + 1), 0);  // at[k * (S + 1) + s]: system s's start in pass k
        for (int s = 0; s < S; s++)
            for (int g = sys[s].g0; g < sys[s].g1; g++) at[(size_t)force_pass_of(b->grp_n_h[g]) * (S + 1) + s + 1]++;
        for (int k = 0; k < kForcePasses; k++) {
            size_t* a = &at[(size_t)k * (S + 1)];
            for (int s = 0; s < S; s++) a[s + 1] += a[s];
            pass[k].resize(a[S]);
        }
        for_each_system(sys, [&](int s) {
            size_t fill[kForcePasses];
            for (int k = 0; k < kForcePasses; k++) fill[k] = at[(size_t)k * (S + 1) + s];
            for (int g = sys[s].g0; g < sys[s].g1; g++) {
                const int k = force_pass_of(b->grp_n_h[g]);
                pass[k][fill[k]++] = g;
            }
            auto by_key = [&](int u, int v) { return zkey[u] < zkey[v] || (zkey[u] == zkey[v] && u < v); };
            for (int k = 0; k < kForcePasses; k++)
                std::sort(pass[k].begin() + at[(size_t)k * (S + 1) + s], pass[k].begin() + fill[k], by_key);
        });
        for (int k = 0; k < kForcePasses; k++)
            if (!pass[k].empty())
                BATCH_TRY(cudaMemcpy(b->d_pass_groups[k].p, pass[k].data(), sizeof(int) * pass[k].size(),
                                     cudaMemcpyHostToDevice));
    }
    BATCH_TRY(cudaMemcpy(b->d_sys.p, sys.data(), sizeof(FFSys) * (size_t)S, cudaMemcpyHostToDevice));
    if (!mc_cell.empty()) {
        BATCH_TRY(cudaMemcpy(b->d_mc_cell.p, mc_cell.data(), sizeof(int) * mc_cell.size(), cudaMemcpyHostToDevice));
        BATCH_TRY(cudaMemcpy(b->d_mc_sys.p, mc_sys.data(), sizeof(int) * mc_sys.size(), cudaMemcpyHostToDevice));
    }
    if (!sc_sys.empty()) {
        BATCH_TRY(cudaMemcpy(b->d_sc_sys.p, sc_sys.data(), sizeof(int) * sc_sys.size(), cudaMemcpyHostToDevice));
        BATCH_TRY(cudaMemcpy(b->d_sc_g0.p, sc_g0.data(), sizeof(int) * sc_g0.size(), cudaMemcpyHostToDevice));
    }
    BATCH_TRY(cudaMemset(b->d_rebuild.p, 1, (size_t)S));
    FFDev& D = b->ff;
    D.n_mc = (int)mc_cell.size();
    D.n_sc = (int)sc_sys.size();
    D.cap = cap;
    D.nbr = b->d_nbr.p;
    return RBX_OK;
}

DevBuf buffers(rbx_batch* b) {
    rbx_buffers rb;
    rbx_context_buffers(b->integ, &rb);
    DevBuf d;
    d.posq = rb.posq;
    d.corr = rb.posq_correction;
    d.velm = rb.velm;
    d.force = rb.force;
    d.stride = rb.stride;
    return d;
}

// Event pair around one launch group when timing is on (never inside a stream capture).
struct Timed {
    rbx_batch* b;
    void* stream;
    int kind, start = -1;
    Timed(rbx_batch* b_, void* s, int k) : b(b_), stream(s), kind(k) {
        if (b->timing) {
            start = b->ev_used;
            cudaEvent_t e = b->event();
            if (e) cudaEventRecord(e, (cudaStream_t)stream); else start = -1;
        }
    }
    ~Timed() {
        if (start < 0) return;
        const int end = b->ev_used;
        cudaEvent_t e = b->event();
        if (!e) return;
        cudaEventRecord(e, (cudaStream_t)stream);
        b->ev_marks.push_back({start, end});
        b->ev_kind.push_back(kind);
    }
};

// Marks every system's lists for a rebuild at the next evaluation. Forces and energies at the state a
// call starts or ends in are formed from lists built at that state, so they are a function of the
// positions alone (not of when earlier calls last rebuilt); the evaluations in between rebuild a
// system's lists when its atoms have moved half the skin.
int force_rebuild(rbx_batch* b, void* stream) {
    BATCH_TRY(cudaMemsetAsync(b->d_rebuild.p, 1, (size_t)b->S, (cudaStream_t)stream));
    return RBX_OK;
}

int forces(rbx_batch* b, void* stream, bool energy) {
    Timed t(b, stream, 0);
    const int n = launch_forces(b->ff, b->prec, buffers(b), energy, stream);
    if (n < 0) return set_error(RBX_ERR_CUDA, "force kernels failed: %s", cudaGetErrorString(cudaGetLastError()));
    b->last_launches += n;
    return RBX_OK;
}

int integrate(rbx_batch* b, void* stream, int kind, double dt) {
    Timed t(b, stream, 1);
    rbx_buffers rb;
    rbx_context_buffers(b->integ, &rb);
    int rc = kind == STEP_PART1 ? rbx_integrate_part1(b->integ, stream, &rb, dt)
             : kind == STEP_PART2 ? rbx_integrate_part2(b->integ, stream, &rb, dt)
                                  : rbx_integrate_fused(b->integ, stream, &rb, dt);
    if (!rc) b->last_launches += 1;
    return rc;
}

int fused(rbx_batch* b, void* stream, double dt) { return integrate(b, stream, STEP_FUSED, dt); }

int capture(rbx_batch* b, double dt) {
    b->drop_graph();
    const bool timing = b->timing;
    b->timing = false;  // no event records inside the capture
    if (!b->cap_stream) BATCH_TRY(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    BATCH_TRY(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeRelaxed));
    int rc = RBX_OK;
    const int before = b->last_launches;
    for (int i = 0; i < b->graph_k && !rc; i++) {
        rc = forces(b, b->cap_stream, false);
        if (!rc) rc = fused(b, b->cap_stream, dt);
    }
    b->graph_launches = b->last_launches - before;
    b->last_launches = before;
    b->timing = timing;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return set_error(RBX_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return set_error(RBX_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    }
    b->graph_dt = dt;
    return RBX_OK;
}

}  // namespace

extern "C" {

int rbx_batch_create(rbx_batch** out, int num_systems, const int* atom_offsets, const double* box_edges,
                     const double* cutoffs, const int* body_indices, const double* masses, const double* charges,
                     const double* sigmas, const double* epsilons, double eps_solvent, int rotation_mode,
                     int precision, int device) {
    if (!out) return set_error(RBX_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (num_systems <= 0 || !atom_offsets || !box_edges || !cutoffs || !body_indices || !masses || !charges ||
        !sigmas || !epsilons)
        return set_error(RBX_ERR_INVALID_ARGUMENT, "need num_systems > 0 and every per-system and per-atom array");
    if (atom_offsets[0] != 0) return set_error(RBX_ERR_INVALID_ARGUMENT, "atom_offsets[0] must be 0");
    for (int s = 0; s < num_systems; s++) {
        if (atom_offsets[s + 1] <= atom_offsets[s]) return set_error(RBX_ERR_INVALID_ARGUMENT, "system %d has no atoms", s);
        if (!(box_edges[s] > 0.0)) return set_error(RBX_ERR_INVALID_ARGUMENT, "system %d: box edge must be positive", s);
        if (!(cutoffs[s] > 0.0) || !(cutoffs[s] < 0.5 * box_edges[s]))
            return set_error(RBX_ERR_INVALID_ARGUMENT, "system %d: the cutoff must lie in (0, box/2)", s);
    }
    if (!(eps_solvent >= 1.0)) return set_error(RBX_ERR_INVALID_ARGUMENT, "reaction-field dielectric must be >= 1");
    const int N = atom_offsets[num_systems];
    rbx_batch* b = new (std::nothrow) rbx_batch();
    if (!b) return set_error(RBX_ERR_INVALID_ARGUMENT, "out of host memory");
    b->S = num_systems;
    b->natoms = N;
    b->prec = precision;
    b->device = device;
    b->offsets.assign(atom_offsets, atom_offsets + num_systems + 1);

    // one integrator over all systems: per-system body ids made unique
    std::vector<int> ids(N, 0);
    long base = 0;
    for (int s = 0; s < num_systems; s++) {
        int mx = 0;
        for (int i = atom_offsets[s]; i < atom_offsets[s + 1]; i++) {
            if (body_indices[i] > 0) {
                ids[i] = (int)(base + body_indices[i]);
                mx = std::max(mx, body_indices[i]);
            }
        }
        base += mx;
        if (base > 2000000000L) { delete b; return set_error(RBX_ERR_INVALID_ARGUMENT, "too many bodies"); }
    }
    int rc = rbx_create(&b->integ, N, ids.data(), masses, rotation_mode, precision, device);
    if (rc) { delete b; return rc; }

    // force field tables: interacting atoms (charge or LJ) system by system and, within a system,
    // body by body (ascending id; each free atom a group of its own)
    std::vector<FFSys> sys(num_systems);
    std::vector<int> iatom, isys, grp_k0, grp_n, gsys, kgrp;
    std::vector<float4> param;
    int cells = 0;
    for (int s = 0; s < num_systems; s++) {
        FFSys& f = sys[s];
        f.a0 = atom_offsets[s];
        f.a1 = atom_offsets[s + 1];
        f.i0 = (int)iatom.size();
        f.g0 = (int)grp_k0.size();
        std::map<int, std::vector<int>> bodies;
        std::vector<int> free_atoms;
        for (int i = f.a0; i < f.a1; i++) {
            if (charges[i] == 0.0 && epsilons[i] == 0.0) continue;
            if (body_indices[i] > 0) bodies[body_indices[i]].push_back(i);
            else free_atoms.push_back(i);
        }
        auto add_group = [&](const std::vector<int>& atoms) {
            grp_k0.push_back((int)iatom.size());
            grp_n.push_back((int)atoms.size());
            gsys.push_back(s);
            for (int i : atoms) {
                kgrp.push_back((int)grp_k0.size() - 1);
                iatom.push_back(i);
                isys.push_back(s);
                const float qs = (float)(std::sqrt(kOne4PiEps0) * charges[i]);
                param.push_back(make_float4(qs, (float)(0.5 * sigmas[i]), (float)std::sqrt(std::max(epsilons[i], 0.0)),
                                            int_bits(ids[i])));
            }
        };
        for (auto& kv : bodies) add_group(kv.second);
        for (int i : free_atoms) add_group(std::vector<int>{i});
        f.i1 = (int)iatom.size();
        f.g1 = (int)grp_k0.size();
        if (f.i1 - f.i0 >= kMaxSystemAtoms) {
            delete b;
            return set_error(RBX_ERR_UNSUPPORTED, "system %d: %d interacting atoms (at most %d)", s, f.i1 - f.i0,
                             kMaxSystemAtoms - 1);
        }
        const double L = box_edges[s], rc_s = cutoffs[s];
        // Pairs are tested by minimum image when the lists are built (and, where cutoff + two radii
        // may reach half the box, when forces are formed), so cutoff + skin + radii may exceed half
        // the box: an image within the cutoff (below half the box) is always the minimum image, and
        // its group pair is always listed.
        f.rl = (float)(rc_s + kSkin);
        f.half_skin2 = (float)(0.25 * kSkin * kSkin);
        f.pair_image = 1;  // until the radii are known (rbx_batch_set_state)
        // cells for the largest grid any set of radii allows (the radii, known with the positions,
        // can only make the cells larger and fewer)
        int nc = (int)std::floor(L / (rc_s + kSkin));
        if (nc < 3) nc = 1;
        if (nc > 256) nc = 256;
        f.c0 = cells;
        f.nc = nc;
        cells += nc * nc * nc;
        f.L = (float)L;
        f.invL = (float)(1.0 / L);
        f.rc2 = (float)(rc_s * rc_s);
        const double krf = (eps_solvent - 1.0) / ((2.0 * eps_solvent + 1.0) * rc_s * rc_s * rc_s);
        f.krf = (float)krf;
        f.crf = (float)(1.0 / rc_s + krf * rc_s * rc_s);
    }
    b->sys_h = sys;
    b->cells_alloc.resize(num_systems);
    for (int s = 0; s < num_systems; s++) b->cells_alloc[s] = sys[s].nc;
    b->iatom_h = iatom;
    b->grp_k0_h = grp_k0;
    b->grp_n_h = grp_n;
    b->box_h.assign(box_edges, box_edges + num_systems);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete b; return set_error(RBX_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e)); }
    const int nint = (int)iatom.size(), ngrp = (int)grp_k0.size();
    rc = upload_vec(b->d_sys, sys);
    if (!rc) rc = upload_vec(b->d_iatom, iatom);
    if (!rc) rc = upload_vec(b->d_isys, isys);
    if (!rc) rc = upload_vec(b->d_param, param);
    if (!rc) rc = upload_vec(b->d_grp_k0, grp_k0);
    if (!rc) rc = upload_vec(b->d_grp_n, grp_n);
    {
        std::vector<int2> kn(grp_k0.size());
        for (size_t g = 0; g < kn.size(); g++) kn[g] = make_int2(grp_k0[g], grp_n[g]);
        if (!rc) rc = upload_vec(b->d_grp_kn, kn);
    }
    if (!rc) rc = upload_vec(b->d_gsys, gsys);
    if (!rc) rc = upload_vec(b->d_kgrp, kgrp);
    std::vector<int> pass_groups[kForcePasses];  // the force passes' groups, by size
    for (int g = 0; g < (int)grp_n.size(); g++) pass_groups[force_pass_of(grp_n[g])].push_back(g);
    for (int k = 0; k < kForcePasses && !rc; k++) rc = upload_vec(b->d_pass_groups[k], pass_groups[k]);
    // atom types: the distinct (scaled charge, sigma/2, sqrt(epsilon)) triples; with at most
    // kMaxTypes of them the force pass reads one 16-byte record per neighbour (position and type)
    // and takes each pair's coefficients from a table of type pairs
    std::vector<float4> types;
    std::vector<int> type_of(param.size(), -1);
    {
        std::map<std::array<float, 3>, int> seen;
        for (size_t k = 0; k < param.size() && (int)types.size() <= kMaxTypes; k++) {
            const std::array<float, 3> key{param[k].x, param[k].y, param[k].z};
            auto it = seen.find(key);
            if (it == seen.end()) {
                it = seen.emplace(key, (int)types.size()).first;
                types.push_back(make_float4(key[0], key[1], key[2], 0.0f));
            }
            type_of[k] = it->second;
        }
        if ((int)types.size() > kMaxTypes) types.clear();
    }
    if (types.empty()) type_of.clear();
    // the type-pair table: (K q_i q_j, 12 C12, 6 C6) with C12 = 4 eps sig^12, C6 = 4 eps sig^6 and
    // Lorentz-Berthelot sig = (sig_i + sig_j)/2, eps = sqrt(eps_i eps_j), formed in FP64 from the
    // FP32 type values (the force is (12 C12 r^-6 - 6 C6) r^-8 r)
    const int nt = (int)types.size();
    std::vector<float4> pair_table((size_t)nt * nt);
    for (int i = 0; i < nt; i++)
        for (int j = 0; j < nt; j++) {
            const double sig = (double)types[i].y + (double)types[j].y, eps = (double)types[i].z * (double)types[j].z;
            const double s6 = sig * sig * sig * sig * sig * sig;
            pair_table[(size_t)i * nt + j] = make_float4((float)((double)types[i].x * (double)types[j].x),
                                                         (float)(48.0 * eps * s6 * s6), (float)(24.0 * eps * s6), 0.0f);
        }
    if (!rc) rc = upload_vec(b->d_types, pair_table);
    if (!rc) rc = upload_vec(b->d_atype, type_of);
    // work lists (filled with the state): at most every cell, and every 64-group chunk
    size_t sc_max = 0;
    for (int s = 0; s < num_systems; s++) sc_max += (size_t)(sys[s].g1 - sys[s].g0 + 63) / 64;
    const int g1 = std::max(ngrp, 1), n1 = std::max(nint, 1);
    if (!rc && (b->d_cell_of.alloc(g1) != cudaSuccess || b->d_cell_list.alloc(g1) != cudaSuccess ||
                b->d_gcen.alloc(g1) != cudaSuccess || b->d_gref.alloc(g1) != cudaSuccess ||
                b->d_gq.alloc(g1) != cudaSuccess || b->d_ncnt.alloc(g1) != cudaSuccess ||
                b->d_cell_count.alloc(cells) != cudaSuccess || b->d_cell_start.alloc(cells + 1) != cudaSuccess ||
                b->d_cell_cursor.alloc(cells) != cudaSuccess || b->d_cpos.alloc(n1) != cudaSuccess ||
                b->d_e_group.alloc(g1) != cudaSuccess || b->d_mc_cell.alloc(std::max(cells, 1)) != cudaSuccess ||
                b->d_mc_sys.alloc(std::max(cells, 1)) != cudaSuccess ||
                b->d_sc_sys.alloc(std::max<size_t>(sc_max, 1)) != cudaSuccess ||
                b->d_sc_g0.alloc(std::max<size_t>(sc_max, 1)) != cudaSuccess ||
                b->d_energy.alloc(num_systems) != cudaSuccess || b->d_ke.alloc(2 * (size_t)num_systems) != cudaSuccess ||
                b->d_user.alloc(3 * (size_t)N) != cudaSuccess || b->d_sys_status.alloc(num_systems) != cudaSuccess ||
                b->d_rebuild.alloc(num_systems) != cudaSuccess || b->d_rebuilds.alloc(num_systems) != cudaSuccess))
        rc = set_error(RBX_ERR_CUDA, "cudaMalloc of force-field arrays failed");
    if (!rc && (cudaMemset(b->d_sys_status.p, 0, sizeof(unsigned int) * (size_t)num_systems) != cudaSuccess ||
                cudaMemset(b->d_cell_count.p, 0, sizeof(int) * (size_t)cells) != cudaSuccess ||
                cudaMemset(b->d_rebuild.p, 1, (size_t)num_systems) != cudaSuccess ||
                cudaMemset(b->d_rebuilds.p, 0, sizeof(unsigned int) * (size_t)num_systems) != cudaSuccess ||
                cudaMemset(b->d_ncnt.p, 0, sizeof(int) * (size_t)g1) != cudaSuccess ||
                cudaMemset(b->d_cell_list.p, 0, sizeof(int) * (size_t)g1) != cudaSuccess))
        rc = set_error(RBX_ERR_CUDA, "initialisation of the force-field arrays failed");
    if (!rc && cudaMallocHost((void**)&b->h_out, sizeof(double) * 3 * (size_t)num_systems) != cudaSuccess)
        rc = set_error(RBX_ERR_CUDA, "pinned allocation failed");
    if (rc) { delete b; return rc; }
    FFDev& D = b->ff;
    D.S = num_systems;
    D.n_int = nint;
    D.n_groups = ngrp;
    D.n_cells = cells;
    D.sys = b->d_sys.p;
    D.iatom = b->d_iatom.p;
    D.isys = b->d_isys.p;
    D.param = b->d_param.p;
    D.grp_k0 = b->d_grp_k0.p;
    D.grp_n = b->d_grp_n.p;
    D.grp_kn = b->d_grp_kn.p;
    D.gsys = b->d_gsys.p;
    D.kgrp = b->d_kgrp.p;
    D.gcen = b->d_gcen.p;
    D.gref = b->d_gref.p;
    D.gq = b->d_gq.p;
    D.cell_of = b->d_cell_of.p;
    D.cell_count = b->d_cell_count.p;
    D.cell_start = b->d_cell_start.p;
    D.cell_cursor = b->d_cell_cursor.p;
    D.cell_list = b->d_cell_list.p;
    D.cpos = b->d_cpos.p;
    D.e_group = b->d_e_group.p;
    D.energy = b->d_energy.p;
    D.fcap = 0.0f;
    D.sys_status = b->d_sys_status.p;
    D.rebuild = b->d_rebuild.p;
    D.rebuilds = b->d_rebuilds.p;
    D.nbr = nullptr;  // allocated with the state (its capacity follows the groups' radii)
    D.ncnt = b->d_ncnt.p;
    D.cap = 0;
    D.types = b->d_types.p;
    D.atype = b->d_atype.p;
    D.ntypes = (int)types.size();
    for (int k = 0; k < kForcePasses; k++) {
        D.n_pass[k] = (int)pass_groups[k].size();
        D.pass_groups[k] = b->d_pass_groups[k].p;
    }
    D.cell_threads = 128;
    D.n_mc = 0;
    D.n_sc = 0;
    D.mc_cell = b->d_mc_cell.p;
    D.mc_sys = b->d_mc_sys.p;
    D.sc_sys = b->d_sc_sys.p;
    D.sc_g0 = b->d_sc_g0.p;
    // the owned OpenMM-layout buffers (forces of non-interacting atoms stay zero)
    rbx_buffers rb;
    if ((rc = rbx_context_buffers(b->integ, &rb))) { delete b; return rc; }
    *out = b;
    return RBX_OK;
}

int rbx_batch_destroy(rbx_batch* b) {
    delete b;
    return RBX_OK;
}

int rbx_batch_set_state(rbx_batch* b, void* stream, const double* positions, const double* velocities) {
    int rc = check(b);
    if (rc) return rc;
    b->u_valid = b->f_valid = false;
    b->drop_graph();
    if (!positions || !velocities) return set_error(RBX_ERR_INVALID_ARGUMENT, "null positions or velocities");
    BATCH_TRY(cudaSetDevice(b->device));
    BATCH_TRY(cudaStreamSynchronize((cudaStream_t)stream));  // no force pass in flight on the old lists
    if ((rc = setup_lists(b, positions))) return rc;
    // positions and velocities into the device buffers, bodies built there (no host round trip)
    if ((rc = rbx_context_load(b->integ, stream, positions, velocities))) return rc;
    rbx_buffers rb;
    if ((rc = rbx_context_buffers(b->integ, &rb))) return rc;
    if ((rc = rbx_upload_state_device(b->integ, stream, &rb))) return rc;
    // body atoms start where the body state puts them (the step kernels' arithmetic), so that a
    // system's trajectory is a function of its body state alone, in or out of a batch
    if ((rc = rbx_context_sync_bodies(b->integ, stream))) return rc;
    if ((rc = sync_host_dof(b->integ))) return rc;
    std::vector<int> body0, free0;
    if ((rc = system_ranges(b->integ, b->offsets, body0, free0, b->dof))) return rc;
    if ((rc = upload_vec(b->d_body0, body0)) || (rc = upload_vec(b->d_free0, free0))) return rc;
    b->body0_h = body0;
    b->free0_h = free0;
    BATCH_TRY(cudaMemsetAsync(b->d_sys_status.p, 0, sizeof(unsigned int) * (size_t)b->S, (cudaStream_t)stream));
    return RBX_OK;
}

int rbx_batch_get_state(rbx_batch* b, void* stream, double* positions, double* velocities) {
    int rc = check(b);
    if (rc) return rc;
    return rbx_context_get_state(b->integ, stream, positions, velocities);
}

int rbx_batch_get_system_state(rbx_batch* b, void* stream, int s, double* positions, double* velocities) {
    int rc = check(b);
    if (rc) return rc;
    if (s < 0 || s >= b->S) return set_error(RBX_ERR_INVALID_ARGUMENT, "system %d outside [0, %d)", s, b->S);
    return rbx_context_get_range(b->integ, stream, b->offsets[s], b->offsets[s + 1] - b->offsets[s], positions,
                                 velocities);
}

int rbx_batch_get_body_state(rbx_batch* b, void* body_rows) {
    int rc = check(b);
    if (rc) return rc;
    return rbx_get_body_state_raw(b->integ, body_rows);
}

int rbx_batch_restore(rbx_batch* b, void* stream, const void* body_rows, const double* positions,
                      const double* velocities) {
    int rc = check(b);
    if (rc) return rc;
    if (!b->d_body0.p) return set_error(RBX_ERR_STATE, "no geometry: call rbx_batch_set_state with the systems first");
    b->u_valid = b->f_valid = false;
    if ((rc = rbx_context_load(b->integ, stream, positions, velocities))) return rc;
    if ((rc = rbx_set_body_state_raw(b->integ, body_rows))) return rc;
    if ((rc = rbx_context_sync_bodies(b->integ, stream))) return rc;
    BATCH_TRY(cudaMemsetAsync(b->d_sys_status.p, 0, sizeof(unsigned int) * (size_t)b->S, (cudaStream_t)stream));
    return RBX_OK;
}

int rbx_batch_step(rbx_batch* b, void* stream, int nsteps, double dt) {
    int rc = check(b);
    if (rc) return rc;
    if (nsteps < 1) return set_error(RBX_ERR_INVALID_ARGUMENT, "nsteps must be >= 1");
    if (!(dt == dt) || dt == 0.0) return set_error(RBX_ERR_INVALID_ARGUMENT, "step size must be finite and non-zero");
    if (!b->d_body0.p) return set_error(RBX_ERR_STATE, "no state: call rbx_batch_set_state first");
    BATCH_TRY(cudaSetDevice(b->device));
    b->last_launches = 0;
    // forces at the starting positions: those the previous step call ended with while nothing has
    // changed the state since (formed, as an evaluation here would form them, from lists built at
    // these positions with the energy variant), else one evaluation. The reference likewise keeps
    // the forces of the last step for the next one (CudaRigidBodyKernels.cpp:421-426).
    if (!b->f_valid && ((rc = force_rebuild(b, stream)) || (rc = forces(b, stream, true)))) return rc;
    b->f_valid = false;
    b->u_valid = false;
    if ((rc = integrate(b, stream, STEP_PART1, dt))) return rc;
    int remaining = nsteps - 1;
    if (b->graph_k > 0 && !b->timing && remaining >= b->graph_k) {
        if (!b->graph || b->graph_dt != dt) {
            if ((rc = capture(b, dt))) return rc;
        }
        while (remaining >= b->graph_k) {
            BATCH_TRY(cudaGraphLaunch(b->graph, (cudaStream_t)stream));
            b->last_launches += b->graph_launches;
            remaining -= b->graph_k;
        }
    }
    for (; remaining > 0; remaining--) {
        if ((rc = forces(b, stream, false)) || (rc = fused(b, stream, dt))) return rc;
    }
    // the last evaluation builds every list at the final positions and also forms their potential
    // energy
    if ((rc = force_rebuild(b, stream)) || (rc = forces(b, stream, true))) return rc;
    if ((rc = integrate(b, stream, STEP_PART2, dt))) return rc;
    b->u_valid = true;
    b->f_valid = true;
    return RBX_OK;
}

int rbx_batch_relax(rbx_batch* b, void* stream, int nsteps, double dt, double max_force, double damping) {
    int rc = check(b);
    if (rc) return rc;
    if (nsteps < 1 || !(dt > 0.0) || !(max_force > 0.0) || !(damping >= 0.0 && damping < 1.0))
        return set_error(RBX_ERR_INVALID_ARGUMENT,
                         "relaxation needs nsteps >= 1, dt > 0, max_force > 0 and 0 <= damping < 1");
    if (!b->d_body0.p) return set_error(RBX_ERR_STATE, "no state: call rbx_batch_set_state first");
    BATCH_TRY(cudaSetDevice(b->device));
    b->last_launches = 0;
    rbx_buffers rb;
    rbx_context_buffers(b->integ, &rb);
    const DevSys sys = device_system(b->integ);
    b->ff.fcap = (float)max_force;
    b->u_valid = false;
    b->f_valid = false;
    if ((rc = force_rebuild(b, stream))) return rc;
    for (int n = 0; n < nsteps && !rc; n++) {
        rc = forces(b, stream, false);
        if (!rc && launch_scale_momenta(b->prec, sys, buffers(b), damping, stream) < 0)
            rc = set_error(RBX_ERR_CUDA, "momentum damping failed");
        if (!rc) rc = rbx_integrate_part1(b->integ, stream, &rb, dt);
        b->last_launches += 2;
    }
    b->ff.fcap = 0.0f;
    if (rc) return rc;
    if (launch_scale_momenta(b->prec, sys, buffers(b), 0.0, stream) < 0) return set_error(RBX_ERR_CUDA, "momentum reset failed");
    return RBX_OK;
}

int rbx_batch_energies(rbx_batch* b, void* stream, double* out) {
    int rc = check(b);
    if (rc) return rc;
    if (!out) return set_error(RBX_ERR_INVALID_ARGUMENT, "null output");
    if (!b->d_body0.p) return set_error(RBX_ERR_STATE, "no state: call rbx_batch_set_state first");
    BATCH_TRY(cudaSetDevice(b->device));
    b->last_launches = 0;
    // the potential energy of the last step call's final positions when it is still current (formed
    // in that call's last force evaluation); otherwise a force evaluation that forms it
    if (!b->u_valid && ((rc = force_rebuild(b, stream)) || (rc = forces(b, stream, true)))) return rc;
    b->u_valid = true;
    b->f_valid = true;
    if (launch_kinetic_systems(b->prec, device_system(b->integ), buffers(b), b->d_body0.p, b->d_free0.p, b->S,
                               b->d_ke.p, stream) < 0)
        return set_error(RBX_ERR_CUDA, "kinetic-energy kernel failed: %s", cudaGetErrorString(cudaGetLastError()));
    b->last_launches += 1;
    cudaStream_t st = (cudaStream_t)stream;
    BATCH_TRY(cudaMemcpyAsync(b->h_out, b->d_energy.p, sizeof(double) * b->S, cudaMemcpyDeviceToHost, st));
    BATCH_TRY(cudaMemcpyAsync(b->h_out + b->S, b->d_ke.p, sizeof(double) * 2 * b->S, cudaMemcpyDeviceToHost, st));
    BATCH_TRY(cudaStreamSynchronize(st));
    for (int s = 0; s < b->S; s++) {
        out[3 * s] = b->h_out[s];
        out[3 * s + 1] = b->h_out[b->S + 2 * s];
        out[3 * s + 2] = b->h_out[b->S + 2 * s + 1];
    }
    return RBX_OK;
}

int rbx_batch_forces(rbx_batch* b, void* stream, double* forces_out, double* energies) {
    int rc = check(b);
    if (rc) return rc;
    if (!b->d_body0.p) return set_error(RBX_ERR_STATE, "no state: call rbx_batch_set_state first");
    BATCH_TRY(cudaSetDevice(b->device));
    b->last_launches = 0;
    if ((rc = force_rebuild(b, stream)) || (rc = forces(b, stream, true))) return rc;
    b->u_valid = true;
    b->f_valid = true;
    cudaStream_t st = (cudaStream_t)stream;
    const DevBuf d = buffers(b);
    if (forces_out) {
        if (launch_forces_to_user(d.force, d.stride, b->natoms, b->d_user.p, stream) < 0)
            return set_error(RBX_ERR_CUDA, "force conversion failed");
        BATCH_TRY(cudaMemcpyAsync(forces_out, b->d_user.p, sizeof(double) * 3 * (size_t)b->natoms, cudaMemcpyDeviceToHost, st));
    }
    if (energies) BATCH_TRY(cudaMemcpyAsync(energies, b->d_energy.p, sizeof(double) * b->S, cudaMemcpyDeviceToHost, st));
    BATCH_TRY(cudaStreamSynchronize(st));
    return RBX_OK;
}

int rbx_batch_get_num_dof(rbx_batch* b, int* dof) {
    int rc = check(b);
    if (rc) return rc;
    if (b->dof.empty()) return set_error(RBX_ERR_STATE, "degrees of freedom are known after rbx_batch_set_state");
    std::copy(b->dof.begin(), b->dof.end(), dof);
    return RBX_OK;
}

int rbx_batch_list_builds(rbx_batch* b, void* stream, unsigned int* counts) {
    int rc = check(b);
    if (rc) return rc;
    if (!counts) return set_error(RBX_ERR_INVALID_ARGUMENT, "null output");
    BATCH_TRY(cudaSetDevice(b->device));
    BATCH_TRY(cudaMemcpyAsync(counts, b->d_rebuilds.p, sizeof(unsigned int) * (size_t)b->S, cudaMemcpyDeviceToHost,
                              (cudaStream_t)stream));
    BATCH_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return RBX_OK;
}

int rbx_batch_memory(const rbx_batch* b, size_t* bytes) {
    int rc = check(b);
    if (rc) return rc;
    if (!bytes) return set_error(RBX_ERR_INVALID_ARGUMENT, "null output");
    size_t n = b->d_sys.bytes() + b->d_iatom.bytes() + b->d_isys.bytes() + b->d_cell_of.bytes() +
               b->d_cell_count.bytes() + b->d_cell_start.bytes() + b->d_cell_cursor.bytes() + b->d_cell_list.bytes() +
               b->d_grp_k0.bytes() + b->d_grp_n.bytes() + b->d_grp_kn.bytes() + b->d_gsys.bytes() + b->d_kgrp.bytes() +
               b->d_mc_cell.bytes() + b->d_mc_sys.bytes() + b->d_sc_sys.bytes() + b->d_sc_g0.bytes() +
               b->d_pass_groups[0].bytes() + b->d_pass_groups[1].bytes() + b->d_pass_groups[2].bytes() +
               b->d_param.bytes() + b->d_cpos.bytes() + b->d_gcen.bytes() + b->d_gref.bytes() + b->d_gq.bytes() +
               b->d_types.bytes() + b->d_rebuild.bytes() + b->d_nbr.bytes() + b->d_ncnt.bytes() + b->d_atype.bytes() +
               b->d_rebuilds.bytes() + b->d_e_group.bytes() + b->d_energy.bytes() + b->d_body0.bytes() +
               b->d_free0.bytes() + b->d_sys_status.bytes() + b->d_ke.bytes() + b->d_user.bytes();
    *bytes = n + (b->integ ? device_bytes(b->integ) : 0);
    return RBX_OK;
}

int rbx_batch_status(rbx_batch* b, void* stream, int* system_status, int* num_failed) {
    int rc = check(b);
    if (rc) return rc;
    if (b->body0_h.empty()) return set_error(RBX_ERR_STATE, "no state: call rbx_batch_set_state first");
    BATCH_TRY(cudaSetDevice(b->device));
    std::vector<unsigned int> fs(b->S);
    BATCH_TRY(cudaMemcpyAsync(fs.data(), b->d_sys_status.p, sizeof(unsigned int) * (size_t)b->S, cudaMemcpyDeviceToHost,
                              (cudaStream_t)stream));
    std::vector<uint8_t> bb, fb;
    unsigned int count = 0;
    if ((rc = failure_flags(b->integ, stream, bb, fb, &count))) return rc;  // synchronises the stream
    std::vector<int> failed(b->S, 0);
    for (int s = 0; s < b->S; s++) {
        bool bad = fs[s] != 0;
        if (count) {
            for (int L = b->body0_h[s]; L < b->body0_h[s + 1] && !bad; L++) bad = bb[L] != 0;
            for (int j = b->free0_h[s]; j < b->free0_h[s + 1] && !bad; j++) bad = fb[j] != 0;
        }
        failed[s] = bad ? RBX_ERR_NUMERIC : RBX_OK;
    }
    int n = 0, first = -1;
    for (int s = 0; s < b->S; s++)
        if (failed[s]) {
            if (first < 0) first = s;
            n++;
        }
    if (system_status) std::copy(failed.begin(), failed.end(), system_status);
    if (num_failed) *num_failed = n;
    if (!n) return RBX_OK;
    return set_error(RBX_ERR_NUMERIC, "%d of %d systems failed (first: system %d): a non-finite state after a step, "
                     "or a force beyond the fixed-point range", n, b->S, first);
}

int rbx_batch_autotune(rbx_batch* b, void* stream, double dt, int trial_steps, int* chosen) {
    int rc = check(b);
    if (rc) return rc;
    if (!b->d_body0.p) return set_error(RBX_ERR_STATE, "no state: call rbx_batch_set_state first");
    if (trial_steps < 1) return set_error(RBX_ERR_INVALID_ARGUMENT, "trial_steps must be >= 1");
    if (!(dt == dt) || dt == 0.0) return set_error(RBX_ERR_INVALID_ARGUMENT, "step size must be finite and non-zero");
    BATCH_TRY(cudaSetDevice(b->device));
    cudaStream_t st = (cudaStream_t)stream;
    // the exact state, restored after the trials (they only change how the work is scheduled)
    int nb = 0;
    if ((rc = rbx_get_num_bodies(b->integ, &nb))) return rc;
    std::vector<double> body((size_t)nb * 14 + 1), x((size_t)3 * b->natoms), v((size_t)3 * b->natoms);
    if ((rc = rbx_batch_get_body_state(b, body.data())) || (rc = rbx_batch_get_state(b, stream, x.data(), v.data())))
        return rc;
    const bool timing = b->timing;
    b->timing = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BATCH_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return set_error(RBX_ERR_CUDA, "cudaEventCreate failed");
    }
    // milliseconds per step of `n` steps after one untimed call of the same length
    auto per_step = [&](int n, float& ms) -> int {
        int r = rbx_batch_step(b, stream, n, dt);
        if (!r && cudaEventRecord(e0, st) != cudaSuccess) r = set_error(RBX_ERR_CUDA, "event record failed");
        if (!r) r = rbx_batch_step(b, stream, n, dt);
        if (!r && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                   cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            r = set_error(RBX_ERR_CUDA, "event timing failed");
        ms /= (float)n;
        return r;
    };
    const int k0 = b->graph_k;
    int best_ct = b->ff.cell_threads, best_k = k0;
    float best = 0.0f, ms = 0.0f;
    b->graph_k = 0;
    b->drop_graph();
    // 1. tile shape of the step kernel (single/mixed; 128 threads only for bodies of at most 32
    // atoms): the integrator launches alone, event-timed over 2 x trial_steps steps after one
    // untimed run, since they are a small share of a step
    int best_nt = 0;
    if (!rc && (rc = rbx_get_tile_threads(b->integ, &best_nt)) == RBX_OK) {
        const int nts[2] = {kThreadsF, kThreadsFNarrow};
        double best_i = 0.0;
        bool any = false;
        for (int nt : nts) {
            if (rbx_set_tile_threads(b->integ, nt) != RBX_OK) continue;  // shape not supported here
            b->timing = true;
            if ((rc = rbx_batch_step(b, stream, trial_steps, dt)) || (rc = rbx_batch_set_timing(b, 1)) ||
                (rc = rbx_batch_step(b, stream, 2 * trial_steps, dt)))
                break;
            double mf = 0.0, mi = 0.0;
            if ((rc = rbx_batch_kernel_times(b, &mf, &mi, nullptr))) break;
            if (!any || mi < best_i) {
                best_i = mi;
                best_nt = nt;
                any = true;
            }
        }
        b->timing = false;
        const int rc1 = rbx_set_tile_threads(b->integ, best_nt);
        if (!rc) rc = rc1;
    }
    // 2. block size of the cell list-build kernel, direct launches
    const int cts[3] = {64, 128, 256};
    for (int i = 0; i < 3 && !rc; i++) {
        if (!b->ff.n_mc && cts[i] != best_ct) continue;
        b->ff.cell_threads = cts[i];
        if ((rc = per_step(trial_steps, ms))) break;
        if (i == 0 || ms < best || !b->ff.n_mc) {
            best = ms;
            best_ct = cts[i];
        }
    }
    b->ff.cell_threads = best_ct;
    // 3. steps per captured graph, where launch overhead matters (steps under 1 ms)
    if (!rc && best < 1.0f) {
        const int ks[3] = {0, 10, 50};
        float best_g = 0.0f;
        for (int i = 0; i < 3 && !rc; i++) {
            b->graph_k = ks[i];
            b->drop_graph();
            if ((rc = per_step(ks[i] ? 2 * ks[i] + 1 : trial_steps, ms))) break;
            if (i == 0 || ms < best_g) {
                best_g = ms;
                best_k = ks[i];
            }
        }
    } else if (!rc) {
        best_k = k0 > 0 ? k0 : 50;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->graph_k = best_k;
    b->drop_graph();
    b->timing = timing;
    b->ev_marks.clear();
    b->ev_kind.clear();
    b->ev_used = 0;
    const int rc2 = rbx_batch_restore(b, stream, body.data(), x.data(), v.data());
    if (rc) return rc;
    if (rc2) return rc2;
    if (chosen) {
        chosen[0] = best_ct;
        chosen[1] = best_k;
    }
    return RBX_OK;
}

int rbx_batch_set_tile_threads(rbx_batch* b, int threads) {
    int rc = check(b);
    if (rc) return rc;
    int cur = 0;
    if ((rc = rbx_get_tile_threads(b->integ, &cur))) return rc;
    if (cur == threads) return RBX_OK;
    b->drop_graph();
    return rbx_set_tile_threads(b->integ, threads);
}

int rbx_batch_get_tile_threads(rbx_batch* b, int* out) {
    int rc = check(b);
    if (rc) return rc;
    return rbx_get_tile_threads(b->integ, out);
}

int rbx_batch_set_tuning(rbx_batch* b, int cell_threads, int graph_steps) {
    int rc = check(b);
    if (rc) return rc;
    if (cell_threads != 64 && cell_threads != 128 && cell_threads != 256)
        return set_error(RBX_ERR_INVALID_ARGUMENT, "cell kernel block size must be 64, 128 or 256");
    if ((rc = rbx_batch_set_graph_steps(b, graph_steps))) return rc;
    if (cell_threads != b->ff.cell_threads) b->drop_graph();
    b->ff.cell_threads = cell_threads;
    return RBX_OK;
}

int rbx_batch_set_graph_steps(rbx_batch* b, int k) {
    int rc = check(b);
    if (rc) return rc;
    if (k < 0) return set_error(RBX_ERR_INVALID_ARGUMENT, "graph run length must be >= 0");
    if (k != b->graph_k) b->drop_graph();
    b->graph_k = k;
    return RBX_OK;
}

int rbx_batch_set_timing(rbx_batch* b, int on) {
    int rc = check(b);
    if (rc) return rc;
    b->timing = on != 0;
    b->ev_marks.clear();
    b->ev_kind.clear();
    b->ev_used = 0;
    return RBX_OK;
}

int rbx_batch_kernel_times(rbx_batch* b, double* ms_forces, double* ms_integrator, int* groups) {
    int rc = check(b);
    if (rc) return rc;
    double t[2] = {0.0, 0.0};
    for (size_t i = 0; i < b->ev_marks.size(); i++) {
        float ms = 0.0f;
        BATCH_TRY(cudaEventSynchronize(b->ev_pool[b->ev_marks[i].second]));
        BATCH_TRY(cudaEventElapsedTime(&ms, b->ev_pool[b->ev_marks[i].first], b->ev_pool[b->ev_marks[i].second]));
        t[b->ev_kind[i]] += ms;
    }
    if (ms_forces) *ms_forces = t[0];
    if (ms_integrator) *ms_integrator = t[1];
    if (groups) *groups = (int)b->ev_marks.size();
    b->ev_marks.clear();
    b->ev_kind.clear();
    b->ev_used = 0;
    return RBX_OK;
}

int rbx_batch_last_launch_count(const rbx_batch* b) { return b ? b->last_launches : 0; }

}  // extern "C"
