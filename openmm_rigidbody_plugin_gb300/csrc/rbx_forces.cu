// rbx_forces.cu -- cutoff Lennard-Jones + reaction-field forces for many independent periodic
// systems, by cell lists (the force provider of the batched and served forms; the drop-in takes
// its forces from the OpenMM Context instead).
//
// Functional form: OpenMM NonbondedForce, CutoffPeriodic method, as documented by OpenMM
//   E = K q_i q_j (1/r + k_rf r^2 - c_rf) + 4 eps_ij ((sig_ij/r)^12 - (sig_ij/r)^6),  r < rc,
// Lorentz-Berthelot combination, minimum image in a cubic box, pairs of one rigid body excluded.
//
// Forces come from neighbour lists of groups: the interacting atoms of one rigid body (or one free
// atom) form a group, and a group's list holds every group whose centroid lies within cutoff +
// skin (0.06 nm) + both groups' radii. A rigid group's atoms stay within its radius of its centroid
// however the body turns, so a list ages only as the centroids move: each system rebuilds its
// lists when one of its centroids has moved half the skin since its last build, and every list is
// rebuilt for the state a call starts or ends in (so the forces there depend only on the
// positions, never on when earlier calls rebuilt). One evaluation, all systems at once:
//   1. ff_gcheck   one thread per group: its atoms' positions (wrapped into the box, with their
//                  type) in list order, its centroid and radius, and the centroid's displacement
//                  since the last build (flags the system's rebuild)
//   then, for the flagged systems only (the kernels return at once for the others):
//   2. ff_bin      cell of each group's centroid and cell counts, cells of at least cutoff + skin
//                  + twice the largest radius per edge
//   3. ff_scan     one block per system: exclusive scan of its cells' counts (and count reset)
//   4. ff_scatter  slot in its cell (single-cell systems keep their group order, no atomics)
//   5. ff_sort     one warp per cell of a multi-cell box: sorts the cell by group index
//   6. ff_gather   cell-ordered centroids and radii, and the build centroids
//   7. ff_build_cells / ff_build_box  one block per cell (27 neighbour cells staged in shared
//                  memory) or per 64 groups of a single-cell box (all groups, minimum image): every
//                  other group in range, in a fixed order, into the group's list
//   8. ff_force_groups  one warp per group (all systems): the group's atoms in shared memory, the
//                  lanes streaming the atoms of the listed groups, pairs within the cutoff; per-lane
//                  partial sums joined by a fixed butterfly, no atomics; forces written as OpenMM
//                  fixed point (2^32) to the slots
//   9. ff_energy   (energy evaluations only) one block per system: fixed-order FP64 sum of its
//                  groups' pair energies.
// The atoms of one group never meet in a list: pairs of one rigid body are excluded, as the
// plugin's ForceField helper removes them (python/forcefield.py:131-138).
#include <cuda_runtime.h>

#include <cstdint>

#include "rbx_internal.h"

namespace rbx {

namespace {

__device__ __forceinline__ float3 atom_position(const DevBuf& B, int prec, int slot) {
    if (prec == PREC_DOUBLE) {
        const double* p = (const double*)B.posq + 4 * (size_t)slot;
        return make_float3((float)p[0], (float)p[1], (float)p[2]);
    }
    const float4 p = ((const float4*)B.posq)[slot];
    if (prec == PREC_MIXED) {
        const float4 c = ((const float4*)B.corr)[slot];
        return make_float3(p.x + c.x, p.y + c.y, p.z + c.z);
    }
    return make_float3(p.x, p.y, p.z);
}

__device__ __forceinline__ int wrap_cell(float x, float invL, int nc) {
    float f = x * invL;
    f -= floorf(f);
    int c = (int)(f * (float)nc);
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

// Position of an interacting atom wrapped into [0, L) and its minimum-image displacement.
__device__ __forceinline__ float3 wrap_box(float3 x, const FFSys& S) {
    x.x -= S.L * floorf(x.x * S.invL);
    x.y -= S.L * floorf(x.y * S.invL);
    x.z -= S.L * floorf(x.z * S.invL);
    return x;
}
__device__ __forceinline__ float3 min_image(float dx, float dy, float dz, const FFSys& S) {
    return make_float3(dx - S.L * rintf(dx * S.invL), dy - S.L * rintf(dy * S.invL), dz - S.L * rintf(dz * S.invL));
}

// 1. Per group: its centroid (the mean of the atoms' minimum-image displacements from its first
// atom, wrapped into the box) and radius, its atoms at their images nearest the centroid (so that
// one periodic shift moves a whole group) with their types, and the rebuild test.
__global__ void ff_gcheck(FFDev D, DevBuf B, int prec) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= D.n_groups) return;
    const int s = D.gsys[g];
    const FFSys S = D.sys[s];
    const int k0 = D.grp_k0[g], n = D.grp_n[g];
    const float3 x0 = atom_position(B, prec, D.iatom[k0]);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int a = 1; a < n; a++) {
        const float3 x = atom_position(B, prec, D.iatom[k0 + a]);
        const float3 d = min_image(x.x - x0.x, x.y - x0.y, x.z - x0.z, S);
        sx += d.x;
        sy += d.y;
        sz += d.z;
    }
    const float inv = 1.0f / (float)n;
    const float3 c = wrap_box(make_float3(x0.x + sx * inv, x0.y + sy * inv, x0.z + sz * inv), S);
    float rho2 = 0.f;
    for (int a = 0; a < n; a++) {
        const int k = k0 + a;
        const float3 x = atom_position(B, prec, D.iatom[k]);
        const float3 d = min_image(x.x - c.x, x.y - c.y, x.z - c.z, S);
        rho2 = fmaxf(rho2, fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)));
        D.cpos[k] = make_float4(c.x + d.x, c.y + d.y, c.z + d.z, D.ntypes ? __int_as_float(D.atype[k]) : D.param[k].x);
    }
    D.gcen[g] = make_float4(c.x, c.y, c.z, sqrtf(rho2));
    if (D.rebuild[s]) return;
    const float4 r = D.gref[g];
    const float3 d = min_image(c.x - r.x, c.y - r.y, c.z - r.z, S);
    if (fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)) > S.half_skin2) D.rebuild[s] = 1;
}

__global__ void ff_bin(FFDev D) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= D.n_groups) return;
    const int s = D.gsys[g];
    if (!D.rebuild[s]) return;
    const FFSys S = D.sys[s];
    if (S.nc == 1) {
        D.cell_of[g] = S.c0;
        return;
    }
    const float4 c = D.gcen[g];
    const int cx = wrap_cell(c.x, S.invL, S.nc), cy = wrap_cell(c.y, S.invL, S.nc), cz = wrap_cell(c.z, S.invL, S.nc);
    const int cell = S.c0 + (cz * S.nc + cy) * S.nc + cx;
    D.cell_of[g] = cell;
    atomicAdd(D.cell_count + cell, 1);
}

// Exclusive scan of one system's cell counts, in chunks of blockDim.x; the counts are reset.
__global__ void ff_scan(FFDev D) {
    __shared__ int s[256];
    if (!D.rebuild[blockIdx.x]) return;
    if (threadIdx.x == 0) D.rebuilds[blockIdx.x]++;
    const FFSys S = D.sys[blockIdx.x];
    const int ncell = S.nc * S.nc * S.nc;
    if (S.nc == 1) {
        if (threadIdx.x == 0) {
            D.cell_start[S.c0] = S.g0;
            D.cell_start[S.c0 + 1] = S.g1;
        }
        return;
    }
    int base = S.g0;
    for (int c0 = 0; c0 < ncell; c0 += blockDim.x) {
        const int c = c0 + threadIdx.x;
        const int v = c < ncell ? D.cell_count[S.c0 + c] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {  // Hillis-Steele inclusive scan
            const int t = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (c < ncell) {
            const int start = base + s[threadIdx.x] - v;
            D.cell_start[S.c0 + c] = start;
            D.cell_cursor[S.c0 + c] = start;
            D.cell_count[S.c0 + c] = 0;
        }
        base += s[blockDim.x - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) D.cell_start[S.c0 + ncell] = base;  // equals S.g1
}

__global__ void ff_scatter(FFDev D) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= D.n_groups) return;
    const int s = D.gsys[g];
    if (!D.rebuild[s]) return;
    if (D.sys[s].nc == 1) {
        D.cell_list[g] = g;  // one cell: group order
        return;
    }
    const int p = atomicAdd(D.cell_cursor + D.cell_of[g], 1);
    D.cell_list[p] = g;
}

// Sort each cell of a multi-cell box by group index, so that every cell, and so every list, is in
// a fixed order. One warp per cell: the cell is staged in shared memory and each lane ranks its
// entries against all of them (the entries are distinct, so the ranks are a permutation); a cell
// larger than the stage falls back to an insertion sort by one lane.
constexpr int kSortWarps = 4, kSortStage = 512;
constexpr int kMaxTypesDev = 32;  // most atom types of the type-pair table (the host's limit)
__global__ void __launch_bounds__(32 * kSortWarps) ff_sort(FFDev D) {
    __shared__ int stage[kSortWarps][kSortStage];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * kSortWarps + warp;
    if (w >= D.n_mc) return;
    if (!D.rebuild[D.mc_sys[w]]) return;
    const int c = D.mc_cell[w];
    const int b = D.cell_start[c], e = D.cell_start[c + 1], n = e - b;
    int* s = stage[warp];
    if (n <= kSortStage) {
        for (int i = lane; i < n; i += 32) s[i] = D.cell_list[b + i];
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            const int v = s[i];
            int rank = 0;
            for (int j = 0; j < n; j++) rank += s[j] < v;
            D.cell_list[b + rank] = v;
        }
    } else if (lane == 0) {
        for (int i = b + 1; i < e; i++) {
            const int v = D.cell_list[i];
            int j = i - 1;
            while (j >= b && D.cell_list[j] > v) {
                D.cell_list[j + 1] = D.cell_list[j];
                j--;
            }
            D.cell_list[j + 1] = v;
        }
    }
}

// Cell-ordered centroids and radii of the rebuilt systems; their build centroids.
__global__ void ff_gather(FFDev D) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.n_groups) return;
    if (!D.rebuild[D.gsys[p]]) return;  // list positions [g0, g1) belong to the system of group p
    const int g = D.cell_list[p];
    const float4 c = D.gcen[g];
    D.gq[p] = c;
    D.gref[g] = c;
}

// Appends a packed group entry to group g's list; a full list marks the system as failed (the
// capacity is sized from the densest system with a wide margin, so this does not happen in a
// liquid).
__device__ __forceinline__ void list_append(const FFDev& D, int g, int s, int& n, unsigned int entry) {
    if (n < D.cap) {
        D.nbr[(size_t)g * D.cap + n] = entry;
    } else if (n == D.cap && D.sys_status) {
        atomicOr(D.sys_status + s, 2u);
    }
    n++;
}

// Group j as a list entry: its index relative to the system's first group.
__device__ __forceinline__ unsigned int pack_group(const FFDev&, const FFSys& S, int j) {
    return (unsigned int)(j - S.g0);
}

// 7a. Lists of multi-cell boxes: one block per cell; its groups kFC at a time, each of the 27
// neighbour cells staged in shared memory kFC groups at a time with its periodic image shift applied
// once (exact for groups in range: the cell edge is at least cutoff + skin + twice the largest
// radius, and there are at least three cells per edge).
template <int kFC>
__global__ void __launch_bounds__(kFC) ff_build_cells(FFDev D) {
    __shared__ float4 sx[kFC];
    __shared__ int sg[kFC];
    const int w = blockIdx.x;
    const int s = D.mc_sys[w];
    if (!D.rebuild[s]) return;
    const int c = D.mc_cell[w];
    const FFSys S = D.sys[s];
    const int b = D.cell_start[c], e = D.cell_start[c + 1];
    const int local = c - S.c0, nc = S.nc;
    const int cx = local % nc, cy = (local / nc) % nc, cz = local / (nc * nc);
    const int t = threadIdx.x;
    for (int i0 = b; i0 < e; i0 += kFC) {
        const int p = i0 + t;
        const bool mine = p < e;
        const float4 ci = mine ? D.gq[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int gi = mine ? D.cell_list[p] : -1;
        int n = 0;
        for (int oz = -1; oz <= 1; oz++) {
            int z = cz + oz;
            const float shz = z < 0 ? -S.L : (z >= nc ? S.L : 0.f);
            z = z < 0 ? z + nc : (z >= nc ? z - nc : z);
            for (int oy = -1; oy <= 1; oy++) {
                int y = cy + oy;
                const float shy = y < 0 ? -S.L : (y >= nc ? S.L : 0.f);
                y = y < 0 ? y + nc : (y >= nc ? y - nc : y);
                for (int ox = -1; ox <= 1; ox++) {
                    int x = cx + ox;
                    const float shx = x < 0 ? -S.L : (x >= nc ? S.L : 0.f);
                    x = x < 0 ? x + nc : (x >= nc ? x - nc : x);
                    const int cn = S.c0 + (z * nc + y) * nc + x;
                    const int qb = D.cell_start[cn], qe = D.cell_start[cn + 1];
                    for (int j0 = qb; j0 < qe; j0 += kFC) {
                        __syncthreads();
                        if (j0 + t < qe) {
                            float4 a = D.gq[j0 + t];
                            a.x += shx;
                            a.y += shy;
                            a.z += shz;
                            sx[t] = a;
                            sg[t] = D.cell_list[j0 + t];
                        }
                        __syncthreads();
                        if (mine) {
                            const int m = min(kFC, qe - j0);
                            for (int j = 0; j < m; j++) {
                                const float4 cq = sx[j];
                                const float dx = ci.x - cq.x, dy = ci.y - cq.y, dz = ci.z - cq.z;
                                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                const float lim = S.rl + ci.w + cq.w;
                                if (r2 < lim * lim && sg[j] != gi) list_append(D, gi, s, n, pack_group(D, S, sg[j]));
                            }
                        }
                    }
                }
            }
        }
        if (mine) D.ncnt[gi] = min(n, D.cap);
    }
}

// 7b. Lists of single-cell boxes (fewer than three list cells per edge): one block per 64 groups,
// all groups of the box streamed through shared memory, minimum image per pair.
constexpr int kBT = 64;
__global__ void __launch_bounds__(kBT) ff_build_box(FFDev D) {
    __shared__ float4 sx[kBT];
    const int s = D.sc_sys[blockIdx.x];
    if (!D.rebuild[s]) return;
    const FFSys S = D.sys[s];
    const int t = threadIdx.x;
    const int gi = D.sc_g0[blockIdx.x] + t;
    const bool mine = gi < S.g1;
    const float4 ci = mine ? D.gcen[gi] : make_float4(0.f, 0.f, 0.f, 0.f);
    int n = 0;
    for (int j0 = S.g0; j0 < S.g1; j0 += kBT) {
        __syncthreads();
        if (j0 + t < S.g1) sx[t] = D.gcen[j0 + t];
        __syncthreads();
        if (mine) {
            const int m = min(kBT, S.g1 - j0);
            for (int j = 0; j < m; j++) {
                const float4 cq = sx[j];
                const float3 d = min_image(ci.x - cq.x, ci.y - cq.y, ci.z - cq.z, S);
                const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
                const float lim = S.rl + ci.w + cq.w;
                if (r2 < lim * lim && j0 + j != gi) list_append(D, gi, s, n, pack_group(D, S, j0 + j));
            }
        }
    }
    if (mine) D.ncnt[gi] = min(n, D.cap);
}

// Compensated FP32 accumulator (Knuth's two-sum): the running sum keeps its rounding error in `lo`.
struct ESum {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float s = hi + x, bp = s - hi;
        lo += (hi - (s - bp)) + (x - bp);
        hi = s;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// A group atom's force as OpenMM fixed point (2^32) in its device slot.
__device__ __forceinline__ void store_force(const FFDev& D, long long* __restrict__ force, int stride, int slot, float fx,
                                            float fy, float fz, int si) {
    if (D.fcap > 0.0f) {  // relaxation: cap the magnitude
        const float f2 = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
        if (f2 > D.fcap * D.fcap) {
            const float s = D.fcap * rsqrtf(f2);
            fx *= s;
            fy *= s;
            fz *= s;
        }
    }
    // keep each component inside the 2^32 fixed-point range (|F| < 2^31 kJ/mol/nm); a non-finite
    // force, or one beyond the range (atoms on top of each other), marks its system as failed
    const float kMaxF = 2.0e9f;
    if (D.fcap <= 0.0f && !(fabsf(fx) < kMaxF && fabsf(fy) < kMaxF && fabsf(fz) < kMaxF) && D.sys_status)
        atomicOr(D.sys_status + si, 1u);
    fx = fminf(fmaxf(fx, -kMaxF), kMaxF);
    fy = fminf(fmaxf(fy, -kMaxF), kMaxF);
    fz = fminf(fmaxf(fz, -kMaxF), kMaxF);
    force[slot] = __float2ll_rn(fx * 0x1p32f);
    force[slot + stride] = __float2ll_rn(fy * 0x1p32f);
    force[slot + 2 * stride] = __float2ll_rn(fz * 0x1p32f);
}

// 8. Forces from the group lists: one warp per group. The group's atoms (KIC at a time) sit in
// shared memory. The lanes take the group's list entries 32 at a time: each finds its listed
// group's periodic shift (the minimum image of its centroid relative to this group's) and drops
// the entry when the centroids lie farther apart than cutoff + both radii (no pair of the two is
// then within the cutoff). The surviving groups' atoms are expanded in list order into a queue of
// (atom, entry) words and streamed, 32 at a time, one per lane (the next 32 are loaded while this
// 32 are paired): each streamed atom is shifted and paired with every group atom. Each lane keeps
// partial sums per group atom; a fixed butterfly of shuffles joins the lanes, so every force is a
// sum in a fixed order, with no atomics. A pair beyond the cutoff adds exactly nothing (its term is
// selected to zero, never multiplied).
// Atoms sit at their images nearest their own group's centroid, so the group shift gives the
// minimum image of every pair within the cutoff when cutoff + two radii < L/2; systems of smaller
// boxes (FFSys::pair_image) take the minimum image per pair as well.
// Groups run in three launches by size (force_pass_of): at most 4 atoms (waters, free atoms) with
// KIC = 4, at most 8 with KIC = 8, the others 12 at a time (fewer registers, and so more warps, for
// the small groups). With at most 32 atom types (PT) each pair's (K q_i q_j, 12 C12, 6 C6) comes
// from a type-pair table in shared memory, else from the atoms' own parameters by
// Lorentz-Berthelot.
// The pair term is OpenMM's CutoffPeriodic form: reaction-field Coulomb and unshifted LJ.
constexpr int kFW = 4;     // warps (groups) per block
constexpr int kQ = 256;    // streamed-atom queue per warp
constexpr int kPassKIC[kForcePasses] = {4, 8, 12};  // group atoms per pass over the list, by launch

// One neighbour (position xj after its shift; w: type bits, or its parameters pj) against the ni
// group atoms in shared memory (NI > 0: exactly NI of them, the loop unrolled without exits).
// RELAX: coincident atoms have no direction and add nothing. PI: the minimum image per pair.
// With PT the group atom's .w holds its row of the type-pair table (type x types) and the table
// gives (K q_i q_j, 12 C12, 6 C6); the LJ force is (12 C12 r^-6 - 6 C6) r^-6 r^-2.
template <int KIC, int NI, bool ENERGY, bool PT, bool RELAX, bool PI>
__device__ __forceinline__ void pair_terms(const float4* xs, const float4* ps, int ni, const FFSys& S,
                                           const float4* ptab, float4 xj, float4 pj, bool valid,
                                           float (&f)[KIC][3], ESum& en) {
    const float4* pcol = PT ? ptab + __float_as_int(xj.w) : nullptr;  // column of the neighbour's type
    const float two_krf = 2.0f * S.krf;
#pragma unroll
    for (int a = 0; a < (NI > 0 ? NI : KIC); a++) {
        if (NI == 0 && a >= ni) break;
        const float4 xi = xs[a];
        float3 d = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        if (PI) d = min_image(d.x, d.y, d.z, S);
        const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
        const bool in = valid && r2 < S.rc2 && !(RELAX && r2 < 1e-8f);
        const float inv_r = rsqrtf(r2), inv_r2 = inv_r * inv_r, inv_r6 = inv_r2 * inv_r2 * inv_r2;
        float4 t;  // K q_i q_j, 12 C12, 6 C6
        if (PT) {
            t = pcol[__float_as_int(xi.w)];
        } else {
            const float4 pi = ps[a];
            const float sig = pi.y + pj.y, sig2 = sig * sig, sig6 = sig2 * sig2 * sig2;
            const float c6 = 4.0f * (pi.z * pj.z) * sig6;
            t = make_float4(pi.x * pj.x, 12.0f * c6 * sig6, 6.0f * c6, 0.0f);
        }
        const float lj = inv_r6 * fmaf(t.y, inv_r6, -t.z);  // 12 C12 r^-12 - 6 C6 r^-6
        float gf = fmaf(t.x, inv_r * inv_r2 - two_krf, lj * inv_r2);
        gf = in ? gf : 0.0f;
        f[a][0] = fmaf(gf, d.x, f[a][0]);
        f[a][1] = fmaf(gf, d.y, f[a][1]);
        f[a][2] = fmaf(gf, d.z, f[a][2]);
        if (ENERGY && in)
            en.add(t.x * (inv_r + S.krf * r2 - S.crf) + inv_r6 * (t.y * (1.0f / 12.0f) * inv_r6 - t.z * (1.0f / 6.0f)));
    }
}

// The pair terms of one streamed neighbour, with the group size and image form chosen (the same
// choice for every lane): exact-size forms for the common sizes (1: a free atom; 3: a water; 5:
// a tetrahedral body; 6: a ring's carbons; 12: a full chunk of a larger body), the general one
// otherwise.
template <int KIC, bool ENERGY, bool PT, bool RELAX, bool PI>
__device__ __forceinline__ void pair_dispatch(const float4* xs, const float4* ps, int ni, const FFSys& S,
                                              const float4* ptab, float4 xj, float4 pj, bool valid,
                                              float (&f)[KIC][3], ESum& en) {
    if (KIC == 4) {
        if (ni == 3) return pair_terms<KIC, (KIC >= 3 ? 3 : 0), ENERGY, PT, RELAX, PI>(xs, ps, ni, S, ptab, xj, pj, valid, f, en);
        if (ni == 1) return pair_terms<KIC, 1, ENERGY, PT, RELAX, PI>(xs, ps, ni, S, ptab, xj, pj, valid, f, en);
    } else if (KIC == 8) {
        if (ni == 5) return pair_terms<KIC, (KIC >= 5 ? 5 : 0), ENERGY, PT, RELAX, PI>(xs, ps, ni, S, ptab, xj, pj, valid, f, en);
        if (ni == 6) return pair_terms<KIC, (KIC >= 6 ? 6 : 0), ENERGY, PT, RELAX, PI>(xs, ps, ni, S, ptab, xj, pj, valid, f, en);
    } else {
        if (ni == KIC) return pair_terms<KIC, KIC, ENERGY, PT, RELAX, PI>(xs, ps, ni, S, ptab, xj, pj, valid, f, en);
    }
    pair_terms<KIC, 0, ENERGY, PT, RELAX, PI>(xs, ps, ni, S, ptab, xj, pj, valid, f, en);
}

template <int KIC, bool ENERGY, bool PT, bool RELAX>
__global__ void __launch_bounds__(32 * kFW, KIC == 4 ? 8 : KIC == 8 ? 6 : 5)
    ff_force_groups(FFDev D, const int* __restrict__ work, int n_work, long long* __restrict__ force, int stride) {
    __shared__ float4 stab[PT ? kMaxTypesDev * kMaxTypesDev : 1];
    __shared__ float4 sxi[kFW][KIC];           // group atoms: position, type or charge
    __shared__ float4 spi[kFW][PT ? 1 : KIC];  // their sqrt(K) q, sigma/2, sqrt(epsilon)
    __shared__ float4 ssh[kFW][32];            // periodic shift of each lane's listed group
    __shared__ int squeue[kFW][kQ];            // streamed atoms: (atom - i0) << 5 | lane of its entry
    const int nt = D.ntypes;
    if (PT) {
        for (int t = threadIdx.x; t < nt * nt; t += blockDim.x) stab[t] = D.types[t];
        __syncthreads();
    }
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int w = blockIdx.x * kFW + warp;
    if (w >= n_work) return;
    constexpr unsigned int kAll = 0xffffffffu;
    const int g = work[w];
    const int s = D.gsys[g];
    const FFSys S = D.sys[s];
    const float4 c = D.gcen[g];
    const int k0 = D.grp_k0[g], ng = D.grp_n[g], n = D.ncnt[g];
    const unsigned int* __restrict__ nb = D.nbr + (size_t)g * D.cap;
    const float4* __restrict__ cpos = D.cpos + S.i0;
    const float4* __restrict__ cpar = D.param + S.i0;
    const float reach = sqrtf(S.rc2) + c.w;
    const bool pim = S.pair_image != 0;
    float4* xs = sxi[warp];
    float4* ps = spi[warp];
    float4* sh = ssh[warp];
    int* queue = squeue[warp];
    double e_sum = 0.0;
    for (int a0 = 0; a0 < ng; a0 += KIC) {
        const int ni = min(KIC, ng - a0);
        __syncwarp();
        if (lane < ni) {
            const int k = k0 + a0 + lane;
            const float4 x = D.cpos[k];
            // with the type-pair table, .w becomes the atom's row offset in it (type x types)
            xs[lane] = PT ? make_float4(x.x, x.y, x.z, __int_as_float(__float_as_int(x.w) * nt)) : x;
            if (!PT) ps[lane] = D.param[k];
        }
        __syncwarp();
        float f[KIC][3];
#pragma unroll
        for (int a = 0; a < KIC; a++) f[a][0] = f[a][1] = f[a][2] = 0.0f;
        ESum en;
        for (int e0 = 0; e0 < n; e0 += 32) {
            int nj = 0, j0 = 0;
            float4 shift = make_float4(0.f, 0.f, 0.f, 0.f);
            if (e0 + lane < n) {
                const int gj = S.g0 + (int)nb[e0 + lane];
                const float4 cj = D.gcen[gj];
                const int2 kn = D.grp_kn[gj];
                const int njg = kn.y, j0g = kn.x;
                const float dx = cj.x - c.x, dy = cj.y - c.y, dz = cj.z - c.z;
                shift = make_float4(-S.L * rintf(dx * S.invL), -S.L * rintf(dy * S.invL), -S.L * rintf(dz * S.invL), 0.f);
                const float ex = dx + shift.x, ey = dy + shift.y, ez = dz + shift.z;
                const float lim = reach + cj.w;
                if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < lim * lim) {
                    nj = njg;
                    j0 = j0g - S.i0;
                }
            }
            __syncwarp();  // the previous batch's readers of sh and queue are done
            sh[lane] = shift;
            int incl = nj;  // inclusive prefix sum of the atom counts over the lanes
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(kAll, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(kAll, incl, 31), excl = incl - nj;
            for (int base = 0; base < total; base += kQ) {
                __syncwarp();
                const int hi = min(incl, base + kQ), lo = max(excl, base);
                // a lane's atoms into the queue: unrolled for up to 6 (every group of the
                // benchmark mix), a loop beyond
                if (hi - lo <= 6) {
#pragma unroll
                    for (int u = 0; u < 6; u++)
                        if (lo + u < hi) queue[lo + u - base] = ((j0 + lo + u - excl) << 5) | lane;
                } else {
                    for (int t = lo; t < hi; t++) queue[t - base] = ((j0 + t - excl) << 5) | lane;
                }
                __syncwarp();
                const int cnt = min(kQ, total - base);
                bool valid = lane < cnt;
                int qv = queue[valid ? lane : 0];
                float4 xq = cpos[qv >> 5];
                for (int q0 = 0; q0 < cnt; q0 += 32) {
                    const int qn = q0 + 32;
                    const bool vn = qn + lane < cnt;
                    int qvn = qv;
                    float4 xqn = xq;
                    if (qn < cnt) {
                        qvn = queue[vn ? qn + lane : qn];
                        xqn = cpos[qvn >> 5];
                    }
                    const float4 sv = sh[qv & 31];
                    const float4 xj = make_float4(xq.x + sv.x, xq.y + sv.y, xq.z + sv.z, xq.w);
                    const float4 pj = PT ? xj : cpar[qv >> 5];
                    if (pim)
                        pair_dispatch<KIC, ENERGY, PT, RELAX, true>(xs, ps, ni, S, stab, xj, pj, valid, f, en);
                    else
                        pair_dispatch<KIC, ENERGY, PT, RELAX, false>(xs, ps, ni, S, stab, xj, pj, valid, f, en);
                    valid = vn;
                    qv = qvn;
                    xq = xqn;
                }
            }
        }
        // join the lanes (every lane ends with the same sums) and store the pass's atoms
#pragma unroll
        for (int a = 0; a < KIC; a++) {
            if (a >= ni) break;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                f[a][0] += __shfl_xor_sync(kAll, f[a][0], o);
                f[a][1] += __shfl_xor_sync(kAll, f[a][1], o);
                f[a][2] += __shfl_xor_sync(kAll, f[a][2], o);
            }
            if (lane == a) store_force(D, force, stride, D.iatom[k0 + a0 + a], f[a][0], f[a][1], f[a][2], s);
        }
        if (ENERGY) {
            double e = en.value();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(kAll, e, o);
            e_sum += e;
        }
    }
    if (ENERGY && lane == 0) D.e_group[g] = 0.5 * e_sum;
}

template <int KIC, bool RELAX>
void launch_force_pass(const FFDev& D, const int* work, int n_work, bool energy, bool typed, long long* f, int stride,
                       cudaStream_t st) {
    const int grid = (n_work + kFW - 1) / kFW;
    if (typed) {
        if (energy) ff_force_groups<KIC, true, true, RELAX><<<grid, 32 * kFW, 0, st>>>(D, work, n_work, f, stride);
        else ff_force_groups<KIC, false, true, RELAX><<<grid, 32 * kFW, 0, st>>>(D, work, n_work, f, stride);
    } else {
        if (energy) ff_force_groups<KIC, true, false, RELAX><<<grid, 32 * kFW, 0, st>>>(D, work, n_work, f, stride);
        else ff_force_groups<KIC, false, false, RELAX><<<grid, 32 * kFW, 0, st>>>(D, work, n_work, f, stride);
    }
}

template <int KIC>
void launch_force_pass(const FFDev& D, const int* work, int n_work, bool energy, bool typed, long long* f, int stride,
                       cudaStream_t st) {
    if (D.fcap > 0.0f) launch_force_pass<KIC, true>(D, work, n_work, energy, typed, f, stride, st);
    else launch_force_pass<KIC, false>(D, work, n_work, energy, typed, f, stride, st);
}

__global__ void ff_energy(FFDev D) {
    __shared__ double s[256];
    const FFSys S = D.sys[blockIdx.x];
    double e = 0.0;
    for (int p = S.g0 + threadIdx.x; p < S.g1; p += blockDim.x) e += D.e_group[p];
    s[threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) D.energy[blockIdx.x] = s[0];
}

__global__ void forces_to_user(const long long* __restrict__ f, int stride, int n, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; c++) out[3 * i + c] = (double)f[i + c * stride] * 0x1p-32;
}

}  // namespace

int launch_forces_to_user(const long long* force, int stride, int natoms, double* out, void* stream) {
    if (natoms == 0) return 0;
    forces_to_user<<<(natoms + 255) / 256, 256, 0, (cudaStream_t)stream>>>(force, stride, natoms, out);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_forces(const FFDev& D, int prec, const DevBuf& B, bool energy, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (D.n_int == 0) return 0;
    const int t = 256, gg = (D.n_groups + t - 1) / t;
    int n = 0;
    ff_gcheck<<<gg, t, 0, st>>>(D, B, prec);
    ff_bin<<<gg, t, 0, st>>>(D);
    ff_scan<<<D.S, 256, 0, st>>>(D);
    ff_scatter<<<gg, t, 0, st>>>(D);
    n += 4;
    if (D.n_mc) {
        ff_sort<<<(D.n_mc + kSortWarps - 1) / kSortWarps, 32 * kSortWarps, 0, st>>>(D);
        n++;
    }
    ff_gather<<<gg, t, 0, st>>>(D);
    n++;
    // list builds: block size of the cell kernel chosen by the autotuner (results do not depend
    // on it: every list is built in the same order)
    if (D.n_mc) {
        switch (D.cell_threads) {
            case 64: ff_build_cells<64><<<D.n_mc, 64, 0, st>>>(D); break;
            case 256: ff_build_cells<256><<<D.n_mc, 256, 0, st>>>(D); break;
            default: ff_build_cells<128><<<D.n_mc, 128, 0, st>>>(D);
        }
        n++;
    }
    if (D.n_sc) {
        ff_build_box<<<D.n_sc, kBT, 0, st>>>(D);
        n++;
    }
    if (cudaMemsetAsync(D.rebuild, 0, (size_t)D.S, st) != cudaSuccess) return -1;
    long long* f = const_cast<long long*>(B.force);
    const bool typed = D.ntypes > 0 && D.ntypes <= kMaxTypesDev;
    if (D.n_pass[0]) {
        launch_force_pass<kPassKIC[0]>(D, D.pass_groups[0], D.n_pass[0], energy, typed, f, B.stride, st);
        n++;
    }
    if (D.n_pass[1]) {
        launch_force_pass<kPassKIC[1]>(D, D.pass_groups[1], D.n_pass[1], energy, typed, f, B.stride, st);
        n++;
    }
    if (D.n_pass[2]) {
        launch_force_pass<kPassKIC[2]>(D, D.pass_groups[2], D.n_pass[2], energy, typed, f, B.stride, st);
        n++;
    }
    if (energy) {
        ff_energy<<<D.S, 256, 0, st>>>(D);
        n++;
    }
    return cudaPeekAtLastError() == cudaSuccess ? n : -1;
}

}  // namespace rbx
