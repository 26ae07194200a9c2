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
// skin (0.1 nm) + both groups' radii. A rigid group's atoms stay within its radius of its centroid
// however the body turns, so a list ages only as the centroids move: each system rebuilds its
// lists when one of its centroids has moved half the skin since its last build, and at the first
// evaluation of every call (so a call's results depend only on the positions it starts from, never
// on when earlier calls rebuilt). One evaluation, all systems at once:
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
//   8. ff_force_groups  one thread per atom (all systems): the atoms of the groups in its group's
//                  list, pairs within the cutoff (minimum image per pair), no atomics; forces
//                  written as OpenMM fixed point (2^32) to the slot, pair terms summed in list order
//   9. ff_energy   (energy evaluations only) one block per system: fixed-order FP64 sum.
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

// 1. Per group: positions and types of its atoms, its centroid (the mean of the atoms' minimum-image
// displacements from its first atom) and radius, and the rebuild test.
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
        const float3 x = wrap_box(atom_position(B, prec, D.iatom[k]), S);
        const float3 d = min_image(x.x - c.x, x.y - c.y, x.z - c.z, S);
        rho2 = fmaxf(rho2, fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)));
        D.cpos[k] = make_float4(x.x, x.y, x.z, D.ntypes ? __int_as_float(D.atype[k]) : D.param[k].x);
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
constexpr int kMaxTypesDev = 256;  // largest type table of the typed force pass (the host's limit)
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
        D.nbr[(size_t)(g >> 5) * 32 * D.cap + (size_t)n * 32 + (g & 31)] = entry;
    } else if (n == D.cap && D.sys_status) {
        atomicOr(D.sys_status + s, 2u);
    }
    n++;
}

// Group j as a list entry: its first atom relative to the system's, and its atom count.
__device__ __forceinline__ unsigned int pack_group(const FFDev& D, const FFSys& S, int j) {
    return ((unsigned int)(D.grp_k0[j] - S.i0) << kGroupAtomBits) | (unsigned int)D.grp_n[j];
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

template <bool ENERGY>
__device__ __forceinline__ void store_force(const FFDev& D, long long* __restrict__ force, int stride, int k, int slot,
                                            float fx, float fy, float fz, const ESum& e, int si) {
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
    if (ENERGY) D.e_atom[k] = 0.5 * e.value();
}

// 8. Forces from the group lists: one thread per atom k, the atoms of every group in its group's
// list, in list order; a pair beyond the cutoff adds exactly nothing (its term is selected to zero).
// The pair term is OpenMM's CutoffPeriodic form: reaction-field Coulomb and unshifted LJ.
template <bool ENERGY, bool TYPED>
__global__ void __launch_bounds__(128) ff_force_groups(FFDev D, long long* __restrict__ force, int stride) {
    __shared__ float4 stype[TYPED ? kMaxTypesDev : 1];
    if (TYPED) {
        for (int t = threadIdx.x; t < D.ntypes; t += blockDim.x) stype[t] = D.types[t];
        __syncthreads();
    }
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= D.n_int) return;
    const int s = D.isys[k];
    const FFSys S = D.sys[s];
    const int g = D.kgrp[k];
    const float4 xi = D.cpos[k];
    const float4 par = D.param[k];  // sqrt(K) q, sigma/2, sqrt(epsilon)
    const int n = D.ncnt[g];
    const unsigned int* __restrict__ nb = D.nbr + (size_t)(g >> 5) * 32 * D.cap + (g & 31);
    const float4* __restrict__ cpos = D.cpos + S.i0;
    const float4* __restrict__ cpar = D.param + S.i0;
    const bool relax = D.fcap > 0.0f;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    ESum en;
    unsigned int next = n > 0 ? nb[0] : 0u;
    for (int e = 0; e < n; e++) {
        const unsigned int w = next;
        if (e + 1 < n) next = nb[(size_t)(e + 1) * 32];  // the next entry's load overlaps this group
        const int j0 = (int)(w >> kGroupAtomBits), nj = (int)(w & (unsigned int)kMaxGroupAtoms);
        for (int a = 0; a < nj; a++) {
            const float4 xq = cpos[j0 + a];
            float qj, sj, ej;
            if (TYPED) {  // one 16-byte record per neighbour; parameters from the type table
                const float4 tq = stype[__float_as_int(xq.w)];
                qj = tq.x;
                sj = tq.y;
                ej = tq.z;
            } else {
                const float4 pq = cpar[j0 + a];
                qj = pq.x;
                sj = pq.y;
                ej = pq.z;
            }
            const float3 d = min_image(xi.x - xq.x, xi.y - xq.y, xi.z - xq.z, S);
            const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
            // relaxation: coincident atoms have no direction
            const bool in = r2 < S.rc2 && !(relax && r2 < 1e-8f);
            const float r2s = in ? r2 : 1.0f;
            const float inv_r = rsqrtf(r2s), inv_r2 = inv_r * inv_r;
            const float qq = par.x * qj;
            const float sig = par.y + sj, eps = par.z * ej;
            const float s2 = sig * sig * inv_r2, s6 = s2 * s2 * s2;
            float gf = qq * (inv_r * inv_r2 - 2.0f * S.krf) + 4.0f * eps * (12.0f * s6 * s6 - 6.0f * s6) * inv_r2;
            gf = in ? gf : 0.0f;
            fx = fmaf(gf, d.x, fx);
            fy = fmaf(gf, d.y, fy);
            fz = fmaf(gf, d.z, fz);
            if (ENERGY && in) en.add(qq * (inv_r + S.krf * r2 - S.crf) + 4.0f * eps * (s6 * s6 - s6));
        }
    }
    store_force<ENERGY>(D, force, stride, k, D.iatom[k], fx, fy, fz, en, s);
}

__global__ void ff_energy(FFDev D) {
    __shared__ double s[256];
    const FFSys S = D.sys[blockIdx.x];
    double e = 0.0;
    for (int p = S.i0 + threadIdx.x; p < S.i1; p += blockDim.x) e += D.e_atom[p];
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
    const int gf = (D.n_int + 127) / 128;
    const bool typed = D.ntypes > 0 && D.ntypes <= kMaxTypesDev;
    if (typed) {
        if (energy) ff_force_groups<true, true><<<gf, 128, 0, st>>>(D, f, B.stride);
        else ff_force_groups<false, true><<<gf, 128, 0, st>>>(D, f, B.stride);
    } else {
        if (energy) ff_force_groups<true, false><<<gf, 128, 0, st>>>(D, f, B.stride);
        else ff_force_groups<false, false><<<gf, 128, 0, st>>>(D, f, B.stride);
    }
    n++;
    if (energy) {
        ff_energy<<<D.S, 256, 0, st>>>(D);
        n++;
    }
    return cudaPeekAtLastError() == cudaSuccess ? n : -1;
}

}  // namespace rbx
