// rbx_forces.cu -- cutoff Lennard-Jones + reaction-field forces for many independent periodic
// systems, by cell lists (the force provider of the batched and served forms; the drop-in takes
// its forces from the OpenMM Context instead).
//
// Functional form: OpenMM NonbondedForce, CutoffPeriodic method, as documented by OpenMM
//   E = K q_i q_j (1/r + k_rf r^2 - c_rf) + 4 eps_ij ((sig_ij/r)^12 - (sig_ij/r)^6),  r < rc,
// Lorentz-Berthelot combination, minimum image in a cubic box, pairs of one rigid body excluded.
//
// Forces come from neighbour lists (Verlet lists with a skin of up to 0.1 nm) that each system
// rebuilds when one of its atoms has moved more than half the skin since its last build, and at the
// first evaluation of every call (so a call's results depend only on the positions it starts from,
// never on when earlier calls rebuilt). One evaluation, all systems at once:
//   1. ff_check    one thread per interacting atom: position (wrapped into the box) in the list
//                  order, and the displacement since the last build (flags the system's rebuild)
//   then, for the flagged systems only (the kernels return at once for the others):
//   2. ff_bin      cell index and cell counts, cells of at least cutoff + skin per edge
//   3. ff_scan     one block per system: exclusive scan of its cells' counts (and count reset)
//   4. ff_scatter  slot in its cell (single-cell systems keep their atom order and need no atomics)
//   5. ff_sort     one warp per cell of a multi-cell box: sorts the cell by atom index
//   6. ff_gather   cell-ordered copies of positions and parameters, and the build positions
//   7. ff_build_cells / ff_build_box  one block per cell (27 neighbour cells staged in shared
//                  memory) or per 64 atoms of a single-cell box (all atoms, minimum image): every
//                  pair within cutoff + skin that is not excluded, in a fixed order, into the lists
//   8. ff_force_list  one thread per atom (all systems): its list, pairs within the cutoff, no
//                  atomics; forces written as OpenMM fixed point (2^32) to the slot; the pair terms
//                  are summed in the list's order, which a call fixes at its first evaluation
//   9. ff_energy   (energy evaluations only) one block per system: fixed-order FP64 sum.
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

// 1. Current positions in the order of the last build, and the rebuild test. The list order of a
// system is fixed between its builds, so the p-th entry stays the same atom (cell_list[p]).
__global__ void ff_check(FFDev D, DevBuf B, int prec) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.n_int) return;
    const int s = D.isys[p];  // list positions [i0, i1) belong to system s, as the atom indices do
    const FFSys S = D.sys[s];
    const int k = D.cell_list[p];
    const float3 x = wrap_box(atom_position(B, prec, D.iatom[k]), S);
    float4 c = D.cpos[p];
    c.x = x.x;
    c.y = x.y;
    c.z = x.z;
    D.cpos[p] = c;
    if (D.rebuild[s]) return;
    const float4 r = D.xref[p];
    const float3 d = min_image(x.x - r.x, x.y - r.y, x.z - r.z, S);
    if (fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)) > S.half_skin2) D.rebuild[s] = 1;
}

__global__ void ff_bin(FFDev D, DevBuf B, int prec) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= D.n_int) return;
    const int s = D.isys[k];
    if (!D.rebuild[s]) return;
    const FFSys S = D.sys[s];
    if (S.nc == 1) {
        D.cell_of[k] = S.c0;
        return;
    }
    const float3 x = atom_position(B, prec, D.iatom[k]);
    const int cx = wrap_cell(x.x, S.invL, S.nc), cy = wrap_cell(x.y, S.invL, S.nc), cz = wrap_cell(x.z, S.invL, S.nc);
    const int c = S.c0 + (cz * S.nc + cy) * S.nc + cx;
    D.cell_of[k] = c;
    atomicAdd(D.cell_count + c, 1);
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
            D.cell_start[S.c0] = S.i0;
            D.cell_start[S.c0 + 1] = S.i1;
        }
        return;
    }
    int base = S.i0;
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
    if (threadIdx.x == 0) D.cell_start[S.c0 + ncell] = base;  // equals S.i1
}

__global__ void ff_scatter(FFDev D) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= D.n_int) return;
    const int s = D.isys[k];
    if (!D.rebuild[s]) return;
    if (D.sys[s].nc == 1) {
        D.cell_list[k] = k;  // one cell: interacting-atom order
        return;
    }
    const int p = atomicAdd(D.cell_cursor + D.cell_of[k], 1);
    D.cell_list[p] = k;
}

// Sort each cell of a multi-cell box by interacting-atom index, so that every cell, and so every
// list, is in a fixed order. One warp per cell: the cell is staged in shared memory and each lane
// ranks its entries against all of them (the entries are distinct, so the ranks are a
// permutation); a cell larger than the stage falls back to an insertion sort by one lane. The one
// cell of a single-cell box is already in order.
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

// Cell-ordered copies (rebuilt systems): position wrapped into [0, L) and scaled charge; sigma/2,
// sqrt(epsilon), body id and device slot; the build positions.
__global__ void ff_gather(FFDev D, DevBuf B, int prec) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.n_int) return;
    const int s = D.isys[p];
    if (!D.rebuild[s]) return;
    const int k = D.cell_list[p];
    const int slot = D.iatom[k];
    const float3 x = wrap_box(atom_position(B, prec, slot), D.sys[s]);
    const float4 q = D.param[k];  // scaled charge, sigma/2, sqrt(eps), body id bits
    const float4 c = make_float4(x.x, x.y, x.z, D.ntypes ? __int_as_float(D.atype[k]) : q.x);
    D.cpos[p] = c;
    D.xref[p] = c;
    D.cpar[p] = make_float4(q.y, q.z, q.w, __int_as_float(slot));
}

// Excluded pairs: the atom itself (same slot) and atoms of the same rigid body. Ids are compared
// as integers: as floats they are denormals, which flush-to-zero arithmetic would make all equal.
__device__ __forceinline__ bool excluded(float4 pi, float4 pq) {
    if (__float_as_int(pi.w) == __float_as_int(pq.w)) return true;
    const int body = __float_as_int(pi.z);
    return body > 0 && __float_as_int(pq.z) == body;
}

// Appends neighbour j (list position) to atom p's list; a full list marks the system as failed
// (the capacity is sized from the densest system with a wide margin, so this does not happen in a
// liquid).
template <class IDX>
__device__ __forceinline__ void list_append(const FFDev& D, int p, int s, int i0, int& n, int j) {
    if (n < D.cap) {
        IDX* nb = (IDX*)D.nbr + (size_t)(p >> 5) * 32 * D.cap + (p & 31);
        nb[(size_t)n * 32] = (IDX)(j - i0);
    } else if (n == D.cap && D.sys_status) {
        atomicOr(D.sys_status + s, 2u);
    }
    n++;
}

// 7a. Lists of multi-cell boxes: one block per cell; its atoms kFC at a time, each of the 27
// neighbour cells staged in shared memory kFC atoms at a time with its periodic image shift applied
// once (exact for pairs within cutoff + skin: the cell edge is at least that and there are at
// least three cells per edge).
template <int kFC, class IDX>
__global__ void __launch_bounds__(kFC) ff_build_cells(FFDev D) {
    __shared__ float4 sx[kFC], sp[kFC];
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
        const float4 xi = mine ? D.cpos[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 pi = mine ? D.cpar[p] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
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
                            float4 a = D.cpos[j0 + t];
                            a.x += shx;
                            a.y += shy;
                            a.z += shz;
                            sx[t] = a;
                            sp[t] = D.cpar[j0 + t];
                        }
                        __syncthreads();
                        if (mine) {
                            const int m = min(kFC, qe - j0);
                            for (int j = 0; j < m; j++) {
                                const float4 xq = sx[j];
                                const float dx = xi.x - xq.x, dy = xi.y - xq.y, dz = xi.z - xq.z;
                                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                if (r2 < S.rl2 && !excluded(pi, sp[j])) list_append<IDX>(D, p, s, S.i0, n, j0 + j);
                            }
                        }
                    }
                }
            }
        }
        if (mine) D.ncnt[p] = min(n, D.cap);
    }
}

// 7b. Lists of single-cell boxes (fewer than three list cells per edge): one block per 64 atoms, all
// atoms of the box streamed through shared memory, minimum image per pair.
constexpr int kBT = 64;
template <class IDX>
__global__ void __launch_bounds__(kBT) ff_build_box(FFDev D) {
    __shared__ float4 sx[kBT], sp[kBT];
    const int s = D.sc_sys[blockIdx.x];
    if (!D.rebuild[s]) return;
    const FFSys S = D.sys[s];
    const int t = threadIdx.x;
    const int p = D.sc_i0[blockIdx.x] + t;
    const bool mine = p < S.i1;
    const float4 xi = mine ? D.cpos[p] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pi = mine ? D.cpar[p] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    int n = 0;
    for (int j0 = S.i0; j0 < S.i1; j0 += kBT) {
        __syncthreads();
        if (j0 + t < S.i1) {
            sx[t] = D.cpos[j0 + t];
            sp[t] = D.cpar[j0 + t];
        }
        __syncthreads();
        if (mine) {
            const int m = min(kBT, S.i1 - j0);
            for (int j = 0; j < m; j++) {
                const float4 xq = sx[j];
                const float3 d = min_image(xi.x - xq.x, xi.y - xq.y, xi.z - xq.z, S);
                const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
                if (r2 < S.rl2 && !excluded(pi, sp[j])) list_append<IDX>(D, p, s, S.i0, n, j0 + j);
            }
        }
    }
    if (mine) D.ncnt[p] = min(n, D.cap);
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

// 8. Forces from the lists: one thread per atom (list position p), its entries in list order; a
// pair beyond the cutoff adds exactly nothing (its term is selected to zero, so the loop does not
// diverge). The pair term is OpenMM's CutoffPeriodic form: reaction-field Coulomb and unshifted LJ.
template <bool ENERGY, class IDX, bool TYPED>
__global__ void __launch_bounds__(128) ff_force_list(FFDev D, long long* __restrict__ force, int stride) {
    __shared__ float4 stype[TYPED ? kMaxTypesDev : 1];
    if (TYPED) {
        for (int t = threadIdx.x; t < D.ntypes; t += blockDim.x) stype[t] = D.types[t];
        __syncthreads();
    }
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.n_int) return;
    const int s = D.isys[p];
    const FFSys S = D.sys[s];
    const float4 xi = D.cpos[p];
    const float4 pi = D.cpar[p];
    const float qi = TYPED ? stype[__float_as_int(xi.w)].x : xi.w;
    const int n = D.ncnt[p];
    const IDX* __restrict__ nb = (const IDX*)D.nbr + (size_t)(p >> 5) * 32 * D.cap + (p & 31);
    const float4* __restrict__ cpos = D.cpos + S.i0;
    const float4* __restrict__ cpar = D.cpar + S.i0;
    const bool relax = D.fcap > 0.0f;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    ESum en;
    // one neighbour's term; `valid` false adds exactly nothing (padding of the last group of loads)
    auto pair = [&](float4 xq, float2 pq, bool valid) {
        float qj, sj, ej;
        if (TYPED) {  // one 16-byte record per neighbour; parameters from the type table
            const float4 tq = stype[__float_as_int(xq.w)];
            qj = tq.x;
            sj = tq.y;
            ej = tq.z;
        } else {
            qj = xq.w;
            sj = pq.x;
            ej = pq.y;
        }
        const float3 d = min_image(xi.x - xq.x, xi.y - xq.y, xi.z - xq.z, S);
        const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
        // relaxation: coincident atoms have no direction
        const bool in = valid && r2 < S.rc2 && !(relax && r2 < 1e-8f);
        const float r2s = in ? r2 : 1.0f;
        const float inv_r = rsqrtf(r2s), inv_r2 = inv_r * inv_r;
        const float qq = qi * qj;
        const float sig = pi.x + sj, eps = pi.y * ej;
        const float s2 = sig * sig * inv_r2, s6 = s2 * s2 * s2;
        float g = qq * (inv_r * inv_r2 - 2.0f * S.krf) + 4.0f * eps * (12.0f * s6 * s6 - 6.0f * s6) * inv_r2;
        g = in ? g : 0.0f;
        fx = fmaf(g, d.x, fx);
        fy = fmaf(g, d.y, fy);
        fz = fmaf(g, d.z, fz);
        if (ENERGY && in) en.add(qq * (inv_r + S.krf * r2 - S.crf) + 4.0f * eps * (s6 * s6 - s6));
    };
    // groups of kU entries: all of a group's index and neighbour loads are issued before its terms
    // are formed (in entry order), so that the dependent index -> position loads overlap
    constexpr int kU = 4;
    for (int e0 = 0; e0 < n; e0 += kU) {
        int jj[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) jj[u] = e0 + u < n ? (int)nb[(size_t)(e0 + u) * 32] : 0;
        float4 xq[kU];
        float2 pq[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            xq[u] = cpos[jj[u]];
            pq[u] = TYPED ? make_float2(0.f, 0.f) : *(const float2*)(cpar + jj[u]);
        }
        // the group's records are all loaded before the first term (the loads are in flight together)
        asm volatile("" ::"f"(xq[0].x), "f"(xq[1].x), "f"(xq[2].x), "f"(xq[3].x));
#pragma unroll
        for (int u = 0; u < kU; u++) pair(xq[u], pq[u], e0 + u < n);
    }
    const int k = D.cell_list[p];
    store_force<ENERGY>(D, force, stride, k, __float_as_int(pi.w), fx, fy, fz, en, s);
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
    const int t = 256, g = (D.n_int + t - 1) / t;
    int n = 0;
    ff_check<<<g, t, 0, st>>>(D, B, prec);
    ff_bin<<<g, t, 0, st>>>(D, B, prec);
    ff_scan<<<D.S, 256, 0, st>>>(D);
    ff_scatter<<<g, t, 0, st>>>(D);
    n += 4;
    if (D.n_mc) {
        ff_sort<<<(D.n_mc + kSortWarps - 1) / kSortWarps, 32 * kSortWarps, 0, st>>>(D);
        n++;
    }
    ff_gather<<<g, t, 0, st>>>(D, B, prec);
    n++;
    // list builds: block size of the cell kernel chosen by the autotuner (results do not depend
    // on it: every list is built in the same order)
    if (D.n_mc) {
        if (D.nbr16) {
            switch (D.cell_threads) {
                case 64: ff_build_cells<64, unsigned short><<<D.n_mc, 64, 0, st>>>(D); break;
                case 256: ff_build_cells<256, unsigned short><<<D.n_mc, 256, 0, st>>>(D); break;
                default: ff_build_cells<128, unsigned short><<<D.n_mc, 128, 0, st>>>(D);
            }
        } else {
            switch (D.cell_threads) {
                case 64: ff_build_cells<64, unsigned int><<<D.n_mc, 64, 0, st>>>(D); break;
                case 256: ff_build_cells<256, unsigned int><<<D.n_mc, 256, 0, st>>>(D); break;
                default: ff_build_cells<128, unsigned int><<<D.n_mc, 128, 0, st>>>(D);
            }
        }
        n++;
    }
    if (D.n_sc) {
        if (D.nbr16) ff_build_box<unsigned short><<<D.n_sc, kBT, 0, st>>>(D);
        else ff_build_box<unsigned int><<<D.n_sc, kBT, 0, st>>>(D);
        n++;
    }
    if (cudaMemsetAsync(D.rebuild, 0, (size_t)D.S, st) != cudaSuccess) return -1;
    long long* f = const_cast<long long*>(B.force);
    const int gf = (D.n_int + 127) / 128;
    const bool typed = D.ntypes > 0 && D.ntypes <= kMaxTypesDev;
#define RBX_FORCE_LIST(E, I, T) ff_force_list<E, I, T><<<gf, 128, 0, st>>>(D, f, B.stride)
    if (D.nbr16) {
        if (typed) { if (energy) RBX_FORCE_LIST(true, unsigned short, true); else RBX_FORCE_LIST(false, unsigned short, true); }
        else { if (energy) RBX_FORCE_LIST(true, unsigned short, false); else RBX_FORCE_LIST(false, unsigned short, false); }
    } else {
        if (typed) { if (energy) RBX_FORCE_LIST(true, unsigned int, true); else RBX_FORCE_LIST(false, unsigned int, true); }
        else { if (energy) RBX_FORCE_LIST(true, unsigned int, false); else RBX_FORCE_LIST(false, unsigned int, false); }
    }
#undef RBX_FORCE_LIST
    n++;
    if (energy) {
        ff_energy<<<D.S, 256, 0, st>>>(D);
        n++;
    }
    return cudaPeekAtLastError() == cudaSuccess ? n : -1;
}

}  // namespace rbx
