// rbx_forces.cu -- cutoff Lennard-Jones + reaction-field forces for many independent periodic
// systems, by cell lists (the force provider of the batched and served forms; the drop-in takes
// its forces from the OpenMM Context instead).
//
// Functional form: OpenMM NonbondedForce, CutoffPeriodic method, as documented by OpenMM
//   E = K q_i q_j (1/r + k_rf r^2 - c_rf) + 4 eps_ij ((sig_ij/r)^12 - (sig_ij/r)^6),  r < rc,
// Lorentz-Berthelot combination, minimum image in a cubic box, pairs of one rigid body excluded.
//
// One evaluation, all systems at once:
//   1. ff_bin      one thread per interacting atom: cell index, cell counts
//   2. ff_scan     one block per system: exclusive scan of its cells' counts (and count reset)
//   3. ff_scatter  one thread per interacting atom: slot in its cell (single-cell systems keep
//                  their atom order and need no atomics)
//   4. ff_sort     one thread per cell of a multi-cell box: sorts the cell by atom index (the
//                  cell contents, and so every force sum, are in a fixed order)
//   5. ff_gather   one thread per atom: cell-ordered copies of positions (wrapped into the box)
//                  and parameters, so that neighbour loads are contiguous
//   6. ff_force_cells / ff_force_box  one block per cell (multi-cell boxes) or per 64 atoms of a
//                  single-cell box: neighbour atoms staged in shared memory, all pairs within the
//                  cutoff, no atomics; forces written as OpenMM fixed point (2^32) to the slot
//   7. ff_energy   (energy evaluations only) one block per system: fixed-order FP64 sum.
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

__global__ void ff_bin(FFDev D, DevBuf B, int prec) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= D.n_int) return;
    const FFSys S = D.sys[D.isys[k]];
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
    const FFSys S = D.sys[D.isys[k]];
    if (S.nc == 1) {
        D.cell_list[k] = k;  // one cell: interacting-atom order
        return;
    }
    const int p = atomicAdd(D.cell_cursor + D.cell_of[k], 1);
    D.cell_list[p] = k;
}

// Sort each cell of a multi-cell box by interacting-atom index, so that every cell, and so every
// force sum, is in a fixed order. One warp per cell: the cell is staged in shared memory and each
// lane ranks its entries against all of them (the entries are distinct, so the ranks are a
// permutation); a cell larger than the stage falls back to an insertion sort by one lane. The one
// cell of a single-cell box is already in order.
constexpr int kSortWarps = 4, kSortStage = 512;
__global__ void __launch_bounds__(32 * kSortWarps) ff_sort(FFDev D) {
    __shared__ int stage[kSortWarps][kSortStage];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * kSortWarps + warp;
    if (w >= D.n_mc) return;
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

// Cell-ordered copies: position wrapped into [0, L) and scaled charge; sigma/2, sqrt(epsilon), body
// id and device slot.
__global__ void ff_gather(FFDev D, DevBuf B, int prec) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.n_int) return;
    const int k = D.cell_list[p];
    const int slot = D.iatom[k];
    const FFSys S = D.sys[D.isys[k]];
    float3 x = atom_position(B, prec, slot);
    x.x -= S.L * floorf(x.x * S.invL);
    x.y -= S.L * floorf(x.y * S.invL);
    x.z -= S.L * floorf(x.z * S.invL);
    const float4 q = D.param[k];  // scaled charge, sigma/2, sqrt(eps), body id bits
    D.cpos[p] = make_float4(x.x, x.y, x.z, q.x);
    D.cpar[p] = make_float4(q.y, q.z, q.w, __int_as_float(slot));
}

constexpr int kFT = 64;  // threads of a single-box force block; also its staged chunk of atoms

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

// The pair's force on i and (energy evaluations) its energy, formed in FP32 and summed with
// compensation, for a pair known to be within the cutoff and not excluded.
template <bool ENERGY>
__device__ __forceinline__ void pair_interact(const FFSys& S, const FFDev& D, float4 xi, float4 pi, float4 xq, float4 pq,
                                              float dx, float dy, float dz, float r2, float& fx, float& fy, float& fz,
                                              ESum& e) {
    if (D.fcap > 0.0f && r2 < 1e-8f) return;  // relaxation: coincident atoms have no direction
    const float inv_r2 = 1.0f / r2, inv_r = rsqrtf(r2);
    const float qq = xi.w * xq.w;
    const float sig = pi.x + pq.x, eps = pi.y * pq.y;
    const float s2 = sig * sig * inv_r2, s6 = s2 * s2 * s2;
    const float g = qq * (inv_r * inv_r2 - 2.0f * S.krf) + 4.0f * eps * (12.0f * s6 * s6 - 6.0f * s6) * inv_r2;
    fx = fmaf(g, dx, fx);
    fy = fmaf(g, dy, fy);
    fz = fmaf(g, dz, fz);
    if (ENERGY) e.add(qq * (inv_r + S.krf * r2 - S.crf) + 4.0f * eps * (s6 * s6 - s6));
}

// Excluded pairs: the atom itself (same slot) and atoms of the same rigid body. Ids are compared
// as integers: as floats they are denormals, which flush-to-zero arithmetic would make all equal.
__device__ __forceinline__ bool excluded(float4 pi, float4 pq) {
    if (__float_as_int(pi.w) == __float_as_int(pq.w)) return true;
    const int body = __float_as_int(pi.z);
    return body > 0 && __float_as_int(pq.z) == body;
}

// Cell kernel (many warps per SM): the cutoff test first, and the neighbour's parameters read from
// shared memory only for pairs within it (about 15 % of the candidates of 27 cells).
template <bool ENERGY>
__device__ __forceinline__ void pair_term_cutoff_first(const FFSys& S, const FFDev& D, float4 xi, float4 pi, float4 xq,
                                                       const float4* __restrict__ pqp, float dx, float dy, float dz,
                                                       float& fx, float& fy, float& fz, ESum& e) {
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (r2 >= S.rc2) return;
    const float4 pq = *pqp;
    if (excluded(pi, pq)) return;
    pair_interact<ENERGY>(S, D, xi, pi, xq, pq, dx, dy, dz, r2, fx, fy, fz, e);
}

// Single-box kernel (few warps, each thread a long loop): the parameters loaded with the position
// and the exclusions tested first keep the loop's dependent chain short (measured on 512 waters:
// 0.19 ms per evaluation against 0.25 ms with the cutoff test first).
template <bool ENERGY>
__device__ __forceinline__ void pair_term_exclusions_first(const FFSys& S, const FFDev& D, float4 xi, float4 pi,
                                                           float4 xq, float4 pq, float dx, float dy, float dz,
                                                           float& fx, float& fy, float& fz, ESum& e) {
    if (excluded(pi, pq)) return;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (r2 >= S.rc2) return;
    pair_interact<ENERGY>(S, D, xi, pi, xq, pq, dx, dy, dz, r2, fx, fy, fz, e);
}

template <bool ENERGY>
__device__ __forceinline__ void store_force(const FFDev& D, long long* __restrict__ force, int stride, int p, float4 pi,
                                            float fx, float fy, float fz, const ESum& e) {
    if (D.fcap > 0.0f) {  // relaxation: cap the magnitude
        const float f2 = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
        if (f2 > D.fcap * D.fcap) {
            const float s = D.fcap * rsqrtf(f2);
            fx *= s;
            fy *= s;
            fz *= s;
        }
    }
    // keep each component inside the 2^32 fixed-point range (|F| < 2^31 kJ/mol/nm)
    const float kMaxF = 2.0e9f;
    fx = fminf(fmaxf(fx, -kMaxF), kMaxF);
    fy = fminf(fmaxf(fy, -kMaxF), kMaxF);
    fz = fminf(fmaxf(fz, -kMaxF), kMaxF);
    const int slot = __float_as_int(pi.w);
    force[slot] = __float2ll_rn(fx * 0x1p32f);
    force[slot + stride] = __float2ll_rn(fy * 0x1p32f);
    force[slot + 2 * stride] = __float2ll_rn(fz * 0x1p32f);
    if (ENERGY) D.e_atom[p] = 0.5 * e.value();
}

// Multi-cell boxes: one block per cell. The block's kFC threads take the cell's atoms (kFC at a
// time: 64, 128 or 256, chosen by the batch's autotuner; a cell of at least a cutoff per edge
// holds 73 or more atoms at liquid density); each of the 27 neighbour cells is staged in shared
// memory, kFC atoms at a time, with its periodic
// image shift applied once (exact for pairs within the cutoff: the cell edge is at least the
// cutoff and there are at least three cells per edge).
template <bool ENERGY, int kFC>
__global__ void __launch_bounds__(kFC) ff_force_cells(FFDev D, long long* __restrict__ force, int stride) {
    __shared__ float4 sx[kFC], sp[kFC];
    const int c = D.mc_cell[blockIdx.x];
    const FFSys S = D.sys[D.mc_sys[blockIdx.x]];
    const int b = D.cell_start[c], e = D.cell_start[c + 1];
    const int local = c - S.c0, nc = S.nc;
    const int cx = local % nc, cy = (local / nc) % nc, cz = local / (nc * nc);
    const int t = threadIdx.x;
    for (int i0 = b; i0 < e; i0 += kFC) {
        const int p = i0 + t;
        const bool mine = p < e;
        const float4 xi = mine ? D.cpos[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 pi = mine ? D.cpar[p] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        float fx = 0.f, fy = 0.f, fz = 0.f;
        ESum en;
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
                    const int n = S.c0 + (z * nc + y) * nc + x;
                    const int qb = D.cell_start[n], qe = D.cell_start[n + 1];
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
                                pair_term_cutoff_first<ENERGY>(S, D, xi, pi, xq, sp + j, xi.x - xq.x, xi.y - xq.y,
                                                               xi.z - xq.z, fx, fy, fz, en);
                            }
                        }
                    }
                }
            }
        }
        if (mine) store_force<ENERGY>(D, force, stride, p, pi, fx, fy, fz, en);
    }
}

// Single-cell boxes (fewer than three cutoffs across): one block per 64 atoms of the box, all
// atoms of the box streamed through shared memory, minimum image per pair. Each atom has kFK
// threads (consecutive lanes), each taking every kFK-th staged neighbour; their partial sums are
// combined by a fixed butterfly of shuffles, so the order of every sum is fixed. Small boxes are
// latency bound: kFK threads per atom give kFK times the parallelism and 1/kFK of the loop.
constexpr int kFK = 8;
template <bool ENERGY>
__global__ void __launch_bounds__(kFT * kFK) ff_force_box(FFDev D, long long* __restrict__ force, int stride) {
    constexpr int NT = kFT * kFK;  // threads, and staged neighbours per barrier pair
    __shared__ float4 sx[NT], sp[NT];
    const FFSys S = D.sys[D.sc_sys[blockIdx.x]];
    const int t = threadIdx.x, k = t % kFK;
    const int p = D.sc_i0[blockIdx.x] + t / kFK;
    const bool mine = p < S.i1;
    const float4 xi = mine ? D.cpos[p] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pi = mine ? D.cpar[p] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    float fx = 0.f, fy = 0.f, fz = 0.f;
    ESum en;
    for (int j0 = S.i0; j0 < S.i1; j0 += NT) {
        __syncthreads();
        if (j0 + t < S.i1) {
            sx[t] = D.cpos[j0 + t];
            sp[t] = D.cpar[j0 + t];
        }
        __syncthreads();
        if (mine) {
            const int m = min(NT, S.i1 - j0);
            for (int j = k; j < m; j += kFK) {
                const float4 xq = sx[j];
                float dx = xi.x - xq.x, dy = xi.y - xq.y, dz = xi.z - xq.z;
                dx -= S.L * rintf(dx * S.invL);
                dy -= S.L * rintf(dy * S.invL);
                dz -= S.L * rintf(dz * S.invL);
                pair_term_exclusions_first<ENERGY>(S, D, xi, pi, xq, sp[j], dx, dy, dz, fx, fy, fz, en);
            }
        }
    }
#pragma unroll
    for (int o = kFK / 2; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
        if (ENERGY) {
            en.hi += __shfl_xor_sync(0xffffffffu, en.hi, o);
            en.lo += __shfl_xor_sync(0xffffffffu, en.lo, o);
        }
    }
    if (mine && k == 0) store_force<ENERGY>(D, force, stride, p, pi, fx, fy, fz, en);
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
    ff_bin<<<g, t, 0, st>>>(D, B, prec);
    ff_scan<<<D.S, 256, 0, st>>>(D);
    ff_scatter<<<g, t, 0, st>>>(D);
    n += 3;
    if (D.n_mc) {
        ff_sort<<<(D.n_mc + kSortWarps - 1) / kSortWarps, 32 * kSortWarps, 0, st>>>(D);
        n++;
    }
    ff_gather<<<g, t, 0, st>>>(D, B, prec);
    n++;
    long long* f = const_cast<long long*>(B.force);
    if (D.n_mc) {
        // block size: results do not depend on it (each atom's pairs are summed in the same order)
        switch (D.cell_threads) {
            case 64:
                if (energy) ff_force_cells<true, 64><<<D.n_mc, 64, 0, st>>>(D, f, B.stride);
                else ff_force_cells<false, 64><<<D.n_mc, 64, 0, st>>>(D, f, B.stride);
                break;
            case 256:
                if (energy) ff_force_cells<true, 256><<<D.n_mc, 256, 0, st>>>(D, f, B.stride);
                else ff_force_cells<false, 256><<<D.n_mc, 256, 0, st>>>(D, f, B.stride);
                break;
            default:
                if (energy) ff_force_cells<true, 128><<<D.n_mc, 128, 0, st>>>(D, f, B.stride);
                else ff_force_cells<false, 128><<<D.n_mc, 128, 0, st>>>(D, f, B.stride);
        }
        n++;
    }
    if (D.n_sc) {
        if (energy) ff_force_box<true><<<D.n_sc, kFT * kFK, 0, st>>>(D, f, B.stride);
        else ff_force_box<false><<<D.n_sc, kFT * kFK, 0, st>>>(D, f, B.stride);
        n++;
    }
    if (energy) {
        ff_energy<<<D.S, 256, 0, st>>>(D);
        n++;
    }
    return cudaPeekAtLastError() == cudaSuccess ? n : -1;
}

}  // namespace rbx
