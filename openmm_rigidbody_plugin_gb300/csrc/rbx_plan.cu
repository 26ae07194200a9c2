// rbx_plan.cu -- re-planning the library order on the device after atoms move to new device
// slots (the ReorderListener of platforms/cuda/src/CudaRigidBodyKernels.cpp:69-113, which OpenMM
// triggers whenever CudaContext::reorderAtoms permutes the atoms).
//
// The library keeps bodies in ascending order of the lowest slot of their atoms and free atoms in
// ascending slot order, so that a tile's atoms occupy a narrow slot range. Every key is a distinct
// slot, so the sort is a counting sort over slot space: each body marks the slot of its key and
// each free atom its own slot, and an exclusive scan of the marks compacts them in slot order.
// The per-body and per-atom arrays then move to the new order with plain gathers, bit for bit.
// Only the greedy packing of bodies into tiles, a sequential O(nb) pass, stays on the host.
#include <cuda_runtime.h>

#include "rbx_internal.h"

namespace rbx {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // items per thread
constexpr int kScanBlock = kScanThreads * kScanItems;

// Slots must be non-negative (checked on the host) and distinct: a slot seen twice sets status.
__global__ void check_slots_kernel(const int* __restrict__ loc, int n, unsigned int* seen, int* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = loc[i];
    const unsigned int bit = 1u << (s & 31);
    if (atomicOr(seen + (s >> 5), bit) & bit) atomicOr(status, 1);
}

// Each body marks the lowest slot of its atoms with its reference index.
__global__ void body_keys_kernel(const int* __restrict__ ref_first, const int* __restrict__ ref_atoms,
                                 const int* __restrict__ loc, int nb, int* mark) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    int key = 0x7fffffff;
    for (int k = ref_first[b]; k < ref_first[b + 1]; k++) key = min(key, loc[ref_atoms[k]]);
    mark[key] = b;
}

// Each free atom marks its slot with its user index.
__global__ void free_marks_kernel(const int* __restrict__ free_atoms, int nf, const int* __restrict__ loc, int* mark) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nf) mark[loc[free_atoms[j]]] = free_atoms[j];
}

__global__ void flags_kernel(const int* __restrict__ mark, int n, int* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = mark[i] >= 0 ? 1 : 0;
}

// Exclusive scan of kScanBlock items per block in place; the block's total goes to sums.
__global__ void __launch_bounds__(kScanThreads) scan_block_kernel(int* data, int n, int* sums) {
    __shared__ int warp_tot[kScanThreads / 32];
    const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    int v[kScanItems], t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? data[base + k] : 0;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = t;  // inclusive scan of the thread totals within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    int run = x - t + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = warp_tot[31];
}

__global__ void scan_add_kernel(int* data, int n, const int* __restrict__ offsets) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += offsets[i / kScanBlock];
}

// Marked entries, in index order, to out[position].
__global__ void compact_kernel(const int* __restrict__ mark, const int* __restrict__ pos, int n, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && mark[i] >= 0) out[pos[i]] = mark[i];
}

// New inverse map, the source position of each body, and body sizes (scanned into atom0_new).
__global__ void inverse_sizes_kernel(PlanMaps M) {
    const int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L > M.nb) return;
    if (L == M.nb) {
        M.atom0_new[M.nb] = 0;
        return;
    }
    const int b = M.lib_body_new[L];
    M.lib_pos_new[b] = L;
    M.idx_body[L] = M.lib_pos_old[b];
    M.atom0_new[L] = M.ref_first[b + 1] - M.ref_first[b];
}

// Per body of the new order: where each of its body atoms came from, and its slot.
__global__ void atom_maps_kernel(PlanMaps M) {
    const int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= M.nb) return;
    const int b = M.lib_body_new[L];
    const int k0 = M.atom0_new[L], k1 = M.atom0_new[L + 1], kold = M.atom0_old[M.lib_pos_old[b]];
    const int r0 = M.ref_first[b];
    for (int j = 0; j < k1 - k0; j++) {
        M.idx_atom[k0 + j] = kold + j;
        M.atom_loc_new[k0 + j] = M.loc[M.ref_atoms[r0 + j]];
    }
}

__global__ void free_maps_kernel(PlanMaps M) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M.nf) return;
    const int u = M.free_new[j];
    M.idx_free[j] = M.free_index_old[u];
    M.free_loc_new[j] = M.loc[u];
}

__global__ void free_index_kernel(const int* __restrict__ free_new, int nf, int* free_index) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nf) free_index[free_new[j]] = j;
}

template <class E>
__global__ void gather_rows_kernel(E* __restrict__ dst, const E* __restrict__ src, int rows, size_t ld, int n,
                                   const int* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (i < n && r < rows) dst[r * ld + i] = src[r * ld + idx[i]];
}

inline int grid(long long n, int t) { return (int)((n + t - 1) / t); }
inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 0 : -1; }

}  // namespace

size_t scan_aux_len(int n) {
    size_t len = 0;
    for (long long m = n; m > 1; m = (m + kScanBlock - 1) / kScanBlock) len += (size_t)((m + kScanBlock - 1) / kScanBlock) + 1;
    return len + 1;
}

int device_exclusive_scan(int* data, int n, int* aux, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n <= 0) return 0;
    const int nblk = grid(n, kScanBlock);
    scan_block_kernel<<<nblk, kScanThreads, 0, st>>>(data, n, aux);
    if (ok()) return -1;
    if (nblk == 1) return 0;
    if (device_exclusive_scan(aux, nblk, aux + nblk, stream)) return -1;
    scan_add_kernel<<<grid(n, 256), 256, 0, st>>>(data, n, aux);
    return ok();
}

int launch_plan_order(const PlanOrder& P, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(P.seen, 0, sizeof(unsigned int) * (size_t)((P.nslots + 31) / 32), st) != cudaSuccess ||
        cudaMemsetAsync(P.status, 0, sizeof(int), st) != cudaSuccess ||
        cudaMemsetAsync(P.mark_body, 0xff, sizeof(int) * (size_t)P.nslots, st) != cudaSuccess ||
        cudaMemsetAsync(P.mark_free, 0xff, sizeof(int) * (size_t)P.nslots, st) != cudaSuccess)
        return -1;
    check_slots_kernel<<<grid(P.natoms, 256), 256, 0, st>>>(P.loc, P.natoms, P.seen, P.status);
    if (P.nb) body_keys_kernel<<<grid(P.nb, 256), 256, 0, st>>>(P.ref_first, P.ref_atoms, P.loc, P.nb, P.mark_body);
    if (P.nf) free_marks_kernel<<<grid(P.nf, 256), 256, 0, st>>>(P.free_old, P.nf, P.loc, P.mark_free);
    if (ok()) return -1;
    // With a duplicated slot the marks of two owners collide and the compaction would write fewer
    // entries than expected; the outputs are then left as they are and the caller reads status.
    const int* marks[2] = {P.mark_body, P.mark_free};
    int* outs[2] = {P.lib_body_new, P.free_new};
    const int counts[2] = {P.nb, P.nf};
    for (int k = 0; k < 2; k++) {
        if (!counts[k]) continue;
        flags_kernel<<<grid(P.nslots, 256), 256, 0, st>>>(marks[k], P.nslots, P.scan);
        if (ok() || device_exclusive_scan(P.scan, P.nslots, P.aux, stream)) return -1;
        compact_kernel<<<grid(P.nslots, 256), 256, 0, st>>>(marks[k], P.scan, P.nslots, outs[k]);
        if (ok()) return -1;
    }
    return 0;
}

int launch_plan_maps(const PlanMaps& M, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (M.nb) {
        inverse_sizes_kernel<<<grid(M.nb + 1, 256), 256, 0, st>>>(M);
        if (ok() || device_exclusive_scan(M.atom0_new, M.nb + 1, M.aux, stream)) return -1;
        atom_maps_kernel<<<grid(M.nb, 128), 128, 0, st>>>(M);
    }
    if (M.nf) {
        free_maps_kernel<<<grid(M.nf, 256), 256, 0, st>>>(M);
        free_index_kernel<<<grid(M.nf, 256), 256, 0, st>>>(M.free_new, M.nf, M.free_index_new);
    }
    return ok();
}

int launch_gather_rows(void* dst, const void* src, int rows, size_t ld, int n, const int* idx, int elem_bytes,
                       void* stream) {
    if (n <= 0 || rows <= 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const dim3 g(grid(n, 256), rows);
    switch (elem_bytes) {
        case 1: gather_rows_kernel<unsigned char><<<g, 256, 0, st>>>((unsigned char*)dst, (const unsigned char*)src, rows, ld, n, idx); break;
        case 4: gather_rows_kernel<int><<<g, 256, 0, st>>>((int*)dst, (const int*)src, rows, ld, n, idx); break;
        case 8: gather_rows_kernel<long long><<<g, 256, 0, st>>>((long long*)dst, (const long long*)src, rows, ld, n, idx); break;
        default: return -1;
    }
    return ok();
}

}  // namespace rbx
