// rbx_refined.cu -- refined ("shadow") energies: the step kernels that also accumulate the
// refined-energy stencils (the COMPMOD == 1 build of platforms/cuda/src/kernels/
// rigidbodyintegrator.cu, switched on by RigidBodyIntegrator::setComputeRefinedEnergies,
// openmmapi/src/RigidBodyIntegrator.cpp:34-38), and the sum of their per-body and per-free-atom
// terms.
//
// After part2 of step n (time t+h), each body and free atom has written to ref_out its correction
// of the translational and rotational kinetic energy and its |F|^2/m + tau.I^-1.tau. The host adds
// the corrections' sums to the plain kinetic energies and scales the last sum by -h^2/24
// (CudaRigidBodyKernels.cpp:118-194, :469-494). The kernels write corrections rather than the
// refined energies themselves so that the FP32 kernels lose nothing to cancellation: the plain
// energies come from the FP64 kinetic-energy reduction.
#include <cuda_runtime.h>

#include "rbx_internal.h"
#include "rbx_step.cuh"

namespace rbx {

namespace {

constexpr int kRefThreads = 256;

// [sum KE_t corrections, sum KE_r corrections, sum |F|^2/m + tau.I^-1.tau] in FP64, fixed order:
// strided per-thread sums, a tree per block, and the last block to finish adds the block sums.
__global__ void __launch_bounds__(kRefThreads) refined_sum_kernel(DevSys S, RefScratch K) {
    __shared__ double sh[3][kRefThreads];
    __shared__ bool s_last;
    const int nbp = S.nb_pad, nfp = S.nf_pad;
    const float* o = S.ref_out;
    const float* f = o + 3 * (size_t)nbp;
    double t = 0.0, r = 0.0, u = 0.0;
    const int gsize = gridDim.x * blockDim.x;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < S.nb; b += gsize) {
        t += (double)o[b];
        r += (double)o[b + nbp];
        u += (double)o[b + 2 * nbp];
    }
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < S.nf; j += gsize) {
        t += (double)f[j];
        u += (double)f[j + nfp];
    }
    sh[0][threadIdx.x] = t;
    sh[1][threadIdx.x] = r;
    sh[2][threadIdx.x] = u;
    __syncthreads();
    for (int w = kRefThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < 3; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; k++) K.partial[3 * blockIdx.x + k] = sh[k][0];
        __threadfence();
        const unsigned int ticket = atomicAdd(K.count, 1u);
        s_last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        double acc[3] = {0.0, 0.0, 0.0};
        for (unsigned int i = 0; i < gridDim.x; i++)
            for (int k = 0; k < 3; k++) acc[k] += ((volatile double*)K.partial)[3 * i + k];
        for (int k = 0; k < 3; k++) K.out[k] = acc[k];
        *K.count = 0u;
    }
}

}  // namespace

int launch_step_refined(int prec, int kind, const DevSys& s, const DevBuf& b, double dt, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    switch (prec) {
        case PREC_SINGLE: return launch_step_p<PREC_SINGLE, true>(kind, s, b, dt, st);
        case PREC_MIXED: return launch_step_p<PREC_MIXED, true>(kind, s, b, dt, st);
        default: return launch_step_p<PREC_DOUBLE, true>(kind, s, b, dt, st);
    }
}

int refined_blocks(const DevSys& s) {
    const int n = s.nb > s.nf ? s.nb : s.nf;
    int blocks = (n + kRefThreads - 1) / kRefThreads;
    if (blocks > 4 * 152) blocks = 4 * 152;
    return blocks < 1 ? 1 : blocks;
}

int launch_refined_sum(const DevSys& s, const RefScratch& k, int n_blocks, void* stream) {
    refined_sum_kernel<<<n_blocks, kRefThreads, 0, (cudaStream_t)stream>>>(s, k);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace rbx
