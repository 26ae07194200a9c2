// rbx_kernels.cu -- sm_103a kernels of the rigid-body integrator: the plain step kernels
// (templates in rbx_step.cuh), kinetic energies, position rebuild from the body state, momentum
// scaling and the layout conversions of the host-buffer API.
// The kinetic-energy kernel reduces [KE_t, KE_r] in FP64 in a fixed order.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <mutex>

#include "../../include/rbx.h"

#include "rbx_fast.cuh"
#include "rbx_internal.h"
#include "rbx_math.cuh"
#include "rbx_step.cuh"

namespace rbx {
// ------------------------------------------------------------------------------------------
// Kinetic energy: [KE_t, KE_r] reduced in FP64, fixed order, last block finishes.
// ------------------------------------------------------------------------------------------
constexpr int kKEThreads = 256;

// Body state and constants of body b as FP64, for either state layout.
template <int P> struct BodyRead {
    static __device__ __forceinline__ void get(const DevSys& S, int b, V3<double>& v, Q4<double>& q, Q4<double>& pi,
                                               double& invm, V3<double>& invI) {
        const int nbp = S.nb_pad;
        if (P == PREC_DOUBLE) {
            const double* st = (const double*)S.state;
            v = v3<double>(st[b + 3 * nbp], st[b + 4 * nbp], st[b + 5 * nbp]);
            q = q4<double>(st[b + 6 * nbp], st[b + 7 * nbp], st[b + 8 * nbp], st[b + 9 * nbp]);
            pi = q4<double>(st[b + 10 * nbp], st[b + 11 * nbp], st[b + 12 * nbp], st[b + 13 * nbp]);
            invm = S.invm[b];
            invI = v3<double>(S.invI[b], S.invI[b + nbp], S.invI[b + 2 * nbp]);
        } else {
            const float* h = (const float*)S.state;
            const float* l = h + 14 * nbp;
            double x[14];
            for (int k = 3; k < 14; k++) x[k] = (double)h[b + k * nbp] + (double)l[b + k * nbp];
            v = v3<double>(x[3], x[4], x[5]);
            q = q4<double>(x[6], x[7], x[8], x[9]);
            pi = q4<double>(x[10], x[11], x[12], x[13]);
            const float* c = S.bconst;
            invm = (double)c[b] + (double)c[b + 7 * nbp];
            invI = v3<double>((double)c[b + nbp] + (double)c[b + 8 * nbp], (double)c[b + 2 * nbp] + (double)c[b + 9 * nbp],
                              (double)c[b + 3 * nbp] + (double)c[b + 10 * nbp]);
        }
    }
};

template <int P>
__global__ void __launch_bounds__(kKEThreads) kinetic_kernel(DevSys S, DevBuf B, KEScratch K) {
    using V4 = typename Tr<P>::V4;
    __shared__ double s_t[kKEThreads], s_r[kKEThreads];
    __shared__ bool s_last;
    double kt = 0.0, kr = 0.0;
    const int gsize = gridDim.x * blockDim.x;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < S.nb; b += gsize) {
        V3<double> v, invI;
        Q4<double> q, pi;
        double invm;
        BodyRead<P>::get(S, b, v, q, pi, invm, invI);
        V3<double> L = qBt(q, pi) * 0.5;
        kt += dot(v, v) / invm;
        kr += dot(L, mul(invI, L));
    }
    const V4* vel = (const V4*)B.velm;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < S.nf; j += gsize) {
        V4 vm = vel[S.free_loc[j]];
        double vx = vm.x, vy = vm.y, vz = vm.z;
        kt += (vx * vx + vy * vy + vz * vz) / (double)vm.w;
    }
    s_t[threadIdx.x] = kt;
    s_r[threadIdx.x] = kr;
    __syncthreads();
    for (int w = kKEThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s_t[threadIdx.x] += s_t[threadIdx.x + w];
            s_r[threadIdx.x] += s_r[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        K.partial[2 * blockIdx.x] = s_t[0];
        K.partial[2 * blockIdx.x + 1] = s_r[0];
        __threadfence();
        unsigned int ticket = atomicAdd(K.count, 1u);
        s_last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        double t = 0.0, r = 0.0;
        for (unsigned int i = 0; i < gridDim.x; i++) {
            t += ((volatile double*)K.partial)[2 * i];
            r += ((volatile double*)K.partial)[2 * i + 1];
        }
        K.out[0] = 0.5 * t;
        K.out[1] = 0.5 * r;
        *K.count = 0u;
    }
}

// [KE_t, KE_r] per system: one block per system over its library-order ranges of bodies and free
// atoms, FP64, fixed-order tree.
template <int P>
__global__ void __launch_bounds__(kKEThreads) kinetic_systems_kernel(DevSys S, DevBuf B, const int* body0,
                                                                     const int* free0, double* out) {
    using V4 = typename Tr<P>::V4;
    __shared__ double s_t[kKEThreads], s_r[kKEThreads];
    const int sys = blockIdx.x;
    double kt = 0.0, kr = 0.0;
    for (int b = body0[sys] + threadIdx.x; b < body0[sys + 1]; b += blockDim.x) {
        V3<double> v, invI;
        Q4<double> q, pi;
        double invm;
        BodyRead<P>::get(S, b, v, q, pi, invm, invI);
        V3<double> L = qBt(q, pi) * 0.5;
        kt += dot(v, v) / invm;
        kr += dot(L, mul(invI, L));
    }
    const V4* vel = (const V4*)B.velm;
    for (int j = free0[sys] + threadIdx.x; j < free0[sys + 1]; j += blockDim.x) {
        V4 vm = vel[S.free_loc[j]];
        double vx = vm.x, vy = vm.y, vz = vm.z;
        kt += (vx * vx + vy * vy + vz * vz) / (double)vm.w;
    }
    s_t[threadIdx.x] = kt;
    s_r[threadIdx.x] = kr;
    __syncthreads();
    for (int w = kKEThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s_t[threadIdx.x] += s_t[threadIdx.x + w];
            s_r[threadIdx.x] += s_r[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[2 * sys] = 0.5 * s_t[0];
        out[2 * sys + 1] = 0.5 * s_r[0];
    }
}

// Scale every momentum by `factor`: body COM velocities and quaternion momenta (both state
// layouts) and the free atoms' velocities (damped relaxation; 0 zeroes them).
template <int P>
__global__ void scale_momenta_kernel(DevSys S, DevBuf B, double factor) {
    using V4 = typename Tr<P>::V4;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S.nb) {
        const int rows[7] = {3, 4, 5, 10, 11, 12, 13};
        if (P == PREC_DOUBLE) {
            double* st = (double*)S.state;
            for (int r : rows) st[i + (size_t)r * S.nb_pad] *= factor;
        } else {
            float* st = (float*)S.state;
            const float f = (float)factor;
            for (int r : rows) {
                st[i + (size_t)r * S.nb_pad] *= f;
                st[i + (size_t)(14 + r) * S.nb_pad] *= f;
            }
        }
    }
    if (i < S.nf) {
        V4* vel = (V4*)B.velm;
        V4 vm = vel[S.free_loc[i]];
        vm.x *= factor;
        vm.y *= factor;
        vm.z *= factor;
        vel[S.free_loc[i]] = vm;
    }
}

// Body-atom positions from the stored body state (r + At(q) d), with exactly the arithmetic of the
// step kernels' position rebuild: after a restore of the body state they equal the positions the
// last step wrote. One thread per body.
template <int P>
__global__ void sync_positions_kernel(DevSys S, DevBuf B) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= S.nb) return;
    const int nbp = S.nb_pad;
    const int a0 = S.atom0[b], a1 = S.atom0[b + 1];
    if (P == PREC_DOUBLE) {
        const double* st = (const double*)S.state;
        const double* d = (const double*)S.d;
        const V3<double> r = v3<double>(st[b], st[b + nbp], st[b + 2 * nbp]);
        const Q4<double> q = q4<double>(st[b + 6 * nbp], st[b + 7 * nbp], st[b + 8 * nbp], st[b + 9 * nbp]);
        for (int k = a0; k < a1; k++) {
            const V3<double> delta = rotate_to_space(q, v3<double>(d[k], d[k + S.nba_pad], d[k + 2 * S.nba_pad]));
            PosIO<P>::store(B, S.atom_loc[k], r, delta);
        }
    } else {
        const float* hi = (const float*)S.state;
        const float* lo = hi + 14 * nbp;
        const float* d = (const float*)S.d;
        float m[9];
        rotation_matrix(q4<float>(hi[b + 6 * nbp], hi[b + 7 * nbp], hi[b + 8 * nbp], hi[b + 9 * nbp]), m);
        const float rf[6] = {hi[b], lo[b], hi[b + nbp], lo[b + nbp], hi[b + 2 * nbp], lo[b + 2 * nbp]};
        for (int k = a0; k < a1; k++) {
            const V3<float> delta = mat_vec(m, v3<float>(d[k], d[k + S.nba_pad], d[k + 2 * S.nba_pad]));
            float* pq = (float*)B.posq + 4 * (size_t)S.atom_loc[k];
            if (P == PREC_MIXED) {
                const ff px = ff_add(ff{rf[0], rf[1]}, delta.x);
                const ff py = ff_add(ff{rf[2], rf[3]}, delta.y);
                const ff pz = ff_add(ff{rf[4], rf[5]}, delta.z);
                *(float2*)pq = make_float2(px.hi, py.hi);
                pq[2] = pz.hi;
                ((float4*)B.corr)[S.atom_loc[k]] = make_float4(px.lo, py.lo, pz.lo, 0.0f);
            } else {
                *(float2*)pq = make_float2(rf[0] + (rf[1] + delta.x), rf[2] + (rf[3] + delta.y));
                pq[2] = rf[4] + (rf[5] + delta.z);
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Free atoms under constraints, through OpenMM's posDelta buffer (mixed4 per slot: float4 in
// single precision, double4 otherwise, the element type of velm). free_delta_kernel writes the
// unconstrained displacement h (v + F/m h/2) of each free atom for the constraint solver
// (freeAtomsDelta, rigidbodyintegrator.cu:270-279); free_apply_delta_kernel moves the atom by the
// corrected displacement and sets its mid-step velocity to that displacement over h. This is the
// Reference platform's step (RigidBodySystem.cpp:172-176 followed by SHAKE) with the
// (R - savedPos)/dt term of part2 (:197) folded into part1; the CUDA reference drops that term
// because it saves the position after the constraints (rigidbodyintegrator.cu:304-305).
// ------------------------------------------------------------------------------------------
template <int P>
__global__ void free_delta_kernel(DevSys S, DevBuf B, void* pos_delta, double dt) {
    using T = typename Tr<P>::R;
    using V4 = typename Tr<P>::V4;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= S.nf) return;
    const int loc = S.free_loc[j];
    const V4 vm = ((const V4*)B.velm)[loc];
    const T w = (T)vm.w, h = (T)dt;
    const V3<T> F = load_force<T>(B.force, loc, B.stride);
    const V3<T> d = (v3<T>((T)vm.x, (T)vm.y, (T)vm.z) + F * (w * (T(0.5) * h))) * h;
    V4 out;
    out.x = d.x; out.y = d.y; out.z = d.z; out.w = 0;
    ((V4*)pos_delta)[loc] = out;
}

template <int P>
__global__ void free_apply_delta_kernel(DevSys S, DevBuf B, const void* pos_delta, double dt) {
    using T = typename Tr<P>::R;
    using V4 = typename Tr<P>::V4;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= S.nf) return;
    const int loc = S.free_loc[j];
    const V4 dm = ((const V4*)pos_delta)[loc];
    const V3<T> d = v3<T>((T)dm.x, (T)dm.y, (T)dm.z);
    const V3<double> x = PosIO<P>::load(B, loc);
    PosIO<P>::store(B, loc, x + cvt<double>(d), v3<T>(T(0), T(0), T(0)));
    V4* vel = (V4*)B.velm;
    V4 vm = vel[loc];
    const T inv = T(1) / (T)dt;
    vm.x = d.x * inv; vm.y = d.y * inv; vm.z = d.z * inv;
    vel[loc] = vm;
}

// ------------------------------------------------------------------------------------------
// Layout conversion for the host-buffer API (user order doubles <-> OpenMM device layout).
// ------------------------------------------------------------------------------------------
__global__ void forces_from_host_kernel(const double* __restrict__ f, const int* __restrict__ loc, int n,
                                        long long* __restrict__ force, int stride) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = loc[i];
    force[s] = __double2ll_rn(f[3 * i] * 0x1p32);
    force[s + stride] = __double2ll_rn(f[3 * i + 1] * 0x1p32);
    force[s + 2 * stride] = __double2ll_rn(f[3 * i + 2] * 0x1p32);
}

template <int P>
__global__ void load_positions_kernel(const double* __restrict__ x, const double* __restrict__ v,
                                      const double* __restrict__ m, const int* __restrict__ loc, int n, DevBuf B) {
    using V4 = typename Tr<P>::V4;
    using P4 = typename Tr<P>::P4;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = loc[i];
    P4 zero;
    zero.x = 0; zero.y = 0; zero.z = 0; zero.w = 0;
    ((P4*)B.posq)[s] = zero;  // charge slot unused by the integrator
    if (Tr<P>::kCorr) ((float4*)B.corr)[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    PosIO<P>::store(B, s, v3<double>(x[3 * i], x[3 * i + 1], x[3 * i + 2]), v3<double>(0.0, 0.0, 0.0));
    V4 vm;
    vm.x = v[3 * i]; vm.y = v[3 * i + 1]; vm.z = v[3 * i + 2];
    vm.w = m[i] == 0.0 ? 0.0 : 1.0 / m[i];
    ((V4*)B.velm)[s] = vm;
}

template <int P>
__global__ void store_positions_kernel(DevBuf B, const int* __restrict__ loc, int n, double* __restrict__ x,
                                       double* __restrict__ v) {
    using V4 = typename Tr<P>::V4;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = loc[i];
    V3<double> p = PosIO<P>::load(B, s);
    x[3 * i] = p.x; x[3 * i + 1] = p.y; x[3 * i + 2] = p.z;
    if (v) {
        V4 vm = ((const V4*)B.velm)[s];
        v[3 * i] = vm.x; v[3 * i + 1] = vm.y; v[3 * i + 2] = vm.z;
    }
}

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------

int launch_sync_positions(int prec, const DevSys& s, const DevBuf& b, void* stream) {
    if (s.nb == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int g = (s.nb + 127) / 128;
    switch (prec) {
        case PREC_SINGLE: sync_positions_kernel<PREC_SINGLE><<<g, 128, 0, st>>>(s, b); break;
        case PREC_MIXED: sync_positions_kernel<PREC_MIXED><<<g, 128, 0, st>>>(s, b); break;
        default: sync_positions_kernel<PREC_DOUBLE><<<g, 128, 0, st>>>(s, b); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_scale_momenta(int prec, const DevSys& s, const DevBuf& b, double factor, void* stream) {
    const int n = s.nb > s.nf ? s.nb : s.nf;
    if (n == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int g = (n + 255) / 256;
    switch (prec) {
        case PREC_SINGLE: scale_momenta_kernel<PREC_SINGLE><<<g, 256, 0, st>>>(s, b, factor); break;
        case PREC_MIXED: scale_momenta_kernel<PREC_MIXED><<<g, 256, 0, st>>>(s, b, factor); break;
        default: scale_momenta_kernel<PREC_DOUBLE><<<g, 256, 0, st>>>(s, b, factor); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_kinetic_systems(int prec, const DevSys& s, const DevBuf& b, const int* body0, const int* free0,
                           int num_systems, double* out, void* stream) {
    if (num_systems <= 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    switch (prec) {
        case PREC_SINGLE: kinetic_systems_kernel<PREC_SINGLE><<<num_systems, kKEThreads, 0, st>>>(s, b, body0, free0, out); break;
        case PREC_MIXED: kinetic_systems_kernel<PREC_MIXED><<<num_systems, kKEThreads, 0, st>>>(s, b, body0, free0, out); break;
        default: kinetic_systems_kernel<PREC_DOUBLE><<<num_systems, kKEThreads, 0, st>>>(s, b, body0, free0, out); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_step(int prec, int kind, const DevSys& s, const DevBuf& b, double dt, void* stream) {
    if (s.ref_start) return launch_step_refined(prec, kind, s, b, dt, stream);
    cudaStream_t st = (cudaStream_t)stream;
    switch (prec) {
        case PREC_SINGLE: return launch_step_p<PREC_SINGLE, false>(kind, s, b, dt, st);
        case PREC_MIXED: return launch_step_p<PREC_MIXED, false>(kind, s, b, dt, st);
        default: return launch_step_p<PREC_DOUBLE, false>(kind, s, b, dt, st);
    }
}

int kinetic_blocks(const DevSys& s) {
    int n = s.nb > s.nf ? s.nb : s.nf;
    int blocks = (n + kKEThreads - 1) / kKEThreads;
    if (blocks > 4 * 152) blocks = 4 * 152;
    return blocks < 1 ? 1 : blocks;
}

int launch_kinetic(int prec, const DevSys& s, const DevBuf& b, const KEScratch& k, int n_blocks, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    switch (prec) {
        case PREC_SINGLE: kinetic_kernel<PREC_SINGLE><<<n_blocks, kKEThreads, 0, st>>>(s, b, k); break;
        case PREC_MIXED: kinetic_kernel<PREC_MIXED><<<n_blocks, kKEThreads, 0, st>>>(s, b, k); break;
        default: kinetic_kernel<PREC_DOUBLE><<<n_blocks, kKEThreads, 0, st>>>(s, b, k); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_free_delta(int prec, const DevSys& s, const DevBuf& b, void* pos_delta, double dt, void* stream) {
    if (s.nf == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int g = (s.nf + 255) / 256;
    switch (prec) {
        case PREC_SINGLE: free_delta_kernel<PREC_SINGLE><<<g, 256, 0, st>>>(s, b, pos_delta, dt); break;
        case PREC_MIXED: free_delta_kernel<PREC_MIXED><<<g, 256, 0, st>>>(s, b, pos_delta, dt); break;
        default: free_delta_kernel<PREC_DOUBLE><<<g, 256, 0, st>>>(s, b, pos_delta, dt); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_free_apply_delta(int prec, const DevSys& s, const DevBuf& b, const void* pos_delta, double dt, void* stream) {
    if (s.nf == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int g = (s.nf + 255) / 256;
    switch (prec) {
        case PREC_SINGLE: free_apply_delta_kernel<PREC_SINGLE><<<g, 256, 0, st>>>(s, b, pos_delta, dt); break;
        case PREC_MIXED: free_apply_delta_kernel<PREC_MIXED><<<g, 256, 0, st>>>(s, b, pos_delta, dt); break;
        default: free_apply_delta_kernel<PREC_DOUBLE><<<g, 256, 0, st>>>(s, b, pos_delta, dt); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_forces_from_host(int prec, const double* f, const int* location, int natoms, long long* force, int stride,
                            void* stream) {
    (void)prec;
    if (natoms == 0) return 0;
    forces_from_host_kernel<<<(natoms + 255) / 256, 256, 0, (cudaStream_t)stream>>>(f, location, natoms, force, stride);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_load_positions(int prec, const double* x, const double* v, const double* m, const int* location, int natoms,
                          const DevBuf& b, void* stream) {
    if (natoms == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    int g = (natoms + 255) / 256;
    switch (prec) {
        case PREC_SINGLE: load_positions_kernel<PREC_SINGLE><<<g, 256, 0, st>>>(x, v, m, location, natoms, b); break;
        case PREC_MIXED: load_positions_kernel<PREC_MIXED><<<g, 256, 0, st>>>(x, v, m, location, natoms, b); break;
        default: load_positions_kernel<PREC_DOUBLE><<<g, 256, 0, st>>>(x, v, m, location, natoms, b); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_store_positions(int prec, const DevBuf& b, const int* location, int natoms, double* x, double* v,
                           void* stream) {
    if (natoms == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    int g = (natoms + 255) / 256;
    switch (prec) {
        case PREC_SINGLE: store_positions_kernel<PREC_SINGLE><<<g, 256, 0, st>>>(b, location, natoms, x, v); break;
        case PREC_MIXED: store_positions_kernel<PREC_MIXED><<<g, 256, 0, st>>>(b, location, natoms, x, v); break;
        default: store_positions_kernel<PREC_DOUBLE><<<g, 256, 0, st>>>(b, location, natoms, x, v); break;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// ------------------------------------------------------------------------------------------
// Kinetic energy without device allocation (rbx_kinetic_energies_static).
//
// Some callers cannot call cudaMalloc: a serving process that has reserved its whole
// device-memory budget up front and admits work only against that reservation, a host
// framework that owns every device allocation through its own pool, or a latency-sensitive
// loop that cannot afford the device synchronisation an allocation may cause. For them the
// reduction's scratch (one pair of partial sums per block and the block ticket counter) lives
// in a fixed static device array of this file instead of memory owned by an integrator handle.
// ------------------------------------------------------------------------------------------
constexpr int kStaticKEMaxBlocks = 1024;
constexpr int kStaticKEItemsPerBlock = kKEThreads * 16;  // bodies (and free atoms) per block
constexpr long long kStaticKEMaxItems = (long long)kStaticKEMaxBlocks * kStaticKEItemsPerBlock;  // 4,194,304
constexpr int kMaxDevices = 64;
// [0, 2*kStaticKEMaxBlocks): per-block partial sums; then one unsigned ticket counter.
// 16 KB + 256 B, resident on every device that loads the library until the process exits.
static __device__ __align__(256) double g_static_ke_scratch[2 * kStaticKEMaxBlocks + 32];

template <int P>
__global__ void __launch_bounds__(kKEThreads) kinetic_static_kernel(DevSys S, DevBuf B, double* scratch, double* out) {
    using V4 = typename Tr<P>::V4;
    __shared__ double s_t[kKEThreads], s_r[kKEThreads];
    __shared__ bool s_last;
    double* partial = scratch;
    unsigned int* count = (unsigned int*)(scratch + 2 * kStaticKEMaxBlocks);
    const int nbp = S.nb_pad;
    const double* st = (const double*)S.state;
    const int first = blockIdx.x * kStaticKEItemsPerBlock;
    const int last = first + kStaticKEItemsPerBlock;
    double kt = 0.0, kr = 0.0;
    for (int b = first + (int)threadIdx.x; b < last && b < S.nb; b += kKEThreads) {
        V3<double> v = v3<double>(st[b + 3 * nbp], st[b + 4 * nbp], st[b + 5 * nbp]);
        Q4<double> q = q4<double>(st[b + 6 * nbp], st[b + 7 * nbp], st[b + 8 * nbp], st[b + 9 * nbp]);
        Q4<double> pi = q4<double>(st[b + 10 * nbp], st[b + 11 * nbp], st[b + 12 * nbp], st[b + 13 * nbp]);
        V3<double> invI = v3<double>(S.invI[b], S.invI[b + nbp], S.invI[b + 2 * nbp]);
        V3<double> L = qBt(q, pi) * 0.5;
        kt += dot(v, v) / S.invm[b];
        kr += dot(L, mul(invI, L));
    }
    const V4* vel = (const V4*)B.velm;
    for (int j = first + (int)threadIdx.x; j < last && j < S.nf; j += kKEThreads) {
        V4 vm = vel[S.free_loc[j]];
        double vx = vm.x, vy = vm.y, vz = vm.z;
        // w = 1/m; a massless slot (w = 0, as OpenMM stores virtual sites) carries no kinetic energy
        if (vm.w != 0) kt += (vx * vx + vy * vy + vz * vz) / (double)vm.w;
    }
    s_t[threadIdx.x] = kt;
    s_r[threadIdx.x] = kr;
    __syncthreads();
    for (int w = kKEThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s_t[threadIdx.x] += s_t[threadIdx.x + w];
            s_r[threadIdx.x] += s_r[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = s_t[0];
        partial[2 * blockIdx.x + 1] = s_r[0];
        __threadfence();
        unsigned int ticket = atomicAdd(count, 1u);
        s_last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        double t = 0.0, r = 0.0;
        for (unsigned int i = 0; i < gridDim.x; i++) {
            t += ((volatile double*)partial)[2 * i];
            r += ((volatile double*)partial)[2 * i + 1];
        }
        out[0] = 0.5 * t;
        out[1] = 0.5 * r;
        *count = 0u;
    }
}

// Device address of the static scratch on the current device. Outside stream capture it is
// looked up on every call (a cudaDeviceReset reloads the module, which may move the array) and
// remembered per device; a call made while `stream` is capturing uses the remembered address,
// so the first call on a device must come before any capture.
static int static_scratch_address(cudaStream_t stream, double** out) {
    static std::mutex mu;
    static void* addr[kMaxDevices] = {};
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(RBX_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(RBX_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(stream, &capture);
    if (e != cudaSuccess) return set_error(RBX_ERR_CUDA, "cudaStreamIsCapturing: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(mu);
    if (capture == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_ke_scratch);
        if (e != cudaSuccess)
            return set_error(RBX_ERR_CUDA, "cudaGetSymbolAddress of the static scratch: %s", cudaGetErrorString(e));
        addr[dev] = p;
    } else if (!addr[dev]) {
        return set_error(RBX_ERR_STATE, "rbx_kinetic_energies_static: the first call on device %d was made "
                         "during stream capture; make one call before capturing", dev);
    }
    *out = (double*)addr[dev];
    return RBX_OK;
}

}  // namespace rbx

extern "C" int rbx_kinetic_energies_static(const double* body_state, int num_bodies, int body_stride,
                                           const double* inv_mass, const double* inv_inertia, const void* velm,
                                           const int* free_slots, int num_free, int precision, void* stream,
                                           double* out_device) {
    using namespace rbx;
    if (num_bodies < 0 || num_free < 0) return set_error(RBX_ERR_INVALID_ARGUMENT, "negative counts");
    if ((long long)num_bodies > kStaticKEMaxItems || (long long)num_free > kStaticKEMaxItems)
        return set_error(RBX_ERR_UNSUPPORTED,
                         "rbx_kinetic_energies_static handles at most %lld bodies and %lld free atoms "
                         "(its fixed scratch holds %d block sums); got %d bodies, %d free atoms",
                         kStaticKEMaxItems, kStaticKEMaxItems, kStaticKEMaxBlocks, num_bodies, num_free);
    if (num_bodies > 0 && (!body_state || !inv_mass || !inv_inertia || body_stride < num_bodies))
        return set_error(RBX_ERR_INVALID_ARGUMENT, "body arrays missing or body_stride < num_bodies");
    // the kernel indexes row r of body b as b + r * body_stride (r <= 13) in 32-bit arithmetic
    if (num_bodies > 0 && (long long)body_stride * 14 > (long long)INT_MAX)
        return set_error(RBX_ERR_UNSUPPORTED, "body_stride %d beyond 32-bit indexing of 14 rows (at most %d)",
                         body_stride, INT_MAX / 14);
    if (num_free > 0 && (!velm || !free_slots)) return set_error(RBX_ERR_INVALID_ARGUMENT, "free-atom arrays missing");
    if (!out_device) return set_error(RBX_ERR_INVALID_ARGUMENT, "null output");
    if (precision < PREC_SINGLE || precision > PREC_DOUBLE) return set_error(RBX_ERR_INVALID_ARGUMENT, "unknown precision");
    cudaStream_t st = (cudaStream_t)stream;
    double* scratch = nullptr;
    int rc = static_scratch_address(st, &scratch);
    if (rc) return rc;
    // The array keeps the previous call's contents: the ticket counter must start at zero.
    cudaError_t e = cudaMemsetAsync(scratch + 2 * kStaticKEMaxBlocks, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return set_error(RBX_ERR_CUDA, "clearing the static scratch: %s", cudaGetErrorString(e));
    DevSys s{};
    s.nb = num_bodies; s.nf = num_free; s.nb_pad = body_stride;
    s.state = const_cast<double*>(body_state); s.invm = inv_mass; s.invI = inv_inertia; s.free_loc = free_slots;
    DevBuf b{};
    b.velm = const_cast<void*>(velm);
    long long items = num_bodies > num_free ? num_bodies : num_free;
    int grid = (int)((items + kStaticKEItemsPerBlock - 1) / kStaticKEItemsPerBlock);
    if (grid < 1) grid = 1;
    switch (precision) {
        case PREC_SINGLE: kinetic_static_kernel<PREC_SINGLE><<<grid, kKEThreads, 0, st>>>(s, b, scratch, out_device); break;
        case PREC_MIXED: kinetic_static_kernel<PREC_MIXED><<<grid, kKEThreads, 0, st>>>(s, b, scratch, out_device); break;
        default: kinetic_static_kernel<PREC_DOUBLE><<<grid, kKEThreads, 0, st>>>(s, b, scratch, out_device); break;
    }
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) return set_error(RBX_ERR_CUDA, "kinetic-energy launch: %s", cudaGetErrorString(e));
    return RBX_OK;
}
