// rbx_kernels.cu -- sm_103a kernels of the rigid-body integrator.
//
// One step kernel serves the three step kinds (part1, part2, fused part2+part1) of the plugin's
// integrateRigidBodyPart1/Part2 and freeAtomsDelta (platforms/cuda/src/kernels/
// rigidbodyintegrator.cu:270-396). A CTA owns one tile: a run of bodies whose atoms are
// contiguous in the library's body-atom order (bodies sorted by size so that a tile holds bodies
// of one kind). Four phases, separated by __syncthreads:
//   0. one thread per body stages its orientation and marks its atoms in shared memory;
//   1. one thread per atom gathers the fixed-point force, rebuilds the COM displacement
//      delta = At(q) d and its torque delta x F, and parks F and tau in shared memory;
//   2. one thread per body sums its atoms' F and tau in a fixed order (deterministic), applies
//      the half kick(s), drift and free rotation (NO-SQUISH or exact) on the FP64 state;
//   3. one thread per atom writes the new position r + At(q) d (or, for part2, the velocity
//      v + omega x delta) to its device slot.
// Free atoms live in separate tiles of the same launch (velocity Verlet).
// The kinetic-energy kernel reduces [KE_t, KE_r] in FP64 in a fixed order.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/rbx.h"

#include "rbx_internal.h"
#include "rbx_math.cuh"

namespace rbx {

// 32-byte aligned double quadruple (the layout of OpenMM's double4 arrays) so that a velm or
// posq element moves with full-width vector accesses.
struct __align__(32) dq4 {
    double x, y, z, w;
};

template <int P> struct Tr;
template <> struct Tr<PREC_SINGLE> {
    using A = float;   // per-atom arithmetic
    using R = float;   // body kinematics and rotation
    using D = float;   // body-frame coordinates in HBM
    using P4 = float4; // posq element
    using V4 = float4; // velm element
    static constexpr bool kCorr = false;
    static constexpr int kTA = kTileAtomsF;
};
template <> struct Tr<PREC_MIXED> {
    using A = float;
    using R = double;
    using D = float;
    using P4 = float4;
    using V4 = dq4;
    static constexpr bool kCorr = true;
    static constexpr int kTA = kTileAtomsF;
};
template <> struct Tr<PREC_DOUBLE> {
    using A = double;
    using R = double;
    using D = double;
    using P4 = dq4;
    using V4 = dq4;
    static constexpr bool kCorr = false;
    static constexpr int kTA = kTileAtomsD;
};

// Fixed-point force (scale 2^32) to floating point.
template <class T> __device__ __forceinline__ T fixed_to(long long v);
template <> __device__ __forceinline__ float fixed_to<float>(long long v) { return __ll2float_rn(v) * 0x1p-32f; }
template <> __device__ __forceinline__ double fixed_to<double>(long long v) { return __ll2double_rn(v) * 0x1p-32; }

template <class T> __device__ __forceinline__ V3<T> load_force(const long long* __restrict__ f, int loc, int stride) {
    return v3<T>(fixed_to<T>(__ldg(f + loc)), fixed_to<T>(__ldg(f + loc + stride)), fixed_to<T>(__ldg(f + loc + 2 * stride)));
}

template <class To, class From> __device__ __forceinline__ V3<To> cvt(V3<From> a) {
    return v3<To>((To)a.x, (To)a.y, (To)a.z);
}
template <class To, class From> __device__ __forceinline__ Q4<To> cvt(Q4<From> a) {
    return q4<To>((To)a.w, (To)a.x, (To)a.y, (To)a.z);
}

// Position read/write in the OpenMM layout of each precision (rigidbodyintegrator.cu:30-64).
template <int P> struct PosIO;
template <> struct PosIO<PREC_SINGLE> {
    static __device__ __forceinline__ V3<double> load(const DevBuf& b, int loc) {
        float4 p = ((const float4*)b.posq)[loc];
        return v3<double>(p.x, p.y, p.z);
    }
    template <class A> static __device__ __forceinline__ void store(const DevBuf& b, int loc, V3<double> base, V3<A> delta) {
        float4* pq = (float4*)b.posq;
        float4 p = pq[loc];
        p.x = (float)base.x + (float)delta.x;
        p.y = (float)base.y + (float)delta.y;
        p.z = (float)base.z + (float)delta.z;
        pq[loc] = p;
    }
};
template <> struct PosIO<PREC_MIXED> {
    static __device__ __forceinline__ V3<double> load(const DevBuf& b, int loc) {
        float4 p = ((const float4*)b.posq)[loc];
        float4 c = ((const float4*)b.corr)[loc];
        return v3<double>((double)p.x + (double)c.x, (double)p.y + (double)c.y, (double)p.z + (double)c.z);
    }
    template <class A> static __device__ __forceinline__ void store(const DevBuf& b, int loc, V3<double> base, V3<A> delta) {
        float4* pq = (float4*)b.posq;
        float4 p = pq[loc];
        double x = base.x + (double)delta.x, y = base.y + (double)delta.y, z = base.z + (double)delta.z;
        p.x = (float)x; p.y = (float)y; p.z = (float)z;
        pq[loc] = p;
        ((float4*)b.corr)[loc] = make_float4((float)(x - (double)p.x), (float)(y - (double)p.y), (float)(z - (double)p.z), 0.0f);
    }
};
template <> struct PosIO<PREC_DOUBLE> {
    static __device__ __forceinline__ V3<double> load(const DevBuf& b, int loc) {
        dq4 p = ((const dq4*)b.posq)[loc];
        return v3<double>(p.x, p.y, p.z);
    }
    template <class A> static __device__ __forceinline__ void store(const DevBuf& b, int loc, V3<double> base, V3<A> delta) {
        dq4* pq = (dq4*)b.posq;
        dq4 p = pq[loc];
        p.x = base.x + (double)delta.x;
        p.y = base.y + (double)delta.y;
        p.z = base.z + (double)delta.z;
        pq[loc] = p;
    }
};

template <class T> struct SmemLayout {
    // byte offsets of the shared-memory arrays of one step CTA
    static constexpr size_t align(size_t x) { return (x + 15) & ~size_t(15); }
};

template <int P> __host__ __device__ constexpr size_t step_smem() {
    using A = typename Tr<P>::A;
    constexpr int TA = Tr<P>::kTA, TB = kTileBodies;
    // sF, sT, sX: 3*TA each (A); sQ: 4*TB (A); sRb: 3*TB (double); sW: 3*TB (A); sBody: TA (uint16)
    return (size_t)3 * 3 * TA * sizeof(A) + 4 * TB * sizeof(A) + 3 * TB * sizeof(double) + 3 * TB * sizeof(A) +
           TA * sizeof(unsigned short) + 64;
}

template <int P, int KIND>
__device__ __forceinline__ void free_atom_tile(const DevSys& S, const DevBuf& B, double dt, int ft) {
    using T = typename Tr<P>::R;  // free-atom velocity/position arithmetic
    using V4 = typename Tr<P>::V4;
    const int j = ft * kFreePerTile + (int)threadIdx.x;
    if (j >= S.nf) return;
    const int loc = __ldg(S.free_loc + j);
    V4* vel = (V4*)B.velm;
    V4 vm = vel[loc];
    V3<T> v = v3<T>((T)vm.x, (T)vm.y, (T)vm.z);
    const T w = (T)vm.w;
    const T halfDt = T(0.5) * (T)dt;
    V3<T> dv = load_force<T>(B.force, loc, B.stride) * (w * halfDt);
    if (KIND != STEP_PART1) v = v + dv;  // second half kick of step n (rigidbodyintegrator.cu:351-358)
    if (KIND != STEP_PART2) {            // first half kick and drift of the next step (:302-310)
        v = v + dv;
        V3<double> x = PosIO<P>::load(B, loc);
        V3<double> nx = x + cvt<double>(v * (T)dt);
        PosIO<P>::store(B, loc, nx, v3<T>(T(0), T(0), T(0)));
    }
    vm.x = v.x; vm.y = v.y; vm.z = v.z;
    vel[loc] = vm;
}

template <int P, int KIND, bool EXACT>
__global__ void __launch_bounds__(kThreads) step_kernel(DevSys S, DevBuf B, double dt) {
    using A = typename Tr<P>::A;
    using R = typename Tr<P>::R;
    using D = typename Tr<P>::D;
    using V4 = typename Tr<P>::V4;
    constexpr int TA = Tr<P>::kTA, TB = kTileBodies;

    if ((int)blockIdx.x >= S.n_body_tiles) {
        free_atom_tile<P, KIND>(S, B, dt, (int)blockIdx.x - S.n_body_tiles);
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    A* sF = (A*)smem;
    A* sT = sF + 3 * TA;
    A* sX = sT + 3 * TA;
    A* sQ = sX + 3 * TA;
    double* sRb = (double*)(sQ + 4 * TB);
    A* sW = (A*)(sRb + 3 * TB);
    unsigned short* sBody = (unsigned short*)(sW + 3 * TB);

    const int tid = threadIdx.x;
    const int b0 = __ldg(S.tile_body0 + blockIdx.x), b1 = __ldg(S.tile_body0 + blockIdx.x + 1);
    const int nbt = b1 - b0;
    const int a0 = __ldg(S.atom0 + b0), nat = __ldg(S.atom0 + b1) - a0;
    const int nbp = S.nb_pad;
    double* __restrict__ st = S.state;

    // Phase 0: stage orientation, mark atoms with their tile-local body.
    if (tid < nbt) {
        const int b = b0 + tid;
        sQ[4 * tid + 0] = (A)st[b + 6 * nbp];
        sQ[4 * tid + 1] = (A)st[b + 7 * nbp];
        sQ[4 * tid + 2] = (A)st[b + 8 * nbp];
        sQ[4 * tid + 3] = (A)st[b + 9 * nbp];
        const int s = __ldg(S.atom0 + b) - a0, e = __ldg(S.atom0 + b + 1) - a0;
        for (int j = s; j < e; j++) sBody[j] = (unsigned short)tid;
    }
    __syncthreads();

    // Phase 1: per-atom force, displacement and torque.
    const D* __restrict__ dg = (const D*)S.d;
    for (int a = tid; a < nat; a += kThreads) {
        const int k = a0 + a;
        const int t = sBody[a];
        Q4<A> q = q4<A>(sQ[4 * t], sQ[4 * t + 1], sQ[4 * t + 2], sQ[4 * t + 3]);
        V3<A> d = v3<A>((A)__ldg(dg + k), (A)__ldg(dg + k + S.nba_pad), (A)__ldg(dg + k + 2 * S.nba_pad));
        const int loc = __ldg(S.atom_loc + k);
        V3<A> F = load_force<A>(B.force, loc, B.stride);
        V3<A> delta = rotate_to_space(q, d);
        V3<A> tau = cross(delta, F);
        sF[3 * a] = F.x; sF[3 * a + 1] = F.y; sF[3 * a + 2] = F.z;
        sT[3 * a] = tau.x; sT[3 * a + 1] = tau.y; sT[3 * a + 2] = tau.z;
        V3<A> x = KIND == STEP_PART2 ? delta : d;
        sX[3 * a] = x.x; sX[3 * a + 1] = x.y; sX[3 * a + 2] = x.z;
    }
    __syncthreads();

    // Phase 2: per-body reduction, kicks, drift, rotation.
    if (tid < nbt) {
        const int b = b0 + tid;
        const int s = __ldg(S.atom0 + b) - a0, e = __ldg(S.atom0 + b + 1) - a0;
        V3<A> Fa = v3<A>(A(0), A(0), A(0)), Ta = Fa;
        for (int j = s; j < e; j++) {
            Fa = Fa + v3<A>(sF[3 * j], sF[3 * j + 1], sF[3 * j + 2]);
            Ta = Ta + v3<A>(sT[3 * j], sT[3 * j + 1], sT[3 * j + 2]);
        }
        V3<double> r = v3<double>(st[b], st[b + nbp], st[b + 2 * nbp]);
        V3<R> v = v3<R>((R)st[b + 3 * nbp], (R)st[b + 4 * nbp], (R)st[b + 5 * nbp]);
        Q4<R> q = q4<R>((R)st[b + 6 * nbp], (R)st[b + 7 * nbp], (R)st[b + 8 * nbp], (R)st[b + 9 * nbp]);
        Q4<R> pi = q4<R>((R)st[b + 10 * nbp], (R)st[b + 11 * nbp], (R)st[b + 12 * nbp], (R)st[b + 13 * nbp]);
        const R invm = (R)__ldg(S.invm + b);
        const V3<R> invI = v3<R>((R)__ldg(S.invI + b), (R)__ldg(S.invI + b + nbp), (R)__ldg(S.invI + b + 2 * nbp));
        const R rdt = (R)dt, halfDt = R(0.5) * rdt;
        const V3<R> F = cvt<R>(Fa);
        const Q4<R> Ctau = qC(q, cvt<R>(Ta));
        const V3<R> dv = F * (invm * halfDt);
        const int kicks = KIND == STEP_FUSED ? 2 : 1;
        for (int kk = 0; kk < kicks; kk++) {
            v = v + dv;
            pi = pi + Ctau * rdt;
        }
        st[b + 3 * nbp] = (double)v.x; st[b + 4 * nbp] = (double)v.y; st[b + 5 * nbp] = (double)v.z;
        if (KIND == STEP_PART2) {
            V3<R> omega = mul(invI, qBt(q, pi)) * R(0.5);
            V3<R> ws = rotate_to_space(q, omega);
            sRb[3 * tid] = (double)v.x; sRb[3 * tid + 1] = (double)v.y; sRb[3 * tid + 2] = (double)v.z;
            sW[3 * tid] = (A)ws.x; sW[3 * tid + 1] = (A)ws.y; sW[3 * tid + 2] = (A)ws.z;
        } else {
            r = r + cvt<double>(v * rdt);
            if (EXACT) {
                const int cls = __ldg(S.cls + b);
                V3<R> I = v3<R>(R(1) / invI.x, R(1) / invI.y, invI.z != R(0) ? R(1) / invI.z : R(0));
                exact_rotation<R>(cls, I, invI, q, pi, rdt);
            } else {
                nosquish_rotation<R>(invI, invI.z != R(0), q, pi, rdt, S.rot_n);
            }
            st[b] = r.x; st[b + nbp] = r.y; st[b + 2 * nbp] = r.z;
            sRb[3 * tid] = r.x; sRb[3 * tid + 1] = r.y; sRb[3 * tid + 2] = r.z;
            sQ[4 * tid] = (A)q.w; sQ[4 * tid + 1] = (A)q.x; sQ[4 * tid + 2] = (A)q.y; sQ[4 * tid + 3] = (A)q.z;
        }
        st[b + 6 * nbp] = (double)q.w; st[b + 7 * nbp] = (double)q.x;
        st[b + 8 * nbp] = (double)q.y; st[b + 9 * nbp] = (double)q.z;
        st[b + 10 * nbp] = (double)pi.w; st[b + 11 * nbp] = (double)pi.x;
        st[b + 12 * nbp] = (double)pi.y; st[b + 13 * nbp] = (double)pi.z;
    }
    __syncthreads();

    // Phase 3: scatter positions (part1, fused) or velocities (part2).
    for (int a = tid; a < nat; a += kThreads) {
        const int k = a0 + a;
        const int t = sBody[a];
        const int loc = __ldg(S.atom_loc + k);
        V3<A> x = v3<A>(sX[3 * a], sX[3 * a + 1], sX[3 * a + 2]);
        if (KIND == STEP_PART2) {
            V3<A> w = v3<A>(sW[3 * t], sW[3 * t + 1], sW[3 * t + 2]);
            V3<A> rel = cross(w, x);
            V4* vel = (V4*)B.velm;
            V4 vm = vel[loc];
            vm.x = sRb[3 * t] + (double)rel.x;
            vm.y = sRb[3 * t + 1] + (double)rel.y;
            vm.z = sRb[3 * t + 2] + (double)rel.z;
            vel[loc] = vm;
        } else {
            Q4<A> q = q4<A>(sQ[4 * t], sQ[4 * t + 1], sQ[4 * t + 2], sQ[4 * t + 3]);
            V3<A> delta = rotate_to_space(q, x);
            PosIO<P>::store(B, loc, v3<double>(sRb[3 * t], sRb[3 * t + 1], sRb[3 * t + 2]), delta);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Kinetic energy: [KE_t, KE_r] reduced in FP64, fixed order, last block finishes.
// ------------------------------------------------------------------------------------------
constexpr int kKEThreads = 256;

template <int P>
__global__ void __launch_bounds__(kKEThreads) kinetic_kernel(DevSys S, DevBuf B, KEScratch K) {
    using V4 = typename Tr<P>::V4;
    __shared__ double s_t[kKEThreads], s_r[kKEThreads];
    __shared__ bool s_last;
    const int nbp = S.nb_pad;
    const double* st = S.state;
    double kt = 0.0, kr = 0.0;
    const int gsize = gridDim.x * blockDim.x;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < S.nb; b += gsize) {
        V3<double> v = v3<double>(st[b + 3 * nbp], st[b + 4 * nbp], st[b + 5 * nbp]);
        Q4<double> q = q4<double>(st[b + 6 * nbp], st[b + 7 * nbp], st[b + 8 * nbp], st[b + 9 * nbp]);
        Q4<double> pi = q4<double>(st[b + 10 * nbp], st[b + 11 * nbp], st[b + 12 * nbp], st[b + 13 * nbp]);
        V3<double> invI = v3<double>(S.invI[b], S.invI[b + nbp], S.invI[b + 2 * nbp]);
        V3<double> L = qBt(q, pi) * 0.5;
        kt += dot(v, v) / S.invm[b];
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
size_t step_smem_bytes(int prec) {
    switch (prec) {
        case PREC_SINGLE: return step_smem<PREC_SINGLE>();
        case PREC_MIXED: return step_smem<PREC_MIXED>();
        default: return step_smem<PREC_DOUBLE>();
    }
}

template <int P, int KIND, bool EXACT>
static int launch_step_t(const DevSys& s, const DevBuf& b, double dt, cudaStream_t stream) {
    static bool configured = false;
    const size_t smem = step_smem<P>();
    if (!configured) {
        if (cudaFuncSetAttribute(step_kernel<P, KIND, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return -1;
        configured = true;
    }
    const int grid = s.n_body_tiles + s.n_free_tiles;
    if (grid == 0) return 0;
    step_kernel<P, KIND, EXACT><<<grid, kThreads, smem, stream>>>(s, b, dt);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template <int P>
static int launch_step_p(int kind, const DevSys& s, const DevBuf& b, double dt, cudaStream_t st) {
    const bool exact = s.rot_n == 0;
    switch (kind) {
        case STEP_PART1: return exact ? launch_step_t<P, STEP_PART1, true>(s, b, dt, st) : launch_step_t<P, STEP_PART1, false>(s, b, dt, st);
        case STEP_PART2: return launch_step_t<P, STEP_PART2, false>(s, b, dt, st);
        default: return exact ? launch_step_t<P, STEP_FUSED, true>(s, b, dt, st) : launch_step_t<P, STEP_FUSED, false>(s, b, dt, st);
    }
}

int launch_step(int prec, int kind, const DevSys& s, const DevBuf& b, double dt, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    switch (prec) {
        case PREC_SINGLE: return launch_step_p<PREC_SINGLE>(kind, s, b, dt, st);
        case PREC_MIXED: return launch_step_p<PREC_MIXED>(kind, s, b, dt, st);
        default: return launch_step_p<PREC_DOUBLE>(kind, s, b, dt, st);
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
    const double* st = S.state;
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

// Device address of the static scratch, looked up once per device (with that device current).
static int static_scratch_address(double** out) {
    static std::mutex mu;
    static void* addr[kMaxDevices] = {};
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(RBX_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(RBX_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_ke_scratch);
        if (e != cudaSuccess)
            return set_error(RBX_ERR_CUDA, "cudaGetSymbolAddress of the static scratch: %s", cudaGetErrorString(e));
        addr[dev] = p;
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
    if (num_free > 0 && (!velm || !free_slots)) return set_error(RBX_ERR_INVALID_ARGUMENT, "free-atom arrays missing");
    if (!out_device) return set_error(RBX_ERR_INVALID_ARGUMENT, "null output");
    if (precision < PREC_SINGLE || precision > PREC_DOUBLE) return set_error(RBX_ERR_INVALID_ARGUMENT, "unknown precision");
    double* scratch = nullptr;
    int rc = static_scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
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
