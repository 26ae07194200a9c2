// rbx_kernels.cu -- sm_103a kernels of the rigid-body integrator.
//
// The step kernels serve the three step kinds (part1, part2, fused part2+part1) of the plugin's
// integrateRigidBodyPart1/Part2 and freeAtomsDelta (platforms/cuda/src/kernels/
// rigidbodyintegrator.cu:270-396). A CTA owns one tile: a run of bodies whose atoms are
// contiguous in the library's body-atom order (bodies ordered by the lowest device slot of their
// atoms, so that a tile's atoms occupy a narrow slot range). Four phases, separated by __syncthreads:
//   0. one thread per body loads its state and stages its orientation, and marks its atoms
//      with the tile-local body index in shared memory;
//   1. one thread per atom gathers the fixed-point force, rebuilds the COM displacement
//      delta = At(q) d and its torque delta x F, and parks F and tau in shared memory;
//   2. one thread per body sums its atoms' F and tau in a fixed order (deterministic, no
//      atomics), applies the half kick(s), drift and free rotation, and writes its state;
//   3. one thread per atom writes the new position r + At(q) d (or, for part2, the velocity
//      v + omega x delta) to its device slot.
// Free atoms live in separate tiles of the same launch (velocity Verlet).
// step_kernel_d runs double precision in FP64 throughout (the reference formulas, the parity
// anchor). step_kernel_f runs single and mixed precision on the FP32 pipe: float-float body
// state, FP32 rotation increments (rbx_fast.cuh), FP32 per-atom work.
// The kinetic-energy kernel reduces [KE_t, KE_r] in FP64 in a fixed order.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/rbx.h"

#include "rbx_fast.cuh"
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
};
template <> struct Tr<PREC_MIXED> {
    using A = float;
    using R = double;  // free-atom arithmetic (velm is FP64)
    using D = float;
    using P4 = float4;
    using V4 = dq4;
    static constexpr bool kCorr = true;
};
template <> struct Tr<PREC_DOUBLE> {
    using A = double;
    using R = double;
    using D = double;
    using P4 = dq4;
    using V4 = dq4;
    static constexpr bool kCorr = false;
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


// Shared memory of the double-precision step kernel: sF, sT, sX 3*TA each; sQ 4*TB; sRb 3*TB
// (double); sW 3*TB; sBody TA (uint16).
constexpr size_t step_smem_d() {
    constexpr int TA = kTileAtomsD, TB = kTileBodies;
    return (size_t)3 * 3 * TA * sizeof(double) + 4 * TB * sizeof(double) + 3 * TB * sizeof(double) +
           3 * TB * sizeof(double) + TA * sizeof(unsigned short) + 64;
}

template <int P, int KIND>
__device__ __forceinline__ void free_atom_tile(const DevSys& S, const DevBuf& B, double dt, int ft) {
    using T = typename Tr<P>::R;  // free-atom velocity/position arithmetic
    using V4 = typename Tr<P>::V4;
    const int j = ft * (int)blockDim.x + (int)threadIdx.x;
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

// Shared-memory carve-up common to both step kernels.
template <class A> struct StepSmem {
    A *sF, *sT, *sX, *sQ, *sW;
    double* sRb;
    unsigned short* sBody;
    template <int TA, int TB> __device__ __forceinline__ void carve(unsigned char* smem) {
        sF = (A*)smem;
        sT = sF + 3 * TA;
        sX = sT + 3 * TA;
        sQ = sX + 3 * TA;
        sRb = (double*)(sQ + 4 * TB);
        sW = (A*)(sRb + 3 * TB);
        sBody = (unsigned short*)(sW + 3 * TB);
    }
};

// Phase 1 (both kernels): per-atom force, displacement from the COM and torque. Each thread
// owns up to TA / kThreads atoms; all of their loads are issued before any is used so that the
// gathers overlap.
template <int P, int KIND, class A, class D>
__device__ __forceinline__ void atom_forces(const DevSys& S, const DevBuf& B, const StepSmem<A>& sm, int a0, int nat) {
    constexpr int APT = kTileAtomsD / kThreads;
    const D* __restrict__ dg = (const D*)S.d;
    int loc[APT];
    V3<A> F[APT], d[APT];
#pragma unroll
    for (int i = 0; i < APT; i++) {
        const int a = threadIdx.x + i * kThreads;
        loc[i] = a < nat ? __ldg(S.atom_loc + a0 + a) : 0;
    }
#pragma unroll
    for (int i = 0; i < APT; i++) {
        const int a = threadIdx.x + i * kThreads;
        if (a < nat) {
            const int k = a0 + a;
            d[i] = v3<A>((A)__ldg(dg + k), (A)__ldg(dg + k + S.nba_pad), (A)__ldg(dg + k + 2 * S.nba_pad));
            F[i] = load_force<A>(B.force, loc[i], B.stride);
        }
    }
#pragma unroll
    for (int i = 0; i < APT; i++) {
        const int a = threadIdx.x + i * kThreads;
        if (a < nat) {
            const int t = sm.sBody[a];
            Q4<A> q = q4<A>(sm.sQ[4 * t], sm.sQ[4 * t + 1], sm.sQ[4 * t + 2], sm.sQ[4 * t + 3]);
            V3<A> delta = rotate_to_space(q, d[i]);
            V3<A> tau = cross(delta, F[i]);
            sm.sF[3 * a] = F[i].x; sm.sF[3 * a + 1] = F[i].y; sm.sF[3 * a + 2] = F[i].z;
            sm.sT[3 * a] = tau.x; sm.sT[3 * a + 1] = tau.y; sm.sT[3 * a + 2] = tau.z;
            V3<A> x = KIND == STEP_PART2 ? delta : d[i];
            sm.sX[3 * a] = x.x; sm.sX[3 * a + 1] = x.y; sm.sX[3 * a + 2] = x.z;
        }
    }
}

// Fixed-order sum of the tile-local atoms [s, e) of one body.
template <class A>
__device__ __forceinline__ void body_sums(const StepSmem<A>& sm, int s, int e, V3<A>& F, V3<A>& T) {
    F = v3<A>(A(0), A(0), A(0));
    T = F;
    for (int j = s; j < e; j++) {
        F = F + v3<A>(sm.sF[3 * j], sm.sF[3 * j + 1], sm.sF[3 * j + 2]);
        T = T + v3<A>(sm.sT[3 * j], sm.sT[3 * j + 1], sm.sT[3 * j + 2]);
    }
}

// Phase 3, part2: atom velocities v + omega_space x delta.
template <int P, class A>
__device__ __forceinline__ void atom_velocities(const DevSys& S, const DevBuf& B, const StepSmem<A>& sm, int a0, int nat) {
    using V4 = typename Tr<P>::V4;
    V4* vel = (V4*)B.velm;
    for (int a = threadIdx.x; a < nat; a += kThreads) {
        const int t = sm.sBody[a];
        const int loc = __ldg(S.atom_loc + a0 + a);
        V3<A> x = v3<A>(sm.sX[3 * a], sm.sX[3 * a + 1], sm.sX[3 * a + 2]);
        V3<A> w = v3<A>(sm.sW[3 * t], sm.sW[3 * t + 1], sm.sW[3 * t + 2]);
        V3<A> rel = cross(w, x);
        V4 vm = vel[loc];
        vm.x = sm.sRb[3 * t] + (double)rel.x;
        vm.y = sm.sRb[3 * t + 1] + (double)rel.y;
        vm.z = sm.sRb[3 * t + 2] + (double)rel.z;
        vel[loc] = vm;
    }
}

// ------------------------------------------------------------------------------------------
// Double precision: FP64 throughout, the plugin's formulas (RigidBody.cpp, rigidbodyintegrator.cu).
// ------------------------------------------------------------------------------------------
template <int KIND, bool EXACT>
__global__ void __launch_bounds__(kThreads) step_kernel_d(DevSys S, DevBuf B, double dt) {
    constexpr int P = PREC_DOUBLE;
    constexpr int TA = kTileAtomsD, TB = kTileBodies;
    if ((int)blockIdx.x >= S.n_body_tiles) {
        free_atom_tile<P, KIND>(S, B, dt, (int)blockIdx.x - S.n_body_tiles);
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    StepSmem<double> sm;
    sm.carve<TA, TB>(smem);
    const int tid = threadIdx.x;
    const int b0 = __ldg(S.tile_body0 + blockIdx.x), b1 = __ldg(S.tile_body0 + blockIdx.x + 1);
    const int nbt = b1 - b0;
    const int a0 = __ldg(S.atom0 + b0), nat = __ldg(S.atom0 + b1) - a0;
    const int nbp = S.nb_pad;
    double* __restrict__ st = (double*)S.state;

    if (tid < nbt) {
        const int b = b0 + tid;
        for (int c = 0; c < 4; c++) sm.sQ[4 * tid + c] = st[b + (6 + c) * nbp];
        const int s = __ldg(S.atom0 + b) - a0, e = __ldg(S.atom0 + b + 1) - a0;
        for (int j = s; j < e; j++) sm.sBody[j] = (unsigned short)tid;
    }
    __syncthreads();
    atom_forces<P, KIND, double, double>(S, B, sm, a0, nat);
    __syncthreads();
    if (tid < nbt) {
        const int b = b0 + tid;
        V3<double> Fa, Ta;
        body_sums(sm, __ldg(S.atom0 + b) - a0, __ldg(S.atom0 + b + 1) - a0, Fa, Ta);
        V3<double> r = v3<double>(st[b], st[b + nbp], st[b + 2 * nbp]);
        V3<double> v = v3<double>(st[b + 3 * nbp], st[b + 4 * nbp], st[b + 5 * nbp]);
        Q4<double> q = q4<double>(st[b + 6 * nbp], st[b + 7 * nbp], st[b + 8 * nbp], st[b + 9 * nbp]);
        Q4<double> pi = q4<double>(st[b + 10 * nbp], st[b + 11 * nbp], st[b + 12 * nbp], st[b + 13 * nbp]);
        const double invm = __ldg(S.invm + b);
        const V3<double> invI = v3<double>(__ldg(S.invI + b), __ldg(S.invI + b + nbp), __ldg(S.invI + b + 2 * nbp));
        const double halfDt = 0.5 * dt;
        const Q4<double> Ctau = qC(q, Ta);
        const V3<double> dv = Fa * (invm * halfDt);
        const int kicks = KIND == STEP_FUSED ? 2 : 1;
        for (int kk = 0; kk < kicks; kk++) {
            v = v + dv;
            pi = pi + Ctau * dt;
        }
        st[b + 3 * nbp] = v.x; st[b + 4 * nbp] = v.y; st[b + 5 * nbp] = v.z;
        if (KIND == STEP_PART2) {
            V3<double> ws = rotate_to_space(q, mul(invI, qBt(q, pi)) * 0.5);
            sm.sRb[3 * tid] = v.x; sm.sRb[3 * tid + 1] = v.y; sm.sRb[3 * tid + 2] = v.z;
            sm.sW[3 * tid] = ws.x; sm.sW[3 * tid + 1] = ws.y; sm.sW[3 * tid + 2] = ws.z;
        } else {
            r = r + v * dt;
            if (EXACT) {
                const int cls = __ldg(S.cls + b);
                V3<double> I = v3<double>(1.0 / invI.x, 1.0 / invI.y, invI.z != 0.0 ? 1.0 / invI.z : 0.0);
                exact_rotation<double>(cls, I, invI, q, pi, dt);
            } else {
                nosquish_rotation<double>(invI, invI.z != 0.0, q, pi, dt, S.rot_n);
            }
            st[b] = r.x; st[b + nbp] = r.y; st[b + 2 * nbp] = r.z;
            sm.sRb[3 * tid] = r.x; sm.sRb[3 * tid + 1] = r.y; sm.sRb[3 * tid + 2] = r.z;
            sm.sQ[4 * tid] = q.w; sm.sQ[4 * tid + 1] = q.x; sm.sQ[4 * tid + 2] = q.y; sm.sQ[4 * tid + 3] = q.z;
            st[b + 6 * nbp] = q.w; st[b + 7 * nbp] = q.x; st[b + 8 * nbp] = q.y; st[b + 9 * nbp] = q.z;
        }
        st[b + 10 * nbp] = pi.w; st[b + 11 * nbp] = pi.x; st[b + 12 * nbp] = pi.y; st[b + 13 * nbp] = pi.z;
    }
    __syncthreads();
    if (KIND == STEP_PART2) {
        atom_velocities<P, double>(S, B, sm, a0, nat);
    } else {
        for (int a = tid; a < nat; a += kThreads) {
            const int t = sm.sBody[a];
            const int loc = __ldg(S.atom_loc + a0 + a);
            Q4<double> q = q4<double>(sm.sQ[4 * t], sm.sQ[4 * t + 1], sm.sQ[4 * t + 2], sm.sQ[4 * t + 3]);
            V3<double> delta = rotate_to_space(q, v3<double>(sm.sX[3 * a], sm.sX[3 * a + 1], sm.sX[3 * a + 2]));
            PosIO<P>::store(B, loc, v3<double>(sm.sRb[3 * t], sm.sRb[3 * t + 1], sm.sRb[3 * t + 2]), delta);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Single and mixed precision: FP32 arithmetic, float-float body state, rotation increments.
// One 256-thread CTA per tile (<= 256 bodies, <= 1024 body atoms), 3 CTAs per SM. Each body's
// rotation matrix is formed once per phase and kept in shared memory, so the per-atom rebuild
// delta = At(q) d costs 9 FMAs.
// ------------------------------------------------------------------------------------------
struct FSmem {
    static constexpr int TA = kTileAtomsF, TB = kTileBodiesF;
    static constexpr int SF = 0;              // 3 x TA: F
    static constexpr int ST = SF + 3 * TA;    // 3 x TA: torque
    static constexpr int SM = ST + 3 * TA;    // 9 x TB: rotation matrix At(q), row-major per body
    static constexpr int SR = SM + 9 * TB;    // 6 x TB: COM (hi, lo) or COM velocity (double)
    static constexpr int SW = SR + 6 * TB;    // 3 x TB: space-frame omega (part2)
    static constexpr int SB = SW + 3 * TB;    // TA ushort: atom -> tile body
    static constexpr int WORDS = SB + TA / 2;
};

// At(q) as a row-major 3x3 matrix (homogeneous quadratic form, equal to Ct(q, B(q, .))).
__device__ __forceinline__ void rotation_matrix(Q4<float> q, float* m) {
    const float ww = q.w * q.w, xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z, wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    m[0] = ww + xx - yy - zz; m[1] = 2.0f * (xy - wz); m[2] = 2.0f * (xz + wy);
    m[3] = 2.0f * (xy + wz); m[4] = ww - xx + yy - zz; m[5] = 2.0f * (yz - wx);
    m[6] = 2.0f * (xz - wy); m[7] = 2.0f * (yz + wx); m[8] = ww - xx - yy + zz;
}
__device__ __forceinline__ V3<float> mat_vec(const float* m, V3<float> d) {
    return v3<float>(fmaf(m[0], d.x, fmaf(m[1], d.y, m[2] * d.z)), fmaf(m[3], d.x, fmaf(m[4], d.y, m[5] * d.z)),
                     fmaf(m[6], d.x, fmaf(m[7], d.y, m[8] * d.z)));
}

template <int P, int KIND, bool EXACT>
__global__ void __launch_bounds__(kThreadsF, 3) step_kernel_f(DevSys S, DevBuf B, double dt_d) {
    constexpr int TA = kTileAtomsF;
    constexpr int APT = TA / kThreadsF;
    if ((int)blockIdx.x >= S.n_body_tiles) {
        free_atom_tile<P, KIND>(S, B, dt_d, (int)blockIdx.x - S.n_body_tiles);
        return;
    }
    extern __shared__ __align__(16) float fsm[];
    float* sF = fsm + FSmem::SF;
    float* sT = fsm + FSmem::ST;
    float* sM = fsm + FSmem::SM;
    float* sR = fsm + FSmem::SR;
    float* sW = fsm + FSmem::SW;
    unsigned short* sBody = (unsigned short*)(fsm + FSmem::SB);
    const int tid = threadIdx.x;
    const int b0 = __ldg(S.tile_body0 + blockIdx.x), b1 = __ldg(S.tile_body0 + blockIdx.x + 1);
    const int nbt = b1 - b0;
    const int a0 = __ldg(S.atom0 + b0), nat = __ldg(S.atom0 + b1) - a0;
    const int nbp = S.nb_pad;
    float* __restrict__ ghi = (float*)S.state;  // state rows 0..13 (hi)
    float* __restrict__ glo = ghi + 14 * nbp;   // rows 14..27 (lo)
    const float dt = (float)dt_d;

    // Phase 0: rotation matrix of the current orientation; atoms -> tile-local body
    if (tid < nbt) {
        const int b = b0 + tid;
        rotation_matrix(q4<float>(ghi[b + 6 * nbp], ghi[b + 7 * nbp], ghi[b + 8 * nbp], ghi[b + 9 * nbp]), sM + 9 * tid);
        const int s0 = __ldg(S.atom0 + b) - a0, e0 = __ldg(S.atom0 + b + 1) - a0;
        for (int j = s0; j < e0; j++) sBody[j] = (unsigned short)tid;
    }
    __syncthreads();

    // Phase 1: per-atom force, displacement from the COM, torque (all loads issued first)
    {
        const float* __restrict__ dg = (const float*)S.d;
        int loc[APT];
        V3<float> F[APT], d[APT];
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * kThreadsF;
            loc[i] = a < nat ? __ldg(S.atom_loc + a0 + a) : 0;
        }
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * kThreadsF;
            if (a < nat) {
                const int k = a0 + a;
                d[i] = v3<float>(__ldg(dg + k), __ldg(dg + k + S.nba_pad), __ldg(dg + k + 2 * S.nba_pad));
                F[i] = load_force<float>(B.force, loc[i], B.stride);
            }
        }
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * kThreadsF;
            if (a < nat) {
                const V3<float> delta = mat_vec(sM + 9 * sBody[a], d[i]);
                const V3<float> tau = cross(delta, F[i]);
                sF[3 * a] = F[i].x; sF[3 * a + 1] = F[i].y; sF[3 * a + 2] = F[i].z;
                sT[3 * a] = tau.x; sT[3 * a + 1] = tau.y; sT[3 * a + 2] = tau.z;
            }
        }
    }
    __syncthreads();

    // Phase 2: kicks, drift and rotation on the float-float state
    if (tid < nbt) {
        const int b = b0 + tid;
        ff x[14];
#pragma unroll
        for (int c = 0; c < 14; c++) x[c] = ff{ghi[b + c * nbp], glo[b + c * nbp]};
        const float* bc = S.bconst;
        const float invm = __ldg(bc + b), invm_lo = __ldg(bc + b + 7 * nbp);
        Rotor R;
        R.invI = v3<float>(__ldg(bc + b + nbp), __ldg(bc + b + 2 * nbp), __ldg(bc + b + 3 * nbp));
        R.g01 = __ldg(bc + b + 4 * nbp);
        R.g12 = __ldg(bc + b + 5 * nbp);
        R.g02 = __ldg(bc + b + 6 * nbp);
        R.invI_lo = v3<float>(__ldg(bc + b + 8 * nbp), __ldg(bc + b + 9 * nbp), __ldg(bc + b + 10 * nbp));
        V3<float> Fa = v3<float>(0.f, 0.f, 0.f), Ta = Fa;
        {
            const int s0 = __ldg(S.atom0 + b) - a0, e0 = __ldg(S.atom0 + b + 1) - a0;
            for (int j = s0; j < e0; j++) {
                Fa = Fa + v3<float>(sF[3 * j], sF[3 * j + 1], sF[3 * j + 2]);
                Ta = Ta + v3<float>(sT[3 * j], sT[3 * j + 1], sT[3 * j + 2]);
            }
        }
        const Q4<float> qh = q4<float>(x[6].hi, x[7].hi, x[8].hi, x[9].hi);
        // half kicks: COM velocity by F/m dt/2 (1/m as hi + lo), pi by C(q, tau) dt
        // (RigidBodySystem.cpp:178-179, :200-201); the fused step applies both halves at once
        const float kick = KIND == STEP_FUSED ? dt : 0.5f * dt;
        const float piscale = KIND == STEP_FUSED ? 2.0f * dt : dt;
        const Q4<float> Ctau = qC(qh, Ta) * piscale;
        x[3] = ff_acc(x[3], fmaf(Fa.x, invm_lo * kick, Fa.x * (invm * kick)));
        x[4] = ff_acc(x[4], fmaf(Fa.y, invm_lo * kick, Fa.y * (invm * kick)));
        x[5] = ff_acc(x[5], fmaf(Fa.z, invm_lo * kick, Fa.z * (invm * kick)));
        x[10] = ff_acc(x[10], Ctau.w); x[11] = ff_acc(x[11], Ctau.x);
        x[12] = ff_acc(x[12], Ctau.y); x[13] = ff_acc(x[13], Ctau.z);
        const Q4<float> ph = q4<float>(x[10].hi, x[11].hi, x[12].hi, x[13].hi);
        if (KIND == STEP_PART2) {
            const V3<float> ws = rotate_to_space(qh, mul(R.invI, qBt(qh, ph)) * 0.5f);
            double* v = (double*)(sR + 6 * tid);
            v[0] = (double)x[3].hi + (double)x[3].lo;
            v[1] = (double)x[4].hi + (double)x[4].lo;
            v[2] = (double)x[5].hi + (double)x[5].lo;
            sW[3 * tid] = ws.x; sW[3 * tid + 1] = ws.y; sW[3 * tid + 2] = ws.z;
        } else {
#pragma unroll
            for (int c = 0; c < 3; c++) x[c] = ff_acc(x[c], fmaf(x[3 + c].hi, dt, x[3 + c].lo * dt));  // drift
            const V3<float> L = qBt(qh, ph) * 0.5f;
            Q4<float> dr;
            if (EXACT) dr = dq_exact(__ldg(S.cls + b), L, R, dt);
            else dr = nosquish_increment(L, R, R.invI.z != 0.0f, dt, S.rot_n);
            const Q4<float> dq = qmul(qh, dr), dp = qmul(ph, dr);
            x[6] = ff_acc(x[6], dq.w); x[7] = ff_acc(x[7], dq.x); x[8] = ff_acc(x[8], dq.y); x[9] = ff_acc(x[9], dq.z);
            x[10] = ff_acc(x[10], dp.w); x[11] = ff_acc(x[11], dp.x);
            x[12] = ff_acc(x[12], dp.y); x[13] = ff_acc(x[13], dp.z);
            // renormalise q: eps = |q|^2 - 1 from exact squares, q <- q (1 - eps/2)
#pragma unroll
            for (int c = 6; c < 10; c++) x[c] = ff_norm(x[c]);
            ff n2 = ff{0.0f, 0.0f};
            float tail = 0.0f;
#pragma unroll
            for (int c = 6; c < 10; c++) {
                const float p = x[c].hi * x[c].hi;
                tail += fmaf(x[c].hi, x[c].hi, -p) + 2.0f * x[c].hi * x[c].lo;
                n2 = ff_acc(n2, p);
            }
            const float eps = ((n2.hi - 1.0f) + n2.lo) + tail;
#pragma unroll
            for (int c = 6; c < 10; c++) x[c] = ff_norm(ff_acc(x[c], -0.5f * eps * x[c].hi));
#pragma unroll
            for (int c = 0; c < 3; c++) {
                x[c] = ff_norm(x[c]);
                sR[6 * tid + 2 * c] = x[c].hi;
                sR[6 * tid + 2 * c + 1] = x[c].lo;
            }
            // positions are rebuilt from exactly the r and q stored below, so that they are a
            // function of the stored state alone (sync_positions_kernel rebuilds them identically)
            rotation_matrix(q4<float>(x[6].hi, x[7].hi, x[8].hi, x[9].hi), sM + 9 * tid);
        }
#pragma unroll
        for (int c = 0; c < 14; c++) {
            const bool normed = KIND != STEP_PART2 && (c < 3 || (c >= 6 && c < 10));
            const ff y = normed ? x[c] : ff_norm(x[c]);
            ghi[b + c * nbp] = y.hi;
            glo[b + c * nbp] = y.lo;
        }
    }
    __syncthreads();

    // Phase 3: positions (part1, fused) or velocities (part2); d is read again (an L2 hit after
    // phase 1) and, for part2, delta rebuilt from the unchanged orientation
    const float* __restrict__ dg3 = (const float*)S.d;
    for (int a = tid; a < nat; a += kThreadsF) {
        const int t = sBody[a];
        const int loc = __ldg(S.atom_loc + a0 + a);
        const int k = a0 + a;
        const V3<float> x = v3<float>(__ldg(dg3 + k), __ldg(dg3 + k + S.nba_pad), __ldg(dg3 + k + 2 * S.nba_pad));
        if (KIND == STEP_PART2) {
            using V4 = typename Tr<P>::V4;
            const V3<float> rel = cross(v3<float>(sW[3 * t], sW[3 * t + 1], sW[3 * t + 2]), mat_vec(sM + 9 * t, x));
            const double* v = (const double*)(sR + 6 * t);
            V4* vel = (V4*)B.velm;
            V4 vm = vel[loc];
            vm.x = v[0] + (double)rel.x;
            vm.y = v[1] + (double)rel.y;
            vm.z = v[2] + (double)rel.z;
            vel[loc] = vm;
        } else {
            const V3<float> delta = mat_vec(sM + 9 * t, x);
            const float* rf = sR + 6 * t;
            // posq.w (the charge) is left untouched: x, y in one 8-byte store, z in 4 bytes
            float* pq = (float*)B.posq + 4 * (size_t)loc;
            if (P == PREC_MIXED) {
                const ff px = ff_add(ff{rf[0], rf[1]}, delta.x);
                const ff py = ff_add(ff{rf[2], rf[3]}, delta.y);
                const ff pz = ff_add(ff{rf[4], rf[5]}, delta.z);
                *(float2*)pq = make_float2(px.hi, py.hi);
                pq[2] = pz.hi;
                ((float4*)B.corr)[loc] = make_float4(px.lo, py.lo, pz.lo, 0.0f);
            } else {
                *(float2*)pq = make_float2(rf[0] + (rf[1] + delta.x), rf[2] + (rf[3] + delta.y));
                pq[2] = rf[4] + (rf[5] + delta.z);
            }
        }
    }
}

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
constexpr size_t step_smem_f() { return (size_t)FSmem::WORDS * 4; }

size_t step_smem_bytes(int prec) { return prec == PREC_DOUBLE ? step_smem_d() : step_smem_f(); }

template <int P, int KIND, bool EXACT> struct StepKernel {
    static constexpr auto fn() { return step_kernel_f<P, KIND, EXACT>; }
};
template <int KIND, bool EXACT> struct StepKernel<PREC_DOUBLE, KIND, EXACT> {
    static constexpr auto fn() { return step_kernel_d<KIND, EXACT>; }
};

template <int P, int KIND, bool EXACT>
static int launch_step_t(const DevSys& s, const DevBuf& b, double dt, cudaStream_t stream) {
    static bool configured = false;
    static int wave = 0;  // resident CTAs of one full wave (float kernels are persistent)
    const size_t smem = P == PREC_DOUBLE ? step_smem_d() : step_smem_f();
    const int threads = P == PREC_DOUBLE ? kThreads : kThreadsF;
    auto kernel = StepKernel<P, KIND, EXACT>::fn();
    if (!configured) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return -1;
        int dev = 0, sms = 0, per_sm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess)
            return -1;
        wave = sms * (per_sm > 0 ? per_sm : 1);
        configured = true;
    }
    const int tiles = s.n_body_tiles + s.n_free_tiles;
    if (tiles == 0) return 0;
    const int grid = tiles;
    (void)wave;
    kernel<<<grid, threads, smem, stream>>>(s, b, dt);
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
