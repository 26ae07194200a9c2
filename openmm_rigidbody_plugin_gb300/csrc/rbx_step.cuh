// rbx_step.cuh -- the step kernels of the rigid-body integrator (sm_103a), as templates shared by
// rbx_kernels.cu (plain steps) and rbx_refined.cu (steps that also accumulate the refined-energy
// stencils). Each translation unit instantiates its own template arguments only.
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
//      (single/mixed: phase 1's loads are issued before phase 0, so that the slot -> force
//      dependency overlaps it: 4 % faster)
//   2. one thread per body sums its atoms' F and tau in a fixed order (deterministic, no
//      atomics; a whole warp per body for bodies of more than 32 atoms), applies the half
//      kick(s), drift and free rotation, and writes its state;
//   3. one thread per atom writes the new position r + At(q) d (or, for part2, the velocity
//      v + omega x delta) to its device slot.
// Free atoms live in separate tiles of the same launch (velocity Verlet), interleaved with the
// body tiles (block_tile).
// step_kernel_d runs double precision in FP64 throughout (the exact rotation in increment form,
// rbx_math.cuh). step_kernel_f runs single and mixed precision on the FP32 pipe: float-float body
// state, FP32 rotation increments (rbx_fast.cuh), FP32 per-atom work.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include "rbx_fast.cuh"
#include "rbx_internal.h"
#include "rbx_math.cuh"
#include "rbx_tiles.h"

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
    using RS = float;  // refined-energy stencil sums
    static constexpr bool kCorr = false;
};
template <> struct Tr<PREC_MIXED> {
    using A = float;
    using R = double;  // FP64 free-atom form (velm is FP64): refined-energy kernels, free_atom_ff's fallback
    using D = float;
    using P4 = float4;
    using V4 = dq4;
    using RS = float;
    static constexpr bool kCorr = true;
};
template <> struct Tr<PREC_DOUBLE> {
    using A = double;
    using R = double;
    using D = double;
    using P4 = dq4;
    using V4 = dq4;
    using RS = double;
    static constexpr bool kCorr = false;
};

// Fixed-point force (scale 2^32) to floating point. The FP32 form converts the two 32-bit halves
// (hi + lo 2^-32, within an ulp of the correctly rounded value): a 64-bit integer conversion
// occupies GB300's narrow FP64 pipe, and this one measured 1 % faster per step.
template <class T> __device__ __forceinline__ T fixed_to(long long v);
template <> __device__ __forceinline__ float fixed_to<float>(long long v) {
    const int hi = (int)(v >> 32);
    const unsigned int lo = (unsigned int)v;
    return fmaf((float)lo, 0x1p-32f, (float)hi);
}
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


// Failure detector: the new state of a body or free atom is checked for a non-finite value (NaN
// or infinity; the check is one sum of already loaded values); a failing unit gets its flag byte
// and the status counter one increment. Finite values never take the branch.
__device__ __forceinline__ bool finite_f(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }
__device__ __forceinline__ bool finite_d(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}
static __device__ __noinline__ void flag_failure(unsigned int* status, uint8_t* flags, int i) {
    if (!status) return;
    flags[i] = 1;
    atomicAdd(status, 1u);
}

// Shared memory of the double-precision step kernel: sF, sT, sX 3*TA each; sQ 4*TB; sRb 3*TB
// (double); sW 3*TB; sBody TA (uint16); sBig one word per warp.
constexpr size_t step_smem_d() {
    constexpr int TA = kTileAtomsD, TB = kTileBodies;
    return (size_t)3 * 3 * TA * sizeof(double) + 4 * TB * sizeof(double) + 3 * TB * sizeof(double) +
           3 * TB * sizeof(double) + TA * sizeof(unsigned short) + (kThreads / 32) * sizeof(unsigned) + 64;
}

// ------------------------------------------------------------------------------------------
// Mixed-precision free atoms in float-float on the FP32 pipe
// ------------------------------------------------------------------------------------------
// Float-float from a double by integer operations: hi is the double truncated to 24 significant
// bits, lo the 29-bit remainder rounded to a float (|hi + lo - d| <= 2^-47 |d|). Zero is exact.
// Returns false for |d| outside [2^-74, 2^127) (the remainder or hi would leave the normal float
// range), infinities and NaN.
__device__ __forceinline__ bool ff_from_double(double d, ff& out) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned int e = (unsigned int)(u >> 52) & 0x7FFu;
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    const unsigned int sign = (unsigned int)(u >> 32) & 0x80000000u;
    if (e == 0u && m == 0ull) {
        out = ff{__uint_as_float(sign), 0.0f};
        return true;
    }
    if (e < 949u || e > 1150u) return false;
    const float hi = __uint_as_float(sign | ((e - 896u) << 23) | (unsigned int)(m >> 29));  // exponent e-1023+127
    const float scale = __uint_as_float((e - 948u) << 23);                                   // 2^(e-1075)
    const float lo = __fmul_rn((float)(unsigned int)(m & 0x1FFFFFFFull), scale);
    out = ff{hi, sign ? -lo : lo};
    return true;
}

// a + b as an exact float-float (two-sum).
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// a * b in float-float (the exact product of the high words by FMA, plus the cross terms).
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    const float hi = __fadd_rn(p, e);
    return ff{hi, __fsub_rn(e, __fsub_rn(hi, p))};
}

__device__ __forceinline__ ff ff_add_ff(ff a, ff b) { return ff_add(ff_add(a, b.hi), b.lo); }

// Fixed-point force (scale 2^32) as float-float: the high word, the top 24 bits of the low word
// and its last 8 bits are each exact floats (the first for |F| < 2^24 kJ/mol/nm).
__device__ __forceinline__ ff fixed_to_ff(long long v) {
    const int hi = (int)(v >> 32);
    const unsigned int lo = (unsigned int)v;
    return ff_add(ff_two_sum((float)hi, __fmul_rn((float)(lo >> 8), 0x1p-24f)), __fmul_rn((float)(lo & 0xFFu), 0x1p-32f));
}

// The free atom's velocity Verlet in mixed precision (rigidbodyintegrator.cu:302-310, :351-358)
// in float-float arithmetic. velm is double4 in OpenMM's mixed mode: its words are split by
// ff_from_double and the new velocity is joined by one FP64 add per component, so an atom issues
// 9 FP64 instructions instead of about 47 on GB300's narrow FP64 pipe. With the free-atom tiles
// interleaved, this measured 0.1374 against 0.1383 ms per step at 1e6 bodies, within run-to-run
// variation: the FP64 pipe no longer limited them. Positions are the
// float-float pair posq + posqCorrection. Returns false, having written nothing, when a velocity,
// 1/m or the step lies outside the split's range; the caller then runs the FP64 form.
template <int KIND>
__device__ __forceinline__ bool free_atom_ff(const DevBuf& B, double dt_d, int loc, double& vsum) {
    dq4* vel = (dq4*)B.velm;
    dq4 vm = vel[loc];
    ff v[3], w, dt;
    if (!ff_from_double(vm.x, v[0]) || !ff_from_double(vm.y, v[1]) || !ff_from_double(vm.z, v[2]) ||
        !ff_from_double(vm.w, w) || !ff_from_double(dt_d, dt))
        return false;
    const ff wh = ff_mul(w, ff{0.5f * dt.hi, 0.5f * dt.lo});  // (1/m) dt/2; halving is exact
    const long long f[3] = {__ldg(B.force + loc), __ldg(B.force + loc + B.stride), __ldg(B.force + loc + 2 * B.stride)};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const ff dv = ff_mul(fixed_to_ff(f[c]), wh);
        if (KIND != STEP_PART1) v[c] = ff_add_ff(v[c], dv);  // second half kick of step n
        if (KIND != STEP_PART2) v[c] = ff_add_ff(v[c], dv);  // first half kick of the next step
    }
    if (KIND != STEP_PART2) {  // drift: posq + posqCorrection += v dt
        float4* pq = (float4*)B.posq;
        float4 p = pq[loc];
        const float4 cr = ((const float4*)B.corr)[loc];
        const ff x0 = ff_add_ff(ff{p.x, cr.x}, ff_mul(v[0], dt));
        const ff x1 = ff_add_ff(ff{p.y, cr.y}, ff_mul(v[1], dt));
        const ff x2 = ff_add_ff(ff{p.z, cr.z}, ff_mul(v[2], dt));
        p.x = x0.hi; p.y = x1.hi; p.z = x2.hi;
        pq[loc] = p;
        ((float4*)B.corr)[loc] = make_float4(x0.lo, x1.lo, x2.lo, 0.0f);
    }
    vm.x = (double)v[0].hi + (double)v[0].lo;
    vm.y = (double)v[1].hi + (double)v[1].lo;
    vm.z = (double)v[2].hi + (double)v[2].lo;
    vel[loc] = vm;
    vsum = vm.x + vm.y + vm.z;
    return true;
}

// Free atoms (velocity Verlet). With REF, part1 and fused steps store alpha = F(t) h/m, and part2
// writes the free atom's refined-energy terms at t+h (the freeAtomsDot stencil of
// CudaRigidBodyKernels.cpp:406-438 and the refinedKineticEnergies / potentialEnergyRefinement
// terms of rigidbodyintegrator.cu:433-469): the kinetic-energy correction
// (m/12) v(t+h).(alpha - beta), beta = F(t+h) h/m, which is (m/2) v(t+h).s/(6h) - (m/2)|v(t+h)|^2
// for the stencil s = h[-v(t-h/2) + 5 v(t+h/2) + 2 v(t+3h/2)], and |F(t+h)|^2/m.
template <int P, int KIND, bool REF>
__device__ __forceinline__ void free_atom_tile(const DevSys& S, const DevBuf& B, double dt, int ft) {
    using T = typename Tr<P>::R;  // free-atom velocity/position arithmetic
    using V4 = typename Tr<P>::V4;
    using RS = typename Tr<P>::RS;
    const int j = ft * (int)blockDim.x + (int)threadIdx.x;
    if (j >= S.nf) return;
    const int loc = __ldg(S.free_loc + j);
    if constexpr (P == PREC_MIXED && !REF) {
        double vsum = 0.0;
        if (free_atom_ff<KIND>(B, dt, loc, vsum)) {
            if (!finite_d(vsum)) flag_failure(S.status, S.free_bad, j);
            return;
        }
    }
    V4* vel = (V4*)B.velm;
    V4 vm = vel[loc];
    V3<T> v = v3<T>((T)vm.x, (T)vm.y, (T)vm.z);
    const T w = (T)vm.w;
    const T halfDt = T(0.5) * (T)dt;
    const V3<T> F = load_force<T>(B.force, loc, B.stride);
    V3<T> dv = F * (w * halfDt);
    if (KIND != STEP_PART1) v = v + dv;  // second half kick of step n (rigidbodyintegrator.cu:351-358)
    if (REF && KIND == STEP_PART2) {
        const RS* st = (const RS*)S.ref_start + kRefBodyRows * (size_t)S.nb_pad;
        const V3<T> al = v3<T>((T)st[j], (T)st[j + S.nf_pad], (T)st[j + 2 * S.nf_pad]);
        float* out = S.ref_out + 3 * (size_t)S.nb_pad;
        out[j] = w != T(0) ? (float)(dot(v, al - dv * T(2)) / (T(12) * w)) : 0.0f;
        out[j + S.nf_pad] = (float)(dot(F, F) * w);
    }
    if (KIND != STEP_PART2) {            // first half kick and drift of the next step (:302-310)
        if (REF) {
            RS* st = (RS*)S.ref_start + kRefBodyRows * (size_t)S.nb_pad;
            st[j] = (RS)(dv.x * T(2)); st[j + S.nf_pad] = (RS)(dv.y * T(2)); st[j + 2 * S.nf_pad] = (RS)(dv.z * T(2));
        }
        v = v + dv;
        V3<double> x = PosIO<P>::load(B, loc);
        V3<double> nx = x + cvt<double>(v * (T)dt);
        PosIO<P>::store(B, loc, nx, v3<T>(T(0), T(0), T(0)));
    }
    vm.x = v.x; vm.y = v.y; vm.z = v.z;
    vel[loc] = vm;
    if (!finite_d((double)(v.x + v.y + v.z))) flag_failure(S.status, S.free_bad, j);
}

// Tile of this block (rbx_tiles.h): the body tile (>= 0) or -1 - the free-atom tile.
__device__ __forceinline__ int block_tile(const DevSys& S) {
    return tile_of_block((int)blockIdx.x, S.n_body_tiles, S.n_free_tiles);
}

// Shared-memory carve-up common to both step kernels.
template <class A> struct StepSmem {
    A *sF, *sT, *sX, *sQ, *sW;
    double* sRb;
    unsigned short* sBody;
    unsigned* sBig;  // large-body ballots, one word per warp
    template <int TA, int TB> __device__ __forceinline__ void carve(unsigned char* smem) {
        sF = (A*)smem;
        sT = sF + 3 * TA;
        sX = sT + 3 * TA;
        sQ = sX + 3 * TA;
        sRb = (double*)(sQ + 4 * TB);
        sW = (A*)(sRb + 3 * TB);
        sBody = (unsigned short*)(sW + 3 * TB);
        sBig = (unsigned*)(sBody + TA);
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

// Bodies of more than a warp's atoms are summed by a whole warp instead of one thread: lane l adds
// the atoms s+l, s+l+32, ... in order and a fixed butterfly of shuffles joins the lanes, so a
// 1024-atom body costs 32 dependent additions instead of 1024 (the plugin sums serially,
// rigidbodyintegrator.cu:367-373). Phase 0 records the tile's large bodies as one ballot per warp
// (masks[w], bit l: tile body 32w + l); they are dealt round-robin to the warps in that order.
// The sums are a function of the body's atoms alone, not of the tile or the warp that forms them.
// This path is compiled into separate kernels (LARGE), launched only for integrators that have such
// bodies (DevSys::large), so that the common case carries none of it.

// The sums of tile body t go to outF[os t + c] and outT[os t + c], c = 0, 1, 2 (out of line: the
// branch is rare and stays out of the callers' register allocation).
template <int NW, class A>
__device__ __noinline__ void warp_body_sums(const unsigned* masks, const int* __restrict__ atom0, int b0, int a0,
                                            const A* sF, const A* sT, A* outF, A* outT, int os) {
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    int k = 0;
    for (int m = 0; m < NW; m++) {
        unsigned bits = masks[m];
        while (bits) {
            const int t = 32 * m + __ffs(bits) - 1;
            bits &= bits - 1;
            if (k++ % NW != warp) continue;
            const int s = __ldg(atom0 + b0 + t) - a0, e = __ldg(atom0 + b0 + t + 1) - a0;
            A f[6] = {A(0), A(0), A(0), A(0), A(0), A(0)};
            for (int j = s + lane; j < e; j += 32) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    f[c] += sF[3 * j + c];
                    f[3 + c] += sT[3 * j + c];
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                for (int c = 0; c < 6; c++) f[c] += __shfl_xor_sync(0xffffffffu, f[c], o);
            }
            if (lane == 0) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    outF[os * t + c] = f[c];
                    outT[os * t + c] = f[3 + c];
                }
            }
        }
    }
}

// Number of large bodies in the tile (block-uniform).
template <int NW> __device__ __forceinline__ int count_large(const unsigned* masks) {
    int n = 0;
#pragma unroll
    for (int m = 0; m < NW; m++) n += __popc(masks[m]);
    return n;
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
// Free rotation of (q, pi) by dt in the integrator's rotation mode (double precision).
template <bool EXACT>
__device__ __forceinline__ void rotate_d(const DevSys& S, int b, V3<double> invI, Q4<double>& q, Q4<double>& pi,
                                         double dt) {
    if (EXACT) {
        const int cls = __ldg(S.cls + b);
        V3<double> I = v3<double>(1.0 / invI.x, 1.0 / invI.y, invI.z != 0.0 ? 1.0 / invI.z : 0.0);
        exact_rotation<double>(cls, I, invI, q, pi, dt);
    } else {
        nosquish_rotation<double>(invI, invI.z != 0.0, q, pi, dt, S.rot_n);
    }
}

// Residency per SM: 3 CTAs for NO-SQUISH (80 registers; shared memory allows 3), 2 for the exact
// rotation (128), 1 with the refined-energy stencils.
template <int KIND, bool EXACT, bool REF, bool LARGE>
__global__ void __launch_bounds__(kThreads, REF ? 1 : EXACT ? 2 : 3) step_kernel_d(DevSys S, DevBuf B, double dt) {
    constexpr int P = PREC_DOUBLE;
    constexpr int TA = kTileAtomsD, TB = kTileBodies;
    const int tile = block_tile(S);
    if (tile < 0) {
        free_atom_tile<P, KIND, REF>(S, B, dt, -1 - tile);
        return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    StepSmem<double> sm;
    sm.carve<TA, TB>(smem);
    const int tid = threadIdx.x;
    const int b0 = __ldg(S.tile_body0 + tile), b1 = __ldg(S.tile_body0 + tile + 1);
    const int nbt = b1 - b0;
    const int a0 = __ldg(S.atom0 + b0), nat = __ldg(S.atom0 + b1) - a0;
    const int nbp = S.nb_pad;
    double* __restrict__ st = (double*)S.state;

    bool big = false;
    if (tid < nbt) {
        const int b = b0 + tid;
        for (int c = 0; c < 4; c++) sm.sQ[4 * tid + c] = st[b + (6 + c) * nbp];
        const int s = __ldg(S.atom0 + b) - a0, e = __ldg(S.atom0 + b + 1) - a0;
        for (int j = s; j < e; j++) sm.sBody[j] = (unsigned short)tid;
        big = e - s > kWarpBody;
    }
    if (LARGE) {
        const unsigned m = __ballot_sync(0xffffffffu, big);
        if ((tid & 31) == 0) sm.sBig[tid >> 5] = m;
    }
    __syncthreads();
    atom_forces<P, KIND, double, double>(S, B, sm, a0, nat);
    __syncthreads();
    if (LARGE && count_large<kThreads / 32>(sm.sBig)) {
        // large bodies' sums parked in sRb (force) and sW (torque) of their tile body
        warp_body_sums<kThreads / 32>(sm.sBig, S.atom0, b0, a0, sm.sF, sm.sT, sm.sRb, sm.sW, 3);
        __syncthreads();
    }
    if (tid < nbt) {
        const int b = b0 + tid;
        V3<double> Fa, Ta;
        const int s = __ldg(S.atom0 + b) - a0, e = __ldg(S.atom0 + b + 1) - a0;
        if (LARGE && e - s > kWarpBody) {
            Fa = v3<double>(sm.sRb[3 * tid], sm.sRb[3 * tid + 1], sm.sRb[3 * tid + 2]);
            Ta = v3<double>(sm.sW[3 * tid], sm.sW[3 * tid + 1], sm.sW[3 * tid + 2]);
        } else {
            body_sums(sm, s, e, Fa, Ta);
        }
        V3<double> r = v3<double>(st[b], st[b + nbp], st[b + 2 * nbp]);
        V3<double> v = v3<double>(st[b + 3 * nbp], st[b + 4 * nbp], st[b + 5 * nbp]);
        Q4<double> q = q4<double>(st[b + 6 * nbp], st[b + 7 * nbp], st[b + 8 * nbp], st[b + 9 * nbp]);
        Q4<double> pi = q4<double>(st[b + 10 * nbp], st[b + 11 * nbp], st[b + 12 * nbp], st[b + 13 * nbp]);
        const double invm = __ldg(S.invm + b);
        const V3<double> invI = v3<double>(__ldg(S.invI + b), __ldg(S.invI + b + nbp), __ldg(S.invI + b + 2 * nbp));
        const double halfDt = 0.5 * dt;
        const Q4<double> Ctau = qC(q, Ta);
        const V3<double> dv = Fa * (invm * halfDt);
        const Q4<double> pin = pi;
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
            if (REF) {
                // end of the stencils at t+h (rigidbodyintegrator.cu:380-384) and the body's terms of
                // refinedKineticEnergies / potentialEnergyRefinement (:433-469), as corrections:
                // KE_t: (m/12) v.(alpha - beta); KE_r: qdot.pi/(6h) - L.I^-1.L/2 with qdot the
                // quaternion stencil closed by q(t+2h) - q(t+h), the virtual rotation from
                // (q(t+h), pi(t+h) + C(q,tau) h) (:238-243), projected off q.
                const double* rs = (const double*)S.ref_start;
                const V3<double> al = v3<double>(rs[b], rs[b + nbp], rs[b + 2 * nbp]);
                Q4<double> qd = q4<double>(rs[b + 3 * nbp], rs[b + 4 * nbp], rs[b + 5 * nbp], rs[b + 6 * nbp]);
                const double dkt = dot(v, al - Fa * (invm * dt)) / (12.0 * invm);
                Q4<double> qf = q, pf = pi + Ctau * dt;
                rotate_d<EXACT>(S, b, invI, qf, pf, dt);
                qd = qd + (qf - q);
                qd = qd - q * dot(qd, q);
                const V3<double> L = qBt(q, pi) * 0.5;
                const double dkr = dot(qd, pi) / (6.0 * dt) - 0.5 * dot(L, mul(invI, L));
                const V3<double> tb = qBt(q, Ctau);
                const double u = dot(Fa, Fa) * invm + dot(tb, mul(invI, tb));
                S.ref_out[b] = (float)dkt; S.ref_out[b + nbp] = (float)dkr; S.ref_out[b + 2 * nbp] = (float)u;
            }
        } else {
            r = r + v * dt;
            const Q4<double> q0 = q;
            rotate_d<EXACT>(S, b, invI, q, pi, dt);
            if (REF) {
                // start of the stencils at t (rigidbodyintegrator.cu:318-321): alpha = F(t) h/m and
                // 0.5 [q(t-h) - q(t)] + 2.5 [q(t+h) - q(t)]; q(t-h) is the virtual rotation by -h from
                // (q(t), pi(t) - C(q,tau) h), taken as the rotation by +h with the momentum reversed
                // (the free rotor is time-reversible)
                Q4<double> qb = q0, pb = (KIND == STEP_FUSED ? pin : pin - Ctau * dt) * -1.0;
                rotate_d<EXACT>(S, b, invI, qb, pb, dt);
                const Q4<double> sq = (qb - q0) * 0.5 + (q - q0) * 2.5;
                const V3<double> al = Fa * (invm * dt);
                double* rs = (double*)S.ref_start;
                rs[b] = al.x; rs[b + nbp] = al.y; rs[b + 2 * nbp] = al.z;
                rs[b + 3 * nbp] = sq.w; rs[b + 4 * nbp] = sq.x; rs[b + 5 * nbp] = sq.y; rs[b + 6 * nbp] = sq.z;
            }
            st[b] = r.x; st[b + nbp] = r.y; st[b + 2 * nbp] = r.z;
            sm.sRb[3 * tid] = r.x; sm.sRb[3 * tid + 1] = r.y; sm.sRb[3 * tid + 2] = r.z;
            sm.sQ[4 * tid] = q.w; sm.sQ[4 * tid + 1] = q.x; sm.sQ[4 * tid + 2] = q.y; sm.sQ[4 * tid + 3] = q.z;
            st[b + 6 * nbp] = q.w; st[b + 7 * nbp] = q.x; st[b + 8 * nbp] = q.y; st[b + 9 * nbp] = q.z;
        }
        st[b + 10 * nbp] = pi.w; st[b + 11 * nbp] = pi.x; st[b + 12 * nbp] = pi.y; st[b + 13 * nbp] = pi.z;
        const double chk = ((r.x + r.y) + (r.z + v.x)) + ((v.y + v.z) + (q.w + q.x)) + ((q.y + q.z) + (pi.w + pi.x)) +
                           (pi.y + pi.z);
        if (!finite_d(chk)) flag_failure(S.status, S.body_bad, b);
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
// One CTA of NT threads per tile (<= NT bodies, <= 4 NT body atoms), 768 threads per SM. Each
// body's rotation matrix is formed once per phase and kept in shared memory, so the per-atom
// rebuild delta = At(q) d costs 9 FMAs.
// ------------------------------------------------------------------------------------------
template <int NT> struct FSmem {
    static constexpr int TA = 4 * NT, TB = NT;
    static constexpr int SF = 0;              // 3 x TA: F
    static constexpr int ST = SF + 3 * TA;    // 3 x TA: torque
    static constexpr int SM = ST + 3 * TA;    // 9 x TB: rotation matrix At(q), row-major per body
    static constexpr int SR = SM + 9 * TB;    // 6 x TB: COM (hi, lo) or COM velocity (double)
    static constexpr int SW = SR + 6 * TB;    // 3 x TB: space-frame omega (part2)
    static constexpr int SB = SW + 3 * TB;    // TA ushort: atom -> tile body
    static constexpr int SG = SB + TA / 2;    // one word per warp: large-body ballots
    static constexpr int WORDS = SG + NT / 32;
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

// FP32 rotation increment dr (q <- q (x) (1 + dr)) for body angular momentum L over dt.
template <bool EXACT>
__device__ __forceinline__ Q4<float> rotation_increment(const DevSys& S, int b, V3<float> L, const Rotor& R, float dt) {
    if (EXACT) return dq_exact(__ldg(S.cls + b), L, R, dt);
    return nosquish_increment(L, R, R.invI.z != 0.0f, dt, S.rot_n);
}

template <int P, int KIND, bool EXACT, bool REF, int NT, bool LARGE>
__global__ void __launch_bounds__(NT, 768 / NT) step_kernel_f(DevSys S, DevBuf B, double dt_d) {
    using FSmem = rbx::FSmem<NT>;
    constexpr int APT = 4;  // body atoms per thread in phase 1
    const int tile = block_tile(S);
    if (tile < 0) {
        free_atom_tile<P, KIND, REF>(S, B, dt_d, -1 - tile);
        return;
    }
    extern __shared__ __align__(16) float fsm[];
    float* sF = fsm + FSmem::SF;
    float* sT = fsm + FSmem::ST;
    float* sM = fsm + FSmem::SM;
    float* sR = fsm + FSmem::SR;
    float* sW = fsm + FSmem::SW;
    unsigned short* sBody = (unsigned short*)(fsm + FSmem::SB);
    unsigned* sBig = (unsigned*)(fsm + FSmem::SG);
    const int tid = threadIdx.x;
    const int b0 = __ldg(S.tile_body0 + tile), b1 = __ldg(S.tile_body0 + tile + 1);
    const int nbt = b1 - b0;
    const int a0 = __ldg(S.atom0 + b0), nat = __ldg(S.atom0 + b1) - a0;
    const int nbp = S.nb_pad;
    float* __restrict__ ghi = (float*)S.state;  // state rows 0..13 (hi)
    float* __restrict__ glo = ghi + 14 * nbp;   // rows 14..27 (lo)
    const float dt = (float)dt_d;

    // Phase 1 loads first (slots, body-frame coordinates; the orientation; then the forces at the
    // slots), so that their latencies overlap phase 0
    {
        const float* __restrict__ dg = (const float*)S.d;
        int loc[APT];
        V3<float> F[APT], d[APT];
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * NT;
            loc[i] = a < nat ? __ldg(S.atom_loc + a0 + a) : 0;
        }
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * NT;
            if (a < nat) {
                const int k = a0 + a;
                d[i] = v3<float>(__ldg(dg + k), __ldg(dg + k + S.nba_pad), __ldg(dg + k + 2 * S.nba_pad));
            }
        }
        Q4<float> q0 = q4<float>(1.0f, 0.0f, 0.0f, 0.0f);
        int s0 = 0, e0 = 0;
        if (tid < nbt) {
            const int b = b0 + tid;
            q0 = q4<float>(ghi[b + 6 * nbp], ghi[b + 7 * nbp], ghi[b + 8 * nbp], ghi[b + 9 * nbp]);
            s0 = __ldg(S.atom0 + b) - a0;
            e0 = __ldg(S.atom0 + b + 1) - a0;
        }
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * NT;
            if (a < nat) F[i] = load_force<float>(B.force, loc[i], B.stride);
        }
        // Phase 0: rotation matrix of the current orientation; atoms -> tile-local body; the
        // tile's large bodies
        if (tid < nbt) {
            rotation_matrix(q0, sM + 9 * tid);
            for (int j = s0; j < e0; j++) sBody[j] = (unsigned short)tid;
        }
        if (LARGE) {
            const unsigned m = __ballot_sync(0xffffffffu, e0 - s0 > kWarpBody);
            if ((tid & 31) == 0) sBig[tid >> 5] = m;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < APT; i++) {
            const int a = tid + i * NT;
            if (a < nat) {
                const V3<float> delta = mat_vec(sM + 9 * sBody[a], d[i]);
                const V3<float> tau = cross(delta, F[i]);
                sF[3 * a] = F[i].x; sF[3 * a + 1] = F[i].y; sF[3 * a + 2] = F[i].z;
                sT[3 * a] = tau.x; sT[3 * a + 1] = tau.y; sT[3 * a + 2] = tau.z;
            }
        }
    }
    __syncthreads();
    if (LARGE && count_large<NT / 32>(sBig)) {
        // large bodies' sums parked in sR (6 words of their tile body; phase 2 reads, then reuses them)
        warp_body_sums<NT / 32>(sBig, S.atom0, b0, a0, sF, sT, sR, sR + 3, 6);
        __syncthreads();
    }

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
            if (LARGE && e0 - s0 > kWarpBody) {
                Fa = v3<float>(sR[6 * tid], sR[6 * tid + 1], sR[6 * tid + 2]);
                Ta = v3<float>(sR[6 * tid + 3], sR[6 * tid + 4], sR[6 * tid + 5]);
            } else {
                for (int j = s0; j < e0; j++) {
                    Fa = Fa + v3<float>(sF[3 * j], sF[3 * j + 1], sF[3 * j + 2]);
                    Ta = Ta + v3<float>(sT[3 * j], sT[3 * j + 1], sT[3 * j + 2]);
                }
            }
        }
        const Q4<float> qh = q4<float>(x[6].hi, x[7].hi, x[8].hi, x[9].hi);
        const Q4<float> pin = q4<float>(x[10].hi, x[11].hi, x[12].hi, x[13].hi);  // before the kicks
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
            if (REF) {
                // end of the refined-energy stencils at t+h (rigidbodyintegrator.cu:380-384) and the
                // body's terms of refinedKineticEnergies / potentialEnergyRefinement (:433-469), as
                // corrections: KE_t: (m/12) v.(alpha - beta), alpha = F(t) h/m, beta = F(t+h) h/m
                // (equal to rdot.v m/(6h) - m|v|^2/2 for the reference's position stencil); KE_r:
                // qdot.pi/(6h) - L.I^-1.L/2 with the quaternion stencil
                //   qdot = 0.5 [q(t-h) - q(t)] + 2.5 [q(t+h) - q(t)] + [q(t+2h) - q(t+h)],
                // q(t-h) - q(t) = q(t) (x) dr_b, the virtual rotation by -h from (q(t), pi(t-h/2))
                // (:318-321), taken as the rotation by +h with the angular momentum reversed (the free
                // rotor is time-reversible); q(t+2h) - q(t+h) = q (x) dr_f, the virtual rotation from
                // (q(t+h), pi(t+h) + C(q,tau) h) (:238-243); qdot projected off q; and
                // |F|^2/m + tau.I^-1.tau in the body frame. Both virtual rotations run here, once per
                // part2, rather than in every fused step.
                const float* rs = (const float*)S.ref_start;
                const V3<float> al = v3<float>(rs[b], rs[b + nbp], rs[b + 2 * nbp]);
                const Q4<float> dqn = q4<float>(rs[b + 3 * nbp], rs[b + 4 * nbp], rs[b + 5 * nbp], rs[b + 6 * nbp]);
                const V3<float> Lb = v3<float>(rs[b + 7 * nbp], rs[b + 8 * nbp], rs[b + 9 * nbp]);
                const V3<float> vh = v3<float>(x[3].hi, x[4].hi, x[5].hi);
                const float dkt = dot(vh, al - Fa * (invm * dt)) / (12.0f * invm);
                const Q4<float> drb = rotation_increment<EXACT>(S, b, Lb * -1.0f, R, dt);
                const Q4<float> drf = rotation_increment<EXACT>(S, b, qBt(qh, ph + Ctau) * 0.5f, R, dt);
                Q4<float> qd = qmul(qh - dqn, drb) * 0.5f + dqn * 2.5f + qmul(qh, drf);
                qd = qd - qh * dot(qd, qh);
                const V3<float> L = qBt(qh, ph) * 0.5f;
                const float dkr = dot(qd, ph) / (6.0f * dt) - 0.5f * dot(L, mul(R.invI, L));
                const V3<float> tb = rotate_to_body(qh, Ta);
                const float u = dot(Fa, Fa) * invm + dot(tb, mul(R.invI, tb));
                S.ref_out[b] = dkt; S.ref_out[b + nbp] = dkr; S.ref_out[b + 2 * nbp] = u;
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; c++) x[c] = ff_acc(x[c], fmaf(x[3 + c].hi, dt, x[3 + c].lo * dt));  // drift
            const V3<float> L = qBt(qh, ph) * 0.5f;
            const Q4<float> dr = rotation_increment<EXACT>(S, b, L, R, dt);
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
            float ren[4];  // the renormalisation's change of q
#pragma unroll
            for (int c = 6; c < 10; c++) {
                ren[c - 6] = -0.5f * eps * x[c].hi;
                x[c] = ff_norm(ff_acc(x[c], ren[c - 6]));
            }
            if (REF) {
                // start of the stencils at t (rigidbodyintegrator.cu:318-321): alpha = F(t) h/m, the
                // increment q(t+h) - q(t) just applied (dq plus the renormalisation), and the body
                // angular momentum L(t-h/2) = Bt(q(t), pi(t) - C(q,tau) h)/2 of the backward virtual
                // rotation, which part2 performs
                const Q4<float> pib = KIND == STEP_FUSED ? pin : pin - Ctau;
                const V3<float> Lb = qBt(qh, pib) * 0.5f;
                const Q4<float> dqn = dq + q4<float>(ren[0], ren[1], ren[2], ren[3]);
                const V3<float> al = Fa * (invm * dt);
                float* rs = (float*)S.ref_start;
                rs[b] = al.x; rs[b + nbp] = al.y; rs[b + 2 * nbp] = al.z;
                rs[b + 3 * nbp] = dqn.w; rs[b + 4 * nbp] = dqn.x; rs[b + 5 * nbp] = dqn.y; rs[b + 6 * nbp] = dqn.z;
                rs[b + 7 * nbp] = Lb.x; rs[b + 8 * nbp] = Lb.y; rs[b + 9 * nbp] = Lb.z;
            }
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
        {
            float chk = 0.0f;
#pragma unroll
            for (int c = 0; c < 14; c++) chk += x[c].hi;
            if (!finite_f(chk)) flag_failure(S.status, S.body_bad, b);
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
    for (int a = tid; a < nat; a += NT) {
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
// Launch: one CTA per tile (body tiles, then free-atom tiles).
// ------------------------------------------------------------------------------------------
template <int NT> constexpr size_t step_smem_f() { return (size_t)FSmem<NT>::WORDS * 4; }

template <int P, int KIND, bool EXACT, bool REF, int NT, bool LARGE> struct StepKernel {
    static constexpr auto fn() { return step_kernel_f<P, KIND, EXACT, REF, NT, LARGE>; }
    static constexpr size_t smem() { return step_smem_f<NT>(); }
    static constexpr int threads() { return NT; }
};
template <int KIND, bool EXACT, bool REF, int NT, bool LARGE> struct StepKernel<PREC_DOUBLE, KIND, EXACT, REF, NT, LARGE> {
    static constexpr auto fn() { return step_kernel_d<KIND, EXACT, REF, LARGE>; }
    static constexpr size_t smem() { return step_smem_d(); }
    static constexpr int threads() { return kThreads; }
};

template <int P, int KIND, bool EXACT, bool REF, int NT, bool LARGE>
int launch_step_nt(const DevSys& s, const DevBuf& b, double dt, cudaStream_t stream) {
    using K = StepKernel<P, KIND, EXACT, REF, NT, LARGE>;
    const size_t smem = K::smem();
    const int threads = K::threads();
    auto kernel = K::fn();
    if (smem > 48 * 1024) {
        // The opt-in above 48 KB of dynamic shared memory is a per-device attribute: remember the
        // devices that have it (one bit each; devices past 63 set it on every launch).
        static std::atomic<unsigned long long> configured{0};
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return -1;
        const unsigned long long bit = dev < 64 ? 1ull << dev : 0ull;
        if (!bit || !(configured.load(std::memory_order_acquire) & bit)) {
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return -1;
            configured.fetch_or(bit, std::memory_order_release);
        }
    }
    const int tiles = s.n_body_tiles + s.n_free_tiles;
    if (tiles == 0) return 0;
    kernel<<<tiles, threads, smem, stream>>>(s, b, dt);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// The kernel for the integrator's bodies (any of more than kWarpBody atoms: the LARGE form) and,
// in single/mixed precision, the block size its tiles were packed for (narrow tiles only without
// large bodies).
template <int P, int KIND, bool EXACT, bool REF>
int launch_step_t(const DevSys& s, const DevBuf& b, double dt, cudaStream_t stream) {
    if (s.large) return launch_step_nt<P, KIND, EXACT, REF, kThreadsF, true>(s, b, dt, stream);
    if (P != PREC_DOUBLE && s.tile_threads == kThreadsFNarrow)
        return launch_step_nt<P, KIND, EXACT, REF, kThreadsFNarrow, false>(s, b, dt, stream);
    return launch_step_nt<P, KIND, EXACT, REF, kThreadsF, false>(s, b, dt, stream);
}

// part2 rotates nothing unless it closes the refined-energy stencils (a virtual rotation).
template <int P, bool REF>
int launch_step_p(int kind, const DevSys& s, const DevBuf& b, double dt, cudaStream_t st) {
    const bool exact = s.rot_n == 0;
    switch (kind) {
        case STEP_PART1:
            return exact ? launch_step_t<P, STEP_PART1, true, REF>(s, b, dt, st) : launch_step_t<P, STEP_PART1, false, REF>(s, b, dt, st);
        case STEP_PART2:
            if constexpr (REF) {
                if (exact) return launch_step_t<P, STEP_PART2, true, true>(s, b, dt, st);
            }
            return launch_step_t<P, STEP_PART2, false, REF>(s, b, dt, st);
        default:
            return exact ? launch_step_t<P, STEP_FUSED, true, REF>(s, b, dt, st) : launch_step_t<P, STEP_FUSED, false, REF>(s, b, dt, st);
    }
}

}  // namespace rbx
