// rbx_setup.cu -- rigid-body setup on the device: geometry and momenta of every body from the atom
// positions and velocities already in the OpenMM-layout buffers (RigidBodySystem::update,
// openmmapi/src/RigidBodySystem.cpp:120-142, without the host round trip of the positions and
// velocities). One thread per body, the arithmetic of rbx_setup.cuh; compiled with -fmad=false so
// that it matches the host setup bit for bit.
#include <cuda_runtime.h>

#include "rbx_internal.h"
#include "rbx_setup.cuh"

namespace rbx {

namespace {

// The atoms of body L (library order) in the device buffers.
struct DevAtoms {
    int n, k0, prec, nba_pad;
    const int* loc;
    const double* bmass;
    DevBuf B;
    void* d;  // body-frame coordinates: float (single, mixed) or double rows of nba_pad
    __device__ double mass(int j) const { return bmass[k0 + j]; }
    __device__ V3<double> pos(int j) const {
        const int s = loc[k0 + j];
        if (prec == PREC_DOUBLE) {
            const double* p = (const double*)B.posq + 4 * (size_t)s;
            return v3<double>(p[0], p[1], p[2]);
        }
        const float4 p = ((const float4*)B.posq)[s];
        if (prec == PREC_MIXED) {
            const float4 c = ((const float4*)B.corr)[s];
            return v3<double>((double)p.x + (double)c.x, (double)p.y + (double)c.y, (double)p.z + (double)c.z);
        }
        return v3<double>(p.x, p.y, p.z);
    }
    __device__ V3<double> vel(int j) const {
        const int s = loc[k0 + j];
        if (prec == PREC_SINGLE) {
            const float4 v = ((const float4*)B.velm)[s];
            return v3<double>(v.x, v.y, v.z);
        }
        const double* v = (const double*)B.velm + 4 * (size_t)s;
        return v3<double>(v[0], v[1], v[2]);
    }
    __device__ void set_d(int j, V3<double> x) const {
        const int k = k0 + j;
        if (prec == PREC_DOUBLE) {
            double* o = (double*)d;
            o[k] = x.x; o[k + nba_pad] = x.y; o[k + 2 * nba_pad] = x.z;
        } else {
            float* o = (float*)d;
            o[k] = (float)x.x; o[k + nba_pad] = (float)x.y; o[k + 2 * nba_pad] = (float)x.z;
        }
    }
};

__global__ void setup_bodies_kernel(DevSys S, DevBuf B, int prec, const double* bmass, SetupOut O) {
    const int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= S.nb) return;
    const int nbp = S.nb_pad;
    DevAtoms at{S.atom0[L + 1] - S.atom0[L], S.atom0[L], prec, S.nba_pad, S.atom_loc, bmass, B, (void*)S.d};
    BodySetup s;
    build_body(at, s);
    const double row[14] = {s.r.x, s.r.y, s.r.z, s.v.x, s.v.y, s.v.z, s.q.w, s.q.x, s.q.y, s.q.z,
                            s.pi.w, s.pi.x, s.pi.y, s.pi.z};
    bool finite = true;
    for (int k = 0; k < 14; k++) finite = finite && isfinite(row[k]);
    if (!finite) atomicOr(O.status, 1u);
    if (prec == PREC_DOUBLE) {
        double* st = (double*)S.state;
        for (int k = 0; k < 14; k++) st[L + (size_t)k * nbp] = row[k];
        double* invm = (double*)S.invm;
        double* invI = (double*)S.invI;
        invm[L] = s.invm;
        for (int k = 0; k < 3; k++) invI[L + (size_t)k * nbp] = s.invI[k];
    } else {
        float* hi = (float*)S.state;
        float* lo = hi + 14 * nbp;
        for (int k = 0; k < 14; k++) {
            const float h = (float)row[k];
            hi[L + (size_t)k * nbp] = h;
            lo[L + (size_t)k * nbp] = (float)(row[k] - (double)h);
        }
        // 1/m and 1/I as float-float (rows 0-3 hi, 7-10 lo); the moment gaps formed in FP64
        const double cst[7] = {s.invm, s.invI[0], s.invI[1], s.invI[2], s.I[0] - s.I[1], s.I[1] - s.I[2],
                               s.I[0] - s.I[2]};
        float* bc = (float*)S.bconst;
        for (int k = 0; k < 7; k++) bc[L + (size_t)k * nbp] = (float)cst[k];
        for (int k = 0; k < 4; k++) bc[L + (size_t)(7 + k) * nbp] = (float)(cst[k] - (double)(float)cst[k]);
    }
    ((uint8_t*)S.cls)[L] = s.cls;
    for (int k = 0; k < 3; k++) O.I[L + (size_t)k * nbp] = s.I[k];
    O.dof[L] = s.dof;
    atomicAdd(O.ndof, s.dof);
}

}  // namespace

int launch_setup_bodies(int prec, const DevSys& s, const DevBuf& b, const double* bmass, const SetupOut& out,
                        void* stream) {
    if (s.nb == 0) return 0;
    setup_bodies_kernel<<<(s.nb + 127) / 128, 128, 0, (cudaStream_t)stream>>>(s, b, prec, bmass, out);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace rbx
