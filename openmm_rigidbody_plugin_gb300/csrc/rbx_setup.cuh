// rbx_setup.cuh -- rigid-body geometry and momenta from atom positions and velocities, usable from
// host and device code (the same arithmetic in both: the host compiles it with FP contraction off
// and the device kernel with -fmad=false, and FP64 division and square root are correctly rounded
// on both, so the host and device setups agree bit for bit).
//
// Follows RigidBody::buildGeometry/buildDynamics (openmmapi/src/RigidBody.cpp:65-142) with the
// robust variants: the longest displacement as the axis of a linear body, an orthonormal vector
// chosen by |component| (the reference compares signed components, RigidBody.cpp:52-53), cyclic
// Jacobi principal axes (the reference's Smith/Kopp solver fails for degenerate moments,
// eigenDecomposition.cpp:162-171), a canonical body frame, and momenta recomputed from scratch.
#pragma once

#include <cstdint>

#include "rbx_math.cuh"

namespace rbx {

struct BodySetup {
    double mass, invm, I[3], invI[3];
    int dof;
    uint8_t cls;
    V3<double> r, v;
    Q4<double> q, pi;
};

// Principal frame by cyclic Jacobi rotations: moments w descending, eigenvectors as the rows of a
// proper rotation A (space -> body).
RBX_HD void principal_axes(const double M[9], double w[3], double A[9]) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a[i][j] = 0.5 * (M[3 * i + j] + M[3 * j + i]);
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off == 0.0 || off <= 1e-36 * diag) break;
        for (int p = 0; p < 2; p++)
            for (int r = p + 1; r < 3; r++) {
                if (a[p][r] == 0.0) continue;
                double theta = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {
                    double akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 3; k++) {
                    double apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 3; k++) {
                    double vkp = v[k][p], vkr = v[k][r];
                    v[k][p] = c * vkp - s * vkr;
                    v[k][r] = s * vkp + c * vkr;
                }
            }
    }
    // moments descending with their eigenvectors: the compare-swaps (0,1), (0,2), (1,2) of a
    // selection sort, on scalars (no run-time indexing of the local arrays)
    double e0 = a[0][0], e1 = a[1][1], e2 = a[2][2];
    V3<double> c0 = v3<double>(v[0][0], v[1][0], v[2][0]), c1 = v3<double>(v[0][1], v[1][1], v[2][1]),
               c2 = v3<double>(v[0][2], v[1][2], v[2][2]);
    if (e1 > e0) { const double t = e0; e0 = e1; e1 = t; const V3<double> u = c0; c0 = c1; c1 = u; }
    if (e2 > e0) { const double t = e0; e0 = e2; e2 = t; const V3<double> u = c0; c0 = c2; c2 = u; }
    if (e2 > e1) { const double t = e1; e1 = e2; e2 = t; const V3<double> u = c1; c1 = c2; c2 = u; }
    w[0] = e0; w[1] = e1; w[2] = e2;
    A[0] = c0.x; A[1] = c0.y; A[2] = c0.z;
    A[3] = c1.x; A[4] = c1.y; A[5] = c1.z;
    A[6] = A[1] * A[5] - A[2] * A[4];
    A[7] = A[2] * A[3] - A[0] * A[5];
    A[8] = A[0] * A[4] - A[1] * A[3];
}

// Unit quaternion of a proper rotation matrix (Shepperd's method, as in MatVec.cpp:344-373).
RBX_HD Q4<double> quaternion_of(const double* M) {
    const double t0 = 1.0 + M[0] + M[4] + M[8], t1 = 1.0 + M[0] - M[4] - M[8], t2 = 1.0 - M[0] + M[4] - M[8],
                 t3 = 1.0 - M[0] - M[4] + M[8];
    int k = 0;
    double tk = t0;
    if (t1 > tk) { k = 1; tk = t1; }
    if (t2 > tk) { k = 2; tk = t2; }
    if (t3 > tk) { k = 3; tk = t3; }
    const double f = 0.5 / sqrt(tk);
    switch (k) {
        case 0: return q4<double>(tk * f, (M[5] - M[7]) * f, (M[6] - M[2]) * f, (M[1] - M[3]) * f);
        case 1: return q4<double>((M[5] - M[7]) * f, tk * f, (M[1] + M[3]) * f, (M[2] + M[6]) * f);
        case 2: return q4<double>((M[6] - M[2]) * f, (M[1] + M[3]) * f, tk * f, (M[5] + M[7]) * f);
        default: return q4<double>((M[1] - M[3]) * f, (M[2] + M[6]) * f, (M[5] + M[7]) * f, tk * f);
    }
}

RBX_HD uint8_t rotation_class(const double I[3]) {
    if (I[2] == 0.0) return ROT_SYMMETRIC_AXIS2;  // linear body
    const double tol = 1e-12 * I[0];
    bool g01 = I[0] - I[1] <= tol, g12 = I[1] - I[2] <= tol;
    if (g01 && g12) return ROT_SPHERICAL;
    if (g01) return ROT_SYMMETRIC_AXIS2;
    if (g12) return ROT_SYMMETRIC_AXIS0;
    return ROT_ASYMMETRIC;
}

// Canonical body frame: each eigenvector row gets its largest-magnitude component positive; a top
// with two equal moments has its degenerate axes fixed by the first atom off the unique axis; a
// spherical top uses the space frame. Equivalent frames therefore never depend on rounding.
RBX_HD void canon_sign(V3<double>& v) {
    double ak = fabs(v.x), ck = v.x;
    if (fabs(v.y) > ak) { ak = fabs(v.y); ck = v.y; }
    if (fabs(v.z) > ak) { ak = fabs(v.z); ck = v.z; }
    if (ck < 0) v = v * -1.0;
}

// The atoms of one body seen through an accessor: n, mass(j), pos(j), vel(j), set_d(j, d).
template <class Atoms> RBX_HD V3<double> delta_of(const Atoms& at, int j, V3<double> rcm) { return at.pos(j) - rcm; }

template <class Atoms>
RBX_HD void canonical_frame(double* A, const double* I, const Atoms& at, V3<double> rcm, double d2max) {
    const uint8_t cls = rotation_class(I);
    if (cls == ROT_SPHERICAL) {
        for (int i = 0; i < 9; i++) A[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    if (cls == ROT_ASYMMETRIC) {
        V3<double> a = v3<double>(A[0], A[1], A[2]), b = v3<double>(A[3], A[4], A[5]);
        canon_sign(a);
        canon_sign(b);
        const V3<double> c = cross(a, b);
        A[0] = a.x; A[1] = a.y; A[2] = a.z; A[3] = b.x; A[4] = b.y; A[5] = b.z; A[6] = c.x; A[7] = c.y; A[8] = c.z;
        return;
    }
    const bool axis0 = cls == ROT_SYMMETRIC_AXIS0;  // the unique axis is row 0, else row 2
    const V3<double> r0 = v3<double>(A[0], A[1], A[2]), r1 = v3<double>(A[3], A[4], A[5]),
                     r2 = v3<double>(A[6], A[7], A[8]);
    V3<double> u = axis0 ? r0 : r2, e1 = axis0 ? r1 : r0;
    canon_sign(u);
    for (int j = 0; j < at.n; j++) {
        const V3<double> d = delta_of(at, j, rcm);
        V3<double> p = d - u * dot(u, d);
        double pp = dot(p, p);
        if (pp > 1e-6 * d2max) {
            e1 = p * (1.0 / sqrt(pp));
            break;
        }
    }
    V3<double> e2 = cross(u, e1);
    const V3<double> a = axis0 ? u : e1, b = axis0 ? e1 : e2, c = axis0 ? e2 : u;
    A[0] = a.x; A[1] = a.y; A[2] = a.z; A[3] = b.x; A[4] = b.y; A[5] = b.z; A[6] = c.x; A[7] = c.y; A[8] = c.z;
}

// Geometry (principal moments, frame, body-frame coordinates via at.set_d) and momenta of one body.
template <class Atoms> RBX_HD void build_body(Atoms& at, BodySetup& out) {
    const int N = at.n;
    double mass = 0.0;
    V3<double> rcm = v3<double>(0.0, 0.0, 0.0);
    for (int j = 0; j < N; j++) {
        const double m = at.mass(j);
        mass += m;
        rcm = rcm + at.pos(j) * m;
    }
    rcm = rcm * (1.0 / mass);
    int jmax = 0;
    double d2max = -1.0;
    for (int j = 0; j < N; j++) {
        const V3<double> d = delta_of(at, j, rcm);
        const double d2 = dot(d, d);
        if (d2 > d2max) { d2max = d2; jmax = j; }
    }
    const double TOL = 1.0e-5;
    V3<double> u = delta_of(at, jmax, rcm) * (1.0 / sqrt(d2max));
    canon_sign(u);
    bool linear = d2max > 0.0;
    for (int j = 0; linear && j < N; j++) {
        const V3<double> d = delta_of(at, j, rcm);
        const double d2 = dot(d, d), udj = dot(u, d);
        linear = d2 < TOL * d2max || fabs(udj * udj / d2 - 1.0) < TOL;
    }
    double A[9];
    if (linear) {
        double moi = 0.0;
        for (int j = 0; j < N; j++) {
            const V3<double> d = delta_of(at, j, rcm);
            moi += at.mass(j) * dot(d, d);
        }
        out.I[0] = out.I[1] = moi;
        out.I[2] = 0.0;
        const double cx = fabs(u.x), cy = fabs(u.y), cz = fabs(u.z);
        int imin = cx < cy ? 0 : 1;
        if (cz < (imin == 0 ? cx : cy)) imin = 2;
        V3<double> e = v3<double>(imin == 0 ? 1.0 : 0.0, imin == 1 ? 1.0 : 0.0, imin == 2 ? 1.0 : 0.0);
        V3<double> vv = e - u * dot(u, e);
        vv = vv * (1.0 / sqrt(dot(vv, vv)));
        V3<double> ww = cross(u, vv);
        const double rows[9] = {vv.x, vv.y, vv.z, ww.x, ww.y, ww.z, u.x, u.y, u.z};
        for (int i = 0; i < 9; i++) A[i] = rows[i];
        out.dof = 5;
    } else {
        double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = 0; j < N; j++) {
            const double m = at.mass(j);
            const V3<double> d = delta_of(at, j, rcm);
            const double d2 = dot(d, d);
            double x[3] = {d.x, d.y, d.z};
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) M[3 * r + c] += ((r == c ? d2 : 0.0) - x[r] * x[c]) * m;
        }
        principal_axes(M, out.I, A);
        canonical_frame(A, out.I, at, rcm, d2max);
        out.dof = 6;
    }
    out.q = quaternion_of(A);
    out.mass = mass;
    out.invm = 1.0 / mass;
    for (int k = 0; k < 3; k++) out.invI[k] = out.I[k] == 0.0 ? 0.0 : 1.0 / out.I[k];
    out.cls = rotation_class(out.I);
    out.r = rcm;
    V3<double> p = v3<double>(0.0, 0.0, 0.0);
    for (int j = 0; j < N; j++) p = p + at.vel(j) * at.mass(j);
    const V3<double> vcm = p * (1.0 / mass);
    V3<double> L = v3<double>(0.0, 0.0, 0.0);
    for (int j = 0; j < N; j++) {
        const V3<double> d = delta_of(at, j, rcm);
        const V3<double> df = v3<double>(A[0] * d.x + A[1] * d.y + A[2] * d.z, A[3] * d.x + A[4] * d.y + A[5] * d.z,
                                         A[6] * d.x + A[7] * d.y + A[8] * d.z);
        at.set_d(j, df);
        const V3<double> body = rotate_to_body(out.q, at.vel(j) - vcm) * at.mass(j);
        L = L + cross(df, body);
    }
    out.v = vcm;
    out.pi = qB(out.q, L * 2.0);
}

}  // namespace rbx
