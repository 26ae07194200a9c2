// rbx_fast.cuh -- FP32 free rotation in increment form and float-float accumulation, for the
// single and mixed precision step kernels.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the body arithmetic of the
// production precisions runs entirely on the FP32 pipe:
//  * Body state (r, v, q, pi) is stored as float-float pairs (hi + lo, about 48 significant bits)
//    and updated by adding FP32 increments with error-free transformations.
//  * A free rotation is returned as the increment dr = r - 1 of the unit quaternion r that
//    right-multiplies q and pi (q <- q (x) r, pi <- pi (x) r; pi = 2 q (x) (0, L) stays valid).
//    Because dr is small and is formed without cancellation, its FP32 rounding error is ~1e-7 of
//    |dr| instead of ~1e-7 absolute.
//  * Exact (mode 0) rotation of an asymmetric top: the body-frame angular momentum over the
//    step follows from the Jacobi-elliptic solution through the addition theorem
//    (sn, cn, dn of u0 + h from their values at u0, which the current state fixes, and of the
//    small argument h = wp dt); the rotation is r = e(phi) (x) mu, with mu the minimal rotation
//    taking L_hat(t) back to L_hat(0) and phi the angle about L_hat(0), whose rate is
//    phi' = omega . (n + n0) / (1 + n . n0), integrated by 3-point Gauss-Legendre quadrature
//    (error about 5e-7 (wp dt)^6 of phi: 4e-10 at |wp dt| = 0.3; thermal water at 2 fs has
//    |wp dt| <= 0.11).
//    This evaluates the same solution as the closed form of openmmapi/src/RigidBody.cpp:241-308
//    (agreement 2e-12 in FP64) without its third-kind elliptic integrals, and with no gauge
//    singularity.
//  * NO-SQUISH (mode n) composes the 5n principal-axis rotations of RigidBody.cpp:189-231 into one
//    increment while tracking the body-frame angular momentum.
#pragma once

#include "rbx_math.cuh"

namespace rbx {

// ------------------------------------------------------------------------------------------
// Float-float scalars
// ------------------------------------------------------------------------------------------
struct ff {
    float hi, lo;
};

// a + b for a float-float a and a float b (two-sum, then renormalise).
__device__ __forceinline__ ff ff_add(ff a, float b) {
    float s = __fadd_rn(a.hi, b);
    float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    e = __fadd_rn(e, a.lo);
    float hi = __fadd_rn(s, e);
    float lo = __fsub_rn(e, __fsub_rn(hi, s));
    return ff{hi, lo};
}

// a + b without the final renormalisation: the rounding error of hi + b is added to lo, so
// hi + lo stays exact to float-float accuracy while |lo| may exceed half an ulp of hi; a chain of
// these is closed by ff_norm before the value is stored.
__device__ __forceinline__ ff ff_acc(ff a, float b) {
    float s = __fadd_rn(a.hi, b);
    float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, __fadd_rn(a.lo, e)};
}
__device__ __forceinline__ ff ff_norm(ff a) {
    float hi = __fadd_rn(a.hi, a.lo);
    return ff{hi, __fsub_rn(a.lo, __fsub_rn(hi, a.hi))};
}

// Split s + e (|e| small against s) into the OpenMM position pair posq = hi, correction = lo.
__device__ __forceinline__ void ff_split(float s, float e, float& hi, float& lo) {
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// ------------------------------------------------------------------------------------------
// Increments of unit quaternions: dq = r - 1, composition (1 + a)(1 + b) - 1 = a + b + a b.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ Q4<float> dq_compose(Q4<float> a, Q4<float> b) { return a + b + qmul(a, b); }

// sin(x) and cos(x) - 1 without cancellation (Taylor series for |x| <= 0.5, else sincosf).
__device__ __forceinline__ void sin_cosm1(float x, float& s, float& cm1) {
    float x2 = x * x;
    if (x2 <= 0.25f) {
        s = x * (1.0f + x2 * (-1.0f / 6.0f + x2 * (1.0f / 120.0f + x2 * (-1.0f / 5040.0f + x2 * (1.0f / 362880.0f)))));
        cm1 = x2 * (-0.5f + x2 * (1.0f / 24.0f + x2 * (-1.0f / 720.0f + x2 * (1.0f / 40320.0f + x2 * (-1.0f / 3628800.0f)))));
    } else {
        float c;
        sincosf(x, &s, &c);
        cm1 = c - 1.0f;
    }
}

// Increment of the rotation by angle `angle` about the unit axis u: (cos(a/2) - 1, sin(a/2) u).
__device__ __forceinline__ Q4<float> dq_axis_angle(V3<float> u, float angle) {
    float s, cm1;
    sin_cosm1(0.5f * angle, s, cm1);
    return q4<float>(cm1, s * u.x, s * u.y, s * u.z);
}

// ------------------------------------------------------------------------------------------
// Jacobi sn, cn - 1, dn - 1 of a small argument: Maclaurin series (Abramowitz & Stegun 16.22)
// for |h| <= 0.125, halving the argument and doubling back with the duplication formulas
//   sn(2h) = 2 s c d / D, cn(2h) - 1 = -2 s^2 d^2 / D, dn(2h) - 1 = -2 m s^2 c^2 / D,
//   D = 1 - m s^4.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void jacobi_small(float h, float m, float& sn, float& cm1, float& dm1) {
    int k = 0;
    while (fabsf(h) > 0.125f && k < 24) {
        h *= 0.5f;
        k++;
    }
    const float u2 = h * h, m2 = m * m, m3 = m2 * m;
    sn = h * (1.0f + u2 * (-(1.0f + m) * (1.0f / 6.0f) +
                           u2 * ((1.0f + 14.0f * m + m2) * (1.0f / 120.0f) +
                                 u2 * (-(1.0f + 135.0f * m + 135.0f * m2 + m3) * (1.0f / 5040.0f) +
                                       u2 * (1.0f + 1228.0f * m + 5478.0f * m2 + 1228.0f * m3 + m2 * m2) *
                                           (1.0f / 362880.0f)))));
    cm1 = u2 * (-0.5f + u2 * ((1.0f + 4.0f * m) * (1.0f / 24.0f) +
                              u2 * (-(1.0f + 44.0f * m + 16.0f * m2) * (1.0f / 720.0f) +
                                    u2 * (1.0f + 408.0f * m + 912.0f * m2 + 64.0f * m3) * (1.0f / 40320.0f))));
    dm1 = m * u2 * (-0.5f + u2 * ((4.0f + m) * (1.0f / 24.0f) +
                                  u2 * (-(16.0f + 44.0f * m + m2) * (1.0f / 720.0f) +
                                        u2 * (64.0f + 912.0f * m + 408.0f * m2 + m3) * (1.0f / 40320.0f))));
    for (int i = 0; i < k; i++) {
        float c = 1.0f + cm1, d = 1.0f + dm1, s2 = sn * sn;
        float D = 1.0f - m * s2 * s2;
        float inv = 1.0f / D;
        float ns = 2.0f * sn * c * d * inv;
        cm1 = -2.0f * s2 * d * d * inv;
        dm1 = -2.0f * m * s2 * c * c * inv;
        sn = ns;
    }
}

// Per-body rotor constants in FP32: inverse principal moments as float-float (hi + lo) and the
// gaps between the moments (g01 = I0 - I1, g12 = I1 - I2, g02 = I0 - I2), computed on the host
// in FP64 so that they keep full relative accuracy for nearly degenerate tops.
struct Rotor {
    V3<float> invI, invI_lo;
    float g01, g12, g02;
};

// ------------------------------------------------------------------------------------------
// NO-SQUISH increment (openmmapi/src/RigidBody.cpp:220-231): 5n principal-axis rotations, each by
// the angle omega_k h of the current body-frame L, composed into one increment dr. The current L
// is recomputed from the step's initial L0 and dr at every substep (L = conj(r) L0 r), so FP32
// rounding does not accumulate along the 5n substeps.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float current_Lk(int k, V3<float> L0, Q4<float> dr) {
    // component k of conj(r) L0 r - L0 = -2 w (v x L0) + 2 v x (v x L0), r = (1 + dr.w, dr.xyz)
    const V3<float> v = v3<float>(dr.x, dr.y, dr.z);
    const float w = 1.0f + dr.w;
    const V3<float> c = cross(v, L0);
    const V3<float> cc = cross(v, c);
    const float d = k == 0 ? (-2.0f * w * c.x + 2.0f * cc.x) : (k == 1 ? (-2.0f * w * c.y + 2.0f * cc.y)
                                                                       : (-2.0f * w * c.z + 2.0f * cc.z));
    const float l0 = k == 0 ? L0.x : (k == 1 ? L0.y : L0.z);
    return l0 + d;
}

__device__ __forceinline__ void nosquish_sub(int k, const Rotor& R, float h, V3<float> L0, Q4<float>& dr) {
    const float Lk = current_Lk(k, L0, dr);
    const float ik = k == 0 ? R.invI.x : (k == 1 ? R.invI.y : R.invI.z);
    const float il = k == 0 ? R.invI_lo.x : (k == 1 ? R.invI_lo.y : R.invI_lo.z);
    const float a = 0.5f * Lk * h;
    const float phi = fmaf(a, il, a * ik);  // omega_k h / 2 (RigidBody.cpp:191)
    float s, cm1;
    sin_cosm1(phi, s, cm1);
    // dr <- (1 + dr) (x) (cos phi + sin phi e_k) - 1
    Q4<float> e = q4<float>(cm1, 0.0f, 0.0f, 0.0f);
    if (k == 0) e.x = s; else if (k == 1) e.y = s; else e.z = s;
    dr = dq_compose(dr, e);
}

__device__ __forceinline__ Q4<float> nosquish_increment(V3<float> L, const Rotor& R, bool axis3, float dt, int n) {
    const float h = dt / (float)n, hh = 0.5f * h;
    Q4<float> dr = q4<float>(0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < n; i++) {
        if (axis3) nosquish_sub(2, R, hh, L, dr);
        nosquish_sub(1, R, hh, L, dr);
        nosquish_sub(0, R, h, L, dr);
        nosquish_sub(1, R, hh, L, dr);
        if (axis3) nosquish_sub(2, R, hh, L, dr);
    }
    return dr;
}

// ------------------------------------------------------------------------------------------
// Exact free rotation, increment form.
// ------------------------------------------------------------------------------------------

// Rotation about a fixed body axis u by angle w dt (used when L lies on a principal axis).
__device__ __forceinline__ Q4<float> dq_uniaxial(int k, float wk, float dt) {
    V3<float> u = v3<float>(k == 0 ? 1.0f : 0.0f, k == 1 ? 1.0f : 0.0f, k == 2 ? 1.0f : 0.0f);
    return dq_axis_angle(u, wk * dt);
}

// Symmetric top with unique axis k (k = -1: spherical): rotation about L at rate |L|/I_perp, then
// spin about axis k at rate (1/I_k - 1/I_perp) L_k.
__device__ __forceinline__ Q4<float> dq_symmetric(int k, float invIp, float invIk, V3<float> L, V3<float> invI, float dt) {
    if (k < 0) {
        V3<float> w = mul(invI, L);  // invI carries its low part here (see dq_exact)
        float wn = sqrtf(dot(w, w));
        if (wn == 0.0f) return q4<float>(0.0f, 0.0f, 0.0f, 0.0f);
        return dq_axis_angle(w * (1.0f / wn), wn * dt);
    }
    float Ln = sqrtf(dot(L, L));
    if (Ln == 0.0f) return q4<float>(0.0f, 0.0f, 0.0f, 0.0f);
    Q4<float> d1 = dq_axis_angle(L * (1.0f / Ln), Ln * invIp * dt);
    float Lk = k == 0 ? L.x : L.z;
    Q4<float> d2 = dq_uniaxial(k, (invIk - invIp) * Lk, dt);
    return dq_compose(d1, d2);
}

// Asymmetric top, I0 > I1 > I2 (moments sorted as in the plugin). Returns the rotation increment.
__device__ __forceinline__ Q4<float> dq_exact_asymmetric(V3<float> Iw, const Rotor& R, float dt) {
    const V3<float> invI = R.invI;
    const V3<float> I = v3<float>(1.0f / invI.x, 1.0f / invI.y, 1.0f / invI.z);
    const float Lsq = dot(Iw, Iw);
    if (Lsq == 0.0f) return q4<float>(0.0f, 0.0f, 0.0f, 0.0f);
    const float perp0 = Iw.y * Iw.y + Iw.z * Iw.z, perp2 = Iw.x * Iw.x + Iw.y * Iw.y;
    // L on a principal axis: stationary rotation about it
    if (perp0 <= 1e-24f * Lsq) return dq_uniaxial(0, Iw.x * invI.x, dt);
    if (perp2 <= 1e-24f * Lsq) return dq_uniaxial(2, Iw.z * invI.z, dt);
    const V3<float> w0 = mul(invI, Iw);
    // r1 = L^2 - 2K I2 and r3 = 2K I0 - L^2 as sums of non-negative terms
    const float r1 = Iw.x * Iw.x * (R.g02 * invI.x) + Iw.y * Iw.y * (R.g12 * invI.y);
    const float r3 = Iw.y * Iw.y * (R.g01 * invI.y) + Iw.z * Iw.z * (R.g02 * invI.z);
    const float l1 = r1 * invI.y / R.g12, l3 = r3 * invI.y / R.g01;
    const bool case1 = l1 < l3;  // L_body = I a (cn, sn, dn); otherwise I a (dn, sn, cn)
    const float lmin = case1 ? l1 : l3, lmax = case1 ? l3 : l1;
    const float c13 = 1.0f / R.g02;
    V3<float> a = v3<float>(sqrtf(r1 * invI.x * c13), sqrtf(lmin), sqrtf(r3 * invI.z * c13));
    if (w0.x < 0.0f) a.x = -a.x;
    if (w0.z < 0.0f) a.z = -a.z;
    const float m = lmin / lmax;
    const float wp = -invI.y * a.x * a.z / (a.y * c13);
    // Jacobi functions at u0, from the state itself
    float s0 = w0.y / a.y;
    s0 = fminf(1.0f, fmaxf(-1.0f, s0));
    const float cx = w0.x / a.x, cz = w0.z / a.z;
    const float c0 = case1 ? cx : cz, d0 = case1 ? cz : cx;
    const V3<float> Ia = mul(I, a);
    const float ms0s0 = m * s0 * s0;
    const float Lm = sqrtf(Lsq), invL = 1.0f / Lm;
    const V3<float> n0 = Iw * invL;
    // body-frame L(t) - L(0) from the addition theorem (Abramowitz & Stegun 16.17)
    auto dL = [&](float t) {
        float sh, cm1, dm1;
        jacobi_small(wp * t, m, sh, cm1, dm1);
        float sh2 = sh * sh;
        float invD = 1.0f / (1.0f - ms0s0 * sh2);
        float ds = (s0 * (cm1 + dm1 + cm1 * dm1) + sh * c0 * d0 + ms0s0 * s0 * sh2) * invD;
        float dc = (c0 * cm1 - s0 * d0 * sh * (1.0f + dm1) + c0 * ms0s0 * sh2) * invD;
        float dd = (d0 * dm1 - m * s0 * c0 * sh * (1.0f + cm1) + d0 * ms0s0 * sh2) * invD;
        return case1 ? v3<float>(Ia.x * dc, Ia.y * ds, Ia.z * dd) : v3<float>(Ia.x * dd, Ia.y * ds, Ia.z * dc);
    };
    // precession angle about L(0): phi = int omega . (n + n0) / (1 + n . n0) dt, 3-point
    // Gauss-Legendre nodes and weights on [0, dt]; the rule's error, (3!)^4 / (7 (6!)^3) dt^7 f^(6),
    // is about 5e-7 (wp dt)^6 of phi, below FP32 rounding for any |wp dt| <= 0.5
    const float glx[3] = {-0.7745966692414834f, 0.0f, 0.7745966692414834f};
    const float glw[3] = {0.5555555555555556f, 0.8888888888888888f, 0.5555555555555556f};
    float phi = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float t = 0.5f * dt * (1.0f + glx[i]);
        V3<float> Lt = Iw + dL(t);
        V3<float> n = Lt * rsqrtf(dot(Lt, Lt));
        V3<float> om = mul(invI, Lt) + mul(R.invI_lo, Lt);
        phi += glw[i] * dot(om, n + n0) / (1.0f + dot(n, n0));
    }
    phi *= 0.5f * dt;
    // minimal rotation mu taking n(dt) to n0, as an increment; dn = n - n0
    V3<float> dLt = dL(dt);
    V3<float> Lt = Iw + dLt;
    float Ltn = sqrtf(dot(Lt, Lt));
    float dLn = (2.0f * dot(Iw, dLt) + dot(dLt, dLt)) / (Ltn + Lm);  // |L(t)| - |L(0)|
    V3<float> dn = (dLt - n0 * dLn) * (1.0f / Ltn);                // n - n0 without cancellation
    float dn2 = dot(dn, dn);
    float q = 1.0f - 0.25f * dn2;  // mu0^2
    float mu0 = sqrtf(fmaxf(q, 0.0f));
    float invN = 0.5f / fmaxf(mu0, 1e-20f);  // 1 / sqrt(4 - |dn|^2)
    V3<float> nv = cross(dn, n0) * invN;   // (n x n0) / N with n = n0 + dn
    Q4<float> dmu = q4<float>(-0.25f * dn2 / (1.0f + mu0), nv.x, nv.y, nv.z);
    Q4<float> de = dq_axis_angle(n0, phi);
    return dq_compose(de, dmu);
}

// Mode-0 rotation increment for any rotation class (closed forms for degenerate tops).
__device__ __forceinline__ Q4<float> dq_exact(int cls, V3<float> L, const Rotor& R, float dt) {
    if (cls == ROT_ASYMMETRIC) return dq_exact_asymmetric(L, R, dt);
    if (cls == ROT_SPHERICAL) return dq_symmetric(-1, 0.0f, 0.0f, L, R.invI + R.invI_lo, dt);
    if (cls == ROT_SYMMETRIC_AXIS0) {
        float Ip = 0.5f * (1.0f / R.invI.y + 1.0f / R.invI.z);
        return dq_symmetric(0, 1.0f / Ip, R.invI.x, L, R.invI, dt);
    }
    float invIp = R.invI.z == 0.0f ? R.invI.x : 1.0f / (0.5f * (1.0f / R.invI.x + 1.0f / R.invI.y));
    return dq_symmetric(2, invIp, R.invI.z, L, R.invI, dt);
}

}  // namespace rbx
