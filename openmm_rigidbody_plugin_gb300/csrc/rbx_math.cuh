// rbx_math.cuh -- quaternion algebra and torque-free rotations (the double-precision step's
// formulas), templated on the scalar type and usable from host and device code.
//
// Conventions follow the plugin (openmmapi/src/MatVec.cpp:495-549): B(q)x = q (x) (0,x),
// C(q)x = (0,x) (x) q, Bt/Ct their transposes; space-to-body rotation A(q)x = Bt(q, C(q, x)) and
// body-to-space At(q)x = Ct(q, B(q, x)). The conjugate momentum is pi = 2 B(q) L_body
// (openmmapi/src/RigidBody.cpp:140), so L_body = Bt(q, pi)/2.
#pragma once

#include <cfloat>
#include <cmath>

#ifdef __CUDACC__
#define RBX_HD __host__ __device__ __forceinline__
#else
#define RBX_HD inline
#endif

namespace rbx {

template <class T> struct V3 { T x, y, z; };
template <class T> struct Q4 { T w, x, y, z; };  // (q0, q1, q2, q3)

template <class T> RBX_HD V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> RBX_HD Q4<T> q4(T a, T b, T c, T d) { return Q4<T>{a, b, c, d}; }
template <class T> RBX_HD T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> RBX_HD T dot(Q4<T> a, Q4<T> b) { return a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> RBX_HD V3<T> cross(V3<T> a, V3<T> b) {
    return v3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> RBX_HD V3<T> operator+(V3<T> a, V3<T> b) { return v3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> RBX_HD V3<T> operator-(V3<T> a, V3<T> b) { return v3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> RBX_HD V3<T> operator*(V3<T> a, T s) { return v3<T>(a.x * s, a.y * s, a.z * s); }
template <class T> RBX_HD V3<T> mul(V3<T> a, V3<T> b) { return v3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class T> RBX_HD Q4<T> operator+(Q4<T> a, Q4<T> b) { return q4<T>(a.w + b.w, a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> RBX_HD Q4<T> operator-(Q4<T> a, Q4<T> b) { return q4<T>(a.w - b.w, a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> RBX_HD Q4<T> operator*(Q4<T> a, T s) { return q4<T>(a.w * s, a.x * s, a.y * s, a.z * s); }

template <class T> RBX_HD Q4<T> qB(Q4<T> q, V3<T> x) {
    return q4<T>(-q.x * x.x - q.y * x.y - q.z * x.z, q.w * x.x - q.z * x.y + q.y * x.z,
                 q.z * x.x + q.w * x.y - q.x * x.z, -q.y * x.x + q.x * x.y + q.w * x.z);
}
template <class T> RBX_HD Q4<T> qC(Q4<T> q, V3<T> x) {
    return q4<T>(-q.x * x.x - q.y * x.y - q.z * x.z, q.w * x.x + q.z * x.y - q.y * x.z,
                 -q.z * x.x + q.w * x.y + q.x * x.z, q.y * x.x - q.x * x.y + q.w * x.z);
}
template <class T> RBX_HD V3<T> qBt(Q4<T> q, Q4<T> y) {
    return v3<T>(-q.x * y.w + q.w * y.x + q.z * y.y - q.y * y.z, -q.y * y.w - q.z * y.x + q.w * y.y + q.x * y.z,
                 -q.z * y.w + q.y * y.x - q.x * y.y + q.w * y.z);
}
template <class T> RBX_HD V3<T> qCt(Q4<T> q, Q4<T> y) {
    return v3<T>(-q.x * y.w + q.w * y.x - q.z * y.y + q.y * y.z, -q.y * y.w + q.z * y.x + q.w * y.y - q.x * y.z,
                 -q.z * y.w - q.y * y.x + q.x * y.y + q.w * y.z);
}
// q (x) e_k for k = 0, 1, 2 (the permutations B1, B2, B3 of MatVec.cpp:526-539)
template <class T> RBX_HD Q4<T> qBk(int k, Q4<T> q) {
    return k == 0 ? q4<T>(-q.x, q.w, q.z, -q.y) : (k == 1 ? q4<T>(-q.y, -q.z, q.w, q.x) : q4<T>(-q.z, q.y, -q.x, q.w));
}
template <class T> RBX_HD V3<T> rotate_to_space(Q4<T> q, V3<T> d) { return qCt(q, qB(q, d)); }  // At(q) d
template <class T> RBX_HD V3<T> rotate_to_body(Q4<T> q, V3<T> x) { return qBt(q, qC(q, x)); }   // A(q) x
template <class T> RBX_HD Q4<T> qmul(Q4<T> a, Q4<T> b) {
    return q4<T>(a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
                 a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x, a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w);
}

template <class T> struct Lim;
template <> struct Lim<double> {
    static constexpr double eps = DBL_EPSILON;
};
template <> struct Lim<float> {
    static constexpr float eps = FLT_EPSILON;
};

template <class T> RBX_HD T tmin(T a, T b) { return a < b ? a : b; }
template <class T> RBX_HD T tmax(T a, T b) { return a > b ? a : b; }
template <class T> RBX_HD T tabs(T a) { return a < T(0) ? -a : a; }

// sin x and cos x. Rotation angles of one step are small: for |x| <= 1/4 the Maclaurin series to
// x^13 and x^14 (truncation below 3e-21 relative, under FP64 rounding) replaces the general-range
// functions, whose argument reduction is costly on GB300's narrow FP64 pipe; larger arguments take
// sincos.
template <class T> RBX_HD void sin_cos(T x, T& s, T& c) {
    const T x2 = x * x;
    if (x2 <= T(0.0625)) {
        s = x * (T(1) + x2 * (T(-1) / T(6) + x2 * (T(1) / T(120) + x2 * (T(-1) / T(5040) + x2 * (T(1) / T(362880) +
              x2 * (T(-1) / T(39916800) + x2 * (T(1) / T(6227020800))))))));
        c = T(1) + x2 * (T(-1) / T(2) + x2 * (T(1) / T(24) + x2 * (T(-1) / T(720) + x2 * (T(1) / T(40320) +
              x2 * (T(-1) / T(3628800) + x2 * (T(1) / T(479001600) + x2 * (T(-1) / T(87178291200))))))));
        return;
    }
    s = sin(x);
    c = cos(x);
}

// Rotation about principal axis k by the angle pi implies (RigidBody.cpp:189-214).
template <class T> RBX_HD void uniaxial(int k, V3<T> invI, Q4<T>& q, Q4<T>& pi, T dt) {
    Q4<T> Bq = qBk(k, q);
    T ik = k == 0 ? invI.x : (k == 1 ? invI.y : invI.z);
    T phi = T(0.25) * dot(pi, Bq) * dt * ik;
    T s, c;
    sin_cos(phi, s, c);
    Q4<T> Bpi = qBk(k, pi);
    q = q * c + Bq * s;
    pi = pi * c + Bpi * s;
}

// NO-SQUISH symmetric splitting with n substeps (RigidBody.cpp:220-231).
template <class T> RBX_HD void nosquish_rotation(V3<T> invI, bool axis3, Q4<T>& q, Q4<T>& pi, T dt, int n) {
    T h = dt / T(n), hh = T(0.5) * h;
    for (int i = 0; i < n; i++) {
        if (axis3) uniaxial(2, invI, q, pi, hh);
        uniaxial(1, invI, q, pi, hh);
        uniaxial(0, invI, q, pi, h);
        uniaxial(1, invI, q, pi, hh);
        if (axis3) uniaxial(2, invI, q, pi, hh);
    }
}

// Rotation classes, fixed per body at setup from its principal moments.
enum RotClass : int { ROT_ASYMMETRIC = 0, ROT_SYMMETRIC_AXIS0 = 1, ROT_SYMMETRIC_AXIS2 = 2, ROT_SPHERICAL = 3 };

// Closed-form free rotation of a top with two equal moments (unique axis k; k = -1 for a
// spherical top): a rotation about the constant body-frame L at rate |L|/I_perp followed by a
// spin about axis k at rate (1/I_k - 1/I_perp) L_k. q and pi are right-multiplied by the same
// unit quaternion, which keeps pi = 2 q (x) (0, L).
template <class T> RBX_HD void symmetric_top_rotation(int k, T invIp, T invIk, V3<T> invI, Q4<T>& q, Q4<T>& pi, T dt) {
    V3<T> L = qBt(q, pi) * T(0.5);
    Q4<T> r = q4<T>(T(1), T(0), T(0), T(0));
    if (k < 0) {
        V3<T> w = mul(invI, L);
        T wn = sqrt(dot(w, w));
        if (wn > T(0)) {
            T a = T(0.5) * wn * dt, sa, ca;
            sin_cos(a, sa, ca);
            const T s = sa / wn;
            r = q4<T>(ca, w.x * s, w.y * s, w.z * s);
        }
    } else {
        T Ln = sqrt(dot(L, L));
        if (Ln > T(0)) {
            T a = T(0.5) * Ln * invIp * dt, sa, ca;
            sin_cos(a, sa, ca);
            const T s = sa / Ln;
            Q4<T> r1 = q4<T>(ca, L.x * s, L.y * s, L.z * s);
            T Lk = k == 0 ? L.x : L.z;
            T b = T(0.5) * (invIk - invIp) * Lk * dt;
            T sb, cb;
            sin_cos(b, sb, cb);
            Q4<T> r2 = k == 0 ? q4<T>(cb, sb, T(0), T(0)) : q4<T>(cb, T(0), T(0), sb);
            r = qmul(r1, r2);
        }
    }
    q = qmul(q, r);
    pi = qmul(pi, r);
    T nq = sqrt(dot(q, q));
    q = q * (T(1) / nq);
}

// ---------------------------------------------------------------------------------------------
// Exact free rotation of an asymmetric top (I.x > I.y > I.z): the Jacobi-elliptic solution of
// RigidBody.cpp:241-308, evaluated in increment form for FP64 on GB300, whose FP64 rate is 1/64 of
// FP32. The closed form spends dozens of FP64 divisions and square roots per body in its Carlson
// iterations (RF, RJ) and AGM, and loses accuracy to cancellation at small rotations (its
// third-kind integrals are differenced). This form spends about a dozen, 5.7x faster per step.
// Against RK4 of the Euler equations in long double it is within 4e-16 (the closed form: 1.4e-11).
// - L(t) in the body frame: the Jacobi functions at u0 + h from their values at u0, which the
//   state fixes, by the addition theorem (Abramowitz & Stegun 16.17). The functions of the small
//   h = wp t come from their Maclaurin series (A&S 16.22) for |h| <= 1/32, and from halving and the
//   duplication formulas above it. The series' first omitted term is below 1e-17 relative there.
// - The rotation: e(phi) (x) mu, with mu the minimal rotation taking L_hat(t) back to L_hat(0).
//   phi is the angle about L_hat(0), with rate omega . (n + n0) / (1 + n . n0), integrated by
//   5-point Gauss-Legendre quadrature. The rule's error, (5!)^4 / (11 (10!)^3) dt^11 f^(10), is
//   about 4e-13 (wp dt)^10 of phi.
// ---------------------------------------------------------------------------------------------

// sn(h), cn(h) - 1, dn(h) - 1 of parameter m for a small argument.
template <class T> RBX_HD void jacobi_small_t(T h, T m, T& sn, T& cm1, T& dm1) {
    int k = 0;
    while (tabs(h) > T(0.03125) && k < 60) {
        h *= T(0.5);
        k++;
    }
    const T u2 = h * h, m2 = m * m, m3 = m2 * m;
    sn = h * (T(1) + u2 * (-(T(1) + m) / T(6) +
                           u2 * ((T(1) + T(14) * m + m2) / T(120) +
                                 u2 * (-(T(1) + T(135) * m + T(135) * m2 + m3) / T(5040) +
                                       u2 * (T(1) + T(1228) * m + T(5478) * m2 + T(1228) * m3 + m2 * m2) / T(362880)))));
    cm1 = u2 * (T(-0.5) + u2 * ((T(1) + T(4) * m) / T(24) +
                                u2 * (-(T(1) + T(44) * m + T(16) * m2) / T(720) +
                                      u2 * (T(1) + T(408) * m + T(912) * m2 + T(64) * m3) / T(40320))));
    dm1 = m * u2 * (T(-0.5) + u2 * ((T(4) + m) / T(24) +
                                    u2 * (-(T(16) + T(44) * m + m2) / T(720) +
                                          u2 * (T(64) + T(912) * m + T(408) * m2 + m3) / T(40320))));
    for (int i = 0; i < k; i++) {  // sn(2h) = 2 s c d / D, cn(2h) - 1 = -2 s^2 d^2 / D, dn(2h) - 1 = -2 m s^2 c^2 / D
        const T c = T(1) + cm1, d = T(1) + dm1, s2 = sn * sn;
        const T inv = T(1) / (T(1) - m * s2 * s2);
        const T ns = T(2) * sn * c * d * inv;
        cm1 = T(-2) * s2 * d * d * inv;
        dm1 = T(-2) * m * s2 * c * c * inv;
        sn = ns;
    }
}

// (cos(a/2) - 1, sin(a/2) u): the increment of the rotation by angle a about the unit axis u, from
// the quarter angle (sin = 2 s c, cos - 1 = -2 s^2: no cancellation at any angle).
template <class T> RBX_HD Q4<T> axis_angle_increment(V3<T> u, T angle) {
    T sh, ch;
    sin_cos(T(0.25) * angle, sh, ch);
    const T s = T(2) * sh * ch, cm1 = T(-2) * sh * sh;
    return q4<T>(cm1, s * u.x, s * u.y, s * u.z);
}

template <class T> RBX_HD void exact_rotation_increment(V3<T> I, V3<T> invI, Q4<T>& q, Q4<T>& pi, T dt) {
    const V3<T> Iw = qBt(q, pi) * T(0.5);
    const T Lsq = dot(Iw, Iw);
    if (Lsq == T(0)) return;
    const T perp0 = Iw.y * Iw.y + Iw.z * Iw.z, perp2 = Iw.x * Iw.x + Iw.y * Iw.y;
    const T tiny = Lim<T>::eps * Lim<T>::eps;
    Q4<T> dr;
    V3<T> Lt = Iw;
    if (perp0 <= tiny * Lsq) {  // L on a principal axis: steady rotation about it
        dr = axis_angle_increment(v3<T>(T(1), T(0), T(0)), Iw.x * invI.x * dt);
    } else if (perp2 <= tiny * Lsq) {
        dr = axis_angle_increment(v3<T>(T(0), T(0), T(1)), Iw.z * invI.z * dt);
    } else {
        const V3<T> w0 = mul(invI, Iw);
        const T g01 = I.x - I.y, g12 = I.y - I.z, g02 = I.x - I.z;
        // L^2 - 2K I2 and 2K I0 - L^2 as sums of non-negative terms
        const T r1 = Iw.x * Iw.x * (g02 * invI.x) + Iw.y * Iw.y * (g12 * invI.y);
        const T r3 = Iw.y * Iw.y * (g01 * invI.y) + Iw.z * Iw.z * (g02 * invI.z);
        const T l1 = r1 * invI.y / g12, l3 = r3 * invI.y / g01;
        const bool case1 = l1 < l3;  // L = I a (cn, sn, dn); otherwise I a (dn, sn, cn)
        const T lmin = case1 ? l1 : l3, lmax = case1 ? l3 : l1;
        const T c13 = T(1) / g02;
        V3<T> a = v3<T>(sqrt(r1 * invI.x * c13), sqrt(lmin), sqrt(r3 * invI.z * c13));
        if (w0.x < T(0)) a.x = -a.x;
        if (w0.z < T(0)) a.z = -a.z;
        const T m = lmin / lmax;
        const T wp = -invI.y * a.x * a.z / (a.y * c13);
        T s0 = w0.y / a.y;
        s0 = tmin(T(1), tmax(T(-1), s0));
        const T cx = w0.x / a.x, cz = w0.z / a.z;
        const T c0 = case1 ? cx : cz, d0 = case1 ? cz : cx;
        const V3<T> Ia = mul(I, a);
        const T ms0s0 = m * s0 * s0;
        const T Lm = sqrt(Lsq);
        const V3<T> n0 = Iw * (T(1) / Lm);
        auto dL = [&](T t) {  // L(t) - L(0)
            T sh, cm1, dm1;
            jacobi_small_t(wp * t, m, sh, cm1, dm1);
            const T sh2 = sh * sh;
            const T invD = T(1) / (T(1) - ms0s0 * sh2);
            const T ds = (s0 * (cm1 + dm1 + cm1 * dm1) + sh * c0 * d0 + ms0s0 * s0 * sh2) * invD;
            const T dc = (c0 * cm1 - s0 * d0 * sh * (T(1) + dm1) + c0 * ms0s0 * sh2) * invD;
            const T dd = (d0 * dm1 - m * s0 * c0 * sh * (T(1) + cm1) + d0 * ms0s0 * sh2) * invD;
            return case1 ? v3<T>(Ia.x * dc, Ia.y * ds, Ia.z * dd) : v3<T>(Ia.x * dd, Ia.y * ds, Ia.z * dc);
        };
        const T glx[5] = {T(-0.906179845938663992797626878299), T(-0.538469310105683091036314420700), T(0),
                          T(0.538469310105683091036314420700), T(0.906179845938663992797626878299)};
        const T glw[5] = {T(0.236926885056189087514264040720), T(0.478628670499366468041291514836),
                          T(0.568888888888888888888888888889), T(0.478628670499366468041291514836),
                          T(0.236926885056189087514264040720)};
        T phi = T(0);
        for (int i = 0; i < 5; i++) {
            const V3<T> L = Iw + dL(T(0.5) * dt * (T(1) + glx[i]));
            const V3<T> n = L * (T(1) / sqrt(dot(L, L)));
            phi += glw[i] * dot(mul(invI, L), n + n0) / (T(1) + dot(n, n0));
        }
        phi *= T(0.5) * dt;
        const V3<T> dLt = dL(dt);
        Lt = Iw + dLt;
        const T Ltn = sqrt(dot(Lt, Lt));
        const T dLn = (T(2) * dot(Iw, dLt) + dot(dLt, dLt)) / (Ltn + Lm);  // |L(t)| - |L(0)|
        const V3<T> dn = (dLt - n0 * dLn) * (T(1) / Ltn);                   // n - n0 without cancellation
        const T dn2 = dot(dn, dn);
        const T mu0 = sqrt(tmax(T(1) - T(0.25) * dn2, T(0)));
        const V3<T> nv = cross(dn, n0) * (T(0.5) / tmax(mu0, T(1e-300)));
        const Q4<T> dmu = q4<T>(T(-0.25) * dn2 / (T(1) + mu0), nv.x, nv.y, nv.z);
        const Q4<T> de = axis_angle_increment(n0, phi);
        dr = de + dmu + qmul(de, dmu);
        Lt = Lt * (Lm / Ltn);  // |L| is invariant: remove the rounding of its length
    }
    q = q + qmul(q, dr);
    q = q * (T(1) / sqrt(dot(q, q)));
    // pi = 2 B(q) L(t) / |q|^2, so that Bt(q, pi) / 2 gives back L(t) exactly whatever the rounding of
    // the normalisation; without the division L and the energy drift by |q|^2 - 1 each step
    pi = qB(q, Lt * (T(2) / dot(q, q)));
}

// Mode-0 free rotation for any body: closed forms for the degenerate classes, the elliptic
// solution otherwise.
template <class T> RBX_HD void exact_rotation(int cls, V3<T> I, V3<T> invI, Q4<T>& q, Q4<T>& pi, T dt) {
    if (cls == ROT_ASYMMETRIC) {
        exact_rotation_increment(I, invI, q, pi, dt);
    } else if (cls == ROT_SPHERICAL) {
        symmetric_top_rotation(-1, T(0), T(0), invI, q, pi, dt);
    } else if (cls == ROT_SYMMETRIC_AXIS0) {
        symmetric_top_rotation(0, T(2) / (I.y + I.z), invI.x, invI, q, pi, dt);
    } else {  // unique axis 2; a linear body has invI.z = 0
        T invIp = invI.z == T(0) ? invI.x : T(2) / (I.x + I.y);
        symmetric_top_rotation(2, invIp, invI.z, invI, q, pi, dt);
    }
}

}  // namespace rbx
