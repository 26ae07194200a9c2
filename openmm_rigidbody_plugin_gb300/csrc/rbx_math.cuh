// rbx_math.cuh -- quaternion algebra, elliptic functions and torque-free rotations, templated on
// the scalar type (float or double) and usable from host and device code.
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
    static constexpr double eps = DBL_EPSILON, tiny = DBL_MIN, huge = DBL_MAX, errtol = 0.001;
    static constexpr double rj_lolim = 4.809554074311741e-103;  // cbrt(5 * DBL_MIN)
    static constexpr double rj_uplim = 9.901548214916537e+101;  // 0.3 * cbrt(0.2 * DBL_MAX)
    static constexpr int levels = 16;
};
template <> struct Lim<float> {
    static constexpr float eps = FLT_EPSILON, tiny = FLT_MIN, huge = FLT_MAX, errtol = 0.03f;
    static constexpr float rj_lolim = 3.888035159154014e-13f;  // cbrt(5 * FLT_MIN)
    static constexpr float rj_uplim = 1.2248353902037021e+12f;  // 0.3 * cbrt(0.2 * FLT_MAX)
    static constexpr int levels = 10;
};

template <class T> RBX_HD T sgn(T x) { return x >= T(0) ? T(1) : T(-1); }
template <class T> RBX_HD T tmin(T a, T b) { return a < b ? a : b; }
template <class T> RBX_HD T tmax(T a, T b) { return a > b ? a : b; }
template <class T> RBX_HD T tabs(T a) { return a < T(0) ? -a : a; }
template <class T> RBX_HD T quiet_nan() { return T(NAN); }

// Jacobi sn, cn, dn of (u | m): arithmetic-geometric mean followed by the descending recursion
// (the method of openmmapi/include/internal/ellipticFunctions.h:34-100).
template <class T> RBX_HD void jacobi_sncndn(T u, T m, T& sn, T& cn, T& dn) {
    const T EPS = Lim<T>::eps;
    if (tabs(m) > T(1)) { sn = cn = dn = quiet_nan<T>(); return; }
    if (tabs(m) < T(2) * EPS) { sn = sin(u); cn = cos(u); dn = T(1); return; }
    if (tabs(m - T(1)) < T(2) * EPS) { sn = tanh(u); cn = T(1) / cosh(u); dn = cn; return; }
    constexpr int N = Lim<T>::levels;
    T mu[N], nu[N];
    int n = 0;
    mu[0] = T(1);
    nu[0] = sqrt(T(1) - m);
    while (tabs(mu[n] - nu[n]) > T(4) * EPS * tabs(mu[n] + nu[n])) {
        mu[n + 1] = T(0.5) * (mu[n] + nu[n]);
        nu[n + 1] = sqrt(mu[n] * nu[n]);
        ++n;
        if (n >= N - 1) { sn = cn = dn = quiet_nan<T>(); return; }
    }
    T s = sin(u * mu[n]), co = cos(u * mu[n]);
    bool tangent = tabs(s) < tabs(co);
    T c = mu[n] * (tangent ? s / co : co / s);
    T d = T(1);
    while (n > 0) {
        n--;
        T cprev = c;
        c = d * cprev;
        T r = (cprev * cprev) / mu[n + 1];
        d = (r + nu[n]) / (r + mu[n]);
    }
    if (tangent) {
        dn = sqrt(T(1) - m) / d;
        cn = dn * sgn(co) / hypot(T(1), c);
        sn = cn * c / sqrt(T(1) - m);
    } else {
        dn = d;
        sn = sgn(s) / hypot(T(1), c);
        cn = c * sn;
    }
}

// Carlson's R_C, R_F and R_J by duplication (B. C. Carlson, Numer. Algorithms 10 (1995) 13-26;
// the variants of ellipticFunctions.h:105-249 with the same stopping tolerances).
template <class T> RBX_HD T carlson_rc(T x, T y) {
    const T lolim = T(5) * Lim<T>::tiny, uplim = T(0.2) * Lim<T>::huge, errtol = T(Lim<T>::errtol);
    if (x < T(0) || y < T(0) || x + y < lolim || x > uplim || y > uplim) return quiet_nan<T>();
    T mu, s;
    for (int n = 0;; n++) {
        mu = (x + y + y) / T(3);
        s = (y + mu) / mu - T(2);
        if (tabs(s) < errtol) break;
        T lam = T(2) * sqrt(x) * sqrt(y) + y;
        x = (x + lam) * T(0.25);
        y = (y + lam) * T(0.25);
        if (n + 1 == 10000) return quiet_nan<T>();
    }
    T series = s * s * (T(0.3) + s * (T(1.0 / 7.0) + s * (T(0.375) + s * T(9.0 / 22.0))));
    return (T(1) + series) / sqrt(mu);
}

template <class T> RBX_HD T carlson_rf(T x, T y, T z) {
    const T lolim = T(5) * Lim<T>::tiny, uplim = T(0.2) * Lim<T>::huge, errtol = T(Lim<T>::errtol);
    if (x < T(0) || y < T(0) || z < T(0) || x + y < lolim || x + z < lolim || y + z < lolim || x > uplim ||
        y > uplim || z > uplim)
        return quiet_nan<T>();
    T mu, X, Y, Z;
    for (int n = 0;; n++) {
        mu = (x + y + z) / T(3);
        X = T(2) - (mu + x) / mu;
        Y = T(2) - (mu + y) / mu;
        Z = T(2) - (mu + z) / mu;
        if (tmax(tabs(X), tmax(tabs(Y), tabs(Z))) < errtol) break;
        T sx = sqrt(x), sy = sqrt(y), sz = sqrt(z);
        T lam = sx * (sy + sz) + sy * sz;
        x = (x + lam) * T(0.25);
        y = (y + lam) * T(0.25);
        z = (z + lam) * T(0.25);
        if (n + 1 == 10000) return quiet_nan<T>();
    }
    T e2 = X * Y - Z * Z, e3 = X * Y * Z;
    T s = T(1) + (T(1.0 / 24.0) * e2 - T(0.1) - T(3.0 / 44.0) * e3) * e2 + T(1.0 / 14.0) * e3;
    return s / sqrt(mu);
}

template <class T> RBX_HD T carlson_rj(T x, T y, T z, T p) {
    const T lolim = Lim<T>::rj_lolim, uplim = Lim<T>::rj_uplim;
    const T errtol = T(Lim<T>::errtol);
    if (x < T(0) || y < T(0) || z < T(0) || x + y < lolim || x + z < lolim || y + z < lolim || p < lolim ||
        x > uplim || y > uplim || z > uplim || p > uplim)
        return quiet_nan<T>();
    const T c1 = T(3.0 / 14.0), c2 = T(1.0 / 3.0), c3 = T(3.0 / 22.0), c4 = T(3.0 / 26.0);
    T sigma = T(0), power4 = T(1), mu, X, Y, Z, P;
    for (int n = 0;; n++) {
        mu = (x + y + z + p + p) * T(0.2);
        X = (mu - x) / mu;
        Y = (mu - y) / mu;
        Z = (mu - z) / mu;
        P = (mu - p) / mu;
        if (tmax(tmax(tabs(X), tabs(Y)), tmax(tabs(Z), tabs(P))) < errtol) break;
        T sx = sqrt(x), sy = sqrt(y), sz = sqrt(z);
        T lam = sx * (sy + sz) + sy * sz;
        T alfa = p * (sx + sy + sz) + sx * sy * sz;
        alfa = alfa * alfa;
        T beta = p * (p + lam) * (p + lam);
        T rc = carlson_rc(alfa, beta);
        if (rc != rc) return quiet_nan<T>();
        sigma += power4 * rc;
        power4 *= T(0.25);
        x = (x + lam) * T(0.25);
        y = (y + lam) * T(0.25);
        z = (z + lam) * T(0.25);
        p = (p + lam) * T(0.25);
        if (n + 1 == 10000) return quiet_nan<T>();
    }
    T ea = X * (Y + Z) + Y * Z, eb = X * Y * Z, ec = P * P;
    T e2 = ea - T(3) * ec, e3 = eb + T(2) * P * (ea - ec);
    T s1 = T(1) + e2 * (-c1 + T(0.75) * c3 * e2 - T(1.5) * c4 * e3);
    T s2 = eb * (T(0.5) * c2 + P * (-c3 - c3 + P * c4));
    T s3 = P * ea * (c2 - P * c3) - c2 * P * ec;
    return T(3) * sigma + power4 * (s1 + s2 + s3) / (mu * sqrt(mu));
}

// Incomplete third-kind term of the exact rotation (ellipticFunctions.h:251-254).
template <class T> RBX_HD T omega_term(T x, T n, T m) {
    T x2 = x * x;
    return (T(-1) / T(3)) * n * x * x2 * carlson_rj(T(1) - x2, T(1) - m * x2, T(1), T(1) + n * x2);
}

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

template <class T> RBX_HD int stair_case(T x) { return x > T(0) ? (int)ceil(x - T(0.5)) : (int)floor(x + T(0.5)); }

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

// Torque-free rotation by the exact Jacobi-elliptic solution of an asymmetric top
// (RigidBody.cpp:241-308). The principal moments must be sorted, I.x >= I.y >= I.z.
template <class T> RBX_HD void exact_rotation_asymmetric(V3<T> I, V3<T> invI, Q4<T>& q, Q4<T>& pi, T dt) {
    const T EPS = Lim<T>::eps;
    const T PI = T(3.14159265358979323846264338328);
    V3<T> Iw = qBt(q, pi) * T(0.5);
    V3<T> w0 = mul(invI, Iw);
    T Lsq = Iw.y * Iw.y + Iw.z * Iw.z;
    if (Lsq < EPS) { uniaxial(0, invI, q, pi, dt); return; }
    Lsq += Iw.x * Iw.x;
    T L = sqrt(Lsq);
    T twoKr = dot(Iw, w0);
    Q4<T> z0 = q4<T>(Iw.z, Iw.y, L - Iw.x, T(0));
    T r1 = Lsq - twoKr * I.z;
    T r3 = twoKr * I.x - Lsq;
    T l1 = r1 * invI.y / (I.y - I.z);
    T l3 = r3 * invI.y / (I.x - I.y);
    T lmin = tmin(l1, l3);
    T c13 = T(1) / (I.x - I.z);
    V3<T> a = v3<T>(sgn(w0.x) * sqrt(r1 * invI.x * c13), sqrt(lmin), sgn(w0.z) * sqrt(r3 * invI.z * c13));
    T m = lmin / tmax(l1, l3);
    T K = carlson_rf(T(0), T(1) - m, T(1));
    T inv2K = T(0.5) / K;
    T s0 = w0.y / a.y;
    T c0, u0;
    int i0;
    if (tabs(s0) < T(1)) {
        c0 = l1 < l3 ? w0.x / a.x : w0.z / a.z;
        u0 = s0 * carlson_rf(T(1) - s0 * s0, T(1) - m * s0 * s0, T(1));
        i0 = stair_case(u0 * inv2K);
    } else {
        a.y = tabs(w0.y);
        s0 = sgn(s0);
        c0 = T(0);
        u0 = s0 * K;
        i0 = 0;
    }
    T wp = -invI.y * a.x * a.z / (a.y * c13);
    T u = wp * dt + u0;
    int jump = stair_case(u * inv2K) - i0;
    T sn, cn, dn, dF;
    jacobi_sncndn(u, m, sn, cn, dn);
    T alpha = I.x * a.x / L;
    T eta = alpha * alpha;
    eta /= T(1) - eta;
    V3<T> Ia = mul(I, a);
    if (l1 < l3) {
        T C = sqrt(m + eta);
        dF = u - u0 + sgn(cn) * omega_term(sn, eta, m) - sgn(c0) * omega_term(s0, eta, m) +
             (alpha / C) * (atan(C * sn / dn) - atan(C * s0 * a.z / w0.z));
        if (jump != 0) dF += T(jump) * T(2) * omega_term(T(1), eta, m);
        Iw = mul(Ia, v3<T>(cn, sn, dn));
    } else {
        T k2eta = m * eta;
        T C = sqrt(T(1) + k2eta);
        dF = u - u0 + sgn(cn) * omega_term(sn, k2eta, m) - sgn(c0) * omega_term(s0, k2eta, m) +
             (alpha / C) * (atan(C * sn / cn) - atan(C * s0 / c0));
        if (jump != 0) dF += T(jump) * (T(2) * omega_term(T(1), k2eta, m) + (alpha / C) * PI);
        Iw = mul(Ia, v3<T>(dn, sn, cn));
    }
    dF *= T(1) + eta;
    T theta = (Lsq * (u - u0) + r3 * dF) / (T(2) * L * I.x * wp);
    T ct, st;
    sin_cos(theta, st, ct);
    Q4<T> z = q4<T>(Iw.z * ct + (-Iw.y) * st, Iw.y * ct + Iw.z * st, (L - Iw.x) * ct + T(0) * st,
                    T(0) * ct + (L - Iw.x) * st);
    // q <- q (x) conj(z0) (x) z, written as z <z0,q> + C(z, Ct(z0, q)) (RigidBody.cpp:305)
    T zq = dot(z0, q);
    Q4<T> cz = qC(z, qCt(z0, q));
    q = z * zq + cz;
    T nq2 = q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z;
    q = q * (T(1) / sqrt(nq2));
    pi = qB(q, Iw * T(2));
}

// Mode-0 free rotation for any body: closed forms for the degenerate classes, the elliptic
// solution otherwise.
template <class T> RBX_HD void exact_rotation(int cls, V3<T> I, V3<T> invI, Q4<T>& q, Q4<T>& pi, T dt) {
    if (cls == ROT_ASYMMETRIC) {
        exact_rotation_asymmetric(I, invI, q, pi, dt);
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
