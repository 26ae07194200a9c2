/*
 * rbx_oracle.c -- CPU restatement (FP64) of the OpenMM rigid-body plugin's integrator.
 *
 * TEST INFRASTRUCTURE ONLY (see rbx_oracle.h). Each function cites the reference file:line whose
 * behaviour it restates; paths are relative to the reference project root.
 *
 * Conventions: quaternions are double[4] = (q0, q1, q2, q3); B(q)x = q (x) (0,x) and
 * C(q)x = (0,x) (x) q in Hamilton products, Bt/Ct their transposes, so that the space-to-body
 * rotation is A(q)x = Bt(q, C(q, x)) and the body-to-space rotation At(q)x = Ct(q, B(q, x))
 * (openmmapi/src/MatVec.cpp:495-549).
 */
#define _POSIX_C_SOURCE 200809L
#include "rbx_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORC_PI 3.14159265358979323846264338328
#define SGN(x) ((x) >= 0 ? 1.0 : -1.0)

static __thread char g_err[256];
const char* orc_last_error(void) { return g_err; }

/* ------------------------------------------------------------------------------------------ */
/* Quaternion and 3-vector algebra (openmmapi/src/MatVec.cpp:495-564)                          */
/* ------------------------------------------------------------------------------------------ */

static void qB(const double* q, const double* x, double* r) {
    r[0] = -q[1] * x[0] - q[2] * x[1] - q[3] * x[2];
    r[1] = q[0] * x[0] - q[3] * x[1] + q[2] * x[2];
    r[2] = q[3] * x[0] + q[0] * x[1] - q[1] * x[2];
    r[3] = -q[2] * x[0] + q[1] * x[1] + q[0] * x[2];
}
static void qC(const double* q, const double* x, double* r) {
    r[0] = -q[1] * x[0] - q[2] * x[1] - q[3] * x[2];
    r[1] = q[0] * x[0] + q[3] * x[1] - q[2] * x[2];
    r[2] = -q[3] * x[0] + q[0] * x[1] + q[1] * x[2];
    r[3] = q[2] * x[0] - q[1] * x[1] + q[0] * x[2];
}
static void qBt(const double* q, const double* y, double* r) {
    r[0] = -q[1] * y[0] + q[0] * y[1] + q[3] * y[2] - q[2] * y[3];
    r[1] = -q[2] * y[0] - q[3] * y[1] + q[0] * y[2] + q[1] * y[3];
    r[2] = -q[3] * y[0] + q[2] * y[1] - q[1] * y[2] + q[0] * y[3];
}
static void qCt(const double* q, const double* y, double* r) {
    r[0] = -q[1] * y[0] + q[0] * y[1] - q[3] * y[2] + q[2] * y[3];
    r[1] = -q[2] * y[0] + q[3] * y[1] + q[0] * y[2] - q[1] * y[3];
    r[2] = -q[3] * y[0] - q[2] * y[1] + q[1] * y[2] + q[0] * y[3];
}
/* Permutations B1, B2, B3 (MatVec.cpp:526-539): q (x) e_k */
static void qBk(int k, const double* q, double* r) {
    if (k == 0) { r[0] = -q[1]; r[1] = q[0]; r[2] = q[3]; r[3] = -q[2]; }
    else if (k == 1) { r[0] = -q[2]; r[1] = -q[3]; r[2] = q[0]; r[3] = q[1]; }
    else { r[0] = -q[3]; r[1] = q[2]; r[2] = -q[1]; r[3] = q[0]; }
}
static void qA(const double* q, const double* x, double* r) { double t[4]; qC(q, x, t); qBt(q, t, r); }
static void qAt(const double* q, const double* x, double* r) { double t[4]; qB(q, x, t); qCt(q, t, r); }
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double dot4(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3]; }
static void cross3(const double* a, const double* b, double* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
/* Hamilton product r = a (x) b (used only by the robust closed forms). */
static void qmul(const double* a, const double* b, double* r) {
    double t0 = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    double t1 = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    double t2 = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    double t3 = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
    r[0] = t0; r[1] = t1; r[2] = t2; r[3] = t3;
}

/* Unit quaternion from a rotation matrix, Shepperd's method (MatVec.cpp:344-373). M row-major. */
static void quat_from_matrix(const double* M, double* q) {
    double a11 = M[0], a22 = M[4], a33 = M[8];
    double Q2[4] = {1.0 + a11 + a22 + a33, 1.0 + a11 - a22 - a33, 1.0 - a11 + a22 - a33, 1.0 - a11 - a22 + a33};
    int imax = 0;
    double vmax = Q2[0];
    for (int i = 1; i < 4; i++)
        if (Q2[i] > vmax) { vmax = Q2[i]; imax = i; }
    double f = 0.5 / sqrt(vmax);
#define AM(i, j) M[3 * (i) + (j)]
    if (imax == 0) {
        q[1] = (AM(1, 2) - AM(2, 1)) * f; q[2] = (AM(2, 0) - AM(0, 2)) * f; q[3] = (AM(0, 1) - AM(1, 0)) * f;
    } else if (imax == 1) {
        q[0] = (AM(1, 2) - AM(2, 1)) * f; q[2] = (AM(0, 1) + AM(1, 0)) * f; q[3] = (AM(0, 2) + AM(2, 0)) * f;
    } else if (imax == 2) {
        q[0] = (AM(2, 0) - AM(0, 2)) * f; q[1] = (AM(0, 1) + AM(1, 0)) * f; q[3] = (AM(1, 2) + AM(2, 1)) * f;
    } else {
        q[0] = (AM(0, 1) - AM(1, 0)) * f; q[1] = (AM(0, 2) + AM(2, 0)) * f; q[2] = (AM(1, 2) + AM(2, 1)) * f;
    }
#undef AM
    q[imax] = vmax * f;
}

/* ------------------------------------------------------------------------------------------ */
/* Special functions (openmmapi/include/internal/ellipticFunctions.h)                          */
/* ------------------------------------------------------------------------------------------ */

/* Jacobi sn, cn, dn by the arithmetic-geometric mean and descending recursion
 * (ellipticFunctions.h:34-100). */
void orc_jacobi_sncndn(double u, double m, double* sn, double* cn, double* dn) {
    const double EPS = DBL_EPSILON;
    if (fabs(m) > 1.0) { *sn = *cn = *dn = NAN; return; }
    if (fabs(m) < 2.0 * EPS) { *sn = sin(u); *cn = cos(u); *dn = 1.0; return; }
    if (fabs(m - 1.0) < 2.0 * EPS) { *sn = tanh(u); *cn = 1.0 / cosh(u); *dn = *cn; return; }
    enum { LEVELS = 16 };
    double mu[LEVELS], nu[LEVELS], c[LEVELS], d[LEVELS];
    int n = 0;
    mu[0] = 1.0;
    nu[0] = sqrt(1.0 - m);
    while (fabs(mu[n] - nu[n]) > 4.0 * EPS * fabs(mu[n] + nu[n])) {
        mu[n + 1] = 0.5 * (mu[n] + nu[n]);
        nu[n + 1] = sqrt(mu[n] * nu[n]);
        ++n;
        if (n >= LEVELS - 1) { *sn = *cn = *dn = NAN; return; }
    }
    double s = sin(u * mu[n]), co = cos(u * mu[n]);
    int tangent = fabs(s) < fabs(co);
    c[n] = mu[n] * (tangent ? s / co : co / s);
    d[n] = 1.0;
    while (n > 0) {
        n--;
        c[n] = d[n + 1] * c[n + 1];
        double r = (c[n + 1] * c[n + 1]) / mu[n + 1];
        d[n] = (r + nu[n]) / (r + mu[n]);
    }
    if (tangent) {
        *dn = sqrt(1.0 - m) / d[0];
        *cn = (*dn) * SGN(co) / hypot(1.0, c[0]);
        *sn = (*cn) * c[0] / sqrt(1.0 - m);
    } else {
        *dn = d[0];
        *sn = SGN(s) / hypot(1.0, c[0]);
        *cn = c[0] * (*sn);
    }
}

/* Carlson's degenerate integral R_C by duplication (ellipticFunctions.h:105-133). */
double orc_carlson_rc(double x, double y) {
    const double lolim = 5.0 * DBL_MIN, uplim = 0.2 * DBL_MAX, errtol = 0.001;
    if (x < 0.0 || y < 0.0 || x + y < lolim || x > uplim || y > uplim) return NAN;
    double mu, s;
    for (int n = 0;; n++) {
        mu = (x + y + y) / 3.0;
        s = (y + mu) / mu - 2.0;
        if (fabs(s) < errtol) break;
        double lam = 2.0 * sqrt(x) * sqrt(y) + y;
        x = (x + lam) * 0.25;
        y = (y + lam) * 0.25;
        if (n + 1 == 10000) return NAN;
    }
    double series = s * s * (0.3 + s * (1.0 / 7.0 + s * (0.375 + s * (9.0 / 22.0))));
    return (1.0 + series) / sqrt(mu);
}

/* Carlson's symmetric integral of the first kind R_F (ellipticFunctions.h:138-181). */
double orc_carlson_rf(double x, double y, double z) {
    const double lolim = 5.0 * DBL_MIN, uplim = 0.2 * DBL_MAX, errtol = 0.001;
    if (x < 0.0 || y < 0.0 || z < 0.0 || x + y < lolim || x + z < lolim || y + z < lolim ||
        x > uplim || y > uplim || z > uplim)
        return NAN;
    double mu, X, Y, Z;
    for (int n = 0;; n++) {
        mu = (x + y + z) / 3.0;
        X = 2.0 - (mu + x) / mu;
        Y = 2.0 - (mu + y) / mu;
        Z = 2.0 - (mu + z) / mu;
        double e = fmax(fabs(X), fmax(fabs(Y), fabs(Z)));
        if (e < errtol) break;
        double sx = sqrt(x), sy = sqrt(y), sz = sqrt(z);
        double lam = sx * (sy + sz) + sy * sz;
        x = (x + lam) * 0.25;
        y = (y + lam) * 0.25;
        z = (z + lam) * 0.25;
        if (n + 1 == 10000) return NAN;
    }
    double e2 = X * Y - Z * Z, e3 = X * Y * Z;
    double s = 1.0 + ((1.0 / 24.0) * e2 - 0.1 - (3.0 / 44.0) * e3) * e2 + (1.0 / 14.0) * e3;
    return s / sqrt(mu);
}

/* Carlson's symmetric integral of the third kind R_J (ellipticFunctions.h:186-249). */
double orc_carlson_rj(double x, double y, double z, double p) {
    const double lolim = pow(5.0 * DBL_MIN, 1.0 / 3.0), uplim = 0.3 * pow(0.2 * DBL_MAX, 1.0 / 3.0);
    const double errtol = 0.001;
    if (x < 0.0 || y < 0.0 || z < 0.0 || x + y < lolim || x + z < lolim || y + z < lolim || p < lolim ||
        x > uplim || y > uplim || z > uplim || p > uplim)
        return NAN;
    const double c1 = 3.0 / 14.0, c2 = 1.0 / 3.0, c3 = 3.0 / 22.0, c4 = 3.0 / 26.0;
    double sigma = 0.0, power4 = 1.0, mu, X, Y, Z, P;
    for (int n = 0;; n++) {
        mu = (x + y + z + p + p) * 0.2;
        X = (mu - x) / mu;
        Y = (mu - y) / mu;
        Z = (mu - z) / mu;
        P = (mu - p) / mu;
        double e = fmax(fmax(fabs(X), fabs(Y)), fmax(fabs(Z), fabs(P)));
        if (e < errtol) break;
        double sx = sqrt(x), sy = sqrt(y), sz = sqrt(z);
        double lam = sx * (sy + sz) + sy * sz;
        double alfa = p * (sx + sy + sz) + sx * sy * sz;
        alfa = alfa * alfa;
        double beta = p * (p + lam) * (p + lam);
        double rc = orc_carlson_rc(alfa, beta);
        if (isnan(rc)) return NAN;
        sigma += power4 * rc;
        power4 *= 0.25;
        x = (x + lam) * 0.25;
        y = (y + lam) * 0.25;
        z = (z + lam) * 0.25;
        p = (p + lam) * 0.25;
        if (n + 1 == 10000) return NAN;
    }
    double ea = X * (Y + Z) + Y * Z, eb = X * Y * Z, ec = P * P;
    double e2 = ea - 3.0 * ec, e3 = eb + 2.0 * P * (ea - ec);
    double s1 = 1.0 + e2 * (-c1 + 0.75 * c3 * e2 - 1.5 * c4 * e3);
    double s2 = eb * (0.5 * c2 + P * (-c3 - c3 + P * c4));
    double s3 = P * ea * (c2 - P * c3) - c2 * P * ec;
    return 3.0 * sigma + power4 * (s1 + s2 + s3) / (mu * sqrt(mu));
}

/* Incomplete third-kind term used by the exact rotation (ellipticFunctions.h:251-254). */
static double omega_term(double x, double n, double m) {
    double x2 = x * x;
    return (-1.0 / 3.0) * n * x * x2 * orc_carlson_rj(1.0 - x2, 1.0 - m * x2, 1.0, 1.0 + n * x2);
}

/* ------------------------------------------------------------------------------------------ */
/* Free rotation (openmmapi/src/RigidBody.cpp:189-308)                                         */
/* ------------------------------------------------------------------------------------------ */

/* Rotation about principal axis k by the angle that pi implies (RigidBody.cpp:189-214). */
static void uniaxial(int k, const double* invI, double* q, double* pi, double dt) {
    double Bq[4], Bpi[4];
    qBk(k, q, Bq);
    double phi = 0.25 * dot4(pi, Bq) * dt * invI[k];
    double s = sin(phi), c = cos(phi);
    qBk(k, pi, Bpi);
    for (int i = 0; i < 4; i++) {
        q[i] = q[i] * c + Bq[i] * s;
        pi[i] = pi[i] * c + Bpi[i] * s;
    }
}

/* NO-SQUISH symmetric splitting with n substeps (RigidBody.cpp:220-231). */
void orc_nosquish_rotation(const double* invI, int dof, double* q, double* pi, double dt, int n) {
    double h = dt / n, hh = 0.5 * h;
    int axis3 = dof == 6;
    for (int i = 0; i < n; i++) {
        if (axis3) uniaxial(2, invI, q, pi, hh);
        uniaxial(1, invI, q, pi, hh);
        uniaxial(0, invI, q, pi, h);
        uniaxial(1, invI, q, pi, hh);
        if (axis3) uniaxial(2, invI, q, pi, hh);
    }
}

static int stair_case(double x) { return x > 0 ? (int)ceil(x - 0.5) : (int)floor(x + 0.5); }

/* Robust closed form for a top with two equal moments about the unique axis k (body frame):
 * the motion is a rotation about the constant body-frame L direction at rate |L|/I_perp
 * followed by a spin about axis k at rate (1/I_k - 1/I_perp) L_k. A spherical top is the case
 * k=-1 (pure rotation about omega). Both q and pi are right-multiplied by the same unit
 * quaternion, which keeps pi = 2 q (x) (0,L). */
static void symmetric_top_rotation(int k, double invIp, double invIk, const double* invI, double* q,
                                   double* pi, double dt) {
    double L[3];
    qBt(q, pi, L);
    for (int i = 0; i < 3; i++) L[i] *= 0.5;
    double r[4] = {1.0, 0.0, 0.0, 0.0};
    if (k < 0) {
        double w[3] = {invI[0] * L[0], invI[1] * L[1], invI[2] * L[2]};
        double wn = sqrt(dot3(w, w));
        if (wn > 0.0) {
            double a = 0.5 * wn * dt, s = sin(a) / wn;
            r[0] = cos(a); r[1] = w[0] * s; r[2] = w[1] * s; r[3] = w[2] * s;
        }
    } else {
        double Ln = sqrt(dot3(L, L));
        if (Ln > 0.0) {
            double a = 0.5 * Ln * invIp * dt, s = sin(a) / Ln;
            double r1[4] = {cos(a), L[0] * s, L[1] * s, L[2] * s};
            double b = 0.5 * (invIk - invIp) * L[k] * dt;
            double r2[4] = {cos(b), 0.0, 0.0, 0.0};
            r2[1 + k] = sin(b);
            qmul(r1, r2, r);
        }
    }
    double t[4];
    qmul(q, r, t); memcpy(q, t, sizeof t);
    qmul(pi, r, t); memcpy(pi, t, sizeof t);
    double nq = sqrt(dot4(q, q));
    for (int i = 0; i < 4; i++) q[i] /= nq;
}

/* Torque-free rotation by the exact Jacobi-elliptic solution (RigidBody.cpp:241-308).
 * With robust=1, spherical, symmetric and linear tops take the closed form above instead of
 * the asymmetric formula, which divides by I0-I1 or I1-I2 (RigidBody.cpp:254-255). */
void orc_exact_rotation(const double* I, const double* invI, double* q, double* pi, double dt, int robust) {
    if (robust) {
        const double tol = 1e-12 * I[0];
        if (invI[2] == 0.0) { symmetric_top_rotation(2, invI[0], 0.0, invI, q, pi, dt); return; }
        int g01 = I[0] - I[1] <= tol, g12 = I[1] - I[2] <= tol;
        if (g01 && g12) { symmetric_top_rotation(-1, 0.0, 0.0, invI, q, pi, dt); return; }
        if (g01) { symmetric_top_rotation(2, 2.0 / (I[0] + I[1]), invI[2], invI, q, pi, dt); return; }
        if (g12) { symmetric_top_rotation(0, 2.0 / (I[1] + I[2]), invI[0], invI, q, pi, dt); return; }
    }
    const double EPS = DBL_EPSILON;
    double Iw[3], w0[3];
    qBt(q, pi, Iw);
    for (int i = 0; i < 3; i++) { Iw[i] *= 0.5; w0[i] = invI[i] * Iw[i]; }
    double Lsq = Iw[1] * Iw[1] + Iw[2] * Iw[2];
    if (Lsq < EPS) { uniaxial(0, invI, q, pi, dt); return; }
    Lsq += Iw[0] * Iw[0];
    double L = sqrt(Lsq);
    double twoKr = dot3(Iw, w0);
    double z0[4] = {Iw[2], Iw[1], L - Iw[0], 0.0};
    double r1 = Lsq - twoKr * I[2];
    double r3 = twoKr * I[0] - Lsq;
    double l1 = r1 * invI[1] / (I[1] - I[2]);
    double l3 = r3 * invI[1] / (I[0] - I[1]);
    double lmin = fmin(l1, l3);
    double c13 = 1.0 / (I[0] - I[2]);
    double a[3] = {SGN(w0[0]) * sqrt(r1 * invI[0] * c13), sqrt(lmin), SGN(w0[2]) * sqrt(r3 * invI[2] * c13)};
    double m = lmin / fmax(l1, l3);
    double K = orc_carlson_rf(0.0, 1.0 - m, 1.0);
    double inv2K = 0.5 / K;
    double s0 = w0[1] / a[1];
    double c0, u0;
    int i0;
    if (fabs(s0) < 1.0) {
        c0 = l1 < l3 ? w0[0] / a[0] : w0[2] / a[2];
        u0 = s0 * orc_carlson_rf(1.0 - s0 * s0, 1.0 - m * s0 * s0, 1.0);
        i0 = stair_case(u0 * inv2K);
    } else {
        a[1] = fabs(w0[1]);
        s0 = SGN(s0);
        c0 = 0.0;
        u0 = s0 * K;
        i0 = 0;
    }
    double wp = -invI[1] * a[0] * a[2] / (a[1] * c13);
    double u = wp * dt + u0;
    int jump = stair_case(u * inv2K) - i0;
    double sn, cn, dn, dF;
    orc_jacobi_sncndn(u, m, &sn, &cn, &dn);
    double alpha = I[0] * a[0] / L;
    double eta = alpha * alpha;
    eta /= 1.0 - eta;
    double Ia[3] = {I[0] * a[0], I[1] * a[1], I[2] * a[2]};
    if (l1 < l3) {
        double C = sqrt(m + eta);
        dF = u - u0 + SGN(cn) * omega_term(sn, eta, m) - SGN(c0) * omega_term(s0, eta, m) +
             (alpha / C) * (atan(C * sn / dn) - atan(C * s0 * a[2] / w0[2]));
        if (jump != 0) dF += jump * 2.0 * omega_term(1.0, eta, m);
        Iw[0] = Ia[0] * cn; Iw[1] = Ia[1] * sn; Iw[2] = Ia[2] * dn;
    } else {
        double k2eta = m * eta;
        double C = sqrt(1.0 + k2eta);
        dF = u - u0 + SGN(cn) * omega_term(sn, k2eta, m) - SGN(c0) * omega_term(s0, k2eta, m) +
             (alpha / C) * (atan(C * sn / cn) - atan(C * s0 / c0));
        if (jump != 0) dF += jump * (2.0 * omega_term(1.0, k2eta, m) + (alpha / C) * ORC_PI);
        Iw[0] = Ia[0] * dn; Iw[1] = Ia[1] * sn; Iw[2] = Ia[2] * cn;
    }
    dF *= 1.0 + eta;
    double theta = (Lsq * (u - u0) + r3 * dF) / (2.0 * L * I[0] * wp);
    double ct = cos(theta), st = sin(theta);
    double z[4];
    z[0] = Iw[2] * ct + (-Iw[1]) * st;
    z[1] = Iw[1] * ct + Iw[2] * st;
    z[2] = (L - Iw[0]) * ct + 0.0 * st;
    z[3] = 0.0 * ct + (L - Iw[0]) * st;
    /* q <- q (x) conj(z0) (x) z, written as z*<z0,q> + C(z, Ct(z0, q)) (RigidBody.cpp:305) */
    double zq = dot4(z0, q), v[3], cz[4];
    qCt(z0, q, v);
    qC(z, v, cz);
    double nq2 = 0.0;
    for (int i = 0; i < 4; i++) { q[i] = z[i] * zq + cz[i]; nq2 += q[i] * q[i]; }
    double inv = 1.0 / sqrt(nq2);
    for (int i = 0; i < 4; i++) q[i] *= inv;
    double twoIw[3] = {Iw[0] * 2.0, Iw[1] * 2.0, Iw[2] * 2.0};
    qB(q, twoIw, pi);
}

/* ------------------------------------------------------------------------------------------ */
/* Symmetric 3x3 eigen-decomposition (openmmapi/src/eigenDecomposition.cpp)                    */
/* ------------------------------------------------------------------------------------------ */

static double det3(const double* a) {
    return a[0] * (a[4] * a[8] - a[7] * a[5]) - a[1] * (a[3] * a[8] - a[6] * a[5]) +
           a[2] * (a[3] * a[7] - a[6] * a[4]);
}

/* Smith's trigonometric eigenvalues, descending (eigenDecomposition.cpp:72-100). */
static void smith_eigenvalues(const double* A, double* w) {
    const double eps = DBL_EPSILON;
    double p1 = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    if (p1 < eps) {
        w[0] = A[0]; w[1] = A[4]; w[2] = A[8];
        double t;
        if (w[0] < w[1]) { t = w[0]; w[0] = w[1]; w[1] = t; }
        if (w[0] < w[2]) { t = w[0]; w[0] = w[2]; w[2] = t; }
        if (w[1] < w[2]) { t = w[1]; w[1] = w[2]; w[2] = t; }
        return;
    }
    double tr = A[0] + A[4] + A[8];
    double qm = tr / 3.0;
    double d[3] = {A[0] - qm, A[4] - qm, A[8] - qm};
    double p2 = dot3(d, d) + 2.0 * p1;
    double p = sqrt(p2 / 6.0);
    double B[9];
    memcpy(B, A, sizeof B);
    B[0] -= qm; B[4] -= qm; B[8] -= qm;
    double r = det3(B) * (3.0 / (p * p2));
    double phi = r <= -1.0 ? ORC_PI / 3.0 : (r >= 1.0 ? 0.0 : acos(r) / 3.0);
    double e0 = qm + 2.0 * p * cos(phi);
    double e2 = qm + 2.0 * p * cos(phi + 2.0 * ORC_PI / 3.0);
    w[0] = e0; w[1] = tr - (e0 + e2); w[2] = e2;
}

/* Normalise a cross-product eigenvector candidate (eigenDecomposition.cpp:37-68). */
static void kopp_finish(double* q, const double* a, double n1tmp, double n2tmp, double thresh) {
    const double eps = DBL_EPSILON;
    double norm = dot3(q, q);
    double n1 = n1tmp + a[0] * a[0], n2 = n2tmp + a[4] * a[4];
    double error = n1 * n2;
    if (n1 <= thresh) { q[0] = 1.0; q[1] = 0.0; q[2] = 0.0; }
    else if (n2 <= thresh) { q[0] = 0.0; q[1] = 1.0; q[2] = 0.0; }
    else if (norm < 4096.0 * eps * eps * error) {
        double t = fabs(a[1]), f = -a[0] / a[1];
        if (fabs(a[4]) > t) { t = fabs(a[4]); f = -a[1] / a[4]; }
        if (fabs(a[5]) > t) f = -a[2] / a[5];
        norm = 1.0 / sqrt(1.0 + f * f);
        q[0] = norm; q[1] = f * norm; q[2] = 0.0;
    } else {
        double s = sqrt(1.0 / norm);
        q[0] *= s; q[1] *= s; q[2] *= s;
    }
}

/* Kopp's cross-product eigenvectors as rows (eigenDecomposition.cpp:104-176). The fallback for
 * an entirely degenerate pair picks any unit vector orthogonal to the first eigenvector (the
 * reference's code for that branch, eigenDecomposition.cpp:162-171, indexes out of range). */
static void kopp_eigenvectors(const double* A, const double* w, double* V) {
    const double eps = DBL_EPSILON;
    double wmax8eps = 8.0 * eps * fabs(w[0]);
    double thresh = wmax8eps * wmax8eps;
    double a[9];
    memcpy(a, A, sizeof a);
    a[3] = a[1]; a[6] = a[2]; a[7] = a[5];
    double n1 = a[1] * a[1] + a[2] * a[2];
    double n2 = a[1] * a[1] + a[5] * a[5];
    double q0[3], q1[3];
    q1[0] = a[1] * a[5] - a[2] * a[4];
    q1[1] = a[2] * a[1] - a[5] * a[0];
    q1[2] = a[1] * a[1];
    a[0] -= w[0]; a[4] -= w[0];
    q0[0] = q1[0] + a[2] * w[0];
    q0[1] = q1[1] + a[5] * w[0];
    q0[2] = a[0] * a[4] - q1[2];
    kopp_finish(q0, a, n1, n2, thresh);
    double t = w[0] - w[1];
    if (fabs(t) > wmax8eps) {
        a[0] += t; a[4] += t;
        double x = q1[0] + a[2] * w[1], y = q1[1] + a[5] * w[1], z = a[0] * a[4] - q1[2];
        q1[0] = x; q1[1] = y; q1[2] = z;
        kopp_finish(q1, a, n1, n2, thresh);
    } else {
        a[0] += w[0]; a[4] += w[0];
        int ok = 0;
        for (int i = 0; i < 3 && !ok; i++) {
            a[4 * i] -= w[1];
            double ai[3] = {a[i], a[3 + i], a[6 + i]};
            double nn = dot3(ai, ai);
            ok = nn > thresh;
            if (ok) {
                cross3(q0, ai, q1);
                double norm = dot3(q1, q1);
                ok = norm > 65536.0 * eps * eps * nn;
                if (ok) { double s = sqrt(1.0 / norm); q1[0] *= s; q1[1] *= s; q1[2] *= s; }
            }
        }
        if (!ok) {
            int k = 0;
            for (int i = 1; i < 3; i++) if (fabs(q0[i]) < fabs(q0[k])) k = i;
            double e[3] = {0.0, 0.0, 0.0};
            e[k] = 1.0;
            cross3(e, q0, q1);
            double s = 1.0 / sqrt(dot3(q1, q1));
            q1[0] *= s; q1[1] *= s; q1[2] *= s;
        }
    }
    double q2[3];
    cross3(q0, q1, q2);
    memcpy(V, q0, sizeof q0); memcpy(V + 3, q1, sizeof q1); memcpy(V + 6, q2, sizeof q2);
}

/* Robust alternative: cyclic Jacobi rotations to machine precision, values sorted descending,
 * eigenvectors as rows of a proper rotation (third row = first x second). */
static void jacobi_eigen(const double* M, double* w, double* V) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) a[i][j] = 0.5 * (M[3 * i + j] + M[3 * j + i]);
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= 1e-36 * diag || off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int r = p + 1; r < 3; r++) {
                if (a[p][r] == 0.0) continue;
                double theta = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
                double t = SGN(theta) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) { /* columns p, r of a */
                    double akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 3; k++) { /* rows p, r of a */
                    double apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 3; k++) { /* eigenvector columns */
                    double vkp = v[k][p], vkr = v[k][r];
                    v[k][p] = c * vkp - s * vkr;
                    v[k][r] = s * vkp + c * vkr;
                }
            }
    }
    int idx[3] = {0, 1, 2};
    for (int i = 0; i < 3; i++)
        for (int j = i + 1; j < 3; j++)
            if (a[idx[j]][idx[j]] > a[idx[i]][idx[i]]) { int t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
    for (int i = 0; i < 3; i++) {
        w[i] = a[idx[i]][idx[i]];
        for (int k = 0; k < 3; k++) V[3 * i + k] = v[k][idx[i]];
    }
    cross3(V, V + 3, V + 6);
}

/* Canonical body frame for the robust oracle, so that equivalent frames never depend on
 * rounding: each eigenvector row gets its largest-magnitude component positive; for a top with
 * two equal moments (relative gap <= 1e-12) the two degenerate axes are fixed by the first atom
 * with a displacement off the unique axis; a spherical top takes the space frame. */
static int rot_class(const double* I) {
    if (I[2] == 0.0) return 2;
    double tol = 1e-12 * I[0];
    int g01 = I[0] - I[1] <= tol, g12 = I[1] - I[2] <= tol;
    if (g01 && g12) return 3;
    if (g01) return 2;
    if (g12) return 1;
    return 0;
}
static void canon_sign(double* v) {
    int k = 0;
    for (int i = 1; i < 3; i++) if (fabs(v[i]) > fabs(v[k])) k = i;
    if (v[k] < 0) { v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2]; }
}
static void canonical_frame(double* A, const double* I, const double* delta, const double* d2, int N) {
    int cls = rot_class(I);
    if (cls == 3) {
        memset(A, 0, 9 * sizeof(double));
        A[0] = A[4] = A[8] = 1.0;
        return;
    }
    if (cls == 0) {
        canon_sign(A); canon_sign(A + 3);
        cross3(A, A + 3, A + 6);
        return;
    }
    int k = cls == 1 ? 0 : 2; /* unique axis */
    double u[3] = {A[3 * k], A[3 * k + 1], A[3 * k + 2]}, e1[3] = {0, 0, 0}, e2[3];
    canon_sign(u);
    double d2max = 0.0;
    for (int j = 0; j < N; j++) d2max = fmax(d2max, d2[j]);
    int found = 0;
    for (int j = 0; j < N && !found; j++) {
        const double* x = delta + 3 * j;
        double ux = dot3(u, x);
        double p[3] = {x[0] - ux * u[0], x[1] - ux * u[1], x[2] - ux * u[2]};
        double pp = dot3(p, p);
        if (pp > 1e-6 * d2max) {
            double s = 1.0 / sqrt(pp);
            e1[0] = p[0] * s; e1[1] = p[1] * s; e1[2] = p[2] * s;
            found = 1;
        }
    }
    if (!found) { memcpy(e1, A + 3 * (k == 0 ? 1 : 0), sizeof e1); }
    cross3(u, e1, e2);
    if (k == 0) { memcpy(A, u, sizeof u); memcpy(A + 3, e1, sizeof e1); memcpy(A + 6, e2, sizeof e2); }
    else { memcpy(A, e1, sizeof e1); memcpy(A + 3, e2, sizeof e2); memcpy(A + 6, u, sizeof u); }
}

void orc_eigen(const double* M, double* w, double* V, int robust) {
    if (robust) { jacobi_eigen(M, w, V); return; }
    smith_eigenvalues(M, w);
    kopp_eigenvectors(M, w, V);
}

/* ------------------------------------------------------------------------------------------ */
/* System of rigid bodies and free atoms (openmmapi/src/RigidBodySystem.cpp)                   */
/* ------------------------------------------------------------------------------------------ */

struct orc_system {
    int natoms, nfree, nbodies, nbodyatoms, ndof, mode, robust;
    int* atom_index;   /* [nfree + nbodyatoms]: free atoms, then body atoms grouped by body */
    double* masses;    /* [natoms] */
    double* free_invm; /* [nfree] */
    double* saved;     /* [3*nfree] */
    int *bN, *bloc, *bdof;
    double *mass, *invm, *I, *invI, *rcm, *pcm, *q, *pi, *force, *torque, *twoKt, *twoKr;
    double* d;     /* [3*nbodyatoms] body-frame positions */
    double* delta; /* [3*nbodyatoms] space-frame displacements from the COM */
    /* refined energies: 0 off, 1 on, 2 on with the reference's free-atom weights */
    int refined;
    double *rdot, *qdot, *posdot; /* [3*nbodies], [4*nbodies], [3*nfree] stencil sums */
};

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

void orc_destroy(orc_system* s) {
    if (!s) return;
    free(s->atom_index); free(s->masses); free(s->free_invm); free(s->saved);
    free(s->bN); free(s->bloc); free(s->bdof);
    free(s->mass); free(s->invm); free(s->I); free(s->invI); free(s->rcm); free(s->pcm);
    free(s->q); free(s->pi); free(s->force); free(s->torque); free(s->twoKt); free(s->twoKr);
    free(s->d); free(s->delta);
    free(s->rdot); free(s->qdot); free(s->posdot);
    free(s);
}

/* cleanBodyIndices (RigidBodySystem.cpp:28-49) plus initialize (RigidBodySystem.cpp:55-114):
 * positive ids are compacted to 1..nbodies in ascending id order; atoms of each body keep their
 * ascending atom order; free atoms come first in atom_index. Robust mode turns ids that occur
 * once into free atoms (the reference keeps them as one-atom bodies). */
orc_system* orc_create(int natoms, const double* masses, const int* body_indices, int mode, int robust) {
    if (natoms <= 0 || mode < 0) { snprintf(g_err, sizeof g_err, "invalid natoms or mode"); return NULL; }
    int maxid = 0;
    for (int i = 0; i < natoms; i++) if (body_indices[i] > maxid) maxid = body_indices[i];
    int* count = xcalloc((size_t)maxid + 1, sizeof(int));
    for (int i = 0; i < natoms; i++) if (body_indices[i] > 0) count[body_indices[i]]++;
    int* newid = xcalloc((size_t)maxid + 1, sizeof(int));
    int nb = 0;
    for (int id = 1; id <= maxid; id++)
        if (count[id] > 0 && !(robust && count[id] == 1)) newid[id] = ++nb;
    orc_system* s = xcalloc(1, sizeof *s);
    s->natoms = natoms; s->mode = mode; s->robust = robust; s->nbodies = nb;
    s->masses = xcalloc(natoms, sizeof(double));
    memcpy(s->masses, masses, natoms * sizeof(double));
    int* bid = xcalloc(natoms, sizeof(int));
    for (int i = 0; i < natoms; i++) bid[i] = body_indices[i] > 0 ? newid[body_indices[i]] : 0;
    s->bN = xcalloc(nb, sizeof(int)); s->bloc = xcalloc(nb, sizeof(int)); s->bdof = xcalloc(nb, sizeof(int));
    int nfree = 0;
    for (int i = 0; i < natoms; i++) {
        if (masses[i] == 0.0) {
            if (bid[i] != 0) { snprintf(g_err, sizeof g_err, "massless atom %d in a rigid body", i); goto fail; }
            continue;
        }
        if (bid[i] == 0) nfree++; else s->bN[bid[i] - 1]++;
    }
    s->nfree = nfree;
    int loc = 0;
    for (int b = 0; b < nb; b++) { s->bloc[b] = loc; loc += s->bN[b]; }
    s->nbodyatoms = loc;
    s->atom_index = xcalloc((size_t)nfree + loc, sizeof(int));
    s->free_invm = xcalloc(nfree, sizeof(double));
    s->saved = xcalloc(3 * (size_t)nfree, sizeof(double));
    int* fill = xcalloc(nb, sizeof(int));
    int f = 0;
    for (int i = 0; i < natoms; i++) {
        if (masses[i] == 0.0) continue;
        if (bid[i] == 0) { s->atom_index[f] = i; s->free_invm[f] = 1.0 / masses[i]; f++; }
        else { int b = bid[i] - 1; s->atom_index[nfree + s->bloc[b] + fill[b]++] = i; }
    }
    free(fill);
#define ALLOC(field, k) s->field = xcalloc((size_t)(k) * (nb ? nb : 1), sizeof(double))
    ALLOC(mass, 1); ALLOC(invm, 1); ALLOC(I, 3); ALLOC(invI, 3); ALLOC(rcm, 3); ALLOC(pcm, 3);
    ALLOC(q, 4); ALLOC(pi, 4); ALLOC(force, 3); ALLOC(torque, 4); ALLOC(twoKt, 1); ALLOC(twoKr, 1);
#undef ALLOC
    s->d = xcalloc(3 * (size_t)loc, sizeof(double));
    s->delta = xcalloc(3 * (size_t)loc, sizeof(double));
    s->rdot = xcalloc(3 * (size_t)(nb ? nb : 1), sizeof(double));
    s->qdot = xcalloc(4 * (size_t)(nb ? nb : 1), sizeof(double));
    s->posdot = xcalloc(3 * (size_t)(nfree ? nfree : 1), sizeof(double));
    free(count); free(newid); free(bid);
    return s;
fail:
    free(count); free(newid); free(bid);
    orc_destroy(s);
    return NULL;
}

/* collinear (RigidBody.cpp:26-45). The reference keeps the last displacement longer than the
 * first one as the axis (it compares against d2[0]); robust mode takes the longest. */
static int collinear(const double* delta, const double* d2, int N, double* u, int robust) {
    const double TOL = 1.0E-5;
    int jmax = 0;
    double d2max = d2[0];
    for (int j = 1; j < N; j++)
        if (d2[j] > (robust ? d2max : d2[0])) { jmax = j; d2max = d2[j]; }
    double s = 1.0 / sqrt(d2max);
    for (int k = 0; k < 3; k++) u[k] = delta[3 * jmax + k] * s;
    int is = 1;
    for (int j = 0; is && j < N; j++) {
        double djdj = d2[j], udj = dot3(u, delta + 3 * j);
        is = is && (djdj < TOL * d2max || fabs(udj * udj / djdj - 1.0) < TOL);
    }
    return is;
}

/* orthonormal (RigidBody.cpp:51-58): project the unit axis with the smallest component of u
 * off u. The reference compares signed components (an axis along -x gives a zero vector);
 * robust mode compares magnitudes. */
static void orthonormal(const double* u, double* v, int robust) {
    double c[3] = {u[0], u[1], u[2]};
    if (robust) for (int k = 0; k < 3; k++) c[k] = fabs(c[k]);
    int imin = c[0] < c[1] ? 0 : 1;
    if (c[2] < c[imin]) imin = 2;
    double e[3] = {0.0, 0.0, 0.0};
    e[imin] = 1.0;
    double uu = dot3(u, u), ue = dot3(u, e);
    for (int k = 0; k < 3; k++) v[k] = uu * e[k] - u[k] * ue;
    double s = 1.0 / sqrt(dot3(v, v));
    for (int k = 0; k < 3; k++) v[k] *= s;
}

/* forceAndTorque (RigidBody.cpp:174-183) */
static void force_and_torque(orc_system* s, int b, const double* F) {
    double f[3] = {0, 0, 0}, tau[3] = {0, 0, 0}, c[3];
    for (int j = 0; j < s->bN[b]; j++) {
        int k = s->bloc[b] + j, i = s->atom_index[s->nfree + k];
        for (int x = 0; x < 3; x++) f[x] += F[3 * i + x];
        cross3(s->delta + 3 * k, F + 3 * i, c);
        for (int x = 0; x < 3; x++) tau[x] += c[x];
    }
    memcpy(s->force + 3 * b, f, sizeof f);
    qC(s->q + 4 * b, tau, s->torque + 4 * b);
}

/* buildGeometry (RigidBody.cpp:65-116) */
static void build_geometry(orc_system* s, int b, const double* R, const double* F) {
    int N = s->bN[b], loc = s->bloc[b];
    const int* atom = s->atom_index + s->nfree + loc;
    double mass = 0.0, rcm[3] = {0, 0, 0};
    for (int j = 0; j < N; j++) {
        int i = atom[j];
        mass += s->masses[i];
        for (int x = 0; x < 3; x++) rcm[x] += R[3 * i + x] * s->masses[i];
    }
    double im = 1.0 / mass;
    for (int x = 0; x < 3; x++) rcm[x] *= im;
    s->mass[b] = mass; s->invm[b] = 1.0 / mass;
    memcpy(s->rcm + 3 * b, rcm, sizeof rcm);
    double* delta = s->delta + 3 * loc;
    double* d2 = xcalloc(N, sizeof(double));
    for (int j = 0; j < N; j++) {
        for (int x = 0; x < 3; x++) delta[3 * j + x] = R[3 * atom[j] + x] - rcm[x];
        d2[j] = dot3(delta + 3 * j, delta + 3 * j);
    }
    double u[3], A[9], *I = s->I + 3 * b, *invI = s->invI + 3 * b;
    /* The reference tests a one-atom body for collinearity too (its cleanBodyIndices keeps an index
     * used once as a body, RigidBodySystem.cpp:37-47): the atom's displacement from its own centre
     * of mass, R - (R*m)*(1/m), is zero or a rounding residue, and in the second case the test
     * passes and the body counts 5 degrees of freedom, otherwise 6 (RigidBody.cpp:88-107). */
    if ((N > 1 || !s->robust) && collinear(delta, d2, N, u, s->robust)) {
        double moi = 0.0;
        for (int j = 0; j < N; j++) moi += s->masses[atom[j]] * d2[j];
        I[0] = moi; I[1] = moi; I[2] = 0.0;
        invI[0] = 1.0 / moi; invI[1] = 1.0 / moi; invI[2] = 0.0;
        double v[3], w[3];
        if (s->robust) canon_sign(u);
        orthonormal(u, v, s->robust);
        cross3(u, v, w);
        if (s->robust) { /* rows v, u x v, u: the molecular axis is body axis 3 */
            memcpy(A, v, sizeof v); memcpy(A + 3, w, sizeof w); memcpy(A + 6, u, sizeof u);
        } else { /* the reference transposes this matrix (RigidBody.cpp:96) */
            for (int k = 0; k < 3; k++) { A[3 * k] = v[k]; A[3 * k + 1] = w[k]; A[3 * k + 2] = u[k]; }
        }
        s->bdof[b] = 5;
    } else {
        double M[9] = {0};
        for (int j = 0; j < N; j++) {
            const double* x = delta + 3 * j;
            double m = s->masses[atom[j]], xx = dot3(x, x);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) M[3 * r + c] += ((-x[c] * x[r]) + (r == c ? xx : 0.0)) * m;
        }
        orc_eigen(M, I, A, s->robust);
        if (s->robust) canonical_frame(A, I, delta, d2, N);
        invI[0] = 1.0 / I[0]; invI[1] = 1.0 / I[1]; invI[2] = 1.0 / I[2];
        s->bdof[b] = 6;
    }
    quat_from_matrix(A, s->q + 4 * b);
    for (int j = 0; j < N; j++)
        for (int r = 0; r < 3; r++) s->d[3 * (loc + j) + r] = dot3(A + 3 * r, delta + 3 * j);
    free(d2);
    force_and_torque(s, b, F);
}

/* buildDynamics (RigidBody.cpp:123-142). The reference adds to pcm without clearing it first;
 * a fresh system starts from zero, and robust mode clears it on every call. */
static void build_dynamics(orc_system* s, int b, const double* V) {
    int N = s->bN[b], loc = s->bloc[b];
    const int* atom = s->atom_index + s->nfree + loc;
    double* pcm = s->pcm + 3 * b;
    if (s->robust) pcm[0] = pcm[1] = pcm[2] = 0.0;
    for (int j = 0; j < N; j++) {
        int i = atom[j];
        for (int x = 0; x < 3; x++) pcm[x] += V[3 * i + x] * s->masses[i];
    }
    double im = 1.0 / s->mass[b];
    double vcm[3] = {pcm[0] * im, pcm[1] * im, pcm[2] * im};
    s->twoKt[b] = dot3(pcm, vcm);
    double L[3] = {0, 0, 0}, dv[3], Adv[3], c[3];
    const double* q = s->q + 4 * b;
    for (int j = 0; j < N; j++) {
        int i = atom[j];
        for (int x = 0; x < 3; x++) dv[x] = V[3 * i + x] - vcm[x];
        double m = s->masses[i];
        qA(q, dv, Adv);
        for (int x = 0; x < 3; x++) Adv[x] *= m;
        cross3(s->d + 3 * (loc + j), Adv, c);
        for (int x = 0; x < 3; x++) L[x] += c[x];
    }
    double twoL[3] = {L[0] * 2.0, L[1] * 2.0, L[2] * 2.0};
    qB(q, twoL, s->pi + 4 * b);
    const double* invI = s->invI + 3 * b;
    double w[3] = {invI[0] * L[0], invI[1] * L[1], invI[2] * L[2]};
    s->twoKr[b] = dot3(L, w);
}

int orc_setup(orc_system* s, const double* R, const double* V, const double* F) {
    /* RigidBodySystem.cpp:130 counts one degree of freedom per free atom (defect D8); the robust
     * oracle counts three */
    s->ndof = s->robust ? 3 * s->nfree : s->nfree;
    for (int b = 0; b < s->nbodies; b++) {
        build_geometry(s, b, R, F);
        s->ndof += s->bdof[b];
    }
    for (int b = 0; b < s->nbodies; b++) build_dynamics(s, b, V);
    return 0;
}

/* updateAtomicPositions (RigidBody.cpp:148-153) */
static void update_positions(orc_system* s, int b, double* R) {
    const double* q = s->q + 4 * b;
    for (int j = 0; j < s->bN[b]; j++) {
        int k = s->bloc[b] + j, i = s->atom_index[s->nfree + k];
        double* dl = s->delta + 3 * k;
        qAt(q, s->d + 3 * k, dl);
        for (int x = 0; x < 3; x++) R[3 * i + x] = s->rcm[3 * b + x] + dl[x];
    }
}

/* updateAtomicVelocities (RigidBody.cpp:159-168) */
static void update_velocities(orc_system* s, int b, double* V) {
    const double* q = s->q + 4 * b;
    const double* invI = s->invI + 3 * b;
    double L[3], w[3], ws[3], c[3];
    qBt(q, s->pi + 4 * b, L);
    for (int x = 0; x < 3; x++) { L[x] *= 0.5; w[x] = invI[x] * L[x]; }
    qAt(q, w, ws);
    double vcm[3];
    for (int x = 0; x < 3; x++) vcm[x] = s->pcm[3 * b + x] * s->invm[b];
    for (int j = 0; j < s->bN[b]; j++) {
        int k = s->bloc[b] + j, i = s->atom_index[s->nfree + k];
        cross3(ws, s->delta + 3 * k, c);
        for (int x = 0; x < 3; x++) V[3 * i + x] = vcm[x] + c[x];
    }
    s->twoKt[b] = dot3(s->pcm + 3 * b, vcm);
    s->twoKr[b] = dot3(L, w);
}

/* Rotation of body b by `dt` from its current q with momentum pi + torque * kick, on copies: the
 * virtualRotation of platforms/cuda/src/kernels/rigidbodyintegrator.cu:238-243. */
static void virtual_rotation(const orc_system* s, int b, double kick, double dt, double* qv) {
    double pv[4];
    for (int x = 0; x < 4; x++) { qv[x] = s->q[4 * b + x]; pv[x] = s->pi[4 * b + x] + s->torque[4 * b + x] * kick; }
    if (s->mode == 0) orc_exact_rotation(s->I + 3 * b, s->invI + 3 * b, qv, pv, dt, s->robust);
    else orc_nosquish_rotation(s->invI + 3 * b, s->bdof[b], qv, pv, dt, s->mode);
}

static void part1_range(orc_system* s, double dt, const double* F, double* V, double* R, int f0, int f1, int b0,
                        int b1) {
    double halfDt = 0.5 * dt;
    if (s->refined) {
        /* Start of the refined-energy stencils at time t, before the kicks. Free atoms: freeAtomsDelta
         * with -dt and freeAtomsDot with factor -1 (CudaRigidBodyKernels.cpp:406-415,
         * rigidbodyintegrator.cu:285-292): the reference stores -(-dt)(v - F/m dt/2) = +dt v(t-dt/2);
         * the stencil that matches the bodies' one (and gives KE for uniform motion) needs -dt v(t-dt/2)
         * (refined == 1). Bodies: rigidbodyintegrator.cu:318-321. */
        const double sgn = s->refined == 2 ? 1.0 : -1.0;
        for (int a = f0; a < f1; a++) {
            int i = s->atom_index[a];
            for (int x = 0; x < 3; x++)
                s->posdot[3 * a + x] = sgn * dt * (V[3 * i + x] - F[3 * i + x] * s->free_invm[a] * halfDt);
        }
        for (int b = b0; b < b1; b++) {
            double qv[4];
            for (int x = 0; x < 3; x++) {
                double v = s->pcm[3 * b + x] * s->invm[b], dv = s->force[3 * b + x] * s->invm[b] * halfDt;
                s->rdot[3 * b + x] = s->rcm[3 * b + x] * 2.5 + (v - dv) * halfDt;
            }
            virtual_rotation(s, b, -dt, -dt, qv);
            for (int x = 0; x < 4; x++) s->qdot[4 * b + x] = qv[x] * 0.5 - s->q[4 * b + x] * 3.0;
        }
    }
    for (int a = f0; a < f1; a++) {
        int i = s->atom_index[a];
        if (s->refined)
            for (int x = 0; x < 3; x++)
                s->posdot[3 * a + x] += 5.0 * dt * (V[3 * i + x] + F[3 * i + x] * s->free_invm[a] * halfDt);
        for (int x = 0; x < 3; x++) {
            V[3 * i + x] += F[3 * i + x] * s->free_invm[a] * halfDt;
            R[3 * i + x] += V[3 * i + x] * dt;
            s->saved[3 * a + x] = R[3 * i + x];
        }
    }
    for (int b = b0; b < b1; b++) {
        double* pcm = s->pcm + 3 * b;
        double* rcm = s->rcm + 3 * b;
        for (int x = 0; x < 3; x++) pcm[x] += s->force[3 * b + x] * halfDt;
        for (int x = 0; x < 4; x++) s->pi[4 * b + x] += s->torque[4 * b + x] * dt;
        double idt = s->invm[b] * dt;
        for (int x = 0; x < 3; x++) rcm[x] += pcm[x] * idt;
        if (s->mode == 0)
            orc_exact_rotation(s->I + 3 * b, s->invI + 3 * b, s->q + 4 * b, s->pi + 4 * b, dt, s->robust);
        else
            orc_nosquish_rotation(s->invI + 3 * b, s->bdof[b], s->q + 4 * b, s->pi + 4 * b, dt, s->mode);
        update_positions(s, b, R);
    }
}

static void part2_range(orc_system* s, double dt, const double* R, const double* F, double* V, int f0, int f1,
                        int b0, int b1) {
    double halfDt = 0.5 * dt, invDt = 1.0 / dt;
    for (int a = f0; a < f1; a++) {
        int i = s->atom_index[a];
        for (int x = 0; x < 3; x++)
            V[3 * i + x] += F[3 * i + x] * s->free_invm[a] * halfDt + (R[3 * i + x] - s->saved[3 * a + x]) * invDt;
    }
    for (int b = b0; b < b1; b++) {
        force_and_torque(s, b, F);
        for (int x = 0; x < 3; x++) s->pcm[3 * b + x] += s->force[3 * b + x] * halfDt;
        for (int x = 0; x < 4; x++) s->pi[4 * b + x] += s->torque[4 * b + x] * dt;
        update_velocities(s, b, V);
    }
    if (!s->refined) return;
    /* End of the stencils at time t+dt, after the kicks. Free atoms: freeAtomsDot with factor 5 on
     * the part1 displacement (added in part1 above) and with factor 2 on dt v(t+3dt/2)
     * (CudaRigidBodyKernels.cpp:428-438). Bodies: rigidbodyintegrator.cu:380-384. */
    for (int a = f0; a < f1; a++) {
        int i = s->atom_index[a];
        for (int x = 0; x < 3; x++)
            s->posdot[3 * a + x] += 2.0 * dt * (V[3 * i + x] + F[3 * i + x] * s->free_invm[a] * halfDt);
    }
    for (int b = b0; b < b1; b++) {
        double qv[4], qq = 0.0;
        for (int x = 0; x < 3; x++) {
            double v = s->pcm[3 * b + x] * s->invm[b], dv = s->force[3 * b + x] * s->invm[b] * halfDt;
            s->rdot[3 * b + x] = s->rcm[3 * b + x] * 2.5 + (v + dv) * dt - s->rdot[3 * b + x];
        }
        virtual_rotation(s, b, dt, dt, qv);
        for (int x = 0; x < 4; x++) s->qdot[4 * b + x] += s->q[4 * b + x] * 1.5 + qv[x];
        for (int x = 0; x < 4; x++) qq += s->qdot[4 * b + x] * s->q[4 * b + x];
        for (int x = 0; x < 4; x++) s->qdot[4 * b + x] -= s->q[4 * b + x] * qq;
    }
}

/* integratePart1 (RigidBodySystem.cpp:170-187) */
void orc_part1(orc_system* s, double dt, const double* F, double* V, double* R) {
    part1_range(s, dt, F, V, R, 0, s->nfree, 0, s->nbodies);
}

/* integratePart2 (RigidBodySystem.cpp:193-204) */
void orc_part2(orc_system* s, double dt, const double* R, const double* F, double* V) {
    part2_range(s, dt, R, F, V, 0, s->nfree, 0, s->nbodies);
}

/* computeKineticEnergies (RigidBodySystem.cpp:210-220) */
void orc_kinetic(orc_system* s, const double* V, double* out) {
    double kt = 0.0, kr = 0.0;
    for (int a = 0; a < s->nfree; a++) {
        int i = s->atom_index[a];
        kt += dot3(V + 3 * i, V + 3 * i) / s->free_invm[a];
    }
    for (int b = 0; b < s->nbodies; b++) { kt += s->twoKt[b]; kr += s->twoKr[b]; }
    out[0] = 0.5 * kt;
    out[1] = 0.5 * kr;
}

void orc_set_refined(orc_system* s, int mode) { s->refined = mode; }

/* Refined kinetic energies and potential-energy refinement after a part2 (the refinedKineticEnergies
 * and potentialEnergyRefinement kernels, rigidbodyintegrator.cu:433-469, summed and scaled as in
 * CudaRigidBodyKernels.cpp:118-194 and :481-494): out = [KE_t, KE_r, U_refinement]. F is the force
 * array of the last part2. */
void orc_refined(orc_system* s, const double* V, const double* F, double dt, double* out) {
    double kt = 0.0, kr = 0.0, u = 0.0;
    for (int a = 0; a < s->nfree; a++) {
        int i = s->atom_index[a];
        kt += dot3(s->posdot + 3 * a, V + 3 * i) * (0.5 / s->free_invm[a]);
        u += dot3(F + 3 * i, F + 3 * i) * s->free_invm[a];
    }
    for (int b = 0; b < s->nbodies; b++) {
        double v[3], tb[3];
        for (int x = 0; x < 3; x++) v[x] = s->pcm[3 * b + x] * s->invm[b];
        kt += dot3(s->rdot + 3 * b, v) / s->invm[b];
        kr += dot4(s->qdot + 4 * b, s->pi + 4 * b);
        qBt(s->q + 4 * b, s->torque + 4 * b, tb);
        u += dot3(s->force + 3 * b, s->force + 3 * b) * s->invm[b];
        for (int x = 0; x < 3; x++) u += tb[x] * s->invI[3 * b + x] * tb[x];
    }
    double factor = 1.0 / (6.0 * dt);
    out[0] = kt * factor;
    out[1] = kr * factor;
    out[2] = -u * dt * dt / 24.0;
}

int orc_num_dof(const orc_system* s) { return s->ndof; }
int orc_num_bodies(const orc_system* s) { return s->nbodies; }
int orc_num_free(const orc_system* s) { return s->nfree; }
int orc_num_body_atoms(const orc_system* s) { return s->nbodyatoms; }
int orc_atom_index(const orc_system* s, int i) { return s->atom_index[i]; }

void orc_get_body(const orc_system* s, int b, double* out) {
    int k = 0;
    out[k++] = s->bN[b]; out[k++] = s->bdof[b]; out[k++] = s->bloc[b]; out[k++] = s->mass[b];
    for (int j = 0; j < 3; j++) out[k++] = s->I[3 * b + j];
    for (int j = 0; j < 3; j++) out[k++] = s->invI[3 * b + j];
    for (int j = 0; j < 3; j++) out[k++] = s->rcm[3 * b + j];
    for (int j = 0; j < 3; j++) out[k++] = s->pcm[3 * b + j];
    for (int j = 0; j < 4; j++) out[k++] = s->q[4 * b + j];
    for (int j = 0; j < 4; j++) out[k++] = s->pi[4 * b + j];
    for (int j = 0; j < 3; j++) out[k++] = s->force[3 * b + j];
    for (int j = 0; j < 4; j++) out[k++] = s->torque[4 * b + j];
    out[k++] = s->twoKt[b];
    out[k++] = s->twoKr[b];
}

void orc_get_body_fixed(const orc_system* s, double* out) {
    memcpy(out, s->d, 3 * (size_t)s->nbodyatoms * sizeof(double));
}

void orc_set_body_state(orc_system* s, int b, const double* rcm, const double* pcm, const double* q,
                        const double* pi) {
    memcpy(s->rcm + 3 * b, rcm, 3 * sizeof(double));
    memcpy(s->pcm + 3 * b, pcm, 3 * sizeof(double));
    memcpy(s->q + 4 * b, q, 4 * sizeof(double));
    memcpy(s->pi + 4 * b, pi, 4 * sizeof(double));
}

void orc_set_body_geometry(orc_system* s, int b, const double* I, const double* d) {
    for (int k = 0; k < 3; k++) {
        s->I[3 * b + k] = I[k];
        s->invI[3 * b + k] = I[k] == 0.0 ? 0.0 : 1.0 / I[k];
    }
    s->bdof[b] = I[2] == 0.0 ? 5 : 6;
    memcpy(s->d + 3 * s->bloc[b], d, 3 * (size_t)s->bN[b] * sizeof(double));
}

/* ------------------------------------------------------------------------------------------ */
/* Threaded fixed-force driver (CPU baseline timing)                                           */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    orc_system* s;
    double dt;
    const double* F;
    double *V, *R;
    int nsteps, f0, f1, b0, b1;
    pthread_barrier_t* bar;
} orc_job;

static void* orc_worker(void* arg) {
    orc_job* j = arg;
    for (int n = 0; n < j->nsteps; n++) {
        part1_range(j->s, j->dt, j->F, j->V, j->R, j->f0, j->f1, j->b0, j->b1);
        pthread_barrier_wait(j->bar);
        part2_range(j->s, j->dt, j->R, j->F, j->V, j->f0, j->f1, j->b0, j->b1);
        pthread_barrier_wait(j->bar);
    }
    return NULL;
}

double orc_run_fixed_force(orc_system* s, double dt, const double* F, double* V, double* R, int nsteps,
                           int nthreads) {
    if (nthreads < 1) nthreads = 1;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (nthreads == 1) {
        for (int n = 0; n < nsteps; n++) { orc_part1(s, dt, F, V, R); orc_part2(s, dt, R, F, V); }
    } else {
        pthread_t* th = xcalloc(nthreads, sizeof(pthread_t));
        orc_job* jobs = xcalloc(nthreads, sizeof(orc_job));
        pthread_barrier_t bar;
        pthread_barrier_init(&bar, NULL, (unsigned)nthreads);
        for (int t = 0; t < nthreads; t++) {
            orc_job* j = &jobs[t];
            j->s = s; j->dt = dt; j->F = F; j->V = V; j->R = R; j->nsteps = nsteps; j->bar = &bar;
            j->f0 = (int)((long)s->nfree * t / nthreads); j->f1 = (int)((long)s->nfree * (t + 1) / nthreads);
            j->b0 = (int)((long)s->nbodies * t / nthreads); j->b1 = (int)((long)s->nbodies * (t + 1) / nthreads);
            pthread_create(&th[t], NULL, orc_worker, j);
        }
        for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
        pthread_barrier_destroy(&bar);
        free(th); free(jobs);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
