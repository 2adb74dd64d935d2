// carlson.cuh -- Carlson's symmetric elliptic integrals R_F, R_C, R_D, R_J in
// FP64 for host and device (the batch role of geokerr_port/cuda/
// carlson_elliptic.cu:77-382 and of the rf/rc/rd/rj routines of
// geokerr_original.f:3444-3762).
//
// Method: B. C. Carlson, "Numerical computation of real or complex elliptic
// integrals", Numerical Algorithms 10 (1995) 13-26.  Each routine applies the
// duplication theorem until the arguments agree to the tolerance r, then
// sums the fifth-order Taylor series in the elementary symmetric functions
// of the scaled deviations (eqs. 2.2, 2.13, 2.28-2.29 and 2.17-2.19 there).
// With r = 1e-16 the truncation error is below FP64 rounding.  R_C with y < 0
// and R_J with p < 0 return Cauchy principal values (eq. 2.14, and the
// transformation of R_J to a positive fourth argument, DLMF 19.20.14).  Invalid arguments give NaN.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define NP_CARLSON_HD __host__ __device__ __forceinline__
#else
#define NP_CARLSON_HD inline
#endif

namespace np {
namespace carlson {

constexpr double kTol = 1e-16;
// (3 kTol)^(-1/6), (3 kTol)^(-1/8) and (kTol / 4)^(-1/6), correctly rounded: literal so
// that the host and device builds stop their duplication loops at the same step
constexpr double kQ_rf = 386.49729393434575, kQ_rc = 87.16855428717356, kQ_rdj = 584.803547642573;
constexpr int kMaxIter = 64;    // each duplication shrinks the deviations by 4

NP_CARLSON_HD double nan_() { return std::nan(""); }

// R_F(x, y, z) = 1/2 int_0^inf dt / sqrt((t+x)(t+y)(t+z)); x, y, z >= 0, at most one zero.
NP_CARLSON_HD double rf(double x, double y, double z) {
    if (!(x >= 0.0 && y >= 0.0 && z >= 0.0) || (x + y == 0.0) || (x + z == 0.0) || (y + z == 0.0)) return nan_();
    const double A0 = (x + y + z) / 3.0;
    double A = A0;
    double Q = kQ_rf * std::fmax(std::fabs(A0 - x), std::fmax(std::fabs(A0 - y), std::fabs(A0 - z)));
    double f = 1.0;     // 4^-m
    for (int m = 0; m < kMaxIter && Q * f >= std::fabs(A); ++m) {
        const double sx = std::sqrt(x), sy = std::sqrt(y), sz = std::sqrt(z);
        const double lam = sx * sy + sx * sz + sy * sz;
        x = 0.25 * (x + lam); y = 0.25 * (y + lam); z = 0.25 * (z + lam);
        A = 0.25 * (A + lam);
        f *= 0.25;
    }
    // scaled deviations X = (A0 - x0) 4^-m / A = (A - x) / A: duplication
    // scales every difference of the arguments by exactly 1/4
    const double Xs = (A - x) / A, Ys = (A - y) / A, Zs = -(Xs + Ys);
    const double E2 = Xs * Ys - Zs * Zs, E3 = Xs * Ys * Zs;
    return (1.0 - E2 / 10.0 + E3 / 14.0 + E2 * E2 / 24.0 - 3.0 * E2 * E3 / 44.0) / std::sqrt(A);
}

// R_C(x, y) = R_F(x, y, y); x >= 0, y != 0; principal value for y < 0.
NP_CARLSON_HD double rc(double x, double y) {
    if (!(x >= 0.0) || y == 0.0 || std::isnan(y)) return nan_();
    double w = 1.0;
    if (y < 0.0) {
        w = std::sqrt(x / (x - y));
        x = x - y;
        y = -y;
    }
    const double A0 = (x + 2.0 * y) / 3.0;
    double A = A0;
    double Q = kQ_rc * std::fabs(A0 - x);
    double f = 1.0;
    for (int m = 0; m < kMaxIter && Q * f >= std::fabs(A); ++m) {
        const double lam = 2.0 * std::sqrt(x) * std::sqrt(y) + y;
        x = 0.25 * (x + lam); y = 0.25 * (y + lam);
        A = 0.25 * (A + lam);
        f *= 0.25;
    }
    const double s = (y - A) / A;      // = (y0 - A0) 4^-m / A
    const double s2 = s * s;
    const double poly = 1.0 + s2 * (3.0 / 10.0 + s * (1.0 / 7.0 + s * (3.0 / 8.0 + s * (9.0 / 22.0 + s * (159.0 / 208.0 + s * (9.0 / 8.0))))));
    return w * poly / std::sqrt(A);
}

// Fifth-order series shared by R_D and R_J (Carlson 1995 eq. 2.19).
NP_CARLSON_HD double rdj_series(double E2, double E3, double E4, double E5) {
    return 1.0 - 3.0 * E2 / 14.0 + E3 / 6.0 + 9.0 * E2 * E2 / 88.0 - 3.0 * E4 / 22.0 - 9.0 * E2 * E3 / 52.0 + 3.0 * E5 / 26.0;
}

// R_D(x, y, z) = R_J(x, y, z, z); x, y >= 0 (not both zero), z > 0.
NP_CARLSON_HD double rd(double x, double y, double z) {
    if (!(x >= 0.0 && y >= 0.0 && z > 0.0) || (x + y == 0.0)) return nan_();
    const double A0 = (x + y + 3.0 * z) / 5.0;
    double A = A0;
    double Q = kQ_rdj *
               std::fmax(std::fabs(A0 - x), std::fmax(std::fabs(A0 - y), std::fabs(A0 - z)));
    double f = 1.0, sum = 0.0;
    for (int m = 0; m < kMaxIter && Q * f >= std::fabs(A); ++m) {
        const double sx = std::sqrt(x), sy = std::sqrt(y), sz = std::sqrt(z);
        const double lam = sx * sy + sx * sz + sy * sz;
        sum += f / (sz * (z + lam));
        x = 0.25 * (x + lam); y = 0.25 * (y + lam); z = 0.25 * (z + lam);
        A = 0.25 * (A + lam);
        f *= 0.25;
    }
    const double X = (A - x) / A, Y = (A - y) / A, Z = -(X + Y) / 3.0;
    const double XY = X * Y, Z2 = Z * Z;
    const double E2 = XY - 6.0 * Z2, E3 = (3.0 * XY - 8.0 * Z2) * Z, E4 = 3.0 * (XY - Z2) * Z2, E5 = XY * Z2 * Z;
    return f * rdj_series(E2, E3, E4, E5) / (A * std::sqrt(A)) + 3.0 * sum;
}

// R_J(x, y, z, p) = 3/2 int_0^inf dt / ((t+p) sqrt((t+x)(t+y)(t+z))); x, y, z >= 0 (at most one
// zero), p != 0; principal value for p < 0.
NP_CARLSON_HD double rj_pos(double x, double y, double z, double p) {
    const double A0 = (x + y + z + 2.0 * p) / 5.0;
    double A = A0;
    const double delta = (p - x) * (p - y) * (p - z);
    double Q = kQ_rdj *
               std::fmax(std::fmax(std::fabs(A0 - x), std::fabs(A0 - y)), std::fmax(std::fabs(A0 - z), std::fabs(A0 - p)));
    double f = 1.0, f3 = 1.0, sum = 0.0;
    for (int m = 0; m < kMaxIter && Q * f >= std::fabs(A); ++m) {
        const double sx = std::sqrt(x), sy = std::sqrt(y), sz = std::sqrt(z), sp = std::sqrt(p);
        const double lam = sx * sy + sx * sz + sy * sz;
        const double d = (sp + sx) * (sp + sy) * (sp + sz);
        const double e = f3 * delta / (d * d);
        sum += f * rc(1.0, 1.0 + e) / d;
        x = 0.25 * (x + lam); y = 0.25 * (y + lam); z = 0.25 * (z + lam); p = 0.25 * (p + lam);
        A = 0.25 * (A + lam);
        f *= 0.25;
        f3 *= 1.0 / 64.0;
    }
    const double X = (A - x) / A, Y = (A - y) / A, Z = (A - z) / A, P = -(X + Y + Z) / 2.0;
    const double P2 = P * P;
    const double E2 = X * Y + X * Z + Y * Z - 3.0 * P2;
    const double E3 = X * Y * Z + 2.0 * E2 * P + 4.0 * P2 * P;
    const double E4 = (2.0 * X * Y * Z + E2 * P + 3.0 * P2 * P) * P;
    const double E5 = X * Y * Z * P2;
    return f * rdj_series(E2, E3, E4, E5) / (A * std::sqrt(A)) + 6.0 * sum;
}

NP_CARLSON_HD double rj(double x, double y, double z, double p) {
    if (!(x >= 0.0 && y >= 0.0 && z >= 0.0) || p == 0.0 || std::isnan(p) || (x + y == 0.0) || (x + z == 0.0) ||
        (y + z == 0.0))
        return nan_();
    if (p > 0.0) return rj_pos(x, y, z, p);
    // p < 0: order x <= y <= z and use the principal-value identity
    // (y - p) R_J(x,y,z,p) = (q - y) R_J(x,y,z,q) - 3 R_F(x,y,z) + 3 sqrt(xyz/(xz - pq)) R_C(xz - pq, -pq)
    // with q = y + (z - y)(y - x)/(y - p) > 0 (so -pq > 0).
    double a = x, b = y, c = z, t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    const double q = b + (c - b) * (b - a) / (b - p);
    const double xz = a * c;
    const double w = xz - p * q;
    const double r = (q - b) * rj_pos(a, b, c, q) - 3.0 * rf(a, b, c) + 3.0 * std::sqrt(a * b * c / w) * rc(w, -p * q);
    return r / (b - p);
}

}  // namespace carlson
}  // namespace np
