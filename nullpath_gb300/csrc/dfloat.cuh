// dfloat.cuh -- double-float arithmetic on the FP32 pipes.
//
// A DF is an unevaluated sum hi + lo of two FP32 values with |lo| <= ulp(hi)/2:
// a 48-bit significand (relative rounding about 2^-48 = 3.6e-15 per operation)
// with the exponent range of FP32.  GB300 issues FP64 at 1/64 of the FP32
// rate, while a DF addition costs 20 FP32 operations and a multiplication 8,
// so arithmetic that needs far more than FP32's 24 bits but not FP64's 53 runs
// several times faster as DF than as FP64.
//
// Algorithms (all with round-to-nearest FP32 operations):
//   two_sum, fast_two_sum   Knuth (TAOCP vol. 2) and Dekker (Numer. Math. 18,
//                           1971) error-free additions;
//   two_prod                error-free product from one FMA;
//   add                     "AccurateDWPlusDW", mul "DWTimesDW3" and div
//                           "DWDivDW2" of Joldes, Muller & Popescu, ACM TOMS
//                           44 (2017): relative errors <= 3u^2, 5u^2 and 15u^2
//                           (u = 2^-24) respectively.
// sin/cos: reduction by multiples of pi/2 with a three-part constant, then
// the Taylor series of sin through z^19 and of cos through z^20 on |z| <=
// pi/4 (truncation < 2e-19).
//
// Every function is __host__ __device__ so the arithmetic can be checked on
// the CPU; host builds must not contract a*b+c (-ffp-contract=off), as the
// device intrinsics below never do.
#pragma once

#include <cmath>

namespace np {

#ifdef __CUDA_ARCH__
#define NP_DF_ADD(a, b) __fadd_rn((a), (b))
#define NP_DF_SUB(a, b) __fsub_rn((a), (b))
#define NP_DF_MUL(a, b) __fmul_rn((a), (b))
#define NP_DF_DIV(a, b) __fdiv_rn((a), (b))
#define NP_DF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define NP_DF_ADD(a, b) ((a) + (b))
#define NP_DF_SUB(a, b) ((a) - (b))
#define NP_DF_MUL(a, b) ((a) * (b))
#define NP_DF_DIV(a, b) ((a) / (b))
#define NP_DF_FMA(a, b, c) std::fmaf((a), (b), (c))
#endif

struct DF {
    float hi, lo;
    DF() = default;
    __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
    // From a double constant (folded at compile time for literal arguments).
    __host__ __device__ constexpr DF(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    __host__ __device__ constexpr DF(int x) : hi((float)x), lo(0.0f) {}
};

__host__ __device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = NP_DF_ADD(a, b);
    const float bb = NP_DF_SUB(s, a);
    const float e = NP_DF_ADD(NP_DF_SUB(a, NP_DF_SUB(s, bb)), NP_DF_SUB(b, bb));
    return DF(s, e);
}
// |a| >= |b| (or a = 0)
__host__ __device__ __forceinline__ DF fast_two_sum(float a, float b) {
    const float s = NP_DF_ADD(a, b);
    return DF(s, NP_DF_SUB(b, NP_DF_SUB(s, a)));
}
__host__ __device__ __forceinline__ DF two_prod(float a, float b) {
    const float p = NP_DF_MUL(a, b);
    return DF(p, NP_DF_FMA(a, b, -p));
}

__host__ __device__ __forceinline__ DF operator+(DF x, DF y) {
    const DF s = two_sum(x.hi, y.hi);
    const DF t = two_sum(x.lo, y.lo);
    const float c = NP_DF_ADD(s.lo, t.hi);
    const DF v = fast_two_sum(s.hi, c);
    const float w = NP_DF_ADD(t.lo, v.lo);
    return fast_two_sum(v.hi, w);
}
__host__ __device__ __forceinline__ DF operator-(DF x) { return DF(-x.hi, -x.lo); }
__host__ __device__ __forceinline__ DF operator-(DF x, DF y) { return x + (-y); }
__host__ __device__ __forceinline__ DF operator*(DF x, DF y) {
    const DF c = two_prod(x.hi, y.hi);
    const float tl0 = NP_DF_MUL(x.lo, y.lo);
    const float tl1 = NP_DF_FMA(x.hi, y.lo, tl0);
    const float cl2 = NP_DF_FMA(x.lo, y.hi, tl1);
    const float cl3 = NP_DF_ADD(c.lo, cl2);
    return fast_two_sum(c.hi, cl3);
}
__host__ __device__ __forceinline__ DF operator*(DF x, float y) {
    const DF c = two_prod(x.hi, y);
    const float cl3 = NP_DF_FMA(x.lo, y, c.lo);
    return fast_two_sum(c.hi, cl3);
}
__host__ __device__ __forceinline__ DF operator*(float y, DF x) { return x * y; }
__host__ __device__ __forceinline__ DF operator/(DF x, DF y) {
    const float th = NP_DF_DIV(x.hi, y.hi);
    const DF r = x - y * th;              // remainder to DF precision
    const float tl = NP_DF_DIV(r.hi, y.hi);
    return fast_two_sum(th, tl);
}
__host__ __device__ __forceinline__ DF& operator+=(DF& x, DF y) { x = x + y; return x; }
__host__ __device__ __forceinline__ DF& operator-=(DF& x, DF y) { x = x - y; return x; }
__host__ __device__ __forceinline__ DF& operator*=(DF& x, DF y) { x = x * y; return x; }

__host__ __device__ __forceinline__ bool operator>(DF x, DF y) { return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo); }
__host__ __device__ __forceinline__ bool operator<(DF x, DF y) { return y > x; }
__host__ __device__ __forceinline__ bool operator<=(DF x, DF y) { return !(x > y); }
__host__ __device__ __forceinline__ bool operator>=(DF x, DF y) { return !(y > x); }

__host__ __device__ __forceinline__ DF fabs(DF x) { return (x.hi < 0.0f) ? -x : x; }
__host__ __device__ __forceinline__ DF fmax(DF x, DF y) { return (y > x) ? y : x; }
__host__ __device__ __forceinline__ bool isfinite(DF x) {
#ifdef __CUDA_ARCH__
    return ::isfinite(x.hi) && ::isfinite(x.lo);
#else
    return std::isfinite(x.hi) && std::isfinite(x.lo);
#endif
}
__host__ __device__ __forceinline__ double df_to_double(DF x) { return (double)x.hi + (double)x.lo; }
__host__ __device__ __forceinline__ float df_to_float(DF x) { return NP_DF_ADD(x.hi, x.lo); }

// sin and cos of a DF angle.  theta - k pi/2 with k = nearest integer to
// theta / (pi/2) (|k| <= 4 here), pi/2 in three FP32 parts so that k * part
// is exact for the first two; then the Taylor series on |z| <= pi/4.
__host__ __device__ __forceinline__ void df_sincos(DF th, DF& sn, DF& cs) {
    const float P1 = 1.57079637050628662109375f;        // fl(pi/2)
    const float P2 = -4.37113882867379e-08f;            // fl(pi/2 - P1)
    const float P3 = -1.71512451e-15f;                  // pi/2 - P1 - P2, rounded
    const float kf = rintf(NP_DF_MUL(th.hi, 0.636619772367581343f));
    const int k = (int)kf;
    DF z = two_sum(th.hi, NP_DF_MUL(-kf, P1));
    z = z + DF(th.lo, 0.0f);
    z = z + two_prod(-kf, P2);
    z = z + DF(NP_DF_MUL(-kf, P3), 0.0f);
    const DF z2 = z * z;
    // sin z = z (1 - z^2/3! + z^4/5! - ...), cos z = 1 - z^2/2! + ...
    DF ps = DF(-1.0 / 121645100408832000.0);            // -1/19!
    ps = ps * z2 + DF(1.0 / 355687428096000.0);         //  1/17!
    ps = ps * z2 + DF(-1.0 / 1307674368000.0);          // -1/15!
    ps = ps * z2 + DF(1.0 / 6227020800.0);              //  1/13!
    ps = ps * z2 + DF(-1.0 / 39916800.0);               // -1/11!
    ps = ps * z2 + DF(1.0 / 362880.0);                  //  1/9!
    ps = ps * z2 + DF(-1.0 / 5040.0);
    ps = ps * z2 + DF(1.0 / 120.0);
    ps = ps * z2 + DF(-1.0 / 6.0);
    ps = ps * z2 + DF(1.0f, 0.0f);
    const DF s = ps * z;
    DF pc = DF(1.0 / 2432902008176640000.0);            //  1/20!
    pc = pc * z2 + DF(-1.0 / 6402373705728000.0);       // -1/18!
    pc = pc * z2 + DF(1.0 / 20922789888000.0);          //  1/16!
    pc = pc * z2 + DF(-1.0 / 87178291200.0);            // -1/14!
    pc = pc * z2 + DF(1.0 / 479001600.0);               //  1/12!
    pc = pc * z2 + DF(-1.0 / 3628800.0);                // -1/10!
    pc = pc * z2 + DF(1.0 / 40320.0);
    pc = pc * z2 + DF(-1.0 / 720.0);
    pc = pc * z2 + DF(1.0 / 24.0);
    pc = pc * z2 + DF(-0.5);
    pc = pc * z2 + DF(1.0f, 0.0f);
    const DF c = pc;
    switch (k & 3) {
        case 0: sn = s; cs = c; break;
        case 1: sn = c; cs = -s; break;
        case 2: sn = -s; cs = -c; break;
        default: sn = -c; cs = s; break;
    }
}

}  // namespace np
