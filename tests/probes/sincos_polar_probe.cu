// Host probe of sincos_polar (nullpath_gb300/csrc/tracer_mixed.cuh): the
// largest error, in ulps of the float nearest the true value, of sin and
// cos over every 7th float of [1e-7, pi) plus every float within 1e-4 of
// pi/4 and 3pi/4, within 1e-3 of pi/2, below 1e-3 and above 3.14, measured
// against libm's double sin/cos of the same float argument.
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "tracer_mixed.cuh"

static double ulp_of(double v) {
    float a = std::fabs((float)v);
    return (double)std::nextafter(a, INFINITY) - (double)a;
}

int main() {
    double es = 0.0, ec = 0.0;
    uint64_t n = 0, k = 0;
    for (float th = 1e-7f; th < 3.14159265f; th = std::nextafter(th, 4.0f), ++k) {
        bool dense = std::fabs(th - 0.785398163f) < 1e-4f || std::fabs(th - 2.35619449f) < 1e-4f ||
                     std::fabs(th - 1.57079633f) < 1e-3f || th < 1e-3f || th > 3.14f;
        if (!dense && k % 7) continue;
        float s, c;
        np::sincos_polar(th, s, c);
        double S = std::sin((double)th), C = std::cos((double)th);
        es = std::fmax(es, std::fabs(s - S) / ulp_of(S));
        ec = std::fmax(ec, std::fabs(c - C) / ulp_of(C));
        ++n;
    }
    std::printf("%llu %.4f %.4f\n", (unsigned long long)n, es, ec);
    return 0;
}
