// Host probe of the double-float arithmetic (nullpath_gb300/csrc/dfloat.cuh):
// reads "op a.hi a.lo b.hi b.lo" lines (op one of + - * / s, floats as %a
// hex) and prints the result pair (for s: sin and cos of a) in %a hex.
#include <cstdio>
#include <cstring>

#include "dfloat.cuh"

int main() {
    char op[4];
    float ah, al, bh, bl;
    while (std::scanf("%3s %a %a %a %a", op, &ah, &al, &bh, &bl) == 5) {
        const np::DF a(ah, al), b(bh, bl);
        np::DF r, r2(0.0f, 0.0f);
        switch (op[0]) {
            case '+': r = a + b; break;
            case '-': r = a - b; break;
            case '*': r = a * b; break;
            case '/': r = a / b; break;
            default: np::df_sincos(a, r, r2); break;
        }
        std::printf("%a %a %a %a\n", r.hi, r.lo, r2.hi, r2.lo);
    }
    return 0;
}
