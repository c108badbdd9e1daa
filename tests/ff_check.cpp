// Host driver for tests/test_float_float.py: applies the float-float scalar
// of the functional library (chinium_gb300/csrc/functional.cuh, xcf::ff) to
// the doubles read from stdin, one "op x [y]" per line, and prints the
// results as doubles (hi + lo) with 17 significant digits.
#include <cstdio>
#include <cstring>

// host compilation (g++): plain inline functions
#define CGB_HD inline
#define CGB_HDN inline
#include "functional.cuh"

using cgb::xcf::ff;
using cgb::xcf::ff_value;
using S = cgb::xcf::Scal<ff>;

int main() {
    char op[16];
    double x, y;
    while (std::scanf("%15s %lf %lf", op, &x, &y) == 3) {
        const ff a(x), b(y);
        ff r;
        if (!std::strcmp(op, "add")) r = a + b;
        else if (!std::strcmp(op, "sub")) r = a - b;
        else if (!std::strcmp(op, "mul")) r = a * b;
        else if (!std::strcmp(op, "div")) r = a / b;
        else if (!std::strcmp(op, "exp")) r = S::exp_(a);
        else if (!std::strcmp(op, "log")) r = S::log_(a);
        else if (!std::strcmp(op, "sqrt")) r = S::sqrt_(a);
        else if (!std::strcmp(op, "cbrt")) r = S::cbrt_(a);
        else if (!std::strcmp(op, "pow3")) r = cgb::xcf::pow3(a, (int)y);
        else if (!std::strcmp(op, "split")) r = a;
        else return 2;
        std::printf("%.17g\n", ff_value(r));
    }
    return 0;
}
