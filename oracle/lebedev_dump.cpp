// Prints the Lebedev-Laikov angular rules that the reference's grid generator
// uses (src/Grid/GridGeneration.cpp:121-125 calls ld_by_order(npoints, ...)).
// This driver is linked against the reference's own src/Grid/sphere_lebedev_rule.cpp,
// compiled where it lies; the printed tables become chinium_gb300/data/lebedev.txt.
// Test infrastructure only: nothing in the product links this file.
#include <cstdio>
#include <cstdlib>
#include <vector>

void ld_by_order(int order, double* x, double* y, double* z, double* w);

int main(int argc, char** argv) {
    for (int i = 1; i < argc; i++) {
        const int n = std::atoi(argv[i]);
        std::vector<double> x(n), y(n), z(n), w(n);
        ld_by_order(n, x.data(), y.data(), z.data(), w.data());
        std::printf("order %d\n", n);
        for (int k = 0; k < n; k++)
            std::printf("%.17g %.17g %.17g %.17g\n", x[k], y[k], z[k], w[k]);
    }
    return 0;
}
