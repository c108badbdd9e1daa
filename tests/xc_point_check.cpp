// Host driver for tests/test_functional_host.py: evaluates the functional
// library the CUDA kernels use (chinium_gb300/csrc/functional.cuh; energy
// density, forward-mode dual-number potentials and second-derivative jets,
// FP64) on the host.  One point per input line:
//   "v 1 nids id.. rho sigma tau"                 restricted
//   "v 2 nids id.. ra rb saa sab sbb ta tb"       unrestricted
// prints eps and the potentials (restricted 3 values, unrestricted 7, in the
// inputs' order; zero where the family has none);
//   "f 1 nids id.. rho sigma"                     restricted, LDA / GGA
//   "f 2 nids id.. ra rb saa sab sbb"             unrestricted, LDA / GGA
// prints eps, the potentials (2 or 5) and the second derivatives in libxc's
// layouts (v2rho2, v2rhosigma, v2sigma2: 3 or 15 values).
#include <cstdio>

#define CGB_HD inline
#define CGB_HDN inline
#include "functional.cuh"

using namespace cgb::xcf;

template <int FAM>
static void point(int ns, const FuncDesc& f, const double* in, double& eps, double* dv) {
    if (ns == 1) eval_unpol<double, FAM>(f, in[0], in[1], in[2], eps, dv);
    else eval_pol<double, FAM>(f, in, eps, dv);
}

template <int FAM>
static void point2(int ns, const FuncDesc& f, const double* in, double& eps, double* dv, double* d2) {
    if (ns == 1) eval_unpol2<double, FAM>(f, in[0], in[1], eps, dv, d2);
    else eval_pol2<double, FAM>(f, in, eps, dv, d2);
}

int main() {
    char mode[4];
    int ns, nids;
    while (std::scanf("%3s %d %d", mode, &ns, &nids) == 3) {
        const bool second = mode[0] == 'f';
        if ((mode[0] != 'v' && !second) || (ns != 1 && ns != 2) || nids < 1 || nids > 4) return 2;
        FuncDesc f{};
        f.nids = nids;
        int fam = 0;
        for (int i = 0; i < nids; i++) {
            if (std::scanf("%d", &f.ids[i]) != 1) return 2;
            const int fi = family_of_id(f.ids[i]);
            if (fi < 0 || (second && fi > 1)) return 3;
            fam = fi > fam ? fi : fam;
        }
        const int nin = second ? (ns == 1 ? 2 : 5) : (ns == 1 ? 3 : 7);
        double in[7] = {0}, dv[7] = {0}, d2[15] = {0}, eps = 0;
        for (int i = 0; i < nin; i++)
            if (std::scanf("%lf", &in[i]) != 1) return 2;
        int nd2 = 0;
        if (second) {
            nd2 = ns == 1 ? 3 : 15;
            if (fam == 0) point2<0>(ns, f, in, eps, dv, d2);
            else point2<1>(ns, f, in, eps, dv, d2);
        } else if (fam == 0) {
            point<0>(ns, f, in, eps, dv);
        } else if (fam == 1) {
            point<1>(ns, f, in, eps, dv);
        } else {
            point<2>(ns, f, in, eps, dv);
        }
        std::printf("%.17g", eps);
        for (int i = 0; i < nin; i++) std::printf(" %.17g", dv[i]);
        for (int i = 0; i < nd2; i++) std::printf(" %.17g", d2[i]);
        std::printf("\n");
    }
    return 0;
}
