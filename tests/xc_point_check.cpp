// Host driver for tests/test_functional_host.py: evaluates the functional
// library the CUDA kernels use (chinium_gb300/csrc/functional.cuh; energy
// density and forward-mode dual-number potentials, FP64) on the host.  One
// point per input line:
//   "1 nids id.. rho sigma tau"                 (restricted)
//   "2 nids id.. ra rb saa sab sbb ta tb"       (unrestricted)
// prints eps and the potentials (vrho, vsigma, vtau in the library's order:
// restricted 3 values, unrestricted 7), zero where the family has none.
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

int main() {
    int ns, nids;
    while (std::scanf("%d %d", &ns, &nids) == 2) {
        if ((ns != 1 && ns != 2) || nids < 1 || nids > 4) return 2;
        FuncDesc f{};
        f.nids = nids;
        int fam = 0;
        for (int i = 0; i < nids; i++) {
            if (std::scanf("%d", &f.ids[i]) != 1) return 2;
            const int fi = family_of_id(f.ids[i]);
            if (fi < 0) return 3;
            fam = fi > fam ? fi : fam;
        }
        const int nin = ns == 1 ? 3 : 7;
        double in[7] = {0}, dv[7] = {0}, eps = 0;
        for (int i = 0; i < nin; i++)
            if (std::scanf("%lf", &in[i]) != 1) return 2;
        if (fam == 0) point<0>(ns, f, in, eps, dv);
        else if (fam == 1) point<1>(ns, f, in, eps, dv);
        else point<2>(ns, f, in, eps, dv);
        std::printf("%.17g", eps);
        for (int i = 0; i < nin; i++) std::printf(" %.17g", dv[i]);
        std::printf("\n");
    }
    return 0;
}
