// Host-side model of the XC problem: basis sets, grid recipes, blocks, and
// the device structures the kernels read.  Layout decisions (HBM):
//   points      x, y, z, w            FP64, block order, each block padded to 8
//   AO store    [block][comp][n_b][ng] FP64, g fastest (coalesced per point)
//   densities   rho (s, G), rho1 (s, 3, G), tau (s, G), sigma (3 or 1, G)
//   potentials  eps (G), vrho (s, G), vsigma (.., G), vtau (s, G)
//   Fock coefs  fcoef (s, 5, G): 1/2 w vrho | w (2 vsigma grad rho ...) xyz | 1/4 w vtau
#pragma once

#include <string>
#include <vector>

namespace cgb {

constexpr int kMaxL = 4;         // highest angular momentum evaluated on the grid
constexpr int kMaxBlockPts = 128;  // GridGeneration.cpp:24 (max_size)

struct Shell {
    int atom;
    int l;
    int type;  // 0 S, 1 Cartesian P, -l pure (reference SubGrid/GridAO convention)
    int first; // first basis function index
    int nprim;
    int prim_off;
    double x, y, z;
    double extent;  // radius beyond which |phi| and |grad phi| < extent_threshold
    double extent_threshold;
};

inline int shell_size(int type) { return type == 0 ? 1 : (type == 1 || type == -1 ? 3 : 2 * (type < 0 ? -type : type) + 1); }

struct BasisSet {
    std::vector<int> Z;
    std::vector<double> xyz;  // natoms x 3, bohr
    std::vector<Shell> shells;
    std::vector<double> exps, coefs;  // coefs libint2-normalised
    int nbasis = 0;
    int natoms() const { return (int)Z.size(); }
};

struct GridRecipe {
    int nshells_total = 0;
    std::string formula;
    std::vector<double> params;
    std::vector<std::pair<int, int>> groups;  // (npoints, nshells)
};

// Data files (package data directory).
const std::string& data_path();
void set_data_path(const std::string& p);
const std::vector<double>& lebedev_rule(int npoints);  // 4*npoints: x y z w
const GridRecipe& grid_recipe(const std::string& grid, int Z);
BasisSet load_basis(const std::string& name, const std::vector<int>& Z, const std::vector<double>& xyz);
// libint2's renormalisation of one contracted shell (primitive factors for
// x^l exp(-a r^2), then unit self-overlap), as Normalization.cpp:11-18 applies it.
std::vector<double> renorm_contraction(int l, const std::vector<double>& e, std::vector<double> c);
void sap_table(int Z, std::vector<double>& radii, std::vector<double>& rv);  // 751 entries each

// Solid-harmonic coefficient table: coef[l][i][k] for function i (m = i - l)
// over Cartesian monomials k (canonical order a = l..0, b = l-a..0).
void solid_harmonic_table(double out[kMaxL + 1][2 * kMaxL + 1][(kMaxL + 1) * (kMaxL + 2) / 2]);

// Shell extent (bohr) for an AO-magnitude threshold.
double shell_extent(const BasisSet& b, const Shell& s, double threshold);

// Per-block descriptor shared by all kernels.
struct BlockDesc {
    int pt_off;     // first padded point
    int ng;         // padded points (multiple of 8, <= 128)
    int nreal;      // real points
    int nb;         // screened basis functions
    int bas_off;    // offset into the block basis-list array
    int nsh;        // screened shells
    int sh_off;     // offset into the block shell-list array
    int pad;
    long long ao_off;  // offset (elements) of component 0 in the AO store
};

}  // namespace cgb
