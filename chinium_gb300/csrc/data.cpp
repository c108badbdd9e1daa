// Data tables (Lebedev rules, SG-n recipes, basis sets, SAP potentials), basis
// construction with libint2's contraction normalisation, the real solid
// harmonic coefficients, and shell extents for screening.
#include <dlfcn.h>

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

#include "common.h"
#include "model.h"

namespace cgb {

namespace {
std::mutex g_mu;
std::string g_data_path;
std::map<int, std::vector<double>> g_lebedev;
std::map<std::string, std::map<int, GridRecipe>> g_recipes;
std::vector<double> g_sap_radii;
std::map<int, std::vector<double>> g_sap;

std::string default_data_path() {
    if (const char* e = std::getenv("CHINIUM_GB300_DATA")) return e;
    Dl_info info;
    if (dladdr((void*)&default_data_path, &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        auto pos = so.rfind('/');
        std::string dir = pos == std::string::npos ? "." : so.substr(0, pos);
        return dir + "/../data";  // library lives in chinium_gb300/_build/
    }
    return "chinium_gb300/data";
}

// Caller holds g_mu.
const std::string& data_path_locked() {
    if (g_data_path.empty()) g_data_path = default_data_path();
    return g_data_path;
}

// Caller holds g_mu.
std::ifstream open_data(const std::string& rel) {
    std::ifstream f(data_path_locked() + "/" + rel);
    if (!f.good()) throw Error(XC_ERR_IO, "missing data file: " + data_path_locked() + "/" + rel);
    return f;
}

void load_lebedev_locked() {
    if (!g_lebedev.empty()) return;
    auto f = open_data("lebedev.txt");
    std::string word;
    while (f >> word) {
        if (word != "order") throw Error(XC_ERR_IO, "corrupt lebedev.txt");
        int n;
        f >> n;
        std::vector<double> v(4 * (size_t)n);
        for (auto& x : v) f >> x;
        if (!f) throw Error(XC_ERR_IO, "corrupt lebedev.txt");
        g_lebedev[n] = std::move(v);
    }
}

void load_recipes_locked(const std::string& grid) {
    if (g_recipes.count(grid)) return;
    auto f = open_data("grids/" + grid + ".txt");
    std::map<int, GridRecipe> m;
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::stringstream ss(line);
        std::string tag;
        int Z, nsh, ngroups;
        ss >> tag >> Z >> nsh >> ngroups;
        if (tag != "element") throw Error(XC_ERR_IO, "corrupt grid recipe " + grid);
        GridRecipe r;
        r.nshells_total = nsh;
        ss >> r.formula;
        double p;
        while (ss >> p) r.params.push_back(p);
        for (int i = 0; i < ngroups; i++) {
            int np, ns;
            f >> np >> ns;
            r.groups.emplace_back(np, ns);
        }
        std::getline(f, line);
        m[Z] = r;
    }
    g_recipes[grid] = std::move(m);
}

void load_sap_locked() {
    if (!g_sap_radii.empty()) return;
    auto f = open_data("sap.txt");
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::stringstream ss(line);
        std::string tag;
        ss >> tag;
        std::vector<double> v;
        double x;
        while (ss >> x) v.push_back(x);
        if (tag == "radii") g_sap_radii = v;
        else g_sap[std::atoi(tag.c_str())] = v;
    }
}

double dfact(int n) {
    double r = 1;
    while (n > 1) {
        r *= n;
        n -= 2;
    }
    return r;
}

double binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    double r = 1;
    for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
    return r;
}

double fact(int n) {
    double r = 1;
    for (int i = 2; i <= n; i++) r *= i;
    return r;
}
}  // namespace

const std::string& data_path() {
    std::lock_guard<std::mutex> lk(g_mu);
    return data_path_locked();
}

void set_data_path(const std::string& p) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_data_path = p;
    g_lebedev.clear();
    g_recipes.clear();
    g_sap_radii.clear();
    g_sap.clear();
}

const std::vector<double>& lebedev_rule(int n) {
    data_path();
    std::lock_guard<std::mutex> lk(g_mu);
    load_lebedev_locked();
    auto it = g_lebedev.find(n);
    if (it == g_lebedev.end()) throw Error(XC_ERR_IO, "no Lebedev rule with " + std::to_string(n) + " points");
    return it->second;
}

const GridRecipe& grid_recipe(const std::string& grid, int Z) {
    data_path();
    std::lock_guard<std::mutex> lk(g_mu);
    load_recipes_locked(grid);
    auto& m = g_recipes[grid];
    auto it = m.find(Z);
    if (it == m.end()) throw Error(XC_ERR_IO, "Missing element grid file in folder! (" + grid + ", Z=" + std::to_string(Z) + ")");
    return it->second;
}

void sap_table(int Z, std::vector<double>& radii, std::vector<double>& rv) {
    data_path();
    std::lock_guard<std::mutex> lk(g_mu);
    load_sap_locked();
    auto it = g_sap.find(Z);
    if (it == g_sap.end()) throw Error(XC_ERR_IO, "no SAP table for Z=" + std::to_string(Z));
    radii = g_sap_radii;
    rv = it->second;
}

// libint2 Shell::renorm (the normalisation Normalization.cpp:11-18 copies):
// primitive factor for x^l exp(-a r^2), then the contraction's self-overlap
// is scaled to one.
std::vector<double> renorm_contraction(int l, const std::vector<double>& e, std::vector<double> c) {
    const double sqrt_pi3 = std::pow(M_PI, 1.5);
    const double df = dfact(2 * l - 1);
    for (size_t p = 0; p < e.size(); p++) {
        const double ta = 2 * e[p];
        c[p] *= std::sqrt(std::pow(2.0, l) * std::pow(ta, l + 1) * std::sqrt(ta) / (sqrt_pi3 * df));
    }
    double norm = 0;
    for (size_t p = 0; p < e.size(); p++)
        for (size_t q = 0; q <= p; q++) {
            const double g = e[p] + e[q];
            norm += (p == q ? 1 : 2) * df * sqrt_pi3 * c[p] * c[q] / (std::pow(2.0, l) * std::pow(g, l + 1) * std::sqrt(g));
        }
    const double f = 1 / std::sqrt(norm);
    for (auto& x : c) x *= f;
    return c;
}

BasisSet load_basis(const std::string& name, const std::vector<int>& Z, const std::vector<double>& xyz) {
    struct RawShell {
        int l;
        std::vector<double> e, c;
    };
    std::map<int, std::vector<RawShell>> table;
    {
        std::unique_lock<std::mutex> lk(g_mu);
        auto f = open_data("basis/" + name + ".txt");
        lk.unlock();
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::stringstream ss(line);
            std::string tag;
            int z, nsh;
            ss >> tag >> z >> nsh;
            if (tag != "element") throw Error(XC_ERR_IO, "corrupt basis file " + name);
            auto& v = table[z];
            for (int i = 0; i < nsh; i++) {
                RawShell r;
                int np;
                f >> r.l >> np;
                r.e.resize(np);
                r.c.resize(np);
                for (int p = 0; p < np; p++) f >> r.e[p] >> r.c[p];
                if (!f) throw Error(XC_ERR_IO, "corrupt basis file " + name);
                v.push_back(r);
            }
            std::getline(f, line);
        }
    }
    BasisSet b;
    b.Z = Z;
    b.xyz = xyz;
    int first = 0;
    for (size_t a = 0; a < Z.size(); a++) {
        auto it = table.find(Z[a]);
        if (it == table.end()) throw Error(XC_ERR_IO, "basis " + name + " has no element Z=" + std::to_string(Z[a]));
        for (auto& r : it->second) {
            if (r.l > kMaxL) throw Error(XC_ERR_UNSUPPORTED, "angular momentum above g is not supported");
            Shell s{};
            s.atom = (int)a;
            s.l = r.l;
            s.type = r.l == 0 ? 0 : (r.l == 1 ? 1 : -r.l);
            s.first = first;
            s.nprim = (int)r.e.size();
            s.prim_off = (int)b.exps.size();
            s.x = xyz[3 * a];
            s.y = xyz[3 * a + 1];
            s.z = xyz[3 * a + 2];
            auto c = renorm_contraction(r.l, r.e, r.c);
            b.exps.insert(b.exps.end(), r.e.begin(), r.e.end());
            b.coefs.insert(b.coefs.end(), c.begin(), c.end());
            first += shell_size(s.type);
            b.shells.push_back(s);
        }
    }
    b.nbasis = first;
    return b;
}

// Real solid harmonics S_lm (Helgaker, Jorgensen, Olsen, Molecular
// Electronic-Structure Theory, eqs. 6.4.47-6.4.50): S_l0 = r^l P_l(cos theta),
// the normalisation the reference's AO/Pure*.hpp tables use.
void solid_harmonic_table(double out[kMaxL + 1][2 * kMaxL + 1][(kMaxL + 1) * (kMaxL + 2) / 2]) {
    for (int l = 0; l <= kMaxL; l++)
        for (int i = 0; i < 2 * kMaxL + 1; i++)
            for (int k = 0; k < (kMaxL + 1) * (kMaxL + 2) / 2; k++) out[l][i][k] = 0;
    for (int l = 0; l <= kMaxL; l++) {
        for (int m = -l; m <= l; m++) {
            const int am = std::abs(m);
            const int twovm = m < 0 ? 1 : 0;  // 2 * v_m
            const double N = 1.0 / (std::pow(2.0, am) * fact(l)) *
                             std::sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0));
            const int vmax2 = 2 * (int)std::floor(am / 2.0 - twovm / 2.0) + twovm;  // 2*(floor(|m|/2 - v_m) + v_m)
            for (int t = 0; t <= (l - am) / 2; t++)
                for (int u = 0; u <= t; u++)
                    for (int v2 = twovm; v2 <= vmax2; v2 += 2) {
                        const int sgn_exp = t + (v2 - twovm) / 2;
                        const double C = ((sgn_exp % 2) ? -1.0 : 1.0) * std::pow(0.25, t) * binom(l, t) *
                                         binom(l - t, am + t) * binom(t, u) * binom(am, v2);
                        const int a = 2 * t + am - 2 * u - v2;
                        const int bb = 2 * u + v2;
                        const int c = l - 2 * t - am;
                        if (a < 0 || bb < 0 || c < 0) continue;
                        const int k = ((l - a) * (l - a + 1)) / 2 + (l - a - bb);
                        out[l][m + l][k] += N * C;
                    }
        }
    }
}

// Conservative radius beyond which every function of the shell and its
// gradient stay below threshold: B(r) = 3 sum_p |c_p| e^{-a_p r^2}
// (r^l + 2 a_p r^{l+1} + l r^{l-1}) bounds |phi| and |grad phi|.
double shell_extent(const BasisSet& b, const Shell& s, double threshold) {
    if (threshold <= 0) return 1e30;
    auto bound = [&](double r) {
        double acc = 0;
        for (int p = 0; p < s.nprim; p++) {
            const double a = b.exps[s.prim_off + p], c = std::fabs(b.coefs[s.prim_off + p]);
            const double rl = std::pow(r, s.l);
            acc += c * std::exp(-a * r * r) * (rl + 2 * a * rl * r + (s.l > 0 ? s.l * std::pow(r, s.l - 1) : 0));
        }
        return 3 * acc;
    };
    double r = 60.0;
    while (r > 0 && bound(r) < threshold) r -= 0.05;
    return r + 0.05;
}

}  // namespace cgb
