// Instantiates fts::FlowGPU with stand-ins for the reference's LevelSet,
// Parameters and VecXd (the member functions Flow uses) and runs one solve of
// a small Kuhn lattice.  Exit code: 0 solved, 10 init refused (no GPU), other
// values = failures.
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "fts_flow.hpp"
#include "fts_gen.h"

struct Vec {
    std::vector<double> v;
    double& operator()(int64_t i) { return v[(size_t)i]; }
    double operator()(int64_t i) const { return v[(size_t)i]; }
};
struct P3 {
    float c[3];
    float operator()(int a) const { return c[a]; }
};
struct T4 {
    int c[4];
    int operator()(int a) const { return c[a]; }
};
struct Mesh {
    std::vector<P3> pts;
    std::vector<T4> tets;
    const std::vector<P3>& p() const { return pts; }
    const std::vector<T4>& t() const { return tets; }
};
struct LevelSet {
    Mesh mesh;
    Vec phi;
    const Mesh& getMesh() const { return mesh; }
    const Vec& getPhi() const { return phi; }
};
struct Parameters {
    std::map<std::string, double> m;
    double operator[](const std::string& k) const {
        auto it = m.find(k);
        return it == m.end() ? 0.0 : it->second;
    }
};

int main() {
    const int n = 9;
    int64_t np, nt;
    fts_gen_kuhn_counts(n, &np, &nt);
    std::vector<float> xyz(3 * np);
    std::vector<int32_t> tets(4 * nt);
    fts_gen_kuhn_mesh(n, 0.0, 1, xyz.data(), tets.data(), nullptr);
    LevelSet ls;
    ls.mesh.pts.resize(np);
    ls.mesh.tets.resize(nt);
    for (int64_t i = 0; i < np; ++i)
        for (int a = 0; a < 3; ++a) ls.mesh.pts[i].c[a] = xyz[3 * i + a];
    for (int64_t k = 0; k < nt; ++k)
        for (int j = 0; j < 4; ++j) ls.mesh.tets[k].c[j] = tets[4 * k + j];
    ls.phi.v.resize(np);
    Vec source{std::vector<double>(np)};
    for (int64_t i = 0; i < np; ++i) {
        double x = xyz[3 * i] - 0.5, y = xyz[3 * i + 1] - 0.5, z = xyz[3 * i + 2] - 0.5;
        double r = std::sqrt(x * x + y * y + z * z);
        ls.phi(i) = r - 0.3;
        source(i) = std::exp(-((x - 0.3) * (x - 0.3) + y * y + z * z) / 0.02);
    }
    Parameters par;
    par.m = {{"Stokes velocity degree", 1}, {"alpha", 0.1}, {"eps", 1e-3},
             {"Stokes tolerance", 1e-9}, {"Viscosity interior", 10.0},
             {"Viscosity exterior", 1.0}, {"Viscosity profile", 0}, {"GF growth", 0.5},
             {"Advection dt", 1.0}};
    fts::FlowGPU<LevelSet, Parameters, Vec> flow;
    if (flow.init(ls, par) != 0) return 10;
    Vec out{std::vector<double>(4 * np, 0.0)};
    if (flow.solve(ls, source, out) != 0) return 2;
    if (!flow.stats().solved || !(flow.stats().rel_residual <= 1e-9)) return 3;
    double vmax = 0.0;
    for (int64_t i = 0; i < 3 * np; ++i) vmax = std::fmax(vmax, std::fabs(out(i)));
    std::printf("FlowGPU solved: %lld iterations, rel residual %.3e, max |u| %.4e\n",
                (long long)flow.stats().iterations, flow.stats().rel_residual, vmax);
    return vmax > 0.0 ? 0 : 4;
}
