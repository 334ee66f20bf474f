// Instantiates fts::FlowGPU with stand-ins for the reference's LevelSet,
// Parameters and VecXd (the member functions Flow uses) and runs two solves on
// a small Kuhn lattice: one without and one with surface tension ("Surface
// tension" > 0: FlowGPU builds the interfacial load itself).  Exit code:
// 0 solved, 10 init refused (no GPU), other values = failures.
//
// argv[1] (optional): a file that receives np (int64) and then, as doubles,
// phi[np], source[np], flow[4 np] of the plain solve, flow[4 np] of the solve
// with surface tension and its load [3 np], for the test to check.
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "fts_flow.hpp"

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

// Kuhn-split n^3 lattice of the unit cube: node (i,j,k) = (i,j,k)/(n-1) with
// index i + n j + n^2 k; cube c split into the 6 monotone paths from its
// corner (0,0,0) to (1,1,1), one per axis permutation.
static void kuhn_lattice(int n, Mesh& m) {
    const double h = 1.0 / (n - 1);
    m.pts.resize((size_t)n * n * n);
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
                m.pts[i + n * (j + n * k)] = {{(float)(i * h), (float)(j * h), (float)(k * h)}};
    const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int off[3] = {1, n, n * n};
    const int c1 = n - 1;
    m.tets.resize((size_t)6 * c1 * c1 * c1);
    for (int c = 0; c < c1 * c1 * c1; ++c) {
        const int base = c % c1 + n * ((c / c1) % c1 + n * (c / (c1 * c1)));
        for (int t = 0; t < 6; ++t) {
            const int a = base + off[perm[t][0]];
            m.tets[6 * c + t] = {{base, a, a + off[perm[t][1]], base + 1 + n + n * n}};
        }
    }
}

int main(int argc, char** argv) {
    const int n = 9;
    LevelSet ls;
    kuhn_lattice(n, ls.mesh);
    const int64_t np = (int64_t)ls.mesh.pts.size();
    ls.phi.v.resize(np);
    Vec source{std::vector<double>(np)};
    for (int64_t i = 0; i < np; ++i) {
        const P3& p = ls.mesh.pts[i];
        double x = p.c[0] - 0.5, y = p.c[1] - 0.5, z = p.c[2] - 0.5;
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
    if (!(vmax > 0.0)) return 4;

    // the same level set with an interfacial tension (parameters/Fig4 *_st1*)
    Parameters par_st = par;
    par_st.m["Surface tension"] = 1.0;
    par_st.m["Node density"] = 2.0;
    fts::FlowGPU<LevelSet, Parameters, Vec> flow_st;
    if (flow_st.init(ls, par_st) != 0) return 5;
    Vec out_st{std::vector<double>(4 * np, 0.0)};
    if (flow_st.solve(ls, source, out_st) != 0) return 6;
    if (!flow_st.stats().solved || !(flow_st.stats().rel_residual <= 1e-9)) return 7;
    const std::vector<double>& load = flow_st.surfaceTensionLoad();
    double fmax = 0.0, dmax = 0.0;
    for (double f : load) fmax = std::fmax(fmax, std::fabs(f));
    for (int64_t i = 0; i < 3 * np; ++i) dmax = std::fmax(dmax, std::fabs(out_st(i) - out(i)));
    std::printf("FlowGPU solved with surface tension: %lld iterations, max |load| %.4e, "
                "max |du| %.4e\n", (long long)flow_st.stats().iterations, fmax, dmax);
    if ((int64_t)load.size() != 3 * np || !(fmax > 0.0) || !(dmax > 0.0)) return 8;

    if (argc > 1) {
        FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 9;
        std::fwrite(&np, sizeof(np), 1, f);
        std::fwrite(ls.phi.v.data(), sizeof(double), np, f);
        std::fwrite(source.v.data(), sizeof(double), np, f);
        std::fwrite(out.v.data(), sizeof(double), 4 * np, f);
        std::fwrite(out_st.v.data(), sizeof(double), 4 * np, f);
        std::fwrite(load.data(), sizeof(double), 3 * np, f);
        std::fclose(f);
    }
    return 0;
}
