// fts_flow.hpp — header-only C++ drop-in for the reference's class Flow
// (src/growth/Flow.hpp:15-63) on top of the C ABI in fts.h.
//
//   Flow::init(const LevelSet&, const Parameters&)           (Flow.cpp:20-85)
//   Flow::solve(const LevelSet&, const VecXd& source, VecXd& flow)  (Flow.cpp:89-94)
//
// FlowGPU<LevelSet, Parameters, VecXd> has the same two members with the same
// argument meaning and return convention (0 success, -1 failure; the early exits
// leave `flow` untouched).  It reads only what Flow reads: the mesh nodes and
// tetrahedra (lset.getMesh().p(), .t()), the level set (lset.getPhi()) and the
// parameter keys of Flow.cpp / ViscosityProfiles.hpp.  Viscosity is computed on
// the GPU from the growth factor with the reference's profile
// (ViscosityProfiles.hpp:27-72), exactly as Flow does.
//
// "Surface tension" > 0 (Flow.cpp:359-363): Flow::fillF_ adds the interfacial
// load of Flow::surfaceTension_ (Flow.cpp:307-341), built from the LevelSet's
// normals, curvature and interface patches.  Those are functions of the level
// set's full distance reset phi_ifn_, which LevelSet keeps private; after
// LevelSet::update the crossing edges of getPhi() and their end values are the
// ones that reset used, so FlowGPU recomputes phi_ifn_ from getPhi() on the GPU
// (fts_ls_distance_reset), then the load (fts_ls_surface_tension, with
// "Node density" as rho), and passes it to fts_solve as `force`.
//
// The template parameters let the header compile inside the reference's build
// (Eigen types, Mesh3D) without this header including any of them.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "fts.h"

namespace fts {

template <class LevelSetT, class ParametersT, class VecT>
class FlowGPU {
public:
    FlowGPU() = default;
    FlowGPU(const FlowGPU&) = delete;
    FlowGPU& operator=(const FlowGPU&) = delete;
    ~FlowGPU() {
        fts_destroy(ctx_);
        fts_ls_destroy(ls_);
    }

    // GB300 options not present in the reference's parameter file.
    void setPrecision(int precision) { precision_ = precision; }
    void setPreconditioner(int pc) { preconditioner_ = pc; }
    void setDevice(int device) { device_ = device; }

    int init(const LevelSetT& lset, const ParametersT& par) {
        fts_params p;
        fts_params_default(&p);
        p.velocity_degree = (int)par["Stokes velocity degree"];
        if (p.velocity_degree < 1) return -1;  // Flow.cpp:23-25
        p.alpha = par["alpha"];
        p.eps = par["eps"];
        double tol = par["Stokes tolerance"];
        if (tol > 0.0) p.tol = tol;            // Flow.cpp:77-79
        int maxit = (int)par["Max. CG iterations"];
        p.max_iter = maxit > 0 ? maxit : -1;   // Flow.cpp:80-82
        p.mu_interior = par["Viscosity interior"];
        p.mu_exterior = par["Viscosity exterior"];
        p.mu_profile = (int)par["Viscosity profile"];
        p.gf_growth = par["GF growth"];
        p.level_sink = par["Level sink"];
        p.growth_threshold = par["Growth threshold"];
        p.rd_iterations = par["RD iterations"];
        p.gf_production = p.rd_iterations > 0.0 ? (double)par["GF production"] : 1.0;
        p.advection_dt = par["Advection dt"];
        p.surface_tension = par["Surface tension"];
        st_ = (float)p.surface_tension;          // Flow.cpp:359
        rho_ = (int)par["Node density"];         // Flow.cpp:361
        p.precision = precision_;
        p.preconditioner = preconditioner_;
        p.device = device_;
        p.warm_start = 1;  // USE_INITIAL_GUESS (Flow.cpp:15)

        const auto& mesh = lset.getMesh();
        const auto& pts = mesh.p();
        const auto& tet = mesh.t();
        np_ = (int64_t)pts.size();
        nt_ = (int64_t)tet.size();
        std::vector<float> xyz((size_t)(3 * np_));
        std::vector<int32_t> t((size_t)(4 * nt_));
        for (int64_t i = 0; i < np_; ++i)
            for (int a = 0; a < 3; ++a) xyz[3 * i + a] = (float)pts[i](a);
        for (int64_t k = 0; k < nt_; ++k)
            for (int j = 0; j < 4; ++j) t[4 * k + j] = (int32_t)tet[k](j);
        fts_mesh m{np_, nt_, xyz.data(), t.data(), nullptr};
        fts_destroy(ctx_);
        ctx_ = nullptr;
        int rc = fts_create(&m, &p, &ctx_);
        if (rc != FTS_OK) {
            std::fprintf(stderr, "FlowGPU::init(): %s: %s\n", fts_status_string(rc),
                         fts_last_error(nullptr));
            return -1;
        }
        fts_ls_destroy(ls_);
        ls_ = nullptr;
        if (st_ > 0.0f) {  // the level-set context that builds the interfacial load
            rc = fts_ls_create(&m, device_, &ls_);
            if (rc != FTS_OK) {
                std::fprintf(stderr, "FlowGPU::init(): %s: %s\n", fts_status_string(rc),
                             fts_ls_last_error(nullptr));
                return -1;
            }
        }
        return 0;
    }

    int solve(const LevelSetT& lset, const VecT& source, VecT& flow) {
        if (!ctx_) return -1;
        const auto& phi = lset.getPhi();
        phi_.assign((size_t)np_, 0.0);
        src_.assign((size_t)np_, 0.0);
        out_.resize((size_t)(4 * np_));
        for (int64_t i = 0; i < np_; ++i) {
            phi_[i] = (double)phi(i);
            src_[i] = (double)source(i);
        }
        for (int64_t i = 0; i < 4 * np_; ++i) out_[i] = (double)flow(i);
        const double* force = nullptr;
        if (st_ > 0.0f) {  // Flow.cpp:359-363
            reset_.resize((size_t)np_);
            force_.resize((size_t)(3 * np_));
            int rs = ls_ ? fts_ls_distance_reset(ls_, phi_.data(), reset_.data()) : FTS_ERR_BAD_INPUT;
            if (rs == FTS_OK)
                rs = fts_ls_surface_tension(ls_, phi_.data(), reset_.data(), (double)st_, rho_,
                                            force_.data(), nullptr);
            if (rs != FTS_OK) {
                std::fprintf(stderr, "FlowGPU::solve(): surface tension: %s: %s\n",
                             fts_status_string(rs), fts_ls_last_error(ls_));
                return -1;
            }
            force = force_.data();
        }
        int rc = fts_solve(ctx_, phi_.data(), src_.data(), nullptr, force, out_.data(), &stats_);
        if (rc != FTS_OK) {
            std::fprintf(stderr, "FlowGPU::solve(): %s: %s\n", fts_status_string(rc),
                         fts_last_error(ctx_));
            return -1;  // Flow.cpp:281-285
        }
        if (stats_.solved)
            for (int64_t i = 0; i < 4 * np_; ++i) flow(i) = out_[i];
        return 0;
    }

    const fts_stats& stats() const { return stats_; }
    // The interfacial load of the last solve, [fx(np), fy(np), fz(np)] (empty
    // when "Surface tension" is 0).
    const std::vector<double>& surfaceTensionLoad() const { return force_; }

private:
    fts_ctx* ctx_ = nullptr;
    fts_ls* ls_ = nullptr;
    float st_ = 0.0f;
    int rho_ = 0;
    std::vector<double> reset_, force_;
    int64_t np_ = 0, nt_ = 0;
    int precision_ = FTS_PREC_FP64;
    int preconditioner_ = FTS_PC_AUTO;
    int device_ = 0;
    std::vector<double> phi_, src_, out_;
    fts_stats stats_{};
};

}  // namespace fts
