// C ABI of libfts (include/fts.h): context lifecycle and the Stokes solve
// pipeline, the GB300 counterpart of Flow::init / Flow::solve
// (src/growth/Flow.cpp:20-94, :218-302).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <vector>
#include <cstring>
#include <exception>
#include <new>

#include "fts_device.cuh"

namespace fts {

void free_all(Ctx& c) {
    void* ptrs[] = {c.xyz, c.tets, c.bnd, c.rowptr, c.cols, c.diag, c.p2t_ptr, c.p2t, c.geom,
                    c.phi, c.src, c.force, c.mu, c.s, c.flow, c.A64, c.A32, c.ell_val,
                    c.ell_col, c.ell_ptr, c.lat_val, c.lat_src, c.lat64, c.pc64, c.pc32, c.dofs, c.xp2t_ptr, c.xp2t,
                    c.b, c.x, c.r, c.w64.q, c.w64.R[0], c.w64.R[1], c.w64.Y[0], c.w64.Y[1],
                    c.w64.W[0], c.w64.W[1], c.w64.X, c.w32.q, c.w32.R[0], c.w32.R[1],
                    c.w32.Y[0], c.w32.Y[1], c.w32.W[0], c.w32.W[1], c.w32.X, c.w32.r0, c.ms,
                    c.os, c.red.partials, c.red.ticket, c.err_flag, c.bicg, c.mf_rec, c.mf_cube, c.mf_rows};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    mg_free(c.mg64);
    mg_free(c.mg32);
    p2mg_free(c.p2mg64);
    p2mg_free(c.p2mg32);
    pmg_free(c.pmg64);
    pmg_free(c.pmg32);
    if (c.ev_fork) cudaEventDestroy(c.ev_fork);
    if (c.ev_join) cudaEventDestroy(c.ev_join);
    if (c.aux_stream) cudaStreamDestroy(c.aux_stream);
    if (c.ms_host) cudaFreeHost(c.ms_host);
    if (c.os_host) cudaFreeHost(c.os_host);
    for (auto& e : c.ev)
        if (e) cudaEventDestroy(e);
    if (c.own_stream) cudaStreamDestroy(c.own_stream);
}

template <typename T>
static void alloc_work(Ctx& c, KrylovWork<T>& w, bool own_r0) {
    w.q = dev_alloc<V4<T>>(c, c.np);
    for (int i = 0; i < 2; ++i) {
        w.R[i] = dev_alloc<V4<T>>(c, c.np);
        w.Y[i] = dev_alloc<V4<T>>(c, c.np);
        w.W[i] = dev_alloc<V4<T>>(c, c.np);
    }
    w.X = dev_alloc<V4<T>>(c, c.np);
    if (own_r0) w.r0 = dev_alloc<V4<T>>(c, c.np);
}

// Sliced-ELL structure (host) of the block graph: slices of 8 rows padded to
// the longest row of the slice.
static void build_ell(Ctx& c) {
    const HostTopology& T = c.topo;
    c.nslices = (c.np + 7) / 8;
    std::vector<int32_t> ptr((size_t)c.nslices + 1, 0);
    for (int64_t s = 0; s < c.nslices; ++s) {
        int32_t kmax = 0;
        for (int64_t r = 8 * s; r < std::min<int64_t>(c.np, 8 * s + 8); ++r)
            kmax = std::max(kmax, T.rowptr[r + 1] - T.rowptr[r]);
        ptr[s + 1] = ptr[s] + 8 * kmax;
    }
    c.ell_slots = ptr[c.nslices];
    std::vector<int32_t> col((size_t)c.ell_slots, 0);
    for (int64_t s = 0; s < c.nslices; ++s) {
        const int32_t kmax = (ptr[s + 1] - ptr[s]) / 8;
        for (int l = 0; l < 8; ++l) {
            const int64_t r = 8 * s + l;
            const int32_t len = r < c.np ? T.rowptr[r + 1] - T.rowptr[r] : 0;
            for (int32_t k = 0; k < kmax; ++k)
                col[ptr[s] + 8 * k + l] = k < len ? T.cols[T.rowptr[r] + k] : 0;
        }
    }
    c.ell_ptr = dev_alloc<int32_t>(c, (size_t)c.nslices + 1);
    c.ell_col = dev_alloc<int32_t>(c, (size_t)c.ell_slots);
    c.ell_val = dev_alloc<float>(c, (size_t)c.ell_slots * 16);
    FTS_CUDA(cudaMemcpy(c.ell_ptr, ptr.data(), ptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    FTS_CUDA(cudaMemcpy(c.ell_col, col.data(), col.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    c.use_ell = true;
}

// Source block of every lattice half-stencil entry: for node v and direction d
// (0 = self, 1..7 = the positive Kuhn directions) the BSR block (v, v + d), or
// -1 where the neighbour is outside the lattice or the block is absent.
void build_lattice(Ctx& c) {
    const HostTopology& T = c.topo;
    const int64_t n = T.lattice_n;
    const int64_t tiles = (c.np + 31) / 32;
    static const int ox[8] = {0, 1, 0, 0, 1, 1, 0, 1}, oy[8] = {0, 0, 1, 0, 1, 0, 1, 1},
                     oz[8] = {0, 0, 0, 1, 0, 1, 1, 1};
    std::vector<int32_t> src((size_t)tiles * 32 * 8, -1);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < c.np; ++v) {
        const int64_t i = v % n, j = (v / n) % n, k = v / (n * n);
        for (int d = 0; d < 8; ++d) {
            if (i + ox[d] >= n || j + oy[d] >= n || k + oz[d] >= n) continue;
            const int64_t w = v + ox[d] + n * (oy[d] + n * oz[d]);
            for (int32_t q = T.rowptr[v]; q < T.rowptr[v + 1]; ++q)
                if (T.cols[q] == w) {
                    src[(size_t)v * 8 + d] = q;
                    break;
                }
        }
    }
    c.lat_src = dev_alloc<int32_t>(c, src.size());
    c.lat_val = dev_alloc<float>(c, (size_t)tiles * 128 * 32);
    FTS_CUDA(cudaMemcpy(c.lat_src, src.data(), src.size() * sizeof(int32_t),
                        cudaMemcpyHostToDevice));
}

void ensure_fp64_work(Ctx& c) {
    if (!c.w64.q) alloc_work<double>(c, c.w64, false);
}

// FP32 operator copy in the storage the context currently selects (built on
// first use; a later parameter update may select the other storage).
void ensure_fp32(Ctx& c) {
    if (!c.matfree) {
        if (c.in_batch) {
            if (!c.A32) c.A32 = dev_alloc<float>(c, (size_t)c.nnzb * 16);
        } else if (c.use_lat) {
            if (!c.lat_val) build_lattice(c);
        } else if (!c.ell_val) {
            build_ell(c);
        }
    }
    if (c.have32) return;
    c.pc32 = dev_alloc<float>(c, (size_t)c.np * 8);
    alloc_work<float>(c, c.w32, true);
    c.have32 = true;
}

int validate_params(const fts_params& p, std::string& err) {
    if (p.velocity_degree != 1 && p.velocity_degree != 2) {
        err = "velocity degree must be 1 (P1-P1 stabilised) or 2 (P2-P1)";
        return FTS_ERR_UNSUPPORTED;
    }
    if (p.velocity_degree == 2 &&
        (p.operator_kind == FTS_OP_MATFREE || p.operator_kind == FTS_OP_STENCIL)) {
        err = "P2-P1 runs on the assembled operator (FTS_OP_AUTO or FTS_OP_ASSEMBLED)";
        return FTS_ERR_UNSUPPORTED;
    }
    if (p.precision != FTS_PREC_FP64 && p.precision != FTS_PREC_MIXED) {
        err = "unknown precision";
        return FTS_ERR_BAD_INPUT;
    }
    if (p.operator_kind < FTS_OP_AUTO || p.operator_kind > FTS_OP_STENCIL) {
        err = "unknown operator kind";
        return FTS_ERR_BAD_INPUT;
    }
    if (p.preconditioner < FTS_PC_AUTO || p.preconditioner > FTS_PC_MULTIGRID_DIAG) {
        err = "unknown preconditioner";
        return FTS_ERR_BAD_INPUT;
    }
    if (p.solver != FTS_SOLVER_MINRES && p.solver != FTS_SOLVER_BICGSTAB) {
        err = "unknown solver";
        return FTS_ERR_BAD_INPUT;
    }
    if (p.solver == FTS_SOLVER_BICGSTAB && p.precision != FTS_PREC_FP64) {
        err = "the reference's BiCGSTAB runs in FP64 only";
        return FTS_ERR_UNSUPPORTED;
    }
    if (!(p.alpha >= 0.0) || !(p.eps >= 0.0)) {
        err = "alpha and eps must be non-negative";
        return FTS_ERR_BAD_INPUT;
    }
    return FTS_OK;
}

// Multigrid needs the Kuhn lattice structure and at least three levels
// (n >= 9); for even n every node on the last layer of each axis must be a
// Dirichlet node (the coarse lattice's last layer sits there).
static int mg_levels(int n) { return (int)mg_chain(n).size(); }

static bool last_layers_dirichlet(const HostTopology& T, int n) {
    const int64_t nvert = (int64_t)n * n * n;  // the lattice's nodes (P2: its vertices)
    for (int64_t v = 0; v < nvert; ++v) {
        const int64_t i = v % n, j = (v / n) % n, k = v / ((int64_t)n * n);
        if ((i == n - 1 || j == n - 1 || k == n - 1) && !T.bnd[v]) return false;
    }
    return true;
}

static void configure_preconditioner(Ctx& c) {
    // P2-P1: the velocity V-cycle has the P2 level above the vertex lattice
    const int n = c.p2 ? c.topo.vertex_lattice_n : c.topo.lattice_n;
    const bool mg_ok = n > 0 && mg_levels(n) >= 3 &&
                       (n % 2 == 1 || last_layers_dirichlet(c.topo, n));
    const bool want_mg = c.par.preconditioner == FTS_PC_MULTIGRID ||
                         c.par.preconditioner == FTS_PC_MULTIGRID_DIAG;
    if (want_mg && !mg_ok) {
        c.last_error = "multigrid needs a Kuhn lattice mesh with n >= 9 (even n: Dirichlet "
                       "nodes on the last layer of every axis)";
        throw (int)FTS_ERR_UNSUPPORTED;
    }
    c.use_mg = mg_ok && c.par.preconditioner != FTS_PC_JACOBI;
    // batched solves keep the pressure diagonal: on batch96 (jumps of mu up to
    // 1e3 across spheres) a pressure V-cycle inside the persistent kernel cut
    // no iterations and its registers slowed every phase
    c.use_pmg = c.use_mg && !c.in_batch && !c.p2 &&
                c.par.preconditioner != FTS_PC_MULTIGRID_DIAG;
    if (c.use_pmg && !c.aux_stream) {
        FTS_CUDA(cudaStreamCreateWithFlags(&c.aux_stream, cudaStreamNonBlocking));
        FTS_CUDA(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming));
        FTS_CUDA(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming));
    }
    if (c.par.operator_kind == FTS_OP_STENCIL && n == 0) {
        c.last_error = "the stencil operator needs a Kuhn lattice mesh";
        throw (int)FTS_ERR_UNSUPPORTED;
    }
    c.use_lat = !c.matfree && !c.in_batch && !c.p2 && n > 0 &&
                (c.par.operator_kind == FTS_OP_AUTO || c.par.operator_kind == FTS_OP_STENCIL);
    // both precisions: the FP64 solve runs its operator on the FP64 half
    // stencil (1 KB/node) as the mixed solve's outer residual does
    c.use_lat64 = c.use_lat && c.par.solver == FTS_SOLVER_MINRES;
    if (c.matfree && (!c.use_mg || c.par.precision != FTS_PREC_MIXED)) {
        c.last_error = "the matrix-free operator runs in mixed precision with the multigrid "
                       "preconditioner (Kuhn lattice, odd n >= 9)";
        throw (int)FTS_ERR_UNSUPPORTED;
    }
    c.crank = (c.par.eps > 0.0 && c.volume > 0.0) ? 1.0 / (c.par.eps * c.volume) : 0.0;
}

void create(Ctx& c, const fts_mesh& m, const fts_params& p) {
    c.par = p;
    c.device = p.device;
    FTS_CUDA(cudaSetDevice(c.device));
    int sms = 0;
    FTS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    c.num_sms = sms > 0 ? sms : 148;
    FTS_CUDA(cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking));
    c.stream = c.own_stream;
    for (auto& e : c.ev) FTS_CUDA(cudaEventCreate(&e));
    const HostTopology& T = c.topo;
    c.np = T.np;
    c.nv = T.nv;
    c.p2 = p.velocity_degree == 2;
    c.nt = T.nt;
    c.nnzb = T.rowptr[T.np];
    c.xyz = dev_alloc<float>(c, 3 * c.nv);
    c.tets = dev_alloc<int32_t>(c, 4 * c.nt);
    c.bnd = dev_alloc<uint8_t>(c, c.np);
    c.rowptr = dev_alloc<int32_t>(c, c.np + 1);
    c.cols = dev_alloc<int32_t>(c, c.nnzb);
    c.diag = dev_alloc<int32_t>(c, c.np);
    c.p2t_ptr = dev_alloc<int32_t>(c, c.np + 1);
    c.p2t = dev_alloc<uint32_t>(c, 4 * c.nt);
    c.geom = dev_alloc<ElemGeom>(c, c.nt);
    c.phi = dev_alloc<double>(c, c.nv);
    c.src = dev_alloc<double>(c, c.nv);
    c.mu = dev_alloc<double>(c, c.nt);
    c.s = dev_alloc<double>(c, c.nv);
    c.flow = dev_alloc<double>(c, 4 * c.np);
    c.matfree = p.operator_kind == FTS_OP_MATFREE;
    // Single solves allocate the FP64 BSR at its first assembly
    // (launch_assemble); batched instances hand its address to the batch's
    // device table when the batch is built, before any assembly.
    if (!c.matfree && c.in_batch) c.A64 = dev_alloc<double>(c, (size_t)c.nnzb * 16);
    c.pc64 = dev_alloc<double>(c, (size_t)c.np * 8);
    c.b = dev_alloc<V4<double>>(c, c.np);
    c.x = dev_alloc<V4<double>>(c, c.np);
    c.r = dev_alloc<V4<double>>(c, c.np);
    if (p.precision == FTS_PREC_FP64) alloc_work<double>(c, c.w64, false);
    c.w64.r0 = c.r;
    c.ms = dev_alloc<MinresScalars>(c, 1);
    c.os = dev_alloc<OuterScalars>(c, 1);
    c.red.partials = dev_alloc<double>(c, kMaxPartials * 4);
    c.red.ticket = dev_alloc<unsigned>(c, 1);
    c.err_flag = dev_alloc<int>(c, 1);
    FTS_CUDA(cudaMallocHost(&c.ms_host, sizeof(MinresScalars)));
    FTS_CUDA(cudaMallocHost(&c.os_host, sizeof(OuterScalars)));
    FTS_CUDA(cudaMemsetAsync(c.red.ticket, 0, sizeof(unsigned), c.stream));
    FTS_CUDA(cudaMemsetAsync(c.err_flag, 0, sizeof(int), c.stream));
    FTS_CUDA(cudaMemsetAsync(c.x, 0, c.np * sizeof(V4<double>), c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.xyz, m.xyz, 3 * c.nv * sizeof(float), cudaMemcpyHostToDevice,
                             c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.tets, m.tets, 4 * c.nt * sizeof(int32_t), cudaMemcpyHostToDevice,
                             c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.bnd, T.bnd.data(), c.np, cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.rowptr, T.rowptr.data(), (c.np + 1) * sizeof(int32_t),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.cols, T.cols.data(), c.nnzb * sizeof(int32_t),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.diag, T.diag.data(), c.np * sizeof(int32_t), cudaMemcpyHostToDevice,
                             c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.p2t_ptr, T.p2t_ptr.data(), (c.np + 1) * sizeof(int32_t),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemcpyAsync(c.p2t, T.p2t.data(), 4 * c.nt * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, c.stream));
    if (c.p2) {
        c.dofs = dev_alloc<int32_t>(c, 10 * c.nt);
        c.xp2t_ptr = dev_alloc<int32_t>(c, c.np + 1);
        c.xp2t = dev_alloc<uint32_t>(c, 10 * c.nt);
        FTS_CUDA(cudaMemcpyAsync(c.dofs, T.dofs.data(), 10 * c.nt * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, c.stream));
        FTS_CUDA(cudaMemcpyAsync(c.xp2t_ptr, T.xp2t_ptr.data(), (c.np + 1) * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, c.stream));
        FTS_CUDA(cudaMemcpyAsync(c.xp2t, T.xp2t.data(), 10 * c.nt * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, c.stream));
    }
    // total volume (for the rank-one constant-pressure term of the preconditioner)
    double vol = 0.0;
#pragma omp parallel for reduction(+ : vol) schedule(static)
    for (int64_t k = 0; k < c.nt; ++k) {
        const int32_t* t = m.tets + 4 * k;
        double q[4][3];
        for (int j = 0; j < 4; ++j)
            for (int a = 0; a < 3; ++a) q[j][a] = (double)m.xyz[3 * (int64_t)t[j] + a];
        double u[3], v[3], w[3];
        for (int a = 0; a < 3; ++a) {
            u[a] = q[1][a] - q[0][a];
            v[a] = q[2][a] - q[0][a];
            w[a] = q[3][a] - q[0][a];
        }
        double det = u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) +
                     u[2] * (v[0] * w[1] - v[1] * w[0]);
        vol += std::fabs(det) / 6.0;
    }
    c.volume = vol;
    configure_preconditioner(c);  // decides the operator storage before any FP32 copy exists
    if (p.precision == FTS_PREC_MIXED) ensure_fp32(c);
    launch_geometry(c, c.err_flag);
    int bad = 0;
    FTS_CUDA(cudaMemcpyAsync(&bad, c.err_flag, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FTS_CUDA(cudaStreamSynchronize(c.stream));
    if (bad) {
        c.last_error = "degenerate tetrahedron (det B == 0)";
        throw 2;
    }
}

static void read_outer(Ctx& c) {
    FTS_CUDA(cudaMemcpyAsync(c.os_host, c.os, sizeof(OuterScalars), cudaMemcpyDeviceToHost,
                             c.stream));
    FTS_CUDA(cudaStreamSynchronize(c.stream));
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// The solve pipeline on device-resident inputs (c.phi, c.src, c.mu / profile,
// c.force).  Returns an fts_status; fills st.
static int solve_device(Ctx& c, bool have_mu, bool have_force, double* flow_out, fts_stats& st) {
    const fts_params& P = c.par;
    const double flt_min = FLT_MIN;
    st.solved = 0;
    if (P.surface_tension > 0.0 && !have_force) {
        // the load needs the level set's interface (normals, curvature,
        // patches): fts_ls_surface_tension computes it
        c.last_error = "\"Surface tension\" > 0 needs its nodal load in `force` "
                       "(fts_ls_surface_tension)";
        return FTS_ERR_UNSUPPORTED;
    }
    // Early exits of Flow::Stokes_ (Flow.cpp:223-228)
    if (P.mu_interior - P.mu_exterior > flt_min && P.rd_iterations > 0.0) {
        // max |source| <= FLT_MIN: nothing to solve
        FTS_CUDA(cudaMemsetAsync(c.err_flag, 0, sizeof(int), c.stream));
        launch_any_abs_above(c, c.src, c.nv, flt_min);
        int any = 0;
        FTS_CUDA(cudaMemcpyAsync(&any, c.err_flag, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        FTS_CUDA(cudaStreamSynchronize(c.stream));
        if (!any) return FTS_OK;
    }
    if (P.advection_dt < flt_min) return FTS_OK;

    FTS_CUDA(cudaMemsetAsync(c.err_flag, 0, sizeof(int), c.stream));
    launch_check_finite(c, c.phi, c.nv);
    launch_check_finite(c, c.src, c.nv);
    if (have_mu) launch_check_finite(c, c.mu, c.nt);
    if (have_force) launch_check_finite(c, c.force, 3 * c.nv);
    FTS_CUDA(cudaEventRecord(c.ev[0], c.stream));
    if (!have_mu) launch_viscosity_profile(c);
    launch_mu_minmax(c);
    launch_source(c);
    if (c.p2) launch_rhs_p2(c, have_force);
    else launch_rhs(c, have_force);
    // the zero-load exit (Flow.cpp:248-251) needs ||F||: computed with the
    // residual kernel on x = 0 below when the matrix exists; here directly.
    if (c.matfree) {
        // no block matrix: pressure weights and the multigrid fine level come
        // straight from the elements
        launch_mf_pc(c);
        setup_preconditioner<float>(c);
    } else if (c.p2) {
        launch_assemble_p2(c);
        launch_preconditioner(c);
        if (P.precision == FTS_PREC_MIXED) {
            ensure_fp32(c);
            launch_to_f32(c);
            setup_preconditioner<float>(c);
        } else {
            setup_preconditioner<double>(c);
        }
    } else if (c.use_lat64) {
        // Kuhn lattice: the FP64 half stencil (and for mixed precision the
        // FP32 one) straight from the elements (no BSR)
        if (P.precision == FTS_PREC_MIXED) ensure_fp32(c);
        launch_assemble_lat(c);
        launch_preconditioner(c);
        if (P.precision == FTS_PREC_MIXED) {
            launch_to_f32(c);
            setup_preconditioner<float>(c);
        } else {
            setup_preconditioner<double>(c);
        }
    } else {
        launch_assemble(c);
        launch_preconditioner(c);
        if (P.precision == FTS_PREC_MIXED) {
            ensure_fp32(c);
            launch_to_f32(c);
            setup_preconditioner<float>(c);
        } else {
            setup_preconditioner<double>(c);
        }
    }
    FTS_CUDA(cudaEventRecord(c.ev[1], c.stream));
    int bad = 0;
    FTS_CUDA(cudaMemcpyAsync(&bad, c.err_flag, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    if (!P.warm_start) FTS_CUDA(cudaMemsetAsync(c.x, 0, c.np * sizeof(V4<double>), c.stream));
    launch_residual64(c);
    read_outer(c);
    st.ms_assembly = elapsed(c.ev[0], c.ev[1]);
    st.mu_min = c.os_host->mu_min;
    st.mu_max = c.os_host->mu_max;
    if (bad) {
        c.last_error = "non-finite value in phi, source, mu or force";
        return FTS_ERR_NAN;
    }
    const double bnorm = std::sqrt(c.os_host->bb);
    st.f_norm = bnorm;
    if (!(bnorm > flt_min)) {
        if (P.verbose) std::printf("  Load zero, nothing to solve.\n");
        return FTS_OK;  // flow untouched (Flow.cpp:248-251)
    }
    if (P.verbose)
        std::printf("  Viscosity min: %g, max: %g\n", st.mu_min, st.mu_max);
    const double tol = P.tol > 0.0 ? P.tol : DBL_EPSILON;
    const long long N = 3 * c.topo.n_interior + c.nv;
    const long long maxit = P.max_iter > 0 ? P.max_iter : 2 * N;
    FTS_CUDA(cudaEventRecord(c.ev[2], c.stream));
    if (P.solver == FTS_SOLVER_BICGSTAB) {
        // the reference's algorithm: stop on the updated residual (Flow.cpp:266-285)
        double err = 0.0;
        int bst = 0;
        long long it = bicgstab_solve(c, tol, maxit, &err, &bst);
        launch_residual64(c);
        read_outer(c);
        FTS_CUDA(cudaEventRecord(c.ev[3], c.stream));
        FTS_CUDA(cudaEventSynchronize(c.ev[3]));
        st.ms_solve = elapsed(c.ev[2], c.ev[3]);
        st.iterations = it;
        st.outer_iterations = 1;
        st.rel_residual = std::sqrt(c.os_host->rr) / bnorm;
        st.error_estimate = err;
        if (bst == 2 || c.os_host->nonfinite) {
            c.last_error = "non-finite value in BiCGSTAB";
            return FTS_ERR_NAN;
        }
        if (!(err <= tol)) {
            c.last_error = "BiCGSTAB stopped above the tolerance";
            return FTS_ERR_NOT_CONVERGED;
        }
        launch_scatter_flow(c, flow_out);
        st.solved = 1;
        return FTS_OK;
    }
    double rel = std::sqrt(c.os_host->rr) / bnorm;
    long long iters = 0, iters32 = 0;
    int outer = 0;
    int status = FTS_OK;
    double est = rel;
    const double floor32 = P.inner_tol > 0.0 ? P.inner_tol
                           : (!c.p2 && c.np >= kInnerTolLargeNodes) ? kInnerTolFloorLarge
                                                                    : kInnerTolFloorSmall;
    while (rel > tol) {
        if (outer >= 40 || iters >= maxit) {
            status = FTS_ERR_NOT_CONVERGED;
            break;
        }
        const double need = tol / rel;  // true reduction still needed
        double achieved = 1.0;
        int ist = 0;
        long long it;
        if (P.precision == FTS_PREC_MIXED) {
            double rt = need / c.pc_ratio32 * 0.5;
            if (rt < floor32) rt = floor32;
            if (rt > 0.5) rt = 0.5;
            launch_prepare_inner32(c);
            it = minres_inner<float>(c, rt, maxit - iters, &achieved, &ist);
            launch_update_x_from32(c);
            iters32 += it;
        } else {
            double rt = need / c.pc_ratio64 * 0.5;
            if (rt > 0.5) rt = 0.5;
            it = minres_inner<double>(c, rt, maxit - iters, &achieved, &ist);
            launch_update_x64(c);
        }
        iters += it;
        ++outer;
        const double prev = rel;
        launch_residual64(c);
        read_outer(c);
        if (c.os_host->nonfinite || ist == 2) {
            status = FTS_ERR_NAN;
            c.last_error = "non-finite value in the Krylov iteration";
            break;
        }
        rel = std::sqrt(c.os_host->rr) / bnorm;
        est = rel;
        if (achieved > 0.0 && it > 0) {
            double ratio = (rel / prev) / achieved;  // true / preconditioned reduction
            if (ratio < 1.0) ratio = 1.0;
            if (ratio > 1e6) ratio = 1e6;
            if (P.precision == FTS_PREC_MIXED) c.pc_ratio32 = ratio;
            else c.pc_ratio64 = ratio;
        }
        if (it == 0 && rel > tol) {
            status = FTS_ERR_NOT_CONVERGED;
            break;
        }
    }
    FTS_CUDA(cudaEventRecord(c.ev[3], c.stream));
    FTS_CUDA(cudaEventSynchronize(c.ev[3]));
    st.ms_solve = elapsed(c.ev[2], c.ev[3]);
    st.iterations = iters;
    st.iterations_fp32 = iters32;
    st.outer_iterations = outer;
    st.rel_residual = rel;
    st.error_estimate = est;
    if (P.verbose)
        std::printf("  finished after %lld iterations and %.3f ms.\n  Error estimate: %g\n",
                    iters, st.ms_solve, est);
    if (status != FTS_OK) return status;  // flow untouched (Flow.cpp:281-285)
    launch_scatter_flow(c, flow_out);
    st.solved = 1;
    return FTS_OK;
}

}  // namespace fts

using namespace fts;

static thread_local std::string g_create_error;

extern "C" {

void fts_params_default(fts_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->velocity_degree = 1;
    p->alpha = 0.032;
    p->eps = 1e-3;
    p->tol = 1e-4;
    p->max_iter = -1;
    p->mu_interior = 1.0;
    p->mu_exterior = 1.0;
    p->mu_profile = 0;
    p->gf_growth = 1.0;
    p->level_sink = 0.0;
    p->growth_threshold = 0.0;
    p->rd_iterations = 0.0;
    p->gf_production = 1.0;
    p->advection_dt = 1.0;
    p->surface_tension = 0.0;
    p->precision = FTS_PREC_FP64;
    p->solver = FTS_SOLVER_MINRES;
    p->preconditioner = FTS_PC_AUTO;
    p->operator_kind = FTS_OP_AUTO;
    p->warm_start = 1;
    p->device = 0;
    p->inner_tol = 0.0;
    p->verbose = 0;
}

const char* fts_status_string(int s) {
    switch (s) {
        case FTS_OK: return "ok";
        case FTS_ERR_BAD_INPUT: return "bad input";
        case FTS_ERR_DEGENERATE_ELEMENT: return "degenerate element";
        case FTS_ERR_NOT_CONVERGED: return "not converged";
        case FTS_ERR_CUDA: return "CUDA error";
        case FTS_ERR_OOM: return "out of device memory";
        case FTS_ERR_UNSUPPORTED: return "unsupported option";
        case FTS_ERR_NAN: return "non-finite value";
        case FTS_ERR_TIMEOUT: return "grid barrier wait ran out";
        default: return "unknown status";
    }
}

const char* fts_last_error(const fts_ctx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->c.last_error.c_str();
}

int fts_create(const fts_mesh* mesh, const fts_params* params, fts_ctx** out) {
    return fts::create_context(mesh, params, out, false);
}

}  // extern "C"

namespace fts {

int create_context(const fts_mesh* mesh, const fts_params* params, fts_ctx** out, bool in_batch) {
    if (!mesh || !out) {
        g_create_error = "null mesh or output pointer";
        return FTS_ERR_BAD_INPUT;
    }
    *out = nullptr;
    fts_params p;
    if (params) p = *params;
    else fts_params_default(&p);
    std::string err;
    int rc = validate_params(p, err);
    if (rc != FTS_OK) {
        g_create_error = err;
        return rc;
    }
    fts_ctx* h = new (std::nothrow) fts_ctx();
    if (!h) return FTS_ERR_OOM;
    try {
        rc = build_topology(*mesh, h->c.topo, err);
        if (rc != FTS_OK) {
            g_create_error = err;
            delete h;
            return rc;
        }
        if (p.velocity_degree == 2) {
            if (in_batch) {
                g_create_error = "batched solves are P1-P1 only";
                delete h;
                return FTS_ERR_UNSUPPORTED;
            }
            rc = extend_p2(*mesh, h->c.topo, err);
            if (rc != FTS_OK) {
                g_create_error = err;
                delete h;
                return rc;
            }
        }
        h->c.in_batch = in_batch;
        create(h->c, *mesh, p);
    } catch (const CudaError& e) {
        g_create_error = e.what;
        free_all(h->c);
        delete h;
        return e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (int code) {
        g_create_error = h->c.last_error;
        free_all(h->c);
        delete h;
        return code;
    } catch (const std::bad_alloc&) {
        g_create_error = "host allocation failed";
        free_all(h->c);
        delete h;
        return FTS_ERR_OOM;
    }
    *out = h;
    return FTS_OK;
}

}  // namespace fts

extern "C" {

static int solve_common(fts_ctx* ctx, const double* phi, const double* source, const double* mu,
                        const double* force, double* flow, fts_stats* stats, bool device) {
    if (!ctx || !phi || !source || !flow) return FTS_ERR_BAD_INPUT;
    Ctx& c = ctx->c;
    fts_stats st;
    std::memset(&st, 0, sizeof(st));
    double t0 = wall_ms();
    c.launches = 0;
    c.spmv_runs = 0;
    c.ms_spmv = 0.0;
    int rc = FTS_OK;
    try {
        FTS_CUDA(cudaSetDevice(c.device));
        const cudaMemcpyKind k = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        FTS_CUDA(cudaMemcpyAsync(c.phi, phi, c.nv * sizeof(double), k, c.stream));
        FTS_CUDA(cudaMemcpyAsync(c.src, source, c.nv * sizeof(double), k, c.stream));
        if (mu) FTS_CUDA(cudaMemcpyAsync(c.mu, mu, c.nt * sizeof(double), k, c.stream));
        if (force) {
            if (!c.force) c.force = dev_alloc<double>(c, 3 * c.nv);
            FTS_CUDA(cudaMemcpyAsync(c.force, force, 3 * c.nv * sizeof(double), k, c.stream));
        }
        if (c.par.precision == FTS_PREC_FP64) ensure_fp64_work(c);
        double* out = device ? flow : c.flow;
        rc = solve_device(c, mu != nullptr, force != nullptr, out, st);
        if (rc == FTS_OK && st.solved && !device) {
            FTS_CUDA(cudaMemcpyAsync(flow, c.flow, 4 * c.nv * sizeof(double),
                                     cudaMemcpyDeviceToHost, c.stream));
        }
        FTS_CUDA(cudaStreamSynchronize(c.stream));
    } catch (const CudaError& e) {
        c.last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (int code) {
        rc = code;
    } catch (const std::bad_alloc&) {
        c.last_error = "host allocation failed";
        rc = FTS_ERR_OOM;
    }
    st.status = rc;
    st.ms_total = wall_ms() - t0;
    st.device_bytes = c.device_bytes;
    st.kernel_launches = c.launches;
    st.spmv_launches = c.spmv_runs;
    st.ms_spmv = c.ms_spmv;
    {
        // algorithmic bytes of one Krylov operator application (kernel A):
        // blocks + column indices + row pointers + x + r1 read + q written
        const double V = c.par.precision == FTS_PREC_MIXED ? 4.0 : 8.0;
        const double nb = (double)c.nnzb, n = (double)c.np;
        st.spmv_bytes = nb * (16.0 * V + 4.0) + 4.0 * (n + 1.0) + 3.0 * 4.0 * n * V;
        if (c.use_lat && c.par.precision == FTS_PREC_MIXED)  // 8 blocks per node; x, r1, q
            st.spmv_bytes = n * (8.0 * 16.0 * 4.0) + 3.0 * 4.0 * n * 4.0;
        if (c.use_lat64 && c.par.precision == FTS_PREC_FP64)  // the same in FP64
            st.spmv_bytes = n * (8.0 * 16.0 * 8.0) + 3.0 * 4.0 * n * 8.0;
        if (c.matfree)  // tets + node->element map + 64 B record per element; map offsets,
                        // flags, x, r1, q per node
            st.spmv_bytes = (double)c.nt * (16.0 + 16.0 + 64.0) + n * (4.0 + 1.0 + 3.0 * 16.0);
        if (c.matfree && c.topo.kuhn_elements) {  // lattice form: coordinates, flags, x, r1,
                                                  // q per node, FP32 mu per element, and the
                                                  // 32 corner sums per cube written and read
            const double m = (double)(c.topo.lattice_n - 1);
            st.spmv_bytes = (double)c.nt * 4.0 + n * (12.0 + 1.0 + 3.0 * 16.0) + m * m * m * 256.0;
        }
        st.spmv_bytes_fp64 = nb * (16.0 * 8.0 + 4.0) + 4.0 * (n + 1.0) + 3.0 * 4.0 * n * 8.0;
    }
    if (stats) *stats = st;
    return rc;
}

int fts_solve(fts_ctx* ctx, const double* phi, const double* source, const double* mu,
              const double* force, double* flow, fts_stats* stats) {
    return solve_common(ctx, phi, source, mu, force, flow, stats, false);
}

int fts_solve_device(fts_ctx* ctx, const double* phi, const double* source, const double* mu,
                     const double* force, double* flow, fts_stats* stats) {
    return solve_common(ctx, phi, source, mu, force, flow, stats, true);
}

int fts_set_stream(fts_ctx* ctx, void* stream) {
    if (!ctx) return FTS_ERR_BAD_INPUT;
    ctx->c.stream = stream ? static_cast<cudaStream_t>(stream) : ctx->c.own_stream;
    return FTS_OK;
}

int fts_update_params(fts_ctx* ctx, const fts_params* params) {
    if (!ctx || !params) return FTS_ERR_BAD_INPUT;
    std::string err;
    int rc = validate_params(*params, err);
    if (rc != FTS_OK) {
        ctx->c.last_error = err;
        return rc;
    }
    if (params->device != ctx->c.device) {
        ctx->c.last_error = "the device of a context cannot change";
        return FTS_ERR_BAD_INPUT;
    }
    if (params->velocity_degree != ctx->c.par.velocity_degree) {
        ctx->c.last_error = "the velocity degree of a context cannot change";
        return FTS_ERR_BAD_INPUT;
    }
    const fts_params old = ctx->c.par;
    ctx->c.par = *params;
    try {
        configure_preconditioner(ctx->c);
    } catch (int code) {
        ctx->c.par = old;
        configure_preconditioner(ctx->c);
        return code;
    }
    return FTS_OK;
}

int fts_reset_guess(fts_ctx* ctx) {
    if (!ctx) return FTS_ERR_BAD_INPUT;
    try {
        FTS_CUDA(cudaSetDevice(ctx->c.device));
        FTS_CUDA(cudaMemsetAsync(ctx->c.x, 0, ctx->c.np * sizeof(V4<double>), ctx->c.stream));
        FTS_CUDA(cudaStreamSynchronize(ctx->c.stream));
    } catch (const CudaError& e) {
        ctx->c.last_error = e.what;
        return FTS_ERR_CUDA;
    }
    return FTS_OK;
}

void fts_destroy(fts_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->c.device);
    if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
    free_all(ctx->c);
    delete ctx;
}

int fts_get_sizes(const fts_ctx* ctx, int64_t* np, int64_t* nnzb, int64_t* n_reduced) {
    if (!ctx) return FTS_ERR_BAD_INPUT;
    if (np) *np = ctx->c.np;
    if (nnzb) *nnzb = ctx->c.nnzb;
    if (n_reduced) *n_reduced = 3 * ctx->c.topo.n_interior + ctx->c.nv;
    return FTS_OK;
}

int fts_get_system(const fts_ctx* ctx, int32_t* rowptr, int32_t* cols, double* vals, double* rhs) {
    if (!ctx) return FTS_ERR_BAD_INPUT;
    const Ctx& c = ctx->c;
    if (c.matfree) return FTS_ERR_UNSUPPORTED;
    try {
        FTS_CUDA(cudaSetDevice(c.device));
        if (vals) ensure_bsr64(const_cast<Ctx&>(c));
        FTS_CUDA(cudaStreamSynchronize(c.stream));
        if (rowptr) std::memcpy(rowptr, c.topo.rowptr.data(), (c.np + 1) * sizeof(int32_t));
        if (cols) std::memcpy(cols, c.topo.cols.data(), c.nnzb * sizeof(int32_t));
        if (vals)
            FTS_CUDA(cudaMemcpy(vals, c.A64, c.nnzb * 16 * sizeof(double), cudaMemcpyDeviceToHost));
        if (rhs) FTS_CUDA(cudaMemcpy(rhs, c.b, c.np * 4 * sizeof(double), cudaMemcpyDeviceToHost));
    } catch (const CudaError& e) {
        const_cast<Ctx&>(c).last_error = e.what;
        return FTS_ERR_CUDA;
    }
    return FTS_OK;
}

int fts_apply(fts_ctx* ctx, int32_t precision, const double* x, double* y) {
    if (!ctx || !x || !y) return FTS_ERR_BAD_INPUT;
    Ctx& c = ctx->c;
    if (c.matfree) return FTS_ERR_UNSUPPORTED;
    try {
        FTS_CUDA(cudaSetDevice(c.device));
        if (precision == FTS_PREC_MIXED && !c.have32) {
            c.last_error = "no FP32 operator assembled";
            return FTS_ERR_BAD_INPUT;
        }
        if (precision != FTS_PREC_MIXED) ensure_bsr64(c);
        FTS_CUDA(cudaMemcpyAsync(c.r, x, c.np * 4 * sizeof(double), cudaMemcpyHostToDevice,
                                 c.stream));
        V4<double>* out = reinterpret_cast<V4<double>*>(c.flow);  // 4*np doubles of scratch
        launch_apply(c, precision, c.r, out);
        FTS_CUDA(cudaMemcpyAsync(y, out, c.np * 4 * sizeof(double), cudaMemcpyDeviceToHost,
                                 c.stream));
        FTS_CUDA(cudaStreamSynchronize(c.stream));
    } catch (const CudaError& e) {
        c.last_error = e.what;
        return FTS_ERR_CUDA;
    }
    return FTS_OK;
}

}  // extern "C"
