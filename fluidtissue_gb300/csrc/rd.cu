// Reaction-diffusion (RD::solve, src/growth/RD.cpp:27-108, :116-172) on one
// GPU: the interior submesh's lumped-mass Laplacian L = diag(1/rowsum M) K is
// assembled by a node-row gather (atomic-free, FP64, the same element
// integrals as the reference's Assembler), then all explicit Euler steps run in
// ONE persistent cooperative launch over the compacted interior nodes, with a
// grid barrier per step (bounded spin, grid_sync.cuh).  The three fields share
// one pass over L per step.  At the benchmark sizes the interior system
// (L + 6 vectors) fits in L2, so a step costs its FP64 arithmetic plus one
// barrier.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fts_device.cuh"
#include "grid_sync.cuh"

namespace fts {

static std::string& g_rd_error() {
    static thread_local std::string e;
    return e;
}

// Element mass factors mq[a][b] = sum_q qw phi_b(q) phi_a(q) with the
// reference's pairwise order ((q0 + q2) + (q1 + q3)); M_e(a,b) = mq[a][b] detB.
struct RdConst {
    double mq[4][4];
    double qw;
};

static RdConst rd_const() {
    const RefConstants R = ref_constants();
    RdConst c;
    c.qw = 0.25 / 6.0;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
            double f[4];
            for (int q = 0; q < 4; ++q) f[q] = R.phi[b][q] * R.phi[a][q];
            c.mq[a][b] = (f[0] * c.qw + f[2] * c.qw) + (f[1] * c.qw + f[3] * c.qw);
        }
    return c;
}

struct RdStep {
    double dt, act, da, dega, inh, di, degi, gprod, gdiff, gdeg, ginh;
    int alive;
};

// One thread per interior node i: row i of K and rowsum M over the interior
// elements around i (all four nodes phi < 0), L(i, j) = K(i, j) / rowsum, in
// the slots of the mesh's node graph.  A row with no interior element stays 0.
__global__ void k_rd_laplacian(int64_t nint, const int32_t* __restrict__ list,
                               const int32_t* __restrict__ rowptr,
                               const int32_t* __restrict__ cols,
                               const int32_t* __restrict__ p2t_ptr,
                               const uint32_t* __restrict__ p2t,
                               const int32_t* __restrict__ tets, const float* __restrict__ xyz,
                               const double* __restrict__ phi, RdConst R,
                               double* __restrict__ lval, int* __restrict__ bad,
                               unsigned long long* __restrict__ nel) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nint;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = list[t];
        const int32_t r0 = rowptr[i], r1 = rowptr[i + 1];
        for (int32_t q = r0; q < r1; ++q) lval[q] = 0.0;
        double msum = 0.0;
        for (int32_t e = p2t_ptr[i]; e < p2t_ptr[i + 1]; ++e) {
            const uint32_t pe = p2t[e];
            const int64_t k = pe >> 2;
            const int a = pe & 3;
            const int4 tt = reinterpret_cast<const int4*>(tets)[k];
            const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
            if (!(phi[ids[0]] < 0.0 && phi[ids[1]] < 0.0 && phi[ids[2]] < 0.0 &&
                  phi[ids[3]] < 0.0))
                continue;
            if (a == 0) atomicAdd(nel, 1ull);  // each interior element once
            double p[4][3];
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int c = 0; c < 3; ++c) p[j][c] = (double)xyz[3 * (int64_t)ids[j] + c];
            double B[3][3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                B[c][0] = p[1][c] - p[0][c];
                B[c][1] = p[2][c] - p[0][c];
                B[c][2] = p[3][c] - p[0][c];
            }
            const double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1];
            const double c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2];
            const double c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
            const double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
            const double detB = fabs(det);
            if (!(detB > 0.0)) {
                atomicOr(bad, 1);
                continue;
            }
            double cof[3][3];
            cof[0][0] = c00;
            cof[0][1] = c01;
            cof[0][2] = c02;
            cof[1][0] = B[0][2] * B[2][1] - B[0][1] * B[2][2];
            cof[1][1] = B[0][0] * B[2][2] - B[0][2] * B[2][0];
            cof[1][2] = B[0][1] * B[2][0] - B[0][0] * B[2][1];
            cof[2][0] = B[0][1] * B[1][2] - B[0][2] * B[1][1];
            cof[2][1] = B[0][2] * B[1][0] - B[0][0] * B[1][2];
            cof[2][2] = B[0][0] * B[1][1] - B[0][1] * B[1][0];
            double g[4][3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const double it0 = cof[r][0] / det, it1 = cof[r][1] / det, it2 = cof[r][2] / det;
                g[0][r] = -it0 - it1 - it2;
                g[1][r] = it0;
                g[2][r] = it1;
                g[3][r] = it2;
            }
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                // K: ux.*vx + uy.*vy + uz.*vz (trial b, test a), constant over the points
                const double gg = g[b][0] * g[a][0] + g[b][1] * g[a][1] + g[b][2] * g[a][2];
                const double tq = gg * R.qw;
                const double kv = ((tq + tq) + (tq + tq)) * detB;
                msum += R.mq[a][b] * detB;
                int32_t slot = r0;
                while (slot < r1 && cols[slot] != ids[b]) ++slot;
                if (slot < r1) lval[slot] += kv;
            }
        }
        if (msum != 0.0)
            for (int32_t q = r0; q < r1; ++q) lval[q] = lval[q] / msum;
    }
}

// State in: full vectors -> device ping buffer (non-interior entries zero, so
// that 0 * value never meets a NaN), sources flagged.
__global__ void k_rd_load(int64_t np, const double* __restrict__ phi,
                          const double* __restrict__ a_in, const double* __restrict__ i_in,
                          const double* __restrict__ g_in, double* __restrict__ u,
                          double* __restrict__ v, double* __restrict__ g) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bool in = phi[i] < 0.0;
        u[i] = in ? a_in[i] : 0.0;
        v[i] = in ? i_in[i] : 0.0;
        g[i] = in ? g_in[i] : 0.0;
    }
}

__global__ void k_rd_sources(int32_t n, const int32_t* __restrict__ src, double gprod,
                             uint8_t* __restrict__ flag, double* __restrict__ g0,
                             double* __restrict__ g1) {
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        flag[src[s]] = 1;
        g0[src[s]] = gprod;
        g1[src[s]] = gprod;
    }
}

// All Euler steps.  Buffers (u, v, g)[0] hold the state; step s reads buffer
// s % 2 and writes the other.  Non-interior entries stay zero in both.
__global__ void __launch_bounds__(256)
k_rd_steps(int64_t nint, const int32_t* __restrict__ list, const int32_t* __restrict__ rowptr,
           const int32_t* __restrict__ cols, const double* __restrict__ lval,
           const uint8_t* __restrict__ srcflag, double* u0, double* v0, double* g0, double* u1,
           double* v1, double* g1, RdStep P, long long steps, BarrierState* bar) {
    for (long long s = 0; s < steps; ++s) {
        const double* u = (s & 1) ? u1 : u0;
        const double* v = (s & 1) ? v1 : v0;
        const double* g = (s & 1) ? g1 : g0;
        double* un = (s & 1) ? u0 : u1;
        double* vn = (s & 1) ? v0 : v1;
        double* gn = (s & 1) ? g0 : g1;
        for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nint;
             t += (int64_t)gridDim.x * blockDim.x) {
            const int32_t i = __ldg(list + t);
            double lu = 0.0, lv = 0.0, lg = 0.0;
            const int32_t r1 = __ldg(rowptr + i + 1);
            for (int32_t q = __ldg(rowptr + i); q < r1; ++q) {
                const double l = __ldg(lval + q);
                const int32_t j = __ldg(cols + q);
                lu = fma(l, u[j], lu);
                lv = fma(l, v[j], lv);
                lg = fma(l, g[j], lg);
            }
            const double ui = u[i], vi = v[i], gi = g[i];
            if (P.alive) {
                const double u2 = ui * ui;
                const double de = 1.0 + P.inh * vi + P.ginh * gi;
                un[i] = ui + P.dt * (-P.da * lu + P.act * (u2 / de) - P.dega * ui);
                vn[i] = vi + P.dt * (-P.di * lv + u2 - P.degi * vi);
            } else {
                un[i] = ui;
                vn[i] = vi;
            }
            gn[i] = srcflag[i] ? P.gprod : gi + P.dt * (-P.gdiff * lg - P.gdeg * gi);
        }
        if (!grid_barrier(bar)) return;
    }
}

}  // namespace fts

using namespace fts;

struct fts_rd {
    int device = 0;
    int num_sms = 148;
    cudaStream_t stream = nullptr;
    HostTopology topo;
    int64_t np = 0, nt = 0;
    float* xyz = nullptr;
    int32_t* tets = nullptr;
    int32_t* rowptr = nullptr;
    int32_t* cols = nullptr;
    int32_t* p2t_ptr = nullptr;
    uint32_t* p2t = nullptr;
    double* lval = nullptr;
    double* phi = nullptr;
    double* in[3] = {nullptr, nullptr, nullptr};
    double* buf[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint8_t* srcflag = nullptr;
    int32_t* list = nullptr;
    int32_t* src = nullptr;
    int32_t src_cap = 0;
    int* bad = nullptr;
    unsigned long long* nel = nullptr;
    BarrierState* bar = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::string last_error;
    int64_t device_bytes = 0;
};

namespace {

template <typename T>
T* rd_alloc(fts_rd& R, size_t n) {
    void* p = nullptr;
    FTS_CUDA(cudaMalloc(&p, n * sizeof(T) + 16));
    R.device_bytes += (int64_t)(n * sizeof(T));
    return static_cast<T*>(p);
}

void rd_free(fts_rd& R) {
    void* ptrs[] = {R.xyz,    R.tets,   R.rowptr, R.cols,   R.p2t_ptr, R.p2t,   R.lval,
                    R.phi,    R.in[0],  R.in[1],  R.in[2],  R.buf[0],  R.buf[1], R.buf[2],
                    R.buf[3], R.buf[4], R.buf[5], R.srcflag, R.list,   R.src,   R.bad,
                    R.nel,    R.bar};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto& e : R.ev)
        if (e) cudaEventDestroy(e);
    if (R.stream) cudaStreamDestroy(R.stream);
}

int grid_of(const fts_rd& R, int64_t work, int per_sm = 8) {
    const int64_t need = std::max<int64_t>(1, (work + 255) / 256);
    return (int)std::min<int64_t>(need, (int64_t)R.num_sms * per_sm);
}

}  // namespace

extern "C" {

int fts_rd_create(const fts_mesh* mesh, int32_t device, fts_rd** out) {
    if (!mesh || !out) return FTS_ERR_BAD_INPUT;
    *out = nullptr;
    fts_rd* R = new (std::nothrow) fts_rd();
    if (!R) return FTS_ERR_OOM;
    R->device = device;
    int rc = FTS_OK;
    try {
        std::string err;
        rc = build_topology(*mesh, R->topo, err);
        if (rc != FTS_OK) throw err;
        FTS_CUDA(cudaSetDevice(device));
        int sms = 0;
        FTS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        R->num_sms = sms > 0 ? sms : 148;
        FTS_CUDA(cudaStreamCreateWithFlags(&R->stream, cudaStreamNonBlocking));
        for (auto& e : R->ev) FTS_CUDA(cudaEventCreate(&e));
        const HostTopology& T = R->topo;
        R->np = T.np;
        R->nt = T.nt;
        const int64_t nnz = T.rowptr[T.np];
        R->xyz = rd_alloc<float>(*R, 3 * R->np);
        R->tets = rd_alloc<int32_t>(*R, 4 * R->nt);
        R->rowptr = rd_alloc<int32_t>(*R, R->np + 1);
        R->cols = rd_alloc<int32_t>(*R, nnz);
        R->p2t_ptr = rd_alloc<int32_t>(*R, R->np + 1);
        R->p2t = rd_alloc<uint32_t>(*R, 4 * R->nt);
        R->lval = rd_alloc<double>(*R, nnz);
        R->phi = rd_alloc<double>(*R, R->np);
        for (auto& p : R->in) p = rd_alloc<double>(*R, R->np);
        for (auto& p : R->buf) p = rd_alloc<double>(*R, R->np);
        R->srcflag = rd_alloc<uint8_t>(*R, R->np);
        R->list = rd_alloc<int32_t>(*R, R->np);
        R->bad = rd_alloc<int>(*R, 1);
        R->nel = rd_alloc<unsigned long long>(*R, 1);
        R->bar = rd_alloc<BarrierState>(*R, 1);
        {
            const BarrierState cfg = barrier_config(kDefaultBarrierLimitNs, -1);
            FTS_CUDA(cudaMemcpy(R->bar, &cfg, sizeof(cfg), cudaMemcpyHostToDevice));
        }
        FTS_CUDA(cudaMemcpy(R->xyz, mesh->xyz, 3 * R->np * sizeof(float), cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(R->tets, mesh->tets, 4 * R->nt * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(R->rowptr, T.rowptr.data(), (R->np + 1) * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(R->cols, T.cols.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(R->p2t_ptr, T.p2t_ptr.data(), (R->np + 1) * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(R->p2t, T.p2t.data(), 4 * R->nt * sizeof(uint32_t),
                            cudaMemcpyHostToDevice));
    } catch (const std::string& e) {
        g_rd_error() = e;
    } catch (const CudaError& e) {
        g_rd_error() = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        g_rd_error() = "host allocation failed";
        rc = FTS_ERR_OOM;
    }
    if (rc != FTS_OK) {
        rd_free(*R);
        delete R;
        return rc;
    }
    *out = R;
    return FTS_OK;
}

int fts_rd_solve(fts_rd* R, const fts_rd_params* P, const double* phi,
                 const int32_t* source_nodes, int32_t n_sources, double* activator,
                 double* inhibitor, double* growth_factor, fts_rd_stats* stats) {
    if (!R || !P || !phi || !activator || !inhibitor || !growth_factor ||
        (n_sources > 0 && !source_nodes) || n_sources < 0)
        return FTS_ERR_BAD_INPUT;
    const double t0 = wall_ms();
    fts_rd_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = FTS_OK;
    try {
        if (P->iterations == 0 || P->dt < FLT_MIN) {  // RD.cpp:31-33
            if (stats) {
                *stats = st;
                stats->ms_total = wall_ms() - t0;
            }
            return FTS_OK;
        }
        if (P->iterations < 0) {
            R->last_error = "negative iteration count";
            return FTS_ERR_BAD_INPUT;
        }
        const int64_t np = R->np;
        // interior nodes (ascending) and the sources' validity, on the host
        std::vector<int32_t> list;
        list.reserve(np);
        for (int64_t i = 0; i < np; ++i)
            if (phi[i] < 0.0) list.push_back((int32_t)i);
        for (int32_t s = 0; s < n_sources; ++s)
            if (source_nodes[s] < 0 || source_nodes[s] >= np || !(phi[source_nodes[s]] < 0.0)) {
                R->last_error = "growth-factor source " + std::to_string(source_nodes[s]) +
                                " is not an interior node";
                return FTS_ERR_BAD_INPUT;
            }
        bool alive = false;
        for (int64_t i = 0; i < np && !alive; ++i)
            alive = std::fabs(activator[i]) >= FLT_MIN || std::fabs(inhibitor[i]) >= FLT_MIN;
        const int64_t nint = (int64_t)list.size();
        FTS_CUDA(cudaSetDevice(R->device));
        cudaStream_t s = R->stream;
        int launches = 0;
        FTS_CUDA(cudaMemcpyAsync(R->phi, phi, np * sizeof(double), cudaMemcpyHostToDevice, s));
        FTS_CUDA(cudaMemcpyAsync(R->in[0], activator, np * sizeof(double), cudaMemcpyHostToDevice, s));
        FTS_CUDA(cudaMemcpyAsync(R->in[1], inhibitor, np * sizeof(double), cudaMemcpyHostToDevice, s));
        FTS_CUDA(cudaMemcpyAsync(R->in[2], growth_factor, np * sizeof(double),
                                 cudaMemcpyHostToDevice, s));
        if (nint > 0)
            FTS_CUDA(cudaMemcpyAsync(R->list, list.data(), nint * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
        if (n_sources > R->src_cap) {
            if (R->src) cudaFree(R->src);
            R->src = nullptr;
            R->src = rd_alloc<int32_t>(*R, n_sources);
            R->src_cap = n_sources;
        }
        if (n_sources > 0)
            FTS_CUDA(cudaMemcpyAsync(R->src, source_nodes, n_sources * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
        FTS_CUDA(cudaMemsetAsync(R->bad, 0, sizeof(int), s));
        FTS_CUDA(cudaMemsetAsync(R->nel, 0, sizeof(unsigned long long), s));
        FTS_CUDA(cudaMemsetAsync(R->srcflag, 0, np, s));
        FTS_CUDA(cudaMemsetAsync(R->bar, 0, kBarrierResetBytes, s));
        FTS_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(R->bar) + kBarrierErrorOffset, 0,
                                 sizeof(int), s));
        static const RdConst K = rd_const();
        if (nint > 0) {
            k_rd_laplacian<<<grid_of(*R, nint), 256, 0, s>>>(nint, R->list, R->rowptr, R->cols,
                                                             R->p2t_ptr, R->p2t, R->tets, R->xyz,
                                                             R->phi, K, R->lval, R->bad, R->nel);
            ++launches;
        }
        double* u0 = R->buf[0];
        double* v0 = R->buf[1];
        double* g0 = R->buf[2];
        double* u1 = R->buf[3];
        double* v1 = R->buf[4];
        double* g1 = R->buf[5];
        k_rd_load<<<grid_of(*R, np), 256, 0, s>>>(np, R->phi, R->in[0], R->in[1], R->in[2], u0,
                                                   v0, g0);
        // the second buffer's non-interior entries must be zero as well
        k_rd_load<<<grid_of(*R, np), 256, 0, s>>>(np, R->phi, R->in[0], R->in[1], R->in[2], u1,
                                                   v1, g1);
        launches += 2;
        if (n_sources > 0) {
            k_rd_sources<<<std::max(1, std::min(R->num_sms, (n_sources + 255) / 256)), 256, 0, s>>>(
                n_sources, R->src, P->gf_production, R->srcflag, g0, g1);
            ++launches;
        }
        int bad = 0;
        unsigned long long nel = 0;
        FTS_CUDA(cudaMemcpyAsync(&bad, R->bad, sizeof(int), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(&nel, R->nel, sizeof(nel), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        if (bad) {
            R->last_error = "degenerate tetrahedron (det B == 0) in the interior submesh";
            return FTS_ERR_DEGENERATE_ELEMENT;
        }
        const double t_setup = wall_ms() - t0;
        RdStep S{P->dt, P->act, P->da, P->dega, P->inh, P->di, P->degi, P->gf_production,
                 P->gf_diffusion, P->gf_degradation, P->gf_inhibition, alive ? 1 : 0};
        long long steps = (long long)P->iterations;
        int per_sm = 0;
        FTS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rd_steps, 256, 0));
        const int blocks = (int)std::max<int64_t>(
            1, std::min<int64_t>((int64_t)std::max(per_sm, 1) * R->num_sms, (nint + 255) / 256));
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3((unsigned)blocks);
        lc.blockDim = dim3(256);
        lc.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        FTS_CUDA(cudaEventRecord(R->ev[0], s));
        if (nint == 0) steps = 0;  // nothing interior: every field is zero
        if (steps > 0)
        FTS_CUDA(cudaLaunchKernelEx(&lc, k_rd_steps, nint, (const int32_t*)R->list,
                                    (const int32_t*)R->rowptr, (const int32_t*)R->cols,
                                    (const double*)R->lval, (const uint8_t*)R->srcflag, u0, v0, g0,
                                    u1, v1, g1, S, steps, R->bar));
        FTS_CUDA(cudaEventRecord(R->ev[1], s));
        ++launches;
        const int fin = (int)(steps & 1);  // buffer holding the result
        BarrierState bs;
        FTS_CUDA(cudaMemcpyAsync(&bs, R->bar, sizeof(bs), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(activator, R->buf[3 * fin], np * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(inhibitor, R->buf[3 * fin + 1], np * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(growth_factor, R->buf[3 * fin + 2], np * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        if (bs.error) {
            R->last_error = "grid barrier timed out in the Euler steps";
            rc = FTS_ERR_TIMEOUT;
        }
        float ms = 0.f;
        FTS_CUDA(cudaEventElapsedTime(&ms, R->ev[0], R->ev[1]));
        st.status = rc;
        st.alive = alive ? 1 : 0;
        st.interior_nodes = nint;
        st.interior_elements = (int64_t)nel;
        st.steps = steps;
        st.ms_setup = t_setup;
        st.ms_steps = ms;
        st.kernel_launches = launches;
    } catch (const CudaError& e) {
        R->last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
        st.status = rc;
    } catch (const std::bad_alloc&) {
        R->last_error = "host allocation failed";
        rc = FTS_ERR_OOM;
        st.status = rc;
    }
    st.ms_total = wall_ms() - t0;
    if (stats) *stats = st;
    return rc;
}

void fts_rd_destroy(fts_rd* R) {
    if (!R) return;
    cudaSetDevice(R->device);
    if (R->stream) cudaStreamSynchronize(R->stream);
    rd_free(*R);
    delete R;
}

const char* fts_rd_last_error(const fts_rd* R) {
    return R ? R->last_error.c_str() : g_rd_error().c_str();
}

}  // extern "C"
