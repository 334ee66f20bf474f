// Batched Stokes solves: many independent systems (uneven mesh sizes, their
// own viscosities and parameters) solved together.  Each instance is assembled
// by the single-solve kernels into its own context; the Krylov iteration of all
// instances then runs in ONE persistent cooperative launch: MINRES over a
// global list of row chunks, with a grid barrier between phases, per-instance
// reductions finished in a fixed order, and per-instance stop flags (converged
// instances drop out of the work).  The velocity preconditioner of an instance
// is the multigrid V-cycle where its mesh is a Kuhn lattice (all instances'
// levels of the same depth are smoothed in one phase, over per-depth chunk
// lists; each coarsest level is solved by one CTA), else 3x3 block Jacobi; the
// pressure block is the diagonal + rank-one term of the single solve.
// The FP64 outer loop (true residual, solution update) runs per instance
// between persistent launches; the whole sequence is captured as a CUDA graph
// and replayed.  An autotuner picks the block size, the chunk length and the
// number of threads per block row (the work split of the SpMV) and, in mixed
// precision, the SpMV's operator storage: the FP32 block rows (BSR), or the
// FP32 lattice half stencil (thread per node, no column indices) on instances
// whose mesh is a Kuhn lattice.
//
// Grid barrier (grid_sync.cuh): every wait has a time limit (a runtime field,
// fts_batch_set_barrier_limit, 2 s by default) after which the kernel records
// an error and returns (no unbounded wait); the solve then reports
// FTS_ERR_TIMEOUT.  With the cooperative launch all blocks are co-resident.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fts_device.cuh"
#include "grid_sync.cuh"
#include "lat_device.cuh"
#include "mg_device.cuh"
#include "reduce.cuh"

namespace fts {

constexpr int kMaxLevels = 10;  // multigrid levels per instance (n <= 513)

static std::string& g_batch_error() {
    static thread_local std::string e;
    return e;
}

template <typename T>
struct BInst {
    int64_t np;
    const int32_t* rowptr;
    const int32_t* cols;
    const T* A;
    const T* pc;
    V4<T>* q;
    V4<T>* R[2];
    V4<T>* Y[2];
    V4<T>* W[2];
    V4<T>* X;
    const V4<T>* r0;
    MinresScalars* s;
    int chunk0, chunk1;  // this instance's range in the chunk list
    int skip;            // 1: not solved in this launch (converged or early exit)
    double rtol;
    long long maxit;
    double crank;
    int use_mg;          // multigrid velocity preconditioner (else block Jacobi)
    int nlev;            // multigrid levels
    const float4* lat;   // FP32 lattice half stencil used by the SpMV phase (else BSR)
    int lat_n;           // its lattice size
    LevelView<T> lv[kMaxLevels];
};

// Rows [row0, row1) of level `depth` of instance `inst` (depth 0: the system's
// block rows).
struct BChunk {
    int inst;
    int row0, row1;
    int depth;
};

// Multigrid schedule of the persistent kernel.
struct BSched {
    const int* cptr;    // chunks of depth d are [cptr[d], cptr[d + 1])
    int max_depth;      // deepest non-coarsest level + 1 over all instances (0: no multigrid)
    const int* coarse;  // instances with multigrid (one coarsest-level solve each)
    int ncoarse;
};

template <typename T>
__device__ __forceinline__ void pc_jacobi_b(const T* __restrict__ pc, int64_t i, const V4<T>& v,
                                            V4<T>& z) {
    const V4<T> p0 = *reinterpret_cast<const V4<T>*>(pc + 8 * i);
    const V4<T> p1 = *reinterpret_cast<const V4<T>*>(pc + 8 * i + 4);
    z.x = p0.x * v.x + p0.y * v.y + p0.z * v.z;
    z.y = p0.y * v.x + p0.w * v.y + p1.x * v.z;
    z.z = p0.z * v.x + p1.x * v.y + p1.y * v.z;
    z.w = p1.z * v.w;
}

__device__ void finalize_beta_b(MinresScalars* s, double beta2, bool init) {
    const bool finite = isfinite(beta2);
    const double beta = beta2 > 0.0 ? sqrt(beta2) : 0.0;
    if (init) {
        s->beta1 = beta;
        s->beta = beta;
        s->oldb = 0.0;
        s->alfa = 0.0;
        s->dbar = 0.0;
        s->epsln = 0.0;
        s->oldeps = 0.0;
        s->delta = 0.0;
        s->gamma = 1.0;
        s->phi = 0.0;
        s->phibar = beta;
        s->cs = -1.0;
        s->sn = 0.0;
        s->target = s->rtol * beta;
        s->status = finite ? 0 : 2;
        s->stop = (!(beta > 0.0) || !finite) ? 1 : 0;
        return;
    }
    const double alfa = s->alfa;
    s->oldb = s->beta;
    s->beta = beta;
    s->oldeps = s->epsln;
    const double delta = s->cs * s->dbar + s->sn * alfa;
    const double gbar = s->sn * s->dbar - s->cs * alfa;
    s->epsln = s->sn * beta;
    s->dbar = -s->cs * beta;
    double gamma = sqrt(gbar * gbar + beta * beta);
    if (gamma < DBL_MIN) gamma = DBL_MIN;
    s->delta = delta;
    s->gamma = gamma;
    s->cs = gbar / gamma;
    s->sn = beta / gamma;
    s->phi = s->cs * s->phibar;
    s->phibar = s->sn * s->phibar;
    s->iters += 1;
    s->c_pending = 1;
    if (!finite || !isfinite(s->phibar)) {
        s->status = 2;
        s->stop = 1;
    } else if (s->phibar <= s->target || !(beta > 0.0)) {
        s->stop = 1;
    } else if (s->iters >= s->maxit) {
        s->status = 1;
        s->stop = 1;
    }
}

// Block sum of NV values, result in thread 0 (all threads must call).
template <int NV>
__device__ __forceinline__ void bsum(double (&v)[NV]) {
    block_sum<NV>(v);
}

// Smoothing-type phase over the depth-d chunks: nodes of level d of every
// active multigrid instance for which level d is not the coarsest.
template <typename T, typename F>
__device__ __forceinline__ void level_phase(const BInst<T>* __restrict__ inst,
                                            const BChunk* __restrict__ chunks, const BSched& S,
                                            int d, F f) {
    for (int ch = S.cptr[d] + blockIdx.x; ch < S.cptr[d + 1]; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        const BInst<T>& I = inst[C.inst];
        if (!I.use_mg || I.s->stop || d + 1 >= I.nlev) continue;
        const LevelView<T> L = I.lv[d];
        for (int64_t v = C.row0 + threadIdx.x; v < C.row1; v += blockDim.x) f(I, L, v);
    }
}

// One V-cycle of every active multigrid instance, level by level across the
// batch; the last post-smoothing step of the finest level is left to the
// caller (fused with preconditioner stage 2).  Returns false when a barrier
// failed.
template <typename T>
__device__ bool batch_vcycle(const BInst<T>* __restrict__ inst, const BChunk* __restrict__ chunks,
                             const BSched& S, BarrierState* bar) {
    const int D = S.max_depth;
    for (int d = 0; d < D; ++d) {
        for (int s = 1; s < kSmooth; ++s) {
            const int mode = s == 1 ? kStepFromZero : kStepRegular;
            level_phase<T>(inst, chunks, S, d, [&](const BInst<T>&, const LevelView<T>& L, int64_t v) {
                T xo[3];
                mg_step_node<T, kSkChecked>(L, v, s, mode, (s & 1) ? L.d0 : L.d1,
                                            (s & 1) ? L.d1 : L.d0, xo, true, true);
            });
            if (!grid_barrier(bar)) return false;
        }
        level_phase<T>(inst, chunks, S, d, [&](const BInst<T>&, const LevelView<T>& L, int64_t v) {
            mg_resid_node<T, kSkChecked>(L, v);
        });
        if (!grid_barrier(bar)) return false;
        // restriction onto level d + 1 (which may be an instance's coarsest)
        for (int ch = S.cptr[d + 1] + blockIdx.x; ch < S.cptr[d + 2]; ch += gridDim.x) {
            const BChunk C = chunks[ch];
            const BInst<T>& I = inst[C.inst];
            if (!I.use_mg || I.s->stop || d + 1 >= I.nlev) continue;
            const LevelView<T> F = I.lv[d], Cv = I.lv[d + 1];
            for (int64_t v = C.row0 + threadIdx.x; v < C.row1; v += blockDim.x)
                mg_restrict_node<T>(F, Cv, v);
        }
        if (!grid_barrier(bar)) return false;
    }
    // coarsest levels: one CTA per instance
    for (int k = blockIdx.x; k < S.ncoarse; k += gridDim.x) {
        const BInst<T>& I = inst[S.coarse[k]];
        if (I.s->stop) continue;
        const LevelView<T> L = I.lv[I.nlev - 1];
        mg_coarse_block<T, kSkChecked>(L, L.n == 3 ? 1 : kCoarse);
    }
    if (!grid_barrier(bar)) return false;
    for (int d = D - 1; d >= 0; --d) {
        level_phase<T>(inst, chunks, S, d, [&](const BInst<T>& I, const LevelView<T>& L, int64_t v) {
            mg_prolong_node<T>(L, I.lv[d + 1], v);
        });
        if (!grid_barrier(bar)) return false;
        level_phase<T>(inst, chunks, S, d, [&](const BInst<T>&, const LevelView<T>& L, int64_t v) {
            mg_resid_first_node<T, kSkChecked>(L, v);
        });
        if (!grid_barrier(bar)) return false;
        const int last = d == 0 ? kSmooth - 2 : kSmooth - 1;
        for (int s = 1; s <= last; ++s) {
            const int mode = s == 1 ? kStepAfterFirst : kStepRegular;
            level_phase<T>(inst, chunks, S, d, [&](const BInst<T>&, const LevelView<T>& L, int64_t v) {
                T xo[3];
                mg_step_node<T, kSkChecked>(L, v, s, mode, (s & 1) ? L.d0 : L.d1,
                                            (s & 1) ? L.d1 : L.d0, xo, true, true);
            });
            if (!grid_barrier(bar)) return false;
        }
    }
    return true;
}

// Multigrid preconditioner stage 2 over the row chunks: the finest level's
// last post-smoothing step gives y.xyz (into Yn); partial n.xyz . y.xyz.
template <typename T>
__device__ void batch_pc2(const BInst<T>* __restrict__ inst, int nchunks,
                          const BChunk* __restrict__ chunks, int rn, int yn,
                          double* __restrict__ part) {
    constexpr int s = kSmooth - 1;
    const int mode = s == 1 ? kStepAfterFirst : kStepRegular;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        const BInst<T>& I = inst[C.inst];
        if (!I.use_mg || I.s->stop) continue;
        const LevelView<T> L = I.lv[0];
        const V4<T>* Rn = I.R[rn];
        V4<T>* Yn = I.Y[yn];
        double acc[1] = {0.0};
        for (int64_t i = C.row0 + threadIdx.x; i < C.row1; i += blockDim.x) {
            T xo[3];
            mg_step_node<T, kSkChecked>(L, i, s, mode, (s & 1) ? L.d0 : L.d1, nullptr, xo, false,
                                        false);
            const V4<T> n = Rn[i];
            V4<T> z = Yn[i];
            z.x = xo[0];
            z.y = xo[1];
            z.z = xo[2];
            Yn[i] = z;
            acc[0] += (double)(n.x * z.x + n.y * z.y + n.z * z.z);
        }
        block_sum<1>(acc);
        if (threadIdx.x == 0) part[(int64_t)ch * 3 + 2] = acc[0];
    }
}

// Preconditioner stage 1 at row i: y.w from the pressure weight; Jacobi gives
// y.xyz, multigrid takes n.xyz as the finest right-hand side (y.xyz follows
// in stage 2).
template <typename T>
__device__ __forceinline__ void batch_pc1(const BInst<T>& I, const LevelView<T>& L0, int64_t i,
                                          const V4<T>& n, V4<T>& z, double (&acc)[3]) {
    if (I.use_mg) {
        z.x = z.y = z.z = T(0);
        z.w = I.pc[8 * i + 6] * n.w;
        L0.b[i] = n.x;
        L0.b[L0.N + i] = n.y;
        L0.b[2 * L0.N + i] = n.z;
        const T bv[3] = {n.x, n.y, n.z};
        mg_first_dir<T>(L0, i, bv);
    } else {
        pc_jacobi_b<T>(I.pc, i, n, z);
        acc[2] += (double)(n.x * z.x) + (double)(n.y * z.y) + (double)(n.z * z.z);
    }
    acc[0] += (double)n.w;
    acc[1] += (double)(n.w * z.w);
}

// The persistent batched MINRES.  TPR threads per block row (4 or 8): with 8,
// two threads share one output component and split the block columns.
template <typename T, int TPR>
__global__ void __launch_bounds__(512)
k_batch_minres(int ninst, BInst<T>* __restrict__ inst, int nchunks,
               const BChunk* __restrict__ chunks, double* __restrict__ part,
               BarrierState* bar, long long max_sweeps, BSched S) {
    constexpr int NP = 3;  // partial values per chunk
    // ---- initialisation: scalars, first Lanczos vector, beta1 --------------
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < ninst; b += gridDim.x * blockDim.x) {
        MinresScalars* s = inst[b].s;
        s->rtol = inst[b].rtol;
        s->maxit = inst[b].maxit;
        s->crank = inst[b].crank;
        s->iters = 0;
        s->c_pending = 0;
        s->status = 0;
        s->ycorr[0] = s->ycorr[1] = 0.0;
        s->stop = inst[b].skip;
    }
    if (!grid_barrier(bar)) return;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        const BInst<T>& I = inst[C.inst];
        double acc[NP] = {0.0, 0.0, 0.0};
        if (!I.s->stop) {
            const LevelView<T> L0 = I.use_mg ? I.lv[0] : LevelView<T>{};
            for (int64_t i = C.row0 + threadIdx.x; i < C.row1; i += blockDim.x) {
                const V4<T> n = I.r0[i];
                I.R[0][i] = n;
                I.R[1][i] = V4<T>{T(0), T(0), T(0), T(0)};
                V4<T> z;
                batch_pc1<T>(I, L0, i, n, z, acc);
                I.Y[0][i] = z;
                I.W[0][i] = V4<T>{T(0), T(0), T(0), T(0)};
                I.W[1][i] = V4<T>{T(0), T(0), T(0), T(0)};
                I.X[i] = V4<T>{T(0), T(0), T(0), T(0)};
            }
        }
        bsum<NP>(acc);
        if (threadIdx.x == 0)
            for (int k = 0; k < NP; ++k) part[(int64_t)ch * NP + k] = acc[k];
    }
    if (!grid_barrier(bar)) return;
    if (S.max_depth > 0) {
        if (!batch_vcycle<T>(inst, chunks, S, bar)) return;
        batch_pc2<T>(inst, nchunks, chunks, 0, 0, part);
        if (!grid_barrier(bar)) return;
    }
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < ninst; b += gridDim.x * blockDim.x) {
        MinresScalars* s = inst[b].s;
        if (s->stop) continue;
        double t[NP] = {0.0, 0.0, 0.0};
        for (int ch = inst[b].chunk0; ch < inst[b].chunk1; ++ch)
            for (int k = 0; k < NP; ++k) t[k] += part[(int64_t)ch * NP + k];
        s->ycorr[0] = s->crank * t[0];
        finalize_beta_b(s, t[2] + t[1] + s->crank * t[0] * t[0], true);
    }
    if (!grid_barrier(bar)) return;

    // ---- iterations -----------------------------------------------------------
    for (long long k = 1; k <= max_sweeps; ++k) {
        const int p = (int)(k & 1);
        const int yk = (int)((k - 1) & 1), yn = (int)(k & 1);
        // A: q = S v, v = (y + ycorr e_p)/beta; partial v.q, v.r1
        for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
            const BChunk C = chunks[ch];
            const BInst<T>& I = inst[C.inst];
            double acc[NP] = {0.0, 0.0, 0.0};
            const MinresScalars* s = I.s;
            if (!s->stop) {
                const T tinv = (T)(1.0 / s->beta);
                const T wadd = (T)s->ycorr[yk];
                const V4<T>* Yv = I.Y[yk];
                const T* y = reinterpret_cast<const T*>(Yv);
                const T* r1 = reinterpret_cast<const T*>(I.R[p]);
                T* q = reinterpret_cast<T*>(I.q);
                const int sub = threadIdx.x % TPR;
                const int r = sub & 3, half = sub >> 2;  // half: column split (TPR = 8)
                const int rows_per_pass = blockDim.x / TPR;
                if (sizeof(T) == 4 && I.lat) {  // lattice half stencil, thread per node
                    const V4<float>* Yf = reinterpret_cast<const V4<float>*>(Yv);
                    const V4<float>* R1f = reinterpret_cast<const V4<float>*>(I.R[p]);
                    V4<float>* qf = reinterpret_cast<V4<float>*>(I.q);
                    const float tf = (float)tinv, wf = (float)wadd;
                    for (int64_t v = C.row0 + threadIdx.x; v < C.row1; v += blockDim.x) {
                        const float4 a = lat_row(I.lat_n, v, I.lat, Yf, wf);
                        V4<float> qv;
                        qv.x = a.x * tf;
                        qv.y = a.y * tf;
                        qv.z = a.z * tf;
                        qv.w = a.w * tf;
                        qf[v] = qv;
                        const V4<float> yv = Yf[v], r1v = R1f[v];
                        const float e0 = yv.x * tf, e1 = yv.y * tf, e2 = yv.z * tf,
                                    e3 = (yv.w + wf) * tf;
                        acc[0] += (double)fmaf(e0, qv.x, fmaf(e1, qv.y, fmaf(e2, qv.z, e3 * qv.w)));
                        acc[1] += (double)fmaf(e0, r1v.x,
                                               fmaf(e1, r1v.y, fmaf(e2, r1v.z, e3 * r1v.w)));
                    }
                } else
                for (int64_t row = C.row0 + threadIdx.x / TPR; row < C.row1; row += rows_per_pass) {
                    T ax = T(0);
                    const int32_t k1 = I.rowptr[row + 1];
                    for (int32_t kk = I.rowptr[row] + half; kk < k1; kk += TPR / 4) {
                        const int32_t j = __ldg(I.cols + kk);
                        const V4<T> a = *reinterpret_cast<const V4<T>*>(I.A + (int64_t)kk * 16 + r * 4);
                        const V4<T> xj = Yv[j];
                        ax = fma(a.x, xj.x, ax);
                        ax = fma(a.y, xj.y, ax);
                        ax = fma(a.z, xj.z, ax);
                        ax = fma(a.w, xj.w + wadd, ax);
                    }
                    if (TPR == 8) {
                        // the 8 lanes of one block row run in lock-step; other rows
                        // of the warp may have left the loop
                        const unsigned grp = 0xffu << ((threadIdx.x & 31) & ~7);
                        ax += __shfl_down_sync(grp, ax, 4, 8);
                    }
                    if (half == 0) {
                        const T qv = ax * tinv;
                        const int64_t e = row * 4 + r;
                        q[e] = qv;
                        const T ve = (y[e] + (r == 3 ? wadd : T(0))) * tinv;
                        acc[0] += (double)(ve * qv);
                        acc[1] += (double)(ve * r1[e]);
                    }
                }
            }
            bsum<NP>(acc);
            if (threadIdx.x == 0)
                for (int kk = 0; kk < NP; ++kk) part[(int64_t)ch * NP + kk] = acc[kk];
        }
        if (!grid_barrier(bar)) return;
        for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < ninst;
             b += gridDim.x * blockDim.x) {
            MinresScalars* s = inst[b].s;
            s->c_pending = 0;  // the previous C phase has finished
            if (s->stop) continue;
            double t0 = 0.0, t1 = 0.0;
            for (int ch = inst[b].chunk0; ch < inst[b].chunk1; ++ch) {
                t0 += part[(int64_t)ch * NP];
                t1 += part[(int64_t)ch * NP + 1];
            }
            const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
            s->alfa = t0 - c1 * t1;
        }
        if (!grid_barrier(bar)) return;
        // B: Lanczos update + Jacobi + rank-one; partial sums
        for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
            const BChunk C = chunks[ch];
            const BInst<T>& I = inst[C.inst];
            double acc[NP] = {0.0, 0.0, 0.0};
            const MinresScalars* s = I.s;
            if (!s->stop) {
                const T c1 = (T)(s->iters >= 1 ? s->beta / s->oldb : 0.0);
                const T c2 = (T)(s->alfa / s->beta);
                V4<T>* R1 = I.R[p];
                const V4<T>* R2 = I.R[1 - p];
                V4<T>* Yn = I.Y[yn];
                const LevelView<T> L0 = I.use_mg ? I.lv[0] : LevelView<T>{};
                for (int64_t i = C.row0 + threadIdx.x; i < C.row1; i += blockDim.x) {
                    const V4<T> qv = I.q[i], a = R1[i], b2 = R2[i];
                    V4<T> n;
                    n.x = qv.x - c1 * a.x - c2 * b2.x;
                    n.y = qv.y - c1 * a.y - c2 * b2.y;
                    n.z = qv.z - c1 * a.z - c2 * b2.z;
                    n.w = qv.w - c1 * a.w - c2 * b2.w;
                    R1[i] = n;
                    V4<T> z;
                    batch_pc1<T>(I, L0, i, n, z, acc);
                    Yn[i] = z;
                }
            }
            bsum<NP>(acc);
            if (threadIdx.x == 0)
                for (int kk = 0; kk < NP; ++kk) part[(int64_t)ch * NP + kk] = acc[kk];
        }
        if (!grid_barrier(bar)) return;
        if (S.max_depth > 0) {
            if (!batch_vcycle<T>(inst, chunks, S, bar)) return;
            batch_pc2<T>(inst, nchunks, chunks, p, yn, part);
            if (!grid_barrier(bar)) return;
        }
        for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < ninst;
             b += gridDim.x * blockDim.x) {
            MinresScalars* s = inst[b].s;
            if (s->stop) continue;
            double t[NP] = {0.0, 0.0, 0.0};
            for (int ch = inst[b].chunk0; ch < inst[b].chunk1; ++ch)
                for (int kk = 0; kk < NP; ++kk) t[kk] += part[(int64_t)ch * NP + kk];
            s->ycorr[yn] = s->crank * t[0];
            finalize_beta_b(s, t[2] + t[1] + s->crank * t[0] * t[0], false);
            if (!s->stop) atomicAdd(&bar->active, 1);
        }
        if (!grid_barrier(bar)) return;
        const int active = *((volatile int*)&bar->active);
        // C: w and x update for instances that completed this iteration
        for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
            const BChunk C = chunks[ch];
            const BInst<T>& I = inst[C.inst];
            const MinresScalars* s = I.s;
            if (!s->c_pending) continue;
            const T inv = (T)(1.0 / s->oldb);
            const T wadd = (T)s->ycorr[yk];
            const T oe = (T)s->oldeps, de = (T)s->delta, ig = (T)(1.0 / s->gamma),
                    ph = (T)s->phi;
            V4<T>* Wprev = I.W[p];
            const V4<T>* Wcur = I.W[1 - p];
            const V4<T>* Yk = I.Y[yk];
            for (int64_t i = C.row0 + threadIdx.x; i < C.row1; i += blockDim.x) {
                const V4<T> y = Yk[i], wp = Wprev[i], wc = Wcur[i];
                V4<T> w, xv = I.X[i];
                w.x = (y.x * inv - oe * wp.x - de * wc.x) * ig;
                w.y = (y.y * inv - oe * wp.y - de * wc.y) * ig;
                w.z = (y.z * inv - oe * wp.z - de * wc.z) * ig;
                w.w = ((y.w + wadd) * inv - oe * wp.w - de * wc.w) * ig;
                Wprev[i] = w;
                xv.x += ph * w.x;
                xv.y += ph * w.y;
                xv.z += ph * w.z;
                xv.w += ph * w.w;
                I.X[i] = xv;
            }
        }
        if (active == 0) break;
        if (!grid_barrier(bar)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) bar->active = 0;
        // (the next A phase does not touch W, X or the active counter; the
        //  counter is read only after the next B-finalise barrier)
    }
}

}  // namespace fts

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

namespace fts {

// Outer-loop state of one instance (device).
struct BOuter {
    const V4<double>* b;
    V4<double>* x;
    V4<double>* r;
    float* r32;            // FP32 inner right-hand side (mixed)
    const void* d;         // inner correction: V4<double> (FP64) or V4<float> (mixed)
    double* flow;          // device staging of the output
    const uint8_t* bnd;
    int64_t np;
    double tol, floor32;
    double bnorm, rel, prev_rel, scale, pc_ratio;
    long long iters, outer, maxit;
    int converged, zero_load, status, first;
};

// r = b - S x (FP64) over the chunk list; partials ||r||^2, ||b||^2 per chunk.
__global__ void __launch_bounds__(256)
k_batch_residual(const BInst<double>* __restrict__ inst64, BOuter* __restrict__ out,
                 int nchunks, const BChunk* __restrict__ chunks, double* __restrict__ part) {
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        const BInst<double>& I = inst64[C.inst];
        const BOuter& O = out[C.inst];
        double acc[2] = {0.0, 0.0};
        if (!O.converged) {
            const int r = threadIdx.x & 3;
            const double* bb = reinterpret_cast<const double*>(O.b);
            double* rr = reinterpret_cast<double*>(O.r);
            for (int64_t row = C.row0 + (threadIdx.x >> 2); row < C.row1; row += blockDim.x >> 2) {
                double ax = 0.0;
                for (int32_t k = I.rowptr[row]; k < I.rowptr[row + 1]; ++k) {
                    const int32_t j = __ldg(I.cols + k);
                    const V4<double> a = *reinterpret_cast<const V4<double>*>(I.A + (int64_t)k * 16 + r * 4);
                    const V4<double> xj = O.x[j];
                    ax = fma(a.x, xj.x, ax);
                    ax = fma(a.y, xj.y, ax);
                    ax = fma(a.z, xj.z, ax);
                    ax = fma(a.w, xj.w, ax);
                }
                const int64_t e = row * 4 + r;
                const double v = bb[e] - ax;
                rr[e] = v;
                acc[0] += v * v;
                acc[1] += bb[e] * bb[e];
            }
        }
        block_sum<2>(acc);
        if (threadIdx.x == 0) {
            part[(int64_t)ch * 3] = acc[0];
            part[(int64_t)ch * 3 + 1] = acc[1];
        }
    }
}

// Per instance: residual norm, convergence, the next inner tolerance, the
// learned true/preconditioned reduction ratio; marks instances to skip.
template <typename T>
__global__ void k_batch_outer(int ninst, BInst<T>* __restrict__ inst, BOuter* __restrict__ out,
                              const double* __restrict__ part, int mixed) {
    const double flt_min = FLT_MIN;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < ninst; b += gridDim.x * blockDim.x) {
        BOuter& O = out[b];
        BInst<T>& I = inst[b];
        if (O.converged) {
            I.skip = 1;
            continue;
        }
        double rr = 0.0, bb = 0.0;
        for (int ch = I.chunk0; ch < I.chunk1; ++ch) {
            rr += part[(int64_t)ch * 3];
            bb += part[(int64_t)ch * 3 + 1];
        }
        if (O.first) {
            O.first = 0;
            O.bnorm = sqrt(bb);
            if (!(O.bnorm > flt_min)) {  // zero load: nothing to solve (Flow.cpp:248-251)
                O.zero_load = 1;
                O.converged = 1;
                I.skip = 1;
                continue;
            }
        } else {
            const MinresScalars* s = I.s;
            O.iters += s->iters;
            O.outer += 1;
            if (s->status == 2 || !isfinite(rr)) {
                O.status = FTS_ERR_NAN;
                O.converged = 1;  // stop working on it; flow stays untouched
                I.skip = 1;
                continue;
            }
            const double achieved = s->beta1 > 0.0 ? s->phibar / s->beta1 : 0.0;
            const double rel_new = sqrt(rr) / O.bnorm;
            if (achieved > 0.0 && s->iters > 0) {
                double ratio = (rel_new / O.rel) / achieved;
                ratio = ratio < 1.0 ? 1.0 : (ratio > 1e6 ? 1e6 : ratio);
                O.pc_ratio = ratio;
            }
        }
        O.rel = sqrt(rr) / O.bnorm;
        O.scale = rr > 0.0 ? 1.0 / sqrt(rr) : 0.0;
        if (O.rel <= O.tol) {
            O.converged = 1;
            I.skip = 1;
            continue;
        }
        if (O.iters >= O.maxit) {
            O.status = FTS_ERR_NOT_CONVERGED;
            O.converged = 1;
            I.skip = 1;
            continue;
        }
        double rt = O.tol / O.rel / O.pc_ratio * 0.5;
        if (mixed && rt < O.floor32) rt = O.floor32;
        if (rt > 0.5) rt = 0.5;
        I.rtol = rt;
        I.maxit = O.maxit - O.iters;
        I.skip = 0;
    }
}

// Mixed: r32 = r / ||r||.  FP64 inner reads r directly.
__global__ void k_batch_prepare32(const BInst<float>* __restrict__ inst, BOuter* __restrict__ out,
                                  int nchunks, const BChunk* __restrict__ chunks) {
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        if (inst[C.inst].skip) continue;
        const BOuter& O = out[C.inst];
        const double sc = O.scale;
        const double* r = reinterpret_cast<const double*>(O.r);
        for (int64_t e = (int64_t)C.row0 * 4 + threadIdx.x; e < (int64_t)C.row1 * 4; e += blockDim.x)
            O.r32[e] = (float)(r[e] * sc);
    }
}

// x += d (FP64 inner) or x += ||r|| d32 (mixed inner), for instances solved in this pass.
template <typename T>
__global__ void k_batch_update(const BInst<T>* __restrict__ inst, BOuter* __restrict__ out,
                               int nchunks, const BChunk* __restrict__ chunks) {
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        if (inst[C.inst].skip) continue;
        const BOuter& O = out[C.inst];
        const double rn = sizeof(T) == 4 ? (O.scale > 0.0 ? 1.0 / O.scale : 0.0) : 1.0;
        const T* d = reinterpret_cast<const T*>(O.d);
        double* x = reinterpret_cast<double*>(O.x);
        for (int64_t e = (int64_t)C.row0 * 4 + threadIdx.x; e < (int64_t)C.row1 * 4; e += blockDim.x)
            x[e] += rn * (double)d[e];
    }
}

// flow = [ux, uy, uz, p] for instances that converged with a load.
__global__ void k_batch_scatter(BOuter* __restrict__ out, int nchunks,
                                const BChunk* __restrict__ chunks) {
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const BChunk C = chunks[ch];
        const BOuter& O = out[C.inst];
        if (!O.converged || O.zero_load || O.status != 0) continue;
        const int64_t np = O.np;
        for (int64_t i = C.row0 + threadIdx.x; i < C.row1; i += blockDim.x) {
            const V4<double> v = O.x[i];
            const bool d = O.bnd[i] != 0;
            O.flow[i] = d ? 0.0 : v.x;
            O.flow[np + i] = d ? 0.0 : v.y;
            O.flow[2 * np + i] = d ? 0.0 : v.z;
            O.flow[3 * np + i] = v.w;
        }
    }
}

}  // namespace fts

using namespace fts;

struct fts_batch {
    std::vector<fts_ctx*> ctx;
    int count = 0;
    int precision = FTS_PREC_FP64;
    int device = 0;
    int num_sms = 148;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;
    // tuned launch shape of the persistent kernel
    fts_batch_config cfg{256, 1024, 4, 0, 0.0, 0, FTS_BATCH_BSR};
    bool tuned = false;
    // device state
    std::vector<BChunk> chunks;   // row chunks (depth 0), then the multigrid levels by depth
    std::vector<int> cptr;        // chunks of depth d: [cptr[d], cptr[d + 1])
    std::vector<int> coarse;      // instances with a multigrid hierarchy
    int nch0 = 0;                 // row chunks
    int max_depth = 0;            // non-coarsest multigrid depths
    BChunk* d_chunks = nullptr;
    size_t chunk_cap = 0;
    int* d_sched = nullptr;       // cptr then coarse (device)
    size_t sched_cap = 0;
    double* d_part = nullptr;
    size_t part_cap = 0;
    BarrierState* d_bar = nullptr;
    BInst<double>* d_inst64 = nullptr;
    BInst<float>* d_inst32 = nullptr;
    BOuter* d_out = nullptr;
    std::vector<BInst<double>> h_inst64;
    std::vector<BInst<float>> h_inst32;
    std::vector<BOuter> h_out;
    cudaGraphExec_t graph = nullptr;
    int graph_outer = 0;
    bool graph_unavailable = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace fts {

// Multigrid level sizes of instance i (empty: block Jacobi).
static std::vector<int> batch_chain(const fts_batch& B, int i) {
    const Ctx& c = B.ctx[i]->c;
    return c.use_mg ? mg_chain(c.topo.lattice_n) : std::vector<int>();
}

static void batch_chunks(fts_batch& B, int chunk_rows) {
    B.chunks.clear();
    B.coarse.clear();
    B.max_depth = 0;
    std::vector<std::vector<int>> chains(B.count);
    for (int i = 0; i < B.count; ++i) {
        const Ctx& c = B.ctx[i]->c;
        chains[i] = batch_chain(B, i);
        if ((int)chains[i].size() > kMaxLevels)
            throw CudaError(cudaErrorInvalidValue, "too many multigrid levels for a batch",
                            __FILE__, __LINE__);
        const int nlev = (int)chains[i].size();
        B.h_inst64[i].use_mg = B.h_inst32[i].use_mg = nlev > 0;
        B.h_inst64[i].nlev = B.h_inst32[i].nlev = nlev;
        if (nlev > 0) {
            B.coarse.push_back(i);
            B.max_depth = std::max(B.max_depth, nlev - 1);
        }
        const int first = (int)B.chunks.size();
        for (int64_t r0 = 0; r0 < c.np; r0 += chunk_rows)
            B.chunks.push_back({i, (int)r0, (int)std::min<int64_t>(c.np, r0 + chunk_rows), 0});
        B.h_inst64[i].chunk0 = B.h_inst32[i].chunk0 = first;
        B.h_inst64[i].chunk1 = B.h_inst32[i].chunk1 = (int)B.chunks.size();
    }
    B.nch0 = (int)B.chunks.size();
    B.cptr.assign(1, 0);
    B.cptr.push_back(B.nch0);
    for (int d = 1; d <= B.max_depth; ++d) {
        for (int i = 0; i < B.count; ++i) {
            if ((int)chains[i].size() <= d) continue;
            const int64_t n = chains[i][d];
            const int64_t N = n * n * n;
            for (int64_t r0 = 0; r0 < N; r0 += chunk_rows)
                B.chunks.push_back({i, (int)r0, (int)std::min<int64_t>(N, r0 + chunk_rows), d});
        }
        B.cptr.push_back((int)B.chunks.size());
    }
    const size_t n = B.chunks.size();
    if (n > B.chunk_cap) {
        if (B.d_chunks) cudaFree(B.d_chunks);
        if (B.d_part) cudaFree(B.d_part);
        B.d_chunks = nullptr;
        B.d_part = nullptr;
        FTS_CUDA(cudaMalloc(&B.d_chunks, n * sizeof(BChunk)));
        FTS_CUDA(cudaMalloc(&B.d_part, n * 3 * sizeof(double)));
        B.chunk_cap = n;
    }
    std::vector<int> sched(B.cptr);
    sched.insert(sched.end(), B.coarse.begin(), B.coarse.end());
    if (sched.size() > B.sched_cap) {
        if (B.d_sched) cudaFree(B.d_sched);
        B.d_sched = nullptr;
        FTS_CUDA(cudaMalloc(&B.d_sched, sched.size() * sizeof(int)));
        B.sched_cap = sched.size();
    }
    FTS_CUDA(cudaMemcpyAsync(B.d_sched, sched.data(), sched.size() * sizeof(int),
                             cudaMemcpyHostToDevice, B.stream));
    FTS_CUDA(cudaMemcpyAsync(B.d_chunks, B.chunks.data(), n * sizeof(BChunk),
                             cudaMemcpyHostToDevice, B.stream));
    FTS_CUDA(cudaMemcpyAsync(B.d_inst64, B.h_inst64.data(), B.count * sizeof(BInst<double>),
                             cudaMemcpyHostToDevice, B.stream));
    FTS_CUDA(cudaMemcpyAsync(B.d_inst32, B.h_inst32.data(), B.count * sizeof(BInst<float>),
                             cudaMemcpyHostToDevice, B.stream));
}

template <typename T, int TPR>
static int coresident_blocks(int threads, int num_sms) {
    int per_sm = 0;
    FTS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_minres<T, TPR>,
                                                           threads, 0));
    return std::max(1, per_sm) * num_sms;
}

// Level views of the instances' multigrid hierarchies (built by the first
// assembly), uploaded with the instance table.
static void batch_levels(fts_batch& B) {
    for (int i = 0; i < B.count; ++i) {
        Ctx& c = B.ctx[i]->c;
        if (!c.use_mg) continue;
        if (B.precision == FTS_PREC_MIXED) {
            for (size_t l = 0; l < c.mg32.L.size(); ++l) B.h_inst32[i].lv[l] = level_view(c.mg32, l);
        } else {
            for (size_t l = 0; l < c.mg64.L.size(); ++l) B.h_inst64[i].lv[l] = level_view(c.mg64, l);
        }
    }
    FTS_CUDA(cudaMemcpyAsync(B.d_inst64, B.h_inst64.data(), B.count * sizeof(BInst<double>),
                             cudaMemcpyHostToDevice, B.stream));
    FTS_CUDA(cudaMemcpyAsync(B.d_inst32, B.h_inst32.data(), B.count * sizeof(BInst<float>),
                             cudaMemcpyHostToDevice, B.stream));
}

template <typename T>
static void launch_persistent(fts_batch& B, long long sweeps) {
    BInst<T>* inst = sizeof(T) == 8 ? reinterpret_cast<BInst<T>*>(B.d_inst64)
                                    : reinterpret_cast<BInst<T>*>(B.d_inst32);
    FTS_CUDA(cudaMemsetAsync(B.d_bar, 0, kBarrierResetBytes, B.stream));
    const int threads = B.cfg.threads;
    const int nch = B.nch0;
    const BSched S{B.d_sched, B.max_depth, B.d_sched + B.cptr.size(), (int)B.coarse.size()};
    int blocks = B.cfg.tpr == 8 ? coresident_blocks<T, 8>(threads, B.num_sms)
                                : coresident_blocks<T, 4>(threads, B.num_sms);
    blocks = std::min(blocks, std::max(nch, B.num_sms));
    B.cfg.blocks = blocks;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)blocks);
    lc.blockDim = dim3((unsigned)threads);
    lc.dynamicSmemBytes = 0;
    lc.stream = B.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    if (B.cfg.tpr == 8)
        FTS_CUDA(cudaLaunchKernelEx(&lc, k_batch_minres<T, 8>, B.count, inst, nch,
                                    (const BChunk*)B.d_chunks, B.d_part, B.d_bar, sweeps, S));
    else
        FTS_CUDA(cudaLaunchKernelEx(&lc, k_batch_minres<T, 4>, B.count, inst, nch,
                                    (const BChunk*)B.d_chunks, B.d_part, B.d_bar, sweeps, S));
}

// Assembly of every instance (the single-solve kernels, no host waits).
static void batch_assemble(fts_batch& B, const std::vector<int>& have_mu) {
    for (int i = 0; i < B.count; ++i) {
        Ctx& c = B.ctx[i]->c;
        c.stream = B.stream;
        FTS_CUDA(cudaMemsetAsync(c.err_flag, 0, sizeof(int), c.stream));
        launch_check_finite(c, c.phi, c.np);
        launch_check_finite(c, c.src, c.np);
        if (have_mu[i]) launch_check_finite(c, c.mu, c.nt);
        if (!have_mu[i]) launch_viscosity_profile(c);
        launch_mu_minmax(c);  // the Schur weight's scale reads the range
        launch_source(c);
        launch_rhs(c, false);
        launch_assemble(c);
        launch_preconditioner(c);
        if (B.precision == FTS_PREC_MIXED) {
            launch_to_f32(c);
            if (c.lat_val) launch_to_lat(c);
            if (c.use_mg) setup_preconditioner<float>(c);
        } else if (c.use_mg) {
            setup_preconditioner<double>(c);
        }
        if (!c.par.warm_start)
            FTS_CUDA(cudaMemsetAsync(c.x, 0, c.np * sizeof(V4<double>), c.stream));
    }
}

// The outer loop for all instances, outer_passes times (device-side decisions).
static void batch_outer_passes(fts_batch& B, int passes, long long sweeps) {
    const int nch = B.nch0;
    const int g = std::min(nch, B.num_sms * 8);
    const bool mixed = B.precision == FTS_PREC_MIXED;
    for (int o = 0; o <= passes; ++o) {
        k_batch_residual<<<g, 256, 0, B.stream>>>(B.d_inst64, B.d_out, nch, B.d_chunks, B.d_part);
        if (mixed)
            k_batch_outer<float><<<(B.count + 127) / 128, 128, 0, B.stream>>>(B.count, B.d_inst32,
                                                                            B.d_out, B.d_part, 1);
        else
            k_batch_outer<double><<<(B.count + 127) / 128, 128, 0, B.stream>>>(B.count, B.d_inst64,
                                                                             B.d_out, B.d_part, 0);
        if (o == passes) break;
        if (mixed) {
            k_batch_prepare32<<<g, 256, 0, B.stream>>>(B.d_inst32, B.d_out, nch, B.d_chunks);
            launch_persistent<float>(B, sweeps);
            k_batch_update<float><<<g, 256, 0, B.stream>>>(B.d_inst32, B.d_out, nch, B.d_chunks);
        } else {
            launch_persistent<double>(B, sweeps);
            k_batch_update<double><<<g, 256, 0, B.stream>>>(B.d_inst64, B.d_out, nch, B.d_chunks);
        }
    }
    k_batch_scatter<<<g, 256, 0, B.stream>>>(B.d_out, nch, B.d_chunks);
    FTS_CUDA(cudaGetLastError());
}

static void batch_reset_outer(fts_batch& B) {
    for (int i = 0; i < B.count; ++i) {
        Ctx& c = B.ctx[i]->c;
        BOuter& O = B.h_out[i];
        O.converged = 0;
        O.zero_load = 0;
        O.status = 0;
        O.first = 1;
        O.iters = 0;
        O.outer = 0;
        O.rel = 1.0;
        O.pc_ratio = B.precision == FTS_PREC_MIXED ? c.pc_ratio32 : c.pc_ratio64;
        O.tol = c.par.tol > 0.0 ? c.par.tol : DBL_EPSILON;
        O.floor32 = c.par.inner_tol > 0.0 ? c.par.inner_tol : kInnerTolFloorLarge;
        const long long N = 3 * c.topo.n_interior + c.np;
        O.maxit = c.par.max_iter > 0 ? c.par.max_iter : 2 * N;
    }
    FTS_CUDA(cudaMemcpyAsync(B.d_out, B.h_out.data(), B.count * sizeof(BOuter),
                             cudaMemcpyHostToDevice, B.stream));
}

static void batch_build(fts_batch& B) {
    B.h_inst64.resize(B.count);
    B.h_inst32.resize(B.count);
    B.h_out.resize(B.count);
    for (int i = 0; i < B.count; ++i) {
        Ctx& c = B.ctx[i]->c;
        BInst<double>& a = B.h_inst64[i];
        std::memset(&a, 0, sizeof(a));
        a.np = c.np;
        a.rowptr = c.rowptr;
        a.cols = c.cols;
        a.A = c.A64;
        a.pc = c.pc64;
        a.q = c.w64.q;
        for (int k = 0; k < 2; ++k) {
            a.R[k] = c.w64.R[k];
            a.Y[k] = c.w64.Y[k];
            a.W[k] = c.w64.W[k];
        }
        a.X = c.w64.X;
        a.r0 = c.r;
        a.s = c.ms;
        a.crank = c.crank;
        a.maxit = 1;
        a.rtol = 0.5;
        BInst<float>& f = B.h_inst32[i];
        std::memset(&f, 0, sizeof(f));
        if (B.precision == FTS_PREC_MIXED && c.topo.lattice_n > 0) build_lattice(c);
        if (B.precision == FTS_PREC_MIXED) {
            f.np = c.np;
            f.rowptr = c.rowptr;
            f.cols = c.cols;
            f.A = c.A32;
            f.pc = c.pc32;
            f.q = c.w32.q;
            for (int k = 0; k < 2; ++k) {
                f.R[k] = c.w32.R[k];
                f.Y[k] = c.w32.Y[k];
                f.W[k] = c.w32.W[k];
            }
            f.X = c.w32.X;
            f.r0 = c.w32.r0;
            f.s = c.ms;
            f.crank = c.crank;
            f.maxit = 1;
            f.rtol = 0.5;
        }
        BOuter& O = B.h_out[i];
        std::memset(&O, 0, sizeof(O));
        O.b = c.b;
        O.x = c.x;
        O.r = c.r;
        O.r32 = B.precision == FTS_PREC_MIXED ? reinterpret_cast<float*>(c.w32.r0) : nullptr;
        O.d = B.precision == FTS_PREC_MIXED ? (const void*)c.w32.X : (const void*)c.w64.X;
        O.flow = c.flow;
        O.bnd = c.bnd;
        O.np = c.np;
    }
    FTS_CUDA(cudaMalloc(&B.d_inst64, B.count * sizeof(BInst<double>)));
    FTS_CUDA(cudaMalloc(&B.d_inst32, B.count * sizeof(BInst<float>)));
    FTS_CUDA(cudaMalloc(&B.d_out, B.count * sizeof(BOuter)));
    FTS_CUDA(cudaMalloc(&B.d_bar, sizeof(BarrierState)));
    {
        const BarrierState cfg = barrier_config(kDefaultBarrierLimitNs, -1);
        FTS_CUDA(cudaMemcpy(B.d_bar, &cfg, sizeof(cfg), cudaMemcpyHostToDevice));
    }
    batch_chunks(B, B.cfg.chunk_rows);
}

// The SpMV operator storage of every instance for a batch-wide format choice.
static void batch_set_format(fts_batch& B, int format) {
    for (int i = 0; i < B.count; ++i) {
        const Ctx& c = B.ctx[i]->c;
        const bool lat = format == FTS_BATCH_LATTICE && c.lat_val != nullptr;
        B.h_inst32[i].lat = lat ? reinterpret_cast<const float4*>(c.lat_val) : nullptr;
        B.h_inst32[i].lat_n = lat ? c.topo.lattice_n : 0;
    }
    B.cfg.spmv_format = format;
}

// Autotuner: time a fixed number of sweeps of the persistent kernel for every
// candidate shape (block size, chunk length, threads per block row and, in
// mixed precision with Kuhn-lattice instances, the SpMV's operator storage) on
// the assembled batch; keep the fastest.
static void batch_tune(fts_batch& B) {
    const bool mixed = B.precision == FTS_PREC_MIXED;
    // a residual pass so that every instance has a right-hand side and a tolerance
    batch_reset_outer(B);
    const int nch0 = B.nch0;
    k_batch_residual<<<std::min(nch0, B.num_sms * 8), 256, 0, B.stream>>>(B.d_inst64, B.d_out, nch0,
                                                                        B.d_chunks, B.d_part);
    if (mixed) {
        k_batch_outer<float><<<(B.count + 127) / 128, 128, 0, B.stream>>>(B.count, B.d_inst32,
                                                                        B.d_out, B.d_part, 1);
        k_batch_prepare32<<<std::min(nch0, B.num_sms * 8), 256, 0, B.stream>>>(B.d_inst32, B.d_out,
                                                                             nch0, B.d_chunks);
    } else {
        k_batch_outer<double><<<(B.count + 127) / 128, 128, 0, B.stream>>>(B.count, B.d_inst64,
                                                                         B.d_out, B.d_part, 0);
    }
    const int threads_c[3] = {128, 256, 512};
    const int chunk_c[3] = {256, 1024, 4096};
    const int tpr_c[2] = {4, 8};
    const long long sweeps = 24;
    fts_batch_config best = B.cfg;
    best.ms_per_sweep = 1e30;
    bool any_lattice = false;
    for (int i = 0; i < B.count; ++i) any_lattice = any_lattice || B.ctx[i]->c.lat_val != nullptr;
    const int nfmt = mixed && any_lattice ? 2 : 1;
    for (int fmt = 0; fmt < nfmt; ++fmt)
    for (int tc : threads_c)
        for (int cc : chunk_c)
            for (int tp : tpr_c) {
                if (fmt == FTS_BATCH_LATTICE && tp != 4) continue;  // BSR instances only
                B.cfg.threads = tc;
                B.cfg.chunk_rows = cc;
                B.cfg.tpr = tp;
                // the shape's chunk list, with the tuning tolerances kept
                FTS_CUDA(cudaMemcpyAsync(B.h_inst64.data(), B.d_inst64,
                                         B.count * sizeof(BInst<double>), cudaMemcpyDeviceToHost,
                                         B.stream));
                FTS_CUDA(cudaMemcpyAsync(B.h_inst32.data(), B.d_inst32,
                                         B.count * sizeof(BInst<float>), cudaMemcpyDeviceToHost,
                                         B.stream));
                FTS_CUDA(cudaStreamSynchronize(B.stream));
                for (auto& a : B.h_inst64) a.rtol = 1e-30, a.maxit = sweeps + 1;
                for (auto& a : B.h_inst32) a.rtol = 1e-30, a.maxit = sweeps + 1;
                batch_set_format(B, fmt);
                batch_chunks(B, cc);
                if (mixed) launch_persistent<float>(B, 2);  // warm-up of this shape
                else launch_persistent<double>(B, 2);
                FTS_CUDA(cudaEventRecord(B.ev[0], B.stream));
                if (mixed) launch_persistent<float>(B, sweeps);
                else launch_persistent<double>(B, sweeps);
                FTS_CUDA(cudaEventRecord(B.ev[1], B.stream));
                FTS_CUDA(cudaEventSynchronize(B.ev[1]));
                BarrierState bs;
                FTS_CUDA(cudaMemcpy(&bs, B.d_bar, sizeof(bs), cudaMemcpyDeviceToHost));
                if (bs.error) throw CudaError(cudaErrorLaunchTimeout, "batched grid barrier", __FILE__, __LINE__);
                float ms = 0.f;
                FTS_CUDA(cudaEventElapsedTime(&ms, B.ev[0], B.ev[1]));
                if (ms / sweeps < best.ms_per_sweep) {
                    best = B.cfg;
                    best.ms_per_sweep = ms / sweeps;
                }
            }
    B.cfg = best;
    batch_set_format(B, best.spmv_format);
    batch_chunks(B, B.cfg.chunk_rows);
    B.tuned = true;
}

static void batch_free(fts_batch& B) {
    for (void* p : {(void*)B.d_chunks, (void*)B.d_part, (void*)B.d_bar, (void*)B.d_inst64,
                    (void*)B.d_inst32, (void*)B.d_out, (void*)B.d_sched})
        if (p) cudaFree(p);
    if (B.graph) cudaGraphExecDestroy(B.graph);
    for (auto& e : B.ev)
        if (e) cudaEventDestroy(e);
    for (fts_ctx* c : B.ctx) fts_destroy(c);
    if (B.own_stream) cudaStreamDestroy(B.own_stream);
}

}  // namespace fts

extern "C" {

int fts_batch_create(int32_t count, const fts_mesh* meshes, const fts_params* params,
                     fts_batch** out) {
    if (!out || count <= 0 || !meshes || !params) return FTS_ERR_BAD_INPUT;
    *out = nullptr;
    fts_batch* B = new (std::nothrow) fts_batch();
    if (!B) return FTS_ERR_OOM;
    B->count = count;
    B->precision = params[0].precision;
    B->device = params[0].device;
    int rc = FTS_OK;
    try {
        FTS_CUDA(cudaSetDevice(B->device));
        int sms = 0;
        FTS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device));
        B->num_sms = sms > 0 ? sms : 148;
        FTS_CUDA(cudaStreamCreateWithFlags(&B->own_stream, cudaStreamNonBlocking));
        B->stream = B->own_stream;
        for (auto& e : B->ev) FTS_CUDA(cudaEventCreate(&e));
        for (int i = 0; i < count; ++i) {
            fts_params p = params[i];
            if (p.precision != B->precision || p.device != B->device) {
                B->last_error = "all instances of a batch share precision and device";
                rc = FTS_ERR_BAD_INPUT;
                break;
            }
            if (p.solver != FTS_SOLVER_MINRES) {
                B->last_error = "batched solves use MINRES";
                rc = FTS_ERR_UNSUPPORTED;
                break;
            }
            fts_ctx* c = nullptr;
            rc = create_context(&meshes[i], &p, &c, true);
            if (rc != FTS_OK) {
                B->last_error = std::string("instance ") + std::to_string(i) + ": " +
                                fts_last_error(nullptr);
                break;
            }
            if (p.precision == FTS_PREC_MIXED) ensure_fp32(c->c);
            else ensure_fp64_work(c->c);
            B->ctx.push_back(c);
        }
        if (rc == FTS_OK) batch_build(*B);
    } catch (const CudaError& e) {
        B->last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (int code) {
        rc = code;
    }
    if (rc != FTS_OK) {
        g_batch_error() = B->last_error;
        batch_free(*B);
        delete B;
        return rc;
    }
    *out = B;
    return FTS_OK;
}

static int batch_solve_common(fts_batch* B, const double* const* phi, const double* const* source,
                              const double* const* mu, double* const* flow, fts_stats* stats,
                              bool device) {
    if (!B || !phi || !source || !flow) return FTS_ERR_BAD_INPUT;
    const double t0 = wall_ms();
    int rc = FTS_OK;
    try {
        FTS_CUDA(cudaSetDevice(B->device));
        const cudaMemcpyKind k = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        std::vector<int> have_mu(B->count, 0);
        for (int i = 0; i < B->count; ++i) {
            Ctx& c = B->ctx[i]->c;
            if (!phi[i] || !source[i] || !flow[i]) return FTS_ERR_BAD_INPUT;
            FTS_CUDA(cudaMemcpyAsync(c.phi, phi[i], c.np * sizeof(double), k, B->stream));
            FTS_CUDA(cudaMemcpyAsync(c.src, source[i], c.np * sizeof(double), k, B->stream));
            if (mu && mu[i]) {
                FTS_CUDA(cudaMemcpyAsync(c.mu, mu[i], c.nt * sizeof(double), k, B->stream));
                have_mu[i] = 1;
            }
        }
        FTS_CUDA(cudaEventRecord(B->ev[0], B->stream));
        batch_assemble(*B, have_mu);
        batch_levels(*B);
        // a barrier failure of any launch of this solve stays recorded
        FTS_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(B->d_bar) + kBarrierErrorOffset, 0,
                                 sizeof(int), B->stream));
        if (!B->tuned) batch_tune(*B);
        batch_reset_outer(*B);
        const int passes = B->precision == FTS_PREC_MIXED ? 4 : 2;
        const long long sweeps = 1LL << 40;  // bounded by the per-instance iteration caps
        // The device-side outer loop as one CUDA graph (captured once per batch).
        if ((!B->graph || B->graph_outer != passes) && !B->graph_unavailable) {
            if (B->graph) {
                cudaGraphExecDestroy(B->graph);
                B->graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            FTS_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
            bool ok = true;
            try {
                batch_outer_passes(*B, passes, sweeps);
            } catch (const CudaError&) {
                ok = false;
            }
            cudaError_t ec = cudaStreamEndCapture(B->stream, &g);
            if (ok && ec == cudaSuccess && g) {
                ok = cudaGraphInstantiate(&B->graph, g, 0) == cudaSuccess;
            } else {
                ok = false;
            }
            if (g) cudaGraphDestroy(g);
            if (!ok) {  // e.g. a driver without capture of cooperative launches
                (void)cudaGetLastError();
                B->graph = nullptr;
                B->graph_unavailable = true;
            }
            B->graph_outer = passes;
        }
        if (B->graph) FTS_CUDA(cudaGraphLaunch(B->graph, B->stream));
        else batch_outer_passes(*B, passes, sweeps);
        // instances that need more outer passes (rare) continue without the graph
        for (int extra = 0; extra < 16; ++extra) {
            FTS_CUDA(cudaMemcpyAsync(B->h_out.data(), B->d_out, B->count * sizeof(BOuter),
                                     cudaMemcpyDeviceToHost, B->stream));
            FTS_CUDA(cudaStreamSynchronize(B->stream));
            bool open = false;
            for (const BOuter& O : B->h_out) open = open || !O.converged;
            if (!open) break;
            batch_outer_passes(*B, 1, sweeps);
        }
        FTS_CUDA(cudaEventRecord(B->ev[1], B->stream));
        BarrierState bs;
        FTS_CUDA(cudaMemcpyAsync(&bs, B->d_bar, sizeof(bs), cudaMemcpyDeviceToHost, B->stream));
        FTS_CUDA(cudaMemcpyAsync(B->h_out.data(), B->d_out, B->count * sizeof(BOuter),
                                 cudaMemcpyDeviceToHost, B->stream));
        FTS_CUDA(cudaStreamSynchronize(B->stream));
        if (bs.error) {
            B->last_error = "batched grid barrier timed out";
            rc = FTS_ERR_TIMEOUT;
        }
        float ms = 0.f;
        FTS_CUDA(cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]));
        for (int i = 0; i < B->count; ++i) {
            Ctx& c = B->ctx[i]->c;
            const BOuter& O = B->h_out[i];
            int st = O.status;
            int bad = 0;
            FTS_CUDA(cudaMemcpy(&bad, c.err_flag, sizeof(int), cudaMemcpyDeviceToHost));
            if (bad) st = FTS_ERR_NAN;
            if (!O.converged && st == FTS_OK) st = FTS_ERR_NOT_CONVERGED;
            const bool solved = st == FTS_OK && O.converged && !O.zero_load;
            if (solved)
                FTS_CUDA(cudaMemcpyAsync(flow[i], c.flow, 4 * c.np * sizeof(double),
                                         device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                         B->stream));
            if (stats) {
                fts_stats& s = stats[i];
                std::memset(&s, 0, sizeof(s));
                s.status = st;
                s.solved = solved ? 1 : 0;
                s.iterations = O.iters;
                s.iterations_fp32 = B->precision == FTS_PREC_MIXED ? O.iters : 0;
                s.outer_iterations = (int)O.outer;
                s.rel_residual = O.rel;
                s.error_estimate = O.rel;
                s.f_norm = O.bnorm;
                s.ms_solve = ms;
                s.device_bytes = c.device_bytes;
            }
            if (st != FTS_OK && rc == FTS_OK) rc = st;
        }
        FTS_CUDA(cudaStreamSynchronize(B->stream));
    } catch (const CudaError& e) {
        B->last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM
             : e.code == cudaErrorLaunchTimeout  ? FTS_ERR_TIMEOUT
                                                 : FTS_ERR_CUDA;
    } catch (int code) {
        rc = code;
    }
    if (stats)
        for (int i = 0; i < B->count; ++i) stats[i].ms_total = wall_ms() - t0;
    return rc;
}

int fts_batch_solve(fts_batch* B, const double* const* phi, const double* const* source,
                    const double* const* mu, double* const* flow, fts_stats* stats) {
    return batch_solve_common(B, phi, source, mu, flow, stats, false);
}

int fts_batch_solve_device(fts_batch* B, const double* const* phi, const double* const* source,
                           const double* const* mu, double* const* flow, fts_stats* stats) {
    return batch_solve_common(B, phi, source, mu, flow, stats, true);
}

int fts_batch_get_config(const fts_batch* B, fts_batch_config* cfg) {
    if (!B || !cfg) return FTS_ERR_BAD_INPUT;
    *cfg = B->cfg;
    cfg->graph = B->graph ? 1 : 0;
    return FTS_OK;
}

int fts_batch_set_barrier_limit(fts_batch* B, double seconds, int32_t absent_block) {
    if (!B || !(seconds > 0.0) || seconds > 3600.0 || absent_block < -1)
        return FTS_ERR_BAD_INPUT;
    try {
        FTS_CUDA(cudaSetDevice(B->device));
        const BarrierState cfg =
            barrier_config((unsigned long long)(seconds * 1e9), (int)absent_block);
        // the whole state: no launch is in flight once the stream has drained
        FTS_CUDA(cudaStreamSynchronize(B->stream));
        FTS_CUDA(cudaMemcpyAsync(B->d_bar, &cfg, sizeof(cfg), cudaMemcpyHostToDevice, B->stream));
        FTS_CUDA(cudaStreamSynchronize(B->stream));
    } catch (const CudaError& e) {
        B->last_error = e.what;
        return FTS_ERR_CUDA;
    }
    return FTS_OK;
}

int fts_batch_set_stream(fts_batch* B, void* stream) {
    if (!B) return FTS_ERR_BAD_INPUT;
    B->stream = stream ? static_cast<cudaStream_t>(stream) : B->own_stream;
    if (B->graph) {
        cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;
    }
    return FTS_OK;
}

const char* fts_batch_last_error(const fts_batch* B) {
    return B ? B->last_error.c_str() : g_batch_error().c_str();
}

void fts_batch_destroy(fts_batch* B) {
    if (!B) return;
    cudaSetDevice(B->device);
    if (B->stream) cudaStreamSynchronize(B->stream);
    batch_free(*B);
    delete B;
}

}  // extern "C"
