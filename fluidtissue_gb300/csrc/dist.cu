// Distance reset of the level set (EuclideanDistance::resetPhi,
// src/fem/EuclideanDistance.cu:45-118): phi_n[k] = +-min_j |ifp_j - p_k|.
//
// The reference runs one thread per mesh node over ALL interface points
// (O(np * n_ifp), every point re-read from global memory by every thread).
// Here the points are sorted along a Morton curve (host, once per call) into
// blocks of 32 with bounding boxes, and blocks of 32 blocks with their own
// boxes; the nodes are taken in Morton order (once per mesh) by CTAs of 256,
// which share a sorted candidate list of blocks (k_dist_cta), and a thread
// scans only the candidate blocks whose box is closer than its current best.
// The first pass finds the minimum squared distance in float; a second pass
// re-evaluates every point within a relative margin of that minimum with
// norm3df, the reference's distance, so the result is the same float as the
// exhaustive minimum of norm3df values (the margin covers the few-ulp
// difference between the squared-distance order and the norm3df order).  The exhaustive kernel (the reference's algorithm) is kept for
// comparison and for bit-exact parity tests.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "fts_device.cuh"

namespace fts {

static std::string& g_dist_error() {
    static thread_local std::string e;
    return e;
}

constexpr int kDistBlock = 32;   // points per block
constexpr int kDistSuper = 32;   // blocks per super-block
constexpr float kDistMargin = 1e-5f;

__device__ __forceinline__ float box_dist2(const float4 lo, const float4 hi, float px, float py,
                                           float pz) {
    const float dx = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.f);
    const float dy = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.f);
    const float dz = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.f);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// The reference's kernel, restated: every node against every point.
__global__ void k_dist_exhaustive(int64_t np, const float* __restrict__ xyz,
                                  const float* __restrict__ ifp, int32_t n_ifp,
                                  double* __restrict__ phi) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < np;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float p0 = xyz[3 * k], p1 = xyz[3 * k + 1], p2 = xyz[3 * k + 2];
        float dmin = FLT_MAX;
        for (int32_t j = 0; j < n_ifp; ++j) {
            const float d = norm3df(ifp[3 * j] - p0, ifp[3 * j + 1] - p1, ifp[3 * j + 2] - p2);
            if (d < dmin) dmin = d;
        }
        double out = dmin;
        if (phi[k] < 0.0f) out = -out;
        phi[k] = out;
    }
}

// Per-node pruned search over all super-blocks (the fallback of k_dist_cta
// when a CTA's candidate list overflows).  pts: sorted points (x, y, z, 0);
// blo/bhi: block boxes; slo/shi: super-block boxes; nb blocks, ns super-blocks.
__device__ float pruned_node(float px, float py, float pz, const float4* __restrict__ pts,
                             int32_t n_ifp, const float4* __restrict__ blo,
                             const float4* __restrict__ bhi, int32_t nb,
                             const float4* __restrict__ slo, const float4* __restrict__ shi,
                             int32_t ns, unsigned long long& mine) {
    {
        float best = FLT_MAX;
        // seed: the super-block with the nearest box first
        int32_t s0 = 0;
        {
            float sb = FLT_MAX;
            for (int32_t s = 0; s < ns; ++s) {
                const float d = box_dist2(__ldg(slo + s), __ldg(shi + s), px, py, pz);
                if (d < sb) {
                    sb = d;
                    s0 = s;
                }
            }
        }
        // pass 1: minimum squared distance (super-block s0, then the others)
        for (int32_t t = 0; t < ns; ++t) {
            const int32_t s = t == 0 ? s0 : (t <= s0 ? t - 1 : t);
            if (box_dist2(__ldg(slo + s), __ldg(shi + s), px, py, pz) > best) continue;
            const int32_t b1 = min(nb, (s + 1) * kDistSuper);
            for (int32_t b = s * kDistSuper; b < b1; ++b) {
                if (box_dist2(__ldg(blo + b), __ldg(bhi + b), px, py, pz) > best) continue;
                const int32_t j1 = min(n_ifp, (b + 1) * kDistBlock);
                for (int32_t j = b * kDistBlock; j < j1; ++j) {
                    const float4 q = __ldg(pts + j);
                    const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                    best = fminf(best, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                }
                mine += (unsigned long long)(j1 - b * kDistBlock);
            }
        }
        // pass 2: norm3df over the candidates within the margin of the minimum
        const float thr = best * (1.f + kDistMargin);
        float dmin = FLT_MAX;
        for (int32_t s = 0; s < ns; ++s) {
            if (box_dist2(__ldg(slo + s), __ldg(shi + s), px, py, pz) > thr) continue;
            const int32_t b1 = min(nb, (s + 1) * kDistSuper);
            for (int32_t b = s * kDistSuper; b < b1; ++b) {
                if (box_dist2(__ldg(blo + b), __ldg(bhi + b), px, py, pz) > thr) continue;
                const int32_t j1 = min(n_ifp, (b + 1) * kDistBlock);
                for (int32_t j = b * kDistBlock; j < j1; ++j) {
                    const float4 q = __ldg(pts + j);
                    const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                    if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= thr) {
                        const float d = norm3df(dx, dy, dz);
                        if (d < dmin) dmin = d;
                    }
                }
            }
        }
        return dmin;
    }
}

// Cooperative pruned search.  Each CTA takes 256 nodes in Morton order (a
// compact brick), so their candidate points are shared: the CTA bounds its
// nodes' box, gets an upper bound U of every node's nearest squared distance
// from the block nearest to the box, keeps the blocks whose box lies within
// U (1 + margin) of the node box, sorts them by that distance (bitonic, in
// shared memory) and each thread walks the sorted list until the box
// distance passes its own best.  Pass 1 and pass 2 are those of the
// per-node search (same expressions), so the result is the same float.
constexpr int kCtaNodes = 256;
constexpr int kCandCap = 2048;

__device__ __forceinline__ float boxbox_dist2(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    const float dx = fmaxf(fmaxf(blo.x - ahi.x, alo.x - bhi.x), 0.f);
    const float dy = fmaxf(fmaxf(blo.y - ahi.y, alo.y - bhi.y), 0.f);
    const float dz = fmaxf(fmaxf(blo.z - ahi.z, alo.z - bhi.z), 0.f);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

__global__ void __launch_bounds__(kCtaNodes)
k_dist_cta(int64_t np, const int32_t* __restrict__ order, const float* __restrict__ xyz,
           const float4* __restrict__ pts, int32_t n_ifp, const float4* __restrict__ blo,
           const float4* __restrict__ bhi, int32_t nb, const float4* __restrict__ slo,
           const float4* __restrict__ shi, int32_t ns, double* __restrict__ phi,
           unsigned long long* __restrict__ scanned) {
    __shared__ unsigned long long cand[kCandCap];
    __shared__ unsigned long long seed;
    __shared__ unsigned int ubits;
    __shared__ int ncand;
    __shared__ unsigned kmin[3], kmax[3];  // node box as order-preserving keys
    __shared__ float bmin[3], bmax[3];
    unsigned long long mine = 0;
    const int64_t nchunks = (np + kCtaNodes - 1) / kCtaNodes;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t slot = c * kCtaNodes + threadIdx.x;
        const bool active = slot < np;
        const int32_t k = active ? order[slot] : 0;
        const float px = active ? xyz[3 * (int64_t)k] : 0.f;
        const float py = active ? xyz[3 * (int64_t)k + 1] : 0.f;
        const float pz = active ? xyz[3 * (int64_t)k + 2] : 0.f;
        if (threadIdx.x == 0) {
            for (int a = 0; a < 3; ++a) {
                kmin[a] = 0xffffffffu;
                kmax[a] = 0u;
            }
            seed = ~0ull;
            ubits = 0u;
            ncand = 0;
        }
        __syncthreads();
        // node box: the float bits with the sign folded (negatives inverted,
        // positives with the top bit set) order like the numbers
        if (active) {
            const float p[3] = {px, py, pz};
            for (int a = 0; a < 3; ++a) {
                const unsigned u = __float_as_uint(p[a]);
                const unsigned key = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
                atomicMin(&kmin[a], key);
                atomicMax(&kmax[a], key);
            }
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            const unsigned a = kmin[threadIdx.x], b = kmax[threadIdx.x];
            bmin[threadIdx.x] = __uint_as_float((a & 0x80000000u) ? (a & 0x7fffffffu) : ~a);
            bmax[threadIdx.x] = __uint_as_float((b & 0x80000000u) ? (b & 0x7fffffffu) : ~b);
        }
        __syncthreads();
        const float4 clo = make_float4(bmin[0], bmin[1], bmin[2], 0.f);
        const float4 chi = make_float4(bmax[0], bmax[1], bmax[2], 0.f);
        // seed: the block nearest to the node box
        for (int32_t b = threadIdx.x; b < nb; b += blockDim.x) {
            const float d = boxbox_dist2(clo, chi, __ldg(blo + b), __ldg(bhi + b));
            atomicMin(&seed, ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)b);
        }
        __syncthreads();
        float best = FLT_MAX;
        if (active) {
            const int32_t b = (int32_t)(seed & 0xffffffffull);
            const int32_t j1 = min(n_ifp, (b + 1) * kDistBlock);
            for (int32_t j = b * kDistBlock; j < j1; ++j) {
                const float4 q = __ldg(pts + j);
                const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                best = fminf(best, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
            }
            mine += (unsigned long long)(j1 - b * kDistBlock);
            atomicMax(&ubits, __float_as_uint(best));  // non-negative: bits order
        }
        __syncthreads();
        const float U = __uint_as_float(ubits) * (1.f + kDistMargin);
        // candidates: super-blocks, then their blocks, within U of the node box
        for (int32_t t = threadIdx.x; t < ns; t += blockDim.x) {
            if (boxbox_dist2(clo, chi, __ldg(slo + t), __ldg(shi + t)) > U) continue;
            const int32_t b1 = min(nb, (t + 1) * kDistSuper);
            for (int32_t b = t * kDistSuper; b < b1; ++b) {
                const float d = boxbox_dist2(clo, chi, __ldg(blo + b), __ldg(bhi + b));
                if (d > U) continue;
                const int at = atomicAdd(&ncand, 1);
                if (at < kCandCap)
                    cand[at] = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)b;
            }
        }
        __syncthreads();
        const int nc = ncand;
        if (nc > kCandCap) {  // too many: the per-node search for this chunk
            if (active) {
                const float d = pruned_node(px, py, pz, pts, n_ifp, blo, bhi, nb, slo, shi, ns,
                                            mine);
                double out = d;
                if (phi[k] < 0.0f) out = -out;
                phi[k] = out;
            }
            __syncthreads();
            continue;
        }
        // bitonic sort of the candidates (padded to a power of two)
        int m = 1;
        while (m < nc) m <<= 1;
        for (int i = nc + threadIdx.x; i < m; i += blockDim.x) cand[i] = ~0ull;
        __syncthreads();
        for (int kk = 2; kk <= m; kk <<= 1)
            for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                for (int i = threadIdx.x; i < m; i += blockDim.x) {
                    const int l = i ^ jj;
                    if (l > i) {
                        const unsigned long long a = cand[i], b = cand[l];
                        const bool up = (i & kk) == 0;
                        if ((a > b) == up) {
                            cand[i] = b;
                            cand[l] = a;
                        }
                    }
                }
                __syncthreads();
            }
        if (active) {
            // pass 1: minimum squared distance over the sorted candidates
            for (int i = 0; i < nc; ++i) {
                const unsigned long long key = cand[i];
                if (__uint_as_float((unsigned)(key >> 32)) > best) break;
                const int32_t b = (int32_t)(key & 0xffffffffull);
                if (box_dist2(__ldg(blo + b), __ldg(bhi + b), px, py, pz) > best) continue;
                const int32_t j1 = min(n_ifp, (b + 1) * kDistBlock);
                for (int32_t j = b * kDistBlock; j < j1; ++j) {
                    const float4 q = __ldg(pts + j);
                    const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                    best = fminf(best, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                }
                mine += (unsigned long long)(j1 - b * kDistBlock);
            }
            // pass 2: norm3df over the points within the margin of the minimum
            const float thr = best * (1.f + kDistMargin);
            float dmin = FLT_MAX;
            for (int i = 0; i < nc; ++i) {
                const unsigned long long key = cand[i];
                if (__uint_as_float((unsigned)(key >> 32)) > thr) break;
                const int32_t b = (int32_t)(key & 0xffffffffull);
                if (box_dist2(__ldg(blo + b), __ldg(bhi + b), px, py, pz) > thr) continue;
                const int32_t j1 = min(n_ifp, (b + 1) * kDistBlock);
                for (int32_t j = b * kDistBlock; j < j1; ++j) {
                    const float4 q = __ldg(pts + j);
                    const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                    if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= thr) {
                        const float d = norm3df(dx, dy, dz);
                        if (d < dmin) dmin = d;
                    }
                }
            }
            double out = dmin;
            if (phi[k] < 0.0f) out = -out;
            phi[k] = out;
        }
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(scanned, mine);
}

}  // namespace fts

using namespace fts;

struct fts_dist {
    int device = 0;
    int num_sms = 148;
    cudaStream_t stream = nullptr;
    int64_t np = 0;
    float* xyz = nullptr;
    int32_t* order = nullptr;  // nodes in Morton order of their coordinates
    double* phi = nullptr;
    float* buf = nullptr;     // points: sorted float4 (pruned) or the raw float3 list
    size_t buf_cap = 0;       // floats
    unsigned long long* scanned = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::string last_error;
};

namespace {

void dist_free(fts_dist& D) {
    for (void* p : {(void*)D.xyz, (void*)D.order, (void*)D.phi, (void*)D.buf, (void*)D.scanned})
        if (p) cudaFree(p);
    for (auto& e : D.ev)
        if (e) cudaEventDestroy(e);
    if (D.stream) cudaStreamDestroy(D.stream);
}

// 10-bit Morton interleave of (x, y, z) quantised to the box.
uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

}  // namespace

namespace fts {

// The reset on device-resident phi (stream-ordered, no host wait): host sort
// of the points, upload, kernel.  Records the kernel between D->ev[0] and
// D->ev[1]; points_scanned is read back only by the caller that waits.
void dist_reset_device(fts_dist* D, const float* ifp, int32_t n_ifp, double* phi_dev,
                       int32_t method, cudaStream_t s, fts_dist_stats* st) {
    const int64_t np = D->np;
    const int grid = (int)std::min<int64_t>((np + 255) / 256, (int64_t)D->num_sms * 8);
    if (n_ifp == 0) {  // the reference's minimum over no point: FLT_MAX
        k_dist_exhaustive<<<grid, 256, 0, s>>>(np, D->xyz, nullptr, 0, phi_dev);
        FTS_CUDA(cudaGetLastError());
        return;
    }
    const double t0 = wall_ms();
    int32_t nb = 0, ns = 0;
    size_t need = 0;
    std::vector<float> host;
    if (method == FTS_DIST_EXHAUSTIVE) {
        need = 3 * (size_t)n_ifp;
    } else {
        // Morton order of the points within their bounding box
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int32_t j = 0; j < n_ifp; ++j)
            for (int c = 0; c < 3; ++c) {
                lo[c] = std::min(lo[c], ifp[3 * j + c]);
                hi[c] = std::max(hi[c], ifp[3 * j + c]);
            }
        std::vector<std::pair<uint32_t, int32_t>> key(n_ifp);
        for (int32_t j = 0; j < n_ifp; ++j) {
            uint32_t q[3];
            for (int c = 0; c < 3; ++c) {
                const float w = hi[c] > lo[c] ? (ifp[3 * j + c] - lo[c]) / (hi[c] - lo[c]) : 0.f;
                q[c] = (uint32_t)std::min(1023.f, std::max(0.f, w * 1023.f));
            }
            key[j] = {spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2), j};
        }
        std::sort(key.begin(), key.end());
        nb = (n_ifp + kDistBlock - 1) / kDistBlock;
        ns = (nb + kDistSuper - 1) / kDistSuper;
        // layout: pts[n_ifp] float4, blo[nb], bhi[nb], slo[ns], shi[ns] (float4 each)
        need = 4 * ((size_t)n_ifp + 2 * (size_t)nb + 2 * (size_t)ns);
        host.assign(need, 0.f);
        float* pts = host.data();
        float* blo = pts + 4 * (size_t)n_ifp;
        float* bhi = blo + 4 * (size_t)nb;
        float* slo = bhi + 4 * (size_t)nb;
        float* shi = slo + 4 * (size_t)ns;
        for (int32_t j = 0; j < n_ifp; ++j)
            for (int c = 0; c < 3; ++c) pts[4 * j + c] = ifp[3 * key[j].second + c];
        for (int32_t b = 0; b < nb; ++b) {
            for (int c = 0; c < 3; ++c) {
                blo[4 * b + c] = FLT_MAX;
                bhi[4 * b + c] = -FLT_MAX;
            }
            for (int32_t j = b * kDistBlock; j < std::min(n_ifp, (b + 1) * kDistBlock); ++j)
                for (int c = 0; c < 3; ++c) {
                    blo[4 * b + c] = std::min(blo[4 * b + c], pts[4 * j + c]);
                    bhi[4 * b + c] = std::max(bhi[4 * b + c], pts[4 * j + c]);
                }
        }
        for (int32_t t = 0; t < ns; ++t) {
            for (int c = 0; c < 3; ++c) {
                slo[4 * t + c] = FLT_MAX;
                shi[4 * t + c] = -FLT_MAX;
            }
            for (int32_t b = t * kDistSuper; b < std::min(nb, (t + 1) * kDistSuper); ++b)
                for (int c = 0; c < 3; ++c) {
                    slo[4 * t + c] = std::min(slo[4 * t + c], blo[4 * b + c]);
                    shi[4 * t + c] = std::max(shi[4 * t + c], bhi[4 * b + c]);
                }
        }
    }
    if (need > D->buf_cap) {
        // the previous contents may still be read by queued work: wait first
        FTS_CUDA(cudaStreamSynchronize(s));
        if (D->buf) cudaFree(D->buf);
        D->buf = nullptr;
        FTS_CUDA(cudaMalloc(&D->buf, need * sizeof(float)));
        D->buf_cap = need;
    }
    const float* src = method == FTS_DIST_EXHAUSTIVE ? ifp : host.data();
    FTS_CUDA(cudaMemcpyAsync(D->buf, src, need * sizeof(float), cudaMemcpyHostToDevice, s));
    // the pageable source must stay valid until the copy has been taken
    if (method != FTS_DIST_EXHAUSTIVE) FTS_CUDA(cudaStreamSynchronize(s));
    FTS_CUDA(cudaMemsetAsync(D->scanned, 0, sizeof(unsigned long long), s));
    if (st) st->ms_setup = wall_ms() - t0;
    FTS_CUDA(cudaEventRecord(D->ev[0], s));
    if (method == FTS_DIST_EXHAUSTIVE) {
        k_dist_exhaustive<<<grid, 256, 0, s>>>(np, D->xyz, D->buf, n_ifp, phi_dev);
    } else {
        const float4* pts = reinterpret_cast<const float4*>(D->buf);
        const float4* blo = pts + n_ifp;
        const float4* bhi = blo + nb;
        const float4* slo = bhi + nb;
        const float4* shi = slo + ns;
        const int cgrid = (int)std::min<int64_t>((np + kCtaNodes - 1) / kCtaNodes,
                                                 (int64_t)D->num_sms * 8);
        k_dist_cta<<<cgrid, kCtaNodes, 0, s>>>(np, D->order, D->xyz, pts, n_ifp, blo, bhi, nb,
                                               slo, shi, ns, phi_dev, D->scanned);
    }
    FTS_CUDA(cudaGetLastError());
    FTS_CUDA(cudaEventRecord(D->ev[1], s));
    if (st) {
        unsigned long long scanned = 0;
        FTS_CUDA(cudaMemcpyAsync(&scanned, D->scanned, sizeof(scanned), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        st->blocks = nb;
        st->points_scanned =
            method == FTS_DIST_EXHAUSTIVE ? np * (int64_t)n_ifp : (int64_t)scanned;
    }
}

}  // namespace fts

extern "C" {

int fts_dist_create(const float* xyz, int64_t np, int32_t device, fts_dist** out) {
    if (!xyz || np <= 0 || !out || np >= (int64_t)1 << 31) return FTS_ERR_BAD_INPUT;
    *out = nullptr;
    fts_dist* D = new (std::nothrow) fts_dist();
    if (!D) return FTS_ERR_OOM;
    D->device = device;
    D->np = np;
    int rc = FTS_OK;
    try {
        FTS_CUDA(cudaSetDevice(device));
        int sms = 0;
        FTS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        D->num_sms = sms > 0 ? sms : 148;
        FTS_CUDA(cudaStreamCreateWithFlags(&D->stream, cudaStreamNonBlocking));
        for (auto& e : D->ev) FTS_CUDA(cudaEventCreate(&e));
        FTS_CUDA(cudaMalloc(&D->xyz, 3 * np * sizeof(float)));
        FTS_CUDA(cudaMalloc(&D->phi, np * sizeof(double)));
        FTS_CUDA(cudaMalloc(&D->scanned, sizeof(unsigned long long)));
        FTS_CUDA(cudaMemcpy(D->xyz, xyz, 3 * np * sizeof(float), cudaMemcpyHostToDevice));
        // the nodes in Morton order (once per mesh): a CTA's 256 nodes form a brick
        {
            float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            for (int64_t k = 0; k < np; ++k)
                for (int c = 0; c < 3; ++c) {
                    lo[c] = std::min(lo[c], xyz[3 * k + c]);
                    hi[c] = std::max(hi[c], xyz[3 * k + c]);
                }
            std::vector<std::pair<uint32_t, int32_t>> key((size_t)np);
            for (int64_t k = 0; k < np; ++k) {
                uint32_t q[3];
                for (int c = 0; c < 3; ++c) {
                    const float w = hi[c] > lo[c] ? (xyz[3 * k + c] - lo[c]) / (hi[c] - lo[c]) : 0.f;
                    q[c] = (uint32_t)std::min(1023.f, std::max(0.f, w * 1023.f));
                }
                key[k] = {spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2),
                          (int32_t)k};
            }
            std::sort(key.begin(), key.end());
            std::vector<int32_t> ord((size_t)np);
            for (int64_t k = 0; k < np; ++k) ord[k] = key[k].second;
            FTS_CUDA(cudaMalloc(&D->order, np * sizeof(int32_t)));
            FTS_CUDA(cudaMemcpy(D->order, ord.data(), np * sizeof(int32_t), cudaMemcpyHostToDevice));
        }
    } catch (const CudaError& e) {
        g_dist_error() = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    }
    if (rc != FTS_OK) {
        dist_free(*D);
        delete D;
        return rc;
    }
    *out = D;
    return FTS_OK;
}

int fts_dist_reset(fts_dist* D, const float* ifp, int32_t n_ifp, double* phi_n, int32_t method,
                   fts_dist_stats* stats) {
    if (!D || !phi_n || n_ifp < 0 || (n_ifp > 0 && !ifp) ||
        (method != FTS_DIST_PRUNED && method != FTS_DIST_EXHAUSTIVE))
        return FTS_ERR_BAD_INPUT;
    const double t0 = wall_ms();
    fts_dist_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = FTS_OK;
    try {
        FTS_CUDA(cudaSetDevice(D->device));
        cudaStream_t s = D->stream;
        FTS_CUDA(cudaMemcpyAsync(D->phi, phi_n, D->np * sizeof(double), cudaMemcpyHostToDevice, s));
        dist_reset_device(D, ifp, n_ifp, D->phi, method, s, &st);
        FTS_CUDA(cudaMemcpyAsync(phi_n, D->phi, D->np * sizeof(double), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        if (n_ifp > 0) FTS_CUDA(cudaEventElapsedTime(&ms, D->ev[0], D->ev[1]));
        st.ms_kernel = ms;
    } catch (const CudaError& e) {
        D->last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        D->last_error = "host allocation failed";
        rc = FTS_ERR_OOM;
    }
    st.status = rc;
    st.ms_total = wall_ms() - t0;
    if (stats) *stats = st;
    return rc;
}

void fts_dist_destroy(fts_dist* D) {
    if (!D) return;
    cudaSetDevice(D->device);
    if (D->stream) cudaStreamSynchronize(D->stream);
    dist_free(*D);
    delete D;
}

const char* fts_dist_last_error(const fts_dist* D) {
    return D ? D->last_error.c_str() : g_dist_error().c_str();
}

}  // extern "C"
