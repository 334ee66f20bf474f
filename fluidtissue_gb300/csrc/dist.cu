// Distance reset of the level set (EuclideanDistance::resetPhi,
// src/fem/EuclideanDistance.cu:45-118): phi_n[k] = +-min_j |ifp_j - p_k|.
//
// The reference runs one thread per mesh node over ALL interface points
// (O(np * n_ifp), every point re-read from global memory by every thread).
// Here the points are binned on the device into the cells of a 64^3 grid
// over their bounding box, cells in Morton order (a counting sort: histogram,
// scan, scatter), and cut into blocks of 32 with bounding boxes, and blocks of
// 32 blocks with their own boxes.  The nodes are taken in Morton order (once
// per mesh) by CTAs of 256, which share a sorted candidate list of blocks
// (k_dist_cta); a thread scans only the candidate blocks whose box is within
// its running threshold, and takes norm3df, the reference's distance, of every
// point within a relative margin of the running minimum squared distance, so
// the result is the same float as the exhaustive minimum of norm3df values
// (the margin covers the few-ulp difference between the squared-distance
// order and the norm3df order).  The exhaustive kernel (the reference's
// algorithm) is kept for comparison and for bit-exact parity tests.
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

// 10-bit Morton interleave.
__host__ __device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Float bits with the sign folded (negatives inverted, positives with the top
// bit set): unsigned order is the order of the numbers.
__device__ __forceinline__ unsigned fkey(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

constexpr int kCellBits = 6;  // cells per axis of the binning grid: 64
constexpr int kCells = 1 << (3 * kCellBits);
constexpr int kScanThreads = 1024;

// Bounding box of the points: keys[0..2] minima, keys[3..5] maxima (set to
// all ones / zero before).
__global__ void k_pts_box(int32_t n, const float* __restrict__ raw, unsigned* __restrict__ keys) {
    unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) {
            const unsigned k = fkey(raw[3 * (int64_t)j + c]);
            lo[c] = min(lo[c], k);
            hi[c] = max(hi[c], k);
        }
    for (int c = 0; c < 3; ++c) {
        lo[c] = __reduce_min_sync(0xffffffffu, lo[c]);
        hi[c] = __reduce_max_sync(0xffffffffu, hi[c]);
    }
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; ++c) {
            atomicMin(keys + c, lo[c]);
            atomicMax(keys + 3 + c, hi[c]);
        }
}

// Cell of each point (Morton code of its 6-bit grid coordinates) and the
// cell histogram.
__global__ void k_pts_cells(int32_t n, const float* __restrict__ raw,
                            const unsigned* __restrict__ keys, uint32_t* __restrict__ cell,
                            uint32_t* __restrict__ counts) {
    float lo[3], sc[3];
    for (int c = 0; c < 3; ++c) {
        lo[c] = fkey_inv(keys[c]);
        const float hi = fkey_inv(keys[3 + c]);
        sc[c] = hi > lo[c] ? (float)(1 << kCellBits) / (hi - lo[c]) : 0.f;
    }
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t code = 0;
        for (int c = 0; c < 3; ++c) {
            const float w = (raw[3 * (int64_t)j + c] - lo[c]) * sc[c];
            const uint32_t q = (uint32_t)fminf(fmaxf(w, 0.f), (float)((1 << kCellBits) - 1));
            code |= spread10(q) << c;
        }
        cell[j] = code;
        atomicAdd(counts + code, 1u);
    }
}

// Exclusive scan of the kCells counts in place, one CTA: each warp scans a
// contiguous chunk of kCells / 32 counts in steps of 32 (coalesced), after the
// chunk totals have been scanned across the warps.
__global__ void __launch_bounds__(kScanThreads) k_cells_scan(uint32_t* __restrict__ counts) {
    __shared__ uint32_t wsum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int kChunk = kCells / (kScanThreads / 32);
    uint32_t* base = counts + (size_t)w * kChunk;
    uint32_t t = 0;
    for (int i = lane; i < kChunk; i += 32) t += base[i];
    t = __reduce_add_sync(0xffffffffu, t);
    if (lane == 0) wsum[w] = t;
    __syncthreads();
    if (w == 0) {
        uint32_t v = wsum[lane], x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wsum[lane] = x - v;  // exclusive
    }
    __syncthreads();
    uint32_t carry = wsum[w];
    for (int i0 = 0; i0 < kChunk; i0 += 32) {
        const uint32_t v = base[i0 + lane];
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        base[i0 + lane] = carry + x - v;
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
}

// Scatter the points to their cell's range (order within a cell is that of
// the atomics: the minimum over a fixed set does not depend on it).
__global__ void k_pts_scatter(int32_t n, const float* __restrict__ raw,
                              const uint32_t* __restrict__ cell, uint32_t* __restrict__ cursor,
                              float4* __restrict__ pts) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t at = atomicAdd(cursor + cell[j], 1u);
        pts[at] = make_float4(raw[3 * (int64_t)j], raw[3 * (int64_t)j + 1],
                              raw[3 * (int64_t)j + 2], 0.f);
    }
}

// Block and super-block boxes: one warp per super-block, one lane per point
// of each of its blocks; the last block is padded to 32 points.
__global__ void k_block_boxes(int32_t n, float4* __restrict__ pts, int32_t nb, int32_t ns,
                              float4* __restrict__ blo, float4* __restrict__ bhi,
                              float4* __restrict__ slo, float4* __restrict__ shi) {
    const int lane = threadIdx.x & 31;
    for (int32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ns;
         t += (gridDim.x * blockDim.x) >> 5) {
        float4 sl = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
        float4 sh = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
        const int32_t b1 = min(nb, (t + 1) * 32);
        for (int32_t b = t * 32; b < b1; ++b) {
            const int32_t j = b * 32 + lane;
            float4 l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
            float4 h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
            if (j < n) {
                l = pts[j];
                h = l;
                l.w = h.w = 0.f;
            } else {  // pad the last block to 32 with points at +inf
                pts[j] = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
            }
            for (int o = 16; o > 0; o >>= 1) {
                l.x = fminf(l.x, __shfl_xor_sync(0xffffffffu, l.x, o));
                l.y = fminf(l.y, __shfl_xor_sync(0xffffffffu, l.y, o));
                l.z = fminf(l.z, __shfl_xor_sync(0xffffffffu, l.z, o));
                h.x = fmaxf(h.x, __shfl_xor_sync(0xffffffffu, h.x, o));
                h.y = fmaxf(h.y, __shfl_xor_sync(0xffffffffu, h.y, o));
                h.z = fmaxf(h.z, __shfl_xor_sync(0xffffffffu, h.z, o));
            }
            if (lane == 0) {
                blo[b] = l;
                bhi[b] = h;
            }
            sl.x = fminf(sl.x, l.x);
            sl.y = fminf(sl.y, l.y);
            sl.z = fminf(sl.z, l.z);
            sh.x = fmaxf(sh.x, h.x);
            sh.y = fmaxf(sh.y, h.y);
            sh.z = fmaxf(sh.z, h.z);
        }
        if (lane == 0) {
            slo[t] = sl;
            shi[t] = sh;
        }
    }
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

// Cooperative pruned search, one pass.  Each CTA takes kCtaNodes nodes in
// Morton order (a compact brick), so their candidate points are shared: the
// CTA bounds its nodes' box, scans a block near that box (the nearest block of
// the nearest super-block), whose values give an upper bound U of every node's
// threshold (below), keeps the blocks whose box lies within U of the node box,
// sorts them by that distance (bitonic, in shared memory) and each thread
// walks the sorted list until the box distance passes its own threshold.
//
// Exactness in one pass: a thread keeps thr = min_j fl(sq_j (1 + margin))
// over the points seen (= fl(best (1 + margin)) by monotone rounding, best =
// the minimum squared distance so far) and takes norm3df of every point with
// sq <= thr at the time it is seen.  thr only decreases, so every point within
// the margin of the final minimum, among them the point with the smallest
// norm3df (the margin covers the ulps between the two orders), is evaluated;
// blocks and the walk are cut at thr, never below it.  The minimum of norm3df
// over a superset of those points that holds only real points is the
// exhaustive minimum, the same float.
constexpr int kCtaNodes = 256;
constexpr int kCandCap = 2048;

__device__ __forceinline__ float boxbox_dist2(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    const float dx = fmaxf(fmaxf(blo.x - ahi.x, alo.x - bhi.x), 0.f);
    const float dy = fmaxf(fmaxf(blo.y - ahi.y, alo.y - bhi.y), 0.f);
    const float dz = fmaxf(fmaxf(blo.z - ahi.z, alo.z - bhi.z), 0.f);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// One block of 32 points (padded with points at +inf, whose sq is inf and
// never passes thr <= FLT_MAX).  First the block's minimum squared distance;
// only if it is within thr, the update thr = min(thr, fl(bmin (1 + margin)))
// (= the running minimum of fl(sq (1 + margin)) over the block's points) and
// the norm3df evaluations of the points with sq <= thr.
__device__ __forceinline__ void scan_block(const float4* q32, float px, float py, float pz,
                                           float& thr, float& dmin) {
    float bmin = INFINITY;
#pragma unroll 8
    for (int j = 0; j < kDistBlock; ++j) {
        const float4 q = q32[j];
        const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
        bmin = fminf(bmin, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    }
    if (bmin <= thr) {
        thr = fminf(thr, bmin * (1.f + kDistMargin));
#pragma unroll 4
        for (int j = 0; j < kDistBlock; ++j) {
            const float4 q = q32[j];
            const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
            if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= thr) dmin = fminf(dmin, norm3df(dx, dy, dz));
        }
    }
}

__global__ void __launch_bounds__(kCtaNodes)
k_dist_cta(int64_t np, const int32_t* __restrict__ order, const float* __restrict__ xyz,
           const float4* __restrict__ pts, int32_t n_ifp, const float4* __restrict__ blo,
           const float4* __restrict__ bhi, int32_t nb, const float4* __restrict__ slo,
           const float4* __restrict__ shi, int32_t ns, double* __restrict__ phi,
           unsigned long long* __restrict__ scanned) {
    __shared__ unsigned long long cand[kCandCap];
    __shared__ float4 stage[kCtaNodes / 32][32];  // one block of points per warp
    __shared__ unsigned long long seed;
    __shared__ unsigned int ubits;
    __shared__ int ncand;
    __shared__ unsigned kmin[3], kmax[3];  // node box as order keys
    __shared__ float bmin[3], bmax[3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
        {  // node box
            const float p[3] = {px, py, pz};
            for (int a = 0; a < 3; ++a) {
                unsigned lo = active ? fkey(p[a]) : 0xffffffffu, hi = active ? fkey(p[a]) : 0u;
                lo = __reduce_min_sync(0xffffffffu, lo);
                hi = __reduce_max_sync(0xffffffffu, hi);
                if (lane == 0) {
                    atomicMin(&kmin[a], lo);
                    atomicMax(&kmax[a], hi);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            bmin[threadIdx.x] = fkey_inv(kmin[threadIdx.x]);
            bmax[threadIdx.x] = fkey_inv(kmax[threadIdx.x]);
        }
        __syncthreads();
        const float4 clo = make_float4(bmin[0], bmin[1], bmin[2], 0.f);
        const float4 chi = make_float4(bmax[0], bmax[1], bmax[2], 0.f);
        if (warp == 0) {  // seed: the nearest block of the super-block nearest to the node box
            unsigned long long key = ~0ull;
            for (int32_t t = lane; t < ns; t += 32) {
                const float d = boxbox_dist2(clo, chi, __ldg(slo + t), __ldg(shi + t));
                key = min(key, ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)t);
            }
            for (int o = 16; o > 0; o >>= 1) key = min(key, __shfl_xor_sync(0xffffffffu, key, o));
            const int32_t b = (int32_t)(key & 0xffffffffull) * kDistSuper + lane;
            key = ~0ull;
            if (b < nb) {
                const float d = boxbox_dist2(clo, chi, __ldg(blo + b), __ldg(bhi + b));
                key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)b;
            }
            for (int o = 16; o > 0; o >>= 1) key = min(key, __shfl_xor_sync(0xffffffffu, key, o));
            if (lane == 0) seed = key;
        }
        __syncthreads();
        const int32_t sb = (int32_t)(seed & 0xffffffffull);
        float thr = FLT_MAX, dmin = FLT_MAX;
        if (active) {
            scan_block(pts + (int64_t)sb * kDistBlock, px, py, pz, thr, dmin);
            mine += (unsigned long long)(min(n_ifp, (sb + 1) * kDistBlock) - sb * kDistBlock);
        }
        {
            unsigned u = active ? __float_as_uint(thr) : 0u;  // non-negative: bits order
            u = __reduce_max_sync(0xffffffffu, u);
            if (lane == 0) atomicMax(&ubits, u);
        }
        __syncthreads();
        const float U = __uint_as_float(ubits);
        // candidates within U of the node box: a warp per super-block, a lane
        // per block, appended in ballot order
        for (int32_t t = warp; t < ns; t += kCtaNodes / 32) {
            if (boxbox_dist2(clo, chi, __ldg(slo + t), __ldg(shi + t)) > U) continue;
            const int32_t b = t * kDistSuper + lane;
            float d = FLT_MAX;
            bool keep = false;
            if (b < nb && b != sb) {
                d = boxbox_dist2(clo, chi, __ldg(blo + b), __ldg(bhi + b));
                keep = d <= U;
            }
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            int base = 0;
            if (lane == 0 && m) base = atomicAdd(&ncand, __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (keep) {
                const int at = base + __popc(m & ((1u << lane) - 1u));
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
                for (int q = threadIdx.x; q < (m >> 1); q += blockDim.x) {  // one pair each
                    const int i = ((q & ~(jj - 1)) << 1) | (q & (jj - 1)), l = i + jj;
                    const unsigned long long a = cand[i], b = cand[l];
                    if ((a > b) == ((i & kk) == 0)) {
                        cand[i] = b;
                        cand[l] = a;
                    }
                }
                __syncthreads();
            }
        // the walk, warp-uniform, in groups of 32 candidates: one lane per
        // candidate tests its block against the warp's node box and the
        // largest threshold of the warp; the blocks that pass are taken in
        // list order, and one that some lane needs is staged once (one
        // coalesced load) and read back as a broadcast from shared memory (the
        // next passing block's points are loaded ahead, into a register).
        float4 wlo, whi;
        {
            unsigned kl[3], kh[3];
            const float p[3] = {px, py, pz};
            for (int a = 0; a < 3; ++a) {
                kl[a] = __reduce_min_sync(0xffffffffu, active ? fkey(p[a]) : 0xffffffffu);
                kh[a] = __reduce_max_sync(0xffffffffu, active ? fkey(p[a]) : 0u);
            }
            wlo = make_float4(fkey_inv(kl[0]), fkey_inv(kl[1]), fkey_inv(kl[2]), 0.f);
            whi = make_float4(fkey_inv(kh[0]), fkey_inv(kh[1]), fkey_inv(kh[2]), 0.f);
        }
        const bool warp_live = __any_sync(0xffffffffu, active);
        int32_t pre_b = -1;
        float4 pre = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int g = 0; warp_live && g < nc; g += 32) {
            // thresholds are non-negative: their bits order like the numbers
            const float tmax =
                __uint_as_float(__reduce_max_sync(0xffffffffu, active ? __float_as_uint(thr) : 0u));
            if (__uint_as_float((unsigned)(cand[g] >> 32)) > tmax) break;
            int32_t bl = -1;
            bool look = false;
            if (g + lane < nc) {
                const unsigned long long key = cand[g + lane];
                bl = (int32_t)(key & 0xffffffffull);
                look = __uint_as_float((unsigned)(key >> 32)) <= tmax &&
                       boxbox_dist2(wlo, whi, __ldg(blo + bl), __ldg(bhi + bl)) <= tmax;
            }
            unsigned m = __ballot_sync(0xffffffffu, look);
            while (m) {
                const int32_t b = __shfl_sync(0xffffffffu, bl, __ffs(m) - 1);
                m &= m - 1;
                const bool need =
                    active && box_dist2(__ldg(blo + b), __ldg(bhi + b), px, py, pz) <= thr;
                if (__ballot_sync(0xffffffffu, need) == 0u) continue;
                const float4 v = pre_b == b ? pre : __ldg(pts + (int64_t)b * kDistBlock + lane);
                if (m) {
                    pre_b = __shfl_sync(0xffffffffu, bl, __ffs(m) - 1);
                    pre = __ldg(pts + (int64_t)pre_b * kDistBlock + lane);
                }
                __syncwarp();
                stage[warp][lane] = v;
                __syncwarp();
                if (need) {
                    scan_block(stage[warp], px, py, pz, thr, dmin);
                    mine += (unsigned long long)(min(n_ifp, (b + 1) * kDistBlock) - b * kDistBlock);
                }
            }
        }
        if (active) {
            double out = dmin;
            if (phi[k] < 0.0f) out = -out;
            phi[k] = out;
        }
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if (lane == 0 && mine) atomicAdd(scanned, mine);
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
    int64_t cap = 0;            // points the buffers below hold
    float* raw = nullptr;       // [3 cap] points as the caller gave them (host uploads)
    uint32_t* cell = nullptr;   // [cap] binning cell of each point
    float4* pts = nullptr;      // [32 nbc] points binned by cell, padded with +inf points
    float4* boxes = nullptr;    // block boxes lo[nbc], hi[nbc], super-block lo[nsc], hi[nsc]
    uint32_t* counts = nullptr; // [kCells] cell histogram, then cursors
    unsigned* keys = nullptr;   // [6] bounding box of the points as order keys
    unsigned long long* scanned = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::string last_error;
};

namespace {

void dist_free(fts_dist& D) {
    for (void* p : {(void*)D.xyz, (void*)D.order, (void*)D.phi, (void*)D.raw, (void*)D.cell,
                    (void*)D.pts, (void*)D.boxes, (void*)D.counts, (void*)D.keys,
                    (void*)D.scanned})
        if (p) cudaFree(p);
    for (auto& e : D.ev)
        if (e) cudaEventDestroy(e);
    if (D.stream) cudaStreamDestroy(D.stream);
}

}  // namespace

namespace fts {

static int64_t blocks_for(int64_t n) { return (n + kDistBlock - 1) / kDistBlock; }
static int64_t supers_for(int64_t n) { return (blocks_for(n) + kDistSuper - 1) / kDistSuper; }

// The reset on device-resident phi, stream-ordered: the points (host or
// device, ifp_on_device) are binned on the device and searched; no host wait
// unless the buffers grow or st asks for the scan count.  Events: D->ev[0]
// before the binning, D->ev[1] before the search kernel, D->ev[2] after it.
void dist_reset_device(fts_dist* D, const float* ifp, bool ifp_on_device, int32_t n_ifp,
                       double* phi_dev, int32_t method, cudaStream_t s, fts_dist_stats* st) {
    const int64_t np = D->np;
    const int grid = (int)std::min<int64_t>((np + 255) / 256, (int64_t)D->num_sms * 8);
    if (n_ifp == 0) {  // the reference's minimum over no point: FLT_MAX
        k_dist_exhaustive<<<grid, 256, 0, s>>>(np, D->xyz, nullptr, 0, phi_dev);
        FTS_CUDA(cudaGetLastError());
        return;
    }
    const double t0 = wall_ms();
    if (n_ifp > D->cap) {
        // the previous buffers may still be read by queued work: wait first
        FTS_CUDA(cudaStreamSynchronize(s));
        for (void** p : {(void**)&D->raw, (void**)&D->cell, (void**)&D->pts, (void**)&D->boxes}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        D->cap = 0;
        // room to grow by a quarter (the interface point count drifts per step)
        const int64_t cap = n_ifp + n_ifp / 4;
        FTS_CUDA(cudaMalloc(&D->raw, 3 * (size_t)cap * sizeof(float)));
        FTS_CUDA(cudaMalloc(&D->cell, (size_t)cap * sizeof(uint32_t)));
        FTS_CUDA(cudaMalloc(&D->pts, (size_t)blocks_for(cap) * kDistBlock * sizeof(float4)));
        FTS_CUDA(cudaMalloc(&D->boxes, 2 * (size_t)(blocks_for(cap) + supers_for(cap)) * sizeof(float4)));
        D->cap = cap;
    }
    const float* raw = ifp;
    if (!ifp_on_device) {  // pageable source: taken by the time the call returns
        FTS_CUDA(cudaMemcpyAsync(D->raw, ifp, 3 * (size_t)n_ifp * sizeof(float),
                                 cudaMemcpyHostToDevice, s));
        raw = D->raw;
    }
    const int32_t nb = (int32_t)blocks_for(n_ifp), ns = (int32_t)supers_for(n_ifp);
    const int64_t nbc = blocks_for(D->cap);
    float4* blo = D->boxes;
    float4* bhi = blo + nbc;
    float4* slo = bhi + nbc;
    float4* shi = slo + supers_for(D->cap);
    FTS_CUDA(cudaMemsetAsync(D->scanned, 0, sizeof(unsigned long long), s));
    FTS_CUDA(cudaEventRecord(D->ev[0], s));
    if (method == FTS_DIST_EXHAUSTIVE) {
        FTS_CUDA(cudaEventRecord(D->ev[1], s));
        k_dist_exhaustive<<<grid, 256, 0, s>>>(np, D->xyz, raw, n_ifp, phi_dev);
    } else {
        const int pgrid = (int)std::min<int64_t>((n_ifp + 255) / 256, (int64_t)D->num_sms * 4);
        FTS_CUDA(cudaMemsetAsync(D->keys, 0xff, 3 * sizeof(unsigned), s));
        FTS_CUDA(cudaMemsetAsync(D->keys + 3, 0, 3 * sizeof(unsigned), s));
        FTS_CUDA(cudaMemsetAsync(D->counts, 0, kCells * sizeof(uint32_t), s));
        k_pts_box<<<pgrid, 256, 0, s>>>(n_ifp, raw, D->keys);
        k_pts_cells<<<pgrid, 256, 0, s>>>(n_ifp, raw, D->keys, D->cell, D->counts);
        k_cells_scan<<<1, kScanThreads, 0, s>>>(D->counts);
        k_pts_scatter<<<pgrid, 256, 0, s>>>(n_ifp, raw, D->cell, D->counts, D->pts);
        k_block_boxes<<<(ns + 7) / 8, 256, 0, s>>>(n_ifp, D->pts, nb, ns, blo, bhi, slo, shi);
        FTS_CUDA(cudaGetLastError());
        FTS_CUDA(cudaEventRecord(D->ev[1], s));
        const int cgrid = (int)std::min<int64_t>((np + kCtaNodes - 1) / kCtaNodes,
                                                 (int64_t)D->num_sms * 8);
        k_dist_cta<<<cgrid, kCtaNodes, 0, s>>>(np, D->order, D->xyz, D->pts, n_ifp, blo, bhi, nb,
                                               slo, shi, ns, phi_dev, D->scanned);
    }
    FTS_CUDA(cudaGetLastError());
    FTS_CUDA(cudaEventRecord(D->ev[2], s));
    if (st) {
        st->ms_setup = wall_ms() - t0;
        unsigned long long scanned = 0;
        FTS_CUDA(cudaMemcpyAsync(&scanned, D->scanned, sizeof(scanned), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        FTS_CUDA(cudaEventElapsedTime(&ms, D->ev[0], D->ev[1]));
        st->ms_setup += ms;
        FTS_CUDA(cudaEventElapsedTime(&ms, D->ev[1], D->ev[2]));
        st->ms_kernel = ms;
        st->blocks = method == FTS_DIST_EXHAUSTIVE ? 0 : nb;
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
        FTS_CUDA(cudaMalloc(&D->counts, kCells * sizeof(uint32_t)));
        FTS_CUDA(cudaMalloc(&D->keys, 6 * sizeof(unsigned)));
        FTS_CUDA(cudaMemcpy(D->xyz, xyz, 3 * np * sizeof(float), cudaMemcpyHostToDevice));
        // the nodes in Morton order (once per mesh): a CTA's nodes form a brick
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
        dist_reset_device(D, ifp, false, n_ifp, D->phi, method, s, &st);
        FTS_CUDA(cudaMemcpyAsync(phi_n, D->phi, D->np * sizeof(double), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
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
