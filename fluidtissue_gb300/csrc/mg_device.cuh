// Per-node bodies of the multigrid V-cycle (internal), shared by the
// single-solve kernels (mg.cu, krylov.cu) and the batched persistent kernel
// (batch.cu).  Lattice offsets are compile-time functions.
//
// Chebyshev smoothing of degree kSmooth on [lambda/10, lambda] of D^-1 K:
//   d_0 = D^-1 r_0 / theta;  r_s = r_{s-1} - K d_{s-1};
//   d_s = ca_s d_{s-1} + cb_s D^-1 r_s;  x_s = x_{s-1} + d_s.
// The first direction d_0 is pointwise, so it is produced together with the
// level's right-hand side (by the restriction, or by the preconditioner stage
// that writes the finest b) or with the post-smoothing residual; the x update
// of d_0 is deferred to the next step so that no kernel writes x while
// another thread of it reads x at a neighbour.
#pragma once

#include <type_traits>

#include "fts_device.cuh"

namespace fts {

// The 15 Kuhn directions: 0 = self, 1..7 = (1,0,0) (0,1,0) (0,0,1) (1,1,0)
// (1,0,1) (0,1,1) (1,1,1), 8..14 = their negatives.
__host__ __device__ __forceinline__ constexpr int off_x(int d) {
    return (d == 1 || d == 4 || d == 5 || d == 7) ? 1
                                                   : ((d == 8 || d == 11 || d == 12 || d == 14) ? -1 : 0);
}
__host__ __device__ __forceinline__ constexpr int off_y(int d) {
    return (d == 2 || d == 4 || d == 6 || d == 7) ? 1
                                                   : ((d == 9 || d == 11 || d == 13 || d == 14) ? -1 : 0);
}
__host__ __device__ __forceinline__ constexpr int off_z(int d) {
    return (d == 3 || d == 5 || d == 6 || d == 7) ? 1
                                                   : ((d == 10 || d == 12 || d == 13 || d == 14) ? -1 : 0);
}

// Tiled stencil layout: 32 consecutive nodes share one tile of kStored x 32
// values (entry q = 9 d + 3 r + c, d = 0..7), so the loads of a warp stay
// inside one contiguous region.
constexpr int kStored = 72;
__host__ __device__ __forceinline__ int64_t kidx(int q, int64_t v) {
    return ((v >> 5) * kStored + q) * 32 + (v & 31);
}

__device__ __forceinline__ int nbr(int i, int j, int k, int d, int n) {
    const int a = i + off_x(d), b = j + off_y(d), c = k + off_z(d);
    if (a < 0 || b < 0 || c < 0 || a >= n || b >= n || c >= n) return -1;
    return a + n * (b + n * c);
}

// Kuhn lattice in the generator's element order: element 6c + t of cube c is
// the monotone path 0 -> e_p0 -> e_p0 + e_p1 -> (1,1,1) of axis permutation t
// ({0,1,2} {0,2,1} {1,0,2} {1,2,0} {2,0,1} {2,1,0}), its local vertex a the
// corner at place a on the path.
__host__ __device__ __forceinline__ constexpr int kuhn_p0(int t) { return t >> 1; }
__host__ __device__ __forceinline__ constexpr int kuhn_p1(int t) {
    return (t == 0 || t == 5) ? 1 : ((t == 1 || t == 3) ? 2 : 0);
}

// The elements holding both v = (i, j, k) and w = v + off(d) (d = 0..7, w
// inside the lattice), in ascending element index (the order of the
// node-element map): f(el, a, b) with a, b the local indices of v and w.  The
// node's corner q in a cube (bits x, y, z) runs from 7 down to 0, which is
// ascending cube index; w is corner q | off(d) of that cube when the two
// share no bit; an element holds a corner when the corner lies on its path.
template <typename F>
__device__ __forceinline__ void kuhn_pair_elements(int n, int i, int j, int k, int d, F&& f) {
    const int m = n - 1;
    const int od = off_x(d) | (off_y(d) << 1) | (off_z(d) << 2);
#pragma unroll
    for (int q = 7; q >= 0; --q) {
        if (q & od) continue;
        const int ci = i - (q & 1), cj = j - ((q >> 1) & 1), ck = k - (q >> 2);
        if (ci < 0 || cj < 0 || ck < 0 || ci >= m || cj >= m || ck >= m) continue;
        const int64_t cube = ci + (int64_t)m * (cj + (int64_t)m * ck);
        const int qw = q | od;
        const int a = __popc(q), b = __popc(qw);
#pragma unroll
        for (int t = 0; t < 6; ++t) {
            const int c1 = 1 << kuhn_p0(t), c2 = c1 | (1 << kuhn_p1(t));
            const bool hv = q == 0 || q == 7 || q == c1 || q == c2;
            const bool hw = qw == 0 || qw == 7 || qw == c1 || qw == c2;
            if (hv && hw) f(6 * cube + t, a, b);
        }
    }
}

template <typename T>
__device__ __forceinline__ T ldk(const T* p) {
    return *p;
}
template <typename T>
__device__ __forceinline__ T ldk(const __half* p) {
    return (T)__half2float(*p);
}

// One level of a hierarchy as the kernels see it.
template <typename T>
struct LevelView {
    using KS = typename MGStore<T>::type;
    int n;
    int64_t N;
    const KS* K;
    const double* ks;    // stencil scale
    const T* Di;
    T* b;
    T* x;
    T* r;
    T* d0;
    T* d1;
    const uint8_t* mask;
    const double* coef;  // 1/theta, (ca_s, cb_s) for s >= 1
};

template <typename T>
inline LevelView<T> level_view(const MG<T>& mg, size_t l) {
    const MGLevel<T>& L = mg.L[l];
    return LevelView<T>{L.n, L.N, L.Kh, mg.scale + l, L.Di, L.b, L.x, L.r, L.d0, L.d1, L.mask,
                        mg.coef + l * kCoefStride};
}

// FP16 stencil layout: per node 9 groups of 8 halfs (16 B each), in tiles of
// 32 nodes: group d < 8 holds entries 0..7 (3r + c) of the block towards
// direction d, group 8 holds entry 8 of the 8 blocks.  A warp's load of one
// group is 512 contiguous bytes; a node's own blocks are 9 loads, a
// neighbour's block 2.  Index in 16-byte units.
__host__ __device__ __forceinline__ int64_t hidx(int g, int64_t v) {
    return ((v >> 5) * 9 + g) * 32 + (v & 31);
}

__device__ __forceinline__ void unpack8(const uint4& u, float f[8]) {
    const __half2* h = reinterpret_cast<const __half2*>(&u);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 a = __half22float2(h[k]);
        f[2 * k] = a.x;
        f[2 * k + 1] = a.y;
    }
}
__device__ __forceinline__ float half_at(const uint4& u, int k) {
    return __half2float(reinterpret_cast<const __half*>(&u)[k]);
}

// How a stencil body treats the lattice boundary.
enum : int {
    kSkChecked = 0,  // one body: a range check and a branch per neighbour
    kSkSplit = 1,    // interior nodes take a check-free body, the others the checked one
    kSkClamped = 2   // one branch-free body: a missing neighbour's loads go to the
                     // node itself and are weighted 0, so every load of the node
                     // can issue before the first use (latency-bound levels, where
                     // nearly every warp holds a boundary node)
};
// Per-node stencil bodies: the check-free interior one, the checked one and
// the clamped one.
enum : int { kBodyChecked = 0, kBodyInner = 1, kBodyClamped = 2 };

// Neighbour w of node v towards direction d for body B; m = 0 marks a
// missing neighbour of the clamped body (w is then v itself).
template <int B>
__device__ __forceinline__ int stencil_nbr(int n, int v, int i, int j, int k, int d, float& m) {
    m = 1.f;
    if (B == kBodyInner) return v + off_x(d) + n * off_y(d) + n * n * off_z(d);
    const int w = nbr(i, j, k, d, n);
    if (B == kBodyClamped && w < 0) {
        m = 0.f;
        return v;
    }
    return w;
}

// y = K x at node v from the FP16 layout (without the level's scale).
// Inner body: all 14 neighbours exist (no range checks, so the compiler can
// issue every load of the node before the first use).
template <int B>
__device__ __forceinline__ void stencil_h_body(int n, int64_t N, int v, int i, int j, int k,
                                               const uint4* __restrict__ K,
                                               const float* __restrict__ x, float y[3]) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const uint4 e8 = __ldg(K + hidx(8, v));
#pragma unroll
    for (int d = 0; d < 8; ++d) {  // self and positive directions: own blocks
        float m;
        const int w = stencil_nbr<B>(n, v, i, j, k, d, m);
        if (B == kBodyChecked && w < 0) continue;
        const float x0 = x[w] * m, x1 = x[N + w] * m, x2 = x[2 * N + w] * m;
        float f[8];
        unpack8(__ldg(K + hidx(d, v)), f);
        const float f8 = half_at(e8, d);
        a0 = fmaf(f[0], x0, fmaf(f[1], x1, fmaf(f[2], x2, a0)));
        a1 = fmaf(f[3], x0, fmaf(f[4], x1, fmaf(f[5], x2, a1)));
        a2 = fmaf(f[6], x0, fmaf(f[7], x1, fmaf(f8, x2, a2)));
    }
#pragma unroll
    for (int d = 1; d < 8; ++d) {  // negative directions: neighbour's block, transposed
        float m;
        const int w = stencil_nbr<B>(n, v, i, j, k, d + 7, m);
        if (B == kBodyChecked && w < 0) continue;
        const float x0 = x[w] * m, x1 = x[N + w] * m, x2 = x[2 * N + w] * m;
        float f[8];
        unpack8(__ldg(K + hidx(d, (int64_t)w)), f);
        const float f8 = half_at(__ldg(K + hidx(8, (int64_t)w)), d);
        a0 = fmaf(f[0], x0, fmaf(f[3], x1, fmaf(f[6], x2, a0)));
        a1 = fmaf(f[1], x0, fmaf(f[4], x1, fmaf(f[7], x2, a1)));
        a2 = fmaf(f[2], x0, fmaf(f[5], x1, fmaf(f8, x2, a2)));
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

// SK (kSk*): the split form has a separate check-free body for interior nodes
// (more registers; the persistent batched kernel, which holds every phase in
// one function, keeps the single checked body).
template <int SK>
__device__ __forceinline__ void stencil_apply_h(int n, int64_t N, int64_t v64,
                                                const uint4* __restrict__ K,
                                                const float* __restrict__ x, float y[3]) {
    const int v = (int)v64;
    const int nn = n * n;
    const int k = v / nn;
    const int rem = v - k * nn;
    const int j = rem / n;
    const int i = rem - j * n;
    if (SK == kSkClamped)
        stencil_h_body<kBodyClamped>(n, N, v, i, j, k, K, x, y);
    else if (SK == kSkSplit && i > 0 && j > 0 && k > 0 && i < n - 1 && j < n - 1 && k < n - 1)
        stencil_h_body<kBodyInner>(n, N, v, i, j, k, K, x, y);
    else
        stencil_h_body<kBodyChecked>(n, N, v, i, j, k, K, x, y);
}

// y = K x at node v (3 components, without the level's scale); x SoA [3][N].
// 32-bit lattice coordinates; interior nodes take the neighbour offsets
// without range checks.
template <typename T, typename KS, int SK = kSkSplit>
__device__ __forceinline__ void stencil_apply(int n, int64_t N, int64_t v64,
                                              const KS* __restrict__ K,
                                              const T* __restrict__ x, T y[3]) {
    if constexpr (std::is_same<KS, __half>::value) {
        stencil_apply_h<SK>(n, N, v64, reinterpret_cast<const uint4*>(K), x, y);
        return;
    }
    const int v = (int)v64;
    const int nn = n * n;
    const int k = v / nn;
    const int rem = v - k * nn;
    const int j = rem / n;
    const int i = rem - j * n;
    const bool inner = SK != kSkClamped && i > 0 && j > 0 && k > 0 && i < n - 1 && j < n - 1 &&
                       k < n - 1;
    T a0 = T(0), a1 = T(0), a2 = T(0);
#pragma unroll
    for (int d = 0; d < 8; ++d) {  // self and positive directions: own blocks
        int w = inner ? v + off_x(d) + n * off_y(d) + nn * off_z(d) : nbr(i, j, k, d, n);
        T m = T(1);
        if (SK == kSkClamped && w < 0) {
            w = v;
            m = T(0);
        }
        if (w < 0) continue;
        const T x0 = x[w] * m, x1 = x[N + w] * m, x2 = x[2 * N + w] * m;
        const KS* kb = K + kidx(d * 9, v64);
        a0 = fma(ldk<T>(kb), x0, fma(ldk<T>(kb + 32), x1, fma(ldk<T>(kb + 64), x2, a0)));
        a1 = fma(ldk<T>(kb + 96), x0, fma(ldk<T>(kb + 128), x1, fma(ldk<T>(kb + 160), x2, a1)));
        a2 = fma(ldk<T>(kb + 192), x0, fma(ldk<T>(kb + 224), x1, fma(ldk<T>(kb + 256), x2, a2)));
    }
#pragma unroll
    for (int d = 1; d < 8; ++d) {  // negative directions: neighbour's block, transposed
        int w = inner ? v - off_x(d) - n * off_y(d) - nn * off_z(d) : nbr(i, j, k, d + 7, n);
        T m = T(1);
        if (SK == kSkClamped && w < 0) {
            w = v;
            m = T(0);
        }
        if (w < 0) continue;
        const T x0 = x[w] * m, x1 = x[N + w] * m, x2 = x[2 * N + w] * m;
        const KS* kb = K + kidx(d * 9, (int64_t)w);
        a0 = fma(ldk<T>(kb), x0, fma(ldk<T>(kb + 96), x1, fma(ldk<T>(kb + 192), x2, a0)));
        a1 = fma(ldk<T>(kb + 32), x0, fma(ldk<T>(kb + 128), x1, fma(ldk<T>(kb + 224), x2, a1)));
        a2 = fma(ldk<T>(kb + 64), x0, fma(ldk<T>(kb + 160), x1, fma(ldk<T>(kb + 256), x2, a2)));
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

// A product rounded on its own (never contracted into a following add).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

template <typename T>
__device__ __forceinline__ void dinv_apply(int64_t N, int64_t v, const T* __restrict__ Di,
                                           const T r[3], T z[3]) {
    const T d0 = Di[v], d1 = Di[N + v], d2 = Di[2 * N + v], d3 = Di[3 * N + v],
            d4 = Di[4 * N + v], d5 = Di[5 * N + v];
    z[0] = d0 * r[0] + d1 * r[1] + d2 * r[2];
    z[1] = d1 * r[0] + d3 * r[1] + d4 * r[2];
    z[2] = d2 * r[0] + d4 * r[1] + d5 * r[2];
}

// d_0 = D^-1 b / theta at node v, from the right-hand side value bv.
template <typename T>
__device__ __forceinline__ void mg_first_dir(const LevelView<T>& L, int64_t v, const T bv[3]) {
    const T ith = (T)L.coef[0];
    T z[3];
    dinv_apply<T>(L.N, v, L.Di, bv, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) L.d0[c * L.N + v] = z[c] * ith;
}

// Step modes: how r and x enter the step.
enum : int {
    kStepRegular = 0,  // r -= K d_in; x += d_out
    kStepFromZero = 1, // x was 0 and d_in = d_0: r = b - K d_in; x = d_in + d_out
    kStepAfterFirst = 2 // r holds b - K x and d_in = d_0 (x not yet updated):
                        // r -= K d_in; x += d_in + d_out
};

// Chebyshev step s >= 1 at node v.  Returns the new x value (3 components),
// written to L.x unless `out` is non-null (the fused caller writes it).
template <typename T, int SK = kSkSplit>
__device__ __forceinline__ void mg_step_node(const LevelView<T>& L, int64_t v, int step, int mode,
                                             const T* __restrict__ din, T* __restrict__ dout,
                                             T xo[3], bool write_x, bool write_rd) {
    const int64_t N = L.N;
    const T A = (T)L.coef[2 * step - 1], B = (T)L.coef[2 * step];
    const T ks = (T)*L.ks;
    T y[3], rr[3], z[3];
    stencil_apply<T, typename MGStore<T>::type, SK>(L.n, N, v, L.K, din, y);
    const T* rin = mode == kStepFromZero ? L.b : L.r;
#pragma unroll
    for (int c = 0; c < 3; ++c) rr[c] = rin[c * N + v] - ks * y[c];
    dinv_apply<T>(N, v, L.Di, rr, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T di = din[c * N + v];
        const T dd = A * di + B * z[c];
        if (write_rd) {
            L.r[c * N + v] = rr[c];
            dout[c * N + v] = dd;
        }
        T xv;
        if (mode == kStepFromZero) xv = di + dd;
        else if (mode == kStepAfterFirst) xv = L.x[c * N + v] + di + dd;
        else xv = L.x[c * N + v] + dd;
        xo[c] = xv;
        if (write_x) L.x[c * N + v] = xv;
    }
}

// r = b - K x at node v.
template <typename T, int SK = kSkSplit>
__device__ __forceinline__ void mg_resid_node(const LevelView<T>& L, int64_t v) {
    const int64_t N = L.N;
    const T ks = (T)*L.ks;
    T y[3];
    stencil_apply<T, typename MGStore<T>::type, SK>(L.n, N, v, L.K, L.x, y);
#pragma unroll
    for (int c = 0; c < 3; ++c) L.r[c * N + v] = L.b[c * N + v] - ks * y[c];
}

// Degree-1 pre-smoothing from zero: r = b - K d_0 at node v (d_0 = D^-1 b /
// theta).  The smoothed x is d_0 itself: the prolongation writes
// x = d_0 + P e, so x is not stored here.
template <typename T, int SK = kSkSplit>
__device__ __forceinline__ void mg_resid_d0_node(const LevelView<T>& L, int64_t v) {
    const int64_t N = L.N;
    const T ks = (T)*L.ks;
    T y[3];
    stencil_apply<T, typename MGStore<T>::type, SK>(L.n, N, v, L.K, L.d0, y);
#pragma unroll
    for (int c = 0; c < 3; ++c) L.r[c * N + v] = L.b[c * N + v] - ks * y[c];
}

// r = b - K x and d_0 = D^-1 r / theta at node v (x is left for the next
// step).  WR = false: r is not stored (degree-1 levels, whose update after
// this is the pointwise x + d_0).
template <typename T, int SK = kSkSplit, bool WR = true>
__device__ __forceinline__ void mg_resid_first_node(const LevelView<T>& L, int64_t v) {
    const int64_t N = L.N;
    const T ks = (T)*L.ks;
    T y[3], rr[3];
    stencil_apply<T, typename MGStore<T>::type, SK>(L.n, N, v, L.K, L.x, y);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        rr[c] = L.b[c * N + v] - ks * y[c];
        if (WR) L.r[c * N + v] = rr[c];
    }
    mg_first_dir<T>(L, v, rr);
}

// The degree-1 post-smoothing of a level at node v, nothing stored:
// xo = x + d_0 with d_0 = D^-1 (b - K x) / theta (the same roundings as
// mg_resid_first_node followed by x + d_0).
template <typename T, int SK = kSkSplit>
__device__ __forceinline__ void mg_post1_node(const LevelView<T>& L, int64_t v, T xo[3]) {
    const int64_t N = L.N;
    const T ks = (T)*L.ks;
    T y[3], rr[3], z[3];
    stencil_apply<T, typename MGStore<T>::type, SK>(L.n, N, v, L.K, L.x, y);
#pragma unroll
    for (int c = 0; c < 3; ++c) rr[c] = L.b[c * N + v] - ks * y[c];
    dinv_apply<T>(N, v, L.Di, rr, z);
    const T ith = (T)L.coef[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) xo[c] = L.x[c * N + v] + mul_rn(z[c], ith);
}

// b_c(I) = sum_a w_a r_f(2I + off[a])  (P^T r), zero on Dirichlet nodes; then
// the coarse level's first direction.  Branch-free: a fine node outside the
// lattice reads node 0 and a Dirichlet one its own r, both with weight 0, so
// every load of the node issues at once.
template <typename T>
__device__ __forceinline__ void mg_restrict_node(const LevelView<T>& F, const LevelView<T>& C,
                                                 int64_t I) {
    const int nf = F.n, nc = C.n;
    const int64_t Nf = F.N, Nc = C.N;
    T a[3] = {T(0), T(0), T(0)};
    if (!C.mask[I]) {
        const int ci = (int)(I % nc), cj = (int)((I / nc) % nc), ck = (int)(I / ((int64_t)nc * nc));
#pragma unroll
        for (int d = 0; d < 15; ++d) {
            int f = nbr(2 * ci, 2 * cj, 2 * ck, d, nf);
            T w = d == 0 ? T(1) : T(0.5);
            if (f < 0) {
                f = 0;
                w = T(0);
            }
            if (F.mask[f]) w = T(0);
            a[0] += w * F.r[f];
            a[1] += w * F.r[Nf + f];
            a[2] += w * F.r[2 * Nf + f];
        }
    }
    C.b[I] = a[0];
    C.b[Nc + I] = a[1];
    C.b[2 * Nc + I] = a[2];
    mg_first_dir<T>(C, I, a);
}

// x_f(f) += sum_{parents J} w x_c(J)  (P e); FROM_D0: x_f = d_0 + P e (a
// degree-1 level, whose pre-smoothed x is d_0).
template <typename T, bool FROM_D0 = false>
__device__ __forceinline__ void mg_prolong_node(const LevelView<T>& F, const LevelView<T>& C,
                                                int64_t f) {
    const T* base = FROM_D0 ? F.d0 : F.x;
    if (F.mask[f]) {
        if (FROM_D0)
            for (int c = 0; c < 3; ++c) F.x[c * F.N + f] = base[c * F.N + f];
        return;
    }
    const int nf = F.n, nc = C.n;
    const int64_t Nf = F.N, Nc = C.N;
    const int fi = (int)(f % nf), fj = (int)((f / nf) % nf), fk = (int)(f / ((int64_t)nf * nf));
    const int Ai = fi >> 1, Aj = fj >> 1, Ak = fk >> 1;
    const int oi = fi & 1, oj = fj & 1, ok = fk & 1;
    // parents A and Bn (Bn = A for a node on the coarse lattice, then weight 0);
    // branch-free, so the masks and the values load together
    const int64_t A = Ai + (int64_t)nc * (Aj + (int64_t)nc * Ak);
    const int64_t Bn = (Ai + oi) + (int64_t)nc * ((Aj + oj) + (int64_t)nc * (Ak + ok));
    const bool on = (oi | oj | ok) == 0;
    const T wa = C.mask[A] ? T(0) : (on ? T(1) : T(0.5));
    const T wb = (on || C.mask[Bn]) ? T(0) : T(0.5);
    const T s0 = wa * C.x[A] + wb * C.x[Bn];
    const T s1 = wa * C.x[Nc + A] + wb * C.x[Nc + Bn];
    const T s2 = wa * C.x[2 * Nc + A] + wb * C.x[2 * Nc + Bn];
    F.x[f] = base[f] + s0;
    F.x[Nf + f] = base[Nf + f] + s1;
    F.x[2 * Nf + f] = base[2 * Nf + f] + s2;
}

// Coarsest level: `steps` Chebyshev steps from zero on L.b by the calling CTA
// alone (every thread of the block must call it).
template <typename T, int SK = kSkSplit>
__device__ __forceinline__ void mg_coarse_block(const LevelView<T>& L, int steps) {
    const int64_t N = L.N;
    for (int64_t v = threadIdx.x; v < N; v += blockDim.x) {
        const T bv[3] = {L.b[v], L.b[N + v], L.b[2 * N + v]};
        mg_first_dir<T>(L, v, bv);
    }
    __syncthreads();
    T xo[3];
    if (steps == 1) {
        for (int64_t v = threadIdx.x; v < N; v += blockDim.x)
            for (int c = 0; c < 3; ++c) L.x[c * N + v] = L.d0[c * N + v];
        __syncthreads();
        return;
    }
    for (int s = 1; s < steps; ++s) {
        const T* din = (s & 1) ? L.d0 : L.d1;
        T* dout = (s & 1) ? L.d1 : L.d0;
        const int mode = s == 1 ? kStepFromZero : kStepRegular;
        for (int64_t v = threadIdx.x; v < N; v += blockDim.x)
            mg_step_node<T, SK>(L, v, s, mode, din, dout, xo, true, true);
        __syncthreads();
    }
}

}  // namespace fts
