// fts_bsr_residual_noalloc: the FP64 block residual r = b - S x with its two
// squared norms, for callers that cannot allocate device memory.
//
// Some callers own all of the GPU's memory through their own allocator or
// arena (a simulation that reserves HBM up front for its time-stepping state),
// or run in a loop that must not stall on the device synchronisation that
// cudaMalloc / cudaFree can trigger.  For them this entry point allocates
// nothing: the caller passes the system, x, b and the outputs (device memory),
// and the grid-reduction scratch lives in the static device array below, of a
// fixed size.  Every GPU that loads libfts.so holds that array until the
// process exits.
//
// Set-up: every call looks up the array's device address with
// cudaGetSymbolAddress for the device that is current (a host-side lookup that
// allocates nothing), so the address stays right after a cudaDeviceReset or a
// context change.  The first call on a device also loads the library's module
// into that device's context; make that first call before any stream capture.
// All calls share the one array and it keeps the previous call's contents, so
// the ticket counter is cleared at the start of every call; two calls whose
// kernels overlap on the GPU (calls on different streams, not ordered by an
// event) race on the array and give wrong norms: serialise them on one stream.
#include <cuda_runtime.h>

#include <cstdint>

#include "fts.h"

namespace {

constexpr int kThreadsNA = 256;
constexpr int kRowsPerBlock = kThreadsNA / 4;  // 4 threads per block row
constexpr int64_t kMaxBlocksNA = FTS_NOALLOC_MAX_NODES / kRowsPerBlock;
static_assert(FTS_NOALLOC_MAX_NODES % kRowsPerBlock == 0, "node limit is a whole number of blocks");

// Per-block partial sums (||r||^2, ||b||^2) followed by the arrival ticket.
constexpr size_t kScratchBytes = (size_t)kMaxBlocksNA * 2 * sizeof(double) + 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// r = b - S x over one block of rows; partials -> scratch; the last block sums
// the partials in block order (deterministic) and writes norms[0..1].
__global__ void __launch_bounds__(kThreadsNA)
k_residual_noalloc(int64_t np, const int32_t* __restrict__ rowptr,
                   const int32_t* __restrict__ cols, const double* __restrict__ A,
                   const double* __restrict__ x, const double* __restrict__ b,
                   double* __restrict__ r, double* __restrict__ norms,
                   unsigned char* __restrict__ scratch) {
    double* part = reinterpret_cast<double*>(scratch);
    unsigned* ticket = reinterpret_cast<unsigned*>(scratch + (size_t)kMaxBlocksNA * 2 * sizeof(double));
    const int q = threadIdx.x & 3;
    const int64_t row = (int64_t)blockIdx.x * kRowsPerBlock + (threadIdx.x >> 2);
    double rr = 0.0, bb = 0.0;
    if (row < np) {
        double acc = 0.0;
        for (int32_t k = rowptr[row]; k < rowptr[row + 1]; ++k) {
            const int64_t j = cols[k];
            const double* a = A + (int64_t)k * 16 + q * 4;
            const double* xj = x + j * 4;
            acc = fma(a[0], xj[0], acc);
            acc = fma(a[1], xj[1], acc);
            acc = fma(a[2], xj[2], acc);
            acc = fma(a[3], xj[3], acc);
        }
        const double be = b[row * 4 + q];
        const double v = be - acc;
        r[row * 4 + q] = v;
        rr = v * v;
        bb = be * be;
    }
    for (int o = 16; o > 0; o >>= 1) {
        rr += __shfl_xor_sync(0xffffffffu, rr, o);
        bb += __shfl_xor_sync(0xffffffffu, bb, o);
    }
    __shared__ double s_rr[kThreadsNA / 32], s_bb[kThreadsNA / 32];
    __shared__ bool am_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s_rr[wid] = rr;
        s_bb[wid] = bb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int w = 0; w < kThreadsNA / 32; ++w) {
            a += s_rr[w];
            c += s_bb[w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = c;
        __threadfence();
        am_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (unsigned i = 0; i < gridDim.x; ++i) {
            a += __ldcg(&part[2 * i]);
            c += __ldcg(&part[2 * i + 1]);
        }
        norms[0] = a;
        norms[1] = c;
        *ticket = 0u;
    }
}

// Device address of the static scratch array in the current device's context,
// looked up on every call (never cached: a cudaDeviceReset or another context
// can place the module at another address).
int scratch_for_current_device(void** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FTS_ERR_CUDA;
    *out = p;
    return FTS_OK;
}

}  // namespace

extern "C" int fts_bsr_residual_noalloc(int64_t np, const int32_t* rowptr, const int32_t* cols,
                                        const double* vals, const double* x, const double* b,
                                        double* r, double* norms, void* stream) {
    if (np <= 0 || !rowptr || !cols || !vals || !x || !b || !r || !norms) return FTS_ERR_BAD_INPUT;
    if (np > FTS_NOALLOC_MAX_NODES) return FTS_ERR_BAD_INPUT;  // scratch holds this many rows
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != FTS_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* base = static_cast<unsigned char*>(scratch);
    unsigned char* ticket = base + (size_t)kMaxBlocksNA * 2 * sizeof(double);
    if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), s) != cudaSuccess) return FTS_ERR_CUDA;
    const unsigned blocks = (unsigned)((np + kRowsPerBlock - 1) / kRowsPerBlock);
    k_residual_noalloc<<<blocks, kThreadsNA, 0, s>>>(np, rowptr, cols, vals, x, b, r, norms, base);
    return cudaGetLastError() == cudaSuccess ? FTS_OK : FTS_ERR_CUDA;
}
