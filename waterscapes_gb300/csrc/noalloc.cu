// Residual of the assembled system for callers that cannot allocate device
// memory.
//
// mpet_residual reduces the residual norms through scratch the context
// obtained from cudaMalloc when it was set up.  Some callers cannot take that
// route: an application whose memory allocator has already claimed the
// device's memory (a caching allocator that reserves the free memory at
// start-up), a code that must not allocate once its initialisation phase is
// over (cudaMalloc and cudaFree synchronise the device and may fail under
// memory pressure), or a caller that only borrows a context another
// component created and may not grow it.  mpet_residual_noalloc gives them
// the same result with no allocation: its reduction scratch is the
// file-scope device array below, NOALLOC_SCRATCH_DOUBLES doubles (256 KiB),
// which every GPU that loads this library holds until the process exits.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object), so the device address is asked for once per
// device with cudaGetSymbolAddress, with that device current, and kept.
// mpet_ctx_create does this eagerly, and also asks for the attributes of this
// file's kernels: with lazy module loading (the CUDA default) that is what
// loads the array and the kernels' code onto the device, so it happens while
// the caller can still spare the memory (256 KiB plus the code), not at the
// first call.  If that early lookup failed, the first
// mpet_residual_noalloc call on the device retries it; make that call
// outside any stream capture.  The call waits for its own stream (it
// returns the norms to the host), so it synchronises the context's stream.
// Every call shares the one array; each call overwrites every slot it reads,
// so nothing carries over from an earlier call, but calls that overlap on
// the GPU (different streams or threads, same device) race on it and must
// be serialised by the caller.
#include <math.h>

#include <mutex>

#include "mpet_internal.cuh"

namespace mpet {

constexpr int NOALLOC_ROWS_PER_BLOCK = 2048;
constexpr int NOALLOC_MAX_BLOCKS = 16384;
constexpr int NOALLOC_SCRATCH_DOUBLES = 2 * NOALLOC_MAX_BLOCKS;
// rows handled by one call at most: 2048 * 16384 = 33,554,432
constexpr int64_t NOALLOC_MAX_ROWS = (int64_t)NOALLOC_ROWS_PER_BLOCK * NOALLOC_MAX_BLOCKS;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[128] = {nullptr};

// device address of the scratch array on the current device (looked up once)
static double* noalloc_scratch(int device) {
    if (device < 0 || device >= 128) fail(MPET_ERR_INVALID, "device index out of range for the static scratch table");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            fail(MPET_ERR_CUDA, std::string("cudaGetSymbolAddress of the residual scratch: ") + cudaGetErrorString(e));
        }
        g_noalloc_ptr[device] = (double*)p;
    }
    return g_noalloc_ptr[device];
}

__device__ __forceinline__ double nb_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double nb_block_sum(double v, double* sh) {
    v = nb_warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        t = nb_warp_sum(t);
    }
    __syncthreads();
    return t;
}

// Block b owns rows [b * NOALLOC_ROWS_PER_BLOCK, ...): r = b - A x for each
// row (LPR lanes per row, each lane summing its entries in increasing order,
// then a butterfly over the lanes) and one partial of (r/d)^2 and (b/d)^2.
template <int LPR>
__global__ void __launch_bounds__(256) k_resid_blocks(int64_t n, const int64_t* __restrict__ rp,
                                                      const int32_t* __restrict__ ci, const double* __restrict__ va,
                                                      const double* __restrict__ x, const double* __restrict__ bvec,
                                                      const double* __restrict__ dinv, double* r, double* part) {
    __shared__ double sh[8];
    const int sub = threadIdx.x & (LPR - 1);
    const int grp = threadIdx.x / LPR;
    constexpr int NGR = 256 / LPR;
    const int64_t r0 = (int64_t)blockIdx.x * NOALLOC_ROWS_PER_BLOCK;
    int64_t r1 = r0 + NOALLOC_ROWS_PER_BLOCK;
    if (r1 > n) r1 = n;
    double s_r = 0.0, s_b = 0.0;
    for (int64_t base = r0; base < r1; base += NGR) {
        const int64_t row = base + grp;
        double acc = 0.0;
        if (row < r1)
            for (int64_t e = rp[row] + sub; e < rp[row + 1]; e += LPR) acc += va[e] * x[ci[e]];
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (row < r1 && sub == 0) {
            const double rr = bvec[row] - acc;
            r[row] = rr;
            const double di = dinv[row];
            s_r += (rr * di) * (rr * di);
            s_b += (bvec[row] * di) * (bvec[row] * di);
        }
    }
    const double t0 = nb_block_sum(s_r, sh);
    const double t1 = nb_block_sum(s_b, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = t0;
        part[NOALLOC_MAX_BLOCKS + blockIdx.x] = t1;
    }
}

// One block sums the nblocks partials (fixed order) into part[0], part[NOALLOC_MAX_BLOCKS].
__global__ void __launch_bounds__(256) k_resid_finish(int nblocks, double* part) {
    __shared__ double sh[8];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += 256) {
        a += part[i];
        b += part[NOALLOC_MAX_BLOCKS + i];
    }
    a = nb_block_sum(a, sh);
    b = nb_block_sum(b, sh);
    if (threadIdx.x == 0) {
        part[0] = a;
        part[NOALLOC_MAX_BLOCKS] = b;
    }
}

// Eager set-up at context creation (the current device is `device`): the
// scratch address, and the code of this file's kernels, which lazy module
// loading would otherwise load (and allocate device memory for) at the first
// call.  A failure here is left for the first call to report.
void noalloc_prepare(int device) {
    try {
        noalloc_scratch(device);
        cudaFuncAttributes fa;
        cudaFuncGetAttributes(&fa, k_resid_blocks<32>);
        cudaFuncGetAttributes(&fa, k_resid_blocks<16>);
        cudaFuncGetAttributes(&fa, k_resid_blocks<8>);
        cudaFuncGetAttributes(&fa, k_resid_blocks<4>);
        cudaFuncGetAttributes(&fa, k_resid_finish);
        cudaGetLastError();
    } catch (const Error&) {
    }
}

static void residual_noalloc(mpet_ctx* c, const double* b, const double* x, double* r, double* norms) {
    const int64_t n = c->N;
    if (n > NOALLOC_MAX_ROWS)
        fail(MPET_ERR_INVALID, "mpet_residual_noalloc handles at most 33,554,432 rows (static scratch of 16384 "
                               "blocks x 2048 rows); this system has " + std::to_string(n));
    if (n == 0) {
        norms[0] = 0.0;
        norms[1] = 0.0;
        return;
    }
    double* part = noalloc_scratch(c->device);
    const int nblocks = (int)((n + NOALLOC_ROWS_PER_BLOCK - 1) / NOALLOC_ROWS_PER_BLOCK);
    const Csr& A = c->A;
    switch (A.lpr) {
        case 32: k_resid_blocks<32><<<nblocks, 256, 0, c->stream>>>(n, A.rp, A.ci, A.v64, x, b, c->dinv, r, part); break;
        case 16: k_resid_blocks<16><<<nblocks, 256, 0, c->stream>>>(n, A.rp, A.ci, A.v64, x, b, c->dinv, r, part); break;
        case 8: k_resid_blocks<8><<<nblocks, 256, 0, c->stream>>>(n, A.rp, A.ci, A.v64, x, b, c->dinv, r, part); break;
        default: k_resid_blocks<4><<<nblocks, 256, 0, c->stream>>>(n, A.rp, A.ci, A.v64, x, b, c->dinv, r, part); break;
    }
    k_resid_finish<<<1, 256, 0, c->stream>>>(nblocks, part);
    MPET_CHECK_LAUNCH();
    double sums[2];
    MPET_CUDA(cudaMemcpyAsync(&sums[0], part, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaMemcpyAsync(&sums[1], part + NOALLOC_MAX_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    norms[0] = sqrt(sums[0]);
    norms[1] = sqrt(sums[1]);
}

}  // namespace mpet

extern "C" int mpet_residual_noalloc(mpet_ctx* c, const double* b, const double* x, double* r, double* norms) {
    if (!c) return MPET_ERR_INVALID;
    try {
        MPET_CUDA(cudaSetDevice(c->device));
        if (!c->assembled) mpet::fail(MPET_ERR_STATE, "mpet_assemble must come first");
        if (!(b && x && r && norms)) mpet::fail(MPET_ERR_INVALID, "NULL argument");
        mpet::residual_noalloc(c, b, x, r, norms);
    } catch (const mpet::Error& e) {
        c->err = e.msg;
        return e.code;
    }
    return MPET_OK;
}
