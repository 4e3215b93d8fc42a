// Krylov solver of the MPET system: block-diagonally preconditioned MINRES
// with one smoothed-aggregation AMG V-cycle per diagonal block, wrapped in
// an FP64 iterative-refinement loop.
//
// Replaces the direct LUSolver(A, "mumps") of src/mpet/mpet/mpetsolver.py:347
// and the PETScKrylovSolver("minres", "hypre_amg") of mpetsolver.py:507-557
// (working twin mpettotalpressuresolver.py:448-493).
//
// Precision: MPET_PRECISION_FP64 runs everything in FP64.  MPET_PRECISION_MIXED
// computes the outer residual r = b - A x with the FP64 matrix and solves
// each correction with FP32 matrix values, FP32 Krylov vectors and an FP32
// AMG (coarsest level solved in FP64), as many sweeps as needed for the
// FP64 preconditioned residual to drop by rtol.
//
// Dirichlet rows: the stored matrix has DirichletBC rows replaced by unit
// rows.  Every Krylov vector has zero Dirichlet entries (the right-hand side
// of a correction has them, and the AMG maps them to zero), so on those
// vectors the stored matrix acts as the symmetric elimination of
// bc_symmetric.py:20-22 without touching the columns.
//
// All reductions are deterministic: a fixed grid of NB_RED blocks writes one
// partial per block and a single block sums the partials in a fixed order.
#include <limits.h>
#include <math.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "mpet_internal.cuh"

namespace mpet {

// True if `bytes` more can be allocated while a fifth of the device memory
// stays free (room for the AMG hierarchies and work vectors allocated later).
bool device_fits(mpet_ctx* c, size_t bytes) {
    size_t free_b = 0, total_b = 0;
    MPET_CUDA(cudaMemGetInfo(&free_b, &total_b));
    return free_b > bytes && free_b - bytes >= total_b / 5;
}

static inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > 2147483647LL) g = 2147483647LL;
    return (int)(g < 1 ? 1 : g);
}

int choose_lpr(int64_t n, int64_t nnz) {
    double avg = n > 0 ? (double)nnz / (double)n : 0.0;
    if (avg >= 48.0) return 32;
    if (avg >= 20.0) return 16;
    if (avg >= 8.0) return 8;
    if (avg >= 3.0) return 4;
    return 1;
}

// ---- vector access -------------------------------------------------------------
// Multi-vector data is node-interleaved (NV values per row).  With NV = 4
// every row's values are one 16-byte-aligned group, accessed by vector
// loads/stores (float4, or two double2 for FP64).

template <typename T, int NV>
struct VecIO {
    static __device__ __forceinline__ void load(const T* p, int64_t row, T* v) {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = p[NV * row + k];
    }
    static __device__ __forceinline__ void store(T* p, int64_t row, const T* v) {
#pragma unroll
        for (int k = 0; k < NV; ++k) p[NV * row + k] = v[k];
    }
};
template <>
struct VecIO<float, 4> {
    static __device__ __forceinline__ void load(const float* p, int64_t row, float* v) {
        const float4 q = reinterpret_cast<const float4*>(p)[row];
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    }
    static __device__ __forceinline__ void store(float* p, int64_t row, const float* v) {
        reinterpret_cast<float4*>(p)[row] = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct VecIO<double, 4> {
    static __device__ __forceinline__ void load(const double* p, int64_t row, double* v) {
        const double2 a = reinterpret_cast<const double2*>(p)[2 * row];
        const double2 b = reinterpret_cast<const double2*>(p)[2 * row + 1];
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ void store(double* p, int64_t row, const double* v) {
        reinterpret_cast<double2*>(p)[2 * row] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(p)[2 * row + 1] = make_double2(v[2], v[3]);
    }
};

// ---- SpMV with fused epilogues -------------------------------------------------------
//
// An epilogue has pre(row), which loads the row's other operands and is
// issued before the row's gather loop so that its latency overlaps the
// gathers, and apply(row, acc, pre, ...), which combines them with A x.

template <typename T, int NV>
struct EpiStore {
    T* y;
    static constexpr int kRed = 0;
    static constexpr bool kSystem = NV == 1;  // runs with the node-block system kernel
    struct Pre {};
    __device__ __forceinline__ Pre pre(int64_t) const { return Pre{}; }
    __device__ __forceinline__ void apply(int64_t row, const T* acc, const Pre&, double&, double&) const {
        VecIO<T, NV>::store(y, row, acc);
    }
};

// y = alpha * (A x) + beta * z   (z may alias y)
template <typename T, int NV>
struct EpiAxpby {
    T* y;
    const T* z;
    T alpha, beta;
    static constexpr int kRed = 0;
    static constexpr bool kSystem = false;
    struct Pre {
        T zz[NV];
    };
    __device__ __forceinline__ Pre pre(int64_t row) const {
        Pre p;
        if (z) VecIO<T, NV>::load(z, row, p.zz);
        else
#pragma unroll
            for (int k = 0; k < NV; ++k) p.zz[k] = T(0);
        return p;
    }
    __device__ __forceinline__ void apply(int64_t row, const T* acc, const Pre& p, double&, double&) const {
        T out[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = alpha * acc[k] + beta * p.zz[k];
        VecIO<T, NV>::store(y, row, out);
    }
};

// One Chebyshev step on D^-1 A: d = c1 d + c2 D^-1 (b - A xin); xout = xin + d.
template <typename T, int NV>
struct EpiCheb {
    const T* b;
    const T* xin;
    T* d;
    T* xout;
    const T* dinv;
    T c1, c2;
    static constexpr int kRed = 0;
    static constexpr bool kSystem = false;
    struct Pre {
        T bb[NV], dd[NV], xx[NV], di;
    };
    __device__ __forceinline__ Pre pre(int64_t row) const {
        Pre p;
        p.di = dinv[row];
        VecIO<T, NV>::load(b, row, p.bb);
        VecIO<T, NV>::load(d, row, p.dd);
        VecIO<T, NV>::load(xin, row, p.xx);
        return p;
    }
    __device__ __forceinline__ void apply(int64_t row, const T* acc, const Pre& p, double&, double&) const {
        T dd[NV], xx[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            dd[k] = c1 * p.dd[k] + c2 * p.di * (p.bb[k] - acc[k]);
            xx[k] = p.xx[k] + dd[k];
        }
        VecIO<T, NV>::store(d, row, dd);
        VecIO<T, NV>::store(xout, row, xx);
    }
};

// a scalar in the working precision: the FP64 value or its FP32 copy
template <typename T>
__device__ __forceinline__ T msc(double d, float f);
template <>
__device__ __forceinline__ double msc<double>(double d, float) { return d; }
template <>
__device__ __forceinline__ float msc<float>(double, float f) { return f; }

// MINRES Lanczos step: y = A v - (beta/oldb) r1; partial v.y
template <typename T>
struct EpiMinres {
    T* y;
    const T* r1;
    const T* v;
    const MinresScalars* sc;
    static constexpr int kRed = 1;
    static constexpr bool kSystem = true;
    struct Pre {
        T r, v;
    };
    __device__ __forceinline__ Pre pre(int64_t row) const { return Pre{r1[row], v[row]}; }
    __device__ __forceinline__ void apply(int64_t row, const T* acc, const Pre& p, double& r0, double&) const {
        const T c = msc<T>(sc->c_r1, sc->f_c_r1);
        const T yy = acc[0] - c * p.r;
        y[row] = yy;
        r0 += (double)p.v * (double)yy;
    }
};

// FP64 residual r = b - A x with partial sums of (r/d)^2 and (b/d)^2.
struct EpiResid64 {
    double* r;
    const double* b;
    const double* dinv;
    static constexpr int kRed = 2;
    static constexpr bool kSystem = true;
    struct Pre {
        double b, di;
    };
    __device__ __forceinline__ Pre pre(int64_t row) const { return Pre{b[row], dinv[row]}; }
    __device__ __forceinline__ void apply(int64_t row, const double* acc, const Pre& p, double& r0,
                                          double& r1) const {
        const double rr = p.b - acc[0];
        r[row] = rr;
        r0 += (rr * p.di) * (rr * p.di);
        r1 += (p.b * p.di) * (p.b * p.di);
    }
};

// Batches: slice s (32 rows, or 32 node-block lanes) belongs to instances
// skl[2s]..skl[2s+1] (lo > hi: no rows); it is skipped, with no load and no
// store, when every one of them has converged (done != 0).  The products of a
// converged instance are never read again in the inner solve.
__device__ __forceinline__ bool slice_frozen(const int32_t* __restrict__ skl, int64_t s,
                                             const double* __restrict__ done) {
    const int lo = skl[2 * s], hi = skl[2 * s + 1];
    for (int i = lo; i <= hi; ++i)
        if (done[i] == 0.0) return false;
    return true;
}

template <typename T, int NV, int LPR, int U, class Epi>
__global__ void __launch_bounds__(256) k_spmv(int64_t n, const int64_t* __restrict__ rp,
                                              const int32_t* __restrict__ ci, const T* __restrict__ va,
                                              const T* __restrict__ x, Epi epi, double* partials,
                                              const int32_t* __restrict__ skl = nullptr,
                                              const double* __restrict__ skip = nullptr) {
    constexpr int RPW = 32 / LPR;  // rows per warp per pass
    const int lane = threadIdx.x & 31;
    const int sub = lane & (LPR - 1);
    const int grp = lane / LPR;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double r0 = 0.0, r1 = 0.0;
    for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {
        // the RPW rows of this pass lie in one 32-row slice (RPW divides 32)
        if (skl && slice_frozen(skl, base >> 5, skip)) continue;
        const int64_t row = base + grp;
        T acc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = T(0);
        typename Epi::Pre pre{};
        if (row < n && sub == 0) pre = epi.pre(row);
        if (row < n) {
            // Chunks of U (column, value) pairs per lane, all issued before the
            // dependent x gathers (U is chosen so that LPR * U covers the
            // longest row: one round trip per row).  Matrix loads are
            // evict-first so x stays resident in L2.  Every address is clamped
            // into the (non-empty) row, so a load issued regardless of its
            // predicate stays in bounds.
            const int64_t e0 = rp[row], e1 = rp[row + 1];
            for (int64_t b = e0; b < e1; b += LPR * U) {
                int32_t cc[U];
                T aa[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int64_t e = b + sub + u * LPR;
                    const int64_t es = e < e1 ? e : e1 - 1;
                    cc[u] = 0;
                    aa[u] = T(0);
                    if (e < e1) {
                        cc[u] = __ldcs(ci + es);
                        aa[u] = __ldcs(va + es);
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (b + sub + u * LPR < e1) {
                        T xv[NV];
                        VecIO<T, NV>::load(x, cc[u], xv);
#pragma unroll
                        for (int k = 0; k < NV; ++k) acc[k] += aa[u] * xv[k];
                    }
                }
            }
        }
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (row < n && sub == 0) epi.apply(row, acc, pre, r0, r1);
    }
    if constexpr (Epi::kRed > 0) {
        __shared__ double sh[8];
        double t0 = block_sum256(r0, sh);
        if (threadIdx.x == 0) partials[blockIdx.x] = t0;
        if constexpr (Epi::kRed > 1) {
            double t1 = block_sum256(r1, sh);
            if (threadIdx.x == 0) partials[NB_RED + blockIdx.x] = t1;
        }
    }
}

// ---- SELL-32 SpMV -------------------------------------------------------------------
//
// One thread owns one row of a 32-row slice; entry k of the slice's rows is
// contiguous, so every column/value load of a warp is one coalesced 128-byte
// line and a warp keeps 32 rows (U gathers each) in flight with no
// cross-lane reduction.  Padding entries carry value 0 and a valid column
// of the row.  The loop bound is the slice width, the same for every lane.
// LATE: the epilogue's own loads come after the accumulation loop, which
// frees their registers during it (more resident warps: the gathers are
// latency-bound), and the slice's entries two chunks ahead are prefetched into
// L2 (k_spmv_sell_late); otherwise the epilogue loads are issued first and
// overlap the loop (k_spmv_sell).
template <typename T, int NV, int U, class Epi, bool LATE>
__device__ __forceinline__ void spmv_sell_body(int64_t n, int64_t nslices, const int64_t* __restrict__ soff,
                                                   const int32_t* __restrict__ sci, const T* __restrict__ sva,
                                                   const T* __restrict__ x, Epi epi, double* partials,
                                                   const int32_t* __restrict__ skl,
                                                   const double* __restrict__ skip) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double r0 = 0.0, r1 = 0.0;
    for (int64_t sl = warp; sl < nslices; sl += nwarps) {
        if (skl && slice_frozen(skl, sl, skip)) continue;
        const int64_t row = sl * 32 + lane;
        const int64_t o1 = soff[sl + 1];
        typename Epi::Pre pre{};
        if (!LATE && row < n) pre = epi.pre(row);
        T acc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = T(0);
        for (int64_t e = soff[sl] + lane; e < o1; e += 32 * U) {
            if (LATE && lane < U) {
                // late variants also pull the slice's entries two chunks ahead into
                // L2 (one 128-byte line per array and chunk row): the dependent
                // loads of the next chunks then wait on L2, not on HBM
                const int64_t pf = e - lane + (int64_t)(2 * U + lane) * 32;
                if (pf < o1) {
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(sci + pf));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(sva + pf));
                }
            }
            int32_t cc[U];
            T aa[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                cc[u] = 0;
                aa[u] = T(0);
                if (e + u * 32 < o1) {
                    cc[u] = __ldcs(sci + e + u * 32);
                    aa[u] = __ldcs(sva + e + u * 32);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (e + u * 32 < o1) {
                    T xv[NV];
                    VecIO<T, NV>::load(x, cc[u], xv);
#pragma unroll
                    for (int k = 0; k < NV; ++k) acc[k] += aa[u] * xv[k];
                }
            }
        }
        if (LATE && row < n) pre = epi.pre(row);
        if (row < n) epi.apply(row, acc, pre, r0, r1);
    }
    if constexpr (Epi::kRed > 0) {
        __shared__ double sh[8];
        double t0 = block_sum256(r0, sh);
        if (threadIdx.x == 0) partials[blockIdx.x] = t0;
        if constexpr (Epi::kRed > 1) {
            double t1 = block_sum256(r1, sh);
            if (threadIdx.x == 0) partials[NB_RED + blockIdx.x] = t1;
        }
    }
}


template <typename T, int NV, int U, class Epi>
__global__ void __launch_bounds__(256) k_spmv_sell(int64_t n, int64_t nslices, const int64_t* __restrict__ soff,
                                                   const int32_t* __restrict__ sci, const T* __restrict__ sva,
                                                   const T* __restrict__ x, Epi epi, double* partials,
                                                   const int32_t* __restrict__ skl = nullptr,
                                                   const double* __restrict__ skip = nullptr) {
    spmv_sell_body<T, NV, U, Epi, false>(n, nslices, soff, sci, sva, x, epi, partials, skl, skip);
}

template <typename T, int NV, int U, class Epi>
__global__ void __launch_bounds__(256, 8) k_spmv_sell_late(int64_t n, int64_t nslices,
                                                          const int64_t* __restrict__ soff,
                                                          const int32_t* __restrict__ sci,
                                                          const T* __restrict__ sva, const T* __restrict__ x,
                                                          Epi epi, double* partials,
                                                          const int32_t* __restrict__ skl = nullptr,
                                                          const double* __restrict__ skip = nullptr) {
    spmv_sell_body<T, NV, U, Epi, true>(n, nslices, soff, sci, sva, x, epi, partials, skl, skip);
}

// SELL-32 with FP16 off-diagonal values (variant 32, FP32 vectors): the
// stored values are a_ij / s (s a power of two), diagonal slots 0; the row's
// result is s * sum + d_i x_i with the FP32 diagonal d_i that keeps the row
// sums of the original matrix.  Six bytes per entry instead of eight.
template <int NV, int U, class Epi>
__global__ void __launch_bounds__(256) k_spmv_sell_h(int64_t n, int64_t nslices, const int64_t* __restrict__ soff,
                                                     const int32_t* __restrict__ sci, const __half* __restrict__ sva,
                                                     const float* __restrict__ dg, float hs,
                                                     const float* __restrict__ x, Epi epi, double* partials,
                                                     const int32_t* __restrict__ skl,
                                                     const double* __restrict__ skip) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double r0 = 0.0, r1 = 0.0;
    for (int64_t sl = warp; sl < nslices; sl += nwarps) {
        if (skl && slice_frozen(skl, sl, skip)) continue;
        const int64_t row = sl * 32 + lane;
        const int64_t o1 = soff[sl + 1];
        typename Epi::Pre pre{};
        if (row < n) pre = epi.pre(row);
        float acc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = 0.f;
        for (int64_t e = soff[sl] + lane; e < o1; e += 32 * U) {
            int32_t cc[U];
            float aa[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                cc[u] = 0;
                aa[u] = 0.f;
                if (e + u * 32 < o1) {
                    cc[u] = __ldcs(sci + e + u * 32);
                    aa[u] = __half2float(__ldcs(sva + e + u * 32));
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (e + u * 32 < o1) {
                    float xv[NV];
                    VecIO<float, NV>::load(x, cc[u], xv);
#pragma unroll
                    for (int k = 0; k < NV; ++k) acc[k] += aa[u] * xv[k];
                }
            }
        }
        if (row < n) {
            float xr[NV];
            VecIO<float, NV>::load(x, row, xr);
            const float d = dg[row];
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] = acc[k] * hs + d * xr[k];
            epi.apply(row, acc, pre, r0, r1);
        }
    }
    if constexpr (Epi::kRed > 0) {
        __shared__ double sh[8];
        double t0 = block_sum256(r0, sh);
        if (threadIdx.x == 0) partials[blockIdx.x] = t0;
        if constexpr (Epi::kRed > 1) {
            double t1 = block_sum256(r1, sh);
            if (threadIdx.x == 0) partials[NB_RED + blockIdx.x] = t1;
        }
    }
}

// largest |a_ij|, i != j, as the bits of a non-negative double (ordered like the values)
__global__ void k_offdiag_absmax(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                 const double* __restrict__ v, unsigned long long* mx) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double m = 0.0;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e)
        if (ci[e] != i) m = fmax(m, fabs(v[e]));
    if (m > 0.0) atomicMax(mx, (unsigned long long)__double_as_longlong(m));
}

// the FP16 SELL values (same slots as k_sell_fill) and the row-sum diagonal
__global__ void k_sell_fill_half(int64_t n, int64_t nslices, const int64_t* __restrict__ rp,
                                 const int32_t* __restrict__ ci, const double* __restrict__ v,
                                 const int64_t* __restrict__ soff, double inv_scale, double scale, __half* sv,
                                 float* dg) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nslices * 32) return;
    const int64_t sl = t >> 5, lane = t & 31, row = t;
    const int64_t w = (soff[sl + 1] - soff[sl]) >> 5;
    const int64_t e0 = row < n ? rp[row] : 0, len = row < n ? rp[row + 1] - e0 : 0;
    double rowsum = 0.0, kept = 0.0;
    for (int64_t k = 0; k < w; ++k) {
        __half h = __float2half_rn(0.f);
        if (k < len) {
            const double a = v[e0 + k];
            rowsum += a;
            if (ci[e0 + k] != row) {
                h = __float2half_rn((float)(a * inv_scale));
                kept += (double)__half2float(h) * scale;
            }
        }
        sv[soff[sl] + k * 32 + lane] = h;
    }
    if (row < n) dg[row] = (float)(rowsum - kept);
}

void build_sell_half(mpet_ctx* c, Csr& A) {
    if (!A.s_off || !A.v64 || A.n == 0 || A.nnz == 0) return;
    int64_t nst = 0;  // stored SELL entries (with padding)
    MPET_CUDA(cudaMemcpyAsync(&nst, A.s_off + A.nslices, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    TmpBuf bm(sizeof(unsigned long long));
    MPET_CUDA(cudaMemsetAsync(bm.p, 0, sizeof(unsigned long long), c->stream));
    k_offdiag_absmax<<<grid_for(A.n, 256), 256, 0, c->stream>>>(A.n, A.rp, A.ci, A.v64, bm.as<unsigned long long>());
    MPET_CHECK_LAUNCH();
    unsigned long long bits = 0;
    MPET_CUDA(cudaMemcpyAsync(&bits, bm.p, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    double mx = 0.0;
    memcpy(&mx, &bits, sizeof(mx));
    if (!(mx > 0.0) || !std::isfinite(mx)) return;  // diagonal matrix: nothing to gain
    // the largest off-diagonal maps to [2^13, 2^14): far from the FP16 maximum, with
    // 2^-24 .. 2^14 (38 binades) of normal and subnormal range below it
    const int e = (int)std::ceil(std::log2(mx)) - 14;
    const double scale = std::ldexp(1.0, e);
    if (!device_fits(c, (size_t)nst * 2 + (size_t)A.n * 4)) return;
    A.s_v16 = c->pool.alloc<__half>(nst);
    A.s_d32 = c->pool.alloc<float>(A.n);
    A.s_h_scale = (float)scale;
    k_sell_fill_half<<<grid_for(A.nslices * 32, 256), 256, 0, c->stream>>>(A.n, A.nslices, A.rp, A.ci, A.v64, A.s_off,
                                                                          1.0 / scale, scale, A.s_v16, A.s_d32);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

__global__ void k_sell_width(int64_t n, int64_t nslices, const int64_t* __restrict__ rp, int64_t* w32) {
    const int64_t sl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (sl >= nslices) return;
    int64_t w = 0;
    const int64_t r1 = (sl + 1) * 32 < n ? (sl + 1) * 32 : n;
    for (int64_t r = sl * 32; r < r1; ++r) {
        const int64_t len = rp[r + 1] - rp[r];
        w = len > w ? len : w;
    }
    w32[sl] = 32 * w;
}

template <typename T>
__global__ void k_sell_fill(int64_t n, int64_t nslices, const int64_t* __restrict__ rp,
                            const int32_t* __restrict__ ci, const T* __restrict__ v,
                            const int64_t* __restrict__ soff, int32_t* sci, T* sv) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nslices * 32) return;
    const int64_t sl = t >> 5, lane = t & 31, row = t;
    const int64_t w = (soff[sl + 1] - soff[sl]) >> 5;
    const int64_t e0 = row < n ? rp[row] : 0, len = row < n ? rp[row + 1] - e0 : 0;
    // padding repeats the row's last column (a valid index of x, and a line
    // the row has just read), or column 0 for an empty row
    const int32_t pad = len > 0 ? ci[e0 + len - 1] : 0;
    for (int64_t k = 0; k < w; ++k) {
        const int64_t q = soff[sl] + k * 32 + lane;
        if (k < len) {
            sci[q] = ci[e0 + k];
            sv[q] = v[e0 + k];
        } else {
            sci[q] = pad;
            sv[q] = T(0);
        }
    }
}

// ---- node-block SpMV of the system matrix --------------------------------------------
//
// One thread owns a P2 node (its 3 displacement rows) or a vertex (its J
// pressure rows); a warp walks a 32-row-group slice.  Per block it loads one
// column id and the block's values (each a coalesced 128-byte line across the
// warp), gathers the 3 displacement or J pressure entries of x and updates
// its 3 or J accumulators.  JM is a compile-time bound on J (loops unrolled).
// UU: the displacement block only (u slices, node columns), x of length Nu.
// FP64 instances are register-bound (each 3 x 3 block is 9 doubles): they load one
// block per iteration, are held to 80 registers (3 resident 256-thread blocks per
// SM) and run as one wave of resident blocks (the reduction partials past the grid
// are written as zeros).
// OCC (FP32 only): held to 64 registers, 4 resident blocks per SM (variant 9).
// PU: the pressure slices only, their displacement (node) columns only.
template <typename T, int JM, class Epi, bool UU = false, bool OCC = false, bool PU = false>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 3 : (OCC ? 4 : 1)) k_spmv_nb(int64_t nnodes, int64_t nv, int64_t Nu, int J, int64_t nsu,
                                                 int64_t ns, const NbSlice* __restrict__ sl,
                                                 const int32_t* __restrict__ perm, const int32_t* __restrict__ cols,
                                                 const T* __restrict__ vals, const T* __restrict__ x, Epi epi,
                                                 double* partials, const int32_t* __restrict__ skl = nullptr,
                                                 const double* __restrict__ skip = nullptr) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double r0 = 0.0, r1 = 0.0;
    for (int64_t s = (PU ? nsu : 0) + warp; s < ns; s += nwarps) {
        if (skl && slice_frozen(skl, s, skip)) continue;
        const NbSlice S = sl[s];
        const int32_t* c2 = cols + S.coff + lane;
        const int32_t* c1 = c2 + (int64_t)S.w2 * 32;
        const T* v2 = vals + S.voff + lane;
        const int64_t g = perm[s * 32 + lane];  // node or vertex of this lane, -1 past the end
        const bool ok = g >= 0;
        if (s < nsu) {
            const int64_t node = g;
            typename Epi::Pre pre[3];
            if (ok)
#pragma unroll
                for (int r = 0; r < 3; ++r) pre[r] = epi.pre(3 * node + r);
            T acc[3] = {T(0), T(0), T(0)};
#pragma unroll(sizeof(T) == 8 ? 1 : 2)
            for (int k = 0; k < S.w2; ++k) {
                const int64_t j = __ldcs(c2 + (int64_t)k * 32);
                T b[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) b[q] = __ldcs(v2 + ((int64_t)k * 9 + q) * 32);
                const T x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
#pragma unroll
                for (int r = 0; r < 3; ++r) acc[r] += b[3 * r] * x0 + b[3 * r + 1] * x1 + b[3 * r + 2] * x2;
            }
            const T* v1 = v2 + (int64_t)S.w2 * 9 * 32;
            const int B1 = 3 * J;
            for (int m = 0; m < (UU ? 0 : S.w1); ++m) {
                const int64_t w = __ldcs(c1 + (int64_t)m * 32);
#pragma unroll
                for (int a = 0; a < JM; ++a) {
                    if (a < J) {
                        const T xp = x[Nu + (int64_t)a * nv + w];
#pragma unroll
                        for (int r = 0; r < 3; ++r) acc[r] += __ldcs(v1 + ((int64_t)m * B1 + r * J + a) * 32) * xp;
                    }
                }
            }
            if (ok)
#pragma unroll
                for (int r = 0; r < 3; ++r) epi.apply(3 * node + r, &acc[r], pre[r], r0, r1);
        } else {
            const int64_t v = g;
            typename Epi::Pre pre[JM];
#pragma unroll
            for (int a = 0; a < JM; ++a)
                if (ok && a < J) pre[a] = epi.pre(Nu + (int64_t)a * nv + v);
            T acc[JM];
#pragma unroll
            for (int a = 0; a < JM; ++a) acc[a] = T(0);
            const int B2 = 3 * J;
#pragma unroll(sizeof(T) == 8 ? 1 : 2)
            for (int k = 0; k < S.w2; ++k) {
                const int64_t j = __ldcs(c2 + (int64_t)k * 32);
                const T x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
#pragma unroll
                for (int a = 0; a < JM; ++a) {
                    if (a < J) {
                        const T* b = v2 + ((int64_t)k * B2 + 3 * a) * 32;
                        acc[a] += __ldcs(b) * x0 + __ldcs(b + 32) * x1 + __ldcs(b + 64) * x2;
                    }
                }
            }
            const T* v1 = v2 + (int64_t)S.w2 * B2 * 32;
            const int B1 = J * J;
            for (int m = 0; m < (PU ? 0 : S.w1); ++m) {
                const int64_t w = __ldcs(c1 + (int64_t)m * 32);
#pragma unroll
                for (int b = 0; b < JM; ++b) {
                    if (b < J) {
                        const T xb = x[Nu + (int64_t)b * nv + w];
#pragma unroll
                        for (int a = 0; a < JM; ++a)
                            if (a < J) acc[a] += __ldcs(v1 + ((int64_t)m * B1 + a * J + b) * 32) * xb;
                    }
                }
            }
            if (ok)
#pragma unroll
                for (int a = 0; a < JM; ++a)
                    if (a < J) epi.apply(Nu + (int64_t)a * nv + v, &acc[a], pre[a], r0, r1);
        }
    }
    if constexpr (Epi::kRed > 0) {
        __shared__ double sh[8];
        const double t0 = block_sum256(r0, sh);
        const double t1 = Epi::kRed > 1 ? block_sum256(r1, sh) : 0.0;
        if (threadIdx.x == 0)
            for (int p = blockIdx.x; p < NB_RED; p += gridDim.x) {
                partials[p] = p == (int)blockIdx.x ? t0 : 0.0;
                if (Epi::kRed > 1) partials[NB_RED + p] = p == (int)blockIdx.x ? t1 : 0.0;
            }
    }
}

// Copies the CSR values into the node-block layout (thread per slice lane).
// A row group's CSR row holds its node columns (3 per node, n2 order) and
// then, network-major, its vertex columns (n1 order).
template <typename T, typename Tin>
__global__ void k_nb_fill(int64_t nnodes, int64_t nv, int64_t Nu, int J, int64_t nsu, int64_t ns,
                          const NbSlice* __restrict__ sl, const int32_t* __restrict__ perm,
                          const int64_t* __restrict__ rp,
                          const Tin* __restrict__ v, const int64_t* __restrict__ n2_ptr,
                          const int32_t* __restrict__ n2_col, const int64_t* __restrict__ n1_ptr,
                          const int32_t* __restrict__ n1_col, int32_t* cols, T* vals, int write_cols) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ns * 32) return;
    const int64_t s = t >> 5;
    const int lane = (int)(t & 31);
    const NbSlice S = sl[s];
    const bool urow = s < nsu;
    const int64_t g = perm[t];  // node or vertex, -1 past the end
    const bool ok = g >= 0;
    const int64_t s2 = ok ? n2_ptr[g] : 0, s1 = ok ? n1_ptr[g] : 0;
    const int d2 = ok ? (int)(n2_ptr[g + 1] - s2) : 0, d1 = ok ? (int)(n1_ptr[g + 1] - s1) : 0;
    const int R = urow ? 3 : J;                       // rows of the group
    const int B2 = urow ? 9 : 3 * J, B1 = urow ? 3 * J : J * J;
    auto row_start = [&](int r) -> int64_t { return urow ? rp[3 * g + r] : rp[Nu + (int64_t)r * nv + g]; };
    for (int k = 0; k < S.w2; ++k) {
        const bool real = k < d2;
        if (write_cols)
            cols[S.coff + (int64_t)k * 32 + lane] = real ? n2_col[s2 + k] : (d2 > 0 ? n2_col[s2 + d2 - 1] : 0);
        for (int r = 0; r < R; ++r) {
            const int64_t e = real ? row_start(r) + 3 * k : 0;
            for (int cc = 0; cc < 3; ++cc)
                vals[S.voff + ((int64_t)k * B2 + r * 3 + cc) * 32 + lane] = real ? (T)v[e + cc] : T(0);
        }
    }
    const int64_t c1 = S.coff + (int64_t)S.w2 * 32, v1 = S.voff + (int64_t)S.w2 * B2 * 32;
    for (int m = 0; m < S.w1; ++m) {
        const bool real = m < d1;
        if (write_cols)
            cols[c1 + (int64_t)m * 32 + lane] = real ? n1_col[s1 + m] : (d1 > 0 ? n1_col[s1 + d1 - 1] : 0);
        for (int r = 0; r < R; ++r) {
            const int64_t base = real ? row_start(r) + 3 * d2 + m : 0;
            for (int b = 0; b < J; ++b)
                vals[v1 + ((int64_t)m * B1 + r * J + b) * 32 + lane] = real ? (T)v[base + (int64_t)b * d1] : T(0);
        }
    }
}

// ---- shared-memory staged SpMV (bulk async copies) ----------------------------------
//
// A CTA walks a list of row tiles; each tile's column ids and values are a
// contiguous range of the CSR arrays, copied to shared memory by one
// cp.async.bulk per array (completion counted on an mbarrier).  Two buffers
// alternate: while the warps reduce tile t from one buffer, the copy of the
// CTA's next tile streams into the other, so HBM is fed by the copy engine
// and the warps only wait on the x gathers (L2) and shared-memory reads.
// The copy start is rounded down and its end up to 4 entries (16 bytes); the
// 64-byte tail of every pool allocation covers the read past the last entry.

constexpr int SPMV_CAP = SPMV_TILE + 8;  // buffer entries (alignment slack)
constexpr int MBAR_SPIN_LIMIT = 1 << 22;    // default bound of a tile wait (try_wait polls)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait for the phase with the given parity; false if it never completed
// within `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = MBAR_SPIN_LIMIT) {
    for (int it = 0; it < limit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

template <typename T>
constexpr size_t staged_smem_bytes() {
    return 128 + 2 * (size_t)SPMV_CAP * (4 + sizeof(T));
}

template <typename T, int NV, int LPR, int U, class Epi>
__global__ void __launch_bounds__(256) k_spmv_staged(const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                                     const T* __restrict__ va, const T* __restrict__ x, Epi epi,
                                                     double* partials, const int32_t* __restrict__ tiles, int ntiles,
                                                     int* err, int spin_limit) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    unsigned char* base = smem + 128;
    constexpr size_t bufb = (size_t)SPMV_CAP * (4 + sizeof(T));
    auto scol = [&](int bb) { return (int32_t*)(base + bb * bufb); };
    auto sval = [&](int bb) { return (T*)(base + bb * bufb + (size_t)SPMV_CAP * 4); };
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int t, int b) {
        const int64_t a0 = rp[tiles[t]] & ~3LL;
        const int64_t a1 = (rp[tiles[t + 1]] + 3) & ~3LL;
        const uint32_t cnt = (uint32_t)(a1 - a0);
        mbar_expect_tx(&bar[b], cnt * (uint32_t)(4 + sizeof(T)));
        bulk_copy_g2s(scol(b), ci + a0, cnt * 4u, &bar[b]);
        bulk_copy_g2s(sval(b), va + a0, cnt * (uint32_t)sizeof(T), &bar[b]);
    };
    const int sub = threadIdx.x & (LPR - 1);
    const int gid = threadIdx.x / LPR;
    constexpr int NGR = 256 / LPR;
    double r0 = 0.0, r1 = 0.0;
    uint32_t ph0 = 0, ph1 = 0;
    bool pending0 = false, pending1 = false;
    int b = 0;
    if (threadIdx.x == 0 && (int)blockIdx.x < ntiles) {
        issue(blockIdx.x, 0);
        pending0 = true;
    }
    bool bad = false;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < ntiles) {
            issue(tn, b ^ 1);
            if (b) pending0 = true; else pending1 = true;
        }
        const bool ok = mbar_wait(&bar[b], b ? ph1 : ph0, spin_limit);
        // a buffer whose wait gave up stays pending at its parity, so the
        // drain below waits for exactly that copy
        if (ok) {
            if (b) { ph1 ^= 1u; pending1 = false; } else { ph0 ^= 1u; pending0 = false; }
        }
        if (__syncthreads_or(!ok)) {
            bad = true;
            break;
        }
        const int64_t rs = tiles[t], re = tiles[t + 1];
        const int64_t a0 = rp[rs] & ~3LL;
        const int32_t* sc = scol(b);
        const T* sv = sval(b);
        for (int64_t rb = rs; rb < re; rb += NGR) {
            const int64_t row = rb + gid;
            T acc[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] = T(0);
            typename Epi::Pre pre{};
            if (row < re && sub == 0) pre = epi.pre(row);
            if (row < re) {
                // batches of U entries per lane: all shared-memory reads, then
                // all x gathers, then the FMAs (indices clamped into the row)
                const int s = (int)(rp[row] - a0), e = (int)(rp[row + 1] - a0);
                for (int q0 = s; q0 < e; q0 += LPR * U) {
                    int32_t cc[U];
                    T aa[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int q = q0 + sub + u * LPR;
                        const int qs = q < e ? q : e - 1;
                        cc[u] = sc[qs];
                        aa[u] = q < e ? sv[qs] : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (q0 + sub + u * LPR < e) {
                            T xv[NV];
                            VecIO<T, NV>::load(x, cc[u], xv);
#pragma unroll
                            for (int k = 0; k < NV; ++k) acc[k] += aa[u] * xv[k];
                        }
                    }
                }
            }
#pragma unroll
            for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < NV; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
            if (row < re && sub == 0) epi.apply(row, acc, pre, r0, r1);
        }
        __syncthreads();  // buffer b consumed before it is refilled
        b ^= 1;
    }
    if (bad) {
        // record the failure and let any copy still in flight land (bounded by
        // the default limit, whatever limit the tile waits had)
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            if (pending0) mbar_wait(&bar[0], ph0);
            if (pending1) mbar_wait(&bar[1], ph1);
        }
        __syncthreads();
    }
    if constexpr (Epi::kRed > 0) {
        __shared__ double sh[8];
        double t0 = block_sum256(r0, sh);
        double t1 = (Epi::kRed > 1) ? block_sum256(r1, sh) : 0.0;
        if (threadIdx.x == 0) {
            for (int p = blockIdx.x; p < NB_RED; p += gridDim.x) {
                partials[p] = p == (int)blockIdx.x ? t0 : 0.0;
                if (Epi::kRed > 1) partials[NB_RED + p] = p == (int)blockIdx.x ? t1 : 0.0;
            }
        }
    }
}

template <typename T, int NV, int LPR, int U, class Epi>
static void launch_staged(mpet_ctx* c, const Csr& A, const T* va, const T* x, const Epi& epi) {
    static int grid = 0;  // resident CTAs on this device (one per instantiation)
    auto kern = k_spmv_staged<T, NV, LPR, U, Epi>;
    const size_t sm = staged_smem_bytes<T>();
    if (grid == 0) {
        MPET_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        int per_sm = 0, nsm = 0, dev = 0;
        MPET_CUDA(cudaGetDevice(&dev));
        MPET_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        MPET_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, sm));
        grid = nsm * (per_sm > 0 ? per_sm : 1);
        if (grid > NB_RED) grid = NB_RED;
    }
    kern<<<grid, 256, sm, c->stream>>>(A.rp, A.ci, va, x, epi, c->partials, A.tiles, A.ntiles, c->dev_err,
                                       c->mbar_spin_limit);
    MPET_CHECK_LAUNCH();
    c->n_launch++;
}

void build_tiles(mpet_ctx* c, Csr& A, const int64_t* rp) {
    A.ntiles = 0;
    A.tiles = nullptr;
    A.max_row = 0;
    for (int64_t r = 0; r < A.n; ++r) A.max_row = std::max<int64_t>(A.max_row, rp[r + 1] - rp[r]);
    if (A.nnz < (int64_t)SPMV_TILE * 64) return;  // small matrices: register kernel
    std::vector<int32_t> t;
    t.push_back(0);
    int64_t start = rp[0];
    for (int64_t r = 0; r < A.n; ++r) {
        const int64_t len = rp[r + 1] - rp[r];
        if (len > SPMV_TILE / 2) return;  // long rows: register kernel
        if (rp[r + 1] - start > SPMV_TILE) {
            t.push_back((int32_t)r);
            start = rp[r];
        }
    }
    t.push_back((int32_t)A.n);
    A.tiles = c->pool.alloc<int32_t>((int64_t)t.size());
    MPET_CUDA(cudaMemcpyAsync(A.tiles, t.data(), sizeof(int32_t) * t.size(), cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    A.ntiles = (int)t.size() - 1;
}

template <typename T>
static const T* vals(const Csr& A);
template <>
const double* vals<double>(const Csr& A) { return A.v64; }
template <>
const float* vals<float>(const Csr& A) { return A.v32; }

// SELL-32 layout of a matrix (slice offsets scanned on the host, column
// ids and values allocated in the precision given, plus FP64 values when
// with64: the system matrix of the mixed path, whose refinement residual is
// FP64); fill_sell copies the current CSR values in (again after every
// change of the values).
void build_sell(mpet_ctx* c, Csr& A, bool fp32, bool with64) {
    if (A.n == 0 || A.nnz == 0) return;
    const int64_t ns = (A.n + 31) / 32;
    int64_t* w = c->pool.alloc<int64_t>(ns + 1);
    k_sell_width<<<grid_for(ns, 256), 256, 0, c->stream>>>(A.n, ns, A.rp, w);
    MPET_CHECK_LAUNCH();
    std::vector<int64_t> off(ns + 1);
    MPET_CUDA(cudaMemcpyAsync(off.data(), w, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    int64_t acc = 0;
    for (int64_t s = 0; s < ns; ++s) {
        const int64_t ws = off[s];
        off[s] = acc;
        acc += ws;
    }
    off[ns] = acc;
    if (!device_fits(c, (size_t)acc * (4 + (fp32 ? 4 : 0) + ((!fp32 || with64) ? 8 : 0)))) return;
    A.nslices = ns;
    A.s_off = w;
    MPET_CUDA(cudaMemcpyAsync(A.s_off, off.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, c->stream));
    A.s_ci = c->pool.alloc<int32_t>(acc);
    if (fp32) A.s_v32 = c->pool.alloc<float>(acc);
    if (!fp32 || with64) A.s_v64 = c->pool.alloc<double>(acc);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    fill_sell(c, A);
}

void fill_sell(mpet_ctx* c, Csr& A) {
    if (!A.s_off) return;
    const int64_t ns = A.nslices;
    if (A.s_v32)
        k_sell_fill<float><<<grid_for(ns * 32, 256), 256, 0, c->stream>>>(A.n, ns, A.rp, A.ci, A.v32, A.s_off,
                                                                          A.s_ci, A.s_v32);
    if (A.s_v64)
        k_sell_fill<double><<<grid_for(ns * 32, 256), 256, 0, c->stream>>>(A.n, ns, A.rp, A.ci, A.v64, A.s_off,
                                                                           A.s_ci, A.s_v64);
    MPET_CHECK_LAUNCH();
}

// Node-block layout of the system matrix: slice widths from the node and
// vertex adjacency counts (host), values filled on the device.
void build_node_blocks(mpet_ctx* c) {
    NodeBlocks& nb = c->A_nb;
    if (c->dim != 3) return;  // 3-row displacement groups
    const int J = c->J;
    std::vector<int64_t> p2(c->nnodes + 1), p1(c->nnodes + 1);
    MPET_CUDA(cudaMemcpyAsync(p2.data(), c->n2_ptr, sizeof(int64_t) * p2.size(), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaMemcpyAsync(p1.data(), c->n1_ptr, sizeof(int64_t) * p1.size(), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    nb.nsu = (c->nnodes + 31) / 32;
    nb.nsp = (c->nv + 31) / 32;
    // lanes take the row groups of each window of NB_WINDOW groups in order of
    // decreasing size (few padded blocks, locality kept within the window)
    constexpr int64_t NB_WINDOW = 2048;
    std::vector<int32_t> perm((nb.nsu + nb.nsp) * 32, -1);
    auto order = [&](int64_t n, int64_t base, int B2, int B1) {
        std::vector<int32_t> idx;
        for (int64_t w0 = 0; w0 < n; w0 += NB_WINDOW) {
            const int64_t w1 = std::min(w0 + NB_WINDOW, n);
            idx.resize(w1 - w0);
            for (int64_t g = w0; g < w1; ++g) idx[g - w0] = (int32_t)g;
            std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) {
                return (p2[a + 1] - p2[a]) * B2 + (p1[a + 1] - p1[a]) * B1 >
                       (p2[b + 1] - p2[b]) * B2 + (p1[b + 1] - p1[b]) * B1;
            });
            std::copy(idx.begin(), idx.end(), perm.begin() + base + w0);
        }
    };
    order(c->nnodes, 0, 9, 3 * J);
    order(c->nv, nb.nsu * 32, 3 * J, J * J);
    std::vector<NbSlice> sl(nb.nsu + nb.nsp);
    int64_t coff = 0, voff = 0;
    for (int64_t s = 0; s < nb.nsu + nb.nsp; ++s) {
        const bool urow = s < nb.nsu;
        int32_t w2 = 0, w1 = 0;
        for (int l = 0; l < 32; ++l) {
            const int32_t g = perm[s * 32 + l];
            if (g < 0) continue;
            w2 = std::max<int32_t>(w2, (int32_t)(p2[g + 1] - p2[g]));
            w1 = std::max<int32_t>(w1, (int32_t)(p1[g + 1] - p1[g]));
        }
        sl[s] = NbSlice{coff, voff, w2, w1};
        coff += (int64_t)(w2 + w1) * 32;
        voff += (urow ? (int64_t)w2 * 9 + (int64_t)w1 * 3 * J : (int64_t)w2 * 3 * J + (int64_t)w1 * J * J) * 32;
    }
    const bool mixed = c->prm.precision == MPET_PRECISION_MIXED;
    const size_t need = (size_t)coff * 4 + (size_t)voff * (mixed ? 4 : 8) + perm.size() * 4;
    if (!device_fits(c, need)) return;  // optional copy: skipped when HBM is short
    nb.ncols = coff;
    nb.nvals = voff;
    nb.nblocks = (p2[c->nnodes] - p2[0]) + (p1[c->nnodes] - p1[0]) + (p2[c->nv] - p2[0]) + (p1[c->nv] - p1[0]);
    nb.sl = c->pool.alloc<NbSlice>((int64_t)sl.size());
    nb.perm = c->pool.alloc<int32_t>((int64_t)perm.size());
    MPET_CUDA(cudaMemcpyAsync(nb.perm, perm.data(), sizeof(int32_t) * perm.size(), cudaMemcpyHostToDevice,
                              c->stream));
    nb.cols = c->pool.alloc<int32_t>(coff);
    if (mixed) nb.v32 = c->pool.alloc<float>(voff);
    // FP64 values: the Krylov matrix of the FP64 path, the refinement residual's of the mixed path
    if (!mixed || device_fits(c, (size_t)voff * 8)) nb.v64 = c->pool.alloc<double>(voff);
    MPET_CUDA(cudaMemcpyAsync(nb.sl, sl.data(), sizeof(NbSlice) * sl.size(), cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->A.nb = &nb;
}

static void fill_node_blocks(mpet_ctx* c) {
    NodeBlocks& nb = c->A_nb;
    if (!nb.sl) return;
    const int64_t ns = nb.nsu + nb.nsp;
    const int G = grid_for(ns * 32, 128);
    int first = 1;
    if (nb.v32) {
        // from the FP32 CSR values when they exist (same rounding as the CSR kernels), else from FP64
        if (c->A.v32)
            k_nb_fill<float, float><<<G, 128, 0, c->stream>>>(c->nnodes, c->nv, c->Nu, c->J, nb.nsu, ns, nb.sl,
                                                              nb.perm, c->A.rp, c->A.v32, c->n2_ptr, c->n2_col,
                                                              c->n1_ptr, c->n1_col, nb.cols, nb.v32, first);
        else
            k_nb_fill<float, double><<<G, 128, 0, c->stream>>>(c->nnodes, c->nv, c->Nu, c->J, nb.nsu, ns, nb.sl,
                                                               nb.perm, c->A.rp, c->A.v64, c->n2_ptr, c->n2_col,
                                                               c->n1_ptr, c->n1_col, nb.cols, nb.v32, first);
        first = 0;
    }
    if (nb.v64)
        k_nb_fill<double, double><<<G, 128, 0, c->stream>>>(c->nnodes, c->nv, c->Nu, c->J, nb.nsu, ns, nb.sl,
                                                            nb.perm, c->A.rp, c->A.v64, c->n2_ptr, c->n2_col,
                                                            c->n1_ptr, c->n1_col, nb.cols, nb.v64, first);
    MPET_CHECK_LAUNCH();
}

// After every change of the system matrix values: its SELL and node-block copies.
void refresh_system_copies(mpet_ctx* c) {
    fill_sell(c, c->A);
    fill_node_blocks(c);
}

template <typename T>
static const T* nb_vals(const NodeBlocks& nb);
template <>
const double* nb_vals<double>(const NodeBlocks& nb) { return nb.v64; }
template <>
const float* nb_vals<float>(const NodeBlocks& nb) { return nb.v32; }

// resident 256-thread blocks of a kernel on the current device (one wave), at most NB_RED
template <class K>
static int one_wave(K kern) {
    int per_sm = 0, nsm = 0, dev = 0;
    MPET_CUDA(cudaGetDevice(&dev));
    MPET_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    MPET_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
    const int g = nsm * (per_sm > 0 ? per_sm : 1);
    return g < NB_RED ? g : NB_RED;
}

template <typename T, class Epi>
static void launch_nb(mpet_ctx* c, const NodeBlocks& nb, const T* x, const Epi& epi, bool occ = false) {
    const int64_t ns = nb.nsu + nb.nsp;
    int blocks = Epi::kRed > 0 ? NB_RED : grid_for(ns * 32, 256);
    if (Epi::kRed == 0 && blocks > 152 * 16) blocks = 152 * 16;
    if (sizeof(T) == 8 && Epi::kRed > 0) {
        static int wave = 0;  // per instantiation (one device type per process)
        if (wave == 0) wave = one_wave(k_spmv_nb<T, 4, Epi>);
        blocks = wave;
    }
    const int J = c->J;
    cudaStream_t st = c->stream;
    const T* v = nb_vals<T>(nb);
    const int32_t* skl = c->skip_done ? nb.skl : nullptr;
    if (occ && sizeof(T) == 4) {
        if (J <= 2)
            k_spmv_nb<T, 2, Epi, false, true><<<blocks, 256, 0, st>>>(c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl,
                                                                      nb.perm, nb.cols, v, x, epi, c->partials, skl,
                                                                      c->skip_done);
        else if (J <= 4)
            k_spmv_nb<T, 4, Epi, false, true><<<blocks, 256, 0, st>>>(c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl,
                                                                      nb.perm, nb.cols, v, x, epi, c->partials, skl,
                                                                      c->skip_done);
        else
            k_spmv_nb<T, 8, Epi, false, true><<<blocks, 256, 0, st>>>(c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl,
                                                                      nb.perm, nb.cols, v, x, epi, c->partials, skl,
                                                                      c->skip_done);
    } else if (J <= 2)
        k_spmv_nb<T, 2, Epi><<<blocks, 256, 0, st>>>(c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl, nb.perm,
                                                     nb.cols, v, x, epi, c->partials, skl, c->skip_done);
    else if (J <= 4)
        k_spmv_nb<T, 4, Epi><<<blocks, 256, 0, st>>>(c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl, nb.perm,
                                                     nb.cols, v, x, epi, c->partials, skl, c->skip_done);
    else
        k_spmv_nb<T, 8, Epi><<<blocks, 256, 0, st>>>(c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl, nb.perm,
                                                     nb.cols, v, x, epi, c->partials, skl, c->skip_done);
    MPET_CHECK_LAUNCH();
    c->n_launch++;
}

// b += the pressure rows' displacement-column products (FP64 right-hand side term)
struct EpiAddRhs {
    double* b;
    static constexpr int kRed = 0;
    static constexpr bool kSystem = true;
    struct Pre {};
    __device__ __forceinline__ Pre pre(int64_t) const { return Pre{}; }
    __device__ __forceinline__ void apply(int64_t row, const double* acc, const Pre&, double&, double&) const {
        b[row] += acc[0];
    }
};

bool rhs_div_from_matrix(mpet_ctx* c, const double* up_prev, double* b) {
    if (!c->A.nb || !c->A.nb->v64 || c->dim != 3) return false;
    const NodeBlocks& nb = *c->A.nb;
    const int64_t ns = nb.nsu + nb.nsp;
    int blocks = grid_for(nb.nsp * 32, 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    const int J = c->J;
    cudaStream_t st = c->stream;
    if (J <= 2)
        k_spmv_nb<double, 2, EpiAddRhs, false, false, true><<<blocks, 256, 0, st>>>(
            c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl, nb.perm, nb.cols, nb.v64, up_prev, EpiAddRhs{b},
            c->partials, nullptr, nullptr);
    else if (J <= 4)
        k_spmv_nb<double, 4, EpiAddRhs, false, false, true><<<blocks, 256, 0, st>>>(
            c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl, nb.perm, nb.cols, nb.v64, up_prev, EpiAddRhs{b},
            c->partials, nullptr, nullptr);
    else
        k_spmv_nb<double, 8, EpiAddRhs, false, false, true><<<blocks, 256, 0, st>>>(
            c->nnodes, c->nv, c->Nu, J, nb.nsu, ns, nb.sl, nb.perm, nb.cols, nb.v64, up_prev, EpiAddRhs{b},
            c->partials, nullptr, nullptr);
    MPET_CHECK_LAUNCH();
    return true;
}

// displacement block of the node-block system copy: u slices only, no vertex columns
template <typename T, class Epi>
static void launch_nb_uu(mpet_ctx* c, const NodeBlocks& nb, const T* x, const Epi& epi) {
    int blocks = Epi::kRed > 0 ? NB_RED : grid_for(nb.nsu * 32, 256);
    if (Epi::kRed == 0 && blocks > 152 * 16) blocks = 152 * 16;
    k_spmv_nb<T, 2, Epi, true><<<blocks, 256, 0, c->stream>>>(c->nnodes, c->nv, c->Nu, c->J, nb.nsu, nb.nsu, nb.sl,
                                                             nb.perm, nb.cols, nb_vals<T>(nb), x, epi, c->partials);
    MPET_CHECK_LAUNCH();
    c->n_launch++;
}

template <typename T>
static const T* sell_vals(const Csr& A);
template <>
const double* sell_vals<double>(const Csr& A) { return A.s_v64; }
template <>
const float* sell_vals<float>(const Csr& A) { return A.s_v32; }

template <typename T, int NV, class Epi>
static void launch_spmv(mpet_ctx* c, const Csr& A, const T* va, const T* x, const Epi& epi) {
    // FP64 products of a matrix tuned on its FP32 copy use their own tuning when they have one
    const bool own64 = sizeof(T) == 8 && A.variant64 >= 0;
    const int variant = own64 ? A.variant64 : A.variant;
    const int lpr = own64 ? A.lpr64 : A.lpr;
    if constexpr (NV == 1 && Epi::kSystem) {
        if ((variant == 8 || variant == 9) && A.nb && nb_vals<T>(*A.nb) && va == vals<T>(A)) {
            launch_nb<T>(c, *A.nb, x, epi, variant == 9);
            return;
        }
    }
    const int32_t* skl = c->skip_done ? A.skl : nullptr;
    const double* skip = c->skip_done;
    if constexpr (sizeof(T) == 4) {
        if (variant == 32 && A.s_v16 && va == vals<T>(A)) {
            int blocks = Epi::kRed > 0 ? NB_RED : grid_for(A.nslices * 32, 256);
            if (Epi::kRed == 0 && blocks > 152 * 16) blocks = 152 * 16;
            k_spmv_sell_h<NV, 4, Epi><<<blocks, 256, 0, c->stream>>>(A.n, A.nslices, A.s_off, A.s_ci, A.s_v16, A.s_d32,
                                                                     A.s_h_scale, (const float*)x, epi, c->partials,
                                                                     skl, skip);
            MPET_CHECK_LAUNCH();
            c->n_launch++;
            return;
        }
    }
    if ((variant & 4) && sell_vals<T>(A) && va == vals<T>(A)) {
        int blocks = Epi::kRed > 0 ? NB_RED : grid_for(A.nslices * 32, 256);
        if (Epi::kRed == 0 && blocks > 152 * 16) blocks = 152 * 16;
        const T* sv = sell_vals<T>(A);
        switch (variant & 3) {
            case 0:
                k_spmv_sell<T, NV, 4, Epi><<<blocks, 256, 0, c->stream>>>(A.n, A.nslices, A.s_off, A.s_ci, sv, x, epi,
                                                                          c->partials, skl, skip);
                break;
            case 1:
                k_spmv_sell<T, NV, 8, Epi><<<blocks, 256, 0, c->stream>>>(A.n, A.nslices, A.s_off, A.s_ci, sv, x, epi,
                                                                          c->partials, skl, skip);
                break;
            case 2:
                k_spmv_sell_late<T, NV, 4, Epi><<<blocks, 256, 0, c->stream>>>(A.n, A.nslices, A.s_off, A.s_ci, sv,
                                                                               x, epi, c->partials, skl, skip);
                break;
            default:
                k_spmv_sell_late<T, NV, 8, Epi><<<blocks, 256, 0, c->stream>>>(A.n, A.nslices, A.s_off, A.s_ci, sv,
                                                                               x, epi, c->partials, skl, skip);
                break;
        }
        MPET_CHECK_LAUNCH();
        c->n_launch++;
        return;
    }
    const bool deep = lpr == 32 && (variant & 1);
    if (A.ntiles > 0 && (variant & 2)) {
        switch (lpr) {
            case 32:
                if (deep) launch_staged<T, NV, 32, 8, Epi>(c, A, va, x, epi);
                else launch_staged<T, NV, 32, 4, Epi>(c, A, va, x, epi);
                return;
            case 16: launch_staged<T, NV, 16, 4, Epi>(c, A, va, x, epi); return;
            case 8: launch_staged<T, NV, 8, 4, Epi>(c, A, va, x, epi); return;
            case 4: launch_staged<T, NV, 4, 4, Epi>(c, A, va, x, epi); return;
            default: launch_staged<T, NV, 1, 4, Epi>(c, A, va, x, epi); return;
        }
    }
    int blocks;
    if (Epi::kRed > 0) {
        blocks = NB_RED;
    } else {
        int64_t rows_per_block = 256 / lpr;
        blocks = grid_for(A.n, (int)rows_per_block);
        if (blocks > 152 * 16) blocks = 152 * 16;
    }
    double* part = c->partials;
    cudaStream_t s = c->stream;
    switch (lpr) {
        case 32:
            if (deep) k_spmv<T, NV, 32, 8, Epi><<<blocks, 256, 0, s>>>(A.n, A.rp, A.ci, va, x, epi, part, skl, skip);
            else k_spmv<T, NV, 32, 4, Epi><<<blocks, 256, 0, s>>>(A.n, A.rp, A.ci, va, x, epi, part, skl, skip);
            break;
        case 16:
            k_spmv<T, NV, 16, 4, Epi><<<blocks, 256, 0, s>>>(A.n, A.rp, A.ci, va, x, epi, part, skl, skip);
            break;
        case 8: k_spmv<T, NV, 8, 4, Epi><<<blocks, 256, 0, s>>>(A.n, A.rp, A.ci, va, x, epi, part, skl, skip); break;
        case 4: k_spmv<T, NV, 4, 4, Epi><<<blocks, 256, 0, s>>>(A.n, A.rp, A.ci, va, x, epi, part, skl, skip); break;
        default: k_spmv<T, NV, 1, 4, Epi><<<blocks, 256, 0, s>>>(A.n, A.rp, A.ci, va, x, epi, part, skl, skip); break;
    }
    MPET_CHECK_LAUNCH();
    c->n_launch++;
}

// Matrix-free product with the first displacement level w (grad u, grad v)
// (+ shift (u, v)) on the 4-wide node layout: a thread owns a P2 node, walks its
// incident cells (node -> cell incidence) and adds its row of each cell's element
// operator, K_mj = sum_{p <= q} T6[mj][pq] a_pq + sh M2[m][j] with the cell's
// a_pq = w |T| kappa (b_p . b_q) and sh = shift |T| (k_mf_cells).  Dirichlet rows
// are the identity and Dirichlet columns are skipped (the cell's mask), as in the
// CSR block.  Reads per product: the incidence, 8 values and NN node ids per
// incident cell (mostly from L2) and the gathered x, against nnz (value + column)
// of the CSR block.
template <typename T, int D, class Epi>
__global__ void __launch_bounds__(256) k_p2lap_mf(int64_t nnodes, const int64_t* __restrict__ inc_ptr,
                                                  const int32_t* __restrict__ inc,
                                                  const int32_t* __restrict__ cell_nodes, const T* __restrict__ cdat,
                                                  const uint8_t* __restrict__ node_bc, const float* __restrict__ tab,
                                                  const T* __restrict__ x, Epi epi) {
    constexpr int NN = Simplex<D>::NN, NQ = D * (D + 1) / 2, NP = NN * (NN + 1) / 2;
    __shared__ float s_t6[NP * NQ];
    __shared__ float s_m2[NN * NN];
    for (int e = threadIdx.x; e < NP * NQ + NN * NN; e += blockDim.x) {
        if (e < NP * NQ) s_t6[e] = tab[e];
        else s_m2[e - NP * NQ] = tab[e];
    }
    __syncthreads();
    double r0 = 0.0, r1 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        const typename Epi::Pre pre = epi.pre(i);
        T acc[4] = {T(0), T(0), T(0), T(0)};
        if (node_bc[i]) {
            VecIO<T, 4>::load(x, i, acc);
        } else {
            const int64_t e1 = inc_ptr[i + 1];
            for (int64_t it = inc_ptr[i]; it < e1; ++it) {
                const int32_t packed = __ldg(inc + it);
                const int64_t cell = packed >> 4;
                const int m = packed & 15;
                T a[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) a[q] = __ldg(cdat + 8 * cell + q);
                uint32_t mask;
                if constexpr (sizeof(T) == 4) mask = __float_as_uint(a[7]);
                else mask = (uint32_t)__double_as_longlong(a[7]);
                const int32_t* cn = cell_nodes + NN * cell;
#pragma unroll
                for (int j = 0; j < NN; ++j) {
                    if ((mask >> j) & 1u) continue;
                    const int lo = m < j ? m : j, hi = m < j ? j : m;
                    const int pr = lo * NN - lo * (lo - 1) / 2 + (hi - lo);
                    T coef = a[NQ] * (T)s_m2[m * NN + j];
#pragma unroll
                    for (int q = 0; q < NQ; ++q) coef += (T)s_t6[pr * NQ + q] * a[q];
                    T xv[4];
                    VecIO<T, 4>::load(x, __ldg(cn + j), xv);
#pragma unroll
                    for (int k = 0; k < 4; ++k) acc[k] += coef * xv[k];
                }
            }
        }
        epi.apply(i, acc, pre, r0, r1);
    }
}

template <typename T, class Epi>
static void launch_p2lap_mf(mpet_ctx* c, const T* x, const Epi& epi) {
    static_assert(Epi::kRed == 0, "no reductions in the matrix-free level");
    int blocks = grid_for(c->nnodes, 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (c->dim == 2)
        k_p2lap_mf<T, 2, Epi><<<blocks, 256, 0, c->stream>>>(c->nnodes, c->inc_ptr, c->inc, c->cell_nodes,
                                                             (const T*)c->mf_cell, c->node_bc, c->mf_tab, x, epi);
    else
        k_p2lap_mf<T, 3, Epi><<<blocks, 256, 0, c->stream>>>(c->nnodes, c->inc_ptr, c->inc, c->cell_nodes,
                                                             (const T*)c->mf_cell, c->node_bc, c->mf_tab, x, epi);
    MPET_CHECK_LAUNCH();
    c->n_launch++;
}

// operator of an AMG level: its CSR copy, the matrix-free first displacement
// level, or the displacement block of the system
template <typename T, int NV, class Epi>
static void level_spmv(mpet_ctx* c, const AmgLevel& L, const T* x, const Epi& epi) {
    if constexpr (NV == 1) {
        if (L.nb_uu) {
            launch_nb_uu<T>(c, *c->A.nb, x, epi);
            return;
        }
    }
    if constexpr (NV == 4) {
        if (L.mf) {
            launch_p2lap_mf<T>(c, x, epi);
            return;
        }
    }
    launch_spmv<T, NV>(c, L.A, vals<T>(L.A), x, epi);
}

template <typename T>
static const T* dinv_of(const AmgLevel& L);
template <>
const double* dinv_of<double>(const AmgLevel& L) { return L.dinv64; }
template <>
const float* dinv_of<float>(const AmgLevel& L) { return L.dinv32; }

// Variant v (bits as in Csr::variant) can run on A with its current lanes
// per row: staged needs row tiles, SELL its copy, 8 entries per lane (CSR)
// 32 lanes per row.
bool spmv_variant_available(const Csr& A, int v) {
    if (v == 32) return A.s_v16 != nullptr;
    if (v == 8) return A.nb != nullptr;
    if (v == 9) return A.nb != nullptr && A.v32 != nullptr;  // FP32 node blocks at 4 blocks per SM
    if (v < 0 || v > 5) return false;
    if (v & 4) return A.s_off != nullptr;  // 6, 7: SELL with late epilogue loads
    if ((v & 2) && A.ntiles == 0) return false;
    if ((v & 1) && A.lpr != 32) return false;
    return true;
}

// Set-up autotuning: time every applicable SpMV variant on this matrix (CSR
// with its lanes per row, half and double that; SELL-32; node blocks) with
// the epilogue it runs in the solver (1 warm-up + median of 7 launches) and
// keep the fastest, the default CSR kernel winning ties within 3%.  Times (ms
// per launch) go to ms_out if given.  A matrix larger than a quarter of L2 is
// timed from a flushed L2 (in the solver it streams from HBM every time); a
// smaller one, a coarse AMG level read by several Chebyshev products in a
// row, is timed warm, as it runs after its first product.
template <typename T, int NV, class Epi>
static void autotune_matrix(mpet_ctx* c, Csr& A, const T* x, const Epi& epi, double* ms_out = nullptr) {
    if (vals<T>(A) == nullptr || A.nnz == 0) return;
    const int64_t l0 = c->n_launch;
    float best = 1e30f;
    int best_v = 0, best_lpr = A.lpr;
    const int lpr0 = A.lpr;
    const double mbytes = (double)A.nnz * (sizeof(T) + 4) + (double)(A.n + 1) * 8;
    const bool flush = mbytes > 32.0 * 1024 * 1024;
    constexpr size_t kFlush = 256u << 20;
    if (!c->l2_flush) c->l2_flush = c->pool.alloc<unsigned char>(kFlush);
    for (int lpr : {lpr0, lpr0 / 2, lpr0 * 2}) {
        if ((lpr < 4 || lpr > 32) && lpr != lpr0) continue;
        A.lpr = lpr;
        for (int v : {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 32}) {
            if (v == 32 && (sizeof(T) != 4 || !A.s_v16 || lpr != lpr0)) continue;
            if (v == 9 && sizeof(T) != 4) continue;
            if (!spmv_variant_available(A, v) || (v >= 4 && v < 8 && (!sell_vals<T>(A) || lpr != lpr0))) continue;
            if ((v == 8 || v == 9) && (!Epi::kSystem || NV != 1 || !nb_vals<T>(*A.nb) || lpr != lpr0)) continue;
            // batches: the staged kernel has no slice skipping
            if (c->ninst > 0 && c->batch_skip && v < 4 && (v & 2)) continue;
            A.variant = v;
            launch_spmv<T, NV>(c, A, vals<T>(A), x, epi);
            float t[7];
            for (int q = 0; q < 7; ++q) {
                if (flush) MPET_CUDA(cudaMemsetAsync(c->l2_flush, q, kFlush, c->stream));
                MPET_CUDA(cudaEventRecord(c->ev0, c->stream));
                launch_spmv<T, NV>(c, A, vals<T>(A), x, epi);
                MPET_CUDA(cudaEventRecord(c->ev1, c->stream));
                MPET_CUDA(cudaEventSynchronize(c->ev1));
                MPET_CUDA(cudaEventElapsedTime(&t[q], c->ev0, c->ev1));
            }
            std::sort(t, t + 7);
            // median; a variant replaces the incumbent only when clearly faster,
            // so near-ties do not flip from one set-up to the next
            const float med = t[3];
            const float ms = med * ((v == 0 && lpr == lpr0) ? 0.97f : 1.0f);
            // (slot 6: the faster node-block kernel)
            if (ms_out && lpr == lpr0 && (v <= 5 || v == 8)) ms_out[v == 8 ? 6 : v] = med;
            if (ms_out && lpr == lpr0 && v == 9 && (ms_out[6] <= 0.0 || med < ms_out[6])) ms_out[6] = med;
            // a later candidate must beat the incumbent by 2%: near-ties keep the
            // earlier (simpler) variant instead of following the timing noise
            if (ms < 0.98f * best || best >= 1e30f) {
                best = ms;
                best_v = v;
                best_lpr = lpr;
            }
        }
    }
    A.variant = best_v;
    A.lpr = best_lpr;
    c->n_launch = l0;
}

void autotune_system(mpet_ctx* c) {
    MPET_CUDA(cudaMemsetAsync(c->kv, 0, sizeof(double) * c->N, c->stream));
    if (c->prm.precision == MPET_PRECISION_MIXED && !c->A.v32) {
        // no FP32 CSR copy (HBM short): the node-block copy is the only FP32 matrix
        if (!(c->A.nb && c->A.nb->v32)) fail(MPET_ERR_NOMEM, "no room for an FP32 copy of the system matrix");
        c->A.variant = 8;
        return;
    }
    c->A.variant64 = -1;
    if (c->A.v32) {
        autotune_matrix<float, 1>(c, c->A, (const float*)c->kv, EpiStore<float, 1>{(float*)c->kd},
                                  c->spmv_variant_ms);
        if (c->A.v64) {
            // the FP64 refinement residual of the mixed path is tuned on its own, with its epilogue
            const int v32 = c->A.variant, l32 = c->A.lpr;
            MPET_CUDA(cudaMemsetAsync(c->kd, 0, sizeof(double) * c->N, c->stream));
            autotune_matrix<double, 1>(c, c->A, (const double*)c->kv, EpiResid64{c->orr, (const double*)c->kd,
                                                                                  c->dinv},
                                       c->spmv_variant_ms64);
            c->A.variant64 = c->A.variant;
            c->A.lpr64 = c->A.lpr;
            c->A.variant = v32;
            c->A.lpr = l32;
        }
    } else {
        autotune_matrix<double, 1>(c, c->A, (const double*)c->kv, EpiStore<double, 1>{(double*)c->kd},
                                   c->spmv_variant_ms);
    }
}

template <typename T, int NV>
static void autotune_hier(mpet_ctx* c, AmgHier& h) {
    for (size_t k = 0; k < h.lev.size(); ++k) {
        AmgLevel& L = h.lev[k];
        const size_t bytes = sizeof(double) * L.A.n * NV;
        for (void* p : {L.x, L.b, L.r, L.d, L.t0}) MPET_CUDA(cudaMemsetAsync(p, 0, bytes, c->stream));
        const T* dinv = dinv_of<T>(L);
        autotune_matrix<T, NV>(c, L.A, (const T*)L.x,
                               EpiCheb<T, NV>{(const T*)L.b, (const T*)L.x, (T*)L.d, (T*)L.t0, dinv, T(0.5), T(0.5)});
        if (k + 1 < h.lev.size()) {
            AmgLevel& C = h.lev[k + 1];
            MPET_CUDA(cudaMemsetAsync(C.x, 0, sizeof(double) * C.A.n * NV, c->stream));
            autotune_matrix<T, NV>(c, L.P, (const T*)C.x, EpiAxpby<T, NV>{(T*)L.t0, (const T*)L.t0, T(1), T(1)});
            autotune_matrix<T, NV>(c, L.R, (const T*)L.r, EpiStore<T, NV>{(T*)C.b});
        }
    }
}

template <typename T>
void spmv(mpet_ctx* c, const Csr& A, int nvec, const T* x, T* y) {
    if (nvec == 4) launch_spmv<T, 4>(c, A, vals<T>(A), x, EpiStore<T, 4>{y});
    else launch_spmv<T, 1>(c, A, vals<T>(A), x, EpiStore<T, 1>{y});
}
template void spmv<double>(mpet_ctx*, const Csr&, int, const double*, double*);
template void spmv<float>(mpet_ctx*, const Csr&, int, const float*, float*);

// ---- vector kernels ----------------------------------------------------------------

template <typename T>
__global__ void k_cheb_first(int64_t n, int nvec, const T* __restrict__ b, const T* __restrict__ dinv, T* d, T* x,
                             T inv_theta) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T v = dinv[i / nvec] * b[i] * inv_theta;
    d[i] = v;
    x[i] = v;
}

template <typename T>
__global__ void k_dense_coarse(int64_t n, int nvec, const double* __restrict__ cinv, const T* __restrict__ b, T* x) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (warp >= n * nvec) return;
    const int64_t row = warp / nvec;
    const int k = (int)(warp % nvec);
    double s = 0.0;
    for (int64_t j = lane; j < n; j += 32) s += cinv[row * n + j] * (double)b[nvec * j + k];
    s = warp_sum(s);
    if (lane == 0) x[nvec * row + k] = (T)s;
}

template <typename T>
__global__ void k_dot(int64_t n, const T* __restrict__ a, const T* __restrict__ b, double* partials) {
    __shared__ double sh[8];
    // a thread's products are summed in the working precision (a few dozen
    // terms), then the thread sums in FP64: no per-element FP64 work
    T acc = T(0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += a[i] * b[i];
    const double s = block_sum256((double)acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

template <typename T>
__global__ void k_copy2(int64_t n, const T* __restrict__ a, T* b, T* c) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T v = a[i];
    b[i] = v;
    c[i] = v;
}

template <typename T>
__global__ void k_mr_v(int64_t n, const T* __restrict__ y, T* v, const MinresScalars* sc) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    v[i] = y[i] * msc<T>(sc->inv_beta, sc->f_inv_beta);
}

template <typename T>
__global__ void k_mr_axpy(int64_t n, T* y, const T* __restrict__ r2, const MinresScalars* sc) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    y[i] -= msc<T>(sc->c_r2, sc->f_c_r2) * r2[i];
}

// w = (v - oldeps w1 - delta w2) / gamma ; d += phi w  (w1, w2 already rotated)
template <typename T>
__global__ void k_mr_update(int64_t n, const T* __restrict__ v, const T* __restrict__ w1, const T* __restrict__ w2,
                            T* w, T* d, const MinresScalars* sc) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T oe = msc<T>(sc->oldeps, sc->f_oldeps), de = msc<T>(sc->delta, sc->f_delta);
    const T ig = msc<T>(sc->inv_gamma, sc->f_inv_gamma), ph = msc<T>(sc->phi, sc->f_phi);
    const T wn = (v[i] - oe * w1[i] - de * w2[i]) * ig;
    w[i] = wn;
    d[i] += ph * wn;
}

// the FP32 copies of the scalars (after every update of the FP64 ones)
__device__ __forceinline__ void mr_mirror(MinresScalars* s) {
    s->f_inv_beta = (float)s->inv_beta;
    s->f_c_r1 = (float)s->c_r1;
    s->f_c_r2 = (float)s->c_r2;
    s->f_oldeps = (float)s->oldeps;
    s->f_delta = (float)s->delta;
    s->f_inv_gamma = (float)s->inv_gamma;
    s->f_phi = (float)s->phi;
}

// One MINRES scalar step (Paige-Saunders recurrences) on the reduced sums.
__device__ void mr_init_one(MinresScalars* s, double t) {
    bool bad = !(t >= 0.0) || isnan(t);
    double b1 = bad ? 0.0 : sqrt(t);
    s->beta1 = b1;
    s->beta = b1;
    s->oldb = 0.0;
    s->dbar = 0.0;
    s->epsln = 0.0;
    s->phibar = b1;
    s->cs = -1.0;
    s->sn = 0.0;
    s->c_r1 = 0.0;
    s->c_r2 = 0.0;
    s->inv_beta = b1 > 0.0 ? 1.0 / b1 : 0.0;
    s->rel = 1.0;
    s->flag = bad ? 1.0 : 0.0;
    s->oldeps = s->delta = s->phi = s->inv_gamma = 0.0;
    mr_mirror(s);
}

__device__ void mr_alfa_one(MinresScalars* s, double t) {
    s->alfa = t;
    s->c_r2 = t * s->inv_beta;
    s->f_c_r2 = (float)s->c_r2;
}

__device__ void mr_beta_one(MinresScalars* s, double t) {
    if (!(t >= 0.0) || isnan(t)) {
        s->flag = 1.0;
        t = 0.0;
    }
    const double oldb = s->beta;
    const double beta = sqrt(t);
    const double oldeps = s->epsln;
    const double delta = s->cs * s->dbar + s->sn * s->alfa;
    const double gbar = s->sn * s->dbar - s->cs * s->alfa;
    const double epsln = s->sn * beta;
    const double dbar = -s->cs * beta;
    double gamma = hypot(gbar, beta);
    if (gamma < 1e-300) gamma = 1e-300;
    const double cs = gbar / gamma, sn = beta / gamma;
    const double phi = cs * s->phibar;
    const double phibar = sn * s->phibar;
    s->oldb = oldb;
    s->beta = beta;
    s->oldeps = oldeps;
    s->delta = delta;
    s->gbar = gbar;
    s->epsln = epsln;
    s->dbar = dbar;
    s->gamma = gamma;
    s->cs = cs;
    s->sn = sn;
    s->phi = phi;
    s->phibar = phibar;
    s->inv_gamma = 1.0 / gamma;
    s->inv_beta = beta > 0.0 ? 1.0 / beta : 0.0;
    s->c_r1 = oldb > 0.0 ? beta / oldb : 0.0;
    s->rel = s->beta1 > 0.0 ? phibar / s->beta1 : 0.0;
    if (beta == 0.0 && phibar > 0.0) s->flag = 1.0;
    mr_mirror(s);
}

__global__ void k_mr_init(MinresScalars* s, const double* partials) {
    __shared__ double sh[8];
    double t = sum_partials(partials, sh);
    if (threadIdx.x == 0) mr_init_one(s, t);
}
__global__ void k_mr_alfa(MinresScalars* s, const double* partials) {
    __shared__ double sh[8];
    double t = sum_partials(partials, sh);
    if (threadIdx.x == 0) mr_alfa_one(s, t);
}
__global__ void k_mr_beta(MinresScalars* s, const double* partials) {
    __shared__ double sh[8];
    double t = sum_partials(partials, sh);
    if (threadIdx.x == 0) mr_beta_one(s, t);
}



__global__ void k_outer_norms(MinresScalars* s, const double* partials) {
    __shared__ double sh[8];
    double a = sum_partials(partials, sh);
    double b = sum_partials(partials + NB_RED, sh);
    if (threadIdx.x == 0) {
        s->nr2 = a;
        s->nb2 = b;
        s->nr = a > 0.0 ? sqrt(a) : 0.0;
        s->inv_nr = s->nr > 0.0 ? 1.0 / s->nr : 0.0;
        s->inv_nb = b > 0.0 ? 1.0 / sqrt(b) : 0.0;
    }
}

// rhs_T = r / ||D^-1 r||  (scale read on the device)
template <typename T>
__global__ void k_scale_to(int64_t n, const double* __restrict__ r, T* out, const MinresScalars* s) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (T)(r[i] * s->inv_nr);
}

template <typename T>
__global__ void k_add_scaled(int64_t n, double* x, const T* __restrict__ d, const MinresScalars* s) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] += s->nr * (double)d[i];
}

__global__ void k_f64_to_f32(int64_t n, const double* __restrict__ a, float* b) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// ---- AMG V-cycle -------------------------------------------------------------------------

template <typename T, int NV>
static void cheb(mpet_ctx* c, AmgHier& h, AmgLevel& L, const T* b, const T* xin, T* xout) {
    const int nv = NV;
    const int64_t n = L.A.n * nv;
    const double hi = 1.1 * L.rho, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
    const double sigma = theta / delta;
    double rho_old = 1.0 / sigma;
    const int64_t lk = &L - &h.lev[0];
    const int s = lk == 0 ? h.cheb_degree0 : (lk >= h.cheb_level_c ? h.cheb_degree_c : h.cheb_degree);
    T* d = (T*)L.d;
    T* t0 = (T*)L.t0;
    T* t1 = (T*)L.t1;
    const T* dinv = dinv_of<T>(L);
    T* cur = (s == 1) ? xout : t0;
    if (!xin) {
        k_cheb_first<T><<<grid_for(n, 256), 256, 0, c->stream>>>(n, nv, b, dinv, d, cur, (T)(1.0 / theta));
        MPET_CHECK_LAUNCH();
        c->n_launch++;
    } else {
        const EpiCheb<T, NV> e{b, xin, d, cur, dinv, T(0), (T)(1.0 / theta)};
        level_spmv<T, NV>(c, L, xin, e);
    }
    for (int j = 1; j < s; ++j) {
        const double rho_new = 1.0 / (2.0 * sigma - rho_old);
        const T c1 = (T)(rho_new * rho_old), c2 = (T)(2.0 * rho_new / delta);
        T* nxt = (j == s - 1) ? xout : (cur == t0 ? t1 : t0);
        level_spmv<T, NV>(c, L, cur, EpiCheb<T, NV>{b, cur, d, nxt, dinv, c1, c2});
        cur = nxt;
        rho_old = rho_new;
    }
}

template <typename T, int NV>
static void vcycle(mpet_ctx* c, AmgHier& h, size_t k, const T* b, T* x) {
    if (k + 1 == h.lev.size()) {
        const int64_t rows = h.ncoarse * NV;
        k_dense_coarse<T><<<grid_for(rows * 32, 256), 256, 0, c->stream>>>(h.ncoarse, NV, h.cinv, b, x);
        MPET_CHECK_LAUNCH();
        c->n_launch++;
        return;
    }
    AmgLevel& L = h.lev[k];
    AmgLevel& C = h.lev[k + 1];
    T* xs = (T*)L.x;
    T* r = (T*)L.r;
    cheb<T, NV>(c, h, L, b, nullptr, xs);
    level_spmv<T, NV>(c, L, xs, EpiAxpby<T, NV>{r, b, T(-1), T(1)});
    launch_spmv<T, NV>(c, L.R, vals<T>(L.R), r, EpiStore<T, NV>{(T*)C.b});
    vcycle<T, NV>(c, h, k + 1, (const T*)C.b, (T*)C.x);
    launch_spmv<T, NV>(c, L.P, vals<T>(L.P), (const T*)C.x, EpiAxpby<T, NV>{xs, xs, T(1), T(1)});
    cheb<T, NV>(c, h, L, b, xs, x);
}

// Per-level profile of one hierarchy: ms[k] = median time of a V-cycle
// started at level k (so level k's own share is ms[k] - ms[k+1]), each of
// `reps` launches from a flushed L2 (in the solver every level is reached
// after the system SpMV has streamed gigabytes through L2); bytes[k] = the
// algorithmic bytes of level k's own work: every matrix entry (value + column
// id) and row pointer once per product, every vector once per read or write
// (2s products with A for Chebyshev degree s, the residual, R and P; the
// dense inverse on the coarsest level).
template <typename T, int NV>
static void profile_levels(mpet_ctx* c, AmgHier& h, int reps, double* ms, double* bytes) {
    constexpr size_t kFlush = 256u << 20;
    if (!c->l2_flush) c->l2_flush = c->pool.alloc<unsigned char>(kFlush);
    const int64_t l0 = c->n_launch;
    const size_t nl = h.lev.size();
    const double sv = sizeof(T);
    for (size_t k = 0; k < nl; ++k) {
        AmgLevel& L = h.lev[k];
        MPET_CUDA(cudaMemsetAsync(L.b, 0, sizeof(double) * L.A.n * NV, c->stream));
        std::vector<float> t;
        for (int q = 0; q <= reps; ++q) {
            MPET_CUDA(cudaMemsetAsync(c->l2_flush, q & 255, kFlush, c->stream));
            MPET_CUDA(cudaEventRecord(c->ev0, c->stream));
            vcycle<T, NV>(c, h, k, (const T*)L.b, (T*)L.x);
            MPET_CUDA(cudaEventRecord(c->ev1, c->stream));
            MPET_CUDA(cudaEventSynchronize(c->ev1));
            float e = 0.f;
            MPET_CUDA(cudaEventElapsedTime(&e, c->ev0, c->ev1));
            if (q > 0) t.push_back(e);
        }
        std::sort(t.begin(), t.end());
        ms[k] = t[t.size() / 2];
        const double n = (double)L.A.n, vec = n * NV * sv, dv = n * sv;
        if (k + 1 == nl) {
            bytes[k] = (double)h.ncoarse * h.ncoarse * 8.0 + 2.0 * h.ncoarse * NV * sv;
            continue;
        }
        const int s = k == 0 ? h.cheb_degree0 : ((int)k >= h.cheb_level_c ? h.cheb_degree_c : h.cheb_degree);
        const double nc = (double)h.lev[k + 1].A.n, vecc = nc * NV * sv;
        // a product with A: the CSR entries and row pointers, or (matrix-free) the
        // incidence and per-cell node ids (NN each), the per-cell data, the row
        // pointers of the incidence and the Dirichlet flags, once each
        const double nn_cell = c->dim == 3 ? 10.0 : 6.0;
        const double mA = L.mf ? (double)c->nc * (2.0 * nn_cell * 4.0 + 8.0 * sv) + n + (n + 1) * 8.0
                               : L.A.nnz * (sv + 4.0) + (n + 1) * 8.0;
        double b = 3 * vec + dv;                              // first Chebyshev step (no product)
        b += (2 * s - 1) * (mA + 5 * vec + dv);               // the other 2s - 1 smoothing products
        b += mA + 3 * vec;                                    // residual
        b += L.R.nnz * (sv + 4.0) + (nc + 1) * 8.0 + vec + vecc;  // restriction
        b += L.P.nnz * (sv + 4.0) + (n + 1) * 8.0 + vecc + 2 * vec;  // prolongation + correction
        bytes[k] = b;
    }
    c->n_launch = l0;
}

void profile_vcycle(mpet_ctx* c, int block, int reps, int* nlev, double* ms, double* bytes) {
    const bool f32 = c->prm.precision == MPET_PRECISION_MIXED;
    AmgHier& h = block == 0 ? c->amg_u : c->amg_p[block - 1];
    *nlev = (int)h.lev.size();
    if (block == 0 && !c->u_elast) {
        if (f32) profile_levels<float, 4>(c, h, reps, ms, bytes);
        else profile_levels<double, 4>(c, h, reps, ms, bytes);
    } else {
        if (f32) profile_levels<float, 1>(c, h, reps, ms, bytes);
        else profile_levels<double, 1>(c, h, reps, ms, bytes);
    }
}

// displacement components (3 per node) <-> the padded 4-wide layout of the
// displacement hierarchy
// (perm: row of each node in a spatially ordered first level, or null)
template <typename T>
__global__ void k_pack34(int64_t nodes, int dim, const T* __restrict__ a, T* b4, const int32_t* __restrict__ perm) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    const T v[4] = {a[dim * i], a[dim * i + 1], dim == 3 ? a[dim * i + 2] : T(0), T(0)};
    VecIO<T, 4>::store(b4, perm ? perm[i] : i, v);
}

template <typename T>
__global__ void k_unpack43(int64_t nodes, int dim, const T* __restrict__ b4, T* a, const int32_t* __restrict__ perm) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    T v[4];
    VecIO<T, 4>::load(b4, perm ? perm[i] : i, v);
    for (int k = 0; k < dim; ++k) a[dim * i + k] = v[k];
}

// rt_k = sum_a Q_ak r_a (fwd) or z_a = sum_k Q_ak zt_k (back) at every vertex,
// with the Q of the vertex's instance
template <typename T, bool FWD>
__global__ void k_modes(int64_t nv, int J, const int32_t* __restrict__ vinst, const double* __restrict__ Q,
                        const T* __restrict__ in, T* out) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const double* q = Q + (vinst ? (int64_t)vinst[v] : 0) * J * J;
    T a_in[MPET_MAX_NETWORKS];
    for (int a = 0; a < J; ++a) a_in[a] = in[(int64_t)a * nv + v];
    for (int k = 0; k < J; ++k) {
        T s = T(0);
        for (int a = 0; a < J; ++a) s += (T)(FWD ? q[a * J + k] : q[k * J + a]) * a_in[a];
        out[(int64_t)k * nv + v] = s;
    }
}

// Block-diagonal preconditioner z = M^-1 r.  The J pressure V-cycles (on the
// networks, or on the network eigenmodes between two vertex-wise
// transforms) are forked onto side streams and run concurrently with the
// displacement V-cycle on the main stream (inside a CUDA graph capture they
// become parallel branches); the main stream joins them at the end.
template <typename T>
static void precond(mpet_ctx* c, const T* r, T* z) {
    cudaStream_t main = c->stream;
    const T* rp = r + c->Nu;
    T* zp = z + c->Nu;
    if (c->net_modes) {
        k_modes<T, true><<<grid_for(c->nv, 256), 256, 0, main>>>(c->nv, c->J, c->vert_inst, c->mode_Q, rp,
                                                                 (T*)c->mode_r);
        MPET_CHECK_LAUNCH();
        c->n_launch++;
        rp = (const T*)c->mode_r;
        zp = (T*)c->mode_z;
    }
    MPET_CUDA(cudaEventRecord(c->ev_fork, main));
    for (int a = 0; a < c->J; ++a) {
        MPET_CUDA(cudaStreamWaitEvent(c->side[a], c->ev_fork, 0));
        c->stream = c->side[a];
        const int64_t off = (int64_t)a * c->nv;
        vcycle<T, 1>(c, c->amg_p[a], 0, rp + off, zp + off);
        MPET_CUDA(cudaEventRecord(c->ev_join[a], c->side[a]));
    }
    c->stream = main;
    AmgHier& hu = c->amg_u;
    if (c->u_elast) {
        // elasticity hierarchy on the interleaved displacement unknowns
        vcycle<T, 1>(c, hu, 0, r, z);
    } else {
        const int64_t nodes = c->nnodes;
        T* bin = (T*)hu.pack_in;
        T* xout = (T*)hu.pack_out;
        k_pack34<T><<<grid_for(nodes, 256), 256, 0, main>>>(nodes, c->dim, r, bin, hu.perm);
        vcycle<T, 4>(c, hu, 0, bin, xout);
        k_unpack43<T><<<grid_for(nodes, 256), 256, 0, main>>>(nodes, c->dim, xout, z, hu.perm);
        MPET_CHECK_LAUNCH();
        c->n_launch += 2;
    }
    for (int a = 0; a < c->J; ++a) MPET_CUDA(cudaStreamWaitEvent(main, c->ev_join[a], 0));
    if (c->net_modes) {
        k_modes<T, false><<<grid_for(c->nv, 256), 256, 0, main>>>(c->nv, c->J, c->vert_inst, c->mode_Q,
                                                                  (const T*)c->mode_z, z + c->Nu);
        MPET_CHECK_LAUNCH();
        c->n_launch++;
    }
}

// ---- MINRES ----------------------------------------------------------------------------

// Three MINRES iterations.  The Lanczos vectors rotate through kr[0..2]
// (r1, r2, y) and the direction vectors through kw[0..2] (w, w1, w2); both
// rotations have period 3, so three iterations start and end in the same
// buffer assignment and can be captured once and replayed as a CUDA graph.
template <typename T>
static void minres_three(mpet_ctx* c) {
    const int64_t n = c->N;
    const int G = grid_for(n, 256);
    T* v = (T*)c->kv;
    T* d = (T*)c->kd;
    int ir1 = 0, ir2 = 1, iy = 2;
    int iw = 0, iw1 = 1, iw2 = 2;
    for (int q = 0; q < 3; ++q) {
        T* r1 = (T*)c->kr[ir1];
        T* r2 = (T*)c->kr[ir2];
        T* y = (T*)c->kr[iy];
        k_mr_v<T><<<G, 256, 0, c->stream>>>(n, y, v, c->sc);
        launch_spmv<T, 1>(c, c->A, vals<T>(c->A), v, EpiMinres<T>{y, r1, v, c->sc});
        c->n_spmv++;
        k_mr_alfa<<<1, 256, 0, c->stream>>>(c->sc, c->partials);
        k_mr_axpy<T><<<G, 256, 0, c->stream>>>(n, y, r2, c->sc);
        MPET_CHECK_LAUNCH();
        c->n_launch += 3;
        const int old1 = ir1;
        ir1 = ir2;
        ir2 = iy;
        iy = old1;
        precond<T>(c, (const T*)c->kr[ir2], (T*)c->kr[iy]);
        k_dot<T><<<NB_RED, 256, 0, c->stream>>>(n, (const T*)c->kr[ir2], (const T*)c->kr[iy], c->partials);
        k_mr_beta<<<1, 256, 0, c->stream>>>(c->sc, c->partials);
        const int oldw1 = iw1;
        iw1 = iw2;
        iw2 = iw;
        iw = oldw1;
        k_mr_update<T><<<G, 256, 0, c->stream>>>(n, v, (const T*)c->kw[iw1], (const T*)c->kw[iw2],
                                                 (T*)c->kw[iw], d, c->sc);
        MPET_CHECK_LAUNCH();
        c->n_launch += 3;
    }
}

// Captures body(c) (issued on c->stream) into an executable graph.
template <class F>
static void capture_graph(mpet_ctx* c, F body, cudaGraphExec_t* out, int64_t* launches, const char* what) {
    if (!c->cap_stream) MPET_CUDA(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    cudaStream_t saved = c->stream;
    const int64_t l0 = c->n_launch, s0 = c->n_spmv;
    c->stream = c->cap_stream;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        try {
            body(c);
        } catch (...) {
            cudaStreamEndCapture(c->cap_stream, &g);
            if (g) cudaGraphDestroy(g);
            c->stream = saved;
            throw;
        }
        e = cudaStreamEndCapture(c->cap_stream, &g);
    }
    c->stream = saved;
    *launches = c->n_launch - l0;
    c->n_launch = l0;
    c->n_spmv = s0;
    if (e != cudaSuccess) fail(MPET_ERR_CUDA, std::string(what) + " graph capture: " + cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *out = nullptr;
        fail(MPET_ERR_CUDA, std::string(what) + " graph instantiate: " + cudaGetErrorString(e));
    }
}

// Whole inner solves as one graph launch: a WHILE conditional node whose body
// is three MINRES iterations followed by a one-thread kernel that counts the
// iterations and keeps the loop going while no breakdown is flagged, the
// target is not reached and the iteration budget lasts (the test the host
// made after every three iterations before).  Target and budget live in
// device memory (LoopCtl), written before each launch.
struct LoopCtl {
    double target;
    int max_iters;
    int iters;
};

__global__ void k_mr_continue(cudaGraphConditionalHandle h, const MinresScalars* sc, LoopCtl* ctl) {
    const int it = ctl->iters + 3;
    ctl->iters = it;
    const bool go = sc->flag == 0.0 && !(sc->rel <= ctl->target) && it < ctl->max_iters;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// batches: continue while some instance is not done (done covers breakdowns)
__global__ void k_bmr_continue(cudaGraphConditionalHandle h, int ni, const double* done, LoopCtl* ctl) {
    __shared__ int open;
    if (threadIdx.x == 0) open = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < ni; i += blockDim.x)
        if (done[i] == 0.0) open = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        const int it = ctl->iters + 3;
        ctl->iters = it;
        cudaGraphSetConditional(h, (open && it < ctl->max_iters) ? 1u : 0u);
    }
}

// Builds a graph of one WHILE node (default 1, reset every launch) whose body is
// captured from body(c, handle) on the capture stream, and instantiates it.
template <class F>
static void build_while_graph(mpet_ctx* c, F body, cudaGraphExec_t* out, int64_t* launches, const char* what) {
    if (!c->cap_stream) MPET_CUDA(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    MPET_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t node;
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        fail(MPET_ERR_CUDA, std::string(what) + " conditional node: " + cudaGetErrorString(e));
    }
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    cudaStream_t saved = c->stream;
    const int64_t l0 = c->n_launch, s0 = c->n_spmv;
    c->stream = c->cap_stream;
    e = cudaStreamBeginCaptureToGraph(c->cap_stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        try {
            body(c, h);
        } catch (...) {
            cudaGraph_t tmp = nullptr;
            cudaStreamEndCapture(c->cap_stream, &tmp);
            c->stream = saved;
            cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t tmp = nullptr;
        e = cudaStreamEndCapture(c->cap_stream, &tmp);
    }
    c->stream = saved;
    *launches = c->n_launch - l0;
    c->n_launch = l0;
    c->n_spmv = s0;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *out = nullptr;
        fail(MPET_ERR_CUDA, std::string(what) + " while-graph: " + cudaGetErrorString(e));
    }
}

template <typename T>
static void capture_minres_graph(mpet_ctx* c) {
    if (!c->loop_ctl) c->loop_ctl = c->pool.alloc<unsigned char>(sizeof(LoopCtl));
    build_while_graph(
        c,
        [](mpet_ctx* cc, cudaGraphConditionalHandle h) {
            minres_three<T>(cc);
            k_mr_continue<<<1, 1, 0, cc->stream>>>(h, cc->sc, (LoopCtl*)cc->loop_ctl);
            MPET_CHECK_LAUNCH();
            cc->n_launch++;
        },
        &c->mr_graph, &c->mr_graph_launches, "MINRES");
}

void destroy_minres_graph(mpet_ctx* c) {
    if (c->mr_graph) cudaGraphExecDestroy(c->mr_graph);
    c->mr_graph = nullptr;
    if (c->mr_graph3) cudaGraphExecDestroy(c->mr_graph3);
    c->mr_graph3 = nullptr;
    if (c->bmr_graph) cudaGraphExecDestroy(c->bmr_graph);
    c->bmr_graph = nullptr;
}

// Launches a whole-solve graph with the given target and budget; the loop
// control comes back to its pinned host copy (read after the caller's sync).
static void run_while_graph(mpet_ctx* c, cudaGraphExec_t g, double target, int max_iters) {
    LoopCtl* hc = (LoopCtl*)c->loop_ctl_host;
    hc->target = target;
    hc->max_iters = max_iters;
    hc->iters = 0;
    MPET_CUDA(cudaMemcpyAsync(c->loop_ctl, hc, sizeof(LoopCtl), cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaGraphLaunch(g, c->stream));
    MPET_CUDA(cudaMemcpyAsync(hc, c->loop_ctl, sizeof(LoopCtl), cudaMemcpyDeviceToHost, c->stream));
}

// The same three iterations replayed as a plain graph with a host check after
// each replay (inner_loop = 1, a test hook to compare with the device loop).
template <typename T>
static int minres_run_host(mpet_ctx* c, double target, int max_iters, int* iters_done) {
    if (!c->mr_graph3)
        capture_graph(c, [](mpet_ctx* cc) { minres_three<T>(cc); }, &c->mr_graph3, &c->mr_graph3_launches,
                      "MINRES");
    int it = 0;
    int status = MPET_OK;
    while (it < max_iters) {
        MPET_CUDA(cudaGraphLaunch(c->mr_graph3, c->stream));
        it += 3;
        c->n_launch += c->mr_graph3_launches;
        c->n_spmv += 3;
        MPET_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        if (c->sc_host->flag != 0.0) {
            status = MPET_ERR_BREAKDOWN;
            break;
        }
        if (c->sc_host->rel <= target) break;
    }
    *iters_done = it;
    return status;
}

template <typename T>
static int minres_run(mpet_ctx* c, double target, int max_iters, int* iters_done) {
    *iters_done = 0;
    if (max_iters <= 0) return MPET_OK;
    if (c->prm.inner_loop == 1) return minres_run_host<T>(c, target, max_iters, iters_done);
    if (!c->mr_graph) capture_minres_graph<T>(c);
    run_while_graph(c, c->mr_graph, target, max_iters);
    MPET_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    const int it = ((LoopCtl*)c->loop_ctl_host)->iters;
    c->n_launch += c->mr_graph_launches * (it / 3);
    c->n_spmv += it;
    *iters_done = it;
    return c->sc_host->flag != 0.0 ? MPET_ERR_BREAKDOWN : MPET_OK;
}

// ---- rigid-motion modes ---------------------------------------------------------------
__global__ void k_fill64(int64_t n, double* y, double v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = v;
}

__global__ void k_axpy64(int64_t n, double* y, double a, const double* __restrict__ x) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}

__global__ void k_finish_dot(const double* __restrict__ partials, double* out) {
    __shared__ double sh[8];
    const double s = sum_partials(partials, sh);
    if (threadIdx.x == 0) *out = s;
}

// a . b over n entries (fixed-order reduction), on the host
static double dot_host(mpet_ctx* c, const double* a, const double* b, int64_t n) {
    k_dot<double><<<NB_RED, 256, 0, c->stream>>>(n, a, b, c->partials);
    k_finish_dot<<<1, 256, 0, c->stream>>>(c->partials, c->partials + 2 * NB_RED - 1);
    MPET_CHECK_LAUNCH();
    double v = 0.0;
    MPET_CUDA(cudaMemcpyAsync(&v, c->partials + 2 * NB_RED - 1, sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    return v;
}

// v -= sum_j (n_j . v) n_j over the pressure kernel vectors of the constrained networks
static void kernel_project(mpet_ctx* c, double* v) {
    const int64_t n = c->N;
    for (int j = 0; j < c->q_nk; ++j) {
        const double* nj = c->q_N + (int64_t)j * n;
        const double t = dot_host(c, nj, v, n);
        k_axpy64<<<grid_for(n, 256), 256, 0, c->stream>>>(n, v, -t, nj);
    }
    MPET_CHECK_LAUNCH();
}

// v_u -= sum_i (P_i . v_u) Q_i over the displacement rows (P, Q: the modes or their duals)
static void rigid_project(mpet_ctx* c, double* v, const double* P, const double* Q, double* coef_out) {
    const int64_t nu = c->Nu;
    for (int i = 0; i < c->nrigid; ++i) {
        const double t = dot_host(c, P + (int64_t)i * nu, v, nu);
        if (coef_out) coef_out[i] = t;
        k_axpy64<<<grid_for(nu, 256), 256, 0, c->stream>>>(nu, v, -t, Q + (int64_t)i * nu);
        MPET_CHECK_LAUNCH();
    }
}

// rhs_T = b / ||D^-1 b|| (the scale read on the device)
template <typename T>
__global__ void k_scale_b(int64_t n, const double* __restrict__ b, T* out, const MinresScalars* s) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (T)(b[i] * s->inv_nb);
}

// Preconditioned norm (b^T M^-1 b)^1/2 of the right-hand side, in the working
// precision, after the first refinement residual (which left ||D^-1 b||^2 in the
// scalars).  The refinement stops when the preconditioned residual is rtol times
// the initial one; after a very good warm start that can lie below what FP64
// residuals resolve, so it also stops when a sweep no longer halves the residual
// and the residual is already below rtol times this norm (PETSc's default test,
// the reference's iterative solves mpetsolver.py:507-556, measures against the
// right-hand side).  rhs and y are scratch vectors (default kr[0], kr[2]).
template <typename T>
static double precond_norm_b(mpet_ctx* c, const double* b, T* rhs = nullptr, T* y = nullptr) {
    const int64_t n = c->N;
    if (!rhs) rhs = (T*)c->kr[0];
    if (!y) y = (T*)c->kr[2];
    k_scale_b<T><<<grid_for(n, 256), 256, 0, c->stream>>>(n, b, rhs, c->sc);
    MPET_CHECK_LAUNCH();
    precond<T>(c, rhs, y);
    k_dot<T><<<NB_RED, 256, 0, c->stream>>>(n, rhs, y, c->partials);
    k_finish_dot<<<1, 256, 0, c->stream>>>(c->partials, c->partials + 2 * NB_RED - 1);
    MPET_CHECK_LAUNCH();
    double q = 0.0;
    MPET_CUDA(cudaMemcpyAsync(&q, c->partials + 2 * NB_RED - 1, sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    return sqrt(q > 0.0 ? q : 0.0) * sqrt(c->sc_host->nb2 > 0.0 ? c->sc_host->nb2 : 0.0);
}

template <typename T>
static int solve_impl(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous) {
    const int64_t n = c->N;
    const int G = grid_for(n, 256);
    if (homogeneous) launch_zero_bc_rows(c, x);
    else launch_set_bc_in_x(c, x);
    if (c->nrigid > 0 || c->q_nk > 0) {
        // multipliers r_i = Z_i . b_u; solve with b - sum_i r_i M Z_i (consistent), and without
        // the components along the pressure kernel vectors
        MPET_CUDA(cudaMemcpyAsync(c->rigid_b, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
        if (c->nrigid > 0) rigid_project(c, c->rigid_b, c->rigid_Z, c->rigid_MZ, c->rigid_r);
        if (c->q_nk > 0) kernel_project(c, c->rigid_b);
        b = c->rigid_b;
    }
    double eta0 = -1.0;
    int iters = 0, outer = 0;
    int status = MPET_OK;
    double relres = 1.0, relres_true = 0.0;
    const bool fp64 = sizeof(T) == 8;
    const int max_outer = c->prm.max_outer > 0 ? c->prm.max_outer : 20;
    const int maxit = c->prm.maxit > 0 ? c->prm.maxit : 5000;
    double eta_b = 0.0, eta_prev = 0.0;
    for (outer = 0; outer < max_outer; ++outer) {
        launch_spmv<double, 1>(c, c->A, c->A.v64, x, EpiResid64{c->orr, b, c->dinv});
        c->n_spmv++;
        k_outer_norms<<<1, 256, 0, c->stream>>>(c->sc, c->partials);
        if (c->nrigid > 0) rigid_project(c, c->orr, c->rigid_Z, c->rigid_MZ, nullptr);  // rounding drift
        if (c->q_nk > 0) kernel_project(c, c->orr);
        T* rhs = (T*)c->kr[0];
        k_scale_to<T><<<G, 256, 0, c->stream>>>(n, c->orr, rhs, c->sc);
        k_copy2<T><<<G, 256, 0, c->stream>>>(n, rhs, (T*)c->kr[1], (T*)c->kr[1]);
        MPET_CHECK_LAUNCH();
        // y = M^-1 r1 into kr[2]
        precond<T>(c, (const T*)c->kr[0], (T*)c->kr[2]);
        k_dot<T><<<NB_RED, 256, 0, c->stream>>>(n, (const T*)c->kr[0], (const T*)c->kr[2], c->partials);
        k_mr_init<<<1, 256, 0, c->stream>>>(c->sc, c->partials);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        const MinresScalars h = *c->sc_host;
        const double nr = sqrt(h.nr2 > 0 ? h.nr2 : 0.0);
        relres_true = h.nb2 > 0 ? sqrt(h.nr2 / h.nb2) : 0.0;
        if (h.flag != 0.0) {
            status = MPET_ERR_BREAKDOWN;
            break;
        }
        const double eta = h.beta1 * nr;
        if (eta0 < 0) eta0 = eta;
        relres = eta0 > 0 ? eta / eta0 : 0.0;
        if (eta == 0.0 || eta <= c->prm.rtol * eta0) break;
        if (outer > 0 && eta > 0.5 * eta_prev) {
            // a sweep that no longer halves the residual: the FP64 floor test, with the
            // right-hand side's norm computed once, when first needed (kw[0], kw[1] are
            // free until their reset below)
            if (eta_b == 0.0) eta_b = precond_norm_b<T>(c, b, (T*)c->kw[0], (T*)c->kw[1]);
            if (eta <= c->prm.rtol * eta_b) break;
        }
        eta_prev = eta;
        if (iters >= maxit) {
            status = MPET_ERR_MAXIT;
            break;
        }
        double target = c->prm.rtol * eta0 / eta;
        if (fp64) {
            if (target < 1e-15) target = 1e-15;
        } else {
            if (target < c->prm.inner_rtol) target = c->prm.inner_rtol;
        }
        MPET_CUDA(cudaMemsetAsync(c->kd, 0, sizeof(T) * n, c->stream));
        for (int q = 0; q < 3; ++q) MPET_CUDA(cudaMemsetAsync(c->kw[q], 0, sizeof(T) * n, c->stream));
        int done = 0;
        MPET_CUDA(cudaEventRecord(c->ev_in0, c->stream));
        int s2 = minres_run<T>(c, target, maxit - iters, &done);
        MPET_CUDA(cudaEventRecord(c->ev_in1, c->stream));
        MPET_CUDA(cudaEventSynchronize(c->ev_in1));
        float ims = 0.f;
        MPET_CUDA(cudaEventElapsedTime(&ims, c->ev_in0, c->ev_in1));
        c->t_inner_ms += ims;
        c->n_inner_its += done;
        iters += done;
        k_add_scaled<T><<<G, 256, 0, c->stream>>>(n, x, (const T*)c->kd, c->sc);
        MPET_CHECK_LAUNCH();
        if (s2 != MPET_OK) {
            status = s2;
            break;
        }
    }
    // (Z_i, u) = 0: remove the modes from the displacement (M-orthogonally), and the kernel
    // components (the constraints set them afterwards)
    if (c->nrigid > 0) rigid_project(c, x, c->rigid_MZ, c->rigid_Z, nullptr);
    if (c->q_nk > 0) kernel_project(c, x);
    if (outer >= max_outer && status == MPET_OK) status = MPET_ERR_MAXIT;
    int derr = 0;
    MPET_CUDA(cudaMemcpyAsync(&derr, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    if (derr) {
        MPET_CUDA(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
        status = MPET_ERR_TIMEOUT;
    }
    if (st) {
        st->iterations = iters;
        st->outer = outer + 1;
        st->status = status;
        st->relres = relres;
        st->relres_true = relres_true;
    }
    return status;
}

void apply_preconditioner(mpet_ctx* c, int precision, const void* r, void* z) {
    if (precision == MPET_PRECISION_MIXED) precond<float>(c, (const float*)r, (float*)z);
    else precond<double>(c, (const double*)r, (double*)z);
}

void residual_norms(mpet_ctx* c, const double* b, const double* x, double* r, double* norms) {
    launch_spmv<double, 1>(c, c->A, c->A.v64, x, EpiResid64{r, b, c->dinv});
    k_outer_norms<<<1, 256, 0, c->stream>>>(c->sc, c->partials);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, c->stream));
    int derr = 0;
    MPET_CUDA(cudaMemcpyAsync(&derr, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    if (derr) {
        MPET_CUDA(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
        fail(MPET_ERR_TIMEOUT, "a staged SpMV copy did not complete within its wait limit");
    }
    norms[0] = sqrt(c->sc_host->nr2);
    norms[1] = sqrt(c->sc_host->nb2);
}

// ---- batches of independent instances -----------------------------------------------
//
// A batch is one mesh made of disjoint instance meshes, so the system and the
// AMG hierarchies are block diagonal and every kernel above runs all
// instances at once.  The Krylov scalars and the refinement loop are per
// instance: the DOFs are cut into chunks of at most BATCH_CHUNK rows of one
// instance; per-chunk partial sums (one block each) are added per instance
// in chunk order, so every per-instance dot and norm is deterministic.

template <typename T>
__global__ void k_seg_dot(const int64_t* __restrict__ lo, const int32_t* __restrict__ len, int64_t nch,
                          const T* __restrict__ a, const T* __restrict__ b, double* part) {
    __shared__ double sh[8];
    const int64_t ch = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < len[ch]; i += 256) {
        const int64_t r = lo[ch] + i;
        s += (double)a[r] * (double)b[r];
    }
    s = block_sum256(s, sh);
    if (threadIdx.x == 0) part[ch] = s;
}

// k_seg_dot for the batched iterations: a converged instance's chunks contribute 0
template <typename T>
__global__ void k_seg_dot_open(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                               const int32_t* __restrict__ inst, const T* __restrict__ a, const T* __restrict__ b,
                               double* part, const double* __restrict__ done) {
    __shared__ double sh[8];
    const int64_t ch = blockIdx.x;
    if (done[inst[ch]] != 0.0) {
        if (threadIdx.x == 0) part[ch] = 0.0;
        return;
    }
    T acc = T(0);  // a thread's 16 products in the working precision, then FP64
    for (int i = threadIdx.x; i < len[ch]; i += 256) {
        const int64_t r = lo[ch] + i;
        acc += a[r] * b[r];
    }
    const double s = block_sum256((double)acc, sh);
    if (threadIdx.x == 0) part[ch] = s;
}

// (r D^-1)^2 and (b D^-1)^2 per chunk
__global__ void k_seg_norms(const int64_t* __restrict__ lo, const int32_t* __restrict__ len, int64_t nch,
                            const double* __restrict__ r, const double* __restrict__ b,
                            const double* __restrict__ dinv, double* part) {
    __shared__ double sh[8];
    const int64_t ch = blockIdx.x;
    double s0 = 0.0, s1 = 0.0;
    for (int i = threadIdx.x; i < len[ch]; i += 256) {
        const int64_t q = lo[ch] + i;
        const double di = dinv[q];
        s0 += (r[q] * di) * (r[q] * di);
        s1 += (b[q] * di) * (b[q] * di);
    }
    s0 = block_sum256(s0, sh);
    s1 = block_sum256(s1, sh);
    if (threadIdx.x == 0) {
        part[ch] = s0;
        part[nch + ch] = s1;
    }
}

// out[v * ninst + i] = sum over instance i's chunks (in order) of part[v * nch + chunk]
__global__ void k_seg_finish(int ninst, const int32_t* __restrict__ cptr, const int32_t* __restrict__ chunks,
                             const double* __restrict__ part, int64_t nch, int nval, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    for (int v = 0; v < nval; ++v) {
        double s = 0.0;
        for (int k = cptr[i]; k < cptr[i + 1]; ++k) s += part[v * nch + chunks[k]];
        out[v * ninst + i] = s;
    }
}

template <typename T>
__global__ void k_seg_scale_from64(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                                   const int32_t* __restrict__ inst, const double* __restrict__ r,
                                   const double* __restrict__ scale, T* out) {
    const int64_t ch = blockIdx.x;
    const double s = scale[inst[ch]];
    for (int i = threadIdx.x; i < len[ch]; i += 256) out[lo[ch] + i] = (T)(r[lo[ch] + i] * s);
}

template <typename T>
__global__ void k_seg_scale(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                            const int32_t* __restrict__ inst, const double* __restrict__ scale, T* v, T* w) {
    const int64_t ch = blockIdx.x;
    const T s = (T)scale[inst[ch]];
    for (int i = threadIdx.x; i < len[ch]; i += 256) {
        v[lo[ch] + i] *= s;
        w[lo[ch] + i] *= s;
    }
}

template <typename T>
__global__ void k_seg_add(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                          const int32_t* __restrict__ inst, const double* __restrict__ scale, double* x,
                          const T* __restrict__ d) {
    const int64_t ch = blockIdx.x;
    const double s = scale[inst[ch]];
    for (int i = threadIdx.x; i < len[ch]; i += 256) x[lo[ch] + i] += s * (double)d[lo[ch] + i];
}

// Per-instance scalars (BatchVals rows of ninst doubles).
enum BatchVals { BV_NR2, BV_NB2, BV_Q, BV_RSCALE, BV_SIN, BV_SOUT, BV_ETA, BV_ETA0, BV_DONE, BV_QB, BV_ETAB,
                 BV_COUNT };

__global__ void k_batch_bscale(int ninst, double* iv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const double nb = sqrt(iv[BV_NB2 * ninst + i]);
    iv[BV_RSCALE * ninst + i] = nb > 0.0 ? 1.0 / nb : 0.0;
}

__global__ void k_batch_rscale(int ninst, double* iv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const double nr = sqrt(iv[BV_NR2 * ninst + i]);
    iv[BV_RSCALE * ninst + i] = nr > 0.0 ? 1.0 / nr : 0.0;
}

// eta_i = sqrt(r_i^T M^-1 r_i) from q_i = rhs_i^T M^-1 rhs_i with rhs_i = r_i / ||D^-1 r_i||
__global__ void k_batch_status(int ninst, double* iv, double rtol, int first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const double nr = sqrt(iv[BV_NR2 * ninst + i]);
    const double q = iv[BV_Q * ninst + i];
    const double beta = q > 0.0 ? sqrt(q) : 0.0;
    const double eta = beta * nr;
    if (first) {
        iv[BV_ETA0 * ninst + i] = eta;
        const double qb = iv[BV_QB * ninst + i];  // the right-hand side's preconditioned norm
        iv[BV_ETAB * ninst + i] = (qb > 0.0 ? sqrt(qb) : 0.0) * sqrt(iv[BV_NB2 * ninst + i]);
    }
    const double eta0 = iv[BV_ETA0 * ninst + i];
    // done at rtol of the initial residual, or (FP64 floor) when a sweep no longer
    // halves the residual and it is below rtol of the right-hand side's norm
    const bool floor = !first && eta > 0.5 * iv[BV_ETA * ninst + i] && eta <= rtol * iv[BV_ETAB * ninst + i];
    const bool done = !(eta > 0.0) || eta <= rtol * eta0 || floor;
    iv[BV_ETA * ninst + i] = eta;
    iv[BV_DONE * ninst + i] = done ? 1.0 : 0.0;
    iv[BV_SIN * ninst + i] = done ? 0.0 : 1.0 / beta;
    iv[BV_SOUT * ninst + i] = done ? 0.0 : nr;
}

// ---- batched MINRES: one Krylov recurrence per instance -------------------------------
//
// The vectors hold all instances; every scalar (alpha, beta, the Givens
// rotation) is per instance, and the dots are per-instance chunk sums.  An
// instance that reaches its target is frozen: its scalars are zeroed at the
// start of the next iteration, so its Lanczos vectors and its correction
// stop changing while the others continue.

template <typename T>
__global__ void k_bmr_v(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                        const int32_t* __restrict__ inst, const T* __restrict__ y, T* v,
                        const MinresScalars* __restrict__ sc, const double* __restrict__ done) {
    const int64_t ch = blockIdx.x;
    if (done[inst[ch]] != 0.0) return;  // a converged instance's chunks are left as they are
    const T ib = msc<T>(sc[inst[ch]].inv_beta, sc[inst[ch]].f_inv_beta);
    for (int i = threadIdx.x; i < len[ch]; i += 256) v[lo[ch] + i] = y[lo[ch] + i] * ib;
}

// y -= c_r1 r1 and the chunk sums of v . y
template <typename T>
__global__ void k_bmr_axpy_dot(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                               const int32_t* __restrict__ inst, T* y, const T* __restrict__ r1,
                               const T* __restrict__ v, const MinresScalars* __restrict__ sc, double* part,
                               const double* __restrict__ done) {
    __shared__ double sh[8];
    const int64_t ch = blockIdx.x;
    if (done[inst[ch]] != 0.0) {
        if (threadIdx.x == 0) part[ch] = 0.0;
        return;
    }
    const T c1 = msc<T>(sc[inst[ch]].c_r1, sc[inst[ch]].f_c_r1);
    T acc = T(0);  // a thread's 16 products in the working precision, then FP64
    for (int i = threadIdx.x; i < len[ch]; i += 256) {
        const int64_t r = lo[ch] + i;
        const T yy = y[r] - c1 * r1[r];
        y[r] = yy;
        acc += v[r] * yy;
    }
    const double s = block_sum256((double)acc, sh);
    if (threadIdx.x == 0) part[ch] = s;
}

template <typename T>
__global__ void k_bmr_axpy(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                           const int32_t* __restrict__ inst, T* y, const T* __restrict__ r2,
                           const MinresScalars* __restrict__ sc, const double* __restrict__ done) {
    const int64_t ch = blockIdx.x;
    if (done[inst[ch]] != 0.0) return;
    const T c2 = msc<T>(sc[inst[ch]].c_r2, sc[inst[ch]].f_c_r2);
    for (int i = threadIdx.x; i < len[ch]; i += 256) y[lo[ch] + i] -= c2 * r2[lo[ch] + i];
}

template <typename T>
__global__ void k_bmr_update(const int64_t* __restrict__ lo, const int32_t* __restrict__ len,
                             const int32_t* __restrict__ inst, const T* __restrict__ v, const T* __restrict__ w1,
                             const T* __restrict__ w2, T* w, T* d, const MinresScalars* __restrict__ sc,
                             const double* __restrict__ done) {
    const int64_t ch = blockIdx.x;
    if (done[inst[ch]] == 1.0) return;  // 2: converged by this iteration's beta, its update still counts
    const MinresScalars& s = sc[inst[ch]];
    const T oe = msc<T>(s.oldeps, s.f_oldeps), de = msc<T>(s.delta, s.f_delta);
    const T ig = msc<T>(s.inv_gamma, s.f_inv_gamma), ph = msc<T>(s.phi, s.f_phi);
    for (int i = threadIdx.x; i < len[ch]; i += 256) {
        const int64_t r = lo[ch] + i;
        const T wn = (v[r] - oe * w1[r] - de * w2[r]) * ig;
        w[r] = wn;
        d[r] += ph * wn;
    }
}

__device__ void mr_freeze(MinresScalars* s) {
    s->inv_beta = 0.0;
    s->c_r1 = 0.0;
    s->c_r2 = 0.0;
    s->phi = 0.0;
    s->inv_gamma = 0.0;
    s->oldeps = 0.0;
    s->delta = 0.0;
    s->alfa = 0.0;
    mr_mirror(s);
}

// start: q_i = rhs_i . M^-1 rhs_i; instances with active_i == 0 start frozen
__global__ void k_bmr_init(int ni, MinresScalars* sc, const double* q, const double* outer_done, double* done) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni) return;
    const bool on = outer_done[i] == 0.0;
    mr_init_one(&sc[i], on ? q[i] : 0.0);
    if (!on) {
        mr_freeze(&sc[i]);
        sc[i].rel = 0.0;
    }
    done[i] = on ? 0.0 : 1.0;
}

// done: 0 open, 2 converged in the previous iteration (its last update was still
// applied), 1 settled; settled instances' chunks are skipped by the vector kernels
__global__ void k_bmr_freeze(int ni, MinresScalars* sc, double* done) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ni && done[i] != 0.0) {
        mr_freeze(&sc[i]);
        done[i] = 1.0;
    }
}

__global__ void k_bmr_alfa(int ni, MinresScalars* sc, const double* t, const double* done) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ni && done[i] == 0.0) mr_alfa_one(&sc[i], t[i]);
}

__global__ void k_bmr_beta(int ni, MinresScalars* sc, const double* t, const double* target, double* done) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni || done[i] != 0.0) return;
    mr_beta_one(&sc[i], t[i]);
    if (sc[i].rel <= target[i] || sc[i].flag != 0.0) done[i] = 2.0;  // the update of this iteration still runs
}

template <typename T>
static void bminres_three(mpet_ctx* c) {
    const int ni = c->ninst;
    const int64_t nch = c->nchunks;
    const int gi = grid_for(ni, 128);
    T* v = (T*)c->kv;
    T* d = (T*)c->kd;
    int ir1 = 0, ir2 = 1, iy = 2;
    int iw = 0, iw1 = 1, iw2 = 2;
    // the products (system SpMV and preconditioner) skip the slices of
    // instances that have converged
    struct SkipScope {
        mpet_ctx* c;
        ~SkipScope() { c->skip_done = nullptr; }
    } scope{c};
    c->skip_done = (c->batch_skip && c->skip_maps) ? c->bdone : nullptr;
    for (int q = 0; q < 3; ++q) {
        T* r1 = (T*)c->kr[ir1];
        T* r2 = (T*)c->kr[ir2];
        T* y = (T*)c->kr[iy];
        k_bmr_freeze<<<gi, 128, 0, c->stream>>>(ni, c->bsc, c->bdone);
        k_bmr_v<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, y, v, c->bsc, c->bdone);
        MPET_CHECK_LAUNCH();
        launch_spmv<T, 1>(c, c->A, vals<T>(c->A), v, EpiStore<T, 1>{y});
        c->n_spmv++;
        k_bmr_axpy_dot<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, y, r1, v, c->bsc,
                                                                 c->ch_part, c->bdone);
        k_seg_finish<<<gi, 128, 0, c->stream>>>(ni, c->inst_cptr, c->inst_chunks, c->ch_part, nch, 1, c->bval);
        k_bmr_alfa<<<gi, 128, 0, c->stream>>>(ni, c->bsc, c->bval, c->bdone);
        k_bmr_axpy<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, y, r2, c->bsc,
                                                             c->bdone);
        MPET_CHECK_LAUNCH();
        c->n_launch += 6;
        const int old1 = ir1;
        ir1 = ir2;
        ir2 = iy;
        iy = old1;
        precond<T>(c, (const T*)c->kr[ir2], (T*)c->kr[iy]);
        k_seg_dot_open<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst,
                                                                (const T*)c->kr[ir2], (const T*)c->kr[iy],
                                                                c->ch_part, c->bdone);
        k_seg_finish<<<gi, 128, 0, c->stream>>>(ni, c->inst_cptr, c->inst_chunks, c->ch_part, nch, 1, c->bval);
        k_bmr_beta<<<gi, 128, 0, c->stream>>>(ni, c->bsc, c->bval, c->btarget, c->bdone);
        const int oldw1 = iw1;
        iw1 = iw2;
        iw2 = iw;
        iw = oldw1;
        k_bmr_update<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, v,
                                                              (const T*)c->kw[iw1], (const T*)c->kw[iw2],
                                                              (T*)c->kw[iw], d, c->bsc, c->bdone);
        MPET_CHECK_LAUNCH();
        c->n_launch += 4;
    }
}

// The batched inner solve as one graph launch (a WHILE node over three batched
// iterations) until every instance is done or the budget is spent.
template <typename T>
static int bminres_run(mpet_ctx* c, int max_iters, int* iters_done) {
    *iters_done = 0;
    if (max_iters <= 0) return MPET_OK;
    if (!c->loop_ctl) c->loop_ctl = c->pool.alloc<unsigned char>(sizeof(LoopCtl));
    if (!c->bmr_graph)
        build_while_graph(
            c,
            [](mpet_ctx* cc, cudaGraphConditionalHandle h) {
                bminres_three<T>(cc);
                k_bmr_continue<<<1, 256, 0, cc->stream>>>(h, cc->ninst, cc->bdone, (LoopCtl*)cc->loop_ctl);
                MPET_CHECK_LAUNCH();
                cc->n_launch++;
            },
            &c->bmr_graph, &c->bmr_graph_launches, "batched MINRES");
    const int ni = c->ninst;
    run_while_graph(c, c->bmr_graph, 0.0, max_iters);
    MPET_CUDA(cudaMemcpyAsync(c->bdone_host, c->bdone, sizeof(double) * ni, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->bsc_host, c->bsc, sizeof(MinresScalars) * ni, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    const int it = ((LoopCtl*)c->loop_ctl_host)->iters;
    c->n_launch += c->bmr_graph_launches * (it / 3);
    c->n_spmv += it;
    *iters_done = it;
    for (int i = 0; i < ni; ++i)
        if (c->bsc_host[i].flag != 0.0) return MPET_ERR_BREAKDOWN;
    return MPET_OK;
}

template <typename T>
static int solve_batch(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous) {
    const int64_t n = c->N;
    const int G = grid_for(n, 256);
    const int ni = c->ninst;
    const int64_t nch = c->nchunks;
    const int gi = grid_for(ni, 128);
    double* iv = c->inst_v;
    if (homogeneous) launch_zero_bc_rows(c, x);
    else launch_set_bc_in_x(c, x);
    int iters = 0, outer = 0;
    int status = MPET_OK;
    double relres = 1.0, relres_true = 0.0;
    const bool fp64 = sizeof(T) == 8;
    const int max_outer = c->prm.max_outer > 0 ? c->prm.max_outer : 20;
    const int maxit = c->prm.maxit > 0 ? c->prm.maxit : 5000;
    T* rhs = (T*)c->kr[0];
    T* y = (T*)c->kr[2];
    std::vector<double> target(ni);
    for (outer = 0; outer < max_outer; ++outer) {
        launch_spmv<double, 1>(c, c->A, c->A.v64, x, EpiResid64{c->orr, b, c->dinv});
        c->n_spmv++;
        k_seg_norms<<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, nch, c->orr, b, c->dinv, c->ch_part);
        k_seg_finish<<<gi, 128, 0, c->stream>>>(ni, c->inst_cptr, c->inst_chunks, c->ch_part, nch, 2,
                                                iv + BV_NR2 * ni);
        if (outer == 0) {
            // right-hand sides scaled by 1 / ||D^-1 b_i||, their preconditioned squared norms (BV_QB)
            k_batch_bscale<<<gi, 128, 0, c->stream>>>(ni, iv);
            k_seg_scale_from64<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, b,
                                                                        iv + BV_RSCALE * ni, rhs);
            precond<T>(c, rhs, y);
            k_seg_dot<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, nch, rhs, y, c->ch_part);
            k_seg_finish<<<gi, 128, 0, c->stream>>>(ni, c->inst_cptr, c->inst_chunks, c->ch_part, nch, 1,
                                                    iv + BV_QB * ni);
            MPET_CHECK_LAUNCH();
        }
        k_batch_rscale<<<gi, 128, 0, c->stream>>>(ni, iv);
        k_seg_scale_from64<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, c->orr,
                                                                    iv + BV_RSCALE * ni, rhs);
        MPET_CHECK_LAUNCH();
        precond<T>(c, rhs, y);
        k_seg_dot<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, nch, rhs, y, c->ch_part);
        k_seg_finish<<<gi, 128, 0, c->stream>>>(ni, c->inst_cptr, c->inst_chunks, c->ch_part, nch, 1,
                                                iv + BV_Q * ni);
        k_batch_status<<<gi, 128, 0, c->stream>>>(ni, iv, c->prm.rtol, outer == 0 ? 1 : 0);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaMemcpyAsync(c->inst_host, iv, sizeof(double) * BV_COUNT * ni, cudaMemcpyDeviceToHost,
                                  c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        const double* h = c->inst_host;
        int active = 0;
        double worst = 0.0, worst_true = 0.0;
        for (int i = 0; i < ni; ++i) {
            const double eta = h[BV_ETA * ni + i], eta0 = h[BV_ETA0 * ni + i];
            const double rr = eta0 > 0.0 ? eta / eta0 : 0.0;
            worst = rr > worst ? rr : worst;
            const double nb2 = h[BV_NB2 * ni + i];
            const double rt = nb2 > 0.0 ? sqrt(h[BV_NR2 * ni + i] / nb2) : 0.0;
            worst_true = rt > worst_true ? rt : worst_true;
            double want = 1.0;
            if (h[BV_DONE * ni + i] == 0.0) {
                ++active;
                want = c->prm.rtol * eta0 / eta;
            }
            target[i] = fp64 ? (want < 1e-15 ? 1e-15 : want) : (want < c->prm.inner_rtol ? c->prm.inner_rtol : want);
        }
        relres = worst;
        relres_true = worst_true;
        if (active == 0) break;
        if (iters >= maxit) {
            status = MPET_ERR_MAXIT;
            break;
        }
        MPET_CUDA(cudaMemcpyAsync(c->btarget, target.data(), sizeof(double) * ni, cudaMemcpyHostToDevice,
                                  c->stream));
        k_copy2<T><<<G, 256, 0, c->stream>>>(n, rhs, (T*)c->kr[1], (T*)c->kr[1]);
        k_bmr_init<<<gi, 128, 0, c->stream>>>(ni, c->bsc, iv + BV_Q * ni, iv + BV_DONE * ni, c->bdone);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaMemsetAsync(c->kd, 0, sizeof(T) * n, c->stream));
        for (int q = 0; q < 3; ++q) MPET_CUDA(cudaMemsetAsync(c->kw[q], 0, sizeof(T) * n, c->stream));
        int done = 0;
        MPET_CUDA(cudaEventRecord(c->ev_in0, c->stream));
        int s2 = bminres_run<T>(c, maxit - iters, &done);
        MPET_CUDA(cudaEventRecord(c->ev_in1, c->stream));
        MPET_CUDA(cudaEventSynchronize(c->ev_in1));
        float ims = 0.f;
        MPET_CUDA(cudaEventElapsedTime(&ims, c->ev_in0, c->ev_in1));
        c->t_inner_ms += ims;
        c->n_inner_its += done;
        iters += done;
        // x_i += ||D^-1 r_i|| d_i for the instances that iterated
        k_seg_add<T><<<(unsigned)nch, 256, 0, c->stream>>>(c->ch_lo, c->ch_len, c->ch_inst, iv + BV_SOUT * ni, x,
                                                           (const T*)c->kd);
        MPET_CHECK_LAUNCH();
        if (s2 != MPET_OK) {
            status = s2;
            break;
        }
    }
    if (outer >= max_outer && status == MPET_OK) status = MPET_ERR_MAXIT;
    int derr = 0;
    MPET_CUDA(cudaMemcpyAsync(&derr, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    if (derr) {
        MPET_CUDA(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
        status = MPET_ERR_TIMEOUT;
    }
    if (st) {
        st->iterations = iters;
        st->outer = outer + 1;
        st->status = status;
        st->relres = relres;
        st->relres_true = relres_true;
    }
    return status;
}

// Chunks of the DOF range per instance (vertex_inst: instance of every mesh
// vertex; an edge node belongs to the instance of its first vertex).
void setup_batch(mpet_ctx* c, int ninst, const int32_t* vertex_inst) {
    std::vector<int64_t> key(c->ne);
    if (c->ne) {
        MPET_CUDA(cudaMemcpyAsync(key.data(), c->edge_key, sizeof(int64_t) * c->ne, cudaMemcpyDeviceToHost,
                                  c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
    }
    std::vector<int32_t> node_inst(c->nnodes);
    for (int64_t v = 0; v < c->nv; ++v) {
        const int32_t i = vertex_inst[v];
        if (i < 0 || i >= ninst) fail(MPET_ERR_INVALID, "instance id out of range");
        node_inst[v] = i;
    }
    for (int64_t e = 0; e < c->ne; ++e) {
        const int32_t i0 = vertex_inst[key[e] / c->nv], i1 = vertex_inst[key[e] % c->nv];
        if (i0 != i1) fail(MPET_ERR_INVALID, "an edge joins two instances: instance meshes must be disjoint");
        node_inst[c->nv + e] = i0;
    }
    std::vector<int64_t> lo;
    std::vector<int32_t> len, inst;
    auto push = [&](int64_t row, int32_t i) {
        if (!lo.empty() && inst.back() == i && lo.back() + len.back() == row && len.back() < BATCH_CHUNK) {
            ++len.back();
            return;
        }
        lo.push_back(row);
        len.push_back(1);
        inst.push_back(i);
    };
    for (int64_t k = 0; k < c->nnodes; ++k)
        for (int d = 0; d < 3; ++d) push(3 * k + d, node_inst[k]);
    for (int a = 0; a < c->J; ++a)
        for (int64_t v = 0; v < c->nv; ++v) push(c->Nu + (int64_t)a * c->nv + v, node_inst[v]);
    const int64_t nch = (int64_t)lo.size();
    std::vector<int32_t> cptr(ninst + 1, 0), order(nch);
    for (int64_t k = 0; k < nch; ++k) cptr[inst[k] + 1]++;
    for (int i = 0; i < ninst; ++i) cptr[i + 1] += cptr[i];
    {
        std::vector<int32_t> fill(cptr.begin(), cptr.end() - 1);
        for (int64_t k = 0; k < nch; ++k) order[fill[inst[k]]++] = (int32_t)k;
    }
    c->ninst = ninst;
    c->nchunks = nch;
    c->ch_lo = c->pool.alloc<int64_t>(nch);
    c->ch_len = c->pool.alloc<int32_t>(nch);
    c->ch_inst = c->pool.alloc<int32_t>(nch);
    c->inst_cptr = c->pool.alloc<int32_t>(ninst + 1);
    c->inst_chunks = c->pool.alloc<int32_t>(nch);
    c->ch_part = c->pool.alloc<double>(2 * nch);
    c->inst_v = c->pool.alloc<double>((int64_t)BV_COUNT * ninst);
    MPET_CUDA(cudaMemcpyAsync(c->ch_lo, lo.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->ch_len, len.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->ch_inst, inst.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->inst_cptr, cptr.data(), sizeof(int32_t) * (ninst + 1), cudaMemcpyHostToDevice,
                              c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->inst_chunks, order.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice,
                              c->stream));
    MPET_CUDA(cudaMemsetAsync(c->inst_v, 0, sizeof(double) * BV_COUNT * ninst, c->stream));
    if (c->inst_host) MPET_CUDA(cudaFreeHost(c->inst_host));
    MPET_CUDA(cudaMallocHost(&c->inst_host, sizeof(double) * BV_COUNT * ninst));
    c->bsc = c->pool.alloc<MinresScalars>(ninst);
    c->bdone = c->pool.alloc<double>(ninst);
    c->btarget = c->pool.alloc<double>(ninst);
    c->bval = c->pool.alloc<double>(ninst);
    MPET_CUDA(cudaMallocHost(&c->bsc_host, sizeof(MinresScalars) * ninst));
    MPET_CUDA(cudaMallocHost(&c->bdone_host, sizeof(double) * ninst));
    c->node_inst = c->pool.alloc<int32_t>(c->nnodes);
    MPET_CUDA(cudaMemcpyAsync(c->node_inst, node_inst.data(), sizeof(int32_t) * c->nnodes, cudaMemcpyHostToDevice,
                              c->stream));
    c->skip_maps = false;
    destroy_minres_graph(c);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

// ---- skip maps of the batched products ------------------------------------------------

// per 32-row slice: lowest and highest instance of its rows (0, -1 without rows)
__global__ void k_skl_rows(int64_t n, int64_t nslices, const int32_t* __restrict__ ri, int ninst, int32_t* skl) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int lo = INT_MAX, hi = -1;
    for (int64_t r = s * 32; r < s * 32 + 32 && r < n; ++r) {
        const int i = ri[r];
        if (i < 0 || i >= ninst) continue;
        lo = i < lo ? i : lo;
        hi = i > hi ? i : hi;
    }
    skl[2 * s] = hi >= 0 ? lo : 0;
    skl[2 * s + 1] = hi;
}

// the system's DOF rows: displacement row r -> node r / dim, pressure row
// Nu + a nv + v -> vertex v (vertices are the first P2 nodes)
__global__ void k_skl_dofs(int64_t N, int64_t Nu, int64_t nv, int dim, int64_t nslices,
                           const int32_t* __restrict__ node_inst, int32_t* skl) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int lo = INT_MAX, hi = -1;
    for (int64_t r = s * 32; r < s * 32 + 32 && r < N; ++r) {
        const int i = r < Nu ? node_inst[r / dim] : node_inst[(r - Nu) % nv];
        lo = i < lo ? i : lo;
        hi = i > hi ? i : hi;
    }
    skl[2 * s] = hi >= 0 ? lo : 0;
    skl[2 * s + 1] = hi;
}

// node-block slices: the node (displacement slices) or vertex (pressure slices) of each lane
__global__ void k_skl_nb(int64_t ns, const int32_t* __restrict__ perm, const int32_t* __restrict__ node_inst,
                         int32_t* skl) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= ns) return;
    int lo = INT_MAX, hi = -1;
    for (int l = 0; l < 32; ++l) {
        const int32_t g = perm[s * 32 + l];
        if (g < 0) continue;
        const int i = node_inst[g];
        lo = i < lo ? i : lo;
        hi = i > hi ? i : hi;
    }
    skl[2 * s] = hi >= 0 ? lo : 0;
    skl[2 * s + 1] = hi;
}

// coarse rows take the instance of the fine rows that prolongate from them
// (all of one instance: instance meshes share no entry)
__global__ void k_coarse_inst(int64_t nf, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                              const int32_t* __restrict__ fi, int32_t* co) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nf) return;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e) atomicMin(co + ci[e], fi[i]);
}

__global__ void k_gather_i32(int64_t n, const int32_t* __restrict__ idx, const int32_t* __restrict__ a, int32_t* b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[idx[i]];
}

static int32_t* skl_of_rows(mpet_ctx* c, int64_t n, const int32_t* ri) {
    const int64_t ns = (n + 31) / 32;
    int32_t* skl = c->pool.alloc<int32_t>(2 * ns);
    k_skl_rows<<<grid_for(ns, 256), 256, 0, c->stream>>>(n, ns, ri, c->ninst, skl);
    MPET_CHECK_LAUNCH();
    return skl;
}

// Instances of every level of a hierarchy whose first level's rows are given
// (inst0: n0 instance ids), and the skip maps of each level's A, P and R.
static void hier_skip_maps(mpet_ctx* c, AmgHier& h, const int32_t* inst0, int64_t n0) {
    // (a kept hierarchy keeps its maps; a rebuilt one starts without)
    if (h.lev.empty() || h.lev[0].A.n != n0 || h.lev[0].nb_uu || h.lev[0].inst) return;
    for (size_t k = 0; k < h.lev.size(); ++k) {
        AmgLevel& L = h.lev[k];
        const int64_t n = L.A.n;
        L.inst = c->pool.alloc<int32_t>(n);
        if (k == 0 && h.iperm) {
            k_gather_i32<<<grid_for(n, 256), 256, 0, c->stream>>>(n, h.iperm, inst0, L.inst);
            MPET_CHECK_LAUNCH();
        } else if (k == 0) {
            MPET_CUDA(cudaMemcpyAsync(L.inst, inst0, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, c->stream));
        } else {
            const AmgLevel& F = h.lev[k - 1];
            if (F.P.n != F.A.n || F.P.m != n) fail(MPET_ERR_STATE, "prolongator shape does not match its levels");
            MPET_CUDA(cudaMemsetAsync(L.inst, 0x7f, sizeof(int32_t) * n, c->stream));
            k_coarse_inst<<<grid_for(F.A.n, 256), 256, 0, c->stream>>>(F.A.n, F.P.rp, F.P.ci, F.inst, L.inst);
            MPET_CHECK_LAUNCH();
        }
        L.A.skl = skl_of_rows(c, n, L.inst);
    }
    for (size_t k = 0; k + 1 < h.lev.size(); ++k) {
        AmgLevel& L = h.lev[k];
        L.P.skl = skl_of_rows(c, L.P.n, L.inst);
        L.R.skl = skl_of_rows(c, L.R.n, h.lev[k + 1].inst);
    }
}

void build_skip_maps(mpet_ctx* c) {
    if (c->ninst <= 0 || !c->node_inst) return;
    if (!c->A.skl) {
        const int64_t ns = (c->N + 31) / 32;
        c->A.skl = c->pool.alloc<int32_t>(2 * ns);
        k_skl_dofs<<<grid_for(ns, 256), 256, 0, c->stream>>>(c->N, c->Nu, c->nv, c->dim, ns, c->node_inst,
                                                              c->A.skl);
        MPET_CHECK_LAUNCH();
    }
    if (c->A.nb && !c->A.nb->skl) {
        NodeBlocks& nb = *c->A.nb;
        const int64_t ns = nb.nsu + nb.nsp;
        nb.skl = c->pool.alloc<int32_t>(2 * ns);
        k_skl_nb<<<grid_for(ns, 256), 256, 0, c->stream>>>(ns, nb.perm, c->node_inst, nb.skl);
        MPET_CHECK_LAUNCH();
    }
    if (!c->u_elast) hier_skip_maps(c, c->amg_u, c->node_inst, c->nnodes);
    for (int a = 0; a < c->J; ++a) hier_skip_maps(c, c->amg_p[a], c->node_inst, c->nv);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->skip_maps = true;
}

void batch_relres(mpet_ctx* c, double* out) {
    const int ni = c->ninst;
    const double* h = c->inst_host;
    for (int i = 0; i < ni; ++i) {
        const double eta0 = h[BV_ETA0 * ni + i];
        out[i] = eta0 > 0.0 ? h[BV_ETA * ni + i] / eta0 : 0.0;
    }
}

// ---- restarted GMRES (non-symmetric transfer matrix) ---------------------------------------
//
// Left-preconditioned GMRES(m) (Saad and Schultz, SIAM J. Sci. Stat. Comput. 7 (1986)
// 856-869) with the block-diagonal preconditioner M, inside the same FP64 refinement loop
// as MINRES: it minimises ||M^-1 (rhs - A d)||_2, a norm that weighs the displacement and
// pressure rows alike (the plain 2-norm is dominated by the displacement rows).  Arnoldi
// by classical Gram-Schmidt applied twice; the small Hessenberg system and its Givens
// rotations live on the host.  Every reduction has a fixed order.

// h[k] = V_k . w for k < m (V_k at V + k * ld); partials[k * NB_RED + block]
template <typename T>
__global__ void __launch_bounds__(256) k_mdot(int64_t n, int m, const T* __restrict__ V, int64_t ld,
                                             const T* __restrict__ w, double* partials) {
    __shared__ double sh[8];
    for (int k = 0; k < m; ++k) {
        double s = 0.0;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            s += (double)V[k * ld + i] * (double)w[i];
        s = block_sum256(s, sh);
        if (threadIdx.x == 0) partials[k * NB_RED + blockIdx.x] = s;
    }
}
__global__ void k_mdot_finish(const double* __restrict__ partials, double* out) {
    __shared__ double sh[8];
    const double v = sum_partials(partials + blockIdx.x * NB_RED, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = v;
}
// w += sum_k coef[k] V_k (coef on the device, k < m)
template <typename T>
__global__ void k_mupdate(int64_t n, int m, const T* __restrict__ V, int64_t ld, const double* __restrict__ coef,
                          double sign, T* w) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = 0; k < m; ++k) s += coef[k] * (double)V[k * ld + i];
    w[i] = (T)((double)w[i] + sign * s);
}
template <typename T>
__global__ void k_gm_scale(int64_t n, const T* __restrict__ a, double f, T* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (T)((double)a[i] * f);
}
template <typename T>
__global__ void k_gm_sub(int64_t n, const T* __restrict__ a, const T* __restrict__ b, T* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}

static void gm_alloc(mpet_ctx* c, int m) {
    if (c->gm_V && c->gm_m >= m) return;
    const int64_t n = c->N;
    c->gm_V = c->pool.alloc<double>((int64_t)(m + 1) * n);
    c->gm_z = c->pool.alloc<double>(n);
    c->gm_w = c->pool.alloc<double>(n);
    c->gm_r = c->pool.alloc<double>(n);
    c->gm_part = c->pool.alloc<double>((int64_t)(m + 1) * NB_RED);
    c->gm_h = c->pool.alloc<double>(m + 1);
    if (c->gm_h_host) cudaFreeHost(c->gm_h_host);
    MPET_CUDA(cudaMallocHost(&c->gm_h_host, sizeof(double) * (m + 1)));
    c->gm_m = m;
}

// V_0..V_{k-1} . w into gm_h (device) and gm_h_host
template <typename T>
static void gm_dots(mpet_ctx* c, const T* V, int k, const T* w) {
    const int64_t n = c->N;
    k_mdot<T><<<NB_RED, 256, 0, c->stream>>>(n, k, V, n, w, c->gm_part);
    k_mdot_finish<<<k, 256, 0, c->stream>>>(c->gm_part, c->gm_h);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaMemcpyAsync(c->gm_h_host, c->gm_h, sizeof(double) * k, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

// d = GMRES(M^-1 A, M^-1 rhs) from d = 0 until ||M^-1 (rhs - A d)||_2 <= target ||M^-1 rhs||_2
template <typename T>
static int gmres_run(mpet_ctx* c, const T* rhs, T* d, double target, int maxit, int* done) {
    const int64_t n = c->N;
    const int G = grid_for(n, 256);
    int m = c->prm.gmres_restart > 0 ? c->prm.gmres_restart : 30;
    if (m > 64) m = 64;
    gm_alloc(c, m);
    T* V = (T*)c->gm_V;
    T* z = (T*)c->gm_z;
    T* w = (T*)c->gm_w;
    T* r = (T*)c->gm_r;
    MPET_CUDA(cudaMemsetAsync(d, 0, sizeof(T) * n, c->stream));
    precond<T>(c, rhs, r);
    gm_dots<T>(c, r, 1, r);
    const double beta0 = sqrt(fmax(c->gm_h_host[0], 0.0));
    double beta = beta0;
    int total = 0;
    *done = 0;
    if (beta0 == 0.0) return MPET_OK;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    while (true) {
        k_gm_scale<T><<<G, 256, 0, c->stream>>>(n, r, 1.0 / beta, V);
        MPET_CHECK_LAUNCH();
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int kk = 0;
        bool conv = false;
        for (int j = 0; j < m && total < maxit; ++j) {
            T* vj = V + (int64_t)j * n;
            launch_spmv<T, 1>(c, c->A, vals<T>(c->A), vj, EpiStore<T, 1>{z});
            c->n_spmv++;
            precond<T>(c, z, w);
            double* h = &H[(size_t)j * (m + 1)];  // column j, rows 0..j+1
            for (int i = 0; i <= j + 1; ++i) h[i] = 0.0;
            for (int pass = 0; pass < 2; ++pass) {
                gm_dots<T>(c, V, j + 1, w);
                for (int i = 0; i <= j; ++i) h[i] += c->gm_h_host[i];
                k_mupdate<T><<<G, 256, 0, c->stream>>>(n, j + 1, V, n, c->gm_h, -1.0, w);
                MPET_CHECK_LAUNCH();
            }
            gm_dots<T>(c, w, 1, w);
            const double hn = sqrt(fmax(c->gm_h_host[0], 0.0));
            h[j + 1] = hn;
            if (hn > 0.0) {
                k_gm_scale<T><<<G, 256, 0, c->stream>>>(n, w, 1.0 / hn, V + (int64_t)(j + 1) * n);
                MPET_CHECK_LAUNCH();
            }
            for (int i = 0; i < j; ++i) {  // earlier rotations
                const double a = h[i], b = h[i + 1];
                h[i] = cs[i] * a + sn[i] * b;
                h[i + 1] = -sn[i] * a + cs[i] * b;
            }
            const double den = hypot(h[j], h[j + 1]);
            cs[j] = den > 0.0 ? h[j] / den : 1.0;
            sn[j] = den > 0.0 ? h[j + 1] / den : 0.0;
            h[j] = den;
            h[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++total;
            kk = j + 1;
            if (fabs(g[j + 1]) <= target * beta0 || hn == 0.0) {
                conv = true;
                break;
            }
        }
        // y = R^-1 g, d += V y
        for (int i = kk - 1; i >= 0; --i) {
            double t = g[i];
            for (int q = i + 1; q < kk; ++q) t -= H[(size_t)q * (m + 1) + i] * y[q];
            const double rii = H[(size_t)i * (m + 1) + i];
            if (!(fabs(rii) > 0.0)) {
                *done = total;
                return MPET_ERR_BREAKDOWN;
            }
            y[i] = t / rii;
        }
        MPET_CUDA(cudaMemcpyAsync(c->gm_h, y.data(), sizeof(double) * kk, cudaMemcpyHostToDevice, c->stream));
        k_mupdate<T><<<G, 256, 0, c->stream>>>(n, kk, V, n, c->gm_h, 1.0, d);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaStreamSynchronize(c->stream));  // y is read from pageable host memory
        if (conv || total >= maxit) {
            *done = total;
            return conv ? MPET_OK : MPET_ERR_MAXIT;
        }
        // restart from r = M^-1 (rhs - A d)
        launch_spmv<T, 1>(c, c->A, vals<T>(c->A), d, EpiStore<T, 1>{w});
        c->n_spmv++;
        k_gm_sub<T><<<G, 256, 0, c->stream>>>(n, rhs, w, z);
        MPET_CHECK_LAUNCH();
        precond<T>(c, z, r);
        gm_dots<T>(c, r, 1, r);
        beta = sqrt(fmax(c->gm_h_host[0], 0.0));
        if (beta <= target * beta0) {
            *done = total;
            return MPET_OK;
        }
    }
}

// FP64 refinement around GMRES in precision T (the MINRES loop of solve_impl, with the
// same preconditioned residual norm as the convergence measure)
template <typename T>
static int solve_gmres(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous) {
    const int64_t n = c->N;
    const int G = grid_for(n, 256);
    {
        int m = c->prm.gmres_restart > 0 ? c->prm.gmres_restart : 30;
        gm_alloc(c, m > 64 ? 64 : m);  // the reduction buffers are used before the first cycle
    }
    if (homogeneous) launch_zero_bc_rows(c, x);
    else launch_set_bc_in_x(c, x);
    double eta0 = -1.0, relres = 1.0, relres_true = 0.0;
    int iters = 0, outer = 0, status = MPET_OK;
    const bool fp64 = sizeof(T) == 8;
    const int max_outer = c->prm.max_outer > 0 ? c->prm.max_outer : 20;
    const int maxit = c->prm.maxit > 0 ? c->prm.maxit : 5000;
    double eta_b = 0.0, eta_prev = 0.0;
    for (outer = 0; outer < max_outer; ++outer) {
        launch_spmv<double, 1>(c, c->A, c->A.v64, x, EpiResid64{c->orr, b, c->dinv});
        c->n_spmv++;
        k_outer_norms<<<1, 256, 0, c->stream>>>(c->sc, c->partials);
        MPET_CHECK_LAUNCH();
        if (outer == 0) eta_b = precond_norm_b<T>(c, b);
        MPET_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        const MinresScalars h = *c->sc_host;
        const double nr = sqrt(h.nr2 > 0 ? h.nr2 : 0.0);
        relres_true = h.nb2 > 0 ? sqrt(h.nr2 / h.nb2) : 0.0;
        // preconditioned norm (r^T M^-1 r)^1/2 of the residual, as MINRES measures it
        T* rhs = (T*)c->kr[0];
        k_scale_to<T><<<G, 256, 0, c->stream>>>(n, c->orr, rhs, c->sc);
        MPET_CHECK_LAUNCH();
        precond<T>(c, rhs, (T*)c->kr[2]);
        gm_dots<T>(c, rhs, 1, (const T*)c->kr[2]);
        const double eta = nr * sqrt(fmax(c->gm_h_host[0], 0.0));
        if (eta0 < 0) eta0 = eta;
        relres = eta0 > 0 ? eta / eta0 : 0.0;
        if (!(eta == eta)) {
            status = MPET_ERR_BREAKDOWN;
            break;
        }
        if (eta == 0.0 || eta <= c->prm.rtol * eta0) break;
        if (outer > 0 && eta > 0.5 * eta_prev && eta <= c->prm.rtol * eta_b) break;  // FP64 floor
        eta_prev = eta;
        if (iters >= maxit) {
            status = MPET_ERR_MAXIT;
            break;
        }
        double target = c->prm.rtol * eta0 / eta;
        if (fp64) {
            if (target < 1e-15) target = 1e-15;
        } else if (target < c->prm.inner_rtol) {
            target = c->prm.inner_rtol;
        }
        int done = 0;
        MPET_CUDA(cudaEventRecord(c->ev_in0, c->stream));
        const int s2 = gmres_run<T>(c, rhs, (T*)c->kd, target, maxit - iters, &done);
        MPET_CUDA(cudaEventRecord(c->ev_in1, c->stream));
        MPET_CUDA(cudaEventSynchronize(c->ev_in1));
        float ims = 0.f;
        MPET_CUDA(cudaEventElapsedTime(&ims, c->ev_in0, c->ev_in1));
        c->t_inner_ms += ims;
        c->n_inner_its += done;
        iters += done;
        k_add_scaled<T><<<G, 256, 0, c->stream>>>(n, x, (const T*)c->kd, c->sc);
        MPET_CHECK_LAUNCH();
        if (s2 == MPET_ERR_BREAKDOWN) {
            status = s2;
            break;
        }
    }
    if (outer >= max_outer && status == MPET_OK) status = MPET_ERR_MAXIT;
    int derr = 0;
    MPET_CUDA(cudaMemcpyAsync(&derr, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    if (derr) {
        MPET_CUDA(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
        status = MPET_ERR_TIMEOUT;
    }
    if (st) {
        st->iterations = iters;
        st->outer = outer + 1;
        st->status = status;
        st->relres = relres;
        st->relres_true = relres_true;
    }
    return status;
}

// ---- constant-pressure constraints ---------------------------------------------------------
//
// The reference borders the system with one R-space unknown per network whose pressure is
// only determined up to a constant (mpetsolver.py:120-124, 209-215):
//   A x + B^T lambda = b,  B x = 0,  B_k = (int phi_v) on the DOFs of network k.
// Solved by the capacitance (Schur complement) method: W = A^-1 B^T (nq solves, redone
// after each assembly), x0 = A^-1 b, lambda = (B W)^-1 B x0, x = x0 - W lambda.

static int solve_plain(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous) {
    const bool mixed = c->prm.precision == MPET_PRECISION_MIXED;
    if (c->gmres)
        return mixed ? solve_gmres<float>(c, b, x, st, homogeneous) : solve_gmres<double>(c, b, x, st, homogeneous);
    if (c->ninst > 0)
        return mixed ? solve_batch<float>(c, b, x, st, homogeneous) : solve_batch<double>(c, b, x, st, homogeneous);
    return mixed ? solve_impl<float>(c, b, x, st, homogeneous) : solve_impl<double>(c, b, x, st, homogeneous);
}

// B_k . x (the load vector against network k's pressures)
static double q_dot(mpet_ctx* c, int k, const double* x) {
    return dot_host(c, c->q_load, x + c->Nu + (int64_t)c->q_net[k] * c->nv, c->nv);
}

// Gauss-Jordan inverse of a small dense matrix (row-major m x m); false when singular
static bool small_inverse(std::vector<double> S, int m, double* inv) {
    std::vector<double> I((size_t)m * m, 0.0);
    for (int k = 0; k < m; ++k) I[k * m + k] = 1.0;
    for (int col = 0; col < m; ++col) {
        int piv = col;
        for (int r = col + 1; r < m; ++r)
            if (fabs(S[r * m + col]) > fabs(S[piv * m + col])) piv = r;
        if (!(fabs(S[piv * m + col]) > 0.0)) return false;
        for (int q = 0; q < m; ++q) {
            std::swap(S[col * m + q], S[piv * m + q]);
            std::swap(I[col * m + q], I[piv * m + q]);
        }
        const double d = S[col * m + col];
        for (int q = 0; q < m; ++q) {
            S[col * m + q] /= d;
            I[col * m + q] /= d;
        }
        for (int r = 0; r < m; ++r)
            if (r != col) {
                const double f = S[r * m + col];
                for (int q = 0; q < m; ++q) {
                    S[r * m + q] -= f * S[col * m + q];
                    I[r * m + q] -= f * I[col * m + q];
                }
            }
    }
    for (int q = 0; q < m * m; ++q) inv[q] = I[q];
    return true;
}

// With the kernel vectors n_j of A among the constrained constant pressures (A n_j = 0,
// e.g. p_1 - p_2 for equal alpha, c = S = 0) and A^+ the solve on their complement:
//   x = A^+ b - W lambda + N a,  W = A^+ B^T,
//   N^T (b - B^T lambda) = 0  (consistency),  B x = 0  (constraints).
static int solve_constrained(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous) {
    const int64_t n = c->N;
    const int nq = c->nq;
    int iters = 0;
    if (c->q_dirty) {
        // kernel of A among the constant pressures of the constrained networks
        TmpBuf e(sizeof(double) * n), ae(sizeof(double) * n * (nq > 0 ? nq : 1));
        for (int k = 0; k < nq; ++k) {
            MPET_CUDA(cudaMemsetAsync(e.p, 0, sizeof(double) * n, c->stream));
            k_fill64<<<grid_for(c->nv, 256), 256, 0, c->stream>>>(c->nv, e.as<double>() + c->Nu +
                                                                   (int64_t)c->q_net[k] * c->nv, 1.0);
            MPET_CHECK_LAUNCH();
            launch_spmv<double, 1>(c, c->A, c->A.v64, e.as<double>(), EpiStore<double, 1>{ae.as<double>() + (int64_t)k * n});
        }
        std::vector<double> Gm((size_t)nq * nq), Q((size_t)nq * nq), lam(nq);
        for (int k = 0; k < nq; ++k)
            for (int l = 0; l <= k; ++l)
                Gm[k * nq + l] = Gm[l * nq + k] =
                    dot_host(c, ae.as<double>() + (int64_t)k * n, ae.as<double>() + (int64_t)l * n, n);
        sym_eig(nq, Gm.data(), Q.data(), lam.data());
        double gmax = 0.0;
        for (int k = 0; k < nq; ++k) gmax = fmax(gmax, fabs(lam[k]));
        c->q_nk = 0;
        for (int j = 0; j < nq; ++j) {
            if (!(fabs(lam[j]) <= 1e-12 * gmax)) continue;
            double nrm = 0.0;
            for (int k = 0; k < nq; ++k) nrm += Q[k * nq + j] * Q[k * nq + j];
            nrm = sqrt(nrm * (double)c->nv);
            double* nj = c->q_N + (int64_t)c->q_nk * n;
            MPET_CUDA(cudaMemsetAsync(nj, 0, sizeof(double) * n, c->stream));
            for (int k = 0; k < nq; ++k)
                k_fill64<<<grid_for(c->nv, 256), 256, 0, c->stream>>>(c->nv, nj + c->Nu + (int64_t)c->q_net[k] * c->nv,
                                                                       Q[k * nq + j] / nrm);
            MPET_CHECK_LAUNCH();
            ++c->q_nk;
        }
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        TmpBuf rhs(sizeof(double) * n);
        for (int k = 0; k < nq; ++k) {
            double* Wk = c->q_W + (int64_t)k * n;
            MPET_CUDA(cudaMemsetAsync(rhs.p, 0, sizeof(double) * n, c->stream));
            MPET_CUDA(cudaMemcpyAsync(rhs.as<double>() + c->Nu + (int64_t)c->q_net[k] * c->nv, c->q_load,
                                      sizeof(double) * c->nv, cudaMemcpyDeviceToDevice, c->stream));
            MPET_CUDA(cudaMemsetAsync(Wk, 0, sizeof(double) * n, c->stream));
            mpet_stats s1{};
            const int s = solve_plain(c, rhs.as<double>(), Wk, &s1, true);
            iters += s1.iterations;
            if (s != MPET_OK) {
                if (st) *st = s1;
                return s;
            }
        }
        // [ -N^T B^T    0  ] [lambda]   [ -N^T b ]
        // [ -B W      B N ] [  a   ] = [ -B x0  ]
        const int nk = c->q_nk, m = nq + nk;
        std::vector<double> Mt((size_t)m * m, 0.0);
        for (int j = 0; j < nk; ++j)
            for (int k = 0; k < nq; ++k) Mt[j * m + k] = -q_dot(c, k, c->q_N + (int64_t)j * n);
        for (int k = 0; k < nq; ++k) {
            for (int l = 0; l < nq; ++l) Mt[(nk + k) * m + l] = -q_dot(c, k, c->q_W + (int64_t)l * n);
            for (int j = 0; j < nk; ++j) Mt[(nk + k) * m + nq + j] = q_dot(c, k, c->q_N + (int64_t)j * n);
        }
        if (!small_inverse(Mt, m, c->q_Sinv)) fail(MPET_ERR_BREAKDOWN, "singular pressure-constraint system");
        c->q_dirty = false;
    }
    const int nk = c->q_nk, m = nq + nk;
    std::vector<double> g(m);
    for (int j = 0; j < nk; ++j) g[j] = -dot_host(c, c->q_N + (int64_t)j * n, b, n);
    const int s = solve_plain(c, b, x, st, homogeneous);
    if (st) st->iterations += iters;
    if (s != MPET_OK) return s;
    for (int k = 0; k < nq; ++k) g[nk + k] = -q_dot(c, k, x);
    std::vector<double> z(m, 0.0);
    for (int r = 0; r < m; ++r)
        for (int q = 0; q < m; ++q) z[r] += c->q_Sinv[r * m + q] * g[q];
    const int G = grid_for(n, 256);
    for (int k = 0; k < nq; ++k) {
        c->q_lambda[k] = z[k];
        k_axpy64<<<G, 256, 0, c->stream>>>(n, x, -z[k], c->q_W + (int64_t)k * n);
    }
    for (int j = 0; j < nk; ++j) k_axpy64<<<G, 256, 0, c->stream>>>(n, x, z[nq + j], c->q_N + (int64_t)j * n);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    return MPET_OK;
}

int solve_system(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous) {
    MPET_CUDA(cudaEventRecord(c->ev_sv0, c->stream));
    int s;
    if (c->gmres && (c->ninst > 0 || c->nrigid > 0))
        fail(MPET_ERR_INVALID, "GMRES (non-symmetric S) is built for single instances without rigid modes");
    if (c->nq > 0) s = solve_constrained(c, b, x, st, homogeneous);
    else s = solve_plain(c, b, x, st, homogeneous);
    MPET_CUDA(cudaEventRecord(c->ev_sv1, c->stream));
    MPET_CUDA(cudaEventSynchronize(c->ev_sv1));
    float ms = 0.f;
    MPET_CUDA(cudaEventElapsedTime(&ms, c->ev_sv0, c->ev_sv1));
    c->t_solve_ms += ms;
    return s;
}

void alloc_krylov(mpet_ctx* c) {
    const int64_t n = c->N;
    c->kv = c->pool.alloc<double>(n);
    c->kd = c->pool.alloc<double>(n);
    for (int q = 0; q < 3; ++q) {
        c->kr[q] = c->pool.alloc<double>(n);
        c->kw[q] = c->pool.alloc<double>(n);
    }
    c->orr = c->pool.alloc<double>(n);
    c->partials = c->pool.alloc<double>(2 * NB_RED);
    c->dev_err = c->pool.alloc<int>(1);
    MPET_CUDA(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
    if (!c->ev_fork) MPET_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    for (int a = 0; a < c->J; ++a) {
        if (!c->side[a]) MPET_CUDA(cudaStreamCreateWithFlags(&c->side[a], cudaStreamNonBlocking));
        if (!c->ev_join[a]) MPET_CUDA(cudaEventCreateWithFlags(&c->ev_join[a], cudaEventDisableTiming));
    }
    c->sc = c->pool.alloc<MinresScalars>(1);
    if (!c->sc_host) MPET_CUDA(cudaMallocHost(&c->sc_host, sizeof(MinresScalars)));
    if (!c->loop_ctl_host) MPET_CUDA(cudaMallocHost(&c->loop_ctl_host, 64));
}

// ---- AMG upload ---------------------------------------------------------------------------

static void upload_csr(mpet_ctx* c, const HostCsr& h, Csr& d, bool fp32) {
    d.n = h.n;
    d.m = h.m;
    d.nnz = (int64_t)h.ci.size();
    d.rp = c->pool.alloc<int64_t>(d.n + 1);
    d.ci = c->pool.alloc<int32_t>(d.nnz);
    d.v64 = c->pool.alloc<double>(d.nnz);
    MPET_CUDA(cudaMemcpyAsync(d.rp, h.rp.data(), sizeof(int64_t) * (d.n + 1), cudaMemcpyHostToDevice, c->stream));
    if (d.nnz) {
        MPET_CUDA(cudaMemcpyAsync(d.ci, h.ci.data(), sizeof(int32_t) * d.nnz, cudaMemcpyHostToDevice, c->stream));
        MPET_CUDA(cudaMemcpyAsync(d.v64, h.v.data(), sizeof(double) * d.nnz, cudaMemcpyHostToDevice, c->stream));
    }
    if (fp32) {
        d.v32 = c->pool.alloc<float>(d.nnz);
        if (d.nnz) k_f64_to_f32<<<grid_for(d.nnz, 256), 256, 0, c->stream>>>(d.nnz, d.v64, d.v32);
        MPET_CHECK_LAUNCH();
    }
    d.lpr = choose_lpr(d.n, d.nnz);
    build_tiles(c, d, h.rp.data());
    build_sell(c, d, fp32, false);
}

// First displacement level: matrix-free products when the per-cell data exist and
// (autotuned) a Chebyshev product is faster that way than with the tuned CSR
// layout (median of 5 launches from a flushed L2), or as forced by mf_mode.
template <typename T>
static void choose_mf(mpet_ctx* c, AmgHier& h) {
    AmgLevel& L = h.lev[0];
    L.mf = false;
    c->mf_ms[0] = c->mf_ms[1] = 0.f;
    // batches keep the CSR level (its products skip converged instances), and
    // so does a first level in a spatial order (the per-cell data are in node order)
    if (!c->mf_cell || c->mf_mode == 0 || (c->ninst > 0 && c->batch_skip) || h.perm) return;
    if (c->mf_mode == 1) {
        L.mf = true;
        return;
    }
    constexpr size_t kFlush = 256u << 20;
    if (!c->l2_flush) c->l2_flush = c->pool.alloc<unsigned char>(kFlush);
    const int64_t l0 = c->n_launch;
    const EpiCheb<T, 4> e{(const T*)L.b, (const T*)L.x, (T*)L.d, (T*)L.t0, dinv_of<T>(L), T(0.5), T(0.5)};
    float med[2];
    for (int v = 0; v < 2; ++v) {
        L.mf = v == 1;
        level_spmv<T, 4>(c, L, (const T*)L.x, e);
        float t[5];
        for (int q = 0; q < 5; ++q) {
            MPET_CUDA(cudaMemsetAsync(c->l2_flush, q, kFlush, c->stream));
            MPET_CUDA(cudaEventRecord(c->ev0, c->stream));
            level_spmv<T, 4>(c, L, (const T*)L.x, e);
            MPET_CUDA(cudaEventRecord(c->ev1, c->stream));
            MPET_CUDA(cudaEventSynchronize(c->ev1));
            MPET_CUDA(cudaEventElapsedTime(&t[q], c->ev0, c->ev1));
        }
        std::sort(t, t + 5);
        med[v] = t[2];
    }
    L.mf = med[1] < med[0];
    c->mf_ms[0] = med[0];
    c->mf_ms[1] = med[1];
    c->n_launch = l0;
}

static double csr_rho(mpet_ctx* c, const Csr& A, const double* dinv);

static void release_csr(mpet_ctx* c, Csr& A) {
    for (void* p : {(void*)A.rp, (void*)A.ci, (void*)A.v64, (void*)A.v32, (void*)A.tiles, (void*)A.s_off,
                    (void*)A.s_ci, (void*)A.s_v32, (void*)A.s_v64, (void*)A.skl, (void*)A.s_v16,
                    (void*)A.s_d32})
        c->pool.release(p);
    A = Csr();
}

void release_hier(mpet_ctx* c, AmgHier& h) {
    for (AmgLevel& L : h.lev) {
        release_csr(c, L.A);
        release_csr(c, L.P);
        release_csr(c, L.R);
        for (void* p : {(void*)L.dinv64, (void*)L.dinv32, L.x, L.b, L.r, L.d, L.t0, L.t1, (void*)L.inst})
            c->pool.release(p);
    }
    h.lev.clear();
    for (void* p : {(void*)h.cinv, h.pack_in, h.pack_out}) c->pool.release(p);
    h.cinv = nullptr;
    h.pack_in = h.pack_out = nullptr;
    h.ncoarse = 0;
    h.perm = h.iperm = nullptr;  // the context owns the permutation
}

void upload_amg(mpet_ctx* c, AmgHier& h, const HostAmg& ha, int nvec, bool fp32) {
    release_hier(c, h);  // the arrays of an earlier set-up
    h.nvec = nvec;
    h.cheb_degree = c->prm.amg_cheb_degree > 0 ? c->prm.amg_cheb_degree : 4;
    h.cheb_degree0 = c->prm.amg_cheb_degree_fine > 0 ? c->prm.amg_cheb_degree_fine : h.cheb_degree;
    h.cheb_degree_c = c->prm.amg_cheb_degree_coarse > 0 ? c->prm.amg_cheb_degree_coarse : h.cheb_degree;
    h.cheb_level_c = c->prm.amg_cheb_coarse_level > 0 ? c->prm.amg_cheb_coarse_level : 2;
    h.lev.resize(ha.lev.size());
    for (size_t k = 0; k < ha.lev.size(); ++k) {
        const HostAmgLevel& hl = ha.lev[k];
        AmgLevel& L = h.lev[k];
        upload_csr(c, hl.A, L.A, fp32);
        if (fp32 && k == 0) build_sell_half(c, L.A);
        L.rho = hl.rho;
        const int64_t n = hl.A.n;
        L.dinv64 = c->pool.alloc<double>(n);
        MPET_CUDA(cudaMemcpyAsync(L.dinv64, hl.dinv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        if (L.rho < 0.0) L.rho = csr_rho(c, L.A, L.dinv64);  // left to the GPU by the host set-up
        if (fp32) {
            L.dinv32 = c->pool.alloc<float>(n);
            k_f64_to_f32<<<grid_for(n, 256), 256, 0, c->stream>>>(n, L.dinv64, L.dinv32);
        }
        if (k + 1 < ha.lev.size()) {
            upload_csr(c, hl.P, L.P, fp32);
            upload_csr(c, hl.R, L.R, fp32);
        }
        const int64_t nn = n * nvec;
        L.x = c->pool.alloc<double>(nn);
        L.b = c->pool.alloc<double>(nn);
        L.r = c->pool.alloc<double>(nn);
        L.d = c->pool.alloc<double>(nn);
        L.t0 = c->pool.alloc<double>(nn);
        L.t1 = c->pool.alloc<double>(nn);
    }
    if (nvec == 4) {
        h.pack_in = c->pool.alloc<double>(ha.lev[0].A.n * 4);
        h.pack_out = c->pool.alloc<double>(ha.lev[0].A.n * 4);
    }
    if (nvec == 4) {
        if (fp32) autotune_hier<float, 4>(c, h); else autotune_hier<double, 4>(c, h);
        if (fp32) choose_mf<float>(c, h); else choose_mf<double>(c, h);
    } else {
        if (fp32) autotune_hier<float, 1>(c, h); else autotune_hier<double, 1>(c, h);
    }
    h.ncoarse = ha.ncoarse;
    h.cinv = c->pool.alloc<double>(ha.ncoarse * ha.ncoarse);
    MPET_CUDA(cudaMemcpyAsync(h.cinv, ha.cinv.data(), sizeof(double) * ha.ncoarse * ha.ncoarse,
                              cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

// Levels built on the GPU (amg_device.cu) come with FP64 matrices, dinv64, rho
// and the coarsest inverse; this adds what upload_amg adds to uploaded ones.
static void finish_device_csr(mpet_ctx* c, Csr& d, bool fp32) {
    if (fp32) {
        d.v32 = c->pool.alloc<float>(d.nnz);
        if (d.nnz) k_f64_to_f32<<<grid_for(d.nnz, 256), 256, 0, c->stream>>>(d.nnz, d.v64, d.v32);
        MPET_CHECK_LAUNCH();
    }
    d.lpr = choose_lpr(d.n, d.nnz);
    std::vector<int64_t> rp(d.n + 1);
    MPET_CUDA(cudaMemcpyAsync(rp.data(), d.rp, sizeof(int64_t) * (d.n + 1), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    build_tiles(c, d, rp.data());
    build_sell(c, d, fp32, false);
}

void finish_device_hier(mpet_ctx* c, AmgHier& h, int nvec, bool fp32) {
    h.nvec = nvec;
    h.cheb_degree = c->prm.amg_cheb_degree > 0 ? c->prm.amg_cheb_degree : 4;
    h.cheb_degree0 = c->prm.amg_cheb_degree_fine > 0 ? c->prm.amg_cheb_degree_fine : h.cheb_degree;
    h.cheb_degree_c = c->prm.amg_cheb_degree_coarse > 0 ? c->prm.amg_cheb_degree_coarse : h.cheb_degree;
    h.cheb_level_c = c->prm.amg_cheb_coarse_level > 0 ? c->prm.amg_cheb_coarse_level : 2;
    for (size_t k = 0; k < h.lev.size(); ++k) {
        AmgLevel& L = h.lev[k];
        finish_device_csr(c, L.A, fp32);
        if (fp32 && k == 0) build_sell_half(c, L.A);
        const int64_t n = L.A.n;
        if (fp32) {
            L.dinv32 = c->pool.alloc<float>(n);
            k_f64_to_f32<<<grid_for(n, 256), 256, 0, c->stream>>>(n, L.dinv64, L.dinv32);
            MPET_CHECK_LAUNCH();
        }
        if (k + 1 < h.lev.size()) {
            finish_device_csr(c, L.P, fp32);
            finish_device_csr(c, L.R, fp32);
        }
        const int64_t nn = n * nvec;
        L.x = c->pool.alloc<double>(nn);
        L.b = c->pool.alloc<double>(nn);
        L.r = c->pool.alloc<double>(nn);
        L.d = c->pool.alloc<double>(nn);
        L.t0 = c->pool.alloc<double>(nn);
        L.t1 = c->pool.alloc<double>(nn);
    }
    if (nvec == 4) {
        h.pack_in = c->pool.alloc<double>(h.lev[0].A.n * 4);
        h.pack_out = c->pool.alloc<double>(h.lev[0].A.n * 4);
        if (fp32) autotune_hier<float, 4>(c, h); else autotune_hier<double, 4>(c, h);
        if (fp32) choose_mf<float>(c, h); else choose_mf<double>(c, h);
    } else {
        if (fp32) autotune_hier<float, 1>(c, h); else autotune_hier<double, 1>(c, h);
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

double device_rho(mpet_ctx* c, const Csr& A, const double* dinv) { return csr_rho(c, A, dinv); }

// ---- displacement block as elasticity AMG ------------------------------------------------
//
// Level 0 is the displacement block of the system itself (its node-block copy,
// Chebyshev on D^-1 A_uu); level 1 the P1 vector elasticity on the free vertices
// reached by the P1-in-P2 embedding of each component; below it smoothed
// aggregation with the six rigid-body modes (amg_setup_block_host).

__global__ void k_lz_init(int64_t n, const double* __restrict__ dinv, const uint8_t* __restrict__ bc, double* s,
                          double* v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    s[i] = dinv[i] > 0.0 ? sqrt(dinv[i]) : 0.0;
    v[i] = (bc && bc[i]) ? 0.0 : 0.5 + (double)((7919LL * i) % 1009LL) / 1009.0;
}
template <typename T>
__global__ void k_lz_mul(int64_t n, const double* __restrict__ s, const double* __restrict__ v, T* w) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) w[i] = (T)(s[i] * v[i]);
}
template <typename T>
__global__ void k_lz_w(int64_t n, const double* __restrict__ s, const T* __restrict__ t, double beta,
                       const double* __restrict__ vprev, double* w) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) w[i] = s[i] * (double)t[i] - beta * vprev[i];
}
__global__ void k_lz_axpy(int64_t n, double* w, double a, const double* __restrict__ v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) w[i] += a * v[i];
}
__global__ void k_lz_next(int64_t n, const double* __restrict__ w, double ib, double* vprev, double* v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    vprev[i] = v[i];
    v[i] = w[i] * ib;
}

// Spectral radius of D^-1 A_uu: 30 Lanczos steps on D^-1/2 A_uu D^-1/2 from the fixed
// start vector of the host setup with the Dirichlet rows zeroed (the iterates stay
// where the row-replaced block acts symmetrically).
template <typename T>
static double nb_uu_rho(mpet_ctx* c, const double* dinv) {
    const int64_t n = c->Nu;
    TmpBuf bs(sizeof(double) * n), bv(sizeof(double) * n), bp(sizeof(double) * n), bw(sizeof(double) * n),
        bt(sizeof(double) * n);
    double *s = bs.as<double>(), *v = bv.as<double>(), *vp = bp.as<double>(), *w = bw.as<double>();
    T* t = bt.as<T>();
    const int G = grid_for(n, 256);
    k_lz_init<<<G, 256, 0, c->stream>>>(n, dinv, c->dof_bc, s, v);
    MPET_CUDA(cudaMemsetAsync(vp, 0, sizeof(double) * n, c->stream));
    MPET_CHECK_LAUNCH();
    double nrm = sqrt(dot_host(c, v, v, n));
    if (!(nrm > 0.0)) return 1.0;
    k_lz_next<<<G, 256, 0, c->stream>>>(n, v, 1.0 / nrm, w, v);  // v /= |v| (w scratch)
    MPET_CUDA(cudaMemsetAsync(vp, 0, sizeof(double) * n, c->stream));
    std::vector<double> al, be(1, 0.0);
    double beta = 0.0;
    TmpBuf bx(sizeof(double) * n);
    T* xin = bx.as<T>();
    for (int k = 0; k < 30; ++k) {
        k_lz_mul<T><<<G, 256, 0, c->stream>>>(n, s, v, xin);
        launch_nb_uu<T>(c, *c->A.nb, xin, EpiStore<T, 1>{t});
        k_lz_w<T><<<G, 256, 0, c->stream>>>(n, s, t, beta, vp, w);
        MPET_CHECK_LAUNCH();
        const double alpha = dot_host(c, w, v, n);
        al.push_back(alpha);
        k_lz_axpy<<<G, 256, 0, c->stream>>>(n, w, -alpha, v);
        beta = sqrt(dot_host(c, w, w, n));
        if (beta <= 1e-14 * fabs(alpha) || k + 1 == 30) break;
        be.push_back(beta);
        k_lz_next<<<G, 256, 0, c->stream>>>(n, w, 1.0 / beta, vp, v);
    }
    return tridiag_max_eig_host(al, be);
}

// Spectral radius of D^-1 A for a CSR level on the device (FP64 values): the host
// set-up's Lanczos iteration (lanczos_rho, amg_setup.cpp) with the same start vector,
// 30 steps on D^-1/2 A D^-1/2, largest Ritz value.
static double csr_rho(mpet_ctx* c, const Csr& A, const double* dinv) {
    const int64_t n = A.n;
    TmpBuf bs(sizeof(double) * n), bv(sizeof(double) * n), bp(sizeof(double) * n), bw(sizeof(double) * n),
        bt(sizeof(double) * n), bx(sizeof(double) * n);
    double *s = bs.as<double>(), *v = bv.as<double>(), *vp = bp.as<double>(), *w = bw.as<double>();
    double *t = bt.as<double>(), *xin = bx.as<double>();
    const int G = grid_for(n, 256);
    k_lz_init<<<G, 256, 0, c->stream>>>(n, dinv, nullptr, s, v);
    MPET_CHECK_LAUNCH();
    double nrm = sqrt(dot_host(c, v, v, n));
    if (!(nrm > 0.0)) return 1.0;
    k_lz_next<<<G, 256, 0, c->stream>>>(n, v, 1.0 / nrm, w, v);  // v /= |v| (w scratch)
    MPET_CUDA(cudaMemsetAsync(vp, 0, sizeof(double) * n, c->stream));
    std::vector<double> al, be(1, 0.0);
    double beta = 0.0;
    for (int k = 0; k < 30 && k < n; ++k) {
        k_lz_mul<double><<<G, 256, 0, c->stream>>>(n, s, v, xin);
        launch_spmv<double, 1>(c, A, A.v64, xin, EpiStore<double, 1>{t});
        k_lz_w<double><<<G, 256, 0, c->stream>>>(n, s, t, beta, vp, w);
        MPET_CHECK_LAUNCH();
        const double alpha = dot_host(c, w, v, n);
        al.push_back(alpha);
        k_lz_axpy<<<G, 256, 0, c->stream>>>(n, w, -alpha, v);
        beta = sqrt(dot_host(c, w, w, n));
        if (beta <= 1e-14 * fabs(alpha) || k + 1 == 30 || k + 1 == n) break;
        be.push_back(beta);
        k_lz_next<<<G, 256, 0, c->stream>>>(n, w, 1.0 / beta, vp, v);
    }
    return tridiag_max_eig_host(al, be);
}

bool setup_u_elasticity(mpet_ctx* c, bool fp32) {
    c->u_elast = false;
    if (c->dim != 3 || !c->A.nb || c->ninst > 0 || c->nrigid > 0) return false;
    if (fp32 ? !c->A.nb->v32 : !c->A.nb->v64) return false;
    if (c->bc_off[1] == c->bc_off[0]) return false;  // no displacement Dirichlet rows: singular block
    const int64_t nv = c->nv, nc = c->nc, Nu = c->Nu, nn = c->nnodes;
    std::vector<uint8_t> bc(nn);
    std::vector<int64_t> n1p(nn + 1), incp(nn + 1), ek(c->ne);
    std::vector<double> geo((size_t)nc * 16), xyz((size_t)nv * 3);
    std::vector<int32_t> cells((size_t)nc * 4);
    auto d2h = [&](void* dst, const void* src, size_t bytes) {
        MPET_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    };
    d2h(bc.data(), c->node_bc, nn);
    d2h(n1p.data(), c->n1_ptr, sizeof(int64_t) * (nn + 1));
    d2h(incp.data(), c->inc_ptr, sizeof(int64_t) * (nn + 1));
    d2h(ek.data(), c->edge_key, sizeof(int64_t) * c->ne);
    d2h(geo.data(), c->geo, sizeof(double) * geo.size());
    d2h(xyz.data(), c->x, sizeof(double) * xyz.size());
    d2h(cells.data(), c->cells, sizeof(int32_t) * cells.size());
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int32_t> n1c(n1p[nv]), inc(incp[nv]);
    d2h(n1c.data(), c->n1_col, sizeof(int32_t) * n1c.size());
    d2h(inc.data(), c->inc, sizeof(int32_t) * inc.size());
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int64_t> vptr(n1p.begin(), n1p.begin() + nv + 1);
    std::vector<int64_t> cidx(nv, -1);
    int64_t nf = 0;
    for (int64_t v = 0; v < nv; ++v)
        if (!bc[v]) cidx[v] = nf++;
    if (nf == 0) return false;
    const double lm = c->prm.formulation == MPET_FORM_TOTAL_PRESSURE ? 0.0 : c->prm.lmbda;
    HostCsr A1;
    p1_elasticity_host(nv, vptr, n1c, std::vector<int64_t>(incp.begin(), incp.begin() + nv + 1), inc, geo, cells,
                       cidx, c->prm.mu, lm, A1);
    // rigid-body modes at the free vertices, about their centroid
    double cx[3] = {0, 0, 0};
    for (int64_t v = 0; v < nv; ++v)
        if (cidx[v] >= 0)
            for (int k = 0; k < 3; ++k) cx[k] += xyz[3 * v + k];
    for (int k = 0; k < 3; ++k) cx[k] /= (double)nf;
    std::vector<double> B1((size_t)3 * nf * 6, 0.0);
    for (int64_t v = 0; v < nv; ++v) {
        const int64_t f = cidx[v];
        if (f < 0) continue;
        const double X = xyz[3 * v] - cx[0], Y = xyz[3 * v + 1] - cx[1], Z = xyz[3 * v + 2] - cx[2];
        double* b0 = &B1[(3 * f) * 6];
        double* b1 = &B1[(3 * f + 1) * 6];
        double* b2 = &B1[(3 * f + 2) * 6];
        b0[0] = 1.0;
        b1[1] = 1.0;
        b2[2] = 1.0;
        b1[3] = -Z; b2[3] = Y;   // e_x x r
        b0[4] = Z;  b2[4] = -X;  // e_y x r
        b0[5] = -Y; b1[5] = X;   // e_z x r
    }
    const int cs = c->prm.amg_coarse_size > 0 ? c->prm.amg_coarse_size : 500;
    HostAmg ha;
    amg_setup_block_host(A1, B1, 6, 3, 0.5 * (c->prm.amg_theta >= 0 ? c->prm.amg_theta : 0.1), cs, 12, ha);
    AmgHier& h = c->amg_u;
    upload_amg(c, h, ha, 1, fp32);
    // level 0: the system's displacement block; P = P1-in-P2 embedding of each component
    HostCsr P0;
    P0.n = Nu;
    P0.m = 3 * nf;
    P0.rp.assign(Nu + 1, 0);
    auto ends = [&](int64_t i, int64_t out[2]) -> int {
        if (bc[i]) return 0;
        if (i < nv) {
            out[0] = i;
            return 1;
        }
        int q = 0;
        const int64_t lo = ek[i - nv] / nv, hi = ek[i - nv] % nv;
        if (cidx[lo] >= 0) out[q++] = lo;
        if (cidx[hi] >= 0) out[q++] = hi;
        return q;
    };
    for (int64_t i = 0; i < nn; ++i) {
        int64_t e2[2];
        const int q = ends(i, e2);
        for (int a = 0; a < 3; ++a) P0.rp[3 * i + a + 1] = q;
    }
    for (int64_t i = 0; i < Nu; ++i) P0.rp[i + 1] += P0.rp[i];
    P0.ci.resize(P0.rp[Nu]);
    P0.v.resize(P0.rp[Nu]);
    for (int64_t i = 0; i < nn; ++i) {
        int64_t e2[2];
        const int q = ends(i, e2);
        for (int a = 0; a < 3; ++a) {
            int64_t p = P0.rp[3 * i + a];
            for (int t = 0; t < q; ++t) {
                P0.ci[p] = (int32_t)(3 * cidx[e2[t]] + a);
                P0.v[p] = i < nv ? 1.0 : 0.5;
                ++p;
            }
        }
    }
    // columns ascending within a row (lo < hi, cidx increasing with the vertex id); the
    // tables index device arrays, so check them before the upload
    for (int64_t i = 0; i < Nu; ++i)
        if (P0.rp[i + 1] < P0.rp[i]) fail(MPET_ERR_INVALID, "embedding row pointers not monotone");
    for (int32_t j : P0.ci)
        if (j < 0 || j >= P0.m) fail(MPET_ERR_INVALID, "embedding column out of range");
    if (h.lev.empty() || h.lev[0].A.n != P0.m) fail(MPET_ERR_INVALID, "elasticity hierarchy size mismatch");
    AmgLevel L0;
    L0.nb_uu = true;
    L0.A.n = L0.A.m = Nu;
    upload_csr(c, P0, L0.P, fp32);
    HostCsr R0;
    {
        R0.n = P0.m;
        R0.m = P0.n;
        R0.rp.assign(R0.n + 1, 0);
        for (int32_t j : P0.ci) R0.rp[j + 1]++;
        for (int64_t i = 0; i < R0.n; ++i) R0.rp[i + 1] += R0.rp[i];
        R0.ci.resize(P0.ci.size());
        R0.v.resize(P0.ci.size());
        std::vector<int64_t> pos(R0.rp.begin(), R0.rp.end() - 1);
        for (int64_t i = 0; i < P0.n; ++i)
            for (int64_t e = P0.rp[i]; e < P0.rp[i + 1]; ++e) {
                const int64_t p = pos[P0.ci[e]]++;
                R0.ci[p] = (int32_t)i;
                R0.v[p] = P0.v[e];
            }
    }
    upload_csr(c, R0, L0.R, fp32);
    L0.dinv64 = c->pool.alloc<double>(Nu);
    MPET_CUDA(cudaMemcpyAsync(L0.dinv64, c->dinv, sizeof(double) * Nu, cudaMemcpyDeviceToDevice, c->stream));
    if (fp32) {
        L0.dinv32 = c->pool.alloc<float>(Nu);
        k_f64_to_f32<<<grid_for(Nu, 256), 256, 0, c->stream>>>(Nu, L0.dinv64, L0.dinv32);
        MPET_CHECK_LAUNCH();
    }
    L0.rho = fp32 ? nb_uu_rho<float>(c, L0.dinv64) : nb_uu_rho<double>(c, L0.dinv64);
    L0.x = c->pool.alloc<double>(Nu);
    L0.b = c->pool.alloc<double>(Nu);
    L0.r = c->pool.alloc<double>(Nu);
    L0.d = c->pool.alloc<double>(Nu);
    L0.t0 = c->pool.alloc<double>(Nu);
    L0.t1 = c->pool.alloc<double>(Nu);
    h.lev.insert(h.lev.begin(), L0);
    {
        AmgLevel& Z = h.lev[0];
        AmgLevel& C = h.lev[1];
        MPET_CUDA(cudaMemsetAsync(C.x, 0, sizeof(double) * C.A.n, c->stream));
        MPET_CUDA(cudaMemsetAsync(Z.t0, 0, sizeof(double) * Nu, c->stream));
        MPET_CUDA(cudaMemsetAsync(Z.r, 0, sizeof(double) * Nu, c->stream));
        if (fp32) {
            autotune_matrix<float, 1>(c, Z.P, (const float*)C.x, EpiAxpby<float, 1>{(float*)Z.t0, (const float*)Z.t0, 1.f, 1.f});
            autotune_matrix<float, 1>(c, Z.R, (const float*)Z.r, EpiStore<float, 1>{(float*)C.b});
        } else {
            autotune_matrix<double, 1>(c, Z.P, (const double*)C.x, EpiAxpby<double, 1>{(double*)Z.t0, (const double*)Z.t0, 1.0, 1.0});
            autotune_matrix<double, 1>(c, Z.R, (const double*)Z.r, EpiStore<double, 1>{(double*)C.b});
        }
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->u_elast = true;
    return true;
}

// ---- public helpers used by the API ------------------------------------------------------

void convert_values_to_f32(mpet_ctx* c) {
    if (!c->A.v32) return;
    k_f64_to_f32<<<grid_for(c->nnz, 256), 256, 0, c->stream>>>(c->nnz, c->A.v64, c->A.v32);
    MPET_CHECK_LAUNCH();
}

}  // namespace mpet
