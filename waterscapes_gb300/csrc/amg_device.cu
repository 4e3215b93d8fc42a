// Smoothed-aggregation set-up on the GPU.
//
// The reference preconditions its iterative path with hypre BoomerAMG, whose
// set-up runs inside PETScKrylovSolver("minres", "hypre_amg")
// (src/mpet/mpet/mpetsolver.py:507; the working twin is
// mpettotalpressuresolver.py:448).  This file builds the engine's
// smoothed-aggregation hierarchies (the recipe of amg_setup_host in
// amg_setup.cpp) from the preconditioner blocks where they are assembled, in
// HBM:
//   strength    |a_ij| >= theta_l sqrt(|a_ii a_jj|) (device, count + fill)
//   aggregates  the host's three greedy passes over the strength graph (a
//               sequential pass over a few MB; the only download per level)
//   T           piecewise constant, unit columns (host, from the aggregates)
//   P           (I - 4/3 rho^-1 D^-1 A) T: A T by the sparse product below,
//               merged with T row by row (device)
//   R = P^T     device transpose (column counts, scatter, row sort)
//   A_c         R (A P), two sparse products (device)
//   rho         30 Lanczos steps on D^-1/2 A D^-1/2 (device, same start vector)
//   coarsest    dense Cholesky inverse (host, a few hundred rows)
// The first displacement prolongator (P1-in-P2 embedding of the free
// vertices) is built on the device too.
//
// Sparse product C = A B: a warp per row of C.  Its column set is marked in a
// per-warp shared-memory bitmap over the row's column window (in chunks of
// 16,384 columns when the window is wider), counted, then written in
// increasing order; each value is then the sum over the row's A entries, in
// their order, of a_ik b_kj (b_kj found by binary search in the sorted row k
// of B), rounded mul then add (no fused multiply-add), which is the order and
// rounding of the host's Gustavson product: the two set-ups give the same
// matrices bit for bit wherever their spectral-radius estimates agree.
#include <limits.h>
#include <math.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "mpet_internal.cuh"

namespace mpet {

namespace {

int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > 2147483647LL) g = 2147483647LL;
    return (int)(g < 1 ? 1 : g);
}

// device FP64 CSR whose arrays come from the context pool
struct DMat {
    int64_t n = 0, m = 0, nnz = 0;
    int64_t* rp = nullptr;
    int32_t* ci = nullptr;
    double* v = nullptr;
};

void dm_release(mpet_ctx* c, DMat& a) {
    c->pool.release(a.rp);
    c->pool.release(a.ci);
    c->pool.release(a.v);
    a = DMat();
}

Csr as_csr(const DMat& a) {
    Csr d;
    d.n = a.n;
    d.m = a.m;
    d.nnz = a.nnz;
    d.rp = a.rp;
    d.ci = a.ci;
    d.v64 = a.v;
    d.lpr = choose_lpr(a.n, a.nnz);
    return d;
}

// ---- exclusive scan of int64 counts into row pointers ---------------------------------

constexpr int SCAN_B = 1024;

__device__ __forceinline__ int64_t block_incl_scan(int64_t v, int64_t* ws) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) ws[w] = v;
    __syncthreads();
    if (w == 0) {
        int64_t s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        ws[lane] = s;
    }
    __syncthreads();
    if (w > 0) v += ws[w - 1];
    __syncthreads();
    return v;
}

// out[i + 1] = inclusive sum of in[] within the block; bsum[block] = block total
__global__ void __launch_bounds__(SCAN_B) k_scan_local(int64_t n, const int64_t* __restrict__ in, int64_t* out,
                                                       int64_t* bsum) {
    __shared__ int64_t ws[32];
    const int64_t i = blockIdx.x * (int64_t)SCAN_B + threadIdx.x;
    const int64_t v = block_incl_scan(i < n ? in[i] : 0, ws);
    if (i < n) out[i + 1] = v;
    if (threadIdx.x == SCAN_B - 1) bsum[blockIdx.x] = v;
}

// exclusive prefix of the block totals, in place (one block)
__global__ void __launch_bounds__(SCAN_B) k_scan_top(int64_t nb, int64_t* bsum) {
    __shared__ int64_t ws[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += SCAN_B) {
        const int64_t i = base + threadIdx.x;
        const int64_t v = i < nb ? bsum[i] : 0;
        const int64_t incl = block_incl_scan(v, ws);
        const int64_t excl = carry + incl - v;
        __syncthreads();
        if (i < nb) bsum[i] = excl;
        if (threadIdx.x == SCAN_B - 1) carry += incl;
        __syncthreads();
    }
}

__global__ void k_scan_add(int64_t n, int64_t* out, const int64_t* __restrict__ bsum) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i == 0) out[0] = 0;
    if (i < n) out[i + 1] += bsum[i / SCAN_B];
}

// rp[0] = 0, rp[i + 1] = cnt[0] + ... + cnt[i]; returns rp[n]
int64_t scan_counts(mpet_ctx* c, const int64_t* cnt, int64_t n, int64_t* rp) {
    if (n == 0) {
        MPET_CUDA(cudaMemsetAsync(rp, 0, sizeof(int64_t), c->stream));
        return 0;
    }
    const int64_t nb = (n + SCAN_B - 1) / SCAN_B;
    TmpBuf bs(sizeof(int64_t) * nb);
    k_scan_local<<<(unsigned)nb, SCAN_B, 0, c->stream>>>(n, cnt, rp, bs.as<int64_t>());
    k_scan_top<<<1, SCAN_B, 0, c->stream>>>(nb, bs.as<int64_t>());
    k_scan_add<<<grid_for(n, 256), 256, 0, c->stream>>>(n, rp, bs.as<int64_t>());
    MPET_CHECK_LAUNCH();
    int64_t total = 0;
    MPET_CUDA(cudaMemcpyAsync(&total, rp + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    return total;
}

// ---- diagonal, strength ---------------------------------------------------------------

// first diagonal entry of each row (0 when absent) and its inverse (0 for 0)
__global__ void k_diag(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                       const double* __restrict__ v, double* dg, double* dinv) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e)
        if (ci[e] == i) {
            d = v[e];
            break;
        }
    dg[i] = fabs(d);
    dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
}

__device__ __forceinline__ bool is_strong(int64_t i, int32_t j, double a, const double* __restrict__ dg, double th) {
    const double v = fabs(a);
    return j != i && v > 0.0 && v >= th * sqrt(dg[i] * dg[j]);
}

template <bool FILL>
__global__ void k_strength(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                           const double* __restrict__ v, const double* __restrict__ dg, double th, int64_t* cnt,
                           const int64_t* __restrict__ srp, int32_t* sci) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t k = 0, p = FILL ? srp[i] : 0;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e)
        if (is_strong(i, ci[e], v[e], dg, th)) {
            if (FILL) sci[p++] = ci[e];
            else ++k;
        }
    if (!FILL) cnt[i] = k;
}

// ---- sparse product C = A B -------------------------------------------------------------

constexpr int SPG_WARPS = 8;    // warps (rows) per 256-thread block
constexpr int SPG_WORDS = 512;  // bitmap words per warp: 16,384 columns per chunk

__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// column window [lo, hi] of each row of C (hi < lo: empty row); B's rows are sorted
__global__ void k_spg_range(int64_t n, const int64_t* __restrict__ arp, const int32_t* __restrict__ aci,
                            const int64_t* __restrict__ brp, const int32_t* __restrict__ bci, int32_t* lo,
                            int32_t* hi) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    int l = INT_MAX, h = -1;
    for (int64_t e = arp[row] + lane; e < arp[row + 1]; e += 32) {
        const int32_t k = aci[e];
        const int64_t b0 = brp[k], b1 = brp[k + 1];
        if (b1 > b0) {
            l = min(l, bci[b0]);
            h = max(h, bci[b1 - 1]);
        }
    }
    l = warp_min(l);
    h = warp_max(h);
    if (lane == 0) {
        lo[row] = l;
        hi[row] = h;
    }
}

// FILL = false: cnt[row] = columns of C's row; FILL = true: write them sorted at crp[row]
template <bool FILL>
__global__ void __launch_bounds__(256) k_spg_sym(int64_t n, const int64_t* __restrict__ arp,
                                                 const int32_t* __restrict__ aci, const int64_t* __restrict__ brp,
                                                 const int32_t* __restrict__ bci, const int32_t* __restrict__ lo,
                                                 const int32_t* __restrict__ hi, int64_t* cnt,
                                                 const int64_t* __restrict__ crp, int32_t* cci) {
    __shared__ uint32_t bm[SPG_WARPS][SPG_WORDS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row = blockIdx.x * (int64_t)SPG_WARPS + w;
    if (row >= n) return;  // whole warps; the kernel synchronises warps only
    uint32_t* B = bm[w];
    const int64_t l = lo[row], h = hi[row];
    int64_t total = 0, out = FILL ? crp[row] : 0;
    constexpr int64_t CAP = (int64_t)SPG_WORDS * 32;
    for (int64_t base = l; base <= h; base += CAP) {
        const int span = (int)min(h - base + 1, CAP);
        const int nw = (span + 31) >> 5;
        for (int q = lane; q < nw; q += 32) B[q] = 0u;
        __syncwarp();
        for (int64_t e = arp[row] + lane; e < arp[row + 1]; e += 32) {
            const int32_t k = aci[e];
            for (int64_t f = brp[k]; f < brp[k + 1]; ++f) {
                const int64_t col = (int64_t)bci[f] - base;
                if (col >= 0 && col < span) atomicOr(&B[col >> 5], 1u << (col & 31));
            }
        }
        __syncwarp();
        if (!FILL) {
            int s = 0;
            for (int q = lane; q < nw; q += 32) s += __popc(B[q]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            total += s;
        } else {
            for (int q0 = 0; q0 < nw; q0 += 32) {
                const int q = q0 + lane;
                uint32_t word = q < nw ? B[q] : 0u;
                const int pc = __popc(word);
                int incl = pc;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                int64_t pos = out + incl - pc;
                while (word) {
                    const int bit = __ffs(word) - 1;
                    cci[pos++] = (int32_t)(base + (q << 5) + bit);
                    word &= word - 1;
                }
                out += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
        __syncwarp();
    }
    if (!FILL && lane == 0) cnt[row] = total;
}

// c_ij = sum over the row's A entries, in order, of a_ik b_kj (mul, then add)
__global__ void k_spg_val(int64_t n, const int64_t* __restrict__ arp, const int32_t* __restrict__ aci,
                          const double* __restrict__ av, const int64_t* __restrict__ brp,
                          const int32_t* __restrict__ bci, const double* __restrict__ bv,
                          const int64_t* __restrict__ crp, const int32_t* __restrict__ cci, double* cv) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const int64_t a0 = arp[row], a1 = arp[row + 1];
    for (int64_t p = crp[row] + lane; p < crp[row + 1]; p += 32) {
        const int32_t j = cci[p];
        double acc = 0.0;
        for (int64_t e = a0; e < a1; ++e) {
            const int32_t k = aci[e];
            int64_t lo = brp[k], hi = brp[k + 1] - 1;
            while (lo <= hi) {
                const int64_t mid = (lo + hi) >> 1;
                const int32_t cj = bci[mid];
                if (cj < j) {
                    lo = mid + 1;
                } else if (cj > j) {
                    hi = mid - 1;
                } else {
                    acc = __dadd_rn(acc, __dmul_rn(av[e], bv[mid]));
                    break;
                }
            }
        }
        cv[p] = acc;
    }
}

DMat spgemm(mpet_ctx* c, const DMat& A, const DMat& B) {
    DMat C;
    C.n = A.n;
    C.m = B.m;
    C.rp = c->pool.alloc<int64_t>(C.n + 1);
    TmpBuf blo(sizeof(int32_t) * (C.n + 1)), bhi(sizeof(int32_t) * (C.n + 1)), bcnt(sizeof(int64_t) * (C.n + 1));
    const unsigned gw = (unsigned)((C.n * 32 + 255) / 256);  // a warp per row
    const unsigned gs = (unsigned)((C.n + SPG_WARPS - 1) / SPG_WARPS);
    if (C.n > 0) {
        k_spg_range<<<gw, 256, 0, c->stream>>>(A.n, A.rp, A.ci, B.rp, B.ci, blo.as<int32_t>(), bhi.as<int32_t>());
        k_spg_sym<false><<<gs, 256, 0, c->stream>>>(A.n, A.rp, A.ci, B.rp, B.ci, blo.as<int32_t>(),
                                                    bhi.as<int32_t>(), bcnt.as<int64_t>(), nullptr, nullptr);
        MPET_CHECK_LAUNCH();
    }
    C.nnz = scan_counts(c, bcnt.as<int64_t>(), C.n, C.rp);
    C.ci = c->pool.alloc<int32_t>(C.nnz);
    C.v = c->pool.alloc<double>(C.nnz);
    if (C.n > 0 && C.nnz > 0) {
        k_spg_sym<true><<<gs, 256, 0, c->stream>>>(A.n, A.rp, A.ci, B.rp, B.ci, blo.as<int32_t>(),
                                                   bhi.as<int32_t>(), nullptr, C.rp, C.ci);
        k_spg_val<<<gw, 256, 0, c->stream>>>(A.n, A.rp, A.ci, A.v, B.rp, B.ci, B.v, C.rp, C.ci, C.v);
        MPET_CHECK_LAUNCH();
    }
    return C;
}

// ---- transpose --------------------------------------------------------------------------

__global__ void k_tr_count(int64_t nnz, const int32_t* __restrict__ ci, unsigned long long* cnt) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < nnz) atomicAdd(cnt + ci[e], 1ull);
}

__global__ void k_tr_fill(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          const double* __restrict__ v, const int64_t* __restrict__ trp, unsigned long long* cur,
                          int32_t* tci, double* tv) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
        const int32_t j = ci[e];
        const int64_t pos = trp[j] + (int64_t)atomicAdd(cur + j, 1ull);
        tci[pos] = (int32_t)i;
        tv[pos] = v[e];
    }
}

// Rows put in column order (the scatter above left them in any order): a warp
// per row marks the row's columns (distinct) in a shared-memory bitmap over
// their window, in chunks of 16,384 columns, and each entry goes to the rank
// of its column, found from the words' prefix counts.  Linear in the row
// length plus the window, however long the row (the coarse levels' rows hold
// thousands of entries).
__global__ void __launch_bounds__(256) k_row_rank(int64_t n, const int64_t* __restrict__ rp,
                                                  const int32_t* __restrict__ ci_in, const double* __restrict__ v_in,
                                                  int32_t* ci, double* v) {
    __shared__ uint32_t bm[SPG_WARPS][SPG_WORDS];
    __shared__ int32_t pre[SPG_WARPS][SPG_WORDS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row = blockIdx.x * (int64_t)SPG_WARPS + w;
    if (row >= n) return;  // whole warps; the kernel synchronises warps only
    uint32_t* B = bm[w];
    int32_t* X = pre[w];
    const int64_t e0 = rp[row], e1 = rp[row + 1];
    int l = INT_MAX, h = -1;
    for (int64_t e = e0 + lane; e < e1; e += 32) {
        l = min(l, ci_in[e]);
        h = max(h, ci_in[e]);
    }
    l = warp_min(l);
    h = warp_max(h);
    constexpr int64_t CAP = (int64_t)SPG_WORDS * 32;
    int64_t done = 0;  // entries of earlier chunks
    for (int64_t base = l; base <= h; base += CAP) {
        const int span = (int)min((int64_t)h - base + 1, CAP);
        const int nw = (span + 31) >> 5;
        for (int q = lane; q < nw; q += 32) B[q] = 0u;
        __syncwarp();
        for (int64_t e = e0 + lane; e < e1; e += 32) {
            const int64_t col = (int64_t)ci_in[e] - base;
            if (col >= 0 && col < span) atomicOr(&B[col >> 5], 1u << (col & 31));
        }
        __syncwarp();
        int carry = 0;
        for (int q0 = 0; q0 < nw; q0 += 32) {
            const int q = q0 + lane;
            const int pc = q < nw ? __popc(B[q]) : 0;
            int incl = pc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (q < nw) X[q] = carry + incl - pc;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        __syncwarp();
        for (int64_t e = e0 + lane; e < e1; e += 32) {
            const int64_t col = (int64_t)ci_in[e] - base;
            if (col >= 0 && col < span) {
                const int wq = (int)(col >> 5), bit = (int)(col & 31);
                const int64_t pos = e0 + done + X[wq] + __popc(B[wq] & ((1u << bit) - 1u));
                ci[pos] = ci_in[e];
                v[pos] = v_in[e];
            }
        }
        done += carry;
        __syncwarp();
    }
}

DMat transpose(mpet_ctx* c, const DMat& P) {
    DMat R;
    R.n = P.m;
    R.m = P.n;
    R.nnz = P.nnz;
    R.rp = c->pool.alloc<int64_t>(R.n + 1);
    R.ci = c->pool.alloc<int32_t>(R.nnz);
    R.v = c->pool.alloc<double>(R.nnz);
    TmpBuf bc(sizeof(int64_t) * (R.n + 1));
    MPET_CUDA(cudaMemsetAsync(bc.p, 0, sizeof(int64_t) * (R.n + 1), c->stream));
    if (P.nnz > 0)
        k_tr_count<<<grid_for(P.nnz, 256), 256, 0, c->stream>>>(P.nnz, P.ci, bc.as<unsigned long long>());
    MPET_CHECK_LAUNCH();
    scan_counts(c, bc.as<int64_t>(), R.n, R.rp);
    MPET_CUDA(cudaMemsetAsync(bc.p, 0, sizeof(int64_t) * (R.n + 1), c->stream));
    TmpBuf tci(sizeof(int32_t) * (R.nnz + 1)), tv(sizeof(double) * (R.nnz + 1));
    if (P.n > 0)
        k_tr_fill<<<grid_for(P.n, 256), 256, 0, c->stream>>>(P.n, P.rp, P.ci, P.v, R.rp,
                                                             bc.as<unsigned long long>(), tci.as<int32_t>(),
                                                             tv.as<double>());
    if (R.n > 0)
        k_row_rank<<<(unsigned)((R.n + SPG_WARPS - 1) / SPG_WARPS), 256, 0, c->stream>>>(
            R.n, R.rp, tci.as<int32_t>(), tv.as<double>(), R.ci, R.v);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(c->stream));  // before the scratch goes
    return R;
}

// ---- prolongators -------------------------------------------------------------------------

// P = T - w D^-1 (A T) row by row: the (sorted) A T row with T's entry merged in
template <bool FILL>
__global__ void k_smooth_p(int64_t n, const int64_t* __restrict__ trp, const int32_t* __restrict__ tci,
                           const double* __restrict__ tv, const int64_t* __restrict__ arp,
                           const int32_t* __restrict__ aci, const double* __restrict__ av,
                           const double* __restrict__ dinv, double w, int64_t* cnt, const int64_t* __restrict__ prp,
                           int32_t* pci, double* pv) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool hasT = trp[i + 1] > trp[i];
    const int32_t tj = hasT ? tci[trp[i]] : -1;
    if (!FILL) {
        int64_t k = arp[i + 1] - arp[i];
        if (hasT) {
            bool found = false;
            for (int64_t e = arp[i]; e < arp[i + 1]; ++e) found = found || aci[e] == tj;
            if (!found) ++k;
        }
        cnt[i] = k;
        return;
    }
    const double t = hasT ? tv[trp[i]] : 0.0;
    const double s = __dmul_rn(-w, dinv[i]);
    int64_t p = prp[i];
    bool placed = !hasT;
    for (int64_t e = arp[i]; e < arp[i + 1]; ++e) {
        const int32_t j = aci[e];
        if (!placed && tj < j) {
            pci[p] = tj;
            pv[p] = t;
            ++p;
            placed = true;
        }
        double x = __dmul_rn(s, av[e]);
        if (j == tj) {
            x = __dadd_rn(x, t);
            placed = true;
        }
        pci[p] = j;
        pv[p] = x;
        ++p;
    }
    if (!placed) {
        pci[p] = tj;
        pv[p] = t;
    }
}

// P1-in-P2 embedding of the free vertices: vertex rows copy their vertex,
// edge-midpoint rows average the free ends; Dirichlet rows are empty
__global__ void k_free_flags(int64_t nv, const uint8_t* __restrict__ bc, int64_t* f) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v < nv) f[v] = bc[v] ? 0 : 1;
}

template <bool FILL>
__global__ void k_embed(int64_t nn, int64_t nv, const uint8_t* __restrict__ bc, const int64_t* __restrict__ ek,
                        const int64_t* __restrict__ cidx, int64_t* cnt, const int64_t* __restrict__ rp, int32_t* ci,
                        double* v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nn) return;
    int64_t k = 0, p = FILL ? rp[i] : 0;
    if (!bc[i]) {
        if (i < nv) {
            if (FILL) {
                ci[p] = (int32_t)cidx[i];
                v[p] = 1.0;
            }
            k = 1;
        } else {
            const int64_t key = ek[i - nv];
            const int64_t ends[2] = {key / nv, key % nv};
            for (int t = 0; t < 2; ++t)
                if (!bc[ends[t]]) {
                    if (FILL) {
                        ci[p] = (int32_t)cidx[ends[t]];
                        v[p] = 0.5;
                        ++p;
                    }
                    ++k;
                }
        }
    }
    if (!FILL) cnt[i] = k;
}

DMat embedding_p0(mpet_ctx* c) {
    const int64_t nn = c->nnodes, nv = c->nv;
    TmpBuf bf(sizeof(int64_t) * (nv + 1)), bcx(sizeof(int64_t) * (nv + 1)), bcnt(sizeof(int64_t) * (nn + 1));
    k_free_flags<<<grid_for(nv, 256), 256, 0, c->stream>>>(nv, c->node_bc, bf.as<int64_t>());
    MPET_CHECK_LAUNCH();
    DMat P;
    P.n = nn;
    P.m = scan_counts(c, bf.as<int64_t>(), nv, bcx.as<int64_t>());
    P.rp = c->pool.alloc<int64_t>(nn + 1);
    k_embed<false><<<grid_for(nn, 256), 256, 0, c->stream>>>(nn, nv, c->node_bc, c->edge_key, bcx.as<int64_t>(),
                                                             bcnt.as<int64_t>(), nullptr, nullptr, nullptr);
    MPET_CHECK_LAUNCH();
    P.nnz = scan_counts(c, bcnt.as<int64_t>(), nn, P.rp);
    P.ci = c->pool.alloc<int32_t>(P.nnz);
    P.v = c->pool.alloc<double>(P.nnz);
    k_embed<true><<<grid_for(nn, 256), 256, 0, c->stream>>>(nn, nv, c->node_bc, c->edge_key, bcx.as<int64_t>(),
                                                            nullptr, P.rp, P.ci, P.v);
    MPET_CHECK_LAUNCH();
    return P;
}

// Smoothed-aggregation prolongator of A at threshold th (false: A is not
// coarsened: no aggregate, or as many aggregates as rows)
template <class Tick>
bool sa_prolongator_device(mpet_ctx* c, const DMat& A, const double* dg, const double* dinv, double rho, double th,
                           DMat& P, Tick& tick) {
    const int64_t n = A.n;
    TmpBuf bcnt(sizeof(int64_t) * (n + 1)), brp(sizeof(int64_t) * (n + 1));
    HostCsr S;
    auto strength = [&](double t) {
        k_strength<false><<<grid_for(n, 256), 256, 0, c->stream>>>(n, A.rp, A.ci, A.v, dg, t, bcnt.as<int64_t>(),
                                                                   nullptr, nullptr);
        MPET_CHECK_LAUNCH();
        const int64_t ns = scan_counts(c, bcnt.as<int64_t>(), n, brp.as<int64_t>());
        TmpBuf bci(sizeof(int32_t) * (ns + 1));
        k_strength<true><<<grid_for(n, 256), 256, 0, c->stream>>>(n, A.rp, A.ci, A.v, dg, t, nullptr,
                                                                  brp.as<int64_t>(), bci.as<int32_t>());
        MPET_CHECK_LAUNCH();
        S.n = S.m = n;
        S.rp.resize(n + 1);
        S.ci.resize(ns);
        MPET_CUDA(cudaMemcpyAsync(S.rp.data(), brp.p, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
        if (ns) MPET_CUDA(cudaMemcpyAsync(S.ci.data(), bci.p, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
    };
    strength(th);
    std::vector<int64_t> agg;
    int64_t nagg = aggregate(S, agg);
    if (nagg == 0 && th > 0.0) {
        strength(0.0);
        nagg = aggregate(S, agg);
    }
    tick(2);
    if (nagg == 0 || nagg >= n) return false;
    std::vector<int64_t> size(nagg, 0);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) size[agg[i]]++;
    std::vector<int64_t> trp(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) trp[i + 1] = trp[i] + (agg[i] >= 0 ? 1 : 0);
    std::vector<int32_t> tci(trp[n]);
    std::vector<double> tv(trp[n]);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) {
            tci[trp[i]] = (int32_t)agg[i];
            tv[trp[i]] = 1.0 / sqrt((double)size[agg[i]]);
        }
    DMat T;
    T.n = n;
    T.m = nagg;
    T.nnz = trp[n];
    T.rp = c->pool.alloc<int64_t>(n + 1);
    T.ci = c->pool.alloc<int32_t>(T.nnz);
    T.v = c->pool.alloc<double>(T.nnz);
    MPET_CUDA(cudaMemcpyAsync(T.rp, trp.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, c->stream));
    if (T.nnz) {
        MPET_CUDA(cudaMemcpyAsync(T.ci, tci.data(), sizeof(int32_t) * T.nnz, cudaMemcpyHostToDevice, c->stream));
        MPET_CUDA(cudaMemcpyAsync(T.v, tv.data(), sizeof(double) * T.nnz, cudaMemcpyHostToDevice, c->stream));
    }
    DMat AT = spgemm(c, A, T);
    const double w = 4.0 / 3.0 / rho;
    P = DMat();
    P.n = n;
    P.m = nagg;
    P.rp = c->pool.alloc<int64_t>(n + 1);
    k_smooth_p<false><<<grid_for(n, 256), 256, 0, c->stream>>>(n, T.rp, T.ci, T.v, AT.rp, AT.ci, AT.v, dinv, w,
                                                               bcnt.as<int64_t>(), nullptr, nullptr, nullptr);
    MPET_CHECK_LAUNCH();
    P.nnz = scan_counts(c, bcnt.as<int64_t>(), n, P.rp);
    P.ci = c->pool.alloc<int32_t>(P.nnz);
    P.v = c->pool.alloc<double>(P.nnz);
    k_smooth_p<true><<<grid_for(n, 256), 256, 0, c->stream>>>(n, T.rp, T.ci, T.v, AT.rp, AT.ci, AT.v, dinv, w,
                                                              nullptr, P.rp, P.ci, P.v);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    dm_release(c, AT);
    dm_release(c, T);
    return true;
}

// ---- spatial order of the first displacement level ----------------------------------

// new row k <- old row iperm[k]: row lengths
__global__ void k_perm_len(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ iperm, int64_t* cnt) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) cnt[k] = rp[iperm[k] + 1] - rp[iperm[k]];
}

// copies old row iperm[k] to new row k, columns through perm (null: unchanged)
__global__ void k_perm_fill(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, const int32_t* __restrict__ iperm,
                            const int32_t* __restrict__ perm, const int64_t* __restrict__ nrp, int32_t* oci,
                            double* ov) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t i = iperm[k], e0 = rp[i], e1 = rp[i + 1], p0 = nrp[k];
    for (int64_t e = e0; e < e1; ++e) {
        oci[p0 + (e - e0)] = perm ? perm[ci[e]] : ci[e];
        ov[p0 + (e - e0)] = v[e];
    }
}

// Pi A Pi^T (cols = true) or Pi A (rows only), rows sorted
DMat permuted(mpet_ctx* c, const DMat& A, const int32_t* perm, const int32_t* iperm, bool cols) {
    DMat B;
    B.n = A.n;
    B.m = A.m;
    B.rp = c->pool.alloc<int64_t>(A.n + 1);
    TmpBuf bcnt(sizeof(int64_t) * (A.n + 1));
    k_perm_len<<<grid_for(A.n, 256), 256, 0, c->stream>>>(A.n, A.rp, iperm, bcnt.as<int64_t>());
    MPET_CHECK_LAUNCH();
    B.nnz = scan_counts(c, bcnt.as<int64_t>(), A.n, B.rp);
    if (B.nnz != A.nnz) fail(MPET_ERR_STATE, "permutation lost entries");
    B.ci = c->pool.alloc<int32_t>(B.nnz);
    B.v = c->pool.alloc<double>(B.nnz);
    if (!cols) {
        k_perm_fill<<<grid_for(A.n, 256), 256, 0, c->stream>>>(A.n, A.rp, A.ci, A.v, iperm, nullptr, B.rp, B.ci, B.v);
        MPET_CHECK_LAUNCH();
        return B;
    }
    TmpBuf tci(sizeof(int32_t) * (B.nnz + 1)), tv(sizeof(double) * (B.nnz + 1));
    k_perm_fill<<<grid_for(A.n, 256), 256, 0, c->stream>>>(A.n, A.rp, A.ci, A.v, iperm, perm, B.rp,
                                                           tci.as<int32_t>(), tv.as<double>());
    k_row_rank<<<(unsigned)((B.n + SPG_WARPS - 1) / SPG_WARPS), 256, 0, c->stream>>>(
        B.n, B.rp, tci.as<int32_t>(), tv.as<double>(), B.ci, B.v);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    return B;
}

uint64_t spread3(uint64_t x) {  // the low 21 bits of x to every third bit
    x &= 0x1fffffULL;
    x = (x | x << 32) & 0x1f00000000ffffULL;
    x = (x | x << 16) & 0x1f0000ff0000ffULL;
    x = (x | x << 8) & 0x100f00f00f00f00fULL;
    x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
    x = (x | x << 2) & 0x1249249249249249ULL;
    return x;
}

// P2 nodes (vertices, then edge midpoints) sorted by the Morton code of their
// position in the mesh's bounding box (21 bits per axis; ties by node id),
// then, within each window of 256 positions (the rows one 256-thread block of
// the SELL kernel takes at a time), by decreasing row length of the first
// level (stable): the Morton order alone mixes vertex rows (about 65 entries)
// and edge rows (10-27) in every 32-row slice, which doubles the SELL padding.
// u_perm[node] = its row of the first displacement level, u_iperm the inverse.
void build_u_perm(mpet_ctx* c, const Csr& A0) {
    if (c->u_perm) return;
    const int64_t nv = c->nv, ne = c->ne, nn = c->nnodes;
    if (nn != nv + ne) fail(MPET_ERR_STATE, "P2 nodes are not vertices + edges");
    std::vector<double> x((size_t)nv * 3);
    std::vector<int64_t> ek(ne);
    MPET_CUDA(cudaMemcpyAsync(x.data(), c->x, sizeof(double) * x.size(), cudaMemcpyDeviceToHost, c->stream));
    if (ne) MPET_CUDA(cudaMemcpyAsync(ek.data(), c->edge_key, sizeof(int64_t) * ne, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    double lo[3] = {x[0], x[1], x[2]}, hi[3] = {x[0], x[1], x[2]};
    for (int64_t v = 0; v < nv; ++v)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], x[3 * v + d]);
            hi[d] = std::max(hi[d], x[3 * v + d]);
        }
    double sc[3];
    for (int d = 0; d < 3; ++d) sc[d] = hi[d] > lo[d] ? 2097151.0 / (hi[d] - lo[d]) : 0.0;
    std::vector<std::pair<uint64_t, int32_t>> key(nn);
    auto code = [&](const double* p) {
        uint64_t m = 0;
        for (int d = 0; d < 3; ++d) {
            double q = (p[d] - lo[d]) * sc[d];
            q = q < 0.0 ? 0.0 : (q > 2097151.0 ? 2097151.0 : q);
            m |= spread3((uint64_t)q) << d;
        }
        return m;
    };
    for (int64_t v = 0; v < nv; ++v) key[v] = {code(&x[3 * v]), (int32_t)v};
    for (int64_t e = 0; e < ne; ++e) {
        const int64_t a = ek[e] / nv, b = ek[e] % nv;
        const double mid[3] = {0.5 * (x[3 * a] + x[3 * b]), 0.5 * (x[3 * a + 1] + x[3 * b + 1]),
                               0.5 * (x[3 * a + 2] + x[3 * b + 2])};
        key[nv + e] = {code(mid), (int32_t)(nv + e)};
    }
    std::sort(key.begin(), key.end());
    std::vector<int64_t> rp(nn + 1);
    MPET_CUDA(cudaMemcpyAsync(rp.data(), A0.rp, sizeof(int64_t) * (nn + 1), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int32_t> perm(nn), iperm(nn);
    for (int64_t k = 0; k < nn; ++k) iperm[k] = key[k].second;
    constexpr int64_t WIN = 256;
    for (int64_t w0 = 0; w0 < nn; w0 += WIN) {
        const int64_t w1 = std::min(w0 + WIN, nn);
        std::stable_sort(iperm.begin() + w0, iperm.begin() + w1, [&](int32_t a, int32_t b) {
            return rp[a + 1] - rp[a] > rp[b + 1] - rp[b];
        });
    }
    for (int64_t k = 0; k < nn; ++k) perm[iperm[k]] = (int32_t)k;
    c->u_perm = c->pool.alloc<int32_t>(nn);
    c->u_iperm = c->pool.alloc<int32_t>(nn);
    MPET_CUDA(cudaMemcpyAsync(c->u_perm, perm.data(), sizeof(int32_t) * nn, cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->u_iperm, iperm.data(), sizeof(int32_t) * nn, cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

}  // namespace

void amg_setup_device(mpet_ctx* c, AmgHier& h, const Csr& A0, bool with_p0, double theta, int coarse_size,
                      int max_levels, int nvec, bool fp32, double ms[2]) {
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto tp = t0;
    // phase k gets the time since the previous tick (after the stream drained)
    auto tick = [&](int k) {
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        const auto now = clk::now();
        c->amg_phase_ms[k] += std::chrono::duration<double, std::milli>(now - tp).count();
        tp = now;
    };
    if (coarse_size < 1) coarse_size = 500;
    if (max_levels < 1) max_levels = 12;
    release_hier(c, h);
    if (!A0.v64) fail(MPET_ERR_STATE, "device AMG set-up needs the FP64 block");
    // the block is reassembled in place by later set-ups: the hierarchy keeps a copy
    DMat A;
    A.n = A0.n;
    A.m = A0.m;
    MPET_CUDA(cudaMemcpyAsync(&A.nnz, A0.rp + A0.n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    int64_t r0 = 0;
    MPET_CUDA(cudaMemcpyAsync(&r0, A0.rp, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    if (r0 != 0) fail(MPET_ERR_STATE, "unexpected row pointer base");
    A.rp = c->pool.alloc<int64_t>(A.n + 1);
    A.ci = c->pool.alloc<int32_t>(A.nnz);
    A.v = c->pool.alloc<double>(A.nnz);
    MPET_CUDA(cudaMemcpyAsync(A.rp, A0.rp, sizeof(int64_t) * (A.n + 1), cudaMemcpyDeviceToDevice, c->stream));
    if (A.nnz) {
        MPET_CUDA(cudaMemcpyAsync(A.ci, A0.ci, sizeof(int32_t) * A.nnz, cudaMemcpyDeviceToDevice, c->stream));
        MPET_CUDA(cudaMemcpyAsync(A.v, A0.v64, sizeof(double) * A.nnz, cudaMemcpyDeviceToDevice, c->stream));
    }
    // the first displacement level in a spatial order (rows and columns), its
    // embedding's rows with it: products over neighbouring rows then share columns
    const bool spatial = with_p0 && c->prm.prec_u_order == 1 && A.n == c->nnodes;
    if (spatial) {
        build_u_perm(c, A0);
        DMat B = permuted(c, A, c->u_perm, c->u_iperm, true);
        dm_release(c, A);
        A = B;
        h.perm = c->u_perm;
        h.iperm = c->u_iperm;
    }
    tick(0);
    while (true) {
        AmgLevel L;
        const int64_t n = A.n;
        L.A = as_csr(A);
        L.dinv64 = c->pool.alloc<double>(n);
        TmpBuf bdg(sizeof(double) * (n + 1));
        k_diag<<<grid_for(n, 256), 256, 0, c->stream>>>(n, A.rp, A.ci, A.v, bdg.as<double>(), L.dinv64);
        MPET_CHECK_LAUNCH();
        L.rho = device_rho(c, L.A, L.dinv64);
        tick(1);
        const bool given = with_p0 && h.lev.empty();
        h.lev.push_back(L);
        if (!given && (n <= coarse_size || (int)h.lev.size() >= max_levels)) break;
        DMat P;
        if (given) {
            P = embedding_p0(c);
            if (P.n != n) fail(MPET_ERR_INVALID, "first-level prolongator has the wrong row count");
            if (spatial) {
                DMat Q = permuted(c, P, nullptr, c->u_iperm, false);
                dm_release(c, P);
                P = Q;
            }
        } else {
            const int sa_level = (int)h.lev.size() - 1 - (with_p0 ? 1 : 0);
            const double th = theta * pow(0.5, (double)sa_level);
            if (!sa_prolongator_device(c, A, bdg.as<double>(), L.dinv64, L.rho, th, P, tick)) break;
        }
        tick(3);
        DMat R = transpose(c, P);
        tick(4);
        DMat AP = spgemm(c, A, P);
        DMat Ac = spgemm(c, R, AP);
        dm_release(c, AP);
        tick(5);
        AmgLevel& cur = h.lev.back();
        cur.P = as_csr(P);
        cur.R = as_csr(R);
        A = Ac;
    }
    // coarsest: dense inverse on the host
    const Csr& last = h.lev.back().A;
    const int64_t nc = last.n;
    if (nc > 6000) fail(MPET_ERR_INVALID, "AMG coarsest level too large for a dense solve");
    std::vector<int64_t> rp(nc + 1);
    std::vector<int32_t> ci(last.nnz);
    std::vector<double> v(last.nnz), dense((size_t)nc * nc, 0.0), inv;
    MPET_CUDA(cudaMemcpyAsync(rp.data(), last.rp, sizeof(int64_t) * (nc + 1), cudaMemcpyDeviceToHost, c->stream));
    if (last.nnz) {
        MPET_CUDA(cudaMemcpyAsync(ci.data(), last.ci, sizeof(int32_t) * last.nnz, cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaMemcpyAsync(v.data(), last.v64, sizeof(double) * last.nnz, cudaMemcpyDeviceToHost, c->stream));
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    for (int64_t i = 0; i < nc; ++i)
        for (int64_t e = rp[i]; e < rp[i + 1]; ++e) dense[i * nc + ci[e]] = v[e];
    if (!cholesky_inverse(dense, nc, inv)) fail(MPET_ERR_INVALID, "AMG coarsest operator is not positive definite");
    h.ncoarse = nc;
    h.cinv = c->pool.alloc<double>(nc * nc);
    MPET_CUDA(cudaMemcpyAsync(h.cinv, inv.data(), sizeof(double) * nc * nc, cudaMemcpyHostToDevice, c->stream));
    tick(6);
    const auto t1 = clk::now();
    finish_device_hier(c, h, nvec, fp32);
    tick(7);
    ms[0] = std::chrono::duration<double, std::milli>(t1 - t0).count();
    ms[1] = std::chrono::duration<double, std::milli>(clk::now() - t1).count();
}

}  // namespace mpet
