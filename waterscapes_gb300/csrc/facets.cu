// Boundary-facet terms of the MPET forms:
//   traction   (s, v)_{ds_m(1)}                       in L0 at t1   (mpetsolver.py:233)
//   flux       dt (I_a, q_a)_{ds_a(1)}                in L1 at t_theta (:249)
//   Robin      lhs: -dt theta (beta_a p_a, q_a)_{ds_a(2)} added to A (:252-253, :336-338)
//              rhs: dt (1-theta) (beta p^n, q) - dt (beta p_robin, q)  in L1 (:254)
// Data are Lagrange interpolants on each facet (P2 for the traction, which
// may depend on the facet normal; P1 for I, beta, p_robin), integrated
// exactly with the triangle tables below.
//
// Accumulation is an owner gather: every boundary node sums the
// contributions of its facets in ascending facet order (incidence built
// once from sorted keys), so no two threads write the same entry and the
// result is deterministic.
#include <cub/cub.cuh>

#include "mpet_internal.cuh"

namespace mpet {

typedef unsigned long long u64;

// int phi_i phi_j / |F| for P2 on a triangle, times 180 (vertices, then
// edges (1,2), (0,2), (0,1))
__constant__ double c_fm2[6][6] = {{6, -1, -1, -4, 0, 0},  {-1, 6, -1, 0, -4, 0},  {-1, -1, 6, 0, 0, -4},
                                   {-4, 0, 0, 32, 16, 16}, {0, -4, 0, 16, 32, 16}, {0, 0, -4, 16, 16, 32}};
// int lambda_v lambda_w lambda_m / |F|, times 60
__constant__ double c_ft1[3][3][3] = {{{6, 2, 2}, {2, 2, 1}, {2, 1, 2}},
                                      {{2, 2, 1}, {2, 6, 2}, {1, 2, 2}},
                                      {{2, 1, 2}, {1, 2, 2}, {2, 2, 6}}};
// 2D boundary facets are segments: int phi_i phi_j / |F| for P2 (vertices, midpoint), times 30,
// and int lambda_v lambda_w lambda_m / |F|, times 12
__constant__ double c_sm2[3][3] = {{4, -1, 2}, {-1, 4, 2}, {2, 2, 16}};
__constant__ double c_st1[2][2][2] = {{{3, 1}, {1, 1}}, {{1, 1}, {1, 3}}};

// Facet tables of the P2 / P1 pair: P2 mass, P1 mass (1 + delta) factor and P1 triple
// products, each divided by |F|.
template <int D>
__device__ __forceinline__ double fm2(int i, int j) { return D == 3 ? c_fm2[i][j] / 180.0 : c_sm2[i][j] / 30.0; }
template <int D>
__device__ __forceinline__ double fm1(int v, int w) { return (v == w ? 2.0 : 1.0) / (D == 3 ? 12.0 : 6.0); }
template <int D>
__device__ __forceinline__ double ft1(int v, int w, int m) {
    return D == 3 ? c_ft1[v][w][m] / 60.0 : c_st1[v][w][m] / 12.0;
}

static inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    return (int)(g < 1 ? 1 : (g > 2147483647LL ? 2147483647LL : g));
}

__device__ __forceinline__ int64_t lb_u64(const u64* a, int64_t n, u64 key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int lb_i32f(const int32_t* a, int n, int32_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// facet P2 nodes, area and outward unit normal (owner cell found through the
// cells of the facet's first vertex)
__global__ void k_facet_geometry(int64_t nf, const int32_t* __restrict__ bf, const double* __restrict__ x,
                                 const int32_t* __restrict__ cells, const int64_t* __restrict__ inc_ptr,
                                 const int32_t* __restrict__ inc, const u64* __restrict__ ekey, int64_t ne,
                                 int64_t nv, int32_t* fnodes, double* geo) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int32_t v[3] = {bf[3 * f], bf[3 * f + 1], bf[3 * f + 2]};
    // ascending vertex order (the facet's local numbering)
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2 - i; ++j)
            if (v[j] > v[j + 1]) {
                const int32_t t = v[j];
                v[j] = v[j + 1];
                v[j + 1] = t;
            }
    const int pr[3][2] = {{1, 2}, {0, 2}, {0, 1}};
    for (int k = 0; k < 3; ++k) fnodes[6 * f + k] = v[k];
    for (int k = 0; k < 3; ++k) {
        const u64 key = (u64)v[pr[k][0]] * (u64)nv + (u64)v[pr[k][1]];
        fnodes[6 * f + 3 + k] = (int32_t)(nv + lb_u64(ekey, ne, key));
    }
    int32_t opp = v[0];
    for (int64_t it = inc_ptr[v[0]]; it < inc_ptr[v[0] + 1]; ++it) {
        const int64_t c = inc[it] >> 4;
        int hit = 0, other = -1;
        for (int q = 0; q < 4; ++q) {
            const int32_t w = cells[4 * c + q];
            if (w == v[0] || w == v[1] || w == v[2]) ++hit; else other = w;
        }
        if (hit == 3) {
            opp = other;
            break;
        }
    }
    double p[3][3], o[3];
    for (int k = 0; k < 3; ++k) {
        for (int d = 0; d < 3; ++d) p[k][d] = x[3 * (int64_t)v[k] + d];
        o[k] = x[3 * (int64_t)opp + k];
    }
    const double e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    const double e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
    double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        n[d] /= len;
        s += n[d] * ((p[0][d] + p[1][d] + p[2][d]) / 3.0 - o[d]);
    }
    if (s < 0.0)
        for (int d = 0; d < 3; ++d) n[d] = -n[d];
    geo[4 * f] = 0.5 * len;
    for (int d = 0; d < 3; ++d) geo[4 * f + 1 + d] = n[d];
}

// segments of a triangle mesh: vertices ascending, then the edge node; length
// and outward unit normal (x, y; z slot 0)
__global__ void k_facet_geometry2(int64_t nf, const int32_t* __restrict__ bf, const double* __restrict__ x,
                                  const int32_t* __restrict__ cells, const int64_t* __restrict__ inc_ptr,
                                  const int32_t* __restrict__ inc, const u64* __restrict__ ekey, int64_t ne,
                                  int64_t nv, int32_t* fnodes, double* geo) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int32_t v0 = bf[2 * f], v1 = bf[2 * f + 1];
    if (v0 > v1) {
        const int32_t t = v0;
        v0 = v1;
        v1 = t;
    }
    fnodes[6 * f] = v0;
    fnodes[6 * f + 1] = v1;
    fnodes[6 * f + 2] = (int32_t)(nv + lb_u64(ekey, ne, (u64)v0 * (u64)nv + (u64)v1));
    fnodes[6 * f + 3] = fnodes[6 * f + 4] = fnodes[6 * f + 5] = -1;
    int32_t opp = v0;
    for (int64_t it = inc_ptr[v0]; it < inc_ptr[v0 + 1]; ++it) {
        const int64_t c = inc[it] >> 4;
        int hit = 0, other = -1;
        for (int q = 0; q < 3; ++q) {
            const int32_t w = cells[3 * c + q];
            if (w == v0 || w == v1) ++hit; else other = w;
        }
        if (hit == 2) {
            opp = other;
            break;
        }
    }
    const double px = x[3 * (int64_t)v1] - x[3 * (int64_t)v0], py = x[3 * (int64_t)v1 + 1] - x[3 * (int64_t)v0 + 1];
    const double len = sqrt(px * px + py * py);
    double n[2] = {py / len, -px / len};
    const double mx = 0.5 * (x[3 * (int64_t)v0] + x[3 * (int64_t)v1]) - x[3 * (int64_t)opp];
    const double my = 0.5 * (x[3 * (int64_t)v0 + 1] + x[3 * (int64_t)v1 + 1]) - x[3 * (int64_t)opp + 1];
    if (n[0] * mx + n[1] * my < 0.0) {
        n[0] = -n[0];
        n[1] = -n[1];
    }
    geo[4 * f] = len;
    geo[4 * f + 1] = n[0];
    geo[4 * f + 2] = n[1];
    geo[4 * f + 3] = 0.0;
}

__global__ void k_facet_keys(int64_t nf, int fn, const int32_t* __restrict__ fnodes, u64* keys) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nf * fn) return;
    const int64_t f = i / fn;
    const int m = (int)(i % fn);
    keys[i] = ((u64)fnodes[6 * f + m] << 32) | (u64)(f * 8 + m);
}

__global__ void k_ptr_u64(const u64* __restrict__ keys, int64_t nkeys, int64_t nrows, int64_t* ptr) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i > nrows) return;
    ptr[i] = lb_u64(keys, nkeys, (u64)i << 32);
}

__global__ void k_low32(const u64* __restrict__ keys, int64_t n, int32_t* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int32_t)(keys[i] & 0xffffffffULL);
}

void build_facets(mpet_ctx* c) {
    cudaStream_t s = c->stream;
    const int64_t nf = c->nf;
    if (nf == 0) return;
    if (nf >= (1LL << 28)) fail(MPET_ERR_INVALID, "too many boundary facets (limit 2^28)");
    c->fnodes = c->pool.alloc<int32_t>(nf * 6);
    c->fgeo = c->pool.alloc<double>(nf * 4);
    if (c->dim == 2)
        k_facet_geometry2<<<grid_for(nf, 128), 128, 0, s>>>(nf, c->bfacets, c->x, c->cells, c->inc_ptr, c->inc,
                                                            (const u64*)c->edge_key, c->ne, c->nv, c->fnodes,
                                                            c->fgeo);
    else
        k_facet_geometry<<<grid_for(nf, 128), 128, 0, s>>>(nf, c->bfacets, c->x, c->cells, c->inc_ptr, c->inc,
                                                           (const u64*)c->edge_key, c->ne, c->nv, c->fnodes,
                                                           c->fgeo);
    MPET_CHECK_LAUNCH();
    const int fn = c->dim == 2 ? 3 : 6;
    const int64_t nk = nf * fn;
    u64* keys = c->pool.alloc<u64>(nk);
    u64* sorted = c->pool.alloc<u64>(nk);
    k_facet_keys<<<grid_for(nk, 256), 256, 0, s>>>(nf, fn, c->fnodes, keys);
    MPET_CHECK_LAUNCH();
    size_t tb = 0;
    MPET_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, sorted, (int)nk, 0, 64, s));
    void* tmp = c->pool.alloc<unsigned char>((int64_t)tb);
    MPET_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tb, keys, sorted, (int)nk, 0, 64, s));
    c->bn_ptr = c->pool.alloc<int64_t>(c->nnodes + 1);
    c->bn_list = c->pool.alloc<int32_t>(nk);
    k_ptr_u64<<<grid_for(c->nnodes + 1, 256), 256, 0, s>>>(sorted, nk, c->nnodes, c->bn_ptr);
    k_low32<<<grid_for(nk, 256), 256, 0, s>>>(sorted, nk, c->bn_list);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(s));
    c->pool.release(tmp);
    c->pool.release(keys);
    c->pool.release(sorted);
}

struct FacetRhsArgs {
    int64_t nnodes, nv, Nu, nf;
    int J;
    const int64_t* bn_ptr;
    const int32_t* bn_list;
    const int32_t* fnodes;
    const double* fgeo;
    const int32_t* markers;  // (1 + J) x nf
    const double* traction;  // nf x FN x D (facet P2 nodes, components)
    const double* flux;      // J x nf x FV (facet vertices)
    const double* beta;      // J x nf x FV (at t_theta)
    const double* probin;    // J x nf x FV
    const double* up;        // previous state
    double* b;
    double dt, theta;
};

template <int D>
__global__ void k_facet_rhs(FacetRhsArgs A) {
    constexpr int FV = Simplex<D>::FV, FN = Simplex<D>::FN;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= A.nnodes) return;
    const int64_t q0 = A.bn_ptr[i], q1 = A.bn_ptr[i + 1];
    if (q0 == q1) return;
    double bu[3] = {0.0, 0.0, 0.0};
    double bp[MPET_MAX_NETWORKS];
    for (int a = 0; a < A.J; ++a) bp[a] = 0.0;
    for (int64_t q = q0; q < q1; ++q) {
        const int64_t f = A.bn_list[q] >> 3;
        const int m = A.bn_list[q] & 7;
        const double area = A.fgeo[4 * f];
        if (A.traction && A.markers[f] == 1) {
            const double* sv = A.traction + FN * D * f;
            for (int j = 0; j < FN; ++j) {
                const double w = area * fm2<D>(m, j);
                for (int k = 0; k < D; ++k) bu[k] += w * sv[D * j + k];
            }
        }
        if (i < A.nv && m < FV) {
            const int32_t* fv = A.fnodes + 6 * f;
            for (int a = 0; a < A.J; ++a) {
                const int mk = A.markers[(int64_t)(1 + a) * A.nf + f];
                if (mk == 1 && A.flux) {
                    const double* Iv = A.flux + ((int64_t)a * A.nf + f) * FV;
                    for (int w = 0; w < FV; ++w) bp[a] += A.dt * area * fm1<D>(m, w) * Iv[w];
                } else if (mk == 2 && A.beta) {
                    const double* bv = A.beta + ((int64_t)a * A.nf + f) * FV;
                    const double* pr = A.probin ? A.probin + ((int64_t)a * A.nf + f) * FV : nullptr;
                    const double* pa = A.up + A.Nu + (int64_t)a * A.nv;
                    for (int v = 0; v < FV; ++v)
                        for (int w = 0; w < FV; ++w) {
                            const double t = area * ft1<D>(v, w, m) * bv[v];
                            bp[a] += A.dt * (1.0 - A.theta) * t * pa[fv[w]];
                            if (pr) bp[a] -= A.dt * t * pr[w];
                        }
                }
            }
        }
    }
    for (int k = 0; k < D; ++k) A.b[D * i + k] += bu[k];
    if (i < A.nv)
        for (int a = 0; a < A.J; ++a) A.b[A.Nu + (int64_t)a * A.nv + i] += bp[a];
}

void launch_facet_rhs(mpet_ctx* c, double dt, const double* up_prev, double* b) {
    if (c->nf == 0 || !c->bn_ptr) return;
    if (!c->f_traction && !c->f_flux && !c->f_beta) return;
    FacetRhsArgs A{};
    A.nnodes = c->nnodes;
    A.nv = c->nv;
    A.Nu = c->Nu;
    A.nf = c->nf;
    A.J = c->J;
    A.bn_ptr = c->bn_ptr;
    A.bn_list = c->bn_list;
    A.fnodes = c->fnodes;
    A.fgeo = c->fgeo;
    A.markers = c->markers;
    A.traction = c->f_traction;
    A.flux = c->f_flux;
    A.beta = c->f_beta;
    A.probin = c->f_probin;
    A.up = up_prev;
    A.b = b;
    A.dt = dt;
    A.theta = c->prm.theta;
    if (c->dim == 2) k_facet_rhs<2><<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A);
    else k_facet_rhs<3><<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A);
    MPET_CHECK_LAUNCH();
}

// Robin matrix: row of p_a at boundary vertex i gains
// -dt theta sum_f |F| sum_v beta_v T[v][m][w] at column p_a(w).
template <int D>
__global__ void k_robin_matrix(int64_t nv, int64_t Nu, int64_t nf, int J, const int64_t* __restrict__ bn_ptr,
                               const int32_t* __restrict__ bn_list, const int32_t* __restrict__ fnodes,
                               const double* __restrict__ fgeo, const int32_t* __restrict__ markers,
                               const double* __restrict__ beta, const int64_t* __restrict__ row_ptr,
                               const int64_t* __restrict__ n2_ptr, const int64_t* __restrict__ n1_ptr,
                               const int32_t* __restrict__ n1_col, const uint8_t* __restrict__ dof_bc, double* v64,
                               float* v32, double* dinv, double dt_theta) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int64_t q0 = bn_ptr[i], q1 = bn_ptr[i + 1];
    if (q0 == q1) return;
    const int64_t s1 = n1_ptr[i];
    const int d1 = (int)(n1_ptr[i + 1] - s1);
    const int d2 = (int)(n2_ptr[i + 1] - n2_ptr[i]);
    for (int a = 0; a < J; ++a) {
        const int64_t row = Nu + (int64_t)a * nv + i;
        if (dof_bc[row]) continue;  // Dirichlet rows stay unit rows
        constexpr int FV = Simplex<D>::FV;
        const int64_t base = row_ptr[row] + D * (int64_t)d2 + (int64_t)a * d1;
        bool touched = false;
        for (int64_t q = q0; q < q1; ++q) {
            const int64_t f = bn_list[q] >> 3;
            const int m = bn_list[q] & 7;
            if (m >= FV || markers[(int64_t)(1 + a) * nf + f] != 2) continue;
            const double area = fgeo[4 * f];
            const double* bv = beta + ((int64_t)a * nf + f) * FV;
            for (int w = 0; w < FV; ++w) {
                double t = 0.0;
                for (int v = 0; v < FV; ++v) t += bv[v] * ft1<D>(v, m, w);
                const int64_t pos = base + lb_i32f(n1_col + s1, d1, fnodes[6 * f + w]);
                v64[pos] += -dt_theta * area * t;
                if (v32) v32[pos] = (float)v64[pos];
            }
            touched = true;
        }
        if (touched) {
            const double dg = fabs(v64[base + lb_i32f(n1_col + s1, d1, (int32_t)i)]);
            dinv[row] = dg > 0.0 ? 1.0 / dg : 1.0;
        }
    }
}

void launch_robin_matrix(mpet_ctx* c, double dt) {
    if (c->nf == 0 || !c->bn_ptr || !c->f_beta_matrix) return;
    auto kern = c->dim == 2 ? k_robin_matrix<2> : k_robin_matrix<3>;
    kern<<<grid_for(c->nv, 128), 128, 0, c->stream>>>(
        c->nv, c->Nu, c->nf, c->J, c->bn_ptr, c->bn_list, c->fnodes, c->fgeo, c->markers, c->f_beta_matrix,
        c->A.rp, c->n2_ptr, c->n1_ptr, c->n1_col, c->dof_bc, c->A.v64, c->A.v32, c->dinv, dt * c->prm.theta);
    MPET_CHECK_LAUNCH();
}

}  // namespace mpet
