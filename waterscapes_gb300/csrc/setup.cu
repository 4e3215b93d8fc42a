// Dofmap, adjacency, CSR sparsity pattern and Dirichlet DOF lists, all
// built on the GPU once per mesh.
//
// The pattern follows DOLFIN's SparsityPatternBuilder as used by
// assemble(self.a) in src/mpet/mpet/mpetsolver.py:335: for every cell the
// dense block over all (30 + 4J) mixed DOFs is inserted, so a row of a P2
// node i holds every displacement DOF of every P2 node sharing a cell with
// i, followed by every pressure DOF of every vertex sharing a cell with i
// (network-major).  Columns are ascending because displacement DOFs come
// first and each list is sorted.
//
// Everything is derived from sorted 64-bit keys (radix sort + unique), which
// keeps the construction deterministic.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "mpet_internal.cuh"

namespace mpet {

typedef unsigned long long u64;


static inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > 2147483647LL) g = 2147483647LL;
    return (int)(g < 1 ? 1 : g);
}

__device__ __forceinline__ int64_t lower_bound_u64(const u64* a, int64_t n, u64 key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int lower_bound_i32(const int32_t* a, int n, int32_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Sort keys in place (ping-pong through a temporary) and keep the unique
// ones; returns a freshly allocated exact-size array from the pool.
static int64_t sort_unique(mpet_ctx* c, u64* keys, int64_t n, int end_bit, u64** out_keys) {
    if (n > 2147483647LL) fail(MPET_ERR_INVALID, "too many adjacency keys for one radix sort");
    int ni = (int)n;
    TmpBuf sorted(sizeof(u64) * (size_t)n);
    size_t tb = 0;
    MPET_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, sorted.as<u64>(), ni, 0, end_bit, c->stream));
    {
        TmpBuf tmp(tb);
        MPET_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, tb, keys, sorted.as<u64>(), ni, 0, end_bit, c->stream));
    }
    TmpBuf nsel(sizeof(int64_t));
    tb = 0;
    MPET_CUDA(cub::DeviceSelect::Unique(nullptr, tb, sorted.as<u64>(), keys, nsel.as<int64_t>(), ni, c->stream));
    {
        TmpBuf tmp(tb);
        MPET_CUDA(cub::DeviceSelect::Unique(tmp.p, tb, sorted.as<u64>(), keys, nsel.as<int64_t>(), ni, c->stream));
    }
    int64_t cnt = 0;
    MPET_CUDA(cudaMemcpyAsync(&cnt, nsel.p, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    u64* o = c->pool.alloc<u64>(cnt);
    MPET_CUDA(cudaMemcpyAsync(o, keys, sizeof(u64) * cnt, cudaMemcpyDeviceToDevice, c->stream));
    *out_keys = o;
    return cnt;
}

static int bits_for(u64 maxval) {
    int b = 1;
    while (b < 64 && (maxval >> b) != 0) ++b;
    return b;
}

// --- kernels ------------------------------------------------------------------

template <int D>
__global__ void k_edge_keys(const int32_t* __restrict__ cells, int64_t nc, int64_t nv, u64* keys) {
    constexpr int NV = Simplex<D>::NV, NE = Simplex<D>::NE;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nc * NE) return;
    int64_t c = idx / NE;
    int e = (int)(idx % NE);
    int64_t a = cells[NV * c + edge_end<D>(e, 0)];
    int64_t b = cells[NV * c + edge_end<D>(e, 1)];
    int64_t lo = a < b ? a : b, hi = a < b ? b : a;
    keys[idx] = (u64)(lo * nv + hi);
}

template <int D>
__global__ void k_cell_nodes(const int32_t* __restrict__ cells, int64_t nc, int64_t nv,
                             const u64* __restrict__ ekey, int64_t ne, int32_t* cell_nodes) {
    constexpr int NV = Simplex<D>::NV, NN = Simplex<D>::NN;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nc * NN) return;
    int64_t c = idx / NN;
    int j = (int)(idx % NN);
    if (j < NV) {
        cell_nodes[idx] = cells[NV * c + j];
        return;
    }
    int e = j - NV;
    int64_t a = cells[NV * c + edge_end<D>(e, 0)];
    int64_t b = cells[NV * c + edge_end<D>(e, 1)];
    int64_t lo = a < b ? a : b, hi = a < b ? b : a;
    int64_t pos = lower_bound_u64(ekey, ne, (u64)(lo * nv + hi));
    cell_nodes[idx] = (int32_t)(nv + pos);
}

// Triangles: gradients of the barycentric coordinates (x, y in slots 3r, 3r+1
// of the 16-double record, z slot 0) and the area in slot 12.
__global__ void k_geometry2(const double* __restrict__ x, const int32_t* __restrict__ cells, int64_t nc,
                            double* geo) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double p[3][2];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 2; ++k) p[i][k] = x[3 * (int64_t)cells[3 * c + i] + k];
    const double e1[2] = {p[1][0] - p[0][0], p[1][1] - p[0][1]};
    const double e2[2] = {p[2][0] - p[0][0], p[2][1] - p[0][1]};
    const double det = e1[0] * e2[1] - e1[1] * e2[0];
    const double id = 1.0 / det;
    // rows of the inverse Jacobian: grad lambda_1 = ( e2y, -e2x)/det, grad lambda_2 = (-e1y, e1x)/det
    double* g = geo + 16 * c;
    for (int q = 0; q < 16; ++q) g[q] = 0.0;
    g[3] = e2[1] * id;
    g[4] = -e2[0] * id;
    g[6] = -e1[1] * id;
    g[7] = e1[0] * id;
    g[0] = -(g[3] + g[6]);
    g[1] = -(g[4] + g[7]);
    g[12] = fabs(det) / 2.0;
}

__global__ void k_geometry(const double* __restrict__ x, const int32_t* __restrict__ cells, int64_t nc,
                           double* geo) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double p[4][3];
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 3; ++k) p[i][k] = x[3 * (int64_t)cells[4 * c + i] + k];
    double e1[3], e2[3], e3[3];
    for (int k = 0; k < 3; ++k) {
        e1[k] = p[1][k] - p[0][k];
        e2[k] = p[2][k] - p[0][k];
        e3[k] = p[3][k] - p[0][k];
    }
    double c23[3] = {e2[1] * e3[2] - e2[2] * e3[1], e2[2] * e3[0] - e2[0] * e3[2], e2[0] * e3[1] - e2[1] * e3[0]};
    double c31[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
    double c12[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    double det = e1[0] * c23[0] + e1[1] * c23[1] + e1[2] * c23[2];
    double id = 1.0 / det;
    double* g = geo + 16 * c;
    for (int k = 0; k < 3; ++k) {
        double b1 = c23[k] * id, b2 = c31[k] * id, b3 = c12[k] * id;
        g[3 + k] = b1;
        g[6 + k] = b2;
        g[9 + k] = b3;
        g[k] = -(b1 + b2 + b3);
    }
    g[12] = fabs(det) / 6.0;
    g[13] = g[14] = g[15] = 0.0;
}

template <int D>
__global__ void k_pairs_n2(const int32_t* __restrict__ cn, int64_t nc, int64_t nnodes, u64* keys) {
    constexpr int NN = Simplex<D>::NN;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nc * NN * NN) return;
    int64_t c = idx / (NN * NN);
    int r = (int)(idx % (NN * NN));
    int m = r / NN, j = r % NN;
    keys[idx] = (u64)cn[NN * c + m] * (u64)nnodes + (u64)cn[NN * c + j];
}

template <int D>
__global__ void k_pairs_n1(const int32_t* __restrict__ cn, const int32_t* __restrict__ cells, int64_t nc,
                           int64_t nv, u64* keys) {
    constexpr int NN = Simplex<D>::NN, NV = Simplex<D>::NV;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nc * NN * NV) return;
    int64_t c = idx / (NN * NV);
    int r = (int)(idx % (NN * NV));
    int m = r / NV, w = r % NV;
    keys[idx] = (u64)cn[NN * c + m] * (u64)nv + (u64)cells[NV * c + w];
}

template <int D>
__global__ void k_pairs_inc(const int32_t* __restrict__ cn, int64_t nc, u64* keys) {
    constexpr int NN = Simplex<D>::NN;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nc * NN) return;
    int64_t c = idx / NN;
    int m = (int)(idx % NN);
    keys[idx] = ((u64)cn[idx] << 32) | (u64)(c * 16 + m);
}

__global__ void k_ptr_from_keys(const u64* __restrict__ keys, int64_t nkeys, int64_t nrows, u64 stride,
                                int64_t* ptr) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i > nrows) return;
    ptr[i] = lower_bound_u64(keys, nkeys, (u64)i * stride);
}

__global__ void k_low_from_keys(const u64* __restrict__ keys, int64_t nkeys, u64 stride, int32_t* out) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= nkeys) return;
    out[p] = (int32_t)(keys[p] % stride);
}

__global__ void k_low32_from_keys(const u64* __restrict__ keys, int64_t nkeys, int32_t* out) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= nkeys) return;
    out[p] = (int32_t)(keys[p] & 0xffffffffULL);
}

__global__ void k_max_degree(const int64_t* __restrict__ ptr, int64_t n, int* out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicMax(out, (int)(ptr[i + 1] - ptr[i]));
}

template <int D>
__global__ void k_ranks(const int32_t* __restrict__ cn, const int32_t* __restrict__ cells, int64_t nc,
                        const int64_t* __restrict__ n2_ptr, const int32_t* __restrict__ n2_col,
                        const int64_t* __restrict__ n1_ptr, const int32_t* __restrict__ n1_col,
                        uint16_t* rank2, uint16_t* rank1) {
    constexpr int NN = Simplex<D>::NN, NV = Simplex<D>::NV, R2 = NN * NN, R1 = NN * NV;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nc * (R2 + R1)) return;
    int64_t c = idx / (R2 + R1);
    int r = (int)(idx % (R2 + R1));
    if (r < R2) {
        int m = r / NN, j = r % NN;
        int32_t i = cn[NN * c + m];
        int64_t s = n2_ptr[i];
        int d = (int)(n2_ptr[i + 1] - s);
        rank2[R2 * c + r] = (uint16_t)lower_bound_i32(n2_col + s, d, cn[NN * c + j]);
    } else {
        r -= R2;
        int m = r / NV, w = r % NV;
        int32_t i = cn[NN * c + m];
        int64_t s = n1_ptr[i];
        int d = (int)(n1_ptr[i + 1] - s);
        rank1[R1 * c + r] = (uint16_t)lower_bound_i32(n1_col + s, d, cells[NV * c + w]);
    }
}

__global__ void k_row_len(int64_t N, int64_t Nu, int64_t nv, int J, int dim, const int64_t* __restrict__ n2_ptr,
                          const int64_t* __restrict__ n1_ptr, int64_t* len) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r > N) return;
    if (r == N) {
        len[r] = 0;
        return;
    }
    int64_t node = r < Nu ? r / dim : (r - Nu) % nv;
    len[r] = dim * (n2_ptr[node + 1] - n2_ptr[node]) + (int64_t)J * (n1_ptr[node + 1] - n1_ptr[node]);
}

__global__ void k_fill_cols(int64_t N, int64_t Nu, int64_t nv, int J, int dim, const int64_t* __restrict__ row_ptr,
                            const int64_t* __restrict__ n2_ptr, const int32_t* __restrict__ n2_col,
                            const int64_t* __restrict__ n1_ptr, const int32_t* __restrict__ n1_col,
                            int32_t* col) {
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < N; r += nwarps) {
        int64_t node = r < Nu ? r / dim : (r - Nu) % nv;
        int64_t s2 = n2_ptr[node], s1 = n1_ptr[node];
        int d2 = (int)(n2_ptr[node + 1] - s2), d1 = (int)(n1_ptr[node + 1] - s1);
        int L = dim * d2 + J * d1;
        int64_t base = row_ptr[r];
        for (int e = lane; e < L; e += 32) {
            int32_t cidx;
            if (e < dim * d2) {
                cidx = dim * n2_col[s2 + e / dim] + e % dim;
            } else {
                int e2 = e - dim * d2;
                int a = e2 / d1;
                cidx = (int32_t)(Nu + (int64_t)a * nv + n1_col[s1 + e2 % d1]);
            }
            col[base + e] = cidx;
        }
    }
}

// a facet has D vertices and D(D-1)/2 edges (every vertex pair)
template <int D>
__global__ void k_bc_flags(const int32_t* __restrict__ bf, const int32_t* __restrict__ mk, int64_t nf, int J,
                           int64_t nv, const u64* __restrict__ ekey, int64_t ne, uint8_t* node_bc,
                           uint8_t* vert_bc) {
    int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int64_t v[D];
    for (int k = 0; k < D; ++k) v[k] = bf[D * f + k];
    if (mk[f] == 0) {
        for (int k = 0; k < D; ++k) node_bc[v[k]] = 1;
        for (int i = 0; i < D; ++i)
            for (int j = i + 1; j < D; ++j) {
                int64_t a = v[i], b = v[j];
                int64_t lo = a < b ? a : b, hi = a < b ? b : a;
                int64_t pos = lower_bound_u64(ekey, ne, (u64)(lo * nv + hi));
                if (pos < ne && ekey[pos] == (u64)(lo * nv + hi)) node_bc[nv + pos] = 1;
            }
    }
    for (int a = 0; a < J; ++a)
        if (mk[(int64_t)(1 + a) * nf + f] == 0)
            for (int k = 0; k < D; ++k) vert_bc[(int64_t)a * nv + v[k]] = 1;
}

__global__ void k_bc_dofs_u(const int32_t* __restrict__ nodes, int64_t n, int dim, int32_t* dofs, uint8_t* dof_bc) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < dim; ++k) {
        int32_t d = dim * nodes[i] + k;
        dofs[dim * i + k] = d;
        dof_bc[d] = 1;
    }
}

__global__ void k_bc_dofs_p(const int32_t* __restrict__ verts, int64_t n, int64_t base, int32_t* dofs,
                            uint8_t* dof_bc) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t d = (int32_t)(base + verts[i]);
    dofs[i] = d;
    dof_bc[d] = 1;
}

// --- host drivers -------------------------------------------------------------------

template <int D>
static void build_topology_d(mpet_ctx* c) {
    constexpr int NE = Simplex<D>::NE, NN = Simplex<D>::NN, NV = Simplex<D>::NV;
    cudaStream_t s = c->stream;
    const int T = 256;
    int64_t nc = c->nc, nv = c->nv;
    // edges
    {
        TmpBuf keys(sizeof(u64) * nc * NE);
        k_edge_keys<D><<<grid_for(nc * NE, T), T, 0, s>>>(c->cells, nc, nv, keys.as<u64>());
        MPET_CHECK_LAUNCH();
        u64* ek = nullptr;
        c->ne = sort_unique(c, keys.as<u64>(), nc * NE, bits_for((u64)nv * (u64)nv), &ek);
        c->edge_key = (int64_t*)ek;
    }
    c->nnodes = nv + c->ne;
    c->cell_nodes = c->pool.alloc<int32_t>(nc * NN);
    k_cell_nodes<D><<<grid_for(nc * NN, T), T, 0, s>>>(c->cells, nc, nv, (const u64*)c->edge_key, c->ne,
                                                     c->cell_nodes);
    MPET_CHECK_LAUNCH();
    c->geo = c->pool.alloc<double>(nc * 16);
    if (D == 3) k_geometry<<<grid_for(nc, T), T, 0, s>>>(c->x, c->cells, nc, c->geo);
    else k_geometry2<<<grid_for(nc, T), T, 0, s>>>(c->x, c->cells, nc, c->geo);
    MPET_CHECK_LAUNCH();
    int64_t nn = c->nnodes;
    // P2 node adjacency
    {
        TmpBuf keys(sizeof(u64) * nc * NN * NN);
        k_pairs_n2<D><<<grid_for(nc * NN * NN, T), T, 0, s>>>(c->cell_nodes, nc, nn, keys.as<u64>());
        MPET_CHECK_LAUNCH();
        u64* uk = nullptr;
        c->n2_nnz = sort_unique(c, keys.as<u64>(), nc * NN * NN, bits_for((u64)nn * (u64)nn), &uk);
        c->n2_ptr = c->pool.alloc<int64_t>(nn + 1);
        c->n2_col = c->pool.alloc<int32_t>(c->n2_nnz);
        k_ptr_from_keys<<<grid_for(nn + 1, T), T, 0, s>>>(uk, c->n2_nnz, nn, (u64)nn, c->n2_ptr);
        k_low_from_keys<<<grid_for(c->n2_nnz, T), T, 0, s>>>(uk, c->n2_nnz, (u64)nn, c->n2_col);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaStreamSynchronize(s));
        c->pool.release(uk);
    }
    // vertices adjacent to each node
    {
        TmpBuf keys(sizeof(u64) * nc * NN * NV);
        k_pairs_n1<D><<<grid_for(nc * NN * NV, T), T, 0, s>>>(c->cell_nodes, c->cells, nc, nv, keys.as<u64>());
        MPET_CHECK_LAUNCH();
        u64* uk = nullptr;
        c->n1_nnz = sort_unique(c, keys.as<u64>(), nc * NN * NV, bits_for((u64)nn * (u64)nv), &uk);
        c->n1_ptr = c->pool.alloc<int64_t>(nn + 1);
        c->n1_col = c->pool.alloc<int32_t>(c->n1_nnz);
        k_ptr_from_keys<<<grid_for(nn + 1, T), T, 0, s>>>(uk, c->n1_nnz, nn, (u64)nv, c->n1_ptr);
        k_low_from_keys<<<grid_for(c->n1_nnz, T), T, 0, s>>>(uk, c->n1_nnz, (u64)nv, c->n1_col);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaStreamSynchronize(s));
        c->pool.release(uk);
    }
    // node -> cell incidence (cells ascending within a node)
    {
        if (nc >= (1LL << 27)) fail(MPET_ERR_INVALID, "too many cells (limit 2^27: cell * 16 + local fits int32)");
        TmpBuf keys(sizeof(u64) * nc * NN);
        k_pairs_inc<D><<<grid_for(nc * NN, T), T, 0, s>>>(c->cell_nodes, nc, keys.as<u64>());
        MPET_CHECK_LAUNCH();
        u64* uk = nullptr;
        int64_t n = sort_unique(c, keys.as<u64>(), nc * NN, 32 + bits_for((u64)nn), &uk);
        if (n != nc * NN) fail(MPET_ERR_INVALID, "degenerate cell (repeated vertex)");
        c->inc_ptr = c->pool.alloc<int64_t>(nn + 1);
        c->inc = c->pool.alloc<int32_t>(n);
        k_ptr_from_keys<<<grid_for(nn + 1, T), T, 0, s>>>(uk, n, nn, 1ULL << 32, c->inc_ptr);
        k_low32_from_keys<<<grid_for(n, T), T, 0, s>>>(uk, n, c->inc);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaStreamSynchronize(s));
        c->pool.release(uk);
    }
    // degree limits of the 16-bit rank tables
    {
        TmpBuf mx(sizeof(int) * 2);
        MPET_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(int) * 2, s));
        k_max_degree<<<grid_for(nn, T), T, 0, s>>>(c->n2_ptr, nn, mx.as<int>());
        k_max_degree<<<grid_for(nn, T), T, 0, s>>>(c->inc_ptr, nn, mx.as<int>() + 1);
        MPET_CHECK_LAUNCH();
        int h[2];
        MPET_CUDA(cudaMemcpyAsync(h, mx.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        MPET_CUDA(cudaStreamSynchronize(s));
        if (h[0] >= 65535) fail(MPET_ERR_INVALID, "node degree too large for 16-bit ranks");
    }
    c->rank2 = c->pool.alloc<uint16_t>(nc * NN * NN);
    c->rank1 = c->pool.alloc<uint16_t>(nc * NN * NV);
    k_ranks<D><<<grid_for(nc * (NN * NN + NN * NV), T), T, 0, s>>>(c->cell_nodes, c->cells, nc, c->n2_ptr, c->n2_col, c->n1_ptr,
                                                 c->n1_col, c->rank2, c->rank1);
    MPET_CHECK_LAUNCH();
}

void build_topology(mpet_ctx* c) {
    if (c->dim == 2) build_topology_d<2>(c);
    else build_topology_d<3>(c);
}

void build_pattern(mpet_ctx* c) {
    cudaStream_t s = c->stream;
    const int T = 256;
    int J = c->J;
    c->Nu = (int64_t)c->dim * c->nnodes;
    c->N = c->Nu + (int64_t)J * c->nv;
    if (c->N >= 2147483647LL) fail(MPET_ERR_INVALID, "too many DOFs for 32-bit column ids");
    int64_t N = c->N;
    c->A.n = c->A.m = N;
    c->A.rp = c->pool.alloc<int64_t>(N + 1);
    {
        TmpBuf len(sizeof(int64_t) * (N + 1));
        k_row_len<<<grid_for(N + 1, T), T, 0, s>>>(N, c->Nu, c->nv, J, c->dim, c->n2_ptr, c->n1_ptr,
                                                   len.as<int64_t>());
        MPET_CHECK_LAUNCH();
        size_t tb = 0;
        MPET_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, len.as<int64_t>(), c->A.rp, (int)(N + 1), s));
        TmpBuf tmp(tb);
        MPET_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, len.as<int64_t>(), c->A.rp, (int)(N + 1), s));
    }
    MPET_CUDA(cudaMemcpyAsync(&c->nnz, c->A.rp + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MPET_CUDA(cudaStreamSynchronize(s));
    c->A.nnz = c->nnz;
    c->A.ci = c->pool.alloc<int32_t>(c->nnz);
    k_fill_cols<<<152 * 16, 256, 0, s>>>(N, c->Nu, c->nv, J, c->dim, c->A.rp, c->n2_ptr, c->n2_col, c->n1_ptr,
                                         c->n1_col, c->A.ci);
    MPET_CHECK_LAUNCH();
    c->A.lpr = choose_lpr(N, c->nnz);
    {
        std::vector<int64_t> rp(N + 1);
        MPET_CUDA(cudaMemcpyAsync(rp.data(), c->A.rp, sizeof(int64_t) * (N + 1), cudaMemcpyDeviceToHost, s));
        MPET_CUDA(cudaStreamSynchronize(s));
        build_tiles(c, c->A, rp.data());
    }
    // preconditioner block patterns: u-Laplacian on n2, P1 blocks on the vertex rows of n1
    c->Lu.n = c->Lu.m = c->nnodes;
    c->Lu.nnz = c->n2_nnz;
    c->Lu.rp = c->n2_ptr;
    c->Lu.ci = c->n2_col;
    c->Lu.lpr = choose_lpr(c->nnodes, c->n2_nnz);
    int64_t p1nnz = 0;
    MPET_CUDA(cudaMemcpyAsync(&p1nnz, c->n1_ptr + c->nv, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MPET_CUDA(cudaStreamSynchronize(s));
    for (int a = 0; a < J; ++a) {
        c->Pp[a].n = c->Pp[a].m = c->nv;
        c->Pp[a].nnz = p1nnz;
        c->Pp[a].rp = c->n1_ptr;
        c->Pp[a].ci = c->n1_col;
        c->Pp[a].lpr = choose_lpr(c->nv, p1nnz);
    }
}

static int64_t compact_flags(mpet_ctx* c, const uint8_t* flags, int64_t n, int32_t** out) {
    TmpBuf buf(sizeof(int32_t) * (n > 0 ? n : 1));
    TmpBuf nsel(sizeof(int));
    size_t tb = 0;
    thrust::counting_iterator<int32_t> it(0);
    MPET_CUDA(cub::DeviceSelect::Flagged(nullptr, tb, it, flags, buf.as<int32_t>(), nsel.as<int>(), (int)n, c->stream));
    {
        TmpBuf tmp(tb);
        MPET_CUDA(cub::DeviceSelect::Flagged(tmp.p, tb, it, flags, buf.as<int32_t>(), nsel.as<int>(), (int)n,
                                             c->stream));
    }
    int cnt = 0;
    MPET_CUDA(cudaMemcpyAsync(&cnt, nsel.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    int32_t* o = c->pool.alloc<int32_t>(cnt);
    if (cnt) MPET_CUDA(cudaMemcpyAsync(o, buf.p, sizeof(int32_t) * cnt, cudaMemcpyDeviceToDevice, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    *out = o;
    return cnt;
}

void build_bc(mpet_ctx* c) {
    cudaStream_t s = c->stream;
    const int T = 256;
    int J = c->J;
    c->node_bc = c->pool.alloc<uint8_t>(c->nnodes);
    c->vert_bc = c->pool.alloc<uint8_t>((int64_t)J * c->nv);
    c->dof_bc = c->pool.alloc<uint8_t>(c->N);
    MPET_CUDA(cudaMemsetAsync(c->node_bc, 0, c->nnodes, s));
    MPET_CUDA(cudaMemsetAsync(c->vert_bc, 0, (size_t)J * c->nv, s));
    MPET_CUDA(cudaMemsetAsync(c->dof_bc, 0, c->N, s));
    if (c->nf > 0) {
        if (c->dim == 2)
            k_bc_flags<2><<<grid_for(c->nf, T), T, 0, s>>>(c->bfacets, c->markers, c->nf, J, c->nv,
                                                            (const u64*)c->edge_key, c->ne, c->node_bc, c->vert_bc);
        else
            k_bc_flags<3><<<grid_for(c->nf, T), T, 0, s>>>(c->bfacets, c->markers, c->nf, J, c->nv,
                                                            (const u64*)c->edge_key, c->ne, c->node_bc, c->vert_bc);
        MPET_CHECK_LAUNCH();
    }
    c->nbc_nodes[0] = compact_flags(c, c->node_bc, c->nnodes, &c->bc_nodes[0]);
    for (int a = 0; a < J; ++a)
        c->nbc_nodes[1 + a] = compact_flags(c, c->vert_bc + (int64_t)a * c->nv, c->nv, &c->bc_nodes[1 + a]);
    c->bc_off[0] = 0;
    c->bc_off[1] = (int64_t)c->dim * c->nbc_nodes[0];
    for (int a = 0; a < J; ++a) c->bc_off[2 + a] = c->bc_off[1 + a] + c->nbc_nodes[1 + a];
    c->nbc_dofs = c->bc_off[1 + J];
    c->bc_dofs = c->pool.alloc<int32_t>(c->nbc_dofs);
    c->bc_vals = c->pool.alloc<double>(c->nbc_dofs);
    MPET_CUDA(cudaMemsetAsync(c->bc_vals, 0, sizeof(double) * (c->nbc_dofs > 0 ? c->nbc_dofs : 1), s));
    if (c->nbc_nodes[0])
        k_bc_dofs_u<<<grid_for(c->nbc_nodes[0], T), T, 0, s>>>(c->bc_nodes[0], c->nbc_nodes[0], c->dim,
                                                                c->bc_dofs, c->dof_bc);
    for (int a = 0; a < J; ++a)
        if (c->nbc_nodes[1 + a])
            k_bc_dofs_p<<<grid_for(c->nbc_nodes[1 + a], T), T, 0, s>>>(
                c->bc_nodes[1 + a], c->nbc_nodes[1 + a], c->Nu + (int64_t)a * c->nv, c->bc_dofs + c->bc_off[1 + a],
                c->dof_bc);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(s));
}

}  // namespace mpet
