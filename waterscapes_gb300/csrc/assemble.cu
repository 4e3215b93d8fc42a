// Element kernels of the MPET operator and right-hand side.
//
// Local tensors restate the forms of src/mpet/mpet/mpetsolver.py:196-201
// (a = lhs(F)) and :233, :249 (sources) for P2 vector displacement and P1
// pressures on affine tetrahedra, integrated exactly: P2 gradients are
// linear, so with g_{j,r} the value of grad(phi_j) at vertex r and
// s_j = sum_r g_{j,r},
//   int d_k phi_m d_l phi_j = |T|/20 (sum_r g_{m,r,k} g_{j,r,l} + s_{m,k} s_{j,l})
//   int lambda_w d_k phi_j  = |T|/20 (g_{j,w,k} + s_{j,k})
//   int lambda_v lambda_w   = |T|/20 (1 + delta_vw),   int grad lambda_v . grad lambda_w = |T| b_v . b_w.
//
// Assembly is a row-owner gather: one warp owns the displacement rows of a
// P2 node (and, for a vertex, its J pressure rows), walks the node's cells
// in ascending order and adds that node's row slice of each cell matrix at
// the CSR positions given by the per-cell rank tables.  Every value is
// written by exactly one warp in a fixed order, so the result is
// deterministic and needs neither atomics nor a cell colouring.
#include <string.h>

#include <algorithm>

#include "mpet_internal.cuh"

namespace mpet {

// int phi_i phi_j / |T| for P2 on a tetrahedron, times 420.
__constant__ double c_m2[10][10] = {
    {6, 1, 1, 1, -6, -6, -6, -4, -4, -4},     {1, 6, 1, 1, -6, -4, -4, -6, -6, -4},
    {1, 1, 6, 1, -4, -6, -4, -6, -4, -6},     {1, 1, 1, 6, -4, -4, -6, -4, -6, -6},
    {-6, -6, -4, -4, 32, 16, 16, 16, 16, 8},  {-6, -4, -6, -4, 16, 32, 16, 16, 8, 16},
    {-6, -4, -4, -6, 16, 16, 32, 8, 16, 16},  {-4, -6, -6, -4, 16, 16, 8, 32, 16, 16},
    {-4, -6, -4, -6, 16, 8, 16, 16, 32, 16},  {-4, -4, -6, -6, 8, 16, 16, 16, 16, 32}};
// int phi_i phi_j / |T| for P2 on a triangle, times 180 (vertices, then edges (1,2), (0,2), (0,1)).
__constant__ double c_m2t[6][6] = {{6, -1, -1, -4, 0, 0},  {-1, 6, -1, 0, -4, 0},  {-1, -1, 6, 0, 0, -4},
                                   {-4, 0, 0, 32, 16, 16}, {0, -4, 0, 16, 32, 16}, {0, 0, -4, 16, 16, 32}};

// int lambda_r lambda_s / |T| = (1 + delta_rs) * KAPPA(D), KAPPA = d! / (d + 2)!
template <int D>
__host__ __device__ constexpr double kappa() { return D == 3 ? 1.0 / 20.0 : 1.0 / 12.0; }

struct MatCoef {
    double mu, lmbda, dt_theta;
    int J;
    double alpha[MPET_MAX_NETWORKS], c[MPET_MAX_NETWORKS], K[MPET_MAX_NETWORKS];
    double S[MPET_MAX_NETWORKS * MPET_MAX_NETWORKS];  // row-major, stride 8
    double Ssum[MPET_MAX_NETWORKS];                   // sum_b S_ab
    const double* Kc;                                  // per-cell K (J x nc) or null
    const double* cc;                                  // per-cell c (J x nc) or null
    const double* Sc;                                  // per-cell S (J x J x nc) or null
    int64_t nc;
    double prec_mu;                                    // weight of the displacement preconditioner block
    double prec_shift;                                 // + prec_shift (u, v) in that block
    // Form-dependent coefficients.  MPET: cpl_a = -alpha_a in (p_a, div v) and (div u, q_a),
    // rhs_cu_a = -alpha_a on (div u^-, q_a), no rank-one term.  Total pressure: cpl = (1, 0, ..),
    // rhs_cu = 0, and the rank-one mass term -(beta_a beta_b / lmbda) (p_b, w_a), beta = alpha
    // with beta_0 = 1, whose previous-time part enters the network rows only (rank_rhs_0 = 0).
    double cpl[MPET_MAX_NETWORKS], rhs_cu[MPET_MAX_NETWORKS];
    double rank_b[MPET_MAX_NETWORKS], rank_rhs[MPET_MAX_NETWORKS], rank_inv;
    double prec_extra[MPET_MAX_NETWORKS];              // + prec_extra_a (p_a, w_a) in pressure block a
    // with scalar coefficients (no per-cell c, K, S): the pressure-pressure block of the
    // system is Cm_ab (p_b, w_a) + [a == b] Kd_a (grad p_a, grad w_a)
    int coef_const;
    double Cm[MPET_MAX_NETWORKS * MPET_MAX_NETWORKS], Kd[MPET_MAX_NETWORKS];
    __device__ __forceinline__ double Kof(int a, int64_t cell) const { return Kc ? Kc[a * nc + cell] : K[a]; }
    __device__ __forceinline__ double cof(int a, int64_t cell) const { return cc ? cc[a * nc + cell] : c[a]; }
    __device__ __forceinline__ double Sof(int a, int b, int64_t cell) const {
        return Sc ? Sc[((int64_t)a * J + b) * nc + cell] : S[a * MPET_MAX_NETWORKS + b];
    }
    __device__ __forceinline__ double Ssumof(int a, int64_t cell) const {
        if (!Sc) return Ssum[a];
        double s = 0.0;
        for (int b = 0; b < J; ++b) s += Sof(a, b, cell);
        return s;
    }
};

struct Geo {
    double b[4][3];
    double vol;
};

__device__ __forceinline__ void load_geo(const double* __restrict__ geo, int64_t c, Geo& G) {
    const double* g = geo + 16 * c;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int k = 0; k < 3; ++k) G.b[r][k] = g[3 * r + k];
    G.vol = g[12];
}

// g_{j,r} (value of grad phi_j at vertex r) for all r, and s_j = sum_r g_{j,r}
// (zero for a vertex of a tetrahedron, grad lambda_j for a vertex of a triangle).
template <int D = 3>
__device__ __forceinline__ void p2_grad_table(const Geo& G, int j, double g[4][3], double s[3]) {
    constexpr int NV = Simplex<D>::NV;
    if (j < NV) {
#pragma unroll
        for (int r = 0; r < NV; ++r) {
            double f = (r == j) ? 3.0 : -1.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) g[r][k] = f * G.b[j][k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) s[k] = D == 3 ? 0.0 : G.b[j][k];
    } else {
        int ea = edge_end<D>(j - NV, 0), eb = edge_end<D>(j - NV, 1);
#pragma unroll
        for (int r = 0; r < NV; ++r)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                g[r][k] = (r == ea ? 4.0 * G.b[eb][k] : 0.0) + (r == eb ? 4.0 * G.b[ea][k] : 0.0);
#pragma unroll
        for (int k = 0; k < 3; ++k) s[k] = 4.0 * (G.b[ea][k] + G.b[eb][k]);
    }
}

// value of grad phi_j at vertex r, plus s_j
template <int D = 3>
__device__ __forceinline__ void p2_grad_at(const Geo& G, int j, int r, double g[3], double s[3]) {
    constexpr int NV = Simplex<D>::NV;
    if (j < NV) {
        double f = (r == j) ? 3.0 : -1.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            g[k] = f * G.b[j][k];
            s[k] = D == 3 ? 0.0 : G.b[j][k];
        }
    } else {
        int ea = edge_end<D>(j - NV, 0), eb = edge_end<D>(j - NV, 1);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            g[k] = (r == ea ? 4.0 * G.b[eb][k] : 0.0) + (r == eb ? 4.0 * G.b[ea][k] : 0.0);
            s[k] = 4.0 * (G.b[ea][k] + G.b[eb][k]);
        }
    }
}

__device__ __forceinline__ int lb_i32(const int32_t* a, int n, int32_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

struct AsmArgs {
    int64_t nnodes, nv, Nu;
    const int64_t* row_ptr;
    const int64_t* n2_ptr;
    const int32_t* n2_col;
    const int64_t* n1_ptr;
    const int32_t* n1_col;
    const int64_t* inc_ptr;
    const int32_t* inc;
    const uint16_t* rank2;
    const uint16_t* rank1;
    const double* geo;
    const uint8_t* dof_bc;
    double* v64;
    float* v32;
    double* dinv;
    int apply_bc;
    const double* Mst;  // per-cell displacement blocks (k_elem_uu) or null
};

// Number of node pairs m <= j of a cell and the index of pair (m, j), m <= j.
template <int D>
__host__ __device__ constexpr int npairs() { return Simplex<D>::NN * (Simplex<D>::NN + 1) / 2; }
// doubles per cell of the staged element data: the displacement blocks, then the
// coupling values C[g][r][k] = |T| kappa (g_{g,r}[k] + s_g[k])
template <int D>
__host__ __device__ constexpr int elem_record() {
    return npairs<D>() * D * D + Simplex<D>::NN * Simplex<D>::NV * D;
}
template <int D>
__device__ __forceinline__ int pair_index(int m, int j) {
    return m * Simplex<D>::NN - m * (m - 1) / 2 + (j - m);
}

// The displacement blocks of one cell's element matrix, computed once per cell:
// with the Gram matrix M_mj[a][b] = |T| kappa (s_m[a] s_j[b] + sum_r g_{m,r}[a] g_{j,r}[b])
// = int dphi_m/dx_a dphi_j/dx_b, the block of rows (m, k) and columns (j, l) is
// B_mj[k][l] = mu M_mj[l][k] + lmbda M_mj[k][l] + [k == l] mu tr M_mj, stored for the
// node pairs m <= j, cell-major (B_jm = B_mj^T), followed by the u-p coupling values
// C[g][r][k] (node g, vertex r, component k).  The row-owner assembly reads them
// instead of recomputing them for every (row node, cell), which keeps the FP64 pipe
// (the bound of the assembly) to the unique work.
template <int D>
__global__ void __launch_bounds__(128) k_elem_uu(int64_t nc, const double* __restrict__ geo, double mu,
                                                 double lmbda, double* Mst) {
    constexpr int NN = Simplex<D>::NN, NV = Simplex<D>::NV, NP = npairs<D>(), DD = D * D;
    const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (cell >= nc) return;
    Geo G;
    load_geo(geo, cell, G);
    const double w20 = G.vol * kappa<D>();
    double* out = Mst + cell * (int64_t)elem_record<D>();
    for (int m = 0; m < NN; ++m) {
        double gm[4][3], sm[3];
        p2_grad_table<D>(G, m, gm, sm);
        double* cpl = out + NP * DD + m * NV * D;
#pragma unroll
        for (int r = 0; r < NV; ++r)
#pragma unroll
            for (int k = 0; k < D; ++k) cpl[r * D + k] = w20 * (gm[r][k] + sm[k]);
        for (int j = m; j < NN; ++j) {
            double gj[4][3], sj[3];
            p2_grad_table<D>(G, j, gj, sj);
            double* o = out + pair_index<D>(m, j) * DD;
            double M[3][3];
            double tr = 0.0;
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b = 0; b < D; ++b) {
                    double acc = sm[a] * sj[b];
#pragma unroll
                    for (int r = 0; r < NV; ++r) acc += gm[r][a] * gj[r][b];
                    M[a][b] = w20 * acc;
                }
#pragma unroll
            for (int a = 0; a < D; ++a) tr += M[a][a];
#pragma unroll
            for (int k = 0; k < D; ++k)
#pragma unroll
                for (int l = 0; l < D; ++l) {
                    double v = mu * M[l][k] + lmbda * M[k][l];
                    if (l == k) v += mu * tr;
                    o[k * D + l] = v;
                }
        }
    }
}

// Task layout of one (node, cell) pair over the warp's lanes: NN*D
// displacement-displacement entries (node j, component k), D*NV
// displacement-pressure couplings (k, vertex w), and for a vertex node
// NN*D pressure-displacement couplings (j, l) and NV pressure-pressure
// entries (w): 30/42/72/76 on tetrahedra, 12/18/30/33 on triangles.
template <int D>
__global__ void __launch_bounds__(256) k_assemble_matrix(AsmArgs A, MatCoef P) {
    constexpr int NV = Simplex<D>::NV, NN = Simplex<D>::NN;
    constexpr int X0 = (NN * D + 31) / 32 * 32;  // first coupling task
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int J = P.J;
    for (int64_t i = warp; i < A.nnodes; i += nwarps) {
        const bool isv = i < A.nv;
        const int64_t s2 = A.n2_ptr[i], s1 = A.n1_ptr[i];
        const int d2 = (int)(A.n2_ptr[i + 1] - s2), d1 = (int)(A.n1_ptr[i + 1] - s1);
        const int L = D * d2 + J * d1;
        const int nrows = D + (isv ? J : 0);
        int64_t rows[3 + MPET_MAX_NETWORKS];
        for (int k = 0; k < D; ++k) rows[k] = D * i + k;
        for (int a = 0; a < J; ++a) rows[D + a] = A.Nu + (int64_t)a * A.nv + i;
        int64_t rp[3 + MPET_MAX_NETWORKS];
        for (int q = 0; q < nrows; ++q) rp[q] = A.row_ptr[rows[q]];
        for (int q = 0; q < nrows; ++q)
            for (int e = lane; e < L; e += 32) A.v64[rp[q] + e] = 0.0;
        __syncwarp();
        for (int64_t it = A.inc_ptr[i]; it < A.inc_ptr[i + 1]; ++it) {
            const int32_t packed = A.inc[it];
            const int64_t cell = packed >> 4;
            const int m = packed & 15;
            Geo G;
            load_geo(A.geo, cell, G);
            const double w20 = G.vol * kappa<D>();
            const uint16_t* rk2 = A.rank2 + cell * (NN * NN) + m * NN;
            const uint16_t* rk1 = A.rank1 + cell * (NN * NV) + m * NV;
            // Lane tasks in class-aligned rounds of 32 (a round runs every branch any of its
            // lanes takes): first the NN*D displacement (node j, row k) tasks; then the
            // u-p coupling tasks (u row k with vertex w, and for vertex rows the p rows with
            // node j, component l); then for vertex rows the (network a, vertex w) pressure tasks.
            const int nx = D * NV + (isv ? NN * D : 0);
            const int ntask = X0 + nx + (isv ? J * NV : 0);
            for (int t = lane; t < ntask; t += 32) {
                if (t < X0) {
                    if (t >= NN * D) continue;
                    const int j = t / D, k = t % D;
                    const int64_t base = rp[k] + D * (int64_t)rk2[j];
                    if (A.Mst) {
                        // row k of B_mj (stored, or the transpose of the stored B_jm)
                        constexpr int DD = D * D;
                        const double* src = A.Mst + cell * (int64_t)elem_record<D>();
                        const bool up = m <= j;
                        src += pair_index<D>(up ? m : j, up ? j : m) * DD;
#pragma unroll
                        for (int l = 0; l < D; ++l) A.v64[base + l] += src[up ? k * D + l : l * D + k];
                        continue;
                    }
                    double M[3][3];
                    {
                        double gm[4][3], sm[3], gj[4][3], sj[3];
                        p2_grad_table<D>(G, m, gm, sm);
                        p2_grad_table<D>(G, j, gj, sj);
#pragma unroll
                        for (int a = 0; a < D; ++a)
#pragma unroll
                            for (int b = 0; b < D; ++b) {
                                double acc = sm[a] * sj[b];
#pragma unroll
                                for (int r = 0; r < NV; ++r) acc += gm[r][a] * gj[r][b];
                                M[a][b] = w20 * acc;
                            }
                    }
                    double tr = 0.0;
#pragma unroll
                    for (int a = 0; a < D; ++a) tr += M[a][a];
#pragma unroll
                    for (int l = 0; l < D; ++l) {
                        double v = P.mu * M[l][k] + P.lmbda * M[k][l];
                        if (l == k) v += P.mu * tr;
                        A.v64[base + l] += v;
                    }
                } else if (t < X0 + nx) {
                    // coupling value w20 (grad phi_node at vertex + s_node)[comp]: u row k with
                    // vertex w (node m at vertex w), or p rows with node j (node j at vertex m)
                    const int x = t - X0;
                    const bool urow = x < D * NV;
                    const int y = x - D * NV;
                    const int gnode = urow ? m : y / D;
                    const int gvert = urow ? x % NV : m;
                    const int comp = urow ? x / NV : y % D;
                    double C;
                    if (A.Mst) {
                        C = A.Mst[cell * (int64_t)elem_record<D>() + npairs<D>() * D * D + (gnode * NV + gvert) * D + comp];
                    } else {
                        double g[3], sg[3];
                        p2_grad_at<D>(G, gnode, gvert, g, sg);
                        C = w20 * (g[comp] + sg[comp]);
                    }
                    for (int a = 0; a < J; ++a) {
                        const int64_t pos = urow ? rp[comp] + D * (int64_t)d2 + (int64_t)a * d1 + rk1[gvert]
                                                 : rp[D + a] + D * (int64_t)rk2[gnode] + comp;
                        A.v64[pos] += P.cpl[a] * C;
                    }
                } else {
                    const int q = t - X0 - nx, a = q / NV, w = q % NV;
                    const double M1 = w20 * (m == w ? 2.0 : 1.0);
                    const double L1 = G.vol * (G.b[m][0] * G.b[w][0] + G.b[m][1] * G.b[w][1] + G.b[m][2] * G.b[w][2]);
                    const int64_t base = rp[D + a] + D * (int64_t)d2 + rk1[w];
                    if (P.coef_const) {
                        for (int b = 0; b < J; ++b) {
                            double v = P.Cm[a * MPET_MAX_NETWORKS + b] * M1;
                            if (a == b) v += P.Kd[a] * L1;
                            A.v64[base + (int64_t)b * d1] += v;
                        }
                    } else {
                        for (int b = 0; b < J; ++b) {
                            double v = -(P.dt_theta * ((a == b ? P.Ssumof(a, cell) : 0.0) - P.Sof(a, b, cell)) +
                                         P.rank_inv * P.rank_b[a] * P.rank_b[b]) * M1;
                            if (a == b) v += -P.cof(a, cell) * M1 - P.dt_theta * P.Kof(a, cell) * L1;
                            A.v64[base + (int64_t)b * d1] += v;
                        }
                    }
                }
            }
            __syncwarp();
        }
        // Dirichlet rows (DirichletBC.apply(A): zero row, unit diagonal)
        int self2 = lb_i32(A.n2_col + s2, d2, (int32_t)i);
        int self1 = isv ? lb_i32(A.n1_col + s1, d1, (int32_t)i) : 0;
        for (int q = 0; q < nrows; ++q) {
            const int64_t dpos = q < D ? rp[q] + D * self2 + q : rp[q] + D * (int64_t)d2 + (int64_t)(q - D) * d1 + self1;
            if (A.apply_bc && A.dof_bc[rows[q]]) {
                for (int e = lane; e < L; e += 32) A.v64[rp[q] + e] = 0.0;
                __syncwarp();
                if (lane == 0) A.v64[dpos] = 1.0;
                __syncwarp();
            }
            if (lane == 0) {
                double dg = fabs(A.v64[dpos]);
                A.dinv[rows[q]] = dg > 0.0 ? 1.0 / dg : 1.0;
            }
        }
        __syncwarp();
        if (A.v32) {
            for (int q = 0; q < nrows; ++q)
                for (int e = lane; e < L; e += 32) A.v32[rp[q] + e] = (float)A.v64[rp[q] + e];
        }
        __syncwarp();
    }
}

// Preconditioner blocks (mpetsolver.py:264-271): mu (grad u, grad v) per
// displacement component on P2 nodes and c_a M + dt theta K_a L +
// dt theta sum_{b != a} S_ab M on P1 vertices; Dirichlet DOFs eliminated
// symmetrically (zero row and column, unit diagonal).
struct PrecArgs {
    int64_t nnodes, nv;
    const int64_t* n2_ptr;
    const int32_t* n2_col;
    const int64_t* n1_ptr;
    const int32_t* n1_col;
    const int64_t* inc_ptr;
    const int32_t* inc;
    const uint16_t* rank2;
    const uint16_t* rank1;
    const double* geo;
    const int32_t* cell_nodes;
    const int32_t* cells;
    const uint8_t* node_bc;
    const uint8_t* vert_bc;
    double* lu;
    double* pp[MPET_MAX_NETWORKS];
    // network eigenmodes (null: one block per network): per instance Q (J x J) and lambda (J)
    const double* mQ;
    const double* mlam;
    const int32_t* cell_inst;
};

template <int D>
__global__ void __launch_bounds__(256) k_assemble_prec(PrecArgs A, MatCoef P) {
    constexpr int NV = Simplex<D>::NV, NN = Simplex<D>::NN;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int J = P.J;
    for (int64_t i = warp; i < A.nnodes; i += nwarps) {
        const bool isv = i < A.nv;
        const int64_t s2 = A.n2_ptr[i], s1 = A.n1_ptr[i];
        const int d2 = (int)(A.n2_ptr[i + 1] - s2), d1 = (int)(A.n1_ptr[i + 1] - s1);
        for (int e = lane; e < d2; e += 32) A.lu[s2 + e] = 0.0;
        if (isv)
            for (int a = 0; a < J; ++a)
                for (int e = lane; e < d1; e += 32) A.pp[a][s1 + e] = 0.0;
        __syncwarp();
        const bool rowbc = A.node_bc[i] != 0;
        for (int64_t it = A.inc_ptr[i]; it < A.inc_ptr[i + 1]; ++it) {
            const int32_t packed = A.inc[it];
            const int64_t cell = packed >> 4;
            const int m = packed & 15;
            Geo G;
            load_geo(A.geo, cell, G);
            const double w20 = G.vol * kappa<D>();
            const int ntask = isv ? NN + NV : NN;
            for (int t = lane; t < ntask; t += 32) {
                if (t < NN) {
                    const int j = t;
                    const int32_t nj = A.cell_nodes[NN * cell + j];
                    if (rowbc || A.node_bc[nj]) continue;
                    double gm[4][3], sm[3], gj[4][3], sj[3];
                    p2_grad_table<D>(G, m, gm, sm);
                    p2_grad_table<D>(G, j, gj, sj);
                    double tr = 0.0;
#pragma unroll
                    for (int a = 0; a < D; ++a) {
                        double acc = sm[a] * sj[a];
#pragma unroll
                        for (int r = 0; r < NV; ++r) acc += gm[r][a] * gj[r][a];
                        tr += acc;
                    }
                    double v = P.prec_mu * w20 * tr;
                    if (P.prec_shift > 0.0)
                        v += P.prec_shift * G.vol * (D == 3 ? c_m2[m][j] / 420.0 : c_m2t[m][j] / 180.0);
                    A.lu[s2 + A.rank2[cell * (NN * NN) + m * NN + j]] += v;
                } else {
                    const int w = t - NN;
                    const int32_t vw = A.cells[NV * cell + w];
                    const double M1 = w20 * (m == w ? 2.0 : 1.0);
                    const double L1 = G.vol * (G.b[m][0] * G.b[w][0] + G.b[m][1] * G.b[w][1] + G.b[m][2] * G.b[w][2]);
                    const int64_t pos = s1 + A.rank1[cell * (NN * NV) + m * NV + w];
                    if (A.mQ) {
                        // mode k: lambda_k M + dt theta (sum_a Q_ak^2 K_a) L  (Dirichlet sets equal for all networks)
                        if (A.vert_bc[i] || A.vert_bc[vw]) continue;
                        const int64_t inst = A.cell_inst ? A.cell_inst[cell] : 0;
                        const double* Q = A.mQ + inst * J * J;
                        for (int k = 0; k < J; ++k) {
                            double kk = 0.0;
                            for (int a = 0; a < J; ++a) kk += Q[a * J + k] * Q[a * J + k] * P.Kof(a, cell);
                            A.pp[k][pos] += A.mlam[inst * J + k] * M1 + P.dt_theta * kk * L1;
                        }
                    } else {
                        for (int a = 0; a < J; ++a) {
                            if (A.vert_bc[(int64_t)a * A.nv + i] || A.vert_bc[(int64_t)a * A.nv + vw]) continue;
                            double sS = P.Ssumof(a, cell) - P.Sof(a, a, cell);
                            A.pp[a][pos] += (P.cof(a, cell) + P.dt_theta * sS + P.prec_extra[a]) * M1 +
                                            P.dt_theta * P.Kof(a, cell) * L1;
                        }
                    }
                }
            }
            __syncwarp();
        }
        if (lane == 0) {
            if (rowbc) A.lu[s2 + lb_i32(A.n2_col + s2, d2, (int32_t)i)] = 1.0;
            if (isv) {
                int self1 = lb_i32(A.n1_col + s1, d1, (int32_t)i);
                for (int a = 0; a < J; ++a)
                    if (A.vert_bc[(int64_t)a * A.nv + i]) A.pp[a][s1 + self1] = 1.0;
            }
        }
        __syncwarp();
    }
}

// --- right-hand side ----------------------------------------------------------

struct RhsArgs {
    int64_t nnodes, nv, Nu;
    const int64_t* inc_ptr;
    const int32_t* inc;
    const double* geo;
    const int32_t* cell_nodes;
    const int32_t* cells;
    const double* up;     // previous state
    const double* f;      // nnodes x 3 or null
    const double* g;      // J x nv or null
    double* b;
    double dt, theta;
};

// Pressure rows of L = rhs(F) (mpetsolver.py:196-201, 261) plus dt g_a q_a
// (L1, :249):  -alpha_a (div u^n, q) - c_a (p_a^n, q)
//   + dt (1-theta) [K_a (grad p_a^n, grad q) + sum_b S_ab (p_a^n - p_b^n, q)] + dt (g_a, q).
// ADJ: the pressure rows of B^T lam for the old-state operator B of those
// rows (no displacement or source term, S transposed).
// DIV = false: without the divergence term (added by rhs_div_from_matrix).
template <int D, bool ADJ, bool DIV = true>
__global__ void __launch_bounds__(128) k_rhs_p(RhsArgs A, MatCoef P) {
    constexpr int NV = Simplex<D>::NV, NN = Simplex<D>::NN;
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= A.nv) return;
    const int J = P.J;
    double acc[MPET_MAX_NETWORKS];
    for (int a = 0; a < J; ++a) acc[a] = 0.0;
    const double omt = A.dt * (1.0 - A.theta);
    for (int64_t it = A.inc_ptr[v]; it < A.inc_ptr[v + 1]; ++it) {
        const int32_t packed = A.inc[it];
        const int64_t cell = packed >> 4;
        const int m = packed & 15;
        Geo G;
        load_geo(A.geo, cell, G);
        const double w20 = G.vol * kappa<D>();
        double cp = 0.0;
        for (int j = 0; j < ((ADJ || !DIV) ? 0 : NN); ++j) {
            double g[3], s[3];
            p2_grad_at<D>(G, j, m, g, s);
            const int64_t nj = A.cell_nodes[NN * cell + j];
            if (D == 3)
                cp += (g[0] + s[0]) * A.up[3 * nj] + (g[1] + s[1]) * A.up[3 * nj + 1] +
                      (g[2] + s[2]) * A.up[3 * nj + 2];
            else
                cp += (g[0] + s[0]) * A.up[2 * nj] + (g[1] + s[1]) * A.up[2 * nj + 1];
        }
        cp *= w20;
        double M1[4], L1[4];
        int32_t vw[4];
        for (int w = 0; w < NV; ++w) {
            vw[w] = A.cells[NV * cell + w];
            M1[w] = w20 * (m == w ? 2.0 : 1.0);
            L1[w] = G.vol * (G.b[m][0] * G.b[w][0] + G.b[m][1] * G.b[w][1] + G.b[m][2] * G.b[w][2]);
        }
        double mp[MPET_MAX_NETWORKS], lp[MPET_MAX_NETWORKS];
        for (int a = 0; a < J; ++a) {
            const double* pa = A.up + A.Nu + (int64_t)a * A.nv;
            double sm = 0.0, sl = 0.0, sg = 0.0;
            for (int w = 0; w < NV; ++w) {
                sm += M1[w] * pa[vw[w]];
                sl += L1[w] * pa[vw[w]];
                if (!ADJ && A.g) sg += M1[w] * A.g[(int64_t)a * A.nv + vw[w]];
            }
            mp[a] = sm;
            lp[a] = sl;
            acc[a] += A.dt * sg;
        }
        double rank = 0.0;
        if (P.rank_inv != 0.0)
            for (int b = 0; b < J; ++b) rank += P.rank_b[b] * mp[b];
        for (int a = 0; a < J; ++a) {
            double t = P.rhs_cu[a] * cp - P.cof(a, cell) * mp[a] + omt * P.Kof(a, cell) * lp[a] - P.rank_rhs[a] * rank;
            for (int b = 0; b < J; ++b) {
                const double sab = P.Sof(a, b, cell);
                if (ADJ) t += omt * (sab * mp[a] - P.Sof(b, a, cell) * mp[b]);
                else if (sab != 0.0) t += omt * sab * (mp[a] - mp[b]);
            }
            acc[a] += t;
        }
    }
    for (int a = 0; a < J; ++a) A.b[A.Nu + (int64_t)a * A.nv + v] = acc[a];
}

// Displacement rows: (f, v) with f the P2 interpolant (L0, mpetsolver.py:233).
template <int D>
__global__ void __launch_bounds__(128) k_rhs_u(RhsArgs A) {
    constexpr int NN = Simplex<D>::NN;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= A.nnodes) return;
    double acc[3] = {0.0, 0.0, 0.0};
    if (A.f) {
        for (int64_t it = A.inc_ptr[i]; it < A.inc_ptr[i + 1]; ++it) {
            const int32_t packed = A.inc[it];
            const int64_t cell = packed >> 4;
            const int m = packed & 15;
            const double vol = A.geo[16 * cell + 12] * (D == 3 ? 1.0 / 420.0 : 1.0 / 180.0);
            for (int j = 0; j < NN; ++j) {
                const int64_t nj = A.cell_nodes[NN * cell + j];
                const double w = vol * (D == 3 ? c_m2[m][j] : c_m2t[m][j]);
                for (int k = 0; k < D; ++k) acc[k] += w * A.f[D * nj + k];
            }
        }
    }
    for (int k = 0; k < D; ++k) A.b[D * i + k] = acc[k];
}

__global__ void k_scatter_bc(const int32_t* __restrict__ dofs, const double* __restrict__ vals, int64_t n,
                             double* b) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) b[dofs[k]] = vals[k];
}

// MatZeroRowsColumns on the row-replaced matrix: for rows that are not
// Dirichlet rows, b -= sum over Dirichlet columns a_rc x_c, then zero them.
__global__ void k_zero_bc_columns(int64_t N, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                  double* v, const uint8_t* __restrict__ dof_bc, double* b,
                                  const double* __restrict__ xbc) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < N; r += nwarps) {
        if (dof_bc[r]) continue;
        double s = 0.0;
        for (int64_t e = rp[r] + lane; e < rp[r + 1]; e += 32) {
            const int32_t col = ci[e];
            if (dof_bc[col]) {
                if (xbc) s += v[e] * xbc[col];
                v[e] = 0.0;
            }
        }
        if (b) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) b[r] -= s;
        }
    }
}

static MatCoef make_coef(const mpet_ctx* c, double dt) {
    MatCoef P{};
    P.mu = c->prm.mu;
    P.lmbda = c->prm.lmbda;
    P.dt_theta = dt * c->prm.theta;
    P.J = c->J;
    for (int a = 0; a < c->J; ++a) {
        P.alpha[a] = c->prm.alpha[a];
        P.c[a] = c->prm.c[a];
        P.K[a] = c->prm.K[a];
        double s = 0.0;
        for (int b = 0; b < c->J; ++b) {
            P.S[a * MPET_MAX_NETWORKS + b] = c->prm.S[a * MPET_MAX_NETWORKS + b];
            s += c->prm.S[a * MPET_MAX_NETWORKS + b];
        }
        P.Ssum[a] = s;
    }
    P.Kc = c->K_cells;
    P.cc = c->c_cells;
    P.Sc = c->S_cells;
    P.nc = c->nc;
    P.prec_mu = c->prm.prec_u_weight > 0.0 ? c->prm.prec_u_weight : c->prm.mu;
    P.prec_shift = c->prm.prec_u_shift > 0.0 ? c->prm.prec_u_shift : 0.0;
    const bool tp = c->prm.formulation == MPET_FORM_TOTAL_PRESSURE;
    P.rank_inv = tp ? 1.0 / c->prm.lmbda : 0.0;
    if (tp) P.lmbda = 0.0;  // 2 mu (eps u, eps v) only
    for (int a = 0; a < c->J; ++a) {
        P.cpl[a] = tp ? (a == 0 ? 1.0 : 0.0) : -c->prm.alpha[a];
        P.rhs_cu[a] = tp ? 0.0 : -c->prm.alpha[a];
        P.rank_b[a] = tp ? (a == 0 ? 1.0 : c->prm.alpha[a]) : 0.0;
        P.rank_rhs[a] = (tp && a > 0) ? P.rank_b[a] * P.rank_inv : 0.0;
        P.prec_extra[a] = !tp ? 0.0
                        : a == 0 ? (c->prm.prec_p0_weight > 0.0 ? c->prm.prec_p0_weight : 1.0)
                                 : c->prm.alpha[a] * c->prm.alpha[a] * P.rank_inv;
        // networks with a constant-pressure constraint (no Dirichlet rows): + dt theta K / diam^2
        P.prec_extra[a] += P.dt_theta * c->prec_p_shift[a];
    }
    P.coef_const = (!P.Kc && !P.cc && !P.Sc) ? 1 : 0;
    for (int a = 0; a < c->J; ++a) {
        for (int b = 0; b < c->J; ++b)
            P.Cm[a * MPET_MAX_NETWORKS + b] =
                -(P.dt_theta * ((a == b ? P.Ssum[a] : 0.0) - P.S[a * MPET_MAX_NETWORKS + b]) +
                  P.rank_inv * P.rank_b[a] * P.rank_b[b]) -
                (a == b ? P.c[a] : 0.0);
        P.Kd[a] = -P.dt_theta * P.K[a];
    }
    return P;
}

static inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > 2147483647LL) g = 2147483647LL;
    return (int)(g < 1 ? 1 : g);
}

void launch_assemble_matrix(mpet_ctx* c, double dt, bool apply_bc, bool write32) {
    AsmArgs A{};
    A.nnodes = c->nnodes;
    A.nv = c->nv;
    A.Nu = c->Nu;
    A.row_ptr = c->A.rp;
    A.n2_ptr = c->n2_ptr;
    A.n2_col = c->n2_col;
    A.n1_ptr = c->n1_ptr;
    A.n1_col = c->n1_col;
    A.inc_ptr = c->inc_ptr;
    A.inc = c->inc;
    A.rank2 = c->rank2;
    A.rank1 = c->rank1;
    A.geo = c->geo;
    A.dof_bc = c->dof_bc;
    A.v64 = c->A.v64;
    A.v32 = write32 ? c->A.v32 : nullptr;
    A.dinv = c->dinv;
    A.apply_bc = apply_bc ? 1 : 0;
    MatCoef P = make_coef(c, dt);
    int64_t warps_needed = c->nnodes;
    int blocks = grid_for(warps_needed * 32, 256);
    if (blocks > 152 * 64) blocks = 152 * 64;
    // staged element data when it fits beside everything else (a fifth of HBM stays free)
    const size_t mst_bytes = (size_t)c->nc * (c->dim == 2 ? elem_record<2>() : elem_record<3>()) * sizeof(double);
    // (kept for later assemblies; decided once per context)
    if (!c->elem_tried) {
        c->elem_tried = true;
        if (device_fits(c, mst_bytes)) c->elem_buf = c->pool.alloc<double>((int64_t)(mst_bytes / sizeof(double)));
    }
    if (c->elem_buf) {
        A.Mst = c->elem_buf;
        if (c->dim == 2)
            k_elem_uu<2><<<grid_for(c->nc, 128), 128, 0, c->stream>>>(c->nc, c->geo, P.mu, P.lmbda, c->elem_buf);
        else if (c->elem_kernel == 1)
            launch_elem_uu_tc(c, P.mu, P.lmbda, c->elem_buf);
        else
            k_elem_uu<3><<<grid_for(c->nc, 128), 128, 0, c->stream>>>(c->nc, c->geo, P.mu, P.lmbda, c->elem_buf);
        MPET_CHECK_LAUNCH();
    }
    if (c->dim == 2) k_assemble_matrix<2><<<blocks, 256, 0, c->stream>>>(A, P);
    else k_assemble_matrix<3><<<blocks, 256, 0, c->stream>>>(A, P);
    MPET_CHECK_LAUNCH();
}

void launch_assemble_prec_blocks(mpet_ctx* c, double dt) {
    PrecArgs A{};
    A.nnodes = c->nnodes;
    A.nv = c->nv;
    A.n2_ptr = c->n2_ptr;
    A.n2_col = c->n2_col;
    A.n1_ptr = c->n1_ptr;
    A.n1_col = c->n1_col;
    A.inc_ptr = c->inc_ptr;
    A.inc = c->inc;
    A.rank2 = c->rank2;
    A.rank1 = c->rank1;
    A.geo = c->geo;
    A.cell_nodes = c->cell_nodes;
    A.cells = c->cells;
    A.node_bc = c->node_bc;
    A.vert_bc = c->vert_bc;
    A.lu = c->Lu.v64;
    for (int a = 0; a < c->J; ++a) A.pp[a] = c->Pp[a].v64;
    A.mQ = c->net_modes ? c->mode_Q : nullptr;
    A.mlam = c->net_modes ? c->mode_lam : nullptr;
    A.cell_inst = c->cell_inst;
    MatCoef P = make_coef(c, dt);
    int blocks = grid_for(c->nnodes * 32, 256);
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (c->dim == 2) k_assemble_prec<2><<<blocks, 256, 0, c->stream>>>(A, P);
    else k_assemble_prec<3><<<blocks, 256, 0, c->stream>>>(A, P);
    MPET_CHECK_LAUNCH();
}

// ---- matrix-free displacement preconditioner level ------------------------------------
//
// The first level of the displacement hierarchy is the block w (grad u, grad v)
// (+ shift (u, v)) on P2 nodes (k_assemble_prec above).  Its entries are, per
// cell, K_mj = w |T| kappa sum_{p <= q} T6[mj][pq] (b_p . b_q) + shift |T| M2[m][j]
// over the barycentric gradients b_1..b_D (b_0 = -(b_1 + ... + b_D) folded into
// the integer table T6), so its product can be formed from D (D + 1) / 2 dot
// products and |T| per cell instead of the 61e6-entry CSR matrix (64^3 cube).
// Per cell: slots 0..NQ-1 = w |T| kappa (b_p . b_q) (p <= q), slot NQ = shift
// |T|, slot 7 = bit mask of the cell's Dirichlet nodes (bit pattern).
template <typename T, int D>
__global__ void k_mf_cells(int64_t nc, const double* __restrict__ geo, const int32_t* __restrict__ cell_nodes,
                           const uint8_t* __restrict__ node_bc, double w, double shift, T* out) {
    constexpr int NN = Simplex<D>::NN;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) return;
    Geo G;
    load_geo(geo, c, G);
    const double f = w * G.vol * kappa<D>();
    T o[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) o[q] = T(0);
    int q = 0;
#pragma unroll
    for (int a = 1; a <= D; ++a)
#pragma unroll
        for (int b = a; b <= D; ++b) {
            double dot = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) dot += G.b[a][k] * G.b[b][k];
            o[q++] = (T)(f * dot);
        }
    o[D * (D + 1) / 2] = (T)(shift * G.vol);
    uint32_t mask = 0;
    for (int j = 0; j < NN; ++j)
        if (node_bc[cell_nodes[NN * c + j]]) mask |= 1u << j;
    if constexpr (sizeof(T) == 4) o[7] = __uint_as_float(mask);
    else o[7] = __longlong_as_double((long long)mask);
#pragma unroll
    for (int k = 0; k < 8; ++k) out[8 * c + k] = o[k];
}

// Host tables of the matrix-free level, as floats: T6 (node pairs m <= j x dot
// products p <= q; integers sum_rs (1 + delta_rs) G[m][r][p] G[j][s][q] with b_0
// folded, symmetrised) and the P2 mass matrix divided by |T| (M2):
// tab = [T6 (NP x NQ), M2 (NN x NN)].
template <int D>
static std::vector<float> mf_table() {
    constexpr int NN = Simplex<D>::NN, NV = Simplex<D>::NV;
    double G[10][4][4] = {};
    for (int i = 0; i < NV; ++i)
        for (int r = 0; r < NV; ++r) G[i][r][i] = (r == i) ? 3.0 : -1.0;
    for (int e = 0; e < Simplex<D>::NE; ++e) {
        const int a = edge_end<D>(e, 0), b = edge_end<D>(e, 1);
        G[NV + e][a][b] += 4.0;
        G[NV + e][b][a] += 4.0;
    }
    std::vector<float> tab;
    for (int m = 0; m < NN; ++m)
        for (int j = m; j < NN; ++j) {
            double Ct[4][4];
            for (int p = 0; p < NV; ++p)
                for (int q = 0; q < NV; ++q) {
                    double s = 0.0;
                    for (int r = 0; r < NV; ++r)
                        for (int t = 0; t < NV; ++t) s += (r == t ? 2.0 : 1.0) * G[m][r][p] * G[j][t][q];
                    Ct[p][q] = s;
                }
            auto cf = [&](int a, int b) { return Ct[a][b] - Ct[0][b] - Ct[a][0] + Ct[0][0]; };
            for (int p = 1; p <= D; ++p)
                for (int q = p; q <= D; ++q) tab.push_back((float)(p == q ? cf(p, p) : cf(p, q) + cf(q, p)));
        }
    // the P2 mass matrices of c_m2 / c_m2t above (host copies), divided by 420 / 180
    static const double m3[10][10] = {
        {6, 1, 1, 1, -6, -6, -6, -4, -4, -4},     {1, 6, 1, 1, -6, -4, -4, -6, -6, -4},
        {1, 1, 6, 1, -4, -6, -4, -6, -4, -6},     {1, 1, 1, 6, -4, -4, -6, -4, -6, -6},
        {-6, -6, -4, -4, 32, 16, 16, 16, 16, 8},  {-6, -4, -6, -4, 16, 32, 16, 16, 8, 16},
        {-6, -4, -4, -6, 16, 16, 32, 8, 16, 16},  {-4, -6, -6, -4, 16, 16, 8, 32, 16, 16},
        {-4, -6, -4, -6, 16, 8, 16, 16, 32, 16},  {-4, -4, -6, -6, 8, 16, 16, 16, 16, 32}};
    static const double m2[6][6] = {{6, -1, -1, -4, 0, 0},  {-1, 6, -1, 0, -4, 0},  {-1, -1, 6, 0, 0, -4},
                                    {-4, 0, 0, 32, 16, 16}, {0, -4, 0, 16, 32, 16}, {0, 0, -4, 16, 16, 32}};
    for (int m = 0; m < NN; ++m)
        for (int j = 0; j < NN; ++j) tab.push_back((float)(D == 3 ? m3[m][j] / 420.0 : m2[m][j] / 180.0));
    return tab;
}

void launch_mf_cells(mpet_ctx* c, double dt) {
    const MatCoef P = make_coef(c, dt);
    const bool f32 = c->prm.precision == MPET_PRECISION_MIXED;
    const size_t bytes = (size_t)c->nc * 8 * (f32 ? 4 : 8);
    if (!c->mf_cell) {
        if (!device_fits(c, bytes)) return;  // optional: the CSR level stands in
        c->mf_cell = c->pool.alloc<unsigned char>((int64_t)bytes);
        const std::vector<float> tab = c->dim == 2 ? mf_table<2>() : mf_table<3>();
        c->mf_tab = c->pool.alloc<float>((int64_t)tab.size());
        MPET_CUDA(cudaMemcpyAsync(c->mf_tab, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice,
                                  c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
    }
    const int G = grid_for(c->nc, 256);
    if (c->dim == 2) {
        if (f32) k_mf_cells<float, 2><<<G, 256, 0, c->stream>>>(c->nc, c->geo, c->cell_nodes, c->node_bc, P.prec_mu,
                                                                P.prec_shift, (float*)c->mf_cell);
        else k_mf_cells<double, 2><<<G, 256, 0, c->stream>>>(c->nc, c->geo, c->cell_nodes, c->node_bc, P.prec_mu,
                                                             P.prec_shift, (double*)c->mf_cell);
    } else {
        if (f32) k_mf_cells<float, 3><<<G, 256, 0, c->stream>>>(c->nc, c->geo, c->cell_nodes, c->node_bc, P.prec_mu,
                                                                P.prec_shift, (float*)c->mf_cell);
        else k_mf_cells<double, 3><<<G, 256, 0, c->stream>>>(c->nc, c->geo, c->cell_nodes, c->node_bc, P.prec_mu,
                                                             P.prec_shift, (double*)c->mf_cell);
    }
    MPET_CHECK_LAUNCH();
}

void launch_rhs(mpet_ctx* c, double dt, const double* up_prev, double* b) {
    RhsArgs A{};
    A.nnodes = c->nnodes;
    A.nv = c->nv;
    A.Nu = c->Nu;
    A.inc_ptr = c->inc_ptr;
    A.inc = c->inc;
    A.geo = c->geo;
    A.cell_nodes = c->cell_nodes;
    A.cells = c->cells;
    A.up = up_prev;
    A.f = c->f_nodes;
    A.g = c->g_vert;
    A.b = b;
    A.dt = dt;
    A.theta = c->prm.theta;
    MatCoef P = make_coef(c, dt);
    // The MPET form's -alpha_a (div u^n, q_a) equals the system's pressure-row,
    // displacement-column block applied to u^n (the same coefficient, the same
    // exact integrals): once the matrix is assembled (and its Dirichlet columns
    // are intact) it comes from one FP64 node-block product over the pressure
    // rows instead of every vertex re-deriving its cells' P2 gradients.
    const bool div_by_matrix = c->dim == 3 && c->prm.formulation == MPET_FORM_MPET && c->assembled &&
                               !c->bc_cols_zeroed && c->A.nb && c->A.nb->v64 && c->rhs_div_matrix;
    if (c->dim == 2) {
        k_rhs_u<2><<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A);
        k_rhs_p<2, false><<<grid_for(c->nv, 128), 128, 0, c->stream>>>(A, P);
    } else {
        k_rhs_u<3><<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A);
        if (div_by_matrix) k_rhs_p<3, false, false><<<grid_for(c->nv, 128), 128, 0, c->stream>>>(A, P);
        else k_rhs_p<3, false><<<grid_for(c->nv, 128), 128, 0, c->stream>>>(A, P);
    }
    MPET_CHECK_LAUNCH();
    if (div_by_matrix && !rhs_div_from_matrix(c, up_prev, b)) fail(MPET_ERR_STATE, "divergence term not added");
    launch_facet_rhs(c, dt, up_prev, b);
    launch_bc_vector(c, b);
}

void launch_bc_vector(mpet_ctx* c, double* b) {
    if (c->nbc_dofs > 0) {
        k_scatter_bc<<<grid_for(c->nbc_dofs, 256), 256, 0, c->stream>>>(c->bc_dofs, c->bc_vals, c->nbc_dofs, b);
        MPET_CHECK_LAUNCH();
    }
}

void launch_set_bc_in_x(mpet_ctx* c, double* x) { launch_bc_vector(c, x); }

void launch_zero_bc_columns(mpet_ctx* c, double* b, const double* xbc) {
    k_zero_bc_columns<<<152 * 16, 256, 0, c->stream>>>(c->N, c->A.rp, c->A.ci, c->A.v64, c->dof_bc, b, xbc);
    MPET_CHECK_LAUNCH();
}

// --- discrete adjoint -----------------------------------------------------------
//
// The time loop solves A_FF y_n = (B x_{n-1} + f_n)_F - A_FD g_n with B the
// old-state operator of rhs(F).  Its adjoint needs B^T lam (below: the
// displacement rows from the coupling block, the pressure rows from
// k_rhs_p<true>), the sensitivity of A and B to a per-cell K_a (the element
// stiffness on the p_a block, scaled by -dt theta and dt (1-theta)) and the
// final-pressure misfit with its gradient.

// Displacement rows of B^T lam: B holds -alpha_a (div u, q_a), so row (i, k)
// is -sum_a alpha_a sum_{cells} int lam_a d_k phi_i.
__global__ void __launch_bounds__(128) k_adj_rhs_u(RhsArgs A, MatCoef P) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= A.nnodes) return;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t it = A.inc_ptr[i]; it < A.inc_ptr[i + 1]; ++it) {
        const int32_t packed = A.inc[it];
        const int64_t cell = packed >> 4;
        const int m = packed & 15;
        Geo G;
        load_geo(A.geo, cell, G);
        const double w20 = G.vol * (1.0 / 20.0);
        for (int w = 0; w < 4; ++w) {
            const int64_t vw = A.cells[4 * cell + w];
            double lam = 0.0;
            for (int a = 0; a < P.J; ++a) lam += P.alpha[a] * A.up[A.Nu + (int64_t)a * A.nv + vw];
            double g[3], sg[3];
            p2_grad_at(G, m, w, g, sg);
#pragma unroll
            for (int k = 0; k < 3; ++k) acc[k] -= w20 * (g[k] + sg[k]) * lam;
        }
    }
    A.b[3 * i] = acc[0];
    A.b[3 * i + 1] = acc[1];
    A.b[3 * i + 2] = acc[2];
}

__global__ void k_zero_rows(const int32_t* __restrict__ dofs, int64_t n, double* b) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) b[dofs[k]] = 0.0;
}

// grad_K[a][cell] += dt |cell| grad lam_a . grad(theta p_a + (1 - theta) p_prev_a)
__global__ void __launch_bounds__(128) k_adj_grad(int64_t nc, int64_t nv, int64_t Nu, int J,
                                                  const double* __restrict__ geo, const int32_t* __restrict__ cells,
                                                  const double* __restrict__ lam, const double* __restrict__ up_prev,
                                                  const double* __restrict__ up, double dt, double theta,
                                                  double* grad) {
    const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (cell >= nc) return;
    Geo G;
    load_geo(geo, cell, G);
    int64_t v[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) v[w] = cells[4 * cell + w];
    for (int a = 0; a < J; ++a) {
        const int64_t o = Nu + (int64_t)a * nv;
        double gl[3] = {0.0, 0.0, 0.0}, gq[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const double l = lam[o + v[w]];
            const double q = theta * up[o + v[w]] + (1.0 - theta) * up_prev[o + v[w]];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                gl[k] += l * G.b[w][k];
                gq[k] += q * G.b[w][k];
            }
        }
        grad[(int64_t)a * nc + cell] += dt * G.vol * (gl[0] * gq[0] + gl[1] * gq[1] + gl[2] * gq[2]);
    }
}

// Misfit 1/2 sum_a d_a^T M d_a, d_a = p_a - p*_a: per vertex (M d_a)_v by a
// gather over the vertex's cells, written to dloss (when given) and folded
// into fixed-grid block partials.
__global__ void __launch_bounds__(256) k_misfit(int64_t nv, int64_t Nu, int J, const int64_t* __restrict__ inc_ptr,
                                                const int32_t* __restrict__ inc, const double* __restrict__ geo,
                                                const int32_t* __restrict__ cells, const double* __restrict__ up,
                                                const double* __restrict__ target, double* dloss, double* partials) {
    __shared__ double sh[8];
    double part = 0.0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        for (int a = 0; a < J; ++a) {
            const double* p = up + Nu + (int64_t)a * nv;
            const double* t = target + (int64_t)a * nv;
            double md = 0.0;
            for (int64_t it = inc_ptr[v]; it < inc_ptr[v + 1]; ++it) {
                const int32_t packed = inc[it];
                const int64_t cell = packed >> 4;
                const int m = packed & 15;
                const double w20 = geo[16 * cell + 12] * (1.0 / 20.0);
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const int64_t vw = cells[4 * cell + w];
                    md += w20 * (m == w ? 2.0 : 1.0) * (p[vw] - t[vw]);
                }
            }
            if (dloss) dloss[Nu + (int64_t)a * nv + v] = md;
            part += 0.5 * (p[v] - t[v]) * md;
        }
    }
    part = block_sum256(part, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = part;
}

__global__ void k_finish_sum(const double* __restrict__ partials, double* out) {
    __shared__ double sh[8];
    const double s = sum_partials(partials, sh);
    if (threadIdx.x == 0) *out = s;
}

static RhsArgs rhs_args(mpet_ctx* c, double dt, const double* state, double* b) {
    RhsArgs A{};
    A.nnodes = c->nnodes;
    A.nv = c->nv;
    A.Nu = c->Nu;
    A.inc_ptr = c->inc_ptr;
    A.inc = c->inc;
    A.geo = c->geo;
    A.cell_nodes = c->cell_nodes;
    A.cells = c->cells;
    A.up = state;
    A.b = b;
    A.dt = dt;
    A.theta = c->prm.theta;
    return A;
}

void launch_adjoint_rhs(mpet_ctx* c, double dt, const double* lam, double* out) {
    RhsArgs A = rhs_args(c, dt, lam, out);
    MatCoef P = make_coef(c, dt);
    k_adj_rhs_u<<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A, P);
    k_rhs_p<3, true><<<grid_for(c->nv, 128), 128, 0, c->stream>>>(A, P);
    MPET_CHECK_LAUNCH();
    launch_zero_bc_rows(c, out);
}

// out = M f on the displacement rows (P2 mass matrix of every component), f at P2 nodes
void launch_mass_u(mpet_ctx* c, const double* f_nodes, double* out) {
    RhsArgs A = rhs_args(c, 0.0, nullptr, out);
    A.f = f_nodes;
    if (c->dim == 2) k_rhs_u<2><<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A);
    else k_rhs_u<3><<<grid_for(c->nnodes, 128), 128, 0, c->stream>>>(A);
    MPET_CHECK_LAUNCH();
}

void launch_zero_bc_rows(mpet_ctx* c, double* b) {
    if (c->nbc_dofs > 0) {
        k_zero_rows<<<grid_for(c->nbc_dofs, 256), 256, 0, c->stream>>>(c->bc_dofs, c->nbc_dofs, b);
        MPET_CHECK_LAUNCH();
    }
}

void launch_adjoint_grad(mpet_ctx* c, double dt, const double* lam, const double* up_prev, const double* up,
                         double* grad) {
    k_adj_grad<<<grid_for(c->nc, 128), 128, 0, c->stream>>>(c->nc, c->nv, c->Nu, c->J, c->geo, c->cells, lam,
                                                             up_prev, up, dt, c->prm.theta, grad);
    MPET_CHECK_LAUNCH();
}

void launch_misfit(mpet_ctx* c, const double* up, const double* target, double* dloss, double* loss_dev) {
    if (dloss) MPET_CUDA(cudaMemsetAsync(dloss, 0, sizeof(double) * c->Nu, c->stream));
    k_misfit<<<NB_RED, 256, 0, c->stream>>>(c->nv, c->Nu, c->J, c->inc_ptr, c->inc, c->geo, c->cells, up, target,
                                             dloss, c->partials);
    k_finish_sum<<<1, 256, 0, c->stream>>>(c->partials, loss_dev);
    MPET_CHECK_LAUNCH();
}

// --- network eigenmodes of the pressure preconditioner --------------------------
//
// The pressure blocks of the system couple the networks through the mass
// terms C_ab M, C = diag(c_a + dt theta sum_{b != a} S_ab) - dt theta S (off
// the diagonal).  With C = Q diag(lambda) Q^T per instance, the preconditioner
// can run one AMG hierarchy per mode k on lambda_k M + dt theta kt_k L,
// kt_k = sum_a Q_ak^2 K_a, between z = Q zt and rt = Q^T r at every vertex: an
// SPD operator that keeps the exact mass coupling of the networks (the
// reference's block-diagonal form, mpetsolver.py:270, drops it and loses
// robustness when dt S >> c) but averages the K_a of the modes (poor when
// the K_a differ by orders of magnitude).  Each instance takes the form with
// the eigenmodes when the square of their condition number of its J x J network operator
// at large t stays below the per-network worst case.

__global__ void k_gather_coef(int ninst, const int64_t* __restrict__ rep, int J, int64_t nc,
                              const double* __restrict__ cc, const double* __restrict__ Sc,
                              const double* __restrict__ Kc, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const int64_t cell = rep[i];
    double* o = out + (int64_t)i * (2 * J + J * J);
    for (int a = 0; a < J; ++a) o[a] = cc ? cc[a * nc + cell] : 0.0;
    for (int q = 0; q < J * J; ++q) o[J + q] = Sc ? Sc[q * nc + cell] : 0.0;
    for (int a = 0; a < J; ++a) o[J + J * J + a] = Kc ? Kc[a * nc + cell] : 0.0;
}

__global__ void k_cell_inst(int64_t nc, const int32_t* __restrict__ cells, const int32_t* __restrict__ vinst,
                            int32_t* cinst) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < nc) cinst[c] = vinst[cells[4 * c]];
}

void set_instances(mpet_ctx* c, int ninst, const int32_t* vertex_inst_host) {
    c->vert_inst = c->pool.alloc<int32_t>(c->nv);
    MPET_CUDA(cudaMemcpyAsync(c->vert_inst, vertex_inst_host, sizeof(int32_t) * c->nv, cudaMemcpyHostToDevice,
                              c->stream));
    c->cell_inst = c->pool.alloc<int32_t>(c->nc);
    k_cell_inst<<<grid_for(c->nc, 256), 256, 0, c->stream>>>(c->nc, c->cells, c->vert_inst, c->cell_inst);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaStreamSynchronize(c->stream));
}

void setup_network_modes(mpet_ctx* c, double dt) {
    const int J = c->J;
    c->net_modes = false;
    if (!c->prm.prec_network_modes || J < 2 || c->prm.formulation != MPET_FORM_MPET || c->gmres) return;
    // the transform mixes the networks at a vertex: all networks need the same Dirichlet vertices
    std::vector<uint8_t> vb((size_t)J * c->nv);
    MPET_CUDA(cudaMemcpyAsync(vb.data(), c->vert_bc, vb.size(), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    for (int a = 1; a < J; ++a)
        if (memcmp(vb.data(), vb.data() + (size_t)a * c->nv, c->nv) != 0) return;
    const int ni = c->ninst > 0 ? c->ninst : 1;
    // coefficients of one cell per instance (per-cell fields hold per-instance constants)
    const int stride = 2 * J + J * J;
    std::vector<double> coef((size_t)ni * stride);
    const bool per_cell = c->c_cells || c->S_cells || (c->ninst > 0 && c->K_cells);
    if (per_cell) {
        std::vector<int64_t> rep(ni, 0);
        if (c->ninst > 0) {
            std::vector<int32_t> ci(c->nc);
            MPET_CUDA(cudaMemcpyAsync(ci.data(), c->cell_inst, sizeof(int32_t) * c->nc, cudaMemcpyDeviceToHost,
                                      c->stream));
            MPET_CUDA(cudaStreamSynchronize(c->stream));
            std::vector<char> seen(ni, 0);
            for (int64_t e = 0; e < c->nc; ++e)
                if (!seen[ci[e]]) {
                    seen[ci[e]] = 1;
                    rep[ci[e]] = e;
                }
        }
        TmpBuf drep(sizeof(int64_t) * ni), dout(sizeof(double) * coef.size());
        MPET_CUDA(cudaMemcpyAsync(drep.p, rep.data(), sizeof(int64_t) * ni, cudaMemcpyHostToDevice, c->stream));
        k_gather_coef<<<grid_for(ni, 128), 128, 0, c->stream>>>(ni, (const int64_t*)drep.p, J, c->nc, c->c_cells,
                                                                 c->S_cells, c->ninst > 0 ? c->K_cells : nullptr,
                                                                 (double*)dout.p);
        MPET_CHECK_LAUNCH();
        MPET_CUDA(cudaMemcpyAsync(coef.data(), dout.p, sizeof(double) * coef.size(), cudaMemcpyDeviceToHost,
                                  c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
    }
    const double dth = dt * c->prm.theta;
    std::vector<double> Q((size_t)ni * J * J), lam((size_t)ni * J), C(J * J), K(J), Qm(J * J), lm(J), Qd(J * J),
        ld(J);
    int used = 0;
    for (int i = 0; i < ni; ++i) {
        const double* o = coef.data() + (size_t)i * stride;
        for (int a = 0; a < J; ++a) {
            double off = 0.0;
            for (int b = 0; b < J; ++b) {
                const double sab = c->S_cells ? o[J + a * J + b] : c->prm.S[a * MPET_MAX_NETWORKS + b];
                if (b != a) {
                    off += sab;
                    C[a * J + b] = -dth * sab;
                }
            }
            C[a * J + a] = (c->c_cells ? o[a] : c->prm.c[a]) + dth * off;
            // the scalar slot holds the mean of a per-cell K of a single instance
            K[a] = (c->ninst > 0 && c->K_cells) ? o[J + J * J + a] : c->prm.K[a];
        }
        // per network (Q = I, lambda = diag C) or per eigenmode of C, whichever
        // keeps the network operator C + t dt theta diag(K) better conditioned
        for (int a = 0; a < J; ++a) {
            for (int b = 0; b < J; ++b) Qd[a * J + b] = a == b ? 1.0 : 0.0;
            ld[a] = C[a * J + a];
        }
        sym_eig(J, C.data(), Qm.data(), lm.data());
        bool modes_ok = true;
        for (int k = 0; k < J; ++k) modes_ok = modes_ok && lm[k] > 0.0;
        const double kd = network_kappa(J, C.data(), K.data(), dth, Qd.data(), ld.data());
        const double km = modes_ok ? network_kappa(J, C.data(), K.data(), dth, Qm.data(), lm.data()) : 1e300;
        // Most eigenvalues of the pressure blocks lie at large t (t >= 1e3), where the modes
        // average K over the networks; the per-network form loses at small t (a few low
        // modes when dt S >> c).  MINRES pays the first about linearly in the square root
        // of its condition number and the second far less: the eigenmodes are taken when
        // their large-t condition number squared stays below the per-network worst case
        // (matched against oracle iteration counts of mixed instances, 8^3 cubes).
        const double kmh = modes_ok ? network_kappa(J, C.data(), K.data(), dth, Qm.data(), lm.data(), 30) : 1e300;
        const bool use = km < kd && kmh * kmh < kd;
        used += use ? 1 : 0;
        std::copy((use ? Qm : Qd).begin(), (use ? Qm : Qd).end(), Q.begin() + (size_t)i * J * J);
        std::copy((use ? lm : ld).begin(), (use ? lm : ld).end(), lam.begin() + (size_t)i * J);
    }
    if (used == 0) return;  // every instance keeps the per-network blocks
    if (!c->mode_Q) {
        c->mode_Q = c->pool.alloc<double>((int64_t)ni * J * J);
        c->mode_lam = c->pool.alloc<double>((int64_t)ni * J);
        c->mode_r = c->pool.alloc<double>((int64_t)J * c->nv);
        c->mode_z = c->pool.alloc<double>((int64_t)J * c->nv);
    }
    MPET_CUDA(cudaMemcpyAsync(c->mode_Q, Q.data(), sizeof(double) * Q.size(), cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->mode_lam, lam.data(), sizeof(double) * lam.size(), cudaMemcpyHostToDevice,
                              c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->net_modes = true;
}

// --- a posteriori error indicators (AdaptiveMPETSolver) ----------------------------
//
// DG0 indicators of adaptivempetsolver.py:82-155 for one step up_prev -> up:
// cell residuals RK_u = f + div sigma(u) - sum_j alpha_j grad p_j (P2 per cell:
// f is the P2 interpolant, div sigma(u) and grad p are constant) and
// RK_p_j = -g_j - c_j (p_j - p_j^-)/dt - alpha_j div(u - u^-)/dt
//          - sum_i S_ij (p_j - p_i)   (P1 per cell; div grad p = 0 for P1),
// interior-facet residuals RE_u = -[sigma(u)] n (linear on the facet; the
// pressure jump vanishes for continuous pressures) and RE_p_j = -K_j [grad p_j] n
// (constant), all squared and integrated exactly with the simplex mass
// matrices; h = cell diameter (largest vertex distance).  A thread per cell
// writes the cell terms, a thread per interior facet its half-weighted facet
// terms 0.5 avg(h) ||RE||_F^2, and a thread per cell adds the terms of its
// interior facets in local order: no atomics, results reproducible.

struct EstArgs {
    int64_t nc, nv, Nu, nfi;
    const double* geo;
    const double* x;
    const int32_t* cells;
    const int32_t* cell_nodes;
    const double* up;
    const double* upp;
    const double* f;
    const double* fp;
    const double* g;
    const int32_t* ifacets;
    const int32_t* cell_facets;
    double dt;
    double* eta_p;
    double* eta_u;
    double* eta_udt;
    double* r4;
    double* fval;
    int32_t* bad;
};

template <int D>
__device__ __forceinline__ double cell_diameter(const EstArgs& A, int64_t cell) {
    constexpr int NV = Simplex<D>::NV;
    double h2 = 0.0;
    for (int r = 0; r < NV; ++r)
        for (int s = r + 1; s < NV; ++s) {
            const int64_t a = A.cells[NV * cell + r], b = A.cells[NV * cell + s];
            double q = 0.0;
            for (int k = 0; k < D; ++k) {
                const double t = A.x[3 * a + k] - A.x[3 * b + k];
                q += t * t;
            }
            h2 = fmax(h2, q);
        }
    return sqrt(h2);
}

// sigma(u) at local vertex r of a cell from the P2 displacement in v
template <int D>
__device__ __forceinline__ void sigma_at_vertex(const EstArgs& A, const Geo& G, const MatCoef& P, int64_t cell,
                                                const double* v, int r, double sg[3][3]) {
    constexpr int NN = Simplex<D>::NN;
    double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int j = 0; j < NN; ++j) {
        double g[3], s[3];
        p2_grad_at<D>(G, j, r, g, s);
        const int64_t nj = A.cell_nodes[NN * cell + j];
        for (int a = 0; a < D; ++a) {
            const double ua = v[D * nj + a];
            for (int b = 0; b < D; ++b) gu[a][b] += ua * g[b];
        }
    }
    double tr = 0.0;
    for (int a = 0; a < D; ++a) tr += gu[a][a];
    for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) sg[a][b] = P.mu * (gu[a][b] + gu[b][a]) + (a == b ? P.lmbda * tr : 0.0);
}

template <int D>
__global__ void __launch_bounds__(128) k_est_cell(EstArgs A, MatCoef P) {
    constexpr int NV = Simplex<D>::NV, NN = Simplex<D>::NN;
    const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (cell >= A.nc) return;
    Geo G;
    load_geo(A.geo, cell, G);
    const int J = P.J;
    int64_t vt[4];
    for (int r = 0; r < NV; ++r) vt[r] = A.cells[NV * cell + r];
    double divs[2][3], tr[2][4];
    for (int st = 0; st < 2; ++st) {
        const double* v = st ? A.upp : A.up;
        for (int a = 0; a < 3; ++a) divs[st][a] = 0.0;
        for (int r = 0; r < NV; ++r) {
            double sg[3][3];
            sigma_at_vertex<D>(A, G, P, cell, v, r, sg);
            double t = 0.0;
            for (int a = 0; a < D; ++a) {
                for (int b = 0; b < D; ++b) divs[st][a] += sg[a][b] * G.b[r][b];
            }
            // div u at vertex r
            for (int j = 0; j < NN; ++j) {
                double g[3], s[3];
                p2_grad_at<D>(G, j, r, g, s);
                const int64_t nj = A.cell_nodes[NN * cell + j];
                for (int a = 0; a < D; ++a) t += v[D * nj + a] * g[a];
            }
            tr[st][r] = t;
        }
        for (int a = 0; a < J; ++a) {
            const double* pa = v + A.Nu + (int64_t)a * A.nv;
            for (int k = 0; k < D; ++k) {
                double gk = 0.0;
                for (int r = 0; r < NV; ++r) gk += pa[vt[r]] * G.b[r][k];
                divs[st][k] -= P.alpha[a] * gk;
            }
        }
    }
    // momentum cell residuals: values at the P2 nodes, integrated with the P2 mass
    const double w2 = G.vol / (D == 3 ? 420.0 : 180.0);
    double iu = 0.0, iudt = 0.0;
    for (int a = 0; a < D; ++a) {
        double R[NN], Rd[NN];
        for (int i = 0; i < NN; ++i) {
            const int64_t ni = A.cell_nodes[NN * cell + i];
            const double fi = A.f ? A.f[D * ni + a] : 0.0;
            const double fpi = A.fp ? A.fp[D * ni + a] : 0.0;
            R[i] = fi + divs[0][a];
            Rd[i] = (R[i] - (fpi + divs[1][a])) / A.dt;
        }
        for (int i = 0; i < NN; ++i)
            for (int j = 0; j < NN; ++j) {
                const double m = D == 3 ? c_m2[i][j] : c_m2t[i][j];
                iu += R[i] * m * R[j];
                iudt += Rd[i] * m * Rd[j];
            }
    }
    const double h = cell_diameter<D>(A, cell);
    const double kv = kappa<D>() * G.vol;
    // mass-equation cell residuals (P1) and the R4p density
    double ip = 0.0, r4 = 0.0;
    for (int j = 0; j < J; ++j) {
        const double* pj = A.up + A.Nu + (int64_t)j * A.nv;
        const double* pjp = A.upp + A.Nu + (int64_t)j * A.nv;
        double R[4], sR = 0.0, qR = 0.0;
        for (int r = 0; r < NV; ++r) {
            double v = -(A.g ? A.g[(int64_t)j * A.nv + vt[r]] : 0.0) - P.c[j] * (pj[vt[r]] - pjp[vt[r]]) / A.dt -
                       P.alpha[j] * (tr[0][r] - tr[1][r]) / A.dt;
            for (int i = 0; i < J; ++i)
                v -= P.S[i * MPET_MAX_NETWORKS + j] * (pj[vt[r]] - A.up[A.Nu + (int64_t)i * A.nv + vt[r]]);
            R[r] = v;
            sR += v;
            qR += v * v;
        }
        ip += kv * (qR + sR * sR);
        double gd[3] = {0.0, 0.0, 0.0};
        for (int r = 0; r < NV; ++r)
            for (int k = 0; k < D; ++k) gd[k] += (pj[vt[r]] - pjp[vt[r]]) * G.b[r][k];
        r4 += P.K[j] * G.vol * (gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2]);
        for (int i = 0; i < J; ++i) {
            const double sij = P.S[i * MPET_MAX_NETWORKS + j];
            if (!(sij > 3.0e-16)) continue;
            const double* pi = A.up + A.Nu + (int64_t)i * A.nv;
            const double* pip = A.upp + A.Nu + (int64_t)i * A.nv;
            double ab = 0.0, sa = 0.0, sb = 0.0;
            for (int r = 0; r < NV; ++r) {
                const double b = pj[vt[r]] - pjp[vt[r]];
                const double a = b - (pi[vt[r]] - pip[vt[r]]);
                ab += a * b;
                sa += a;
                sb += b;
            }
            r4 += sij * kv * (ab + sa * sb);
        }
    }
    A.eta_u[cell] = h * h * w2 * iu;
    A.eta_udt[cell] = h * h * w2 * iudt;
    A.eta_p[cell] = h * h * ip;
    A.r4[cell] = r4;
}

template <int D>
__global__ void __launch_bounds__(128) k_est_facet(EstArgs A, MatCoef P) {
    constexpr int NV = Simplex<D>::NV;
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= A.nfi) return;
    const int64_t cp = A.ifacets[4 * f], cm = A.ifacets[4 * f + 2];
    const int op = A.ifacets[4 * f + 1];
    Geo Gp, Gm;
    load_geo(A.geo, cp, Gp);
    load_geo(A.geo, cm, Gm);
    const double nb = sqrt(Gp.b[op][0] * Gp.b[op][0] + Gp.b[op][1] * Gp.b[op][1] + Gp.b[op][2] * Gp.b[op][2]);
    double n[3];
    for (int k = 0; k < 3; ++k) n[k] = -Gp.b[op][k] / nb;
    const double area = D * Gp.vol * nb;
    const int J = P.J;
    double sq = 0.0, sqd = 0.0, sv[3] = {0, 0, 0}, svd[3] = {0, 0, 0};
    for (int r = 0; r < NV; ++r) {
        if (r == op) continue;
        const int32_t vr = A.cells[NV * cp + r];
        int rm = -1;
        for (int q = 0; q < NV; ++q)
            if (A.cells[NV * cm + q] == vr) rm = q;
        if (rm < 0) {
            *A.bad = 1;
            return;
        }
        double e[3] = {0, 0, 0}, e0[3] = {0, 0, 0};
        for (int st = 0; st < 2; ++st) {
            const double* v = st ? A.upp : A.up;
            double sp[3][3], sm[3][3];
            sigma_at_vertex<D>(A, Gp, P, cp, v, r, sp);
            sigma_at_vertex<D>(A, Gm, P, cm, v, rm, sm);
            double* out = st ? e0 : e;
            for (int a = 0; a < D; ++a) {
                double t = 0.0;
                for (int b = 0; b < D; ++b) t += (sp[a][b] - sm[a][b]) * n[b];
                out[a] = -t;
            }
        }
        for (int a = 0; a < D; ++a) {
            const double ed = (e[a] - e0[a]) / A.dt;
            sq += e[a] * e[a];
            sqd += ed * ed;
            sv[a] += e[a];
            svd[a] += ed;
        }
    }
    const double cF = area / (D * (D + 1));
    const double iu = cF * (sq + sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
    const double iudt = cF * (sqd + svd[0] * svd[0] + svd[1] * svd[1] + svd[2] * svd[2]);
    double ip = 0.0;
    for (int j = 0; j < J; ++j) {
        const double* pj = A.up + A.Nu + (int64_t)j * A.nv;
        double t = 0.0;
        for (int r = 0; r < NV; ++r) {
            const double a = pj[A.cells[NV * cp + r]], b = pj[A.cells[NV * cm + r]];
            for (int k = 0; k < D; ++k) t += (a * Gp.b[r][k] - b * Gm.b[r][k]) * n[k];
        }
        const double re = -P.K[j] * t;
        ip += area * re * re;
    }
    const double hav = 0.5 * (cell_diameter<D>(A, cp) + cell_diameter<D>(A, cm));
    A.fval[3 * f] = 0.5 * hav * iu;
    A.fval[3 * f + 1] = 0.5 * hav * iudt;
    A.fval[3 * f + 2] = 0.5 * hav * ip;
}

template <int D>
__global__ void k_est_gather(EstArgs A) {
    constexpr int NV = Simplex<D>::NV;
    const int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (cell >= A.nc) return;
    double u = A.eta_u[cell], ud = A.eta_udt[cell], p = A.eta_p[cell];
    for (int k = 0; k < NV; ++k) {
        const int64_t fid = A.cell_facets[NV * cell + k];
        if (fid < 0) continue;
        u += A.fval[3 * fid];
        ud += A.fval[3 * fid + 1];
        p += A.fval[3 * fid + 2];
    }
    A.eta_u[cell] = u;
    A.eta_udt[cell] = ud;
    A.eta_p[cell] = p;
}

// index check of the caller's facet tables before any kernel reads through them
__global__ void k_est_validate(int64_t nc, int nvc, int64_t nfi, const int32_t* __restrict__ ifacets,
                               const int32_t* __restrict__ cell_facets, int32_t* bad) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nfi) {
        const int32_t a = ifacets[4 * i], oa = ifacets[4 * i + 1], b = ifacets[4 * i + 2], ob = ifacets[4 * i + 3];
        if (a < 0 || a >= nc || b < 0 || b >= nc || oa < 0 || oa >= nvc || ob < 0 || ob >= nvc) *bad = 1;
    }
    if (i < nc)
        for (int k = 0; k < nvc; ++k) {
            const int32_t fid = cell_facets[(int64_t)nvc * i + k];
            if (fid < -1 || fid >= nfi) *bad = 1;
        }
}

__global__ void __launch_bounds__(256) k_sum_array(int64_t n, const double* __restrict__ v, double* partials) {
    __shared__ double sh[8];
    double part = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        part += v[i];
    part = block_sum256(part, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = part;
}

int launch_error_indicators(mpet_ctx* c, double dt, const double* up, const double* up_prev, const double* f,
                            const double* fp, const double* g, int64_t nfi, const int32_t* ifacets,
                            const int32_t* cell_facets, double* eta_p, double* eta_u, double* eta_udt,
                            double* r4_host) {
    if (!c->est_bad) {
        c->est_bad = c->pool.alloc<int32_t>(1);
        c->est_r4 = c->pool.alloc<double>(c->nc);
        c->est_sum = c->pool.alloc<double>(1);
    }
    if (nfi > c->est_fval_cap) {
        c->est_fval = c->pool.alloc<double>(3 * (nfi > 0 ? nfi : 1));
        c->est_fval_cap = nfi;
    }
    const int nvc = c->dim + 1;
    MPET_CUDA(cudaMemsetAsync(c->est_bad, 0, sizeof(int32_t), c->stream));
    const int64_t nmax = nfi > c->nc ? nfi : c->nc;
    k_est_validate<<<grid_for(nmax, 256), 256, 0, c->stream>>>(c->nc, nvc, nfi, ifacets, cell_facets, c->est_bad);
    MPET_CHECK_LAUNCH();
    int32_t bad = 0;
    MPET_CUDA(cudaMemcpyAsync(&bad, c->est_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    if (bad) return 1;
    EstArgs A{};
    A.nc = c->nc;
    A.nv = c->nv;
    A.Nu = c->Nu;
    A.nfi = nfi;
    A.geo = c->geo;
    A.x = c->x;
    A.cells = c->cells;
    A.cell_nodes = c->cell_nodes;
    A.up = up;
    A.upp = up_prev;
    A.f = f;
    A.fp = fp;
    A.g = g;
    A.ifacets = ifacets;
    A.cell_facets = cell_facets;
    A.dt = dt;
    A.eta_p = eta_p;
    A.eta_u = eta_u;
    A.eta_udt = eta_udt;
    A.r4 = c->est_r4;
    A.fval = c->est_fval;
    A.bad = c->est_bad;
    MatCoef P = make_coef(c, dt);
    if (c->dim == 2) {
        k_est_cell<2><<<grid_for(c->nc, 128), 128, 0, c->stream>>>(A, P);
        if (nfi > 0) k_est_facet<2><<<grid_for(nfi, 128), 128, 0, c->stream>>>(A, P);
        k_est_gather<2><<<grid_for(c->nc, 256), 256, 0, c->stream>>>(A);
    } else {
        k_est_cell<3><<<grid_for(c->nc, 128), 128, 0, c->stream>>>(A, P);
        if (nfi > 0) k_est_facet<3><<<grid_for(nfi, 128), 128, 0, c->stream>>>(A, P);
        k_est_gather<3><<<grid_for(c->nc, 256), 256, 0, c->stream>>>(A);
    }
    k_sum_array<<<NB_RED, 256, 0, c->stream>>>(c->nc, c->est_r4, c->partials);
    k_finish_sum<<<1, 256, 0, c->stream>>>(c->partials, c->est_sum);
    MPET_CHECK_LAUNCH();
    MPET_CUDA(cudaMemcpyAsync(&bad, c->est_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaMemcpyAsync(r4_host, c->est_sum, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    return bad ? 1 : 0;
}

}  // namespace mpet
