/* Assembly of the MPET system in C with OpenMP (test infrastructure and CPU
 * baseline; the oracle).
 *
 * The same matrices as oracle/mpet.py, built without the (cells x nloc x
 * nloc) dense arrays that limit the numpy restatement to small meshes:
 *
 *  - oracle_node_adjacency: for every P2 node the sorted set of P2 nodes that
 *    share a cell with it (vertices come first, since vertex ids < nv);
 *  - oracle_system_pattern: the DOLFIN sparsity rule of fem.assemble_csr
 *    (the union of dense mixed cell blocks), row by row: a displacement row
 *    of node i holds d columns per node of adj(i), then for each network a
 *    the pressure columns of the vertices in adj(i); a pressure row of vertex
 *    v holds the same for node v.  Columns come out sorted;
 *  - oracle_assemble: values of a = lhs(F) (OracleMPET.local_matrix,
 *    src/mpet/mpet/mpetsolver.py:196-201) on that pattern, the pressure rows
 *    of the previous-state operator B (b_p = B up_, OracleMPET.rhs_L without
 *    data terms, mpetsolver.py:196-201, 261, 356), the preconditioner's
 *    scalar P2 block w (grad u, grad v) on the node pattern and, per network
 *    (or network eigenmode), lam_k M + dt theta kk_k L on the vertex pattern
 *    (OracleMPET.preconditioner_blocks, mpetsolver.py:264-271);
 *  - oracle_dirichlet_rows: DirichletBC.apply on the system (rows zeroed,
 *    unit diagonal, pattern kept).
 *
 * Cells are processed colour by colour (no two cells of a colour share a
 * vertex), so the additions need no atomics; each entry's sum runs over its
 * cells in colour order, so values agree with the numpy oracle to round-off.
 * Exact integration as in oracle/fem.py: gradients of P2 functions are linear
 * and every term is a polynomial of degree <= 2.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXN2 10 /* P2 nodes of a tetrahedron */
#define MAXV 4

static const int TET_EDGES[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
static const int TRI_EDGES[3][2] = {{1, 2}, {0, 2}, {0, 1}};

static int cmp_i64(const void* a, const void* b) {
    const int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/* node -> cell incidence (CSR over nnodes) */
static void incidence(int64_t nc, int n2, const int64_t* cn, int64_t nnodes, int64_t** ptr_out, int64_t** idx_out) {
    int64_t* ptr = (int64_t*)calloc((size_t)nnodes + 1, sizeof(int64_t));
    for (int64_t c = 0; c < nc; ++c)
        for (int i = 0; i < n2; ++i) ptr[cn[c * n2 + i] + 1]++;
    for (int64_t i = 0; i < nnodes; ++i) ptr[i + 1] += ptr[i];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)nnodes);
    memcpy(fill, ptr, sizeof(int64_t) * (size_t)nnodes);
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ptr[nnodes] > 0 ? ptr[nnodes] : 1));
    for (int64_t c = 0; c < nc; ++c)
        for (int i = 0; i < n2; ++i) idx[fill[cn[c * n2 + i]]++] = c;
    free(fill);
    *ptr_out = ptr;
    *idx_out = idx;
}

/* sorted unique nodes sharing a cell with `node`, written to out (capacity cap); returns count */
static int64_t gather_adj(int64_t node, int n2, const int64_t* cn, const int64_t* iptr, const int64_t* iidx,
                          int64_t* buf) {
    int64_t m = 0;
    for (int64_t e = iptr[node]; e < iptr[node + 1]; ++e) {
        const int64_t c = iidx[e];
        for (int j = 0; j < n2; ++j) buf[m++] = cn[c * n2 + j];
    }
    qsort(buf, (size_t)m, sizeof(int64_t), cmp_i64);
    int64_t u = 0;
    for (int64_t k = 0; k < m; ++k)
        if (u == 0 || buf[k] != buf[u - 1]) buf[u++] = buf[k];
    return u;
}

/* Node adjacency: adj_ptr (nnodes + 1) must be preallocated; when adj_idx is
 * NULL only the pointers (and the count of vertex neighbours per node, degv)
 * are computed; call again with adj_idx of size adj_ptr[nnodes]. */
int oracle_node_adjacency(int64_t nc, int n2, const int64_t* cn, int64_t nnodes, int64_t nv, int64_t* adj_ptr,
                          int32_t* degv, int32_t* adj_idx) {
    int64_t *iptr, *iidx;
    incidence(nc, n2, cn, nnodes, &iptr, &iidx);
    int64_t maxinc = 0;
    for (int64_t i = 0; i < nnodes; ++i)
        if (iptr[i + 1] - iptr[i] > maxinc) maxinc = iptr[i + 1] - iptr[i];
    int bad = 0;
#pragma omp parallel
    {
        int64_t* buf = (int64_t*)malloc(sizeof(int64_t) * (size_t)(maxinc * n2 + 1));
        if (!buf) {
#pragma omp atomic write
            bad = 1;
        }
#pragma omp for schedule(dynamic, 4096)
        for (int64_t i = 0; i < nnodes; ++i) {
            if (!buf) continue;
            const int64_t u = gather_adj(i, n2, cn, iptr, iidx, buf);
            if (!adj_idx) {
                adj_ptr[i + 1] = u;
                int32_t dv = 0;
                for (int64_t k = 0; k < u; ++k) dv += buf[k] < nv;
                degv[i] = dv;
            } else {
                for (int64_t k = 0; k < u; ++k) adj_idx[adj_ptr[i] + k] = (int32_t)buf[k];
            }
        }
        free(buf);
    }
    if (!adj_idx) {
        adj_ptr[0] = 0;
        for (int64_t i = 0; i < nnodes; ++i) adj_ptr[i + 1] += adj_ptr[i];
    }
    free(iptr);
    free(iidx);
    return bad ? -1 : 0;
}

/* Row pointers (N + 1) of the mixed system; if ci is not NULL also the columns. */
void oracle_system_pattern(int d, int J, int64_t nnodes, int64_t nv, const int64_t* adj_ptr, const int32_t* degv,
                           const int32_t* adj_idx, int64_t* rp, int32_t* ci) {
    const int64_t Nu = (int64_t)d * nnodes, N = Nu + (int64_t)J * nv;
    if (!ci) {
        rp[0] = 0;
        for (int64_t r = 0; r < N; ++r) {
            const int64_t node = r < Nu ? r / d : (r - Nu) % nv;
            const int64_t deg = adj_ptr[node + 1] - adj_ptr[node];
            rp[r + 1] = rp[r] + d * deg + (int64_t)J * degv[node];
        }
        return;
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < N; ++r) {
        const int64_t node = r < Nu ? r / d : (r - Nu) % nv;
        const int32_t* a = adj_idx + adj_ptr[node];
        const int64_t deg = adj_ptr[node + 1] - adj_ptr[node];
        int32_t* out = ci + rp[r];
        for (int64_t k = 0; k < deg; ++k)
            for (int q = 0; q < d; ++q) *out++ = (int32_t)(d * (int64_t)a[k] + q);
        for (int b = 0; b < J; ++b)
            for (int64_t k = 0; k < degv[node]; ++k) *out++ = (int32_t)(Nu + (int64_t)b * nv + a[k]);
    }
}

/* Greedy colouring of cells: cells sharing a vertex get different colours.
 * Returns the number of colours (colour[c] in [0, ncol)), -1 on failure. */
int oracle_colour_cells(int64_t nc, int nvc, const int64_t* cells, int64_t nv, int32_t* colour) {
    int64_t *vptr, *vidx;
    incidence(nc, nvc, cells, nv, &vptr, &vidx);
    int ncol = 0;
    uint64_t used[4];
    for (int64_t c = 0; c < nc; ++c) colour[c] = -1;
    for (int64_t c = 0; c < nc; ++c) {
        memset(used, 0, sizeof(used));
        for (int i = 0; i < nvc; ++i) {
            const int64_t v = cells[c * nvc + i];
            for (int64_t e = vptr[v]; e < vptr[v + 1]; ++e) {
                const int32_t k = colour[vidx[e]];
                if (k >= 0) used[k >> 6] |= 1ull << (k & 63);
            }
        }
        int k = 0;
        while (k < 256 && (used[k >> 6] >> (k & 63)) & 1ull) ++k;
        if (k == 256) {
            free(vptr);
            free(vidx);
            return -1;
        }
        colour[c] = k;
        if (k + 1 > ncol) ncol = k + 1;
    }
    free(vptr);
    free(vidx);
    return ncol;
}

typedef struct {
    int d, J;
    int64_t nc, nv, nnodes;
    const double* x;          /* nv x d */
    const int64_t* cells;     /* nc x (d+1), sorted vertex ids */
    const int64_t* cn;        /* nc x n2, P2 nodes (vertices, then edges in UFC order) */
    double mu, lmbda, theta, dt;
    const double* alpha;      /* J */
    const double* c;          /* J */
    const double* K;          /* J x nc per-cell permeability */
    const double* S;          /* J x J */
    double u_weight;          /* w of the preconditioner's P2 block */
    const double* lam;        /* J: mass coefficient of preconditioner block k */
    const double* kk;         /* J x nc: permeability of preconditioner block k */
} oasm;

static double det3(const double J[3][3]) {
    return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

/* barycentric gradients b[m][k] and volume of cell c */
static double cell_geometry(const oasm* P, int64_t cell, double b[MAXV][3]) {
    const int d = P->d;
    const int64_t* v = P->cells + cell * (d + 1);
    double Jm[3][3] = {{0}};
    for (int i = 0; i < d; ++i)
        for (int k = 0; k < d; ++k) Jm[k][i] = P->x[v[i + 1] * d + k] - P->x[v[0] * d + k];
    double det, inv[3][3];
    if (d == 3) {
        det = det3(Jm);
        inv[0][0] = (Jm[1][1] * Jm[2][2] - Jm[1][2] * Jm[2][1]) / det;
        inv[0][1] = (Jm[0][2] * Jm[2][1] - Jm[0][1] * Jm[2][2]) / det;
        inv[0][2] = (Jm[0][1] * Jm[1][2] - Jm[0][2] * Jm[1][1]) / det;
        inv[1][0] = (Jm[1][2] * Jm[2][0] - Jm[1][0] * Jm[2][2]) / det;
        inv[1][1] = (Jm[0][0] * Jm[2][2] - Jm[0][2] * Jm[2][0]) / det;
        inv[1][2] = (Jm[0][2] * Jm[1][0] - Jm[0][0] * Jm[1][2]) / det;
        inv[2][0] = (Jm[1][0] * Jm[2][1] - Jm[1][1] * Jm[2][0]) / det;
        inv[2][1] = (Jm[0][1] * Jm[2][0] - Jm[0][0] * Jm[2][1]) / det;
        inv[2][2] = (Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0]) / det;
    } else {
        det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
        inv[0][0] = Jm[1][1] / det;
        inv[0][1] = -Jm[0][1] / det;
        inv[1][0] = -Jm[1][0] / det;
        inv[1][1] = Jm[0][0] / det;
    }
    /* rows of J^-1 are grad lambda_1..lambda_d; grad lambda_0 = -sum */
    for (int k = 0; k < d; ++k) {
        double s = 0.0;
        for (int m = 1; m <= d; ++m) {
            b[m][k] = inv[m - 1][k];
            s += inv[m - 1][k];
        }
        b[0][k] = -s;
    }
    return fabs(det) / (d == 3 ? 6.0 : 2.0);
}

/* Local tensors of one cell: Mg[i][j][k][l] = int d_k phi_i d_l phi_j,
 * Cp[i][k][w] = int lambda_w d_k phi_i, M1, L1 (P1 mass and stiffness). */
static void cell_tensors(const oasm* P, int64_t cell, double Mg[MAXN2][MAXN2][3][3], double Cp[MAXN2][3][MAXV],
                         double M1[MAXV][MAXV], double L1[MAXV][MAXV]) {
    const int d = P->d, n = d + 1, n2 = d == 3 ? 10 : 6;
    double b[MAXV][3];
    const double vol = cell_geometry(P, cell, b);
    const double w0 = (d == 3 ? 6.0 / 120.0 : 2.0 / 24.0); /* d!/(d+2)! */
    double W[MAXV][MAXV];
    for (int r = 0; r < n; ++r)
        for (int s = 0; s < n; ++s) W[r][s] = w0 * (r == s ? 2.0 : 1.0);
    /* gradient of P2 basis i at vertex r */
    double g[MAXN2][MAXV][3];
    memset(g, 0, sizeof(g));
    for (int m = 0; m < n; ++m)
        for (int r = 0; r < n; ++r)
            for (int k = 0; k < d; ++k) g[m][r][k] = (4.0 * (m == r) - 1.0) * b[m][k];
    for (int e = 0; e < n2 - n; ++e) {
        const int a = d == 3 ? TET_EDGES[e][0] : TRI_EDGES[e][0];
        const int bb = d == 3 ? TET_EDGES[e][1] : TRI_EDGES[e][1];
        for (int k = 0; k < d; ++k) {
            g[n + e][a][k] = 4.0 * b[bb][k];
            g[n + e][bb][k] = 4.0 * b[a][k];
        }
    }
    /* Wg[j][r][l] = sum_s W[r][s] g[j][s][l] */
    double Wg[MAXN2][MAXV][3];
    for (int j = 0; j < n2; ++j)
        for (int r = 0; r < n; ++r)
            for (int l = 0; l < d; ++l) {
                double s = 0.0;
                for (int q = 0; q < n; ++q) s += W[r][q] * g[j][q][l];
                Wg[j][r][l] = s;
            }
    for (int i = 0; i < n2; ++i)
        for (int j = 0; j < n2; ++j)
            for (int k = 0; k < d; ++k)
                for (int l = 0; l < d; ++l) {
                    double s = 0.0;
                    for (int r = 0; r < n; ++r) s += g[i][r][k] * Wg[j][r][l];
                    Mg[i][j][k][l] = s * vol;
                }
    for (int i = 0; i < n2; ++i)
        for (int k = 0; k < d; ++k)
            for (int w = 0; w < n; ++w) {
                double s = 0.0;
                for (int r = 0; r < n; ++r) s += W[w][r] * g[i][r][k];
                Cp[i][k][w] = s * vol;
            }
    for (int v = 0; v < n; ++v)
        for (int w = 0; w < n; ++w) {
            M1[v][w] = W[v][w] * vol;
            double s = 0.0;
            for (int k = 0; k < d; ++k) s += b[v][k] * b[w][k];
            L1[v][w] = s * vol;
        }
}

/* position of `key` in the sorted array a[0..n) (must be present) */
static inline int64_t find_pos(const int32_t* a, int64_t n, int32_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Values (added into zeroed arrays): A (system, nnz of rp), B (pressure rows
 * of the previous-state operator, offset rp[Nu]), Lu (P2 block on adj),
 * Pk (J blocks on the vertex pattern: row v holds adj(v)'s vertex prefix;
 * block k at Pk + k * pnnz).  Any output may be NULL. */
int oracle_assemble(const oasm* P, int ncol, const int32_t* colour, const int64_t* adj_ptr, const int32_t* degv,
                    const int32_t* adj_idx, const int64_t* rp, const int64_t* vp, double* A, double* B, double* Lu,
                    double* Pk) {
    const int d = P->d, n = d + 1, n2 = d == 3 ? 10 : 6, J = P->J;
    const int64_t nc = P->nc, nv = P->nv, Nu = (int64_t)d * P->nnodes;
    const int64_t pnnz = vp ? vp[nv] : 0;
    const double mu = P->mu, lm = P->lmbda, th = P->theta, dt = P->dt;
    double Ssum[16];
    for (int a = 0; a < J; ++a) {
        Ssum[a] = 0.0;
        for (int b = 0; b < J; ++b) Ssum[a] += P->S[a * J + b];
    }
    for (int col = 0; col < ncol; ++col) {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t cell = 0; cell < nc; ++cell) {
            if (colour[cell] != col) continue;
            double Mg[MAXN2][MAXN2][3][3], Cp[MAXN2][3][MAXV], M1[MAXV][MAXV], L1[MAXV][MAXV];
            cell_tensors(P, cell, Mg, Cp, M1, L1);
            const int64_t* nodes = P->cn + cell * n2;
            int64_t pos[MAXN2][MAXN2];
            for (int i = 0; i < n2; ++i) {
                const int32_t* ai = adj_idx + adj_ptr[nodes[i]];
                const int64_t di = adj_ptr[nodes[i] + 1] - adj_ptr[nodes[i]];
                for (int j = 0; j < n2; ++j) pos[i][j] = find_pos(ai, di, (int32_t)nodes[j]);
            }
            /* displacement rows */
            for (int i = 0; i < n2; ++i) {
                const int64_t node = nodes[i];
                const int64_t deg = adj_ptr[node + 1] - adj_ptr[node];
                double tr[MAXN2];
                for (int j = 0; j < n2; ++j) {
                    double s = 0.0;
                    for (int k = 0; k < d; ++k) s += Mg[i][j][k][k];
                    tr[j] = s;
                }
                if (Lu)
                    for (int j = 0; j < n2; ++j) Lu[adj_ptr[node] + pos[i][j]] += P->u_weight * tr[j];
                if (!A) continue;
                for (int k = 0; k < d; ++k) {
                    const int64_t base = rp[d * node + k];
                    for (int j = 0; j < n2; ++j)
                        for (int l = 0; l < d; ++l)
                            A[base + pos[i][j] * d + l] +=
                                mu * tr[j] * (k == l) + mu * Mg[i][j][l][k] + lm * Mg[i][j][k][l];
                    for (int a = 0; a < J; ++a)
                        for (int w = 0; w < n; ++w)
                            A[base + d * deg + (int64_t)a * degv[node] + pos[i][w]] += -P->alpha[a] * Cp[i][k][w];
                }
            }
            /* pressure rows: vertex m of the cell (P2 node m) */
            for (int m = 0; m < n; ++m) {
                const int64_t v = nodes[m];
                const int64_t deg = adj_ptr[v + 1] - adj_ptr[v];
                const int64_t dv = degv[v];
                for (int a = 0; a < J; ++a) {
                    const int64_t row = Nu + (int64_t)a * nv + v;
                    const int64_t base = rp ? rp[row] : 0;
                    const double Ka = P->K[(int64_t)a * nc + cell];
                    if (A || B) {
                        for (int j = 0; j < n2; ++j)
                            for (int l = 0; l < d; ++l) {
                                const double val = -P->alpha[a] * Cp[j][l][m];
                                if (A) A[base + pos[m][j] * d + l] += val;
                                if (B) B[base - rp[Nu] + pos[m][j] * d + l] += val;
                            }
                        for (int b = 0; b < J; ++b)
                            for (int w = 0; w < n; ++w) {
                                const int64_t o = base + d * deg + (int64_t)b * dv + pos[m][w];
                                const double sab = (Ssum[a] * (a == b) - P->S[a * J + b]) * M1[m][w];
                                double va = -dt * th * sab;
                                double vb = dt * (1.0 - th) * sab;
                                if (a == b) {
                                    va += -P->c[a] * M1[m][w] - dt * th * Ka * L1[m][w];
                                    vb += -P->c[a] * M1[m][w] + dt * (1.0 - th) * Ka * L1[m][w];
                                }
                                if (A) A[o] += va;
                                if (B) B[o - rp[Nu]] += vb;
                            }
                    }
                }
                if (Pk)
                    for (int k = 0; k < J; ++k) {
                        const double kk = P->kk[(int64_t)k * nc + cell];
                        for (int w = 0; w < n; ++w)
                            Pk[(int64_t)k * pnnz + vp[v] + pos[m][w]] +=
                                P->lam[k] * M1[m][w] + dt * th * kk * L1[m][w];
                    }
            }
        }
    }
    return 0;
}

/* DirichletBC.apply on the system: zero the rows of the listed DOFs, unit diagonal. */
void oracle_dirichlet_rows(int64_t nbc, const int64_t* dofs, const int64_t* rp, const int32_t* ci, double* A) {
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nbc; ++q) {
        const int64_t r = dofs[q];
        for (int64_t e = rp[r]; e < rp[r + 1]; ++e) A[e] = ci[e] == r ? 1.0 : 0.0;
    }
}

/* y[Nu..N) = B x (pressure rows of the previous-state operator), y[0..Nu) = 0 */
void oracle_rhs_prev(int64_t N, int64_t Nu, const int64_t* rp, const int32_t* ci, const double* B, const double* x,
                     double* y) {
    const int64_t off = rp[Nu];
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < N; ++r) {
        double s = 0.0;
        if (r >= Nu)
            for (int64_t e = rp[r]; e < rp[r + 1]; ++e) s += B[e - off] * x[ci[e]];
        y[r] = s;
    }
}

/* krylov.aggregate in C (same three greedy passes, same order, so the same
 * aggregates): S is the strength graph (CSR without the diagonal); agg gets
 * the aggregate of each node (-1 = isolated); returns the aggregate count. */
int64_t oracle_aggregate(int64_t n, const int64_t* ptr, const int32_t* idx, int64_t* agg) {
    int64_t nagg = 0;
    for (int64_t i = 0; i < n; ++i) agg[i] = -1;
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -1 || ptr[i + 1] == ptr[i]) continue;
        int free_all = 1;
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e)
            if (agg[idx[e]] != -1) {
                free_all = 0;
                break;
            }
        if (!free_all) continue;
        agg[i] = nagg;
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) agg[idx[e]] = nagg;
        ++nagg;
    }
    int64_t* agg2 = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!agg2) return -1;
    memcpy(agg2, agg, sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -1) continue;
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e)
            if (agg[idx[e]] != -1) {
                agg2[i] = agg[idx[e]];
                break;
            }
    }
    memcpy(agg, agg2, sizeof(int64_t) * (size_t)n);
    free(agg2);
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -1 || ptr[i + 1] == ptr[i]) continue;
        agg[i] = nagg;
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e)
            if (agg[idx[e]] == -1) agg[idx[e]] = nagg;
        ++nagg;
    }
    return nagg;
}
