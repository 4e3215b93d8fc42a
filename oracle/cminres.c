/* Preconditioned MINRES with the block smoothed-aggregation V-cycles of
 * oracle/krylov.py, in C with OpenMP (test infrastructure and CPU baseline;
 * the oracle).
 *
 * The same algorithm as krylov.minres (Paige-Saunders recurrences, stop when
 * phibar <= rtol * beta1) and krylov.SAHierarchy.vcycle / _cheb (Chebyshev on
 * D^-1 A over [rho/30, 1.1 rho] times 1.1, degree `cheb`, pre- and
 * post-smoothing, dense coarsest inverse) and krylov.block_preconditioner
 * (one hierarchy shared by the displacement components, one per pressure
 * block, optional network-mode transform Q).  The hierarchies are built by
 * the Python oracle and passed in as CSR arrays; this file only runs them, on
 * every host thread (the reference's iterative path is PETSc MINRES with
 * hypre, src/mpet/mpet/mpetsolver.py:507-556, which this stands in for).
 * Reductions use OpenMP: results agree with the Python oracle to round-off,
 * not bitwise.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int64_t n, m;
    const int64_t* rp;
    const int32_t* ci;
    const double* v;
} ocsr;

typedef struct {
    ocsr A, P, R;          /* P, R unused on the coarsest level */
    const double* dinv;
    double rho;
} olevel;

typedef struct {
    int nlev;
    const olevel* lev;
    int64_t ncoarse;
    const double* cinv;    /* dense inverse of the coarsest operator, row-major */
    int cheb;
    double* work;          /* oracle_hier_work(...) doubles */
} ohier;

static void spmv(const ocsr* A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A->n; ++i) {
        double s = 0.0;
        for (int64_t e = A->rp[i]; e < A->rp[i + 1]; ++e) s += A->v[e] * x[A->ci[e]];
        y[i] = s;
    }
}

static void cheb(const olevel* L, int degree, const double* b, double* x, double* r, double* d) {
    const int64_t n = L->A.n;
    const double hi = 1.1 * L->rho, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
    const double sigma = theta / delta;
    double rho_old = 1.0 / sigma;
    spmv(&L->A, x, r);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        d[i] = L->dinv[i] * (b[i] - r[i]) / theta;
        x[i] += d[i];
    }
    for (int k = 1; k < degree; ++k) {
        spmv(&L->A, x, r);
        const double rho_new = 1.0 / (2.0 * sigma - rho_old);
        const double c1 = rho_new * rho_old, c2 = 2.0 * rho_new / delta;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            d[i] = c1 * d[i] + c2 * L->dinv[i] * (b[i] - r[i]);
            x[i] += d[i];
        }
        rho_old = rho_new;
    }
}

/* work per level k: r, d, t (size n_k), then the next level's right-hand side and
 * solution (size n_{k+1}) */
static void vcycle(const ohier* H, int k, const double* b, double* x, double** W) {
    const olevel* L = &H->lev[k];
    const int64_t n = L->A.n;
    if (k == H->nlev - 1) {
        const int64_t m = H->ncoarse;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < m; ++i) {
            double s = 0.0;
            for (int64_t j = 0; j < m; ++j) s += H->cinv[i * m + j] * b[j];
            x[i] = s;
        }
        return;
    }
    double* r = W[5 * k];
    double* d = W[5 * k + 1];
    double* t = W[5 * k + 2];
    double* bc = W[5 * k + 3];
    double* xc = W[5 * k + 4];
    memset(x, 0, sizeof(double) * n);
    cheb(L, H->cheb, b, x, r, d);
    spmv(&L->A, x, r);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) t[i] = b[i] - r[i];
    spmv(&L->R, t, bc);
    vcycle(H, k + 1, bc, xc, W);
    spmv(&L->P, xc, r);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] += r[i];
    cheb(L, H->cheb, b, x, r, d);
}

/* One hierarchy applied to a right-hand side (b and x of the first level's size). */
static void happly(const ohier* H, const double* b, double* x) {
    double* W[5 * 16];
    int64_t off = 0;
    for (int k = 0; k < H->nlev && k < 16; ++k) {
        const int64_t n = H->lev[k].A.n;
        const int64_t nc = (k + 1 < H->nlev) ? H->lev[k + 1].A.n : 1;
        for (int q = 0; q < 5; ++q) {
            W[5 * k + q] = H->work + off;
            off += q < 3 ? n : nc;
        }
    }
    vcycle(H, 0, b, x, W);
}

/* work doubles a hierarchy needs (at most 16 levels) */
int64_t oracle_hier_work(int nlev, const int64_t* sizes) {
    int64_t w = 0;
    for (int k = 0; k < nlev; ++k) w += 3 * sizes[k] + 2 * (k + 1 < nlev ? sizes[k + 1] : 1);
    return w;
}

typedef struct {
    int64_t Nu, nv, nnodes;
    int dim, J;
    const ohier* hu;
    const ohier* hp;       /* J hierarchies */
    const double* Q;       /* J x J row-major or NULL */
    double* scratch;       /* 2 * max(nnodes, J * nv) doubles */
} oprec;

static void precond(const oprec* M, const double* r, double* z) {
    const int64_t nn = M->nnodes, nv = M->nv;
    double* bi = M->scratch;
    double* xo = M->scratch + (nn > M->J * nv ? nn : M->J * nv);
    for (int k = 0; k < M->dim; ++k) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < nn; ++i) bi[i] = r[M->dim * i + k];
        happly(M->hu, bi, xo);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < nn; ++i) z[M->dim * i + k] = xo[i];
    }
    const double* rp = r + M->Nu;
    double* zp = z + M->Nu;
    const int J = M->J;
    if (M->Q) {
#pragma omp parallel for schedule(static)
        for (int64_t v = 0; v < nv; ++v)
            for (int k = 0; k < J; ++k) {
                double s = 0.0;
                for (int a = 0; a < J; ++a) s += M->Q[a * J + k] * rp[a * nv + v];
                bi[k * nv + v] = s;
            }
    } else {
        memcpy(bi, rp, sizeof(double) * J * nv);
    }
    for (int a = 0; a < J; ++a) happly(&M->hp[a], bi + a * nv, xo + a * nv);
    if (M->Q) {
#pragma omp parallel for schedule(static)
        for (int64_t v = 0; v < nv; ++v)
            for (int a = 0; a < J; ++a) {
                double s = 0.0;
                for (int k = 0; k < J; ++k) s += M->Q[a * J + k] * xo[k * nv + v];
                zp[a * nv + v] = s;
            }
    } else {
        memcpy(zp, xo, sizeof(double) * J * nv);
    }
}

static double dot(int64_t n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* x += MINRES(A, b - A x); returns iterations, writes phibar/beta1 to *rel. */
int oracle_minres(const ocsr* A, const double* b, double* x, const oprec* M, double rtol, int maxit,
                  double* rel) {
    const int64_t n = A->n;
    double* buf = (double*)calloc((size_t)n * 9, sizeof(double));
    if (!buf) return -1;
    double *r1 = buf, *r2 = buf + n, *y = buf + 2 * n, *v = buf + 3 * n, *w1 = buf + 4 * n, *w2 = buf + 5 * n,
           *t = buf + 6 * n;
    spmv(A, x, t);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) r1[i] = b[i] - t[i];
    precond(M, r1, y);
    const double beta1 = sqrt(fmax(dot(n, r1, y), 0.0));
    *rel = 1.0;
    if (beta1 == 0.0) {
        free(buf);
        return 0;
    }
    double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0;
    memcpy(r2, r1, sizeof(double) * n);
    int it = 0;
    while (it < maxit) {
        ++it;
        const double s = 1.0 / beta;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) v[i] = s * y[i];
        spmv(A, v, y);
        if (it >= 2) {
            const double c = beta / oldb;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) y[i] -= c * r1[i];
        }
        const double alfa = dot(n, v, y);
        const double c2 = alfa / beta;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            y[i] -= c2 * r2[i];
            r1[i] = r2[i];
            r2[i] = y[i];
        }
        precond(M, r2, y);
        oldb = beta;
        beta = sqrt(fmax(dot(n, r2, y), 0.0));
        const double oldeps = epsln;
        const double delta = cs * dbar + sn * alfa;
        const double gbar = sn * dbar - cs * alfa;
        epsln = sn * beta;
        dbar = -cs * beta;
        double gamma = hypot(gbar, beta);
        if (gamma < 1e-300) gamma = 1e-300;
        cs = gbar / gamma;
        sn = beta / gamma;
        const double phi = cs * phibar;
        phibar = sn * phibar;
        const double ig = 1.0 / gamma;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            const double wn = (v[i] - oldeps * w1[i] - delta * w2[i]) * ig;
            w1[i] = w2[i];
            w2[i] = wn;
            x[i] += phi * wn;
        }
        *rel = phibar / beta1;
        if (phibar <= rtol * beta1) break;
    }
    free(buf);
    return it;
}
