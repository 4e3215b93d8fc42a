// Host-side smoothed-aggregation AMG setup for one scalar SPD block.
//
// The reference's iterative path preconditions with hypre BoomerAMG
// (PETScKrylovSolver("minres", "hypre_amg"), src/mpet/mpet/mpetsolver.py:507)
// applied to the block-diagonal form of mpetsolver.py:264-271.  This file
// builds instead one smoothed-aggregation hierarchy per diagonal block:
//   strength   |a_ij| >= theta_l sqrt(|a_ii a_jj|), i != j, theta_l = theta 2^-l
//              (0 on a level that has no strong connection)
//   aggregates three greedy passes (root + free neighbourhood, attach,
//              leftovers), isolated rows (Dirichlet unit rows) unaggregated
//   T          piecewise constant, columns scaled to unit 2-norm
//   P          (I - 4/3 rho^-1 D^-1 A) T, rho = spectral radius of D^-1 A
//              from 30 Lanczos steps on D^-1/2 A D^-1/2 (fixed start vector)
//   A_c        P^T A P (Gustavson sparse products, rows sorted)
//   coarsest   explicit inverse via Cholesky (FP64)
// The V-cycle itself runs on the GPU (solve.cu).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "mpet_internal.cuh"

namespace mpet {

static void transpose(const HostCsr& A, HostCsr& T) {
    T.n = A.m;
    T.m = A.n;
    const int64_t nnz = (int64_t)A.ci.size();
    T.rp.assign(T.n + 1, 0);
    T.ci.resize(nnz);
    T.v.resize(nnz);
    for (int64_t e = 0; e < nnz; ++e) T.rp[A.ci[e] + 1]++;
    for (int64_t i = 0; i < T.n; ++i) T.rp[i + 1] += T.rp[i];
    std::vector<int64_t> pos(T.rp.begin(), T.rp.end() - 1);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) {
            int64_t p = pos[A.ci[e]]++;
            T.ci[p] = (int32_t)i;
            T.v[p] = A.v[e];
        }
}

// C = A * B (Gustavson, dense accumulator per thread, columns sorted).
static void spgemm(const HostCsr& A, const HostCsr& B, HostCsr& C) {
    C.n = A.n;
    C.m = B.m;
    C.rp.assign(C.n + 1, 0);
    const int64_t n = A.n;
#pragma omp parallel
    {
        std::vector<int64_t> mark(B.m, -1);
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n; ++i) {
            int64_t cnt = 0;
            for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) {
                const int32_t k = A.ci[e];
                for (int64_t f = B.rp[k]; f < B.rp[k + 1]; ++f) {
                    const int32_t j = B.ci[f];
                    if (mark[j] != i) {
                        mark[j] = i;
                        ++cnt;
                    }
                }
            }
            C.rp[i + 1] = cnt;
        }
    }
    for (int64_t i = 0; i < n; ++i) C.rp[i + 1] += C.rp[i];
    const int64_t nnz = C.rp[n];
    C.ci.resize(nnz);
    C.v.resize(nnz);
#pragma omp parallel
    {
        std::vector<int64_t> mark(B.m, -1);
        std::vector<double> acc(B.m, 0.0);
        std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n; ++i) {
            cols.clear();
            for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) {
                const int32_t k = A.ci[e];
                const double a = A.v[e];
                for (int64_t f = B.rp[k]; f < B.rp[k + 1]; ++f) {
                    const int32_t j = B.ci[f];
                    if (mark[j] != i) {
                        mark[j] = i;
                        acc[j] = 0.0;
                        cols.push_back(j);
                    }
                    acc[j] += a * B.v[f];
                }
            }
            std::sort(cols.begin(), cols.end());
            int64_t p = C.rp[i];
            for (int32_t j : cols) {
                C.ci[p] = j;
                C.v[p] = acc[j];
                ++p;
            }
        }
    }
}

static void csr_matvec(const HostCsr& A, const std::vector<double>& x, std::vector<double>& y) {
    y.assign(A.n, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        double s = 0.0;
        for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) s += A.v[e] * x[A.ci[e]];
        y[i] = s;
    }
}

static double diag_of(const HostCsr& A, int64_t i) {
    for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e)
        if (A.ci[e] == i) return A.v[e];
    return 0.0;
}

// Largest eigenvalue of a symmetric tridiagonal matrix (diagonal a, off-
// diagonal b[1..m-1]) by Sturm-sequence bisection.
static double tridiag_max_eig(const std::vector<double>& a, const std::vector<double>& b) {
    const int m = (int)a.size();
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < m; ++i) {
        const double r = (i > 0 ? fabs(b[i]) : 0.0) + (i + 1 < m ? fabs(b[i + 1]) : 0.0);
        lo = fmin(lo, a[i] - r);
        hi = fmax(hi, a[i] + r);
    }
    auto below = [&](double x) {  // eigenvalues < x
        int cnt = 0;
        double d = 1.0;
        for (int i = 0; i < m; ++i) {
            d = a[i] - x - (i > 0 ? b[i] * b[i] / d : 0.0);
            if (d == 0.0) d = -1e-300;
            if (d < 0.0) ++cnt;
        }
        return cnt;
    };
    for (int it = 0; it < 200 && hi - lo > 1e-12 * fmax(1.0, fabs(hi)); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (below(mid) >= m) hi = mid; else lo = mid;
    }
    return hi;
}

double tridiag_max_eig_host(const std::vector<double>& a, const std::vector<double>& b) {
    return tridiag_max_eig(a, b);
}

// Spectral radius of D^-1 A: 30 Lanczos steps on D^-1/2 A D^-1/2 (same
// spectrum, symmetric) from x_i = 0.5 + ((7919 i) mod 1009)/1009, then the
// largest Ritz value.
static double lanczos_rho(const HostCsr& A, const std::vector<double>& dinv, int steps) {
    const int64_t n = A.n;
    std::vector<double> s(n), v(n), vprev(n, 0.0), w(n), t;
    for (int64_t i = 0; i < n; ++i) s[i] = dinv[i] > 0.0 ? sqrt(dinv[i]) : 0.0;
    double nrm = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        v[i] = 0.5 + (double)((7919LL * i) % 1009LL) / 1009.0;
        nrm += v[i] * v[i];
    }
    nrm = sqrt(nrm);
    for (int64_t i = 0; i < n; ++i) v[i] /= nrm;
    std::vector<double> al, be(1, 0.0);
    double beta = 0.0;
    for (int k = 0; k < steps && k < n; ++k) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) w[i] = s[i] * v[i];
        csr_matvec(A, w, t);
        double alpha = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : alpha)
        for (int64_t i = 0; i < n; ++i) {
            w[i] = s[i] * t[i] - beta * vprev[i];
            alpha += w[i] * v[i];
        }
        al.push_back(alpha);
        double nb = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : nb)
        for (int64_t i = 0; i < n; ++i) {
            w[i] -= alpha * v[i];
            nb += w[i] * w[i];
        }
        beta = sqrt(nb);
        if (beta <= 1e-14 * fabs(alpha) || k + 1 == steps || k + 1 == n) break;
        be.push_back(beta);
        const double ib = 1.0 / beta;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            vprev[i] = v[i];
            v[i] = w[i] * ib;
        }
    }
    return tridiag_max_eig(al, be);
}

static void strength(const HostCsr& A, double theta, HostCsr& S) {
    const int64_t n = A.n;
    std::vector<double> d(n);
    for (int64_t i = 0; i < n; ++i) d[i] = fabs(diag_of(A, i));
    S.n = S.m = n;
    S.rp.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        int64_t cnt = 0;
        for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) {
            const int32_t j = A.ci[e];
            const double v = fabs(A.v[e]);
            if (j != i && v > 0.0 && v >= theta * sqrt(d[i] * d[j])) ++cnt;
        }
        S.rp[i + 1] = S.rp[i] + cnt;
    }
    S.ci.resize(S.rp[n]);
    for (int64_t i = 0; i < n; ++i) {
        int64_t p = S.rp[i];
        for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) {
            const int32_t j = A.ci[e];
            const double v = fabs(A.v[e]);
            if (j != i && v > 0.0 && v >= theta * sqrt(d[i] * d[j])) S.ci[p++] = j;
        }
    }
}

int64_t aggregate(const HostCsr& S, std::vector<int64_t>& agg) {
    const int64_t n = S.n;
    agg.assign(n, -1);
    int64_t nagg = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -1) continue;
        const int64_t b = S.rp[i], e = S.rp[i + 1];
        if (b == e) continue;
        bool free = true;
        for (int64_t q = b; q < e && free; ++q) free = agg[S.ci[q]] == -1;
        if (!free) continue;
        agg[i] = nagg;
        for (int64_t q = b; q < e; ++q) agg[S.ci[q]] = nagg;
        ++nagg;
    }
    std::vector<int64_t> agg2(agg);
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -1) continue;
        for (int64_t q = S.rp[i]; q < S.rp[i + 1]; ++q)
            if (agg[S.ci[q]] != -1) {
                agg2[i] = agg[S.ci[q]];
                break;
            }
    }
    agg.swap(agg2);
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -1) continue;
        const int64_t b = S.rp[i], e = S.rp[i + 1];
        if (b == e) continue;
        agg[i] = nagg;
        for (int64_t q = b; q < e; ++q)
            if (agg[S.ci[q]] == -1) agg[S.ci[q]] = nagg;
        ++nagg;
    }
    return nagg;
}

bool cholesky_inverse(std::vector<double>& a, int64_t n, std::vector<double>& inv) {
    // in-place lower Cholesky of a (row-major n x n)
    for (int64_t j = 0; j < n; ++j) {
        double s = a[j * n + j];
        for (int64_t k = 0; k < j; ++k) s -= a[j * n + k] * a[j * n + k];
        if (!(s > 0.0)) return false;
        const double l = sqrt(s);
        a[j * n + j] = l;
        for (int64_t i = j + 1; i < n; ++i) {
            double t = a[i * n + j];
            for (int64_t k = 0; k < j; ++k) t -= a[i * n + k] * a[j * n + k];
            a[i * n + j] = t / l;
        }
    }
    inv.assign(n * n, 0.0);
    std::vector<double> y(n);
    for (int64_t col = 0; col < n; ++col) {
        for (int64_t i = 0; i < n; ++i) {
            double t = (i == col) ? 1.0 : 0.0;
            for (int64_t k = 0; k < i; ++k) t -= a[i * n + k] * y[k];
            y[i] = t / a[i * n + i];
        }
        for (int64_t i = n - 1; i >= 0; --i) {
            double t = y[i];
            for (int64_t k = i + 1; k < n; ++k) t -= a[k * n + i] * inv[k * n + col];
            inv[i * n + col] = t / a[i * n + i];
        }
    }
    return true;
}

// Threads for the setup: the affinity set, capped by a cgroup CPU quota
// (containers often expose every core but grant only a fraction).
int host_threads() {
    int n = 1;
#ifdef _OPENMP
    n = omp_get_num_procs();
#endif
    long quota = -1, period = -1;
    if (FILE* f = fopen("/sys/fs/cgroup/cpu.max", "r")) {
        char q[64] = {0};
        if (fscanf(f, "%63s %ld", q, &period) == 2 && strcmp(q, "max") != 0) quota = atol(q);
        fclose(f);
    } else if (FILE* f1 = fopen("/sys/fs/cgroup/cpu/cpu.cfs_quota_us", "r")) {
        if (fscanf(f1, "%ld", &quota) != 1) quota = -1;
        fclose(f1);
        if (FILE* f2 = fopen("/sys/fs/cgroup/cpu/cpu.cfs_period_us", "r")) {
            if (fscanf(f2, "%ld", &period) != 1) period = -1;
            fclose(f2);
        }
    }
    if (quota > 0 && period > 0) {
        long q = quota / period;
        if (q < 1) q = 1;
        if (q < n) n = (int)q;
    }
    if (n > 32) n = 32;
    return n < 1 ? 1 : n;
}

// Smoothed-aggregation prolongator of level A (threshold th); false when the
// level cannot be coarsened.
static bool sa_prolongator(const HostCsr& A, const std::vector<double>& dinv, double rho, double th, HostCsr& P) {
    const int64_t n = A.n;
    HostCsr S;
    strength(A, th, S);
    std::vector<int64_t> agg;
    int64_t nagg = aggregate(S, agg);
    if (nagg == 0 && th > 0.0) {
        strength(A, 0.0, S);
        nagg = aggregate(S, agg);
    }
    if (nagg == 0 || nagg >= n) return false;
    std::vector<int64_t> size(nagg, 0);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) size[agg[i]]++;
    HostCsr T;
    T.n = n;
    T.m = nagg;
    T.rp.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) T.rp[i + 1] = T.rp[i] + (agg[i] >= 0 ? 1 : 0);
    T.ci.resize(T.rp[n]);
    T.v.resize(T.rp[n]);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) {
            T.ci[T.rp[i]] = (int32_t)agg[i];
            T.v[T.rp[i]] = 1.0 / sqrt((double)size[agg[i]]);
        }
    // P = T - (4/3/rho) D^-1 A T
    HostCsr AT;
    spgemm(A, T, AT);
    const double w = 4.0 / 3.0 / rho;
    P = HostCsr();
    P.n = n;
    P.m = nagg;
    P.rp.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        // union of T row (<= 1 entry) and AT row, both sorted
        int64_t cnt = AT.rp[i + 1] - AT.rp[i];
        if (T.rp[i + 1] > T.rp[i]) {
            const int32_t j = T.ci[T.rp[i]];
            bool found = false;
            for (int64_t e = AT.rp[i]; e < AT.rp[i + 1]; ++e)
                if (AT.ci[e] == j) found = true;
            if (!found) ++cnt;
        }
        P.rp[i + 1] = P.rp[i] + cnt;
    }
    P.ci.resize(P.rp[n]);
    P.v.resize(P.rp[n]);
    for (int64_t i = 0; i < n; ++i) {
        int64_t p = P.rp[i];
        const bool hasT = T.rp[i + 1] > T.rp[i];
        const int32_t tj = hasT ? T.ci[T.rp[i]] : -1;
        const double tv = hasT ? T.v[T.rp[i]] : 0.0;
        bool placed = !hasT;
        for (int64_t e = AT.rp[i]; e < AT.rp[i + 1]; ++e) {
            const int32_t j = AT.ci[e];
            if (!placed && tj < j) {
                P.ci[p] = tj;
                P.v[p] = tv;
                ++p;
                placed = true;
            }
            double v = -w * dinv[i] * AT.v[e];
            if (j == tj) {
                v += tv;
                placed = true;
            }
            P.ci[p] = j;
            P.v[p] = v;
            ++p;
        }
        if (!placed) {
            P.ci[p] = tj;
            P.v[p] = tv;
            ++p;
        }
    }
    return true;
}

void amg_setup_host(HostCsr A, const HostCsr* P0, double theta, int coarse_size, int max_levels, HostAmg& out,
                    int nthreads, bool rho0_device) {
    out.lev.clear();
    if (coarse_size < 1) coarse_size = 500;
    if (max_levels < 1) max_levels = 12;
#ifdef _OPENMP
    omp_set_num_threads(nthreads > 0 ? nthreads : host_threads());
#endif
    while (true) {
        HostAmgLevel L;
        const int64_t n = A.n;
        L.dinv.resize(n);
        for (int64_t i = 0; i < n; ++i) {
            const double d = diag_of(A, i);
            L.dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
        }
        // the first level's spectral radius is only needed by its smoother when P0
        // is given: with rho0_device it is estimated on the GPU after the upload
        // (rho < 0 marks that), the same Lanczos iteration on the same start vector
        const bool given = P0 != nullptr && out.lev.empty();
        L.rho = (given && rho0_device) ? -1.0 : lanczos_rho(A, L.dinv, 30);
        L.A = std::move(A);
        out.lev.push_back(std::move(L));
        HostAmgLevel& cur = out.lev.back();
        if (!given && (n <= coarse_size || (int)out.lev.size() >= max_levels)) break;
        HostCsr P;
        if (given) {
            if (P0->n != n) fail(MPET_ERR_INVALID, "first-level prolongator has the wrong row count");
            P = *P0;
        } else {
            // the threshold halves per aggregation level; a level without any
            // strong connection is aggregated on its full graph (threshold 0)
            const int sa_level = (int)out.lev.size() - 1 - (P0 != nullptr ? 1 : 0);
            const double th = theta * pow(0.5, (double)sa_level);
            if (!sa_prolongator(cur.A, cur.dinv, cur.rho, th, P)) break;
        }
        HostCsr R;
        transpose(P, R);
        HostCsr AP, Ac;
        spgemm(cur.A, P, AP);
        spgemm(R, AP, Ac);
        cur.P = std::move(P);
        cur.R = std::move(R);
        A = std::move(Ac);
    }
    // coarsest: dense inverse
    HostAmgLevel& last = out.lev.back();
    const int64_t nc = last.A.n;
    if (nc > 6000) fail(MPET_ERR_INVALID, "AMG coarsest level too large for a dense solve");
    std::vector<double> dense(nc * nc, 0.0);
    for (int64_t i = 0; i < nc; ++i)
        for (int64_t e = last.A.rp[i]; e < last.A.rp[i + 1]; ++e) dense[i * nc + last.A.ci[e]] = last.A.v[e];
    out.ncoarse = nc;
    if (!cholesky_inverse(dense, nc, out.cinv))
        fail(MPET_ERR_INVALID, "AMG coarsest operator is not positive definite");
}

// ---- smoothed aggregation for the displacement block (vector elasticity) ----------
//
// The same recipe with a near-nullspace of rigid-body modes (Vanek, Mandel and
// Brezina, Computing 56 (1996) 179-196): unknowns come in nodes (3 displacement
// components at the first level, the coarse unknowns of an aggregate below);
// strength and aggregation act on the node graph with Frobenius norms of the
// node blocks; the tentative prolongator of an aggregate is the orthonormal
// factor Q of its near-nullspace rows B_agg = Q R (Gram-Schmidt with rank
// detection), and R gives the coarse near-nullspace; P = (I - 4/3 rho^-1 D^-1 A) T.

static bool check_csr(const HostCsr& A) {
    if ((int64_t)A.rp.size() != A.n + 1 || A.rp[0] != 0) return false;
    for (int64_t i = 0; i < A.n; ++i)
        if (A.rp[i + 1] < A.rp[i]) return false;
    if (A.rp[A.n] != (int64_t)A.ci.size() || A.ci.size() != A.v.size()) return false;
    for (int32_t j : A.ci)
        if (j < 0 || j >= A.m) return false;
    return true;
}

// C = T - w D^-1 (A T), rows of T and A T sorted
static void smooth_prolongator(const HostCsr& A, const HostCsr& T, const std::vector<double>& dinv, double w,
                               HostCsr& P) {
    HostCsr AT;
    spgemm(A, T, AT);
    const int64_t n = T.n;
    P = HostCsr();
    P.n = n;
    P.m = T.m;
    P.rp.assign(n + 1, 0);
    std::vector<std::vector<std::pair<int32_t, double>>> rows(n);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        auto& r = rows[i];
        int64_t a = T.rp[i], ae = T.rp[i + 1], b = AT.rp[i], be = AT.rp[i + 1];
        const double f = -w * dinv[i];
        while (a < ae || b < be) {
            if (b >= be || (a < ae && T.ci[a] < AT.ci[b])) {
                r.emplace_back(T.ci[a], T.v[a]);
                ++a;
            } else if (a >= ae || AT.ci[b] < T.ci[a]) {
                r.emplace_back(AT.ci[b], f * AT.v[b]);
                ++b;
            } else {
                r.emplace_back(T.ci[a], T.v[a] + f * AT.v[b]);
                ++a;
                ++b;
            }
        }
    }
    for (int64_t i = 0; i < n; ++i) P.rp[i + 1] = P.rp[i] + (int64_t)rows[i].size();
    P.ci.resize(P.rp[n]);
    P.v.resize(P.rp[n]);
    for (int64_t i = 0; i < n; ++i) {
        int64_t p = P.rp[i];
        for (auto& e : rows[i]) {
            P.ci[p] = e.first;
            P.v[p] = e.second;
            ++p;
        }
    }
}

// Node strength graph: nodes own the unknowns node_ptr[k]..node_ptr[k+1].
static void node_strength(const HostCsr& A, const std::vector<int64_t>& node_ptr, double theta, HostCsr& S) {
    const int64_t nn = (int64_t)node_ptr.size() - 1;
    std::vector<int32_t> node_of(A.n);
    for (int64_t k = 0; k < nn; ++k)
        for (int64_t i = node_ptr[k]; i < node_ptr[k + 1]; ++i) node_of[i] = (int32_t)k;
    std::vector<std::vector<std::pair<int32_t, double>>> nb(nn);
    std::vector<double> dnorm(nn, 0.0);
#pragma omp parallel
    {
        std::vector<double> acc(nn, 0.0);
        std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 256)
        for (int64_t k = 0; k < nn; ++k) {
            cols.clear();
            for (int64_t i = node_ptr[k]; i < node_ptr[k + 1]; ++i)
                for (int64_t e = A.rp[i]; e < A.rp[i + 1]; ++e) {
                    const int32_t q = node_of[A.ci[e]];
                    if (acc[q] == 0.0) cols.push_back(q);
                    acc[q] += A.v[e] * A.v[e];
                }
            std::sort(cols.begin(), cols.end());
            for (int32_t q : cols) {
                if (q == k) dnorm[k] = sqrt(acc[q]);
                else nb[k].emplace_back(q, sqrt(acc[q]));
                acc[q] = 0.0;
            }
        }
    }
    S = HostCsr();
    S.n = S.m = nn;
    S.rp.assign(nn + 1, 0);
    for (int64_t k = 0; k < nn; ++k) {
        int64_t cnt = 0;
        for (auto& e : nb[k])
            if (e.second > 0.0 && e.second >= theta * sqrt(dnorm[k] * dnorm[e.first])) ++cnt;
        S.rp[k + 1] = S.rp[k] + cnt;
    }
    S.ci.resize(S.rp[nn]);
    S.v.assign(S.rp[nn], 1.0);
    for (int64_t k = 0; k < nn; ++k) {
        int64_t p = S.rp[k];
        for (auto& e : nb[k])
            if (e.second > 0.0 && e.second >= theta * sqrt(dnorm[k] * dnorm[e.first])) S.ci[p++] = e.first;
    }
}

void amg_setup_block_host(const HostCsr& A1, const std::vector<double>& B1, int nb_cols, int bs, double theta,
                          int coarse_size, int max_levels, HostAmg& out) {
    out.lev.clear();
    if (!check_csr(A1) || A1.n % bs != 0 || (int64_t)B1.size() != A1.n * nb_cols)
        fail(MPET_ERR_INVALID, "block AMG input is inconsistent");
    HostCsr A = A1;
    std::vector<double> B = B1;  // A.n x nb_cols, row-major
    std::vector<int64_t> node_ptr(A.n / bs + 1);
    for (size_t k = 0; k < node_ptr.size(); ++k) node_ptr[k] = (int64_t)k * bs;
    if (coarse_size < 1) coarse_size = 500;
    if (max_levels < 1) max_levels = 12;
#ifdef _OPENMP
    omp_set_num_threads(host_threads());
#endif
    int sa_level = 0;
    while (true) {
        HostAmgLevel L;
        const int64_t n = A.n;
        L.dinv.resize(n);
        for (int64_t i = 0; i < n; ++i) {
            const double d = diag_of(A, i);
            L.dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
        }
        L.rho = lanczos_rho(A, L.dinv, 30);
        L.A = A;
        out.lev.push_back(L);
        HostAmgLevel& cur = out.lev.back();
        if (n <= coarse_size || (int)out.lev.size() >= max_levels) break;
        const double th = theta * pow(0.5, (double)sa_level);
        HostCsr S;
        node_strength(A, node_ptr, th, S);
        std::vector<int64_t> agg;
        int64_t nagg = aggregate(S, agg);
        if (nagg == 0 && th > 0.0) {
            node_strength(A, node_ptr, 0.0, S);
            nagg = aggregate(S, agg);
        }
        const int64_t nn = (int64_t)node_ptr.size() - 1;
        if (nagg == 0 || nagg >= nn) break;
        // tentative prolongator: per aggregate, Gram-Schmidt on its near-nullspace rows
        std::vector<std::vector<int64_t>> members(nagg);
        for (int64_t k = 0; k < nn; ++k)
            if (agg[k] >= 0) members[agg[k]].push_back(k);
        std::vector<int> kcols(nagg, 0);
        std::vector<std::vector<double>> Qs(nagg), Rs(nagg);
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t g = 0; g < nagg; ++g) {
            std::vector<int64_t> dofs;
            for (int64_t k : members[g])
                for (int64_t i = node_ptr[k]; i < node_ptr[k + 1]; ++i) dofs.push_back(i);
            const int64_t m = (int64_t)dofs.size();
            std::vector<double> Q(m * nb_cols), R(nb_cols * nb_cols, 0.0);
            for (int64_t r = 0; r < m; ++r)
                for (int q = 0; q < nb_cols; ++q) Q[r * nb_cols + q] = B[dofs[r] * nb_cols + q];
            double scale = 0.0;
            for (double v : Q) scale = fmax(scale, fabs(v));
            int kept = 0;
            std::vector<double> cols(m * nb_cols);  // kept orthonormal columns, column-major
            for (int q = 0; q < nb_cols; ++q) {
                std::vector<double> v(m);
                for (int64_t r = 0; r < m; ++r) v[r] = Q[r * nb_cols + q];
                double n0 = 0.0;
                for (double t : v) n0 += t * t;
                n0 = sqrt(n0);
                for (int pass = 0; pass < 2; ++pass)
                    for (int c2 = 0; c2 < kept; ++c2) {
                        double d = 0.0;
                        for (int64_t r = 0; r < m; ++r) d += cols[c2 * m + r] * v[r];
                        R[c2 * nb_cols + q] += d;
                        for (int64_t r = 0; r < m; ++r) v[r] -= d * cols[c2 * m + r];
                    }
                double nv2 = 0.0;
                for (double t : v) nv2 += t * t;
                nv2 = sqrt(nv2);
                if (nv2 <= 1e-10 * fmax(n0, scale * sqrt((double)m)) || kept == m) continue;
                for (int64_t r = 0; r < m; ++r) cols[kept * m + r] = v[r] / nv2;
                R[kept * nb_cols + q] = nv2;
                ++kept;
            }
            kcols[g] = kept;
            Qs[g].assign(cols.begin(), cols.begin() + (size_t)kept * m);
            Rs[g].assign(R.begin(), R.begin() + (size_t)kept * nb_cols);
        }
        std::vector<int64_t> cptr(nagg + 1, 0);
        for (int64_t g = 0; g < nagg; ++g) cptr[g + 1] = cptr[g] + kcols[g];
        const int64_t nc = cptr[nagg];
        HostCsr T;
        T.n = n;
        T.m = nc;
        T.rp.assign(n + 1, 0);
        std::vector<int64_t> dof_agg(n, -1), dof_row(n, -1);
        for (int64_t g = 0; g < nagg; ++g) {
            int64_t r = 0;
            for (int64_t k : members[g])
                for (int64_t i = node_ptr[k]; i < node_ptr[k + 1]; ++i) {
                    dof_agg[i] = g;
                    dof_row[i] = r++;
                }
        }
        for (int64_t i = 0; i < n; ++i) T.rp[i + 1] = T.rp[i] + (dof_agg[i] >= 0 ? kcols[dof_agg[i]] : 0);
        T.ci.resize(T.rp[n]);
        T.v.resize(T.rp[n]);
        for (int64_t i = 0; i < n; ++i) {
            const int64_t g = dof_agg[i];
            if (g < 0) continue;
            const int64_t m = (int64_t)Qs[g].size() / (kcols[g] > 0 ? kcols[g] : 1);
            int64_t p = T.rp[i];
            for (int q = 0; q < kcols[g]; ++q) {
                T.ci[p] = (int32_t)(cptr[g] + q);
                T.v[p] = Qs[g][q * m + dof_row[i]];
                ++p;
            }
        }
        std::vector<double> Bc(nc * nb_cols, 0.0);
        for (int64_t g = 0; g < nagg; ++g)
            for (int q = 0; q < kcols[g]; ++q)
                for (int c2 = 0; c2 < nb_cols; ++c2) Bc[(cptr[g] + q) * nb_cols + c2] = Rs[g][q * nb_cols + c2];
        HostCsr P;
        smooth_prolongator(A, T, cur.dinv, 4.0 / 3.0 / cur.rho, P);
        HostCsr R;
        transpose(P, R);
        HostCsr AP, Ac;
        spgemm(A, P, AP);
        spgemm(R, AP, Ac);
        cur.P = std::move(P);
        cur.R = std::move(R);
        A = std::move(Ac);
        B.swap(Bc);
        node_ptr = cptr;
        ++sa_level;
    }
    HostAmgLevel& last = out.lev.back();
    const int64_t nc = last.A.n;
    if (nc > 6000) fail(MPET_ERR_INVALID, "AMG coarsest level too large for a dense solve");
    std::vector<double> dense(nc * nc, 0.0);
    for (int64_t i = 0; i < nc; ++i)
        for (int64_t e = last.A.rp[i]; e < last.A.rp[i + 1]; ++e) dense[i * nc + last.A.ci[e]] = last.A.v[e];
    out.ncoarse = nc;
    if (!cholesky_inverse(dense, nc, out.cinv))
        fail(MPET_ERR_INVALID, "AMG coarsest operator is not positive definite");
    for (auto& L : out.lev)
        if (!check_csr(L.A) || (L.P.n > 0 && (!check_csr(L.P) || !check_csr(L.R))))
            fail(MPET_ERR_INVALID, "block AMG produced an inconsistent level");
}

// P1 vector elasticity mu (grad u, grad v) + mu (grad u^T, grad v) + lmbda (div u, div v)
// on the free vertices (3 unknowns each, interleaved): the Galerkin operator of the P2
// displacement block under the P1-in-P2 embedding (the embedding is exact, so the
// product P^T A P is the P1 stiffness).  Rows are owned per vertex, cells taken from the
// vertex incidence in ascending order (deterministic); the pattern is the vertex
// adjacency restricted to free vertices.
void p1_elasticity_host(int64_t nv, const std::vector<int64_t>& vptr, const std::vector<int32_t>& vadj,
                        const std::vector<int64_t>& inc_ptr, const std::vector<int32_t>& inc,
                        const std::vector<double>& geo, const std::vector<int32_t>& cells,
                        const std::vector<int64_t>& cidx, double mu, double lmbda, HostCsr& A) {
    int64_t nf = 0;
    for (int64_t v = 0; v < nv; ++v)
        if (cidx[v] >= 0) nf = std::max(nf, cidx[v] + 1);
    A = HostCsr();
    A.n = A.m = 3 * nf;
    A.rp.assign(A.n + 1, 0);
    std::vector<int64_t> row_of(nf, -1);
    for (int64_t v = 0; v < nv; ++v)
        if (cidx[v] >= 0) row_of[cidx[v]] = v;
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t v = row_of[f];
        int64_t cnt = 0;
        for (int64_t e = vptr[v]; e < vptr[v + 1]; ++e) cnt += cidx[vadj[e]] >= 0;
        for (int a = 0; a < 3; ++a) A.rp[3 * f + a + 1] = 3 * cnt;
    }
    for (int64_t i = 0; i < A.n; ++i) A.rp[i + 1] += A.rp[i];
    A.ci.resize(A.rp[A.n]);
    A.v.assign(A.rp[A.n], 0.0);
#ifdef _OPENMP
    omp_set_num_threads(host_threads());
#endif
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t v = row_of[f];
        std::vector<int32_t> fcols;
        for (int64_t e = vptr[v]; e < vptr[v + 1]; ++e)
            if (cidx[vadj[e]] >= 0) fcols.push_back(vadj[e]);
        const int64_t w = (int64_t)fcols.size();
        for (int a = 0; a < 3; ++a)
            for (int64_t q = 0; q < w; ++q)
                for (int b = 0; b < 3; ++b) A.ci[A.rp[3 * f + a] + 3 * q + b] = (int32_t)(3 * cidx[fcols[q]] + b);
        for (int64_t it = inc_ptr[v]; it < inc_ptr[v + 1]; ++it) {
            const int64_t cell = inc[it] >> 4;
            const int m = inc[it] & 15;
            const double* g = &geo[16 * cell];
            const double vol = g[12];
            for (int s = 0; s < 4; ++s) {
                const int32_t ws = cells[4 * cell + s];
                if (cidx[ws] < 0) continue;
                const int64_t q = std::lower_bound(fcols.begin(), fcols.end(), ws) - fcols.begin();
                const double* bm = g + 3 * m;
                const double* bs = g + 3 * s;
                const double dot = bm[0] * bs[0] + bm[1] * bs[1] + bm[2] * bs[2];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        A.v[A.rp[3 * f + a] + 3 * q + b] +=
                            vol * ((a == b ? mu * dot : 0.0) + mu * bm[b] * bs[a] + lmbda * bm[a] * bs[b]);
            }
        }
    }
}

// Symmetric eigendecomposition A = Q diag(lam) Q^T of a small n x n matrix
// (row-major, n <= 8) by cyclic Jacobi rotations (Golub & Van Loan,
// Matrix Computations, 4th ed., sec. 8.5.2); Q column i is eigenvector i.
void sym_eig(int n, const double* A_in, double* Q, double* lam) {
    std::vector<double> A(A_in, A_in + n * n);
    for (int i = 0; i < n * n; ++i) Q[i] = 0.0;
    for (int i = 0; i < n; ++i) Q[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += A[i * n + j] * A[i * n + j];
                if (i != j) off += A[i * n + j] * A[i * n + j];
            }
        if (off <= 1e-30 * tot) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (apq == 0.0) continue;
                const double tau = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = t * cs;
                for (int k = 0; k < n; ++k) {  // A <- A J
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = cs * akp - sn * akq;
                    A[k * n + q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^T A
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = cs * apk - sn * aqk;
                    A[q * n + k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {  // Q <- Q J
                    const double qkp = Q[k * n + p], qkq = Q[k * n + q];
                    Q[k * n + p] = cs * qkp - sn * qkq;
                    Q[k * n + q] = sn * qkp + cs * qkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) lam[i] = A[i * n + i];
}

// Worst condition number, over t in [1, 1e6] (the ratio of stiffness to
// mass eigenvalues from the smoothest to the finest P1 mode), of the
// preconditioned network operator P(t)^-1 (C + t g diag(K)) for
// P(t) = Q (diag(lam) + t g diag(kt)) Q^T, kt_k = sum_a Q_ak^2 K_a.
double network_kappa(int J, const double* C, const double* K, double g, const double* Q, const double* lam,
                     int first_step) {
    double worst = 1.0;
    std::vector<double> A(J * J), P(J * J), L(J * J), W(J * J), T(J * J), V(J * J), ev(J);
    std::vector<double> kt(J);
    for (int k = 0; k < J; ++k) {
        kt[k] = 0.0;
        for (int a = 0; a < J; ++a) kt[k] += Q[a * J + k] * Q[a * J + k] * K[a];
    }
    for (int step = first_step; step <= 60; ++step) {
        const double t = pow(10.0, 0.1 * step);
        for (int a = 0; a < J; ++a)
            for (int b = 0; b < J; ++b) {
                A[a * J + b] = C[a * J + b] + (a == b ? t * g * K[a] : 0.0);
                double p = 0.0;
                for (int k = 0; k < J; ++k) p += Q[a * J + k] * (lam[k] + t * g * kt[k]) * Q[b * J + k];
                P[a * J + b] = p;
            }
        // P = L L^T (Cholesky), W = L^-1 A L^-T, eigenvalues of W
        for (int i = 0; i < J; ++i)
            for (int j = 0; j <= i; ++j) {
                double sum = P[i * J + j];
                for (int k = 0; k < j; ++k) sum -= L[i * J + k] * L[j * J + k];
                if (i == j) {
                    if (!(sum > 0.0)) return 1e300;
                    L[i * J + i] = sqrt(sum);
                } else {
                    L[i * J + j] = sum / L[j * J + j];
                }
            }
        for (int col = 0; col < J; ++col)  // T = L^-1 A (forward substitution per column)
            for (int i = 0; i < J; ++i) {
                double sum = A[i * J + col];
                for (int k = 0; k < i; ++k) sum -= L[i * J + k] * T[k * J + col];
                T[i * J + col] = sum / L[i * J + i];
            }
        for (int row = 0; row < J; ++row)  // W = T L^-T
            for (int i = 0; i < J; ++i) {
                double sum = T[row * J + i];
                for (int k = 0; k < i; ++k) sum -= W[row * J + k] * L[i * J + k];
                W[row * J + i] = sum / L[i * J + i];
            }
        sym_eig(J, W.data(), V.data(), ev.data());
        double lo = ev[0], hi = ev[0];
        for (int k = 1; k < J; ++k) {
            lo = std::min(lo, ev[k]);
            hi = std::max(hi, ev[k]);
        }
        if (!(lo > 0.0)) return 1e300;
        worst = std::max(worst, hi / lo);
    }
    return worst;
}

}  // namespace mpet
