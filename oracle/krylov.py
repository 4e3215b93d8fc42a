"""Preconditioned MINRES and smoothed-aggregation AMG on the CPU (oracle).

Test infrastructure and CPU baseline.  The reference's iterative path is
``PETScKrylovSolver("minres", "hypre_amg")`` on the block-diagonal
preconditioner form (src/mpet/mpet/mpetsolver.py:264-271, 502-557; working
twin src/mpet/mpet/mpettotalpressuresolver.py:414-505).  PETSc KSP MINRES
(Paige-Saunders) and an AMG preconditioner are restated here: hypre's
classical BoomerAMG is replaced by smoothed aggregation (one hierarchy per
diagonal block), which is the method the GPU path implements.

The AMG follows the standard SA recipe: symmetric strength of connection
(threshold halved per level, 0 when a level has no strong connection),
greedy three-pass aggregation, piecewise-constant tentative prolongator
(near-nullspace = constants per scalar block), Jacobi-smoothed prolongator
P = (I - omega/rho D^-1 A) T with omega = 4/3, Galerkin coarse operators
P^T A P, Chebyshev smoothing on D^-1 A over [rho/30, 1.1 rho], and a dense
Cholesky solve on the coarsest level.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp


def strength(A, theta):
    A = A.tocsr()
    d = np.abs(A.diagonal())
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    cols = A.indices
    v = np.abs(A.data)
    keep = (rows != cols) & (v >= theta * np.sqrt(d[rows] * d[cols])) & (v > 0)
    S = sp.csr_matrix((np.ones(keep.sum()), (rows[keep], cols[keep])), shape=A.shape)
    S.sort_indices()
    return S


def aggregate(S):
    """Standard greedy aggregation (three passes).  Returns agg id per node (-1 = isolated)."""
    n = S.shape[0]
    ptr, idx = S.indptr, S.indices
    agg = np.full(n, -1, dtype=np.int64)
    nagg = 0
    # pass 1: node whose strong neighbourhood is entirely free starts an aggregate
    for i in range(n):
        if agg[i] != -1:
            continue
        nb = idx[ptr[i]:ptr[i + 1]]
        if nb.size == 0:
            continue
        if np.all(agg[nb] == -1):
            agg[i] = nagg
            agg[nb] = nagg
            nagg += 1
    # pass 2: attach free nodes to a neighbouring aggregate (first one found)
    agg2 = agg.copy()
    for i in range(n):
        if agg[i] != -1:
            continue
        nb = idx[ptr[i]:ptr[i + 1]]
        for j in nb:
            if agg[j] != -1:
                agg2[i] = agg[j]
                break
    agg = agg2
    # pass 3: remaining free nodes with neighbours form new aggregates
    for i in range(n):
        if agg[i] != -1:
            continue
        nb = idx[ptr[i]:ptr[i + 1]]
        if nb.size == 0:
            continue
        agg[i] = nagg
        free = nb[agg[nb] == -1]
        agg[free] = nagg
        nagg += 1
    return agg, nagg


def lanczos_rho(A, Dinv, steps=30):
    """Spectral radius of D^-1 A: ``steps`` Lanczos steps (no reorthogonalisation) on
    D^-1/2 A D^-1/2 from x_i = 0.5 + ((7919 i) mod 1009) / 1009, largest Ritz value."""
    n = A.shape[0]
    s = np.sqrt(np.where(Dinv > 0, Dinv, 0.0))
    i = np.arange(n, dtype=np.int64)
    v = 0.5 + ((7919 * i) % 1009) / 1009.0
    v = v / np.linalg.norm(v)
    vprev = np.zeros(n)
    al, be = [], []
    beta = 0.0
    for k in range(min(steps, n)):
        w = s * (A @ (s * v)) - beta * vprev
        alpha = float(w @ v)
        al.append(alpha)
        w = w - alpha * v
        beta = float(np.linalg.norm(w))
        if beta <= 1e-14 * abs(alpha) or k + 1 == steps or k + 1 == n:
            break
        be.append(beta)
        vprev, v = v, w / beta
    if not be:
        return max(al)
    return float(sla.eigh_tridiagonal(np.array(al), np.array(be), eigvals_only=True)[-1])


def p1_in_p2_embedding(dm, bc_nodes):
    """Prolongator from the P1 functions vanishing at the displacement Dirichlet
    nodes to P2: vertex values copied, edge-midpoint values averaged; Dirichlet
    rows are zero and coarse DOFs are the non-Dirichlet vertices in order."""
    nv, ne = dm.nv, dm.ne
    isbc = np.zeros(dm.nnodes, dtype=bool)
    isbc[np.asarray(bc_nodes, dtype=np.int64)] = True
    cidx = np.full(nv, -1, dtype=np.int64)
    free = ~isbc[:nv]
    cidx[free] = np.arange(free.sum())
    rows = np.concatenate([np.arange(nv), nv + np.arange(ne), nv + np.arange(ne)])
    cols = np.concatenate([np.arange(nv), dm.edges[:, 0], dm.edges[:, 1]])
    vals = np.concatenate([np.ones(nv), 0.5 * np.ones(ne), 0.5 * np.ones(ne)])
    keep = (~isbc[rows]) & (cidx[cols] >= 0)
    return sp.csr_matrix((vals[keep], (rows[keep], cidx[cols[keep]])), shape=(dm.nnodes, int(free.sum())))


class SAHierarchy:
    """Smoothed-aggregation hierarchy; ``P0`` (optional) replaces aggregation on
    the first level (the strength threshold then counts aggregation levels);
    ``aggregate_fn`` (optional) replaces ``aggregate`` by an equivalent (the C
    restatement in cbaseline.aggregate)."""

    def __init__(self, A, theta=0.0, coarse_size=500, max_levels=12, cheb_degree=2, P0=None, aggregate_fn=None):
        self.levels = []
        agg_fn = aggregate if aggregate_fn is None else aggregate_fn
        self.cheb_degree = cheb_degree
        A = A.tocsr()
        while True:
            n = A.shape[0]
            D = A.diagonal().copy()
            Dinv = np.where(D != 0, 1.0 / np.where(D != 0, D, 1.0), 0.0)
            DinvA = sp.diags(Dinv) @ A
            rho = lanczos_rho(A, Dinv)
            lev = {"A": A, "Dinv": Dinv, "rho": rho}
            self.levels.append(lev)
            given = P0 is not None and len(self.levels) == 1
            if not given and (n <= coarse_size or len(self.levels) >= max_levels):
                break
            if given:
                P = P0.tocsr()
            else:
                th = theta * 0.5 ** (len(self.levels) - 1 - (1 if P0 is not None else 0))
                S = strength(A, th)
                agg, nagg = agg_fn(S)
                if nagg == 0 and th > 0.0:
                    agg, nagg = agg_fn(strength(A, 0.0))
                if nagg == 0 or nagg >= n:
                    break
                rows = np.nonzero(agg >= 0)[0]
                sizes = np.bincount(agg[rows], minlength=nagg)
                T = sp.csr_matrix((1.0 / np.sqrt(sizes[agg[rows]]), (rows, agg[rows])), shape=(n, nagg))
                P = (T - (4.0 / 3.0 / rho) * (DinvA @ T)).tocsr()
            R = P.T.tocsr()
            lev["P"], lev["R"] = P, R
            A = (R @ A @ P).tocsr()
            A.sort_indices()
        Ac = self.levels[-1]["A"].toarray()
        self.coarse = sla.cho_factor(Ac)

    def _cheb(self, lev, b, x):
        A, Dinv, rho = lev["A"], lev["Dinv"], lev["rho"]
        hi, lo = 1.1 * rho, 1.1 * rho / 30.0
        theta = 0.5 * (hi + lo)
        delta = 0.5 * (hi - lo)
        sigma = theta / delta
        rho_old = 1.0 / sigma
        r = Dinv * (b - A @ x)
        d = r / theta
        x = x + d
        for _ in range(1, self.cheb_degree):
            r = Dinv * (b - A @ x)
            rho_new = 1.0 / (2.0 * sigma - rho_old)
            d = rho_new * rho_old * d + (2.0 * rho_new / delta) * r
            x = x + d
            rho_old = rho_new
        return x

    def vcycle(self, b, k=0):
        lev = self.levels[k]
        if k == len(self.levels) - 1:
            return sla.cho_solve(self.coarse, b)
        x = self._cheb(lev, b, np.zeros_like(b))
        r = b - lev["A"] @ x
        xc = self.vcycle(lev["R"] @ r, k + 1)
        x = x + lev["P"] @ xc
        x = self._cheb(lev, b, x)
        return x

    def operator_complexity(self):
        return sum(l["A"].nnz for l in self.levels) / self.levels[0]["A"].nnz


def block_preconditioner(hier_u, hier_p, d, Nu, nv, Q=None):
    """z = blockdiag(AMG(Lu) per displacement component, AMG(P_a) per network) r;
    with Q (J x J orthogonal) the pressure hierarchies act on the network
    eigenmodes: z_p = Q AMG_k((Q^T r_p)_k) vertex by vertex."""
    J = len(hier_p)

    def apply(r):
        z = np.empty_like(r)
        ru = r[:Nu].reshape(-1, d)
        zu = np.stack([hier_u.vcycle(np.ascontiguousarray(ru[:, k])) for k in range(d)], 1)
        z[:Nu] = zu.ravel()
        rp = r[Nu:].reshape(J, nv)
        if Q is not None:
            rp = Q.T @ rp
        zp = np.stack([hier_p[a].vcycle(np.ascontiguousarray(rp[a])) for a in range(J)])
        if Q is not None:
            zp = Q @ zp
        z[Nu:] = zp.ravel()
        return z
    return apply


def minres(A, b, M=None, x0=None, rtol=1e-10, maxiter=1000):
    """Preconditioned MINRES (Paige-Saunders recurrences).

    Stops when the preconditioned residual estimate phibar <= rtol * beta1.
    Returns (x, iterations, history of phibar / beta1).
    """
    n = b.shape[0]
    x = np.zeros(n) if x0 is None else x0.copy()
    Mf = (lambda v: v) if M is None else M
    r1 = b - A @ x
    y = Mf(r1)
    beta1 = math.sqrt(max(float(r1 @ y), 0.0))
    hist = [1.0]
    if beta1 == 0.0:
        return x, 0, hist
    oldb, beta, dbar, epsln, phibar = 0.0, beta1, 0.0, 0.0, beta1
    cs, sn = -1.0, 0.0
    w = np.zeros(n)
    w2 = np.zeros(n)
    r2 = r1.copy()
    it = 0
    while it < maxiter:
        it += 1
        s = 1.0 / beta
        v = s * y
        y = A @ v
        if it >= 2:
            y = y - (beta / oldb) * r1
        alfa = float(v @ y)
        y = y - (alfa / beta) * r2
        r1 = r2
        r2 = y
        y = Mf(r2)
        oldb = beta
        beta = math.sqrt(max(float(r2 @ y), 0.0))
        oldeps = epsln
        delta = cs * dbar + sn * alfa
        gbar = sn * dbar - cs * alfa
        epsln = sn * beta
        dbar = -cs * beta
        gamma = max(math.hypot(gbar, beta), 1e-300)
        cs = gbar / gamma
        sn = beta / gamma
        phi = cs * phibar
        phibar = sn * phibar
        w1 = w2
        w2 = w
        w = (v - oldeps * w1 - delta * w2) / gamma
        x = x + phi * w
        hist.append(phibar / beta1)
        if phibar <= rtol * beta1:
            break
    return x, it, hist
