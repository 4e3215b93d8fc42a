"""FP64 CPU restatement of the ``AdaptiveMPETSolver`` error estimators
(test infrastructure, oracle).

Follows src/mpet/mpet/adaptivempetsolver.py:82-227:

* cell and interior-facet residuals of the momentum equation (:122-128),
  RK_u = f + div sigma(u) - sum_i grad(alpha_i p_i) and
  RE_u = sum_i jump(alpha_i p_i, n) - jump(sigma(u), n), and their values at the
  previous time with f_ (:126-128);
* residuals of the mass equations (:132-136), RK_p_j = -g_j - c_j (p_j - p_j^-)/dt
  - alpha_j div(u - u^-)/dt + K_j div grad p_j - sum_i S_ij (p_j - p_i) and
  RE_p_j = -K_j jump(grad p_j, n);
* the DG0 indicators (:144-146)
  zeta_u_K = h^2 ||RK_u||_K^2 + sum_F avg(h) avg(w) ||RE_u||_F^2 (interior facets),
  zeta_p_K (sum over networks), zeta_u_dt_K (the residuals' difference quotient);
* R4p (:148-155) = sum_j ||K_j^1/2 grad(p_j - p_j^-)||^2
  + sum_{i: S_ij > eps} (S_ij ((p_j - p_j^-) - (p_i - p_i^-)), p_j - p_j^-);
* the time bookkeeping of estimate_error_at_t, add_to_indicators,
  compute_error_indicators and compute_error_estimate (:170-227) and the marking
  rules maximal_mark / dorfler_mark (:10-61).

Quadrature is exact for the discrete fields: u in P2, p in P1, f and f_ as P2
interpolants (the right-hand side's convention) and g as P1 interpolants, so
every integrand is a polynomial integrated with the mass matrices.  h is the
cell diameter (largest vertex distance, UFL ``CellDiameter``).  The pressure
jump term of RE_u vanishes for continuous P1 pressures and is not formed.
"""
from __future__ import annotations

import math

import numpy as np

from . import fem

DOLFIN_EPS = 3.0e-16


def interior_facets(cells):
    """Interior facets of a simplicial mesh: (nfi, 4) rows (cell+, local vertex
    opposite the facet in cell+, cell-, its local opposite vertex) with cell+ <
    cell-, ordered by the facet's sorted vertex tuple; and (nc, d+1) ids of the
    interior facet opposite each local vertex (-1 on the boundary)."""
    cells = np.sort(np.asarray(cells, dtype=np.int64), axis=1)
    nc, n1 = cells.shape
    keys = []
    for k in range(n1):
        keys.append(np.delete(cells, k, axis=1))
    F = np.stack(keys, 1).reshape(nc * n1, n1 - 1)               # facet k of cell c at c * n1 + k
    uniq, inv, cnt = np.unique(F, axis=0, return_inverse=True, return_counts=True)
    inv = inv.ravel()
    order = np.argsort(inv, kind="stable")
    ids = inv[order]
    first = np.ones(ids.shape[0], dtype=bool)
    first[1:] = ids[1:] != ids[:-1]
    starts = np.nonzero(first)[0]
    interior = cnt[ids[starts]] == 2
    a = order[starts[interior]]
    b = order[starts[interior] + 1]
    rows = np.stack([a // n1, a % n1, b // n1, b % n1], 1)
    cell_facets = np.full(nc * n1, -1, dtype=np.int64)
    cell_facets[a] = np.arange(a.shape[0])
    cell_facets[b] = np.arange(a.shape[0])
    return rows.astype(np.int64), cell_facets.reshape(nc, n1)


class Estimators:
    """Indicators of one MPET state pair (up, up_prev) on the mesh of an OracleMPET."""

    def __init__(self, om):
        self.om = om
        dm = om.dm
        self.d = dm.d
        self.ifacets, self.cell_facets = interior_facets(dm.cells)
        X = dm.x[dm.cells]
        diff = X[:, :, None, :] - X[:, None, :, :]
        self.h = np.sqrt((diff ** 2).sum(-1)).reshape(X.shape[0], -1).max(1)
        self.g = fem.p2_gradient_vertex_values(om.bgrad)            # (nc, n2, n1, d)

    def _fields(self, up):
        om, dm, d = self.om, self.om.dm, self.d
        U = up[:dm.Nu].reshape(dm.nnodes, d)[dm.cell_nodes]          # (nc, n2, d)
        G = np.einsum("cja,cjrb->crab", U, self.g)                   # grad u at the vertices
        tr = np.einsum("craa->cr", G)
        sig = om.mu * (G + np.swapaxes(G, 2, 3)) + om.lmbda * tr[:, :, None, None] * np.eye(d)
        divsig = np.einsum("crab,crb->ca", sig, om.bgrad)
        P = [up[dm.Nu + a * dm.nv: dm.Nu + (a + 1) * dm.nv] for a in range(om.J)]
        gradp = [np.einsum("cr,crk->ck", p[dm.cells], om.bgrad) for p in P]
        return sig, tr, divsig, P, gradp

    def indicators(self, up, up_prev, dt, f_nodes=None, f_prev_nodes=None, g_vert=None):
        """(eta_p_K, eta_u_K, eta_u_dt_K, R4p) for the step up_prev -> up."""
        om, dm, d, J = self.om, self.om.dm, self.d, self.om.J
        sig, tr, divsig, P, gradp = self._fields(up)
        sig_, tr_, divsig_, P_, gradp_ = self._fields(up_prev)
        nc = dm.cells.shape[0]
        zf = np.zeros((dm.nnodes, d))
        f = zf if f_nodes is None else np.asarray(f_nodes).reshape(dm.nnodes, d)
        f_ = zf if f_prev_nodes is None else np.asarray(f_prev_nodes).reshape(dm.nnodes, d)
        cn = dm.cell_nodes
        RKc = divsig - sum(om.alpha[a] * gradp[a] for a in range(J))
        RKc_ = divsig_ - sum(om.alpha[a] * gradp_[a] for a in range(J))
        RK = f[cn] + RKc[:, None, :]
        RK_ = f_[cn] + RKc_[:, None, :]
        RKdt = (RK - RK_) / dt
        quad2 = lambda V: np.einsum("cia,cij,cja->c", V, om.M2, V)  # noqa: E731
        h2 = self.h ** 2
        eta_u = h2 * quad2(RK)
        eta_udt = h2 * quad2(RKdt)
        S = om.S
        eta_p = np.zeros(nc)
        for j in range(J):
            gj = np.zeros(dm.nv) if g_vert is None else np.asarray(g_vert)[j]
            R = (-gj[dm.cells] - om.c[j] * (P[j] - P_[j])[dm.cells] / dt
                 - om.alpha[j] * (tr - tr_) / dt
                 - sum(S[i, j] * (P[j] - P[i])[dm.cells] for i in range(J)))
            eta_p += h2 * np.einsum("cv,cvw,cw->c", R, om.M1, R)
        # interior facets
        cp, op, cm, omn = (self.ifacets[:, k] for k in range(4))
        bo = om.bgrad[cp, op]                                         # (nfi, d)
        nb = np.linalg.norm(bo, axis=1)
        n = -bo / nb[:, None]
        area = d * om.vol[cp] * nb
        havg = 0.5 * (self.h[cp] + self.h[cm])
        vp = dm.cells[cp]
        vm = dm.cells[cm]
        nfi = cp.shape[0]
        e = np.zeros((nfi, d, d))
        e_ = np.zeros((nfi, d, d))
        for r in range(d + 1):
            keep = op != r
            # local index of the same vertex in cell-
            rm = np.argmax(vm == vp[:, r][:, None], axis=1)
            sp_ = sig[cp, r] - sig[cm, rm]
            sp0 = sig_[cp, r] - sig_[cm, rm]
            val = -np.einsum("fab,fb->fa", sp_, n)
            val0 = -np.einsum("fab,fb->fa", sp0, n)
            # facet vertex slot: position of r among the vertices other than op
            slot = r - (op < r).astype(np.int64)
            idx = np.nonzero(keep)[0]
            e[idx, slot[idx]] = val[idx]
            e_[idx, slot[idx]] = val0[idx]
        cF = area / (d * (d + 1))

        def facet_quad(E):
            return cF * ((E ** 2).sum((1, 2)) + (E.sum(1) ** 2).sum(1))
        fu = 0.5 * havg * facet_quad(e)
        fudt = 0.5 * havg * facet_quad((e - e_) / dt)
        fp = np.zeros(nfi)
        for j in range(J):
            Kj = float(np.mean(om.Kc[j]))
            RE = -Kj * np.einsum("fk,fk->f", gradp[j][cp] - gradp[j][cm], n)
            fp += 0.5 * havg * area * RE ** 2
        for k in range(d + 1):
            fid = self.cell_facets[:, k]
            ok = fid >= 0
            eta_u[ok] += fu[fid[ok]]
            eta_udt[ok] += fudt[fid[ok]]
            eta_p[ok] += fp[fid[ok]]
        # R4p
        r4 = 0.0
        dP = [P[j] - P_[j] for j in range(J)]
        for j in range(J):
            Kj = float(np.mean(om.Kc[j]))
            gd = np.einsum("cr,crk->ck", dP[j][dm.cells], om.bgrad)
            r4 += Kj * float(np.sum(om.vol * (gd ** 2).sum(1)))
            for i in range(J):
                if S[i, j] > DOLFIN_EPS:
                    a = (dP[j] - dP[i])[dm.cells]
                    b = dP[j][dm.cells]
                    r4 += S[i, j] * float(np.einsum("cv,cvw,cw->", a, om.M1, b))
        return eta_p, eta_u, eta_udt, r4


class EstimatorHistory:
    """The lists and indicator fields of adaptivempetsolver.py:157-227."""

    def __init__(self, nc):
        self.eta_1s, self.eta_2s, self.eta_3s, self.eta_4s = [], [], [], []
        self.eta_1Ks = np.zeros(nc)
        self.eta_2Ks = np.zeros(nc)
        self.eta_3Ks = np.zeros(nc)

    def estimate(self, eta_p_K, eta_u_K, eta_u_dt_K, r4p, tau):
        self.eta_1s.append(tau * eta_p_K.sum())
        self.eta_2s.append(eta_u_K.sum())
        self.eta_3s.append(tau * math.sqrt(eta_u_dt_K.sum()))
        self.eta_4s.append(tau * r4p)

    def add_to_indicators(self, eta_p_K, eta_u_K, eta_u_dt_K, tau):
        self.eta_1Ks += tau * eta_p_K
        self.eta_3Ks = tau * np.sqrt(eta_u_dt_K)
        self.eta_2Ks = np.maximum(self.eta_2Ks, eta_u_K)

    def error_indicators(self):
        return self.eta_2Ks + self.eta_3Ks + np.sqrt(self.eta_1Ks)

    def error_estimate(self):
        etas = (math.sqrt(sum(self.eta_1s)), math.sqrt(max(self.eta_2s)), sum(self.eta_3s),
                math.sqrt(sum(self.eta_4s)))
        return sum(etas), etas


def maximal_mark(etas, fraction):
    """adaptivempetsolver.py:10-32."""
    etas = np.asarray(etas)
    marked = np.zeros(etas.shape[0], dtype=bool)
    marked[np.argsort(-etas)[:math.ceil(fraction * etas.shape[0])]] = True
    return marked


def dorfler_mark(etas, fraction):
    """adaptivempetsolver.py:34-61 (sequential accumulation in sorted order)."""
    etas = np.asarray(etas)
    marked = np.zeros(etas.shape[0], dtype=bool)
    stop = fraction * np.sum(etas)
    eta = 0.0
    for i in np.argsort(-etas):
        if eta >= stop:
            break
        marked[i] = True
        eta += etas[i]
    return marked
