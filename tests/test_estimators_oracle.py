"""The estimator oracle (oracle/estimators.py, adaptivempetsolver.py:82-227)
checked against an independent evaluation by numerical quadrature: second
derivatives of the P2 basis for div sigma(u), fields evaluated at Gauss points
of every cell and of every interior facet; the zero residuals of a linear
displacement with constant pressures; the marking rules (:10-61)."""
import math

import numpy as np
import pytest

import mms
from helpers import make_oracle


def _setup(dim, n=3, J=2, seed=0):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, UnitCubeMesh, UnitSquareMesh
    mesh = UnitSquareMesh(n) if dim == 2 else UnitCubeMesh(n)
    params = dict(J=J, E=10.0, nu=0.3, alpha=(0.5, 0.7), c=(0.2, 0.1), K=(0.3, 0.05),
                  S=((0.0, 0.4), (0.4, 0.0)))
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    om = make_oracle(problem, 1.0)
    rng = np.random.default_rng(seed)
    up = rng.standard_normal(om.dm.N)
    up_prev = rng.standard_normal(om.dm.N)
    f = rng.standard_normal((om.dm.nnodes, dim))
    f_ = rng.standard_normal((om.dm.nnodes, dim))
    g = rng.standard_normal((J, om.dm.nv))
    return om, up, up_prev, f, f_, g


def _brute(om, up, up_prev, dt, f, f_, g):
    """The same indicators by quadrature (degree-exact rules from tests/mms.py)."""
    from oracle import fem
    dm = om.dm
    d, J = dm.d, om.J
    lam, wt = mms.simplex_quadrature(d, 6)
    edges = fem.local_edges(d)
    phi = np.concatenate([lam * (2 * lam - 1)] + [4 * lam[:, [a]] * lam[:, [b]] for (a, b) in edges], 1)
    B = om.bgrad                                                   # (nc, n1, d)
    nc = B.shape[0]
    H = [4 * np.einsum("ck,cl->ckl", B[:, r], B[:, r]) for r in range(d + 1)]
    H += [4 * (np.einsum("ck,cl->ckl", B[:, a], B[:, b]) + np.einsum("ck,cl->ckl", B[:, b], B[:, a]))
          for (a, b) in edges]
    H = np.stack(H, 1)                                             # (nc, n2, d, d)
    gtab = fem.p2_gradient_vertex_values(B)                         # (nc, n2, n1, d)
    X = dm.x[dm.cells]
    h = np.sqrt(((X[:, :, None] - X[:, None]) ** 2).sum(-1)).reshape(nc, -1).max(1)
    mu, lm = om.mu, om.lmbda

    def fields(v):
        U = v[:dm.Nu].reshape(dm.nnodes, d)[dm.cell_nodes]
        D2 = np.einsum("cja,cjkl->cakl", U, H)                      # d2 u_a / dx_k dx_l
        divsig = (mu * (np.einsum("cakk->ca", D2) + np.einsum("cbab->ca", D2))
                  + lm * np.einsum("cbab->ca", D2))
        gq = np.einsum("qr,cjrk->cqjk", lam, gtab)                  # grad phi_j at the points
        Gq = np.einsum("cja,cqjb->cqab", U, gq)
        P = [v[dm.Nu + a * dm.nv: dm.Nu + (a + 1) * dm.nv] for a in range(J)]
        gp = [np.einsum("cr,crk->ck", p[dm.cells], B) for p in P]
        return U, divsig, Gq, P, gp
    U, ds, Gq, P, gp = fields(up)
    U_, ds_, Gq_, P_, gp_ = fields(up_prev)
    w = wt[None, :] * om.vol[:, None]
    cn = dm.cell_nodes
    fq = np.einsum("qj,cja->cqa", phi, f[cn])
    fq_ = np.einsum("qj,cja->cqa", phi, f_[cn])
    RK = fq + (ds - sum(om.alpha[a] * gp[a] for a in range(J)))[:, None]
    RK_ = fq_ + (ds_ - sum(om.alpha[a] * gp_[a] for a in range(J)))[:, None]
    eta_u = h ** 2 * np.sum(w[..., None] * RK ** 2, (1, 2))
    eta_udt = h ** 2 * np.sum(w[..., None] * ((RK - RK_) / dt) ** 2, (1, 2))
    divu = np.einsum("cqaa->cq", Gq)
    divu_ = np.einsum("cqaa->cq", Gq_)
    eta_p = np.zeros(nc)
    S = om.S
    for j in range(J):
        pq = lambda p: np.einsum("qr,cr->cq", lam, p[dm.cells])  # noqa: E731
        R = (-pq(g[j]) - om.c[j] * (pq(P[j]) - pq(P_[j])) / dt - om.alpha[j] * (divu - divu_) / dt
             - sum(S[i, j] * (pq(P[j]) - pq(P[i])) for i in range(J)))
        eta_p += h ** 2 * np.sum(w * R ** 2, 1)
    # interior facets by quadrature on the facet simplex
    from oracle.estimators import interior_facets
    rows, _ = interior_facets(dm.cells)
    if d == 2:
        gx, gw = np.polynomial.legendre.leggauss(6)
        flam = np.stack([0.5 * (1 - gx), 0.5 * (1 + gx)], 1)
        fw = 0.5 * gw
    else:
        flam, fw = mms.simplex_quadrature(2, 6)
    for (cp, op, cm, omn) in rows:
        vp = dm.cells[cp]
        verts = [r for r in range(d + 1) if r != op]
        xs = dm.x[vp[verts]]
        nvec = -B[cp, op] / np.linalg.norm(B[cp, op])
        area = d * om.vol[cp] * np.linalg.norm(B[cp, op])
        hav = 0.5 * (h[cp] + h[cm])
        acc = np.zeros(3)
        for qf in range(fw.shape[0]):
            xq = flam[qf] @ xs

            def grad_at(c, v):
                Xc = dm.x[dm.cells[c]]
                T = np.vstack([Xc.T, np.ones(d + 1)])
                lamc = np.linalg.solve(T, np.append(xq, 1.0))
                Uc = v[:dm.Nu].reshape(dm.nnodes, d)[dm.cell_nodes[c]]
                gph = np.einsum("r,jrk->jk", lamc, gtab[c])
                return np.einsum("ja,jb->ab", Uc, gph)

            def sig(G):
                return mu * (G + G.T) + lm * np.trace(G) * np.eye(d)
            e = -(sig(grad_at(cp, up)) - sig(grad_at(cm, up))) @ nvec
            e0 = -(sig(grad_at(cp, up_prev)) - sig(grad_at(cm, up_prev))) @ nvec
            acc[0] += fw[qf] * e @ e
            acc[1] += fw[qf] * ((e - e0) / dt) @ ((e - e0) / dt)
        rep = 0.0
        for j in range(J):
            Kj = float(np.mean(om.Kc[j]))
            rep += (Kj * (gp[j][cp] - gp[j][cm]) @ nvec) ** 2
        for c in (cp, cm):
            eta_u[c] += 0.5 * hav * area * acc[0]
            eta_udt[c] += 0.5 * hav * area * acc[1]
            eta_p[c] += 0.5 * hav * area * rep
    return eta_p, eta_u, eta_udt


@pytest.mark.parametrize("dim", [2, 3])
def test_indicators_match_quadrature(dim):
    from oracle.estimators import Estimators
    om, up, up_prev, f, f_, g = _setup(dim, n=3 if dim == 2 else 2)
    dt = 0.1
    est = Estimators(om)
    got = est.indicators(up, up_prev, dt, f, f_, g)
    ref = _brute(om, up, up_prev, dt, f, f_, g)
    for a, b in zip(got[:3], ref):
        assert np.allclose(a, b, rtol=1e-11, atol=1e-12 * np.abs(b).max())


@pytest.mark.parametrize("dim", [2, 3])
def test_linear_displacement_constant_pressure_has_zero_residuals(dim):
    from oracle.estimators import Estimators
    om, _, _, _, _, _ = _setup(dim, n=3 if dim == 2 else 2)
    dm = om.dm
    rng = np.random.default_rng(3)
    Aff = rng.standard_normal((dim, dim))
    u = dm.node_x @ Aff.T
    up = np.zeros(dm.N)
    up[:dm.Nu] = u.ravel()
    up[dm.Nu:] = 0.7
    est = Estimators(om)
    eta_p, eta_u, eta_udt, r4 = est.indicators(up, up, 0.1)
    # div sigma = 0, sigma continuous, grad p = 0; the mass residual keeps the transfer
    # and source terms only, which vanish for equal pressures and g = 0
    assert np.abs(eta_u).max() < 1e-20 and np.abs(eta_udt).max() < 1e-20
    assert np.abs(eta_p).max() < 1e-20 and abs(r4) < 1e-20


def test_marking_rules():
    from oracle.estimators import dorfler_mark, maximal_mark
    etas = np.array([0.1, 0.5, 0.2, 0.05, 0.15])
    assert maximal_mark(etas, 0.4).tolist() == [False, True, True, False, False]
    assert maximal_mark(etas, 1.0).all() and not maximal_mark(etas, 0.0).any()
    # 0.5 covers 0.5 of 1.0 => stop before the next one when fraction = 0.5
    assert dorfler_mark(etas, 0.5).tolist() == [False, True, False, False, False]
    assert dorfler_mark(etas, 0.6).tolist() == [False, True, True, False, False]
    assert not dorfler_mark(etas, 0.0).any()


@pytest.mark.parametrize("dim,n", [(2, 4), (3, 3)])
def test_host_facet_tables_match_oracle(dim, n):
    """The engine's interior-facet tables (built on the host) equal the oracle's."""
    from oracle.estimators import interior_facets
    from waterscapes_gb300 import UnitCubeMesh, UnitSquareMesh
    from waterscapes_gb300.adaptive import interior_facet_tables
    mesh = UnitSquareMesh(n) if dim == 2 else UnitCubeMesh(n)
    a, b = interior_facet_tables(mesh.cells())
    ra, rb = interior_facets(mesh.cells())
    assert np.array_equal(a, ra) and np.array_equal(b, rb)
    # every interior facet appears twice in the cell table, boundary facets not at all
    nb = mesh.num_boundary_facets()
    assert (b >= 0).sum() == 2 * a.shape[0]
    assert (b < 0).sum() == nb


def test_host_marking_rules_match_oracle():
    from oracle.estimators import dorfler_mark as od, maximal_mark as om_
    from waterscapes_gb300.adaptive import dorfler_mark, maximal_mark
    rng = np.random.default_rng(2)
    etas = np.round(rng.random(200), 2)                 # ties included
    for fr in (0.0, 0.1, 0.33, 0.5, 0.9, 1.0):
        assert np.array_equal(maximal_mark(etas, fr), om_(etas, fr))
        assert np.array_equal(dorfler_mark(etas, fr), od(etas, fr))
