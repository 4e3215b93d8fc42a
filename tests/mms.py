"""Manufactured solutions and error norms for the MPET convergence tests.

Restates the setup of src/mpet/test/test_convergence_mpetsolver.py:21-179:
u_k = sin(2 pi x + pi/2) sin(2 pi y + pi/2) sin(omega t + t), omega = 2 pi,
p_i = -i * (same), total pressure p0 = lambda div u - sum alpha_i p_i,
sigma = 2 mu eps(u) + p0 I, f = -div sigma and
g_i = -c_i dp_i/dt - alpha_i/lambda d/dt(p0 + sum_j alpha_j p_j)
      + div(K_i grad p_i) - sum_j S_ij (p_i - p_j).
Dirichlet data everywhere except a traction (sigma n) on the x = 1 edge.
3D variant: same construction with a third factor sin(2 pi z + pi/2).
"""
from __future__ import annotations

import math

import numpy as np
import sympy


def exact_solutions(params, dim=2):
    J = params["J"]
    nu, E = params["nu"], params["E"]
    alpha, c, K, S = params["alpha"], params["c"], params["K"], params["S"]
    lmbda = nu * E / ((1.0 - 2.0 * nu) * (1.0 + nu))
    mu = E / (2.0 * (1.0 + nu))
    pi = sympy.pi
    x = sympy.symbols("x0:%d" % dim)
    t = sympy.symbols("t")
    phi = sympy.sin(2 * pi * t + t)
    for k in range(dim):
        phi = phi * sympy.sin(2 * pi * x[k] + pi / 2)
    u = [phi for _ in range(dim)]
    p = [0] + [-(i) * phi for i in range(1, J + 1)]
    div_u = sum(sympy.diff(u[i], x[i]) for i in range(dim))
    p[0] = lmbda * div_u - sum(alpha[i] * p[i + 1] for i in range(J))
    grad_u = [[sympy.diff(u[i], x[j]) for j in range(dim)] for i in range(dim)]
    eps = [[(grad_u[i][j] + grad_u[j][i]) / 2 for j in range(dim)] for i in range(dim)]
    sigma = [[2 * mu * eps[i][j] + (p[0] if i == j else 0) for j in range(dim)] for i in range(dim)]
    f = [-sum(sympy.diff(sigma[i][j], x[j]) for j in range(dim)) for i in range(dim)]
    g = []
    for i in range(J):
        gi = (-c[i] * sympy.diff(p[i + 1], t)
              - alpha[i] / lmbda * sympy.diff(p[0] + sum(alpha[j] * p[j + 1] for j in range(J)), t)
              + sum(sympy.diff(K[i] * sympy.diff(p[i + 1], x[j]), x[j]) for j in range(dim))
              - sum(S[i][j] * (p[i + 1] - p[j + 1]) for j in range(J)))
        g.append(gi)
    args = list(x) + [t]
    lam = lambda e: sympy.lambdify(args, e, "numpy")
    U = [lam(e) for e in u]
    dU = [[lam(sympy.diff(u[i], x[j])) for j in range(dim)] for i in range(dim)]
    P = [lam(e) for e in p[1:]]
    P0 = lam(p[0])
    dP = [[lam(sympy.diff(p[i + 1], x[j])) for j in range(dim)] for i in range(J)]
    F = [lam(e) for e in f]
    G = [lam(e) for e in g]
    SIG = [[lam(sigma[i][j]) for j in range(dim)] for i in range(dim)]

    def bcast(fn, xx, tt):
        v = fn(*[xx[:, k] for k in range(dim)], tt)
        return np.broadcast_to(np.asarray(v, dtype=np.float64), (xx.shape[0],)).copy()

    data = {
        "u_bar": lambda xx, tt: np.stack([bcast(U[k], xx, tt) for k in range(dim)], 1),
        "p_bar": [(lambda i: (lambda xx, tt: bcast(P[i], xx, tt)))(i) for i in range(J)],
        "f": lambda xx, tt: np.stack([bcast(F[k], xx, tt) for k in range(dim)], 1),
        "g": [(lambda i: (lambda xx, tt: bcast(G[i], xx, tt)))(i) for i in range(J)],
        "s": lambda xx, tt, nn: np.stack(
            [sum(bcast(SIG[i][j], xx, tt) * nn[:, j] for j in range(dim)) for i in range(dim)], 1),
    }
    exact = {
        "u": lambda xx, tt: np.stack([bcast(U[k], xx, tt) for k in range(dim)], 1),
        "du": lambda xx, tt: np.stack([np.stack([bcast(dU[i][j], xx, tt) for j in range(dim)], 1)
                                       for i in range(dim)], 1),
        "p": [(lambda i: (lambda xx, tt: bcast(P[i], xx, tt)))(i) for i in range(J)],
        "p0": lambda xx, tt: bcast(P0, xx, tt),
        "dp": [(lambda i: (lambda xx, tt: np.stack([bcast(dP[i][j], xx, tt) for j in range(dim)], 1)))(i)
               for i in range(J)],
    }
    return data, exact


def simplex_quadrature(d, n=6):
    """Collapsed Gauss rule on the d-simplex: barycentric points, weights summing to 1."""
    g, w = np.polynomial.legendre.leggauss(n)
    g = 0.5 * (g + 1.0)
    w = 0.5 * w
    if d == 2:
        U, V = np.meshgrid(g, g, indexing="ij")
        WU, WV = np.meshgrid(w, w, indexing="ij")
        xi = U.ravel()
        eta = (V * (1 - U)).ravel()
        wt = (WU * WV * (1 - U)).ravel() * 2.0
        lam = np.stack([1 - xi - eta, xi, eta], 1)
        return lam, wt
    U, V, W = np.meshgrid(g, g, g, indexing="ij")
    WU, WV, WW = np.meshgrid(w, w, w, indexing="ij")
    a = U.ravel()
    b = (V * (1 - U)).ravel()
    cc = (W * (1 - U) * (1 - V)).ravel()
    wt = (WU * WV * WW * (1 - U) ** 2 * (1 - V)).ravel() * 6.0
    lam = np.stack([1 - a - b - cc, a, b, cc], 1)
    return lam, wt


def errornorms(om, up, t, exact):
    """L2 and H1 (full) errors of u and each p_a at time t, high-order quadrature."""
    from oracle import fem
    dm = om.dm
    d, J = dm.d, dm.J if hasattr(dm, "J") else om.J
    J = om.J
    lam, wt = simplex_quadrature(d, 6 if d == 2 else 5)
    cells = dm.cells
    X = dm.x[cells]                                   # (nc, d+1, d)
    xq = np.einsum("qr,crk->cqk", lam, X)             # (nc, nq, d)
    nc, nq = xq.shape[0], xq.shape[1]
    xf = xq.reshape(-1, d)
    edges = fem.local_edges(d)
    n1 = d + 1
    phi = np.concatenate([lam * (2 * lam - 1)] + [4 * lam[:, [a]] * lam[:, [b]] for (a, b) in edges], 1)
    g = fem.p2_gradient_vertex_values(om.bgrad)        # (nc, n2, n1, d)
    dphi = np.einsum("qr,cirk->cqik", lam, g)          # (nc, nq, n2, d)
    cn = dm.cell_nodes
    U = up[:dm.Nu].reshape(dm.nnodes, d)[cn]          # (nc, n2, d)
    uh = np.einsum("qi,cik->cqk", phi, U)
    duh = np.einsum("cqij,cik->cqkj", dphi, U)        # [c,q,comp,deriv]
    ue = exact["u"](xf, t).reshape(nc, nq, d)
    due = exact["du"](xf, t).reshape(nc, nq, d, d)
    vol = om.vol[:, None]
    w = wt[None, :] * vol
    eL2 = np.sum(w[..., None] * (uh - ue) ** 2)
    eH1 = eL2 + np.sum(w[..., None, None] * (duh - due) ** 2)
    res = {"uL2": math.sqrt(eL2), "uH1": math.sqrt(eH1), "pL2": [], "pH1": []}
    for a in range(J):
        P = up[dm.Nu + a * dm.nv: dm.Nu + (a + 1) * dm.nv][cells]
        ph = np.einsum("qr,cr->cq", lam, P)
        dph = np.einsum("crk,cr->ck", om.bgrad, P)[:, None, :]
        pe = exact["p"][a](xf, t).reshape(nc, nq)
        dpe = exact["dp"][a](xf, t).reshape(nc, nq, d)
        l2 = np.sum(w * (ph - pe) ** 2)
        h1 = l2 + np.sum(w[..., None] * (dph - dpe) ** 2)
        res["pL2"].append(math.sqrt(l2))
        res["pH1"].append(math.sqrt(h1))
    return res


def rates(errors, hs):
    return [math.log(errors[i + 1] / errors[i]) / math.log(hs[i + 1] / hs[i]) for i in range(len(hs) - 1)]
