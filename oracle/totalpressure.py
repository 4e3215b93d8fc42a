"""FP64 CPU restatement of ``MPETTotalPressureSolver`` (test infrastructure, oracle).

The total-pressure formulation adds the field p0 = lambda div u - sum_i alpha_i p_i
(src/mpet/mpet/mpettotalpressuresolver.py:164-305).  Unknowns in block-natural
order: u (P2 vector), p0 (P1), p_1 .. p_A (P1), so the pressure fields of this
oracle are numbered 0..A with field 0 the total pressure.  Forms
(mpettotalpressuresolver.py:262-270, theta-weighted pm for the network fields):

    2 mu (eps u, eps v) + (p0, div v)
  + (div u - p0 / lambda - sum_i alpha_i p_i / lambda, w0)
  - sum_i c_i (p_i - p_i^-, w_i)
  - sum_i alpha_i / lambda (p0 - p0^- + sum_j alpha_j (p_j - p_j^-), w_i)
  - sum_i dt K_i (grad pm_i, grad w_i) - sum_ij dt S_ij (pm_i - pm_j, w_i)

with L0, L1 and the Robin form L2 as in the MPET solver, the network terms
carried by fields 1..A, and no boundary condition on p0
(mpettotalpressuresolver.py:117-137).  The preconditioner form
(mpettotalpressuresolver.py:276-283): mu (grad u, grad v) + (p0, w0)
+ sum_i [alpha_i^2 / lambda + c_i + dt theta sum_{j != i} S_ij] (p_i, w_i)
+ dt theta K_i (grad p_i, grad w_i).  The time loop is ``solve_direct``
(mpettotalpressuresolver.py:331-395): the same time levels as the MPET solver.
"""
from __future__ import annotations

import numpy as np

from . import fem
from .mpet import OracleMPET


def expand_params(params):
    """MPET-style parameters over the A + 1 pressure fields: field 0 is p0 (alpha 1
    in the rank-one coupling, c = K = S = 0), fields 1..A are the networks."""
    A = int(params["J"])
    S = np.zeros((A + 1, A + 1))
    S[1:, 1:] = np.asarray(params["S"], dtype=np.float64).reshape(A, A)
    out = dict(params)
    out.update(J=A + 1, alpha=(1.0,) + tuple(float(a) for a in params["alpha"]),
               c=(0.0,) + tuple(float(a) for a in params["c"]),
               K=(0.0,) + tuple(params["K"]), S=tuple(map(tuple, S)))
    return out


def expand_data(data):
    """Per-network data lists (g, I, beta, p_robin, p_bar) shifted by the p0 field."""
    data = dict(data or {})
    for key in ("g", "I", "beta", "p_robin", "p_bar"):
        if data.get(key) is not None:
            data[key] = [None] + list(data[key])
    return data


class OracleTotalPressure(OracleMPET):
    """``params`` are the problem's (J = number of networks A); continuity markers
    are given per network; the p0 field carries no boundary condition."""

    def __init__(self, x, cells, bfacets, bfacet_cells, params, theta=0.5,
                 momentum_markers=None, continuity_markers=None):
        A = int(params["J"])
        nf = np.asarray(bfacets).shape[0]
        cm = None
        if continuity_markers is not None:
            cm = [np.full(nf, -1)] + [np.asarray(continuity_markers[a]) for a in range(A)]
        super().__init__(x, cells, bfacets, bfacet_cells, expand_params(params), theta, momentum_markers, cm)
        self.A = A
        self.beta_tp = np.asarray(self.alpha, dtype=np.float64)    # (1, alpha_1 .. alpha_A)

    def local_matrix(self, dt, beta_cells=None):
        d, J = self.d, self.J
        nc = self.vol.shape[0]
        n2 = self.dm.nloc2
        n1 = d + 1
        mu, lm, th = self.mu, self.lmbda, self.theta
        Mg = self.Mg
        tr = np.einsum("cijkk->cij", Mg)
        uu = mu * np.einsum("cij,kl->cikjl", tr, np.eye(d)) + mu * np.transpose(Mg, (0, 1, 4, 2, 3))
        Ae = np.zeros((nc, self.dm.nloc, self.dm.nloc))
        Ae[:, :d * n2, :d * n2] = uu.reshape(nc, d * n2, d * n2)
        Cf = self.C.reshape(nc, d * n2, n1)
        o0 = d * n2
        Ae[:, :d * n2, o0:o0 + n1] = Cf
        Ae[:, o0:o0 + n1, :d * n2] = np.transpose(Cf, (0, 2, 1))
        Ssum = self.S.sum(axis=1)
        bt = self.beta_tp
        for a in range(J):
            o = d * n2 + a * n1
            for b_ in range(J):
                ob = d * n2 + b_ * n1
                blk = (-bt[a] * bt[b_] / lm - dt * th * (Ssum[a] * (a == b_) - self.S[a, b_])) * self.M1
                if a == b_:
                    blk = blk - self.c[a] * self.M1 - dt * th * self.Kc[a][:, None, None] * self.L1
                Ae[:, o:o + n1, ob:ob + n1] += blk
        return Ae

    def rhs_L(self, up_prev, dt):
        """b = assemble(L): the previous-time terms of the network rows."""
        d, J = self.d, self.J
        dm = self.dm
        th = self.theta
        n1 = d + 1
        nc = self.vol.shape[0]
        cd = self.cell_dofs
        n2 = dm.nloc2
        p_loc = [up_prev[cd[:, d * n2 + a * n1: d * n2 + (a + 1) * n1]] for a in range(J)]
        bt = self.beta_tp
        mp = [np.einsum("cvw,cw->cv", self.M1, p_loc[a]) for a in range(J)]
        tot = sum(bt[b_] * mp[b_] for b_ in range(J))
        bl = np.zeros((nc, dm.nloc))
        for a in range(1, J):
            o = d * n2 + a * n1
            val = -self.c[a] * mp[a] - bt[a] / self.lmbda * tot
            val += dt * (1.0 - th) * self.Kc[a][:, None] * np.einsum("cvw,cw->cv", self.L1, p_loc[a])
            for b_ in range(J):
                coef = self.S[a, b_]
                if coef != 0.0:
                    val += dt * (1.0 - th) * coef * (mp[a] - mp[b_])
            bl[:, o:o + n1] = val
        return fem.assemble_vector(cd, bl, dm.N)

    def step(self, up_prev, t0, dt, data=None, return_system=False):
        return super().step(up_prev, t0, dt, expand_data(data), return_system)

    def solve_direct(self, up0, t0, T, dt, data=None):
        return super().solve_direct(up0, t0, T, dt, expand_data(data))

    def dirichlet_values(self, t, data):
        if data is not None and data.get("p_bar") is not None and len(data["p_bar"]) == self.A:
            data = expand_data(data)
        return super().dirichlet_values(t, data)

    def preconditioner_blocks(self, dt, u_weight=None, p0_weight=1.0, modes=None):
        """mu (grad u, grad v), p0_weight (p0, w0) and the network blocks of
        mpettotalpressuresolver.py:276-283, Dirichlet DOFs eliminated."""
        dm = self.dm
        tr = np.einsum("cijkk->cij", self.Mg)
        w = self.mu if u_weight is None else float(u_weight)
        Lu = fem.assemble_csr(dm.cell_nodes, w * tr, dm.nnodes)
        bcs = self.dirichlet_dofs()
        Lu, _ = self.zero_rows_columns(Lu, [bcs[0][0]])
        blocks = [Lu, fem.assemble_csr(dm.cells, p0_weight * self.M1, dm.nv)]
        th = self.theta
        for a in range(1, self.J):
            sS = sum(self.S[a, b_] for b_ in range(self.J) if b_ != a)
            m = self.alpha[a] ** 2 / self.lmbda + self.c[a] + dt * th * sS
            loc = m * self.M1 + dt * th * self.Kc[a][:, None, None] * self.L1
            Pa = fem.assemble_csr(dm.cells, loc, dm.nv)
            Pa, _ = self.zero_rows_columns(Pa, [bcs[1 + a][0]])
            blocks.append(Pa)
        return blocks
