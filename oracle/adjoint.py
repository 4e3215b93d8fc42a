"""FP64 discrete adjoint of the MPET time loop (test infrastructure, oracle).

The reference has no adjoint: this differentiates the oracle's own
restatement of ``solve_direct`` (mpetsolver.py:382-462, forms :196-261) with
respect to the per-cell permeability fields K_a (DG0).

Forward, per step n = 1..N, with x_n = E_F y_n + E_D g_n (free / Dirichlet):

    A(K)_FF y_n = (B(K) x_{n-1} + f_n)_F - A(K)_FD g_n

where A is the assembled matrix and B the old-state operator of L = rhs(F):
the pressure rows -alpha_a (div u, q) - c_a (p_a, q)
+ dt (1-theta) [K_a (grad p_a, grad q) + sum_b S_ab (p_a - p_b, q)]
(the momentum rows of L hold no state).  The loss is the L2 misfit of the
final pressures, 1/2 sum_a (p_a - p*_a)^T M (p_a - p*_a), M the P1 mass
matrix.  The adjoint runs backwards:

    A_FF^T lam_N = (W (x_N - x*))_F,    A_FF^T lam_n = (B^T lam_{n+1})_F,

lam zero on the Dirichlet DOFs, and, because dA/dK_a(e) = -dt theta L_e and
dB/dK_a(e) = dt (1-theta) L_e on the p_a block (L_e the element stiffness),

    dL/dK_a(e) = dt sum_n |e| grad lam_a,n . grad(theta p_a,n + (1-theta) p_a,n-1).

Robin terms are not differentiated for theta < 1 (their (1-theta) part sits
in B); the solver raises for that combination.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import fem


def old_state_matrix(om, dt):
    """B with rhs_L(x) == B @ x (mpetsolver.py:196-201, 261)."""
    d, J = om.d, om.J
    dm = om.dm
    nc = om.vol.shape[0]
    n2, n1 = dm.nloc2, d + 1
    th = om.theta
    Cf = om.C.reshape(nc, d * n2, n1)
    Ssum = om.S.sum(axis=1)
    nloc = dm.nloc
    Be = np.zeros((nc, nloc, nloc))
    for a in range(J):
        o = d * n2 + a * n1
        Be[:, o:o + n1, :d * n2] = -om.alpha[a] * np.transpose(Cf, (0, 2, 1))
        for b_ in range(J):
            ob = d * n2 + b_ * n1
            blk = -dt * (1.0 - th) * om.S[a, b_] * om.M1
            if a == b_:
                blk = blk + (-om.c[a] + dt * (1.0 - th) * Ssum[a]) * om.M1 \
                    + dt * (1.0 - th) * om.Kc[a][:, None, None] * om.L1
            Be[:, o:o + n1, ob:ob + n1] += blk
    cd = om.cell_dofs
    rows = np.repeat(cd, nloc, axis=1).ravel()
    cols = np.tile(cd, (1, nloc)).ravel()
    return sp.coo_matrix((Be.ravel(), (rows, cols)), shape=(dm.N, dm.N)).tocsr()


def pressure_mass(om):
    """W: the P1 mass matrix on every pressure block, zero on the displacement rows."""
    dm = om.dm
    M = fem.assemble_csr(dm.cells, om.M1, dm.nv)
    blocks = [sp.csr_matrix((dm.Nu, dm.Nu))] + [M] * om.J
    return sp.block_diag(blocks, format="csr")


def misfit(om, x, p_target):
    """(loss, dloss/dx) of 1/2 sum_a (p_a - p*_a)^T M (p_a - p*_a); p_target is (J, nv)."""
    dm = om.dm
    W = pressure_mass(om)
    diff = np.zeros(dm.N)
    diff[dm.Nu:] = x[dm.Nu:] - np.asarray(p_target, dtype=np.float64).ravel()
    g = W @ diff
    return 0.5 * float(diff @ g), g


def forward(om, up0, t0, nsteps, dt, data):
    """States x_0..x_N of the solve_direct loop (LU)."""
    T = t0 + nsteps * dt
    xs = [np.array(up0, dtype=np.float64)]
    for up, t in om.solve_direct(up0, t0, T - 0.5 * dt, dt, data):
        xs.append(up.copy())
    return xs


def gradient(om, xs, p_target, dt, data=None, t0=0.0):
    """(loss, dL/dK) with dL/dK of shape (J, nc), from the states of ``forward``."""
    data = data or {}
    if om.theta < 1.0 and data.get("beta") is not None:
        raise NotImplementedError("Robin terms are not differentiated for theta < 1")
    dm = om.dm
    A = om.assemble_matrix(dt, t0, data)
    dofs = om.dirichlet_dofs()
    bc = np.unique(np.concatenate([dd for _, dd in dofs]))
    As, _ = om.zero_rows_columns(A, [bc])
    lu = spla.splu(As.T.tocsc())
    B = old_state_matrix(om, dt)
    loss, seed = misfit(om, xs[-1], p_target)
    th = om.theta
    cells = dm.cells
    grad = np.zeros((om.J, om.vol.shape[0]))
    for n in range(len(xs) - 1, 0, -1):
        seed = seed.copy()
        seed[bc] = 0.0
        lam = lu.solve(seed)
        for a in range(om.J):
            base = dm.Nu + a * dm.nv
            la = lam[base + cells]
            q = th * xs[n][base + cells] + (1.0 - th) * xs[n - 1][base + cells]
            grad[a] += dt * np.einsum("cvw,cv,cw->c", om.L1, la, q)
        seed = B.T @ lam
    return loss, grad
