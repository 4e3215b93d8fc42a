"""FP64 CPU restatement of ``MPETSolver`` (test infrastructure, oracle).

Follows, line by line in meaning:

* forms ``a``, ``L``, ``L0``, ``L1`` and the Robin split:
  src/mpet/mpet/mpetsolver.py:178-261;
* the block-diagonal preconditioner form: mpetsolver.py:264-271 (with
  ``dt*theta*inner(...)`` in place of the ``dt*theta**inner(...)`` typo at
  :270, as in the working twin mpettotalpressuresolver.py:276-283);
* ``step``: mpetsolver.py:317-379 and ``solve_direct``: mpetsolver.py:382-462
  (time levels: ``L`` at t0, ``L1`` at t0 + theta dt, ``L0`` and Dirichlet
  values at t1);
* ``DirichletBC.apply`` (topological: every DOF in the closure of a facet
  marked 0; rows zeroed, unit diagonal, ``b[dof] = value``) and
  ``apply_symmetric`` / ``MatZeroRowsColumns``: src/mpet/mpet/bc_symmetric.py:11-22;
* elastic stress and parameter conversion: src/mpet/mpet/mpetproblem.py:8-24.

Data terms are Lagrange interpolants integrated exactly: f in P2 (vector),
g, I, beta, p_robin in P1, the traction s in P2 on each boundary facet.
MUMPS LU is replaced by SuperLU (scipy.sparse.linalg.splu).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import fem

DIRICHLET, NEUMANN, ROBIN = 0, 1, 2


def convert_to_mu_lmbda(E, nu):
    """mpetproblem.py:13-16."""
    mu = E / (2.0 * (1.0 + nu))
    lmbda = nu * E / ((1.0 - 2.0 * nu) * (1.0 + nu))
    return mu, lmbda


def convert_to_E_nu(mu, lmbda):
    """mpetproblem.py:8-11."""
    E = mu * (3 * lmbda + 2 * mu) / (lmbda + mu)
    nu = lmbda / (2 * (lmbda + mu))
    return E, nu


def _facet_geometry(x, facets, owner_cells, cells):
    """Facet measure and outward unit normal of boundary facets."""
    d = x.shape[1]
    X = x[facets]
    if d == 3:
        cr = np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0])
        area = 0.5 * np.linalg.norm(cr, axis=1)
        n = cr / np.linalg.norm(cr, axis=1)[:, None]
    else:
        t = X[:, 1] - X[:, 0]
        area = np.linalg.norm(t, axis=1)
        n = np.stack([t[:, 1], -t[:, 0]], 1) / area[:, None]
    oc = cells[owner_cells]
    # opposite vertex: the owner-cell vertex absent from the facet
    opp = np.empty(facets.shape[0], dtype=np.int64)
    for k in range(oc.shape[1]):
        mask = np.all(oc[:, k:k + 1] != facets, axis=1)
        opp[mask] = oc[mask, k]
    centroid = X.mean(axis=1)
    s = np.sign(np.einsum("fd,fd->f", n, centroid - x[opp]))
    n = n * s[:, None]
    return area, n


class OracleMPET:
    """Assembly, boundary conditions and direct solves of the MPET system.

    Parameters mirror ``MPETProblem.params`` (J, E, nu, alpha, K, S, c;
    mpetproblem.py:169-180) and ``MPETSolver.params`` (theta).  Markers are
    one integer per boundary facet (0 Dirichlet, 1 Neumann, 2 Robin).
    """

    def __init__(self, x, cells, bfacets, bfacet_cells, params, theta=1.0,
                 momentum_markers=None, continuity_markers=None):
        self.dm = fem.DofMap(x, cells, params["J"])
        dm = self.dm
        self.d = dm.d
        self.J = int(params["J"])
        self.params = params
        self.theta = float(theta)
        if "mu" in params:
            self.mu, self.lmbda = float(params["mu"]), float(params["lmbda"])
        else:
            self.mu, self.lmbda = convert_to_mu_lmbda(float(params["E"]), float(params["nu"]))
        self.alpha = np.asarray(params["alpha"], dtype=np.float64)
        self.c = np.asarray(params["c"], dtype=np.float64)
        # K_a: a constant or a per-cell (DG0) array; Kc[a] holds one value per cell
        nc0 = np.asarray(cells).shape[0]
        self.Kc = np.stack([np.broadcast_to(np.asarray(k, dtype=np.float64), (nc0,)) for k in params["K"]])
        self.S = np.asarray(params["S"], dtype=np.float64).reshape(self.J, self.J)
        self.bfacets = np.sort(np.asarray(bfacets, dtype=np.int64), axis=1)
        self.bfacet_cells = np.asarray(bfacet_cells, dtype=np.int64)
        nf = self.bfacets.shape[0]
        self.mmark = np.full(nf, -1) if momentum_markers is None else np.asarray(momentum_markers)
        self.cmark = [np.full(nf, -1) if continuity_markers is None else np.asarray(continuity_markers[a])
                      for a in range(self.J)]
        b, vol = fem.simplex_geometry(dm.x, dm.cells)
        self.bgrad, self.vol = b, vol
        g = fem.p2_gradient_vertex_values(b)
        self.Mg = fem.local_gradient_products(g, vol)      # (nc,10,10,3,3)
        self.C = fem.local_coupling(g, vol)                  # (nc,10,3,4)
        self.M1 = fem.p1_mass_reference(self.d)[None] * vol[:, None, None]
        self.L1 = np.einsum("cvk,cwk->cvw", b, b) * vol[:, None, None]
        self.M2 = fem.p2_mass_reference(self.d)[None] * vol[:, None, None]
        self.cell_dofs = dm.cell_dofs()
        # facet data
        self.farea, self.fnormal = _facet_geometry(dm.x, self.bfacets, self.bfacet_cells, dm.cells)
        self._facet_nodes()

    # --- facets -------------------------------------------------------------
    def _facet_nodes(self):
        dm = self.dm
        f = self.bfacets
        fd = self.d - 1
        nv = dm.nv
        edge_key = dm.edges[:, 0] * nv + dm.edges[:, 1]
        fe = []
        for (a, b) in fem.local_edges(fd):
            k = f[:, a] * nv + f[:, b]
            idx = np.searchsorted(edge_key, k)
            assert np.all(edge_key[idx] == k)
            fe.append(nv + idx)
        self.facet_p2_nodes = np.concatenate([f] + [e[:, None] for e in fe], axis=1)
        self.fM1 = fem.p1_mass_reference(fd)[None] * self.farea[:, None, None]
        self.fM2 = fem.p2_mass_reference(fd)[None] * self.farea[:, None, None]
        self.fT1 = fem.p1_triple_reference(fd)[None] * self.farea[:, None, None, None]

    # --- local blocks ---------------------------------------------------------
    def local_matrix(self, dt, beta_cells=None):
        """(nc, nloc, nloc) local matrices of a = lhs(F) (mpetsolver.py:196-201, 260)."""
        d, J = self.d, self.J
        nc = self.vol.shape[0]
        n2 = self.dm.nloc2
        n1 = d + 1
        mu, lm, th = self.mu, self.lmbda, self.theta
        Mg = self.Mg
        tr = np.einsum("cijkk->cij", Mg)
        uu = (mu * np.einsum("cij,kl->cikjl", tr, np.eye(d))
              + mu * np.transpose(Mg, (0, 1, 4, 2, 3))  # [c,i,k,j,l] = Mg[c,i,j,l,k]
              + lm * np.transpose(Mg, (0, 1, 3, 2, 4)))  # [c,i,k,j,l] = Mg[c,i,j,k,l]
        nloc = self.dm.nloc
        Ae = np.zeros((nc, nloc, nloc))
        Ae[:, :d * n2, :d * n2] = uu.reshape(nc, d * n2, d * n2)
        Cf = self.C.reshape(nc, d * n2, n1)  # [c, (i,k), w]
        Ssum = self.S.sum(axis=1)
        for a in range(J):
            o = d * n2 + a * n1
            Ae[:, :d * n2, o:o + n1] = -self.alpha[a] * Cf
            Ae[:, o:o + n1, :d * n2] = -self.alpha[a] * np.transpose(Cf, (0, 2, 1))
            for b_ in range(J):
                ob = d * n2 + b_ * n1
                blk = -dt * th * (Ssum[a] * (a == b_) - self.S[a, b_]) * self.M1
                if a == b_:
                    blk = blk - self.c[a] * self.M1 - dt * th * self.Kc[a][:, None, None] * self.L1
                Ae[:, o:o + n1, ob:ob + n1] += blk
        return Ae

    # --- global matrix --------------------------------------------------------
    def assemble_matrix(self, dt, t=0.0, data=None):
        """assemble(a) + sum of Robin matrices (mpetsolver.py:335-338)."""
        A = fem.assemble_csr(self.cell_dofs, self.local_matrix(dt), self.dm.N)
        data = data or {}
        beta = data.get("beta")
        if beta is not None:
            R = self._robin_matrix(dt, beta, t)
            if R is not None:
                # PETSc MatAXPY(DIFFERENT_NONZERO_PATTERN): union pattern, stored
                # zeros kept (a SciPy sum would drop them)
                A, R = A.tocoo(), R.tocoo()
                A = sp.coo_matrix((np.concatenate([A.data, R.data]),
                                   (np.concatenate([A.row, R.row]), np.concatenate([A.col, R.col]))),
                                  shape=A.shape).tocsr()
                A.sort_indices()
        return A

    def _robin_matrix(self, dt, beta, t):
        rows, cols, vals = [], [], []
        dm = self.dm
        for a in range(self.J):
            if beta[a] is None:
                continue
            sel = np.nonzero(self.cmark[a] == ROBIN)[0]
            if sel.size == 0:
                continue
            fv = self.bfacets[sel]
            bv = _eval_scalar(beta[a], dm.x[fv.ravel()], t).reshape(fv.shape)
            loc = -dt * self.theta * np.einsum("fv,fvij->fij", bv, self.fT1[sel])
            dofs = dm.Nu + a * dm.nv + fv
            rows.append(np.repeat(dofs, dofs.shape[1], axis=1).ravel())
            cols.append(np.tile(dofs, (1, dofs.shape[1])).ravel())
            vals.append(loc.ravel())
        if not rows:
            return None
        N = dm.N
        return sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                             shape=(N, N)).tocsr()

    # --- right-hand side ----------------------------------------------------------
    def rhs_L(self, up_prev, dt):
        """b = assemble(L), L = rhs(F) with up_ = up_prev (mpetsolver.py:196-201, 261, 356)."""
        d, J = self.d, self.J
        dm = self.dm
        th = self.theta
        n1 = d + 1
        nc = self.vol.shape[0]
        cd = self.cell_dofs
        n2 = dm.nloc2
        u_loc = up_prev[cd[:, :d * n2]]                      # (nc, 30)
        p_loc = [up_prev[cd[:, d * n2 + a * n1: d * n2 + (a + 1) * n1]] for a in range(J)]
        Cf = self.C.reshape(nc, d * n2, n1)
        Ssum = self.S.sum(axis=1)
        bl = np.zeros((nc, dm.nloc))
        for a in range(J):
            o = d * n2 + a * n1
            val = -self.alpha[a] * np.einsum("ciw,ci->cw", Cf, u_loc)
            val -= self.c[a] * np.einsum("cvw,cw->cv", self.M1, p_loc[a])
            val += dt * (1.0 - th) * self.Kc[a][:, None] * np.einsum("cvw,cw->cv", self.L1, p_loc[a])
            for b_ in range(J):
                coef = self.S[a, b_]
                if coef != 0.0:
                    val += dt * (1.0 - th) * coef * np.einsum("cvw,cw->cv", self.M1, p_loc[a] - p_loc[b_])
            bl[:, o:o + n1] = val
        return fem.assemble_vector(cd, bl, dm.N)

    def rhs_L1(self, up_prev, dt, t_theta, data):
        """sum_a assemble(L1[a]) at t0 + theta dt (mpetsolver.py:244-254, 359-365)."""
        dm = self.dm
        b = np.zeros(dm.N)
        g = data.get("g")
        I = data.get("I")
        beta = data.get("beta")
        p_robin = data.get("p_robin")
        for a in range(self.J):
            base = dm.Nu + a * dm.nv
            if g is not None and g[a] is not None:
                gv = _eval_scalar(g[a], dm.x, t_theta)
                loc = dt * np.einsum("cvw,cw->cv", self.M1, gv[self.dm.cells])
                b += np.bincount((base + dm.cells).ravel(), weights=loc.ravel(), minlength=dm.N)
            if I is not None and I[a] is not None:
                sel = np.nonzero(self.cmark[a] == NEUMANN)[0]
                if sel.size:
                    fv = self.bfacets[sel]
                    Iv = _eval_scalar(I[a], dm.x[fv.ravel()], t_theta).reshape(fv.shape)
                    loc = dt * np.einsum("fvw,fw->fv", self.fM1[sel], Iv)
                    b += np.bincount((base + fv).ravel(), weights=loc.ravel(), minlength=dm.N)
            if beta is not None and beta[a] is not None:
                sel = np.nonzero(self.cmark[a] == ROBIN)[0]
                if sel.size:
                    fv = self.bfacets[sel]
                    bv = _eval_scalar(beta[a], dm.x[fv.ravel()], t_theta).reshape(fv.shape)
                    pr = (np.zeros(fv.shape) if p_robin is None or p_robin[a] is None else
                          _eval_scalar(p_robin[a], dm.x[fv.ravel()], t_theta).reshape(fv.shape))
                    pn = up_prev[base + fv]
                    T = self.fT1[sel]
                    loc = dt * (1.0 - self.theta) * np.einsum("fv,fw,fvwq->fq", bv, pn, T)
                    loc -= dt * np.einsum("fv,fw,fvwq->fq", bv, pr, T)
                    b += np.bincount((base + fv).ravel(), weights=loc.ravel(), minlength=dm.N)
        return b

    def rhs_L0(self, t1, data):
        """assemble(L0) at t1: f.v dx + s.v ds_m(1) (mpetsolver.py:231-233, 368-372)."""
        dm = self.dm
        d = self.d
        b = np.zeros(dm.N)
        f = data.get("f")
        s = data.get("s")
        if f is not None:
            fv = np.asarray(f(dm.node_x, t1), dtype=np.float64).reshape(dm.nnodes, d)
            cn = dm.cell_nodes
            loc = np.einsum("cij,cjk->cik", self.M2, fv[cn])  # (nc, 10, d)
            dofs = d * cn[:, :, None] + np.arange(d)[None, None, :]
            b += np.bincount(dofs.ravel(), weights=loc.ravel(), minlength=dm.N)
        if s is not None:
            sel = np.nonzero(self.mmark == NEUMANN)[0]
            if sel.size:
                fn = self.facet_p2_nodes[sel]
                xs = dm.node_x[fn.ravel()]
                nrm = np.repeat(self.fnormal[sel], fn.shape[1], axis=0)
                sv = np.asarray(s(xs, t1, nrm), dtype=np.float64).reshape(fn.shape[0], fn.shape[1], d)
                loc = np.einsum("fij,fjk->fik", self.fM2[sel], sv)
                dofs = d * fn[:, :, None] + np.arange(d)[None, None, :]
                b += np.bincount(dofs.ravel(), weights=loc.ravel(), minlength=dm.N)
        return b

    # --- Dirichlet conditions -----------------------------------------------------------
    def dirichlet_dofs(self):
        """Per field: sorted DOFs in the closure of facets marked 0 (DirichletBC, mpetsolver.py:63-84)."""
        dm = self.dm
        d = self.d
        out = []
        sel = np.nonzero(self.mmark == DIRICHLET)[0]
        nodes = np.unique(self.facet_p2_nodes[sel].ravel())
        out.append((nodes, (d * nodes[:, None] + np.arange(d)[None, :]).ravel()))
        for a in range(self.J):
            sel = np.nonzero(self.cmark[a] == DIRICHLET)[0]
            verts = np.unique(self.bfacets[sel].ravel())
            out.append((verts, dm.Nu + a * dm.nv + verts))
        return out

    def dirichlet_values(self, t, data):
        dm = self.dm
        d = self.d
        dofs_all, vals_all = [], []
        bcs = self.dirichlet_dofs()
        nodes, dofs = bcs[0]
        ub = data.get("u_bar")
        if ub is None:
            v = np.zeros(dofs.shape[0])
        else:
            v = np.asarray(ub(dm.node_x[nodes], t), dtype=np.float64).reshape(nodes.shape[0], d).ravel()
        dofs_all.append(dofs)
        vals_all.append(v)
        pb = data.get("p_bar")
        for a in range(self.J):
            verts, dofs = bcs[1 + a]
            if pb is None or pb[a] is None:
                v = np.zeros(dofs.shape[0])
            else:
                v = _eval_scalar(pb[a], dm.x[verts], t)
            dofs_all.append(dofs)
            vals_all.append(v)
        return dofs_all, vals_all

    @staticmethod
    def apply_bc_matrix(A, dofs):
        """DirichletBC.apply(A): zero the rows, unit diagonal (pattern kept)."""
        A = A.tocsr(copy=True)
        for dd in dofs:
            for r in dd:
                A.data[A.indptr[r]:A.indptr[r + 1]] = 0.0
        A = A.tolil() if False else A
        diag_pos = _diag_positions(A)
        for dd in dofs:
            A.data[diag_pos[dd]] = 1.0
        return A

    @staticmethod
    def apply_bc_vector(b, dofs, vals):
        b = b.copy()
        for dd, vv in zip(dofs, vals):
            b[dd] = vv
        return b

    @staticmethod
    def zero_rows_columns(A, dofs, b=None, x=None):
        """PETSc MatZeroRowsColumns(A, dofs, diag=1, x, b) (bc_symmetric.py:11-18).

        b <- b - A[:, dofs] x[dofs] on the other rows, b[dofs] = x[dofs]
        (PETSc fixes b[dofs] = diag * x[dofs]); pattern kept.
        """
        A = A.tocsr(copy=True)
        dofs = np.unique(np.concatenate([np.asarray(d, dtype=np.int64) for d in dofs]))
        isbc = np.zeros(A.shape[0], dtype=bool)
        isbc[dofs] = True
        if b is not None:
            b = b.copy()
            xd = np.zeros(A.shape[0])
            xd[dofs] = x[dofs]
            b -= A @ xd
            b[dofs] = x[dofs]
        rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
        kill = isbc[rows] | isbc[A.indices]
        A.data[kill] = 0.0
        A.data[_diag_positions(A)[dofs]] = 1.0
        return A, b

    # --- preconditioner blocks (mpetsolver.py:264-271) ---------------------------------
    def network_modes(self, dt, form="auto"):
        """(Q, lambda) of the pressure blocks; see ``network_modes`` (module level)."""
        K = np.array([float(np.mean(self.Kc[a])) for a in range(self.J)])
        return network_modes(self.J, self.theta, self.S, self.c, K, dt, form)

    def preconditioner_blocks(self, dt, u_weight=None, modes=None):
        """Scalar SPD blocks: w (grad u, grad v) on P2 nodes (w = mu in the
        reference form, mpetsolver.py:269) and, per network,
        c_a M + dt theta K_a L + dt theta sum_{b != a} S_ab M on P1 vertices,
        with the Dirichlet DOFs eliminated symmetrically (unit diagonal).
        With modes = (Q, lambda) from network_modes, block k is instead
        lambda_k M + dt theta (sum_a Q_ak^2 K_a) L."""
        dm = self.dm
        nc = self.vol.shape[0]
        tr = np.einsum("cijkk->cij", self.Mg)
        cn = dm.cell_nodes
        w = self.mu if u_weight is None else float(u_weight)
        Lu = fem.assemble_csr(cn, w * tr, dm.nnodes)
        bcs = self.dirichlet_dofs()
        Lu, _ = self.zero_rows_columns(Lu, [bcs[0][0]])
        blocks = [Lu]
        for a in range(self.J):
            if modes is not None:
                Q, lam = modes
                kk = sum(Q[b_, a] ** 2 * self.Kc[b_] for b_ in range(self.J))
                loc = lam[a] * self.M1 + dt * self.theta * kk[:, None, None] * self.L1
            else:
                sS = sum(self.S[a, b_] for b_ in range(self.J) if b_ != a)
                loc = ((self.c[a] + dt * self.theta * sS) * self.M1
                       + dt * self.theta * self.Kc[a][:, None, None] * self.L1)
            Pa = fem.assemble_csr(dm.cells, loc, dm.nv)
            Pa, _ = self.zero_rows_columns(Pa, [bcs[1 + a][0]])
            blocks.append(Pa)
        return blocks

    # --- steps ---------------------------------------------------------------------------
    def step(self, up_prev, t0, dt, data=None, return_system=False):
        """One ``MPETSolver.step(dt)``: assemble, BC, LU, rhs, solve (mpetsolver.py:317-379)."""
        data = data or {}
        th = self.theta
        A = self.assemble_matrix(dt, t0, data)
        t_theta = t0 + th * dt
        t1 = t0 + dt
        b = self.rhs_L(up_prev, dt)
        b += self.rhs_L1(up_prev, dt, t_theta, data)
        b += self.rhs_L0(t1, data)
        dofs, vals = self.dirichlet_values(t1, data)
        Abc = self.apply_bc_matrix(A, dofs)
        bbc = self.apply_bc_vector(b, dofs, vals)
        x = spla.splu(Abc.tocsc()).solve(bbc)
        if return_system:
            return x, Abc, bbc, A, b
        return x

    def solve_direct(self, up0, t0, T, dt, data=None):
        """Generator of (up, t) as in ``solve_direct`` (mpetsolver.py:382-462)."""
        data = data or {}
        th = self.theta
        A = self.assemble_matrix(dt, t0, data)
        dofs0, _ = self.dirichlet_values(t0, data)
        Abc = self.apply_bc_matrix(A, dofs0)
        lu = spla.splu(Abc.tocsc())
        t = float(t0)
        up_ = np.array(up0, dtype=np.float64, copy=True)
        while t < T - 1e-9:
            t_theta = t + th * dt
            t1 = t + dt
            b = self.rhs_L(up_, dt)
            b += self.rhs_L1(up_, dt, t_theta, data)
            b += self.rhs_L0(t1, data)
            dofs, vals = self.dirichlet_values(t1, data)
            b = self.apply_bc_vector(b, dofs, vals)
            up = lu.solve(b)
            t = t1
            yield up, t
            up_ = up


def network_modes(J, theta, S, c, K_mean, dt, form="auto"):
    """(Q, lambda) of the pressure blocks: per network (Q = I, lambda =
    diag C) or per eigenmode of the network mass coupling C = Q diag(lambda)
    Q^T, C = diag(c_a + dt theta sum_{b != a} S_ab) - dt theta S (off the
    diagonal).  With kappa(form, T) the worst condition number of
    P(t)^-1 (C + t dt theta diag(K)) over t in T (K = the mean permeability of
    each network), "auto" takes the eigenmodes when
    kappa(modes, [1e3, 1e6])^2 < kappa(networks, [1, 1e6]): most eigenvalues of
    the pressure blocks lie at large t, where the modes average K."""
    S = np.asarray(S, dtype=np.float64).reshape(J, J)
    c = np.asarray(c, dtype=np.float64)
    dth = dt * theta
    C = -dth * S.copy()
    for a in range(J):
        C[a, a] = c[a] + dth * sum(S[a, b_] for b_ in range(J) if b_ != a)
    lam, Q = np.linalg.eigh(C)
    per_net = (np.eye(J), np.diag(C).copy())
    if form == "networks":
        return per_net
    if form == "modes":
        return Q, lam
    K = np.asarray(K_mean, dtype=np.float64)

    def kappa(Qx, lx, first=0):
        kt = (Qx ** 2).T @ K
        worst = 1.0
        for t in 10.0 ** (0.1 * np.arange(first, 61)):
            A = C + t * dth * np.diag(K)
            P = Qx @ np.diag(lx + t * dth * kt) @ Qx.T
            ev = np.linalg.eigvalsh(np.linalg.solve(np.linalg.cholesky(P), np.linalg.solve(
                np.linalg.cholesky(P), A).T).T)
            worst = max(worst, ev.max() / ev.min())
        return worst
    kd = kappa(*per_net)
    if np.all(lam > 0) and kappa(Q, lam) < kd and kappa(Q, lam, 30) ** 2 < kd:
        return Q, lam
    return per_net


def _diag_positions(A):
    """Index into A.data of each diagonal entry (must exist)."""
    n = A.shape[0]
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(A.indptr))
    hit = np.nonzero(A.indices == rows)[0]
    pos = np.full(n, -1, dtype=np.int64)
    pos[rows[hit]] = hit
    assert np.all(pos >= 0), "a diagonal entry is missing from the pattern"
    return pos


def _eval_scalar(fn, x, t):
    v = fn(x, t) if callable(fn) else fn
    v = np.asarray(v, dtype=np.float64)
    if v.ndim == 0:
        v = np.full(x.shape[0], float(v))
    return v.reshape(x.shape[0])
