"""Batches of independent MPET problems advanced together on one GB300.

The reference runs one problem per ``MPETSolver``.  Here a list of
``MPETProblem`` instances (same number of networks, same mu, lambda, alpha;
their own meshes, K, c, S and boundary data) becomes one disjoint union
mesh: instance i is translated by i * L along x (L = widest instance + 1),
so every assembly, right-hand side, SpMV and V-cycle kernel processes all
instances in one launch, and the per-instance data (K_a, c_a, S_ab) become
per-cell fields.  ``mpet_set_batch`` makes the refinement loop converge
every instance to ``rtol`` on its own.  ``step`` / ``solve_direct`` behave
as for one problem and advance every instance; ``instance_vector`` returns
instance i's state in that instance's own DOF order.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .mesh import Mesh, MeshFunction
from .problem import Constant, Expression, MPETProblem, is_zero
from .solver import MPETSolver, _torch


class BatchExpression(Expression):
    """Per-instance data on the union mesh: a point with x0 in
    [i L, (i + 1) L) belongs to instance i and is evaluated there in that
    instance's own coordinates (x0 - i L + lo)."""

    def __init__(self, exprs, L, vector, lo=0.0, gdim=3):
        self.exprs = list(exprs)
        self.L = float(L)
        self.lo = float(lo)
        self.vector = vector
        self.gdim = gdim
        super().__init__(self._eval)

    def is_zero(self):
        return all(is_zero(e) for e in self.exprs)

    def _one(self, e, x, t, n):
        torch = _torch()
        m = x.shape[0]
        shape = (m, 3) if self.vector else (m,)
        if is_zero(e):
            return torch.zeros(shape, dtype=torch.float64, device=x.device)
        if isinstance(e, Constant) or isinstance(e, (int, float, tuple, list)):
            val = e.values() if isinstance(e, Constant) else e
            if self.vector:
                val = tuple(float(a) for a in (val if isinstance(val, (tuple, list)) else (val,) * 3))
                return torch.tensor(val, dtype=torch.float64, device=x.device).expand(m, 3)
            return torch.full((m,), float(val), dtype=torch.float64, device=x.device)
        if n is not None:
            try:
                v = e.fn(x, t, n)
            except TypeError:
                v = e.fn(x, t)
        else:
            v = e(x, t)
        v = torch.as_tensor(v, dtype=torch.float64, device=x.device)
        return v.reshape(shape) if v.numel() == int(np.prod(shape)) else v.expand(shape)

    def _eval(self, x, t, n=None):
        torch = _torch()
        x = torch.as_tensor(x, dtype=torch.float64)
        inst = torch.floor(x[:, 0] / self.L).long()
        out = torch.zeros((x.shape[0], 3) if self.vector else (x.shape[0],), dtype=torch.float64, device=x.device)
        for i in torch.unique(inst).tolist():
            sel = torch.nonzero(inst == i).flatten()
            xi = x[sel].clone()
            xi[:, 0] += self.lo - i * self.L
            out[sel] = self._one(self.exprs[i], xi, t, None if n is None else n[sel])
        return out


def _union_mesh(meshes):
    """Disjoint union of the instance meshes, instance i shifted by i * L along x."""
    lo = min(float(m.coordinates()[:, 0].min()) for m in meshes)
    hi = max(float(m.coordinates()[:, 0].max()) for m in meshes)
    L = (hi - lo) + 1.0
    xs, cs, bfs, bcs = [], [], [], []
    voff = coff = 0
    for i, m in enumerate(meshes):
        x = m.coordinates().copy()
        x[:, 0] += i * L - lo
        xs.append(x)
        cs.append(m.cells().astype(np.int64) + voff)
        bfs.append(m.boundary_facets().astype(np.int64) + voff)
        bcs.append(m.boundary_facet_cells().astype(np.int64) + coff)
        voff += m.num_vertices()
        coff += m.num_cells()
    u = Mesh(np.concatenate(xs), np.concatenate(cs))
    # each instance's facets are already sorted by vertex key, and the offsets
    # keep that order across instances
    u._bfacets = np.ascontiguousarray(np.concatenate(bfs).astype(np.int32))
    u._bfacet_cell = np.ascontiguousarray(np.concatenate(bcs).astype(np.int32))
    return u, L, lo


class MPETBatchSolver(MPETSolver):
    """``MPETSolver`` over a list of independent problems (one launch per kernel
    for all of them)."""

    def __init__(self, problems, params=None):
        problems = list(problems)
        if not problems:
            raise ValueError("empty batch")
        J = int(problems[0].params["J"])
        lame0 = problems[0].lame()
        alpha0 = [float(a) for a in problems[0].params["alpha"]]
        for p in problems:
            if int(p.params["J"]) != J:
                raise ValueError("every instance needs the same number of networks")
            if p.lame() != lame0 or [float(a) for a in p.params["alpha"]] != alpha0:
                raise ValueError("mu, lambda and alpha must be equal across the batch (K, c, S may differ)")
            if p.mesh.gdim != 3:
                raise NotImplementedError("the GPU engine assembles tetrahedral (3D) meshes only")
        mesh, L, lo = _union_mesh([p.mesh for p in problems])
        self.instances = problems
        self.ninst = len(problems)
        nvs = np.array([p.mesh.num_vertices() for p in problems], dtype=np.int64)
        ncs = np.array([p.mesh.num_cells() for p in problems], dtype=np.int64)
        self.vertex_offsets = np.concatenate([[0], np.cumsum(nvs)])
        self.cell_offsets = np.concatenate([[0], np.cumsum(ncs)])
        # per-cell fields of the per-instance coefficients
        K = np.concatenate([np.stack([np.broadcast_to(np.asarray(p.params["K"][a], dtype=np.float64),
                                                      (p.mesh.num_cells(),)) for a in range(J)])
                            for p in problems], axis=1)
        c = np.concatenate([np.repeat(np.asarray([float(v) for v in p.params["c"]])[:, None], p.mesh.num_cells(), 1)
                            for p in problems], axis=1)
        S = np.concatenate([np.repeat(np.asarray([[float(v) for v in row] for row in p.params["S"]])
                                      .reshape(J, J)[:, :, None], p.mesh.num_cells(), 2) for p in problems], axis=2)
        if not np.array_equal(S, np.transpose(S, (1, 0, 2))):
            raise NotImplementedError("MINRES needs a symmetric S in every instance")
        uparams = dict(problems[0].params)
        uparams.update(J=J, K=tuple(K[a] for a in range(J)), c=tuple(float(np.mean(c[a])) for a in range(J)),
                       S=tuple(tuple(float(np.mean(S[a, b])) for b in range(J)) for a in range(J)))
        up = MPETProblem(mesh, Constant(float(problems[0].time)), params=uparams)
        X = lambda get, vec: BatchExpression([get(p) for p in problems], L, vec, lo)  # noqa: E731
        up.f = X(lambda p: p.f, True)
        up.s = X(lambda p: p.s, True)
        up.u_bar = X(lambda p: p.u_bar, True)
        for name in ("g", "I", "beta", "p_robin", "p_bar"):
            setattr(up, name, [X((lambda a, nm: (lambda p: getattr(p, nm)[a]))(a, name), False) for a in range(J)])
        cat = lambda arrs: np.concatenate(arrs)  # noqa: E731
        up.momentum_boundary_markers = MeshFunction(mesh)
        up.momentum_boundary_markers._values = cat([p.momentum_boundary_markers.array() for p in problems])
        for a in range(J):
            mf = MeshFunction(mesh)
            mf._values = cat([p.continuity_boundary_markers[a].array() for p in problems])
            up.continuity_boundary_markers[a] = mf
        self._L, self._lo = L, lo
        super().__init__(up, params)
        torch = _torch()
        self._c_cells = torch.as_tensor(np.ascontiguousarray(c), device=self.device)
        self._S_cells = torch.as_tensor(np.ascontiguousarray(S.reshape(J * J, -1)), device=self.device)
        self._ctx.call("mpet_set_cell_coefficients", _lib._ptr(self._c_cells), _lib._ptr(self._S_cells))
        vinst = np.repeat(np.arange(self.ninst, dtype=np.int32), nvs)
        self._ctx.call("mpet_set_batch", self.ninst, _lib._ptr(np.ascontiguousarray(vinst)))
        self._build_maps()

    def _build_maps(self):
        """Union DOF indices of every instance in the instance's own order
        (vertices, then its edges sorted, u interleaved; then the networks)."""
        torch = _torch()
        edges = self.edges()
        einst = np.searchsorted(self.vertex_offsets, edges[:, 0], side="right") - 1
        eoff = np.concatenate([[0], np.cumsum(np.bincount(einst, minlength=self.ninst))])
        self._maps = []
        for i in range(self.ninst):
            v0, v1 = self.vertex_offsets[i], self.vertex_offsets[i + 1]
            nodes = np.concatenate([np.arange(v0, v1), self.nv + np.arange(eoff[i], eoff[i + 1])])
            u = (3 * nodes[:, None] + np.arange(3)[None, :]).ravel()
            p = [self.Nu + a * self.nv + np.arange(v0, v1) for a in range(self.J)]
            self._maps.append(torch.as_tensor(np.concatenate([u] + p), device=self.device))

    def instance_vector(self, i, vec=None):
        """Instance i's part of a union vector (default: ``up``) in its own DOF order."""
        v = self.up.vector() if vec is None else vec
        return v[self._maps[i]]

    def batch_relres(self):
        out = np.zeros(self.ninst)
        self._ctx.call("mpet_get_batch_relres", _lib._ptr(out))
        return out
