"""``AdaptiveMPETSolver``: a posteriori error estimators of the MPET solver on
one GB300 (src/mpet/mpet/adaptivempetsolver.py:64-240).

The DG0 indicators zeta_p_K, zeta_u_K and zeta_u_dt_K and the scalar R4p
(:114-155) are computed by the engine (``mpet_error_indicators``: a thread per
cell for the cell residuals, a thread per interior facet for the jump terms,
exact integration of the discrete fields).  The time bookkeeping of
``estimate_error_at_t``, ``add_to_indicators``, ``compute_error_indicators`` and
``compute_error_estimate`` (:157-227) and the marking rules ``maximal_mark`` and
``dorfler_mark`` (:10-61) act on those fields.  Indicator fields are CUDA
float64 tensors with one value per cell; the marking rules return one bool per
cell (the reference returns a cell ``MeshFunction("bool")``).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .problem import Constant, Expression
from .solver import MPETSolver, _torch


def interior_facet_tables(cells):
    """(ifacets (nfi x 4): cell+, local vertex opposite the facet in cell+,
    cell-, its local opposite vertex; cell_facets (nc x (d+1)): the interior
    facet opposite each local vertex, -1 on the boundary), for cells with
    ascending vertex ids."""
    cells = np.sort(np.asarray(cells, dtype=np.int64), axis=1)
    nc, n1 = cells.shape
    owner = np.repeat(np.arange(nc), n1)
    local = np.tile(np.arange(n1), nc)
    # facet opposite local vertex k: the cell's other vertices, ascending
    keys = np.stack([np.delete(cells, k, axis=1) for k in range(n1)], 1).reshape(nc * n1, n1 - 1)
    order = np.lexsort(keys.T[::-1])
    ks = keys[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    a = order[:-1][same]
    b = order[1:][same]
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    ifacets = np.stack([owner[lo], local[lo], owner[hi], local[hi]], 1).astype(np.int32)
    cell_facets = np.full(nc * n1, -1, dtype=np.int32)
    ids = np.arange(lo.shape[0], dtype=np.int32)
    cell_facets[lo] = ids
    cell_facets[hi] = ids
    return np.ascontiguousarray(ifacets), cell_facets.reshape(nc, n1)


def _values(indicators):
    if hasattr(indicators, "detach"):
        return indicators.detach().cpu().numpy()
    return np.asarray(indicators)


def maximal_mark(indicators, fraction):
    """Mark the ceil(fraction * num_cells) cells with the largest indicators
    (adaptivempetsolver.py:10-32)."""
    etas = _values(indicators)
    marked = np.zeros(etas.shape[0], dtype=bool)
    marked[np.argsort(-etas)[:math.ceil(fraction * etas.shape[0])]] = True
    return marked


def dorfler_mark(indicators, fraction):
    """Mark the largest indicators until their sum reaches fraction times the
    total (adaptivempetsolver.py:34-61): cell k of the descending order is
    marked while the sum of the cells before it is below the limit."""
    etas = _values(indicators)
    order = np.argsort(-etas)
    before = np.concatenate([[0.0], np.cumsum(etas[order])[:-1]])
    marked = np.zeros(etas.shape[0], dtype=bool)
    marked[order[before < fraction * np.sum(etas)]] = True
    return marked


class AdaptiveMPETSolver:
    """Error estimation around an inner MPETSolver (adaptivempetsolver.py:64-80)."""

    def __init__(self, problem, f_, params=None):
        self.problem = problem
        self.f_ = f_
        self.params = self.default_params()
        if params is not None:
            inner = params.get("MPETSolver")
            self.params.update({k: v for k, v in params.items() if k != "MPETSolver"})
            if inner is not None:
                self.params["MPETSolver"].update(inner)
        inner = dict(self.params["MPETSolver"])
        for key in ("dt", "T", "t", "theta"):
            if isinstance(inner.get(key), Constant):
                inner[key] = float(inner[key])
        self.inner_solver = MPETSolver(problem, params=inner)
        self._init_error_estimators()

    @staticmethod
    def default_params():
        """adaptivempetsolver.py:229-240."""
        return {"MPETSolver": MPETSolver.default_params(), "alpha": 0.1, "beta": 2, "tau_max": 0.2,
                "tau_min": 0.0, "marking_fraction": 1.0}

    def _init_error_estimators(self):
        torch = _torch()
        s = self.inner_solver
        mesh = self.problem.mesh
        ifacets, cell_facets = interior_facet_tables(mesh.cells())
        dev = s.device
        self._nfi = ifacets.shape[0]
        self._ifacets = torch.as_tensor(ifacets, device=dev)
        self._cell_facets = torch.as_tensor(np.ascontiguousarray(cell_facets), device=dev)
        nc = mesh.num_cells()
        f64 = dict(dtype=torch.float64, device=dev)
        self._eta = [torch.zeros(nc, **f64) for _ in range(3)]
        self.eta_1s, self.eta_2s, self.eta_3s, self.eta_4s = [], [], [], []
        self.eta_1Ks = torch.zeros(nc, **f64)
        self.eta_2Ks = torch.zeros(nc, **f64)
        self.eta_3Ks = torch.zeros(nc, **f64)

    def _data(self, t, dt):
        """f at t and f_ at its own time (the ``t`` keyword of the expression, else
        t - dt) at the P2 nodes; g at t at the vertices."""
        torch = _torch()
        s, p = self.inner_solver, self.problem
        xn = s._node_coordinates()
        f = s._eval(p.f, xn, t, True).reshape(-1).contiguous()
        t_prev = t - dt
        if isinstance(self.f_, Expression) and "t" in self.f_.kwargs:
            t_prev = float(self.f_.kwargs["t"])
        f_ = s._eval(self.f_, xn, t_prev, True).reshape(-1).contiguous()
        xv = xn[:s.nv]
        g = torch.stack([s._eval(gi, xv, t, False) for gi in p.g], 0).contiguous()
        return f, f_, g

    def indicators(self, dt=None):
        """(eta_p_K, eta_u_K, eta_u_dt_K, R4p) of the inner solver's last step
        (up_ -> up) at the current time."""
        s = self.inner_solver
        dt = float(s.dt) if dt is None else float(dt)
        f, f_, g = self._data(float(self.problem.time), dt)
        r4 = ctypes.c_double()
        eta_p, eta_u, eta_udt = (e.clone() for e in self._eta)
        s.ctx.call("mpet_error_indicators", dt, _lib._ptr(s.up.vector()), _lib._ptr(s.up_.vector()),
                   _lib._ptr(f), _lib._ptr(f_), _lib._ptr(g), self._nfi, _lib._ptr(self._ifacets),
                   _lib._ptr(self._cell_facets), _lib._ptr(eta_p), _lib._ptr(eta_u), _lib._ptr(eta_udt),
                   ctypes.byref(r4))
        return eta_p, eta_u, eta_udt, r4.value

    def estimate_error_at_t(self):
        """adaptivempetsolver.py:170-188."""
        eta_p_K_m, eta_u_K_m, eta_u_dt_K_m, r4 = self.indicators()
        tau_m = float(self.inner_solver.dt)
        self.eta_1s.append(tau_m * float(eta_p_K_m.sum()))
        self.eta_2s.append(float(eta_u_K_m.sum()))
        self.eta_3s.append(tau_m * math.sqrt(float(eta_u_dt_K_m.sum())))
        self.eta_4s.append(tau_m * r4)
        return (eta_p_K_m, eta_u_K_m, eta_u_dt_K_m, tau_m)

    def add_to_indicators(self, eta_Ks):
        """adaptivempetsolver.py:190-198."""
        torch = _torch()
        eta_p_K_m, eta_u_K_m, eta_u_dt_K_m, tau_m = eta_Ks
        self.eta_1Ks.add_(tau_m * eta_p_K_m)
        self.eta_3Ks = tau_m * torch.sqrt(eta_u_dt_K_m)
        self.eta_2Ks = torch.maximum(self.eta_2Ks, eta_u_K_m)

    def pop_error_estimators(self):
        """Remove the last entry of each estimator list (adaptivempetsolver.py:200-205)."""
        self.eta_1s.pop()
        self.eta_2s.pop()
        self.eta_3s.pop()
        self.eta_4s.pop()

    def compute_error_indicators(self):
        """eta_K = eta_2K + eta_3K + sqrt(eta_1K) (adaptivempetsolver.py:207-215)."""
        return self.eta_2Ks + self.eta_3Ks + _torch().sqrt(self.eta_1Ks)

    def compute_error_estimate(self):
        """(eta, (eta_1, eta_2, eta_3, eta_4)) summed over time
        (adaptivempetsolver.py:217-225)."""
        etas = (math.sqrt(float(np.sum(self.eta_1s))), math.sqrt(float(np.max(self.eta_2s))),
                float(np.sum(self.eta_3s)), math.sqrt(float(np.sum(self.eta_4s))))
        return (sum(etas), etas)

