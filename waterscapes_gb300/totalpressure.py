"""``MPETTotalPressureSolver`` on one GB300: the total-pressure formulation
(src/mpet/mpet/mpettotalpressuresolver.py:16-514) on the same engine as the
MPET solver.

Unknowns: u (P2 vector), the total pressure p0 = lmbda div u - sum_i alpha_i p_i
(P1) and the network pressures p_1 .. p_A (P1), in that block order, so
``up.split()`` gives (u, p0, p1, .., pA) as the reference's mixed function
does (mpettotalpressuresolver.py:206-214).  The engine assembles the form of
mpettotalpressuresolver.py:262-270 (``MPET_FORM_TOTAL_PRESSURE``): pressure
field 0 is p0, with no boundary condition (mpettotalpressuresolver.py:117-137),
and the network data (g, I, beta, p_robin, p_bar, markers) go to fields 1..A.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .mesh import INVALID_MARKER, MeshFunction
from .solver import MPETSolver


class _FieldView:
    """The problem seen with p0 as pressure field 0: per-network lists get a
    leading empty entry, the parameters a leading (alpha 1, c = K = S = 0) field.
    Reads through to the problem at every access, so data set on the problem
    after the solver is created are used."""

    def __init__(self, problem):
        object.__setattr__(self, "_p", problem)
        object.__setattr__(self, "_p0_markers", MeshFunction(problem.mesh, INVALID_MARKER))

    def __getattr__(self, name):
        p = object.__getattribute__(self, "_p")
        if name in ("g", "I", "beta", "p_robin", "p_bar"):
            return [None] + list(getattr(p, name))
        if name == "continuity_boundary_markers":
            return [object.__getattribute__(self, "_p0_markers")] + list(p.continuity_boundary_markers)
        if name == "p_has_nullspace":
            return [False] + list(p.p_has_nullspace)
        if name == "params":
            return expand_params(p.params)
        return getattr(p, name)

    def __setattr__(self, name, value):
        setattr(object.__getattribute__(self, "_p"), name, value)


def expand_params(params):
    A = int(params["J"])
    S = np.zeros((A + 1, A + 1))
    S[1:, 1:] = np.asarray([[float(v) for v in row] for row in params["S"]], dtype=np.float64).reshape(A, A)
    out = dict(params)
    out.update(J=A + 1, alpha=(1.0,) + tuple(float(a) for a in params["alpha"]),
               c=(0.0,) + tuple(float(a) for a in params["c"]),
               K=(0.0,) + tuple(params["K"]), S=tuple(map(tuple, S)))
    return out


class MPETTotalPressureSolver(MPETSolver):
    """Total-pressure MPET solver; default parameters of
    mpettotalpressuresolver.py:146-162 (theta = 0.5, dt = 0.05) plus engine keys."""

    def __init__(self, problem, params=None):
        self.total_problem = problem
        self.A = int(problem.params["J"])
        super().__init__(_FieldView(problem), params)

    @staticmethod
    def default_params():
        p = MPETSolver.default_params()
        p.update({"dt": 0.05, "t": 0.0, "T": 1.0, "theta": 0.5, "direct_solver": True, "testing": False,
                  # 2 mu (grad u, grad v) for the 2 mu (eps u, eps v) block and 1 / (2 w) (p0, w0)
                  # for the total pressure balance the blocks; the reference form has mu and 1
                  # (mpettotalpressuresolver.py:276-283)
                  "prec_u_weight": "2mu", "prec_p0_weight": "auto"})
        return p

    def _make_params(self):
        prm = super()._make_params()
        uw = prm.prec_u_weight
        w0 = self.params["prec_p0_weight"]
        prm.prec_p0_weight = 0.5 / uw if w0 == "auto" else float(w0)
        prm.formulation = _lib.FORMULATION["total_pressure"]
        prm.prec_network_modes = 0
        return prm

    def solve(self):
        """mpettotalpressuresolver.py:508-512: the time loop, with ``direct_solver``
        selecting nothing on this engine (one iterative GPU solve per step)."""
        return self.solve_direct()
