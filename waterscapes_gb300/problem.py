"""MPET problem description (mirrors src/mpet/mpet/mpetproblem.py).

``MPETProblem(mesh, time, params)`` keeps the reference's parameter dict
(J, E, nu, alpha, K, S, c; mpetproblem.py:169-180) and attribute protocol
(f, g, s, I, beta, p_robin, u_bar, p_bar, momentum/continuity boundary
markers, u_has_nullspace, p_has_nullspace; mpetproblem.py:113-166).

Data fields are :class:`Constant` values or :class:`Expression` callables
``fn(x, t)`` evaluated at DOF coordinates ``x`` (a float64 tensor of shape
(n, 3) on the solver's device) and the current time ``t`` read from the
problem's ``time`` Constant, as DOLFIN's ``Expression(..., t=time)`` does.
"""
from __future__ import annotations

from .mesh import INVALID_MARKER, MeshFunction


def convert_to_E_nu(mu, lmbda):
    """mpetproblem.py:8-11."""
    E = mu * (3 * lmbda + 2 * mu) / (lmbda + mu)
    nu = lmbda / (2 * (lmbda + mu))
    return (E, nu)


def convert_to_mu_lmbda(E, nu):
    """mpetproblem.py:13-16."""
    mu = E / (2.0 * ((1.0 + nu)))
    lmbda = nu * E / ((1.0 - 2.0 * nu) * (1.0 + nu))
    return (mu, lmbda)


class Constant:
    """Mutable scalar or vector constant (DOLFIN ``Constant`` stand-in)."""

    def __init__(self, value):
        self._v = value

    def assign(self, value):
        self._v = float(value) if not isinstance(value, (tuple, list)) else tuple(value)

    def values(self):
        return self._v

    def __float__(self):
        return float(self._v)

    def __repr__(self):
        return "Constant(%r)" % (self._v,)

    def is_zero(self):
        v = self._v
        if isinstance(v, (tuple, list)):
            return all(float(a) == 0.0 for a in v)
        return float(v) == 0.0


class Expression:
    """Space-time function ``fn(x, t)``; ``x`` is an (n, 3) tensor."""

    def __init__(self, fn, **kwargs):
        self.fn = fn
        self.kwargs = kwargs

    def __call__(self, x, t):
        return self.fn(x, t)

    def is_zero(self):
        return False


def is_zero(v):
    if v is None:
        return True
    if isinstance(v, (int, float)):
        return float(v) == 0.0
    if hasattr(v, "is_zero"):
        return v.is_zero()
    return False


class MPETProblem:
    """Multiple-network poroelasticity problem (see mpetproblem.py:26-101).

    (1) -div(sigma(u) - sum_j alpha_j p_j I) = f
    (2) c_j dp_j/dt + alpha_j div(du/dt) - div K_j grad p_j + sum_i S_ji (p_j - p_i) = g_j
    with sigma(u) = 2 mu eps(u) + lambda div(u) I.  Facet markers:
    0 Dirichlet, 1 Neumann, 2 Robin; unmarked facets hold INVALID_MARKER.
    """

    def __init__(self, mesh, time, params=None):
        self.mesh = mesh
        self.time = time
        self.params = self.default_parameters()
        if params is not None:
            self.params.update(params)
        Js = range(int(self.params["J"]))
        gdim = mesh.geometry().dim()
        self.f = Constant((0.0,) * gdim)
        self.s = Constant((0.0,) * gdim)
        self.g = [Constant(0.0) for i in Js]
        self.I = [Constant(0.0) for i in Js]
        self.beta = [Constant(0.0) for i in Js]
        self.p_robin = [Constant(0.0) for i in Js]
        self.u_bar = Constant((0.0,) * gdim)
        self.p_bar = [Constant(0.0) for i in Js]
        self.momentum_boundary_markers = MeshFunction(mesh, INVALID_MARKER)
        self.continuity_boundary_markers = [MeshFunction(mesh, INVALID_MARKER) for i in Js]
        self.u_has_nullspace = False
        self.p_has_nullspace = list(False for i in Js)

    @classmethod
    def default_parameters(cls):
        """mpetproblem.py:169-180 (the reference's defaults, 'X' key included)."""
        return {"J": 1, "rho": Constant(1.0), "nu": Constant(0.479), "E": Constant(1500),
                "alpha": (Constant(1.0),), "K": (Constant(1.0),), "X": ((Constant(1.0),),),
                "c": (Constant(1.0),)}

    def lame(self):
        """(mu, lmbda) from the parameters: E, nu as in the reference, or mu, lmbda directly."""
        p = self.params
        if "mu" in p and "lmbda" in p:
            return float(p["mu"]), float(p["lmbda"])
        return convert_to_mu_lmbda(float(p["E"]), float(p["nu"]))
