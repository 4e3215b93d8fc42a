"""Discrete adjoint of the MPET time loop with respect to per-cell permeability.

The reference has no adjoint.  This differentiates the time loop that
``MPETSolver.solve_direct`` runs (mpetsolver.py:382-462, as the GPU engine
discretises it) for the loss

    L(K) = 1/2 sum_a (p_a(T) - p*_a)^T M (p_a(T) - p*_a),

the L2 misfit of the final pressures (M the P1 mass matrix), with respect
to the per-cell fields K_a (shape J x num_cells).  The forward pass keeps a
checkpoint every ``checkpoint_every`` steps; the backward pass recomputes
each segment from its checkpoint and runs the adjoint steps of that segment
in reverse:

    A^T lam_N = dL/dx_N,   A^T lam_n = B^T lam_{n+1},   lam = 0 on Dirichlet DOFs,
    dL/dK_a(e) = dt sum_n |e| grad lam_a,n . grad(theta p_a,n + (1 - theta) p_a,n-1)

(``mpet_pressure_misfit``, ``mpet_adjoint_rhs``, ``mpet_adjoint_step``).
``pressure_misfit`` wraps it in a ``torch.autograd.Function``.
"""
from __future__ import annotations

import ctypes

from . import _lib


def _torch():
    import torch
    return torch


class MisfitAdjoint:
    """Forward/backward driver over an ``MPETSolver`` (its problem, BCs and dt).

    ``p_target`` is a (J, num_vertices) tensor; the loop runs ``nsteps`` steps
    of size ``solver.params["dt"]`` from ``t0`` and the initial state ``up0``
    (default: the solver's ``up_`` when the driver is built)."""

    def __init__(self, solver, p_target, nsteps, checkpoint_every=5, t0=None, up0=None):
        torch = _torch()
        self.solver = solver
        self.nsteps = int(nsteps)
        self.every = max(1, int(checkpoint_every))
        self.dt = float(solver.params["dt"])
        self.t0 = float(solver.problem.time) if t0 is None else float(t0)
        f64 = dict(dtype=torch.float64, device=solver.device)
        self.p_target = torch.as_tensor(p_target, **f64).reshape(solver.J, solver.nv).contiguous()
        src = solver.up_.vector() if up0 is None else torch.as_tensor(up0, **f64)
        self.up0 = src.clone()
        self.checkpoints = {}
        self.x_final = None
        self.stats = {"forward_iterations": [], "adjoint_iterations": []}

    # --- pieces ------------------------------------------------------------------
    def _set_K(self, K):
        self.solver.set_cell_permeability(K)
        self.solver._assemble(self.dt)

    def _step(self, x_prev, n, guess=None):
        """State n from state n - 1 (n = 1..nsteps); the solve starts from
        ``guess`` when given (else from x_prev)."""
        s = self.solver
        s.up_.assign(x_prev)
        st = s._advance(self.dt, self.t0 + (n - 1) * self.dt, guess)
        self.stats["forward_iterations"].append(st.iterations)
        return s.up.vector().clone()

    def misfit(self, x, with_grad=True):
        torch = _torch()
        loss = ctypes.c_double()
        d = torch.empty_like(x) if with_grad else None
        self.solver.ctx.call("mpet_pressure_misfit", _lib._ptr(x), _lib._ptr(self.p_target), ctypes.byref(loss),
                             _lib._ptr(d))
        return loss.value, d

    # --- passes ------------------------------------------------------------------
    def forward(self, K, guesses=None, keep_states=False):
        """Run the loop with permeability K; returns the loss (checkpoints kept).

        ``guesses[n]`` (optional) is the initial guess of step n's solve, e.g.
        the states of a nearby K: the solves then resolve the difference to
        the solver's relative tolerance (finite differences need that).
        ``keep_states`` keeps every state in ``self.states``."""
        self._set_K(K)
        self.K = self.solver._K_cells
        x = self.up0.clone()
        self.checkpoints = {0: x.clone()}
        self.states = [x.clone()] if keep_states else None
        for n in range(1, self.nsteps + 1):
            x = self._step(x, n, None if guesses is None else guesses[n])
            if n % self.every == 0 and n < self.nsteps:
                self.checkpoints[n] = x.clone()
            if keep_states:
                self.states.append(x.clone())
        self.x_final = x
        return self.misfit(x, with_grad=False)[0]

    def backward(self):
        """dL/dK (J x num_cells) for the K of the last forward pass."""
        torch = _torch()
        s = self.solver
        if s._K_cells is not self.K or s._assembled_dt != self.dt:
            self._set_K(self.K)
        _, seed = self.misfit(self.x_final)
        grad = torch.zeros_like(self.K)
        lam = torch.empty_like(seed)
        starts = sorted(self.checkpoints)
        for start in reversed(starts):
            end = min(start + self.every, self.nsteps)
            xs = [self.checkpoints[start]]
            for n in range(start + 1, end + 1):
                xs.append(self.x_final if n == self.nsteps else self._step(xs[-1], n))
            for n in range(end, start, -1):
                st = _lib.MpetStats()
                s.ctx.call("mpet_adjoint_step", self.dt, _lib._ptr(seed), _lib._ptr(xs[n - start - 1]),
                           _lib._ptr(xs[n - start]), _lib._ptr(lam), _lib._ptr(grad), ctypes.byref(st))
                self.stats["adjoint_iterations"].append(st.iterations)
                s.ctx.call("mpet_adjoint_rhs", self.dt, _lib._ptr(lam), _lib._ptr(seed))
        return grad

    def loss_and_grad(self, K):
        loss = self.forward(K)
        return loss, self.backward()


def _function_class():
    torch = _torch()

    class PressureMisfit(torch.autograd.Function):
        """L(K) with the hand-written discrete adjoint as its backward."""

        @staticmethod
        def forward(ctx, K, driver):
            loss = driver.forward(K.detach())
            ctx.driver = driver
            return torch.tensor(loss, dtype=torch.float64, device=K.device)

        @staticmethod
        def backward(ctx, g):
            return g * ctx.driver.backward(), None

    return PressureMisfit


_FN = None


def pressure_misfit(solver, K, p_target, nsteps, checkpoint_every=5, t0=None, up0=None):
    """Differentiable final-pressure misfit of ``nsteps`` time steps as a
    function of the per-cell permeability tensor K (J x num_cells)."""
    global _FN
    if _FN is None:
        _FN = _function_class()
    driver = MisfitAdjoint(solver, p_target, nsteps, checkpoint_every, t0, up0)
    return _FN.apply(K, driver)
