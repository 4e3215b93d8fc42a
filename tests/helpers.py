"""Shared set-up for parity tests: one MPET case built both for the GPU
engine (waterscapes_gb300.MPETSolver) and the CPU oracle (oracle.mpet)."""
import math

import numpy as np

from waterscapes_gb300 import (CompiledSubDomain, Constant, Expression, MPETProblem, UnitCubeMesh,
                               convert_to_E_nu)

CFG1 = dict(mu=1.0e3, lmbda=1.0e4, alpha=(0.5, 0.5), c=(1e-4, 1e-4), K=(1e-3, 1e-2),
            S=((0.0, 0.1), (0.1, 0.0)), dt=0.0125)


def cfg_params(J):
    """Material sets of the two cube workloads: A=2 (16^3 case) and A=4 (64^3 case)."""
    if J == 2:
        d = dict(CFG1)
    elif J == 4:
        S = np.full((4, 4), 1e-2)
        np.fill_diagonal(S, 0.0)
        d = dict(mu=1.0e3, lmbda=1.0e4, alpha=(0.25,) * 4, c=(1e-4,) * 4, K=(1e-4, 1e-3, 1e-2, 1e-1),
                 S=tuple(tuple(r) for r in S), dt=0.01)
    else:
        S = np.zeros((J, J))
        d = dict(mu=1.0e3, lmbda=1.0e4, alpha=tuple(0.3 + 0.1 * a for a in range(J)),
                 c=tuple(1e-3 * (a + 1) for a in range(J)), K=tuple(10.0 ** (-3 + a) for a in range(J)),
                 S=tuple(tuple(r) for r in S), dt=0.02)
    E, nu = convert_to_E_nu(d["mu"], d["lmbda"])
    params = dict(J=J, E=E, nu=nu, alpha=d["alpha"], c=d["c"], K=d["K"], S=d["S"])
    return params, d["dt"]


def p_bar_fn(a):
    """p_a = sin(2 pi t) x0 (a + 1) on the boundary (the cube workloads' data)."""
    return lambda x, t: math.sin(2 * math.pi * t) * x[:, 0] * (a + 1)


def make_problem(n, J, time=None, all_dirichlet=True):
    mesh = UnitCubeMesh(n)
    time = time or Constant(0.0)
    params, dt = cfg_params(J)
    problem = MPETProblem(mesh, time, params=params)
    if all_dirichlet:
        CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
        for a in range(J):
            CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.p_bar = [Expression(p_bar_fn(a)) for a in range(J)]
    return problem, dt


def make_oracle(problem, theta=1.0):
    from oracle.mpet import OracleMPET
    m = problem.mesh
    J = int(problem.params["J"])
    return OracleMPET(m.coordinates(), m.cells(), m.boundary_facets(), m.boundary_facet_cells(),
                      problem.params, theta, problem.momentum_boundary_markers.array(),
                      [problem.continuity_boundary_markers[a].array() for a in range(J)])


def oracle_data(J):
    return {"p_bar": [p_bar_fn(a) for a in range(J)]}
