"""Batches of independent instances against one solver per instance.

Each instance of a batch (own mesh size, K, c, S, boundary data) must follow
the trajectory of the same problem solved alone: within 1e-8 relative per
step for FP64 and mixed precision (every instance converged to its own
1e-10), and within 1e-8 of the oracle's LU solution.
"""
import math

import numpy as np
import pytest

from helpers import make_oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _instance(n, K, c, s12, amp, J=2):
    from waterscapes_gb300 import (CompiledSubDomain, Constant, Expression, MPETProblem, UnitCubeMesh,
                                   convert_to_E_nu)
    E, nu = convert_to_E_nu(1.0e3, 1.0e4)
    params = dict(J=J, E=E, nu=nu, alpha=(0.5, 0.5), c=c, K=K, S=((0.0, s12), (s12, 0.0)))
    problem = MPETProblem(UnitCubeMesh(n), Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(J):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.p_bar = [Expression((lambda a: lambda x, t: amp * math.sin(2 * math.pi * t) * x[:, 0] * (a + 1))(a))
                     for a in range(J)]
    return problem


def _batch_problems():
    rng = np.random.default_rng(7)
    out = []
    for n in (2, 4, 3):
        K = tuple(10.0 ** rng.uniform(-5, -1, 2))
        c = tuple(10.0 ** rng.uniform(-5, -3, 2))
        out.append(_instance(n, K, c, 10.0 ** rng.uniform(-3, 0), rng.uniform(0.5, 2.0)))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_instances(precision):
    from waterscapes_gb300 import MPETBatchSolver, MPETSolver
    dt, steps = 0.02, 3
    params = dict(dt=dt, T=steps * dt, theta=1.0, precision=precision, rtol=1e-10)
    bs = MPETBatchSolver(_batch_problems(), params)
    batch_states = []
    for up, t in bs.solve_direct():
        batch_states.append([bs.instance_vector(i).cpu().numpy() for i in range(bs.ninst)])
        assert np.all(bs.batch_relres() <= 1e-10)
    assert len(batch_states) == steps
    for i, p in enumerate(_batch_problems()):
        s = MPETSolver(p, dict(params))
        om = make_oracle(p)
        data = {"p_bar": [p.p_bar[a].fn for a in range(2)]}
        ref = [u.copy() for u, _ in om.solve_direct(np.zeros(om.dm.N), 0.0, steps * dt - 0.5 * dt, dt, data)]
        for k, (up, t) in enumerate(s.solve_direct()):
            single = up.vector().cpu().numpy()
            b = batch_states[k][i]
            assert np.linalg.norm(b - single) <= 1e-8 * np.linalg.norm(single)
            assert np.linalg.norm(b - ref[k]) <= 1e-8 * np.linalg.norm(ref[k])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_skipping_converged_instances_keeps_results(precision):
    """The batched products skip the rows of instances that have converged
    (mpet_set_batch_skip, on by default); every instance's trajectory must be
    the one it follows when every product runs over all instances (within
    the 1e-8 bar: the two runs may tune different SpMV kernels)."""
    from waterscapes_gb300 import MPETBatchSolver
    dt, steps = 0.02, 2
    params = dict(dt=dt, T=steps * dt, theta=1.0, precision=precision, rtol=1e-10)
    runs = []
    for skip in (1, 0):
        bs = MPETBatchSolver(_batch_problems(), params)
        bs._ctx.call("mpet_set_batch_skip", skip)
        states = []
        for up, t in bs.solve_direct():
            assert np.all(bs.batch_relres() <= 1e-10)
            states.append([bs.instance_vector(i).cpu().numpy() for i in range(bs.ninst)])
        runs.append(states)
        bs.ctx.close()
    for k in range(steps):
        for i in range(3):
            a, b = runs[0][k][i], runs[1][k][i]
            assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)
