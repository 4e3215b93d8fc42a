"""AdaptiveMPETSolver's error indicators on the GPU path against the estimator
oracle (oracle/estimators.py, itself checked against quadrature), for triangles
and tetrahedra: the three DG0 indicator fields and R4p of one step within
1e-11, the time bookkeeping over a solve_direct run (estimate_error_at_t,
add_to_indicators, compute_error_indicators, compute_error_estimate), the
marking rules on the GPU fields, and the range check of the facet tables.
"""
import ctypes

import numpy as np
import pytest

import mms
from helpers import make_oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

PARAMS = dict(J=2, c=(0.3, 0.4), alpha=(0.4, 0.6), K=(0.2, 0.3), S=((0.0, 1.5), (1.5, 0.0)), E=520.0, nu=0.47)


def _wrap(fn, dim):
    from waterscapes_gb300 import Expression
    return Expression(lambda x, t: torch.as_tensor(np.asarray(fn(x[:, :dim].detach().cpu().numpy(), t),
                                                              dtype=np.float64), device=x.device))


def _adaptive(dim, n, dt, T):
    from waterscapes_gb300 import (AdaptiveMPETSolver, CompiledSubDomain, Constant, Expression, MPETProblem,
                                   UnitCubeMesh, UnitSquareMesh)
    data, _ = mms.exact_solutions(PARAMS, dim)
    mesh = UnitSquareMesh(n) if dim == 2 else UnitCubeMesh(n)
    time = Constant(0.0)
    problem = MPETProblem(mesh, time, params=PARAMS)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(2):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.u_bar = _wrap(data["u_bar"], dim)
    problem.p_bar = [_wrap(data["p_bar"][a], dim) for a in range(2)]
    problem.f = _wrap(data["f"], dim)
    problem.g = [_wrap(data["g"][a], dim) for a in range(2)]
    time_ = Constant(0.0)
    f_ = Expression(_wrap(data["f"], dim).fn, t=time_)
    params = AdaptiveMPETSolver.default_params()
    params["MPETSolver"].update(dt=dt, T=T, theta=1.0, precision="fp64", rtol=1e-11)
    return AdaptiveMPETSolver(problem, f_, params), problem, data, time_


def _oracle_indicators(problem, data, up, up_prev, dt, t, t_prev):
    from oracle.estimators import Estimators
    om = make_oracle(problem, 1.0)
    dm = om.dm
    f = data["f"](dm.node_x, t)
    f_ = data["f"](dm.node_x, t_prev)
    g = np.stack([data["g"][j](dm.x, t) for j in range(2)])
    return Estimators(om).indicators(up, up_prev, dt, f, f_, g)


@pytest.mark.parametrize("dim,n", [(2, 6), (3, 3)])
def test_indicators_match_oracle(dim, n):
    dt = 0.05
    ad, problem, data, time_ = _adaptive(dim, n, dt, 10 * dt)
    s = ad.inner_solver
    rng = np.random.default_rng(11)
    up_prev = rng.standard_normal(s.N) * 1e-2
    s.up_.assign(torch.tensor(up_prev))
    t0 = 0.1
    problem.time.assign(t0)
    time_.assign(t0)
    s.step(dt)
    eta_p, eta_u, eta_udt, r4 = ad.indicators()
    up = s.up.vector().cpu().numpy()
    ref = _oracle_indicators(problem, data, up, up_prev, dt, t0 + dt, t0)
    for got, want in zip((eta_p, eta_u, eta_udt), ref[:3]):
        got = got.cpu().numpy()
        assert np.allclose(got, want, rtol=1e-11, atol=1e-13 * np.abs(want).max())
    assert abs(r4 - ref[3]) <= 1e-11 * abs(ref[3])


def test_time_bookkeeping_and_marking():
    from oracle.estimators import EstimatorHistory, dorfler_mark as od, maximal_mark as om_
    from waterscapes_gb300.adaptive import dorfler_mark, maximal_mark
    dt = 0.1
    ad, problem, data, time_ = _adaptive(2, 6, dt, 0.3)
    s = ad.inner_solver
    hist = EstimatorHistory(problem.mesh.num_cells())
    t_prev = 0.0
    for up, t in s.solve_direct():
        eta = ad.estimate_error_at_t()
        ad.add_to_indicators(eta)
        ref = _oracle_indicators(problem, data, up.vector().cpu().numpy(), s.up_.vector().cpu().numpy(), dt, t,
                                 t_prev)
        hist.estimate(*ref, dt)
        hist.add_to_indicators(ref[0], ref[1], ref[2], dt)
        time_.assign(t)
        t_prev = t
    eta, etas = ad.compute_error_estimate()
    eta_r, etas_r = hist.error_estimate()
    assert np.allclose(etas, etas_r, rtol=1e-10) and abs(eta - eta_r) <= 1e-10 * eta_r
    ind = ad.compute_error_indicators()
    ind_r = hist.error_indicators()
    assert np.allclose(ind.cpu().numpy(), ind_r, rtol=1e-10, atol=1e-14 * ind_r.max())
    for fr in (0.2, 0.5, 1.0):
        assert np.array_equal(maximal_mark(ind, fr), om_(ind.cpu().numpy(), fr))
        assert np.array_equal(dorfler_mark(ind, fr), od(ind.cpu().numpy(), fr))
    ad.pop_error_estimators()
    assert len(ad.eta_1s) == 2


def test_bad_facet_table_is_an_error_code():
    from waterscapes_gb300 import _lib
    dt = 0.05
    ad, problem, data, time_ = _adaptive(2, 3, dt, 10 * dt)
    s = ad.inner_solver
    s.step(dt)
    bad = ad._ifacets.clone()
    bad[0, 2] = problem.mesh.num_cells()              # a cell index past the end
    out = [torch.zeros(problem.mesh.num_cells(), dtype=torch.float64, device=s.device) for _ in range(3)]
    r4 = ctypes.c_double()
    lib = _lib.load()
    rc = lib.mpet_error_indicators(s.ctx.h, ctypes.c_double(dt), _lib._ptr(s.up.vector()),
                                   _lib._ptr(s.up_.vector()), None, None, None, ctypes.c_int64(ad._nfi),
                                   _lib._ptr(bad), _lib._ptr(ad._cell_facets), _lib._ptr(out[0]),
                                   _lib._ptr(out[1]), _lib._ptr(out[2]), ctypes.byref(r4))
    assert rc == -1
    # the context stays usable
    eta_p, eta_u, eta_udt, r4v = ad.indicators()
    assert torch.isfinite(eta_u).all() and np.isfinite(r4v)
