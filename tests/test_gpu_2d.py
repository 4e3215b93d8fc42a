"""Triangles (2D) on the GPU path against the oracle, and the reference's own
2D convergence tests run on the GPU.

* sparsity pattern bit-exact, matrix and right-hand side within 1e-12
  (sources f, g, traction on x = 1; theta = 1 and 0.5), one step within 1e-8
  of the SuperLU solution;
* the rate thresholds of src/mpet/test/test_convergence_mpetsolver.py:234-239
  (UnitSquareMesh 8, 16, 32; theta = 1 with M = 8, 32, 128 steps and
  theta = 0.5 with M = 4, 8, 16), the errors measured on the GPU solutions.
"""
import math

import numpy as np
import pytest

import mms
from helpers import make_oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REF_PARAMS = dict(J=2, c=(0.3, 0.4), alpha=(0.4, 0.6), K=(0.2, 0.3), S=((0.0, 2.0), (1.0, 0.0)), E=520.0, nu=0.47)
SYM_PARAMS = dict(REF_PARAMS, S=((0.0, 1.5), (1.5, 0.0)))


def _wrap(fn, vector=False):
    """numpy data function of (x, t) -> torch function of GPU points (n x 3, z = 0)."""
    from waterscapes_gb300 import Expression

    def f(x, t):
        v = fn(x[:, :2].detach().cpu().numpy(), t)
        return torch.as_tensor(np.asarray(v, dtype=np.float64), device=x.device)
    return Expression(f)


def _wrap_traction(fn):
    from waterscapes_gb300 import Expression

    def f(x, t, n):
        v = fn(x[:, :2].detach().cpu().numpy(), t, n[:, :2].detach().cpu().numpy())
        return torch.as_tensor(np.asarray(v, dtype=np.float64), device=x.device)
    return Expression(f)


def _problem_2d(n, params, data):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, UnitSquareMesh
    J = params["J"]
    mesh = UnitSquareMesh(n)
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    CompiledSubDomain(lambda x: np.abs(x[:, 0] - 1.0) < 1e-12).mark(problem.momentum_boundary_markers, 1)
    for a in range(J):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.u_bar = _wrap(data["u_bar"], True)
    problem.p_bar = [_wrap(data["p_bar"][a]) for a in range(J)]
    problem.f = _wrap(data["f"], True)
    problem.g = [_wrap(data["g"][a]) for a in range(J)]
    problem.s = _wrap_traction(data["s"])
    return problem


def _solver(problem, dt, T, theta, precision="fp64", rtol=1e-11):
    from waterscapes_gb300 import MPETSolver
    return MPETSolver(problem, dict(dt=dt, T=T, theta=theta, precision=precision, rtol=rtol))


@pytest.mark.parametrize("n,J", [(2, 1), (3, 2), (4, 3)])
def test_pattern_bit_exact_2d(n, J):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, UnitSquareMesh
    params = dict(REF_PARAMS, J=J, c=(0.3,) * J, alpha=(0.4,) * J, K=(0.2,) * J,
                  S=tuple(tuple(0.5 * (a != b) for b in range(J)) for a in range(J)))
    problem = MPETProblem(UnitSquareMesh(n), Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    s = _solver(problem, 0.1, 1.0, 1.0)
    om = make_oracle(problem)
    A = om.assemble_matrix(0.1)
    rp, ci = s.pattern()
    assert s.N == om.dm.N and s.nnz == A.nnz
    assert np.array_equal(rp, A.indptr.astype(np.int64))
    assert np.array_equal(ci, A.indices.astype(np.int32))


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_matrix_rhs_and_step_2d(theta):
    data, exact = mms.exact_solutions(SYM_PARAMS, 2)
    problem = _problem_2d(6, SYM_PARAMS, data)
    dt = 0.05
    s = _solver(problem, dt, 10 * dt, theta)
    om = make_oracle(problem, theta)
    t0 = 0.1
    problem.time.assign(t0)
    s._assemble(dt)
    A = om.assemble_matrix(dt, t0, data)
    dofs, _ = om.dirichlet_values(t0 + dt, data)
    Abc = om.apply_bc_matrix(A, dofs)
    v = s.matrix_values()
    assert np.allclose(v, Abc.data, rtol=1e-12, atol=1e-13 * np.abs(Abc.data).max())
    rng = np.random.default_rng(3)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, t0, dt, data)
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(t0)
    s.step(dt)
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def _rates_gpu(theta, ms, precision):
    data, exact = mms.exact_solutions(SYM_PARAMS, 2)
    errs = {k: [] for k in ("uL2", "uH1", "p0L2", "p1L2", "p0H1", "p1H1")}
    hs = []
    for n, M in zip((8, 16, 32), ms):
        problem = _problem_2d(n, SYM_PARAMS, data)
        s = _solver(problem, 1.0 / M, 1.0, theta, precision=precision, rtol=1e-10)
        for up, t in s.solve():
            pass
        om = make_oracle(problem, theta)
        e = mms.errornorms(om, up.vector().cpu().numpy(), t, exact)
        errs["uL2"].append(e["uL2"])
        errs["uH1"].append(e["uH1"])
        for a in range(2):
            errs["p%dL2" % a].append(e["pL2"][a])
            errs["p%dH1" % a].append(e["pH1"][a])
        hs.append(problem.mesh.hmin())
    return {k: mms.rates(v, hs) for k, v in errs.items()}


@pytest.mark.parametrize("theta,ms,precision", [(1.0, (8, 32, 128), "fp64"), (0.5, (4, 8, 16), "fp64"),
                                                (0.5, (4, 8, 16), "mixed")])
def test_reference_rate_thresholds_on_gpu(theta, ms, precision):
    """test_convergence_mpetsolver.py:234-239 with the GPU solution (S symmetrised:
    MINRES needs S = S^T; the reference's S has S12 = 2, S21 = 1)."""
    r = _rates_gpu(theta, ms, precision)
    assert r["uH1"][-1] > 1.70
    assert r["uL2"][-1] > 1.70
    assert r["p0L2"][-1] > 1.70
    assert r["p1L2"][-1] > 1.70
    assert r["p0H1"][-1] > 0.95
    assert r["p1H1"][-1] > 0.95


@pytest.mark.parametrize("theta,ms,precision", [(1.0, (8, 32, 128), "fp64"), (0.5, (4, 8, 16), "fp64"),
                                                (0.5, (4, 8, 16), "mixed")])
def test_reference_rate_thresholds_nonsymmetric_S_gmres(theta, ms, precision):
    """test_convergence_mpetsolver.py:234-239 with the reference's own transfer matrix
    S = ((0, 2), (1, 0)) (:112-118): a non-symmetric system, solved by GMRES."""
    data, exact = mms.exact_solutions(REF_PARAMS, 2)
    errs = {k: [] for k in ("uL2", "uH1", "p0L2", "p1L2", "p0H1", "p1H1")}
    hs = []
    for n, M in zip((8, 16, 32), ms):
        problem = _problem_2d(n, REF_PARAMS, data)
        s = _solver(problem, 1.0 / M, 1.0, theta, precision=precision, rtol=1e-10)
        for up, t in s.solve():
            assert s.last_stats["status"] == 0
        om = make_oracle(problem, theta)
        e = mms.errornorms(om, up.vector().cpu().numpy(), t, exact)
        errs["uL2"].append(e["uL2"])
        errs["uH1"].append(e["uH1"])
        for a in range(2):
            errs["p%dL2" % a].append(e["pL2"][a])
            errs["p%dH1" % a].append(e["pH1"][a])
        hs.append(problem.mesh.hmin())
    r = {k: mms.rates(v, hs) for k, v in errs.items()}
    assert r["uH1"][-1] > 1.70
    assert r["uL2"][-1] > 1.70
    assert r["p0L2"][-1] > 1.70
    assert r["p1L2"][-1] > 1.70
    assert r["p0H1"][-1] > 0.95
    assert r["p1H1"][-1] > 0.95


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonsymmetric_S_step_matches_oracle(precision):
    """One step with S12 = 2, S21 = 1 (GMRES) against the oracle's SuperLU solve."""
    data, exact = mms.exact_solutions(REF_PARAMS, 2)
    problem = _problem_2d(6, REF_PARAMS, data)
    dt = 0.05
    s = _solver(problem, dt, 10 * dt, 1.0, precision=precision, rtol=1e-11)
    om = make_oracle(problem, 1.0)
    rng = np.random.default_rng(8)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    t0 = 0.1
    x_ref = om.step(up_prev, t0, dt, data)
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(t0)
    st = s.step(dt)
    assert st.status == 0
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
