"""GPU parity of the assemble + solve path against the CPU oracle.

All engine calls go through the C ABI (libmpetgpu via ctypes).  Bars:
sparsity bit-exact; matrix / right-hand side within 1e-12 relative (FP64,
different summation order); solutions within 1e-8 relative of the SuperLU
solution for both precisions (the spec bar is 1e-8 against FP64).
"""
import ctypes
import math

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():
    from waterscapes_gb300 import _lib
    return _lib


def _solver(problem, dt, **kw):
    from waterscapes_gb300 import MPETSolver
    params = dict(dt=dt, T=10 * dt, theta=1.0)
    params.update(kw)
    return MPETSolver(problem, params)


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("n,J", [(2, 1), (2, 2), (3, 4), (4, 2)])
def test_pattern_bit_exact(n, J):
    problem, dt = make_problem(n, J)
    s = _solver(problem, dt)
    om = make_oracle(problem)
    A = om.assemble_matrix(dt)
    rp, ci = s.pattern()
    assert s.N == om.dm.N and s.nnz == A.nnz
    assert np.array_equal(rp, A.indptr.astype(np.int64))
    assert np.array_equal(ci, A.indices.astype(np.int32))
    assert np.array_equal(s.edges(), om.dm.edges)


@pytest.mark.parametrize("n,J,apply_bc", [(3, 2, 1), (3, 4, 1), (3, 2, 0), (2, 3, 1)])
def test_matrix_values(n, J, apply_bc):
    problem, dt = make_problem(n, J)
    s = _solver(problem, dt)
    om = make_oracle(problem)
    A = om.assemble_matrix(dt)
    if apply_bc:
        dofs, _ = om.dirichlet_values(dt, oracle_data(J))
        A = om.apply_bc_matrix(A, dofs)
    s.ctx.call("mpet_assemble", dt, apply_bc)
    v = s.matrix_values()
    scale = np.abs(A.data).max()
    assert np.allclose(v, A.data, rtol=1e-12, atol=1e-13 * scale)


def _f_expr(x, t):
    return (x * x) * (1.0 + t)


def _g_expr(a):
    return lambda x, t: x[:, 0] * x[:, 1] * (a + 1) + t


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_rhs_parity(theta):
    from waterscapes_gb300 import Expression
    J = 2
    problem, dt = make_problem(3, J)
    problem.f = Expression(_f_expr)
    problem.g = [Expression(_g_expr(a)) for a in range(J)]
    s = _solver(problem, dt, theta=theta)
    om = make_oracle(problem, theta)
    rng = np.random.default_rng(1)
    up_prev = rng.standard_normal(om.dm.N)
    t0 = 0.3
    t_theta, t1 = t0 + theta * dt, t0 + dt
    data = oracle_data(J)
    data["f"] = _f_expr
    data["g"] = [_g_expr(a) for a in range(J)]
    b = om.rhs_L(up_prev, dt) + om.rhs_L1(up_prev, dt, t_theta, data) + om.rhs_L0(t1, data)
    dofs, vals = om.dirichlet_values(t1, data)
    b = om.apply_bc_vector(b, dofs, vals)
    s._set_sources(t_theta, t1)
    s._set_bc_values(t1)
    up = torch.tensor(up_prev, dtype=torch.float64, device=s.device)
    bg = torch.empty(s.N, dtype=torch.float64, device=s.device)
    s.ctx.call("mpet_rhs", dt, _lib()._ptr(up), _lib()._ptr(bg))
    torch.cuda.synchronize()
    assert np.allclose(_np(bg), b, rtol=1e-12, atol=1e-13 * np.abs(b).max())
    # once the matrix is assembled, the pressure rows' -alpha (div u^n, q) term comes from
    # the system's pressure-row, displacement-column block (an FP64 node-block product)
    s.ctx.call("mpet_assemble", dt, 1)
    bm = torch.empty(s.N, dtype=torch.float64, device=s.device)
    s.ctx.call("mpet_rhs", dt, _lib()._ptr(up), _lib()._ptr(bm))
    torch.cuda.synchronize()
    assert np.allclose(_np(bm), b, rtol=1e-12, atol=1e-13 * np.abs(b).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,J", [(4, 2), (3, 4)])
def test_step_matches_direct_solve(precision, n, J):
    problem, dt = make_problem(n, J)
    s = _solver(problem, dt, precision=precision, rtol=1e-11)
    om = make_oracle(problem)
    rng = np.random.default_rng(2)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, 0.0, dt, oracle_data(J))
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(0.0)
    st = s.step(dt)
    x = _np(s.up.vector())
    err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    assert st.status == 0
    assert err <= 1e-8, (err, s.last_stats)
    assert float(problem.time) == pytest.approx(dt)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_direct_sequence(precision):
    J = 2
    problem, dt = make_problem(4, J)
    s = _solver(problem, dt, precision=precision, T=6 * dt)
    om = make_oracle(problem)
    ref = list(om.solve_direct(np.zeros(om.dm.N), 0.0, 6 * dt, dt, oracle_data(J)))
    got = []
    for up, t in s.solve():
        got.append((_np(up.vector()).copy(), t))
    assert len(got) == len(ref) == 6
    for (xg, tg), (xr, tr) in zip(got, ref):
        assert tg == pytest.approx(tr)
        assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)
    assert len(s.solver_monitor["niter"]) == 6


def test_apply_symmetric_matches_zero_rows_columns():
    J = 2
    problem, dt = make_problem(3, J)
    s = _solver(problem, dt, precision="fp64")
    om = make_oracle(problem)
    data = oracle_data(J)
    A = om.assemble_matrix(dt)
    dofs, vals = om.dirichlet_values(dt, data)
    Abc = om.apply_bc_matrix(A, dofs)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(om.dm.N)
    xbc = np.zeros(om.dm.N)
    for d, v in zip(dofs, vals):
        xbc[d] = v
        b[d] = v
    As, bs = om.zero_rows_columns(Abc, dofs, b, xbc)
    s.ctx.call("mpet_assemble", dt, 1)
    bg = torch.tensor(b, device=s.device)
    xg = torch.tensor(xbc, device=s.device)
    s.ctx.call("mpet_apply_symmetric", _lib()._ptr(bg), _lib()._ptr(xg))
    v = s.matrix_values()
    assert np.allclose(v, As.data, rtol=1e-12, atol=1e-13 * np.abs(As.data).max())
    assert np.allclose(_np(bg), bs, rtol=1e-12, atol=1e-12 * np.abs(bs).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_spmv_parity(precision):
    J = 4
    problem, dt = make_problem(3, J)
    s = _solver(problem, dt, precision=precision)
    om = make_oracle(problem)
    A = om.apply_bc_matrix(om.assemble_matrix(dt), om.dirichlet_values(dt, oracle_data(J))[0])
    s.ctx.call("mpet_assemble", dt, 1)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(om.dm.N)
    y_ref = A @ x
    y64 = torch.empty(s.N, dtype=torch.float64, device=s.device)
    xg = torch.tensor(x, device=s.device)
    # every SpMV variant that can run on this matrix (CSR register / staged,
    # SELL-32), not only the autotuned one
    ran = []
    for v in (0, 1, 2, 3, 4, 5, 8):
        try:
            s.ctx.call("mpet_set_spmv_variant", v)
        except _lib().MpetError:
            continue
        ran.append(v)
        s.ctx.call("mpet_spmv", 0, _lib()._ptr(xg), _lib()._ptr(y64))
        torch.cuda.synchronize()
        assert np.allclose(_np(y64), y_ref, rtol=1e-12, atol=1e-12 * np.abs(y_ref).max())
        if precision == "mixed":
            y32 = torch.empty(s.N, dtype=torch.float32, device=s.device)
            x32 = torch.tensor(x, dtype=torch.float32, device=s.device)
            s.ctx.call("mpet_spmv", 1, _lib()._ptr(x32), _lib()._ptr(y32))
            torch.cuda.synchronize()
            assert np.linalg.norm(_np(y32) - y_ref) <= 1e-5 * np.linalg.norm(y_ref)
    assert 4 in ran and 5 in ran and 8 in ran


def test_residual_matches_oracle():
    J = 2
    problem, dt = make_problem(4, J)
    s = _solver(problem, dt, precision="mixed")
    om = make_oracle(problem)
    A = om.apply_bc_matrix(om.assemble_matrix(dt), om.dirichlet_values(dt, oracle_data(J))[0])
    s.ctx.call("mpet_assemble", dt, 1)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(om.dm.N)
    b = rng.standard_normal(om.dm.N)
    r_ref = b - A @ x
    dinv = 1.0 / np.abs(A.diagonal())
    nr_ref, nb_ref = np.linalg.norm(r_ref * dinv), np.linalg.norm(b * dinv)
    r = torch.empty(s.N, dtype=torch.float64, device=s.device)
    norms = np.zeros(2)
    bg = torch.tensor(b, device=s.device)
    xg = torch.tensor(x, device=s.device)
    s.ctx.call("mpet_residual", _lib()._ptr(bg), _lib()._ptr(xg), _lib()._ptr(r), _lib()._ptr(norms))
    assert np.allclose(_np(r), r_ref, rtol=1e-12, atol=1e-12 * np.abs(r_ref).max())
    assert norms[0] == pytest.approx(nr_ref, rel=1e-12)
    assert norms[1] == pytest.approx(nb_ref, rel=1e-12)


def test_theta_half_step_matches_direct_solve():
    J = 2
    problem, dt = make_problem(4, J)
    s = _solver(problem, dt, precision="mixed", theta=0.5, rtol=1e-11)
    om = make_oracle(problem, theta=0.5)
    rng = np.random.default_rng(6)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, 0.0, dt, oracle_data(J))
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(0.0)
    s.step(dt)
    x = _np(s.up.vector())
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def _facet_problem(theta):
    """Neumann traction on x=1 (momentum), flux on x=0 (network 0), Robin on y=1 (network 1)."""
    from waterscapes_gb300 import CompiledSubDomain, Constant, Expression
    J = 2
    problem, dt = make_problem(3, J)
    near = lambda v, c: abs(v - c) < 1e-12
    CompiledSubDomain(lambda x: near(x[:, 0], 1.0)).mark(problem.momentum_boundary_markers, 1)
    CompiledSubDomain(lambda x: near(x[:, 0], 0.0)).mark(problem.continuity_boundary_markers[0], 1)
    CompiledSubDomain(lambda x: near(x[:, 1], 1.0)).mark(problem.continuity_boundary_markers[1], 2)
    s = lambda x, t, n: (1.0 + t) * n * x[:, :1]
    I0 = lambda x, t: x[:, 1] + t
    beta1 = lambda x, t: 2.0 + x[:, 2] + t
    pr1 = lambda x, t: x[:, 0] * (1.0 + t)
    problem.s = Expression(s)
    problem.I = [Expression(I0), Constant(0.0)]
    problem.beta = [Constant(0.0), Expression(beta1)]
    problem.p_robin = [Constant(0.0), Expression(pr1)]
    data = oracle_data(J)
    data.update({"s": s, "I": [I0, None], "beta": [None, beta1], "p_robin": [None, pr1]})
    return problem, dt, data


def test_facet_terms_matrix_and_rhs():
    theta = 0.5
    problem, dt, data = _facet_problem(theta)
    s = _solver(problem, dt, theta=theta, precision="fp64")
    om = make_oracle(problem, theta)
    t0 = 0.2
    problem.time.assign(t0)
    s._assemble(dt)
    A = om.assemble_matrix(dt, t0, data)
    dofs, _ = om.dirichlet_values(t0 + dt, data)
    A = om.apply_bc_matrix(A, dofs)
    v = s.matrix_values()
    assert np.allclose(v, A.data, rtol=1e-12, atol=1e-13 * np.abs(A.data).max())
    rng = np.random.default_rng(7)
    up_prev = rng.standard_normal(om.dm.N)
    t_theta, t1 = t0 + theta * dt, t0 + dt
    b = om.rhs_L(up_prev, dt) + om.rhs_L1(up_prev, dt, t_theta, data) + om.rhs_L0(t1, data)
    dofs, vals = om.dirichlet_values(t1, data)
    b = om.apply_bc_vector(b, dofs, vals)
    s._set_sources(t_theta, t1)
    s._set_facet_sources(t_theta, t1)
    s._set_bc_values(t1)
    up = torch.tensor(up_prev, dtype=torch.float64, device=s.device)
    bg = torch.empty(s.N, dtype=torch.float64, device=s.device)
    s.ctx.call("mpet_rhs", dt, _lib()._ptr(up), _lib()._ptr(bg))
    torch.cuda.synchronize()
    assert np.allclose(_np(bg), b, rtol=1e-12, atol=1e-13 * np.abs(b).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_facet_terms_step_matches_direct_solve(precision):
    problem, dt, data = _facet_problem(1.0)
    s = _solver(problem, dt, precision=precision, rtol=1e-11)
    om = make_oracle(problem)
    rng = np.random.default_rng(8)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, 0.0, dt, data)
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(0.0)
    s.step(dt)
    x = _np(s.up.vector())
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ellipsoid_per_cell_permeability_step(precision):
    """Jittered ellipsoidal shell with log-normal per-cell K_a (the brain-like case)."""
    from waterscapes_gb300 import CompiledSubDomain, Constant, EllipsoidShellMesh, Expression, MPETProblem
    from helpers import p_bar_fn
    mesh = EllipsoidShellMesh(3, seed=3)
    J = 2
    rng = np.random.default_rng(9)
    K = [10.0 ** rng.normal(-3.0 + a, 0.5, size=mesh.num_cells()) for a in range(J)]
    problem = MPETProblem(mesh, Constant(0.0), params=dict(J=J, E=2909.09, nu=0.4545, alpha=(0.25, 0.25),
                                                           c=(1e-4, 1e-4), K=K, S=((0.0, 1e-2), (1e-2, 0.0))))
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(J):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.p_bar = [Expression(p_bar_fn(a)) for a in range(J)]
    dt = 0.01
    s = _solver(problem, dt, precision=precision, rtol=1e-11)
    om = make_oracle(problem)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, 0.0, dt, oracle_data(J))
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(0.0)
    s.step(dt)
    x = _np(s.up.vector())
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_assembly_and_solve_are_deterministic():
    J = 2
    problem, dt = make_problem(4, J)
    s = _solver(problem, dt, precision="mixed")
    s.ctx.call("mpet_assemble", dt, 1)
    v1 = s.matrix_values()
    s.ctx.call("mpet_assemble", dt, 1)
    v2 = s.matrix_values()
    assert np.array_equal(v1, v2)
    problem.time.assign(0.0)
    s.step(dt)
    x1 = _np(s.up.vector()).copy()
    problem.time.assign(0.0)
    s.step(dt)
    x2 = _np(s.up.vector()).copy()
    assert np.array_equal(x1, x2)


def test_preconditioner_spmv_variants_agree_and_symmetric():
    """The block AMG preconditioner gives the same z = M^-1 r with every SpMV
    variant of its matrices (CSR register, SELL-32 with 4 / 8 entries per
    batch; rectangular prolongations and restrictions included), and M^-1 is
    symmetric (MINRES needs it)."""
    problem, dt = make_problem(5, 2)
    s = _solver(problem, dt, precision="fp64")
    s._assemble(dt)
    rng = np.random.default_rng(11)
    r = torch.tensor(rng.standard_normal(s.N), device=s.device)
    q = torch.tensor(rng.standard_normal(s.N), device=s.device)
    out = {}
    for v in (0, 4, 5):
        s.ctx.call("mpet_set_hierarchy_spmv_variant", v)
        z = torch.empty_like(r)
        s.ctx.call("mpet_apply_preconditioner", 0, _lib()._ptr(r), _lib()._ptr(z))
        w = torch.empty_like(r)
        s.ctx.call("mpet_apply_preconditioner", 0, _lib()._ptr(q), _lib()._ptr(w))
        torch.cuda.synchronize()
        out[v] = (_np(z), _np(w))
    z0 = out[0][0]
    assert np.all(np.isfinite(z0)) and np.linalg.norm(z0) > 0
    for v in (4, 5):
        assert np.linalg.norm(out[v][0] - z0) <= 1e-12 * np.linalg.norm(z0)
    z, w = out[0]
    rq = float(_np(q) @ z)
    qr = float(_np(r) @ w)
    assert abs(rq - qr) <= 1e-10 * (abs(rq) + abs(qr))
