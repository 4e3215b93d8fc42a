"""Edge cases of the GPU path: the largest network count, one network with
every boundary-term kind, a single-cell mesh, and the error codes the C ABI
returns instead of faulting (call order, bad sizes, aliased vectors,
overlapping batch instances).
"""
import ctypes

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _solver(problem, dt, **kw):
    from waterscapes_gb300 import MPETSolver
    params = dict(dt=dt, T=10 * dt, theta=1.0, rtol=1e-11)
    params.update(kw)
    return MPETSolver(problem, params)


def _step_check(problem, dt, data, precision, theta=1.0, tol=1e-8):
    s = _solver(problem, dt, precision=precision, theta=theta)
    om = make_oracle(problem, theta)
    rng = np.random.default_rng(21)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, 0.0, dt, data)
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(0.0)
    s.step(dt)
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= tol * np.linalg.norm(x_ref)
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_eight_networks_step(precision):
    """J = 8 (MPET_MAX_NETWORKS) with a dense symmetric transfer matrix."""
    problem, dt = make_problem(2, 8)
    S = np.full((8, 8), 3e-2)
    np.fill_diagonal(S, 0.0)
    problem.params["S"] = tuple(map(tuple, S))
    _step_check(problem, dt, oracle_data(8), precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_one_network_flux_and_robin(precision):
    """J = 1: traction on x=1, flux on x=0 and Robin on y=1 for the single network."""
    from waterscapes_gb300 import CompiledSubDomain, Constant, Expression
    problem, dt = make_problem(3, 1)
    near = lambda v, c: abs(v - c) < 1e-12  # noqa: E731
    CompiledSubDomain(lambda x: near(x[:, 0], 1.0)).mark(problem.momentum_boundary_markers, 1)
    CompiledSubDomain(lambda x: near(x[:, 0], 0.0)).mark(problem.continuity_boundary_markers[0], 1)
    CompiledSubDomain(lambda x: near(x[:, 1], 1.0)).mark(problem.continuity_boundary_markers[0], 2)
    s = lambda x, t, n: (1.0 + t) * n * x[:, :1]  # noqa: E731
    I0 = lambda x, t: x[:, 1] + t  # noqa: E731
    beta0 = lambda x, t: 1.5 + x[:, 2]  # noqa: E731
    pr0 = lambda x, t: x[:, 0] - t  # noqa: E731
    problem.s = Expression(s)
    problem.I = [Expression(I0)]
    problem.beta = [Expression(beta0)]
    problem.p_robin = [Expression(pr0)]
    data = oracle_data(1)
    data.update({"s": s, "I": [I0], "beta": [beta0], "p_robin": [pr0]})
    _step_check(problem, dt, data, precision)


def test_single_cube_mesh():
    """The smallest mesh: one hexahedron split in 6 tetrahedra (every node on the boundary
    except none: all DOFs are Dirichlet or boundary-adjacent)."""
    problem, dt = make_problem(1, 2)
    _step_check(problem, dt, oracle_data(2), "fp64")


def test_error_codes_instead_of_faults():
    from waterscapes_gb300 import _lib
    lib = _lib.load()
    ctx = ctypes.c_void_p()
    assert lib.mpet_ctx_create(0, ctypes.byref(ctx)) == 0
    try:
        # call order: nothing set up yet
        assert lib.mpet_assemble(ctx, ctypes.c_double(0.1), 1) == -7
        st = _lib.MpetStats()
        assert lib.mpet_solve(ctx, None, None, ctypes.byref(st)) == -7
        # bad sizes: 9 networks
        problem, dt = make_problem(1, 2)
        m = problem.mesh
        x = np.ascontiguousarray(m.coordinates())
        cells = np.ascontiguousarray(m.cells(), dtype=np.int32)
        bf = np.ascontiguousarray(m.boundary_facets(), dtype=np.int32)
        markers = np.zeros((10, bf.shape[0]), dtype=np.int32)
        rc = lib.mpet_mesh_upload(ctx, x.shape[0], _lib._ptr(x), cells.shape[0], _lib._ptr(cells),
                                  bf.shape[0], _lib._ptr(bf), _lib._ptr(markers), 9)
        assert rc == -1
        msg = lib.mpet_last_error(ctx).decode()
        assert msg
    finally:
        lib.mpet_ctx_destroy(ctx)


def test_aliased_vectors_and_overlapping_instances_rejected():
    from waterscapes_gb300 import _lib
    problem, dt = make_problem(2, 2)
    s = _solver(problem, dt)
    s._assemble(dt)
    v = torch.zeros(s.N, dtype=torch.float64, device=s.device)
    st = _lib.MpetStats()
    lib = _lib.load()
    h = s.ctx.h
    assert lib.mpet_step(h, ctypes.c_double(dt), _lib._ptr(v), _lib._ptr(v), ctypes.byref(st)) == -1
    assert lib.mpet_adjoint_rhs(h, ctypes.c_double(dt), _lib._ptr(v), _lib._ptr(v)) == -1
    # a batch partition whose instances share an edge
    inst = np.zeros(s.nv, dtype=np.int32)
    inst[0] = 1
    assert lib.mpet_set_batch(h, 2, _lib._ptr(inst)) == -1
    # the context stays usable
    s.step(dt)
    assert torch.isfinite(s.up.vector()).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_elasticity_preconditioner_form(precision):
    """prec_u_form = "elasticity" (the displacement block of the system with rigid-body-mode
    aggregation) gives the oracle's step with fewer MINRES iterations than the vector
    Laplacian form."""
    import ctypes
    problem, dt = make_problem(6, 2)
    om = make_oracle(problem, 1.0)
    data = oracle_data(2)
    rng = np.random.default_rng(4)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, 0.0, dt, data)
    its = {}
    for form in ("laplacian", "elasticity"):
        s = _solver(problem, dt, precision=precision, prec_u_form=form)
        s.up_.assign(torch.tensor(up_prev))
        problem.time.assign(0.0)
        st = s.step(dt)
        x = s.up.vector().cpu().numpy()
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
        v = ctypes.c_int32()
        s.ctx.call("mpet_get_prec_info", ctypes.byref(v))
        assert v.value == (1 if form == "elasticity" else 0)
        its[form] = st.iterations
    assert its["elasticity"] < its["laplacian"]
