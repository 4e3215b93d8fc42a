"""The matrix-free first level of the displacement preconditioner against its
CSR copy.

The block w (grad u, grad v) (+ shift (u, v) when the displacement has rigid
modes) of mpetsolver.py:269 is applied from per-cell data (k_p2lap_mf) or from
the assembled CSR block; both are the same operator, so one preconditioner
application agrees to round-off (FP64: 1e-12; FP32: 1e-4 relative, the FP32
sums running in a different order), and a step with the matrix-free level is
the oracle's step.  Cases: the Kuhn cube (3D), the unit square (2D) and the
donut known answer (pure traction: the shifted block, no Dirichlet nodes).
"""
import ctypes

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _apply(s, mode, dt):
    from waterscapes_gb300 import _lib
    s.ctx.call("mpet_set_prec_matrix_free", mode)
    s.ctx.call("mpet_setup_preconditioner", dt)
    used = ctypes.c_int32()
    s.ctx.call("mpet_get_prec_matrix_free", ctypes.byref(used), None)
    assert used.value == mode
    mixed = s.params["precision"] == "mixed"
    dtype = torch.float32 if mixed else torch.float64
    r = torch.tensor(np.random.default_rng(4).standard_normal(s.N), dtype=dtype, device=s.device)
    z = torch.empty_like(r)
    s.ctx.call("mpet_apply_preconditioner", 1 if mixed else 0, _lib._ptr(r), _lib._ptr(z))
    torch.cuda.synchronize()
    return z.double().cpu().numpy()


def _square(n):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, UnitSquareMesh
    params = dict(J=2, c=(0.3, 0.4), alpha=(0.4, 0.6), K=(0.2, 0.3), S=((0.0, 1.5), (1.5, 0.0)), E=520.0, nu=0.47)
    problem = MPETProblem(UnitSquareMesh(n), Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(2):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    return problem, 0.1


@pytest.mark.parametrize("case,precision", [("cube", "fp64"), ("cube", "mixed"), ("square", "fp64")])
def test_matrix_free_level_matches_csr_level(case, precision):
    from waterscapes_gb300 import MPETSolver
    problem, dt = make_problem(5, 2) if case == "cube" else _square(8)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision=precision, rtol=1e-11))
    s.ctx.call("mpet_assemble", dt, 1)
    z0 = _apply(s, 0, dt)
    z1 = _apply(s, 1, dt)
    tol = 1e-12 if precision == "fp64" else 1e-4
    assert np.linalg.norm(z1 - z0) <= tol * np.linalg.norm(z0)
    # a step with the matrix-free level (still forced on for the next set-up)
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    if case == "cube":
        om = make_oracle(problem)
        x_ref = om.step(np.zeros(om.dm.N), 0.0, dt, oracle_data(2))
        x = s.up.vector().cpu().numpy()
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_matrix_free_level_with_rigid_modes():
    """Donut known answer (test_donut.py:70-71) with the matrix-free shifted block."""
    from waterscapes_gb300 import MPETSolver
    from waterscapes_gb300.mesh import AnnulusMesh
    from test_gpu_nullspace import _donut_problem
    problem = _donut_problem(AnnulusMesh(40.0, 60.0, 8, 64))
    s = MPETSolver(problem, dict(dt=0.1, theta=1.0, T=0.2, precision="fp64", rtol=1e-12))
    s.ctx.call("mpet_set_prec_matrix_free", 1)
    for up, t in s.solve():
        pass
    p = up.split(deepcopy=True)[1].cpu().numpy()
    assert np.abs(p + 0.2).max() <= 1e-8
