"""The allocation-free residual entry point against the regular one.

mpet_residual_noalloc serves callers that cannot allocate device memory
(their allocator already owns the device's free memory, or they may not
allocate after start-up).  It must give what mpet_residual gives, on two
calls in a row (the static scratch keeps the previous call's contents), and
the device's free memory must not change across a call.  Two systems are
checked: a 3D cube (32 lanes per row in the residual kernel) and a 2D
square (16 lanes per row).  The test passes both when this file runs alone
in a fresh process and after the other tests; the file name makes pytest
collect it last.
"""
import numpy as np
import pytest

from helpers import make_problem

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _square_problem():
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, UnitSquareMesh
    params = dict(J=2, c=(0.3, 0.4), alpha=(0.4, 0.6), K=(0.2, 0.3), S=((0.0, 1.5), (1.5, 0.0)), E=520.0, nu=0.47)
    problem = MPETProblem(UnitSquareMesh(6), Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(2):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    return problem, 0.1


@pytest.mark.parametrize("case", ["cube", "square"])
def test_residual_noalloc_matches_residual_twice(case):
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = make_problem(4, 2) if case == "cube" else _square_problem()
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="mixed"))
    s.ctx.call("mpet_assemble", dt, 1)
    rng = np.random.default_rng(11)
    for call in range(2):
        x = torch.tensor(rng.standard_normal(s.N), device=s.device)
        b = torch.tensor(rng.standard_normal(s.N) * (call + 1), device=s.device)
        r_ref = torch.empty(s.N, dtype=torch.float64, device=s.device)
        r_new = torch.full((s.N,), float("nan"), dtype=torch.float64, device=s.device)
        n_ref = np.zeros(2)
        n_new = np.zeros(2)
        s.ctx.call("mpet_residual", _lib._ptr(b), _lib._ptr(x), _lib._ptr(r_ref), _lib._ptr(n_ref))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(s.device)[0]
        s.ctx.call("mpet_residual_noalloc", _lib._ptr(b), _lib._ptr(x), _lib._ptr(r_new), _lib._ptr(n_new))
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(s.device)[0] == free_before
        rr, rn = r_ref.cpu().numpy(), r_new.cpu().numpy()
        assert np.allclose(rn, rr, rtol=1e-12, atol=1e-12 * np.abs(rr).max())
        assert n_new[0] == pytest.approx(n_ref[0], rel=1e-12)
        assert n_new[1] == pytest.approx(n_ref[1], rel=1e-12)
