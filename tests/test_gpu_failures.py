"""Failure detection on the GPU path, without faulting the GPU.

Each failure is made on the host side (an iteration limit of 1, a NaN in the
previous state or in the Dirichlet data, a wait bound of zero polls) and
must come back as a status code from the C ABI, with the context still
usable for a correct step afterwards:

* MPET_ERR_MAXIT when the Krylov iteration limit is reached;
* MPET_ERR_BREAKDOWN for non-finite data (the reference would hand PETSc a
  NaN right-hand side; here the first reduction flags it);
* MPET_ERR_TIMEOUT when the staged SpMV's bounded mbarrier waits give up:
  with a bound of 0 polls every tile wait gives up at once, the kernel sets
  the device error flag, waits for its copies in flight under the default
  bound and exits; the next call with the default bound is correct.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MAXIT, BREAKDOWN, TIMEOUT = -4, -5, -6


def _oracle_step(problem, dt):
    om = make_oracle(problem)
    return om.step(np.zeros(om.dm.N), 0.0, dt, oracle_data(int(problem.params["J"])))


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_iteration_limit_then_usable(precision):
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = make_problem(3, 2)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision=precision, maxit=1, rtol=1e-11))
    with pytest.raises(_lib.MpetError) as e:
        s.step(dt)
    assert e.value.code == MAXIT
    # the same context, with a usable limit, gives the oracle's step
    s._prm.maxit = 5000
    s.ctx.call("mpet_update_params", ctypes.byref(s._prm))
    s._assembled_dt = s._prec_dt = None
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    assert _rel(s.up.vector().cpu().numpy(), _oracle_step(problem, dt)) <= 1e-8


@pytest.mark.parametrize("where", ["previous_state", "dirichlet_data"])
def test_nonfinite_data_is_reported_then_usable(where):
    from waterscapes_gb300 import Expression, MPETSolver, _lib
    problem, dt = make_problem(3, 2)
    good = list(problem.p_bar)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="mixed", rtol=1e-11))
    if where == "previous_state":
        # an interior pressure DOF (a Dirichlet DOF of up_ is replaced by its boundary value)
        bc = set(s._bcs[1]["dofs"].cpu().numpy().tolist())
        dof = next(d for d in range(s.Nu, s.Nu + s.nv) if d not in bc)
        s.up_.vector()[dof] = float("nan")
    else:
        problem.p_bar = [Expression(lambda x, t: torch.full((x.shape[0],), float("nan"), dtype=torch.float64,
                                                            device=x.device))] + good[1:]
    with pytest.raises(_lib.MpetError) as e:
        s.step(dt)
    assert e.value.code == BREAKDOWN
    # clean data on the same context (the state a failed step leaves is unspecified)
    problem.p_bar = good
    s.up_.vector().zero_()
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    assert _rel(s.up.vector().cpu().numpy(), _oracle_step(problem, dt)) <= 1e-8


def test_staged_spmv_wait_timeout_is_reported_then_usable():
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = make_problem(4, 2)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="fp64"))
    s.ctx.call("mpet_assemble", dt, 1)
    rng = np.random.default_rng(3)
    x = torch.tensor(rng.standard_normal(s.N), device=s.device)
    b = torch.tensor(rng.standard_normal(s.N), device=s.device)
    r_ref = torch.empty(s.N, dtype=torch.float64, device=s.device)
    n_ref = np.zeros(2)
    s.ctx.call("mpet_residual", _lib._ptr(b), _lib._ptr(x), _lib._ptr(r_ref), _lib._ptr(n_ref))
    torch.cuda.synchronize()
    ran = []
    for variant in (2, 3):                       # staged tiles; 3 = deeper batches (32 lanes per row only)
        if s.ctx.lib.mpet_set_spmv_variant(s.ctx.h, variant) != 0:
            continue
        ran.append(variant)
        s.ctx.call("mpet_set_wait_limit", 0)
        r = torch.zeros(s.N, dtype=torch.float64, device=s.device)
        n = np.zeros(2)
        rc = s.ctx.lib.mpet_residual(s.ctx.h, _lib._ptr(b), _lib._ptr(x), _lib._ptr(r), _lib._ptr(n))
        assert rc == TIMEOUT
        s.ctx.call("mpet_set_wait_limit", 1 << 22)
        s.ctx.call("mpet_residual", _lib._ptr(b), _lib._ptr(x), _lib._ptr(r), _lib._ptr(n))
        torch.cuda.synchronize()
        rr, rn = r_ref.cpu().numpy(), r.cpu().numpy()
        assert np.allclose(rn, rr, rtol=1e-12, atol=1e-12 * np.abs(rr).max())
        assert n[0] == pytest.approx(n_ref[0], rel=1e-12)
    assert 2 in ran
