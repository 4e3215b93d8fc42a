"""GPU discrete adjoint (per-cell K) against the oracle's adjoint and against
central finite differences of the GPU forward model.

Bars: misfit and B^T lam within 1e-12 relative (FP64, different summation
order); FP64 gradient within 1e-8 relative of the oracle's LU adjoint; the
mixed-precision gradient within 1e-6 of the FP64 one; central differences
(h = 1e-6 along K-relative random directions) within 1e-5 of the adjoint;
checkpoint spacing and the autograd wrapper agree to 1e-9 (each driver
rebuilds the preconditioner, whose autotuned SpMV variant may sum in another
order).
"""
import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _case(n=3, J=2, theta=1.0, precision="fp64", seed=0):
    from waterscapes_gb300 import MPETSolver
    problem, dt = make_problem(n, J)
    nc = problem.mesh.num_cells()
    rng = np.random.default_rng(seed)
    base = np.asarray(problem.params["K"], dtype=np.float64)
    K = np.stack([base[a] * np.exp(0.5 * rng.standard_normal(nc)) for a in range(J)])
    s = MPETSolver(problem, dict(dt=dt, T=10 * dt, theta=theta, precision=precision, rtol=1e-13))
    om = make_oracle(problem, theta=theta)
    om.Kc = K.copy()
    target = 0.05 * rng.standard_normal((J, problem.mesh.num_vertices()))
    return s, om, K, target, dt, rng


def _dev(a, s):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=s.device)


def test_misfit_matches_oracle():
    from oracle import adjoint as oadj
    s, om, K, target, dt, rng = _case()
    x = rng.standard_normal(s.N)
    from waterscapes_gb300.adjoint import MisfitAdjoint
    drv = MisfitAdjoint(s, target, 1)
    loss, d = drv.misfit(_dev(x, s))
    ref_loss, ref_d = oadj.misfit(om, x, target)
    assert abs(loss - ref_loss) <= 1e-12 * abs(ref_loss)
    assert np.abs(d.cpu().numpy() - ref_d).max() <= 1e-12 * np.abs(ref_d).max()


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_adjoint_rhs_matches_oracle(theta):
    from oracle import adjoint as oadj
    s, om, K, target, dt, rng = _case(theta=theta)
    s.set_cell_permeability(K)
    lam = rng.standard_normal(s.N)
    bc = np.unique(np.concatenate([dd for _, dd in om.dirichlet_dofs()]))
    lam[bc] = 0.0
    out = torch.empty(s.N, dtype=torch.float64, device=s.device)
    from waterscapes_gb300 import _lib
    s.ctx.call("mpet_adjoint_rhs", dt, _lib._ptr(_dev(lam, s)), _lib._ptr(out))
    torch.cuda.synchronize()
    ref = oadj.old_state_matrix(om, dt).T @ lam
    ref[bc] = 0.0
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def _gpu_grad(s, K, target, nsteps, every=2):
    from waterscapes_gb300.adjoint import MisfitAdjoint
    s.problem.time.assign(0.0)
    drv = MisfitAdjoint(s, target, nsteps, checkpoint_every=every, t0=0.0,
                        up0=torch.zeros(s.N, dtype=torch.float64, device=s.device))
    loss, g = drv.loss_and_grad(_dev(K, s))
    return loss, g.cpu().numpy(), drv


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_gradient_matches_oracle_adjoint(theta):
    from oracle import adjoint as oadj
    s, om, K, target, dt, rng = _case(theta=theta)
    nsteps = 4
    loss, g, _ = _gpu_grad(s, K, target, nsteps)
    xs = oadj.forward(om, np.zeros(om.dm.N), 0.0, nsteps, dt, oracle_data(2))
    ref_loss, ref_g = oadj.gradient(om, xs, target, dt, oracle_data(2))
    assert abs(loss - ref_loss) <= 1e-9 * abs(ref_loss)
    assert np.linalg.norm(g - ref_g) <= 1e-8 * np.linalg.norm(ref_g)


def test_mixed_gradient_matches_fp64():
    s64, _, K, target, dt, _ = _case(precision="fp64")
    s32, _, _, _, _, _ = _case(precision="mixed")
    _, g64, _ = _gpu_grad(s64, K, target, 4)
    _, g32, _ = _gpu_grad(s32, K, target, 4)
    assert np.linalg.norm(g32 - g64) <= 1e-6 * np.linalg.norm(g64)


def test_gradient_matches_central_differences():
    s, _, K, target, dt, rng = _case(seed=3)
    nsteps = 3
    loss, g, drv = _gpu_grad(s, K, target, nsteps)
    h = 1e-6
    for _ in range(4):
        dK = K * rng.standard_normal(K.shape)
        lp = drv.forward(_dev(K + h * dK, s))
        lm = drv.forward(_dev(K - h * dK, s))
        fd = (lp - lm) / (2.0 * h)
        ad = float(np.sum(g * dK))
        assert abs(fd - ad) <= 1e-5 * abs(ad)


def test_checkpoint_spacing_and_autograd():
    from waterscapes_gb300.adjoint import pressure_misfit
    s, _, K, target, dt, _ = _case(seed=5)
    _, g1, _ = _gpu_grad(s, K, target, 5, every=1)
    _, g3, _ = _gpu_grad(s, K, target, 5, every=3)
    assert np.linalg.norm(g1 - g3) <= 1e-9 * np.linalg.norm(g1)
    Kt = _dev(K, s).requires_grad_(True)
    s.problem.time.assign(0.0)
    loss = pressure_misfit(s, Kt, target, 5, checkpoint_every=2, t0=0.0,
                           up0=torch.zeros(s.N, dtype=torch.float64, device=s.device))
    (gK,) = torch.autograd.grad(2.0 * loss, Kt)
    assert np.linalg.norm(gK.cpu().numpy() - 2.0 * g1) <= 1e-9 * np.linalg.norm(2.0 * g1)
