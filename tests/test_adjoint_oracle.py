"""The oracle's discrete adjoint against its own forward model (CPU).

* the assembled old-state operator B reproduces rhs(F) (the vector the time
  loop assembles from the previous state);
* the adjoint gradient of the final-pressure misfit with respect to the
  per-cell K_a fields matches central finite differences of the LU forward
  model along random directions, for theta = 1 and theta = 0.5.
"""
import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data
from oracle import adjoint


def _case(n, J, theta, seed=0):
    problem, dt = make_problem(n, J)
    om = make_oracle(problem, theta=theta)
    rng = np.random.default_rng(seed)
    nc = om.vol.shape[0]
    base = np.asarray(problem.params["K"], dtype=np.float64)
    om.Kc = np.stack([base[a] * np.exp(0.5 * rng.standard_normal(nc)) for a in range(J)])
    return om, dt, rng


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_old_state_matrix_reproduces_rhs(theta):
    om, dt, rng = _case(2, 2, theta)
    x = rng.standard_normal(om.dm.N)
    B = adjoint.old_state_matrix(om, dt)
    ref = om.rhs_L(x, dt)
    assert np.abs(B @ x - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_adjoint_gradient_matches_central_differences(theta):
    om, dt, rng = _case(2, 2, theta, seed=1)
    data = oracle_data(2)
    nsteps = 4
    x0 = np.zeros(om.dm.N)
    target = 0.05 * rng.standard_normal((2, om.dm.nv))
    xs = adjoint.forward(om, x0, 0.0, nsteps, dt, data)
    loss, grad = adjoint.gradient(om, xs, target, dt, data)
    assert loss > 0.0
    K0 = om.Kc.copy()
    h = 1e-6

    def loss_at(K):
        om.Kc = K
        return adjoint.misfit(om, adjoint.forward(om, x0, 0.0, nsteps, dt, data)[-1], target)[0]

    for _ in range(3):
        dK = K0 * rng.standard_normal(K0.shape)
        fd = (loss_at(K0 + h * dK) - loss_at(K0 - h * dK)) / (2.0 * h)
        ad = float(np.sum(grad * dK))
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-14
    om.Kc = K0
