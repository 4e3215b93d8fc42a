"""Rigid-motion nullspace of the displacement on the GPU path.

* the donut known answer of src/mpet/test/test_donut.py:16-71 (J = 1, c = 0,
  alpha = 1, K = 1e-2, S = 0, E = 500, nu = 0.35; traction s = t n on the whole
  boundary, p = -t on the whole boundary, u_has_nullspace, dt = 0.1, T = 0.2):
  the pressure is the constant -0.2 at T, checked at every vertex to 1e-8 and
  through ||p||_L2 / sqrt(|Omega|) = 0.2 to 1e-10, as the reference asserts.
  The reference reads donut2D.h5; the exact solution is constant, so an annulus
  of the same kind (inner radius 40, outer radius 60, holding the point (0, 50))
  carries the same answer.  The 3D variant runs on an ellipsoidal shell.
* a random right-hand side on a shell with pure traction: the GPU solution is
  the oracle's solution of the bordered system (multipliers r for the L2-
  orthonormal rigid motions), and the displacement is L2-orthogonal to every
  rigid motion.
"""
import math

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from helpers import make_oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _donut_problem(mesh, J=1):
    from waterscapes_gb300 import CompiledSubDomain, Constant, Expression, MPETProblem
    params = dict(J=J, alpha=(1.0,) * J, K=(1e-2,) * J, S=((0.0,) * J,) * J, c=(0.0,) * J, nu=0.35, E=500.0)
    time = Constant(0.0)
    problem = MPETProblem(mesh, time, params=params)
    d = mesh.geometry().dim()
    problem.s = Expression(lambda x, t, n: float(t) * n[:, :d])
    problem.u_has_nullspace = True
    on_boundary = CompiledSubDomain.on_boundary()
    on_boundary.mark(problem.momentum_boundary_markers, 1)
    problem.p_bar = [Expression(lambda x, t: torch.full((x.shape[0],), -float(t), dtype=torch.float64,
                                                        device=x.device)) for _ in range(J)]
    for a in range(J):
        on_boundary.mark(problem.continuity_boundary_markers[a], 0)
    return problem


def _mass(om, field):
    """Oracle P1 vertex mass (field "p") or P2 vector mass on the displacement DOFs ("u")."""
    dm = om.dm
    if field == "p":
        cd, loc, n = dm.cells, om.M1, dm.nv
    else:
        d = dm.d
        cn = dm.cell_nodes
        cd = (d * cn[:, :, None] + np.arange(d)[None, None, :]).reshape(cn.shape[0], -1)
        loc = np.einsum("cij,kl->cikjl", om.M2, np.eye(d)).reshape(cn.shape[0], cd.shape[1], cd.shape[1])
        n = dm.Nu
    rows = np.repeat(cd, cd.shape[1], axis=1).ravel()
    cols = np.tile(cd, (1, cd.shape[1])).ravel()
    return sp.csr_matrix((loc.ravel(), (rows, cols)), shape=(n, n))


def _run_donut(mesh, precision):
    from waterscapes_gb300 import MPETSolver
    problem = _donut_problem(mesh)
    solver = MPETSolver(problem, dict(dt=0.1, theta=1.0, T=0.2, precision=precision, rtol=1e-12))
    t = None
    for up, t in solver.solve():
        pass
    assert abs(t - 0.2) < 1e-12
    u, p, r = up.split(deepcopy=True)
    return solver, make_oracle(problem), u.cpu().numpy(), p.cpu().numpy(), r.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_constant_on_the_donut_2d(precision):
    from waterscapes_gb300.mesh import AnnulusMesh
    mesh = AnnulusMesh(40.0, 60.0, 8, 64)
    solver, om, u, p, r = _run_donut(mesh, precision)
    assert solver.nrigid == 3 and r.shape == (3,)
    x = np.asarray(mesh.coordinates())
    i = int(np.argmin(np.hypot(x[:, 0], x[:, 1] - 50.0)))
    assert np.hypot(x[i, 0], x[i, 1] - 50.0) < 1e-12      # (0, 50) is a vertex of the annulus
    assert abs(p[i] + 0.2) < 1e-8
    assert np.abs(p + 0.2).max() < 1e-8
    M = _mass(om, "p")
    vol = M.sum()
    assert abs(math.sqrt(p @ (M @ p)) / math.sqrt(vol) - 0.2) < 1e-10
    assert np.abs(u).max() < 1e-8


def test_constant_on_the_shell_3d():
    from waterscapes_gb300.mesh import EllipsoidShellMesh
    mesh = EllipsoidShellMesh(3)
    solver, om, u, p, r = _run_donut(mesh, "mixed")
    assert solver.nrigid == 6 and r.shape == (6,)
    assert np.abs(p + 0.2).max() < 1e-8
    M = _mass(om, "p")
    assert abs(math.sqrt(p @ (M @ p)) / math.sqrt(M.sum()) - 0.2) < 1e-10
    assert np.abs(u).max() < 1e-8


@pytest.mark.parametrize("dim,precision", [(2, "fp64"), (3, "fp64"), (3, "mixed")])
def test_bordered_system_against_oracle(dim, precision):
    """Pure traction (every boundary facet Neumann for the displacement), Dirichlet
    pressure, random previous state: the GPU step equals the oracle's direct solve
    of the bordered system [A, B^T; B, 0] with B_i = (M Z_i)^T on the displacement."""
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, MPETSolver
    from waterscapes_gb300.mesh import AnnulusMesh, EllipsoidShellMesh
    from waterscapes_gb300.nullspace import rigid_motions
    mesh = AnnulusMesh(1.0, 2.0, 4, 24) if dim == 2 else EllipsoidShellMesh(2)
    J = 2
    params = dict(J=J, alpha=(0.5, 0.7), K=(0.3, 0.1), S=((0.0, 0.2), (0.2, 0.0)), c=(0.1, 0.2), nu=0.3, E=10.0)
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    on_boundary = CompiledSubDomain.on_boundary()
    on_boundary.mark(problem.momentum_boundary_markers, 1)
    for a in range(J):
        on_boundary.mark(problem.continuity_boundary_markers[a], 0)
    problem.u_has_nullspace = True
    dt = 0.05
    solver = MPETSolver(problem, dict(dt=dt, theta=1.0, T=10 * dt, precision=precision, rtol=1e-12))
    om = make_oracle(problem, 1.0)
    data = {"f": lambda x, t: np.stack([np.sin(x[:, k] + t) for k in range(dim)], 1),
            "g": [lambda x, t: x[:, 0] * (1 + t), lambda x, t: np.cos(x[:, 1])],
            "u_bar": lambda x, t: np.zeros((x.shape[0], dim)),
            "p_bar": [lambda x, t: 0.1 * x[:, 0] + t, lambda x, t: -0.2 * x[:, 1]]}
    from waterscapes_gb300 import Expression

    def wrap(fn):
        return Expression(lambda x, t: torch.as_tensor(np.asarray(fn(x[:, :dim].cpu().numpy(), t)),
                                                       device=x.device))
    problem.f = wrap(data["f"])
    problem.g = [wrap(g) for g in data["g"]]
    problem.p_bar = [wrap(p) for p in data["p_bar"]]
    rng = np.random.default_rng(5)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    t0 = 0.1
    # oracle: assembled system, pressure Dirichlet rows, bordered with the rigid motions
    _, Abc, bbc, _, _ = om.step(up_prev, t0, dt, data, return_system=True)
    Z = rigid_motions(mesh, om.dm.node_x).reshape(-1, om.dm.Nu)
    Mu = _mass(om, "u")
    assert np.allclose(Z @ (Mu @ Z.T), np.eye(Z.shape[0]), atol=1e-12)
    B = np.zeros((Z.shape[0], om.dm.N))
    B[:, :om.dm.Nu] = (Mu @ Z.T).T
    K = sp.bmat([[Abc, sp.csr_matrix(B).T], [sp.csr_matrix(B), None]]).tocsc()
    sol = spla.spsolve(K, np.concatenate([bbc, np.zeros(Z.shape[0])]))
    x_ref, r_ref = sol[:om.dm.N], sol[om.dm.N:]
    solver.up_.assign(torch.tensor(up_prev))
    problem.time.assign(t0)
    solver.step(dt)
    x = solver.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    r = solver.up.split()[-1].cpu().numpy()
    assert np.allclose(r, r_ref, rtol=1e-7, atol=1e-9 * np.abs(r_ref).max())
    # displacement L2-orthogonal to the rigid motions
    assert np.abs(B[:, :om.dm.Nu] @ x[:om.dm.Nu]).max() <= 1e-10 * np.linalg.norm(x[:om.dm.Nu])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_donut_with_pressure_nullspaces_against_oracle(precision):
    """The second case of src/mpet/test/test_donut.py:73-131 (J = 2, c = 0, alpha = 1,
    K = (1e-2, 1e-1), S = 0; traction t n everywhere, u_has_nullspace; both pressures
    only determined up to constants, p_has_nullspace = (True, True); network 0 marked
    Neumann, network 1 unmarked): one step equals the oracle's LU solve of the system
    bordered by the rigid motions and the two constant-pressure constraints, the
    pressures have zero mean, and the multipliers agree; then the reference's time loop
    (dt = 0.1, T = 0.2) runs through."""
    from waterscapes_gb300 import CompiledSubDomain, Constant, Expression, MPETProblem, MPETSolver
    from waterscapes_gb300.mesh import AnnulusMesh
    from waterscapes_gb300.nullspace import rigid_motions
    mesh = AnnulusMesh(1.0, 2.0, 4, 24)
    params = dict(J=2, c=(0.0, 0.0), alpha=(1.0, 1.0), K=(1e-2, 1e-1), S=((0.0, 0.0), (0.0, 0.0)), E=500.0,
                  nu=0.35)
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    problem.s = Expression(lambda x, t, n: float(t) * n[:, :2])
    problem.u_has_nullspace = True
    problem.p_has_nullspace = (True, True)
    on_boundary = CompiledSubDomain.on_boundary()
    on_boundary.mark(problem.momentum_boundary_markers, 1)
    on_boundary.mark(problem.continuity_boundary_markers[0], 1)
    dt, t0 = 0.1, 0.1
    solver = MPETSolver(problem, dict(dt=dt, theta=1.0, T=0.2, precision=precision, rtol=1e-12))
    assert solver.nq == 2 and solver.nrigid == 3
    om = make_oracle(problem, 1.0)
    data = {"s": lambda x, t, n: t * n}
    rng = np.random.default_rng(9)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    _, Abc, bbc, _, _ = om.step(up_prev, t0, dt, data, return_system=True)
    Nu, nv, N = om.dm.Nu, om.dm.nv, om.dm.N
    Z = rigid_motions(mesh, om.dm.node_x).reshape(-1, Nu)
    Mu = _mass(om, "u")
    Mp = _mass(om, "p")
    load = np.asarray(Mp.sum(axis=1)).ravel()                 # int phi_v
    B = np.zeros((Z.shape[0] + 2, N))
    B[:Z.shape[0], :Nu] = (Mu @ Z.T).T
    for a in range(2):
        B[Z.shape[0] + a, Nu + a * nv: Nu + (a + 1) * nv] = load
    K = sp.bmat([[Abc, sp.csr_matrix(B).T], [sp.csr_matrix(B), None]]).tocsc()
    sol = spla.spsolve(K, np.concatenate([bbc, np.zeros(B.shape[0])]))
    x_ref, lam_ref = sol[:N], sol[N:]
    solver.up_.assign(torch.tensor(up_prev))
    problem.time.assign(t0)
    st = solver.step(dt)
    assert st.status == 0
    x = solver.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    assert np.abs(B[Z.shape[0]:] @ x).max() <= 1e-10 * np.abs(load).sum() * np.abs(x[Nu:]).max()
    parts = solver.up.split()
    assert len(parts) == 1 + 2 + 1 + 2
    r, q0, q1 = (v.cpu().numpy() for v in parts[3:])
    assert np.allclose(r, lam_ref[:3], rtol=1e-6, atol=1e-8 * np.abs(lam_ref).max())
    assert np.allclose(np.concatenate([q0, q1]), lam_ref[3:], rtol=1e-6, atol=1e-8 * np.abs(lam_ref).max())
    # the reference's loop: t = 0.1, 0.2
    problem.time.assign(0.0)
    solver.up_.vector().zero_()
    ts = [t for _, t in solver.solve()]
    assert len(ts) == 2 and abs(ts[-1] - 0.2) < 1e-12
