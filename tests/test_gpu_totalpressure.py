"""MPETTotalPressureSolver on the GPU path against the total-pressure oracle
(oracle/totalpressure.py) and the reference's own rate thresholds:

* sparsity pattern bit-exact (triangles and tetrahedra), matrix within 1e-12
  and one step within 1e-8 of the SuperLU solution (theta = 0.5 and 1, FP64
  and mixed precision, traction on x = 1);
* src/mpet/test/test_convergence_totalpressuresolver.py:153-229 on the GPU
  solutions (UnitSquareMesh 8, 16, 32; theta = 0.5 with 4, 8, 16 steps and
  theta = 1 with 8, 32, 128 steps; L2 rates of the network pressures above
  1.85 and 1.87);
* pure traction with rigid-motion modes: the GPU step is the oracle's bordered
  solve.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import mms

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TP_PARAMS = dict(J=2, c=(1.0, 1.0), alpha=(1.0, 1.0), K=(1.0, 1.0), S=((1.0, 1.0), (1.0, 1.0)), E=1.0, nu=0.35)
CUBE_PARAMS = dict(J=2, c=(1e-4, 2e-4), alpha=(0.5, 0.4), K=(1e-3, 1e-2), S=((0.0, 0.1), (0.1, 0.0)),
                   E=2.7e3, nu=0.4)


def _wrap(fn, dim):
    from waterscapes_gb300 import Expression
    return Expression(lambda x, t: torch.as_tensor(np.asarray(fn(x[:, :dim].detach().cpu().numpy(), t),
                                                              dtype=np.float64), device=x.device))


def _wrap_traction(fn, dim):
    from waterscapes_gb300 import Expression
    return Expression(lambda x, t, n: torch.as_tensor(np.asarray(
        fn(x[:, :dim].detach().cpu().numpy(), t, n[:, :dim].detach().cpu().numpy()), dtype=np.float64),
        device=x.device))


def _problem(mesh, params, data, traction=True):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem
    dim = mesh.geometry().dim()
    J = params["J"]
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    if traction:
        CompiledSubDomain(lambda x: np.abs(x[:, 0] - 1.0) < 1e-12).mark(problem.momentum_boundary_markers, 1)
    for a in range(J):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.u_bar = _wrap(data["u_bar"], dim)
    problem.p_bar = [_wrap(data["p_bar"][a], dim) for a in range(J)]
    problem.f = _wrap(data["f"], dim)
    problem.g = [_wrap(data["g"][a], dim) for a in range(J)]
    problem.s = _wrap_traction(data["s"], dim)
    return problem


def _oracle(problem, theta):
    from oracle.totalpressure import OracleTotalPressure
    m = problem.mesh
    J = int(problem.params["J"])
    return OracleTotalPressure(m.coordinates(), m.cells(), m.boundary_facets(), m.boundary_facet_cells(),
                               problem.params, theta, problem.momentum_boundary_markers.array(),
                               [problem.continuity_boundary_markers[a].array() for a in range(J)])


def _solver(problem, dt, T, theta, precision="fp64", rtol=1e-11):
    from waterscapes_gb300 import MPETTotalPressureSolver
    return MPETTotalPressureSolver(problem, dict(dt=dt, T=T, theta=theta, precision=precision, rtol=rtol))


def _mesh(dim, n):
    from waterscapes_gb300 import UnitCubeMesh, UnitSquareMesh
    return UnitSquareMesh(n) if dim == 2 else UnitCubeMesh(n)


@pytest.mark.parametrize("dim,n", [(2, 3), (3, 2)])
def test_pattern_bit_exact(dim, n):
    data, _ = mms.exact_solutions(TP_PARAMS, dim)
    problem = _problem(_mesh(dim, n), TP_PARAMS, data)
    s = _solver(problem, 0.1, 1.0, 0.5)
    om = _oracle(problem, 0.5)
    A = om.assemble_matrix(0.1)
    rp, ci = s.pattern()
    assert s.N == om.dm.N and s.nnz == A.nnz
    assert np.array_equal(rp, A.indptr.astype(np.int64))
    assert np.array_equal(ci, A.indices.astype(np.int32))


@pytest.mark.parametrize("dim,params,theta,precision", [
    (2, TP_PARAMS, 0.5, "fp64"), (2, TP_PARAMS, 1.0, "mixed"),
    (3, CUBE_PARAMS, 0.5, "fp64"), (3, CUBE_PARAMS, 1.0, "mixed")])
def test_matrix_and_step(dim, params, theta, precision):
    data, _ = mms.exact_solutions(params, dim)
    problem = _problem(_mesh(dim, 6 if dim == 2 else 4), params, data)
    dt = 0.05
    s = _solver(problem, dt, 10 * dt, theta, precision)
    om = _oracle(problem, theta)
    t0 = 0.1
    problem.time.assign(t0)
    s._assemble(dt)
    A = om.assemble_matrix(dt, t0, data)
    dofs, _ = om.dirichlet_values(t0 + dt, data)
    Abc = om.apply_bc_matrix(A, dofs)
    v = s.matrix_values()
    assert np.allclose(v, Abc.data, rtol=1e-12, atol=1e-13 * np.abs(Abc.data).max())
    rng = np.random.default_rng(7)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    x_ref = om.step(up_prev, t0, dt, data)
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(t0)
    s.step(dt)
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    u, p0, p1, p2 = s.up.split()
    assert p0.shape[0] == om.dm.nv and p2.shape[0] == om.dm.nv


def _rates_gpu(theta, ms, precision):
    data, exact = mms.exact_solutions(TP_PARAMS, 2)
    ex = dict(exact, p=[exact["p0"]] + list(exact["p"]),
              dp=[lambda xx, tt: np.zeros((xx.shape[0], 2))] + list(exact["dp"]))
    errs = {k: [] for k in ("uL2", "uH1", "p1L2", "p2L2", "p1H1", "p2H1")}
    hs = []
    for n, M in zip((8, 16, 32), ms):
        problem = _problem(_mesh(2, n), TP_PARAMS, data)
        s = _solver(problem, 1.0 / M, 1.0, theta, precision=precision, rtol=1e-10)
        for up, t in s.solve():
            pass
        e = mms.errornorms(_oracle(problem, theta), up.vector().cpu().numpy(), t, ex)
        errs["uL2"].append(e["uL2"])
        errs["uH1"].append(e["uH1"])
        for a in (1, 2):
            errs["p%dL2" % a].append(e["pL2"][a])
            errs["p%dH1" % a].append(e["pH1"][a])
        hs.append(problem.mesh.hmin())
    return {k: mms.rates(v, hs) for k, v in errs.items()}


@pytest.mark.parametrize("theta,ms,precision", [(0.5, (4, 8, 16), "fp64"), (1.0, (8, 32, 128), "fp64"),
                                                (0.5, (4, 8, 16), "mixed")])
def test_reference_rate_thresholds_on_gpu(theta, ms, precision):
    """test_convergence_totalpressuresolver.py:223-228 with the GPU solutions."""
    r = _rates_gpu(theta, ms, precision)
    assert r["uL2"][-1] > 1.70
    assert r["uH1"][-1] > 1.70
    assert r["p1L2"][-1] > 1.85
    assert r["p2L2"][-1] > 1.87
    assert r["p1H1"][-1] > 0.95
    assert r["p2H1"][-1] > 0.95


def test_rigid_modes_bordered_against_oracle():
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem
    from waterscapes_gb300.mesh import AnnulusMesh
    from waterscapes_gb300.nullspace import rigid_motions
    mesh = AnnulusMesh(1.0, 2.0, 4, 24)
    params = dict(TP_PARAMS, S=((0.0, 0.5), (0.5, 0.0)))
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 1)
    for a in range(2):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.u_has_nullspace = True
    data = {"f": lambda x, t: np.stack([np.sin(x[:, 0] + t), np.cos(x[:, 1])], 1),
            "g": [lambda x, t: x[:, 0] * (1 + t), lambda x, t: np.cos(x[:, 1])],
            "p_bar": [lambda x, t: 0.1 * x[:, 0] + t, lambda x, t: -0.2 * x[:, 1]]}
    problem.f = _wrap(data["f"], 2)
    problem.g = [_wrap(g, 2) for g in data["g"]]
    problem.p_bar = [_wrap(p, 2) for p in data["p_bar"]]
    dt, t0 = 0.05, 0.1
    s = _solver(problem, dt, 10 * dt, 0.5, "fp64", rtol=1e-12)
    om = _oracle(problem, 0.5)
    rng = np.random.default_rng(5)
    up_prev = rng.standard_normal(om.dm.N) * 1e-2
    _, Abc, bbc, _, _ = om.step(up_prev, t0, dt, data, return_system=True)
    Z = rigid_motions(mesh, om.dm.node_x).reshape(-1, om.dm.Nu)
    cn = om.dm.cell_nodes
    cd = (2 * cn[:, :, None] + np.arange(2)[None, None, :]).reshape(cn.shape[0], -1)
    loc = np.einsum("cij,kl->cikjl", om.M2, np.eye(2)).reshape(cn.shape[0], cd.shape[1], cd.shape[1])
    Mu = sp.csr_matrix((loc.ravel(), (np.repeat(cd, cd.shape[1], 1).ravel(), np.tile(cd, (1, cd.shape[1])).ravel())),
                       shape=(om.dm.Nu, om.dm.Nu))
    B = np.zeros((Z.shape[0], om.dm.N))
    B[:, :om.dm.Nu] = (Mu @ Z.T).T
    K = sp.bmat([[Abc, sp.csr_matrix(B).T], [sp.csr_matrix(B), None]]).tocsc()
    x_ref = spla.spsolve(K, np.concatenate([bbc, np.zeros(Z.shape[0])]))[:om.dm.N]
    s.up_.assign(torch.tensor(up_prev))
    problem.time.assign(t0)
    s.step(dt)
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
