"""CPU oracle checks, pinned to the reference's own tests.

* convergence rates of src/mpet/test/test_convergence_mpetsolver.py:234-239
  (2D, theta = 1 with M = 8, 32, 128 and theta = 0.5 with M = 4, 8, 16);
* sparsity counts of the Kuhn cube (DOLFIN rule) at the workload sizes;
* symmetric Dirichlet elimination (bc_symmetric.py) gives the same solution
  as row replacement;
* preconditioned MINRES + SA-AMG (pressure blocks per network or per network
  eigenmode) reaches the SuperLU solution.
"""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spla

import mms
from helpers import make_oracle, make_problem, oracle_data
from oracle import fem, krylov
from oracle.mpet import OracleMPET
from waterscapes_gb300.mesh import CompiledSubDomain, MeshFunction, UnitCubeMesh, UnitSquareMesh

REF_PARAMS = dict(J=2, c=(0.3, 0.4), alpha=(0.4, 0.6), K=(0.2, 0.3), S=((0.0, 2.0), (1.0, 0.0)), E=520.0, nu=0.47)


def _rates_2d(theta, ns, ms):
    data, exact = mms.exact_solutions(REF_PARAMS, 2)
    errs = {k: [] for k in ("uL2", "uH1", "p0L2", "p1L2", "p0H1", "p1H1")}
    hs = []
    for n, M in zip(ns, ms):
        mesh = UnitSquareMesh(n)
        mm = MeshFunction(mesh)
        CompiledSubDomain.on_boundary().mark(mm, 0)
        CompiledSubDomain(lambda x: np.abs(x[:, 0] - 1.0) < 1e-12).mark(mm, 1)
        cm = [MeshFunction(mesh) for _ in range(2)]
        for m in cm:
            CompiledSubDomain.on_boundary().mark(m, 0)
        om = OracleMPET(mesh.coordinates(), mesh.cells(), mesh.boundary_facets(), mesh.boundary_facet_cells(),
                        REF_PARAMS, theta, mm.array(), [m.array() for m in cm])
        for up, t in om.solve_direct(np.zeros(om.dm.N), 0.0, 1.0, 1.0 / M, data):
            pass
        e = mms.errornorms(om, up, t, exact)
        errs["uL2"].append(e["uL2"])
        errs["uH1"].append(e["uH1"])
        for a in range(2):
            errs["p%dL2" % a].append(e["pL2"][a])
            errs["p%dH1" % a].append(e["pH1"][a])
        hs.append(mesh.hmin())
    return {k: mms.rates(v, hs) for k, v in errs.items()}


@pytest.mark.parametrize("theta,ms", [(1.0, (8, 32, 128)), (0.5, (4, 8, 16))])
def test_convergence_rates_match_reference_thresholds(theta, ms):
    r = _rates_2d(theta, (8, 16, 32), ms)
    # thresholds of test_convergence_mpetsolver.py:234-239
    assert r["uH1"][-1] > 1.70
    assert r["uL2"][-1] > 1.70
    assert r["p0L2"][-1] > 1.70
    assert r["p1L2"][-1] > 1.70
    assert r["p0H1"][-1] > 0.95
    assert r["p1H1"][-1] > 0.95


@pytest.mark.parametrize("A,n", [(2, 2), (4, 2), (2, 3), (4, 3), (1, 2)])
def test_sparsity_counts_kuhn_cube(A, n):
    m = UnitCubeMesh(n)
    dm = fem.DofMap(m.coordinates(), m.cells(), A)
    import scipy.sparse as sp
    r, c = fem.pattern_coo(dm.cell_dofs())
    P = sp.coo_matrix((np.ones(r.size), (r, c)), shape=(dm.N, dm.N)).tocsr()
    poly = {2: 2910 * n**3 + 2010 * n**2 + 432 * n + 25, 4: 3870 * n**3 + 2946 * n**2 + 720 * n + 49}
    if A in poly:
        assert P.nnz == poly[A]
    # every row holds its diagonal
    assert np.all(P.diagonal() > 0)


def test_dof_counts_of_workloads():
    for n, A, N in [(16, 2, 117637), (64, 4, 7538567), (32, 2, 895749)]:
        nodes = (2 * n + 1) ** 3
        nv = (n + 1) ** 3
        assert 3 * nodes + A * nv == N


def test_symmetric_elimination_matches_row_replacement():
    problem, dt = make_problem(3, 2)
    om = make_oracle(problem)
    data = oracle_data(2)
    x, Abc, bbc, A, b = om.step(np.zeros(om.dm.N), 0.0, dt, data, return_system=True)
    dofs, vals = om.dirichlet_values(dt, data)
    xbc = np.zeros(om.dm.N)
    for d, v in zip(dofs, vals):
        xbc[d] = v
    As, bs = om.zero_rows_columns(A, dofs, b, xbc)
    assert abs(As - As.T).max() < 1e-12 * abs(As).max()
    xs = spla.splu(As.tocsc()).solve(bs)
    assert np.linalg.norm(xs - x) <= 1e-10 * np.linalg.norm(x)


@pytest.mark.parametrize("modes", ["networks", "modes", "auto"])
def test_minres_amg_reaches_lu_solution(modes):
    problem, dt = make_problem(4, 4)
    om = make_oracle(problem)
    data = oracle_data(4)
    x, Abc, bbc, A, b = om.step(np.zeros(om.dm.N), 0.0, dt, data, return_system=True)
    dofs, vals = om.dirichlet_values(dt, data)
    x0 = np.zeros(om.dm.N)
    for d, v in zip(dofs, vals):
        x0[d] = v
    r0 = bbc - Abc @ x0
    md = om.network_modes(dt, form=modes)
    blocks = om.preconditioner_blocks(dt, u_weight=om.mu + om.lmbda, modes=md)
    P0 = krylov.p1_in_p2_embedding(om.dm, om.dirichlet_dofs()[0][0])
    hu = krylov.SAHierarchy(blocks[0], theta=0.1, cheb_degree=4, P0=P0)
    hp = [krylov.SAHierarchy(B, theta=0.1, cheb_degree=4) for B in blocks[1:]]
    M = krylov.block_preconditioner(hu, hp, 3, om.dm.Nu, om.dm.nv, Q=md[0])
    d, it, hist = krylov.minres(Abc, r0, M, rtol=1e-11, maxiter=3000)
    assert hist[-1] <= 1e-11
    assert np.linalg.norm(x0 + d - x) <= 1e-8 * np.linalg.norm(x)
