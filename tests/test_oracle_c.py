"""The oracle's C restatement of MINRES + SA V-cycles (oracle/cminres.c, the
multithreaded CPU baseline) against the Python oracle (oracle/krylov.py) on the
same hierarchies: same iteration count within one, solutions within 1e-8 of
each other and of the SuperLU step."""
import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data


@pytest.mark.parametrize("modes", [False, True])
def test_c_minres_matches_python(modes):
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = os.path.join(root, "oracle", "_build", "liboracle.so")
    if not os.path.exists(so):
        sys.path.insert(0, root)
        import __graft_entry__
        __graft_entry__.build_oracle()
    from oracle import cbaseline, krylov
    problem, dt = make_problem(5, 4)
    om = make_oracle(problem, 1.0)
    data = oracle_data(4)
    x_ref, Abc, bbc, _, _ = om.step(np.zeros(om.dm.N), 0.0, dt, data, return_system=True)
    md = om.network_modes(dt, "modes" if modes else "networks")
    blocks = om.preconditioner_blocks(dt, u_weight=om.mu + om.lmbda, modes=md)
    P0 = krylov.p1_in_p2_embedding(om.dm, om.dirichlet_dofs()[0][0])
    hu = krylov.SAHierarchy(blocks[0], theta=0.1, cheb_degree=4, P0=P0)
    hp = [krylov.SAHierarchy(B, theta=0.1, cheb_degree=4) for B in blocks[1:]]
    Q = md[0] if modes else None
    M = krylov.block_preconditioner(hu, hp, 3, om.dm.Nu, om.dm.nv, Q=Q)
    # symmetric elimination of the Dirichlet rows as the solver does
    dofs, vals = om.dirichlet_values(dt, data)
    x0 = np.zeros(om.dm.N)
    for d_, v_ in zip(dofs, vals):
        x0[d_] = v_
    r0 = bbc - Abc @ x0
    d_py, it_py, _ = krylov.minres(Abc, r0, M, rtol=1e-10, maxiter=3000)
    d_c, it_c, rel = cbaseline.minres(Abc, r0, hu, hp, 3, om.dm.Nu, om.dm.nv, Q=Q, rtol=1e-10, maxiter=3000)
    assert abs(it_c - it_py) <= 1 and rel <= 1e-10
    assert np.linalg.norm(d_c - d_py) <= 1e-8 * np.linalg.norm(d_py)
    x = x0 + d_c
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def _csystem(problem, dt, theta, K=None):
    from oracle.cbaseline import CSystem
    p = problem.params
    J = int(p["J"])
    mu, lmbda = problem.lame()
    m = problem.mesh
    return CSystem(m.coordinates(), m.cells(), J, mu, lmbda, p["alpha"], p["c"], p["K"] if K is None else K, p["S"],
                   theta, dt, m.boundary_facets())


def _ensure_built():
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if not os.path.exists(os.path.join(root, "oracle", "_build", "liboracle.so")):
        sys.path.insert(0, root)
        import __graft_entry__
        __graft_entry__.build_oracle()


@pytest.mark.parametrize("n,J,theta,percell", [(3, 2, 1.0, False), (3, 4, 0.5, False), (4, 2, 1.0, True)])
def test_c_assembly_matches_oracle(n, J, theta, percell):
    """oracle/cassemble.c against OracleMPET (numpy): the Dirichlet-row system
    (pattern bit-exact, values to 1e-13 of the largest), the previous-state
    operator (B up_ = rhs_L), the preconditioner blocks and the Dirichlet DOFs."""
    _ensure_built()
    problem, dt = make_problem(n, J)
    nc = problem.mesh.num_cells()
    K = None
    if percell:
        rng = np.random.default_rng(5)
        K = [np.asarray(problem.params["K"][a]) * 10.0 ** rng.normal(0, 0.5, nc) for a in range(J)]
        problem.params["K"] = tuple(K)
    om = make_oracle(problem, theta)
    cs = _csystem(problem, dt, theta, K)
    bcs = om.dirichlet_dofs()
    dofs = np.concatenate([b[1] for b in bcs])
    assert np.array_equal(np.sort(dofs), np.sort(cs.bc_dofs))
    Abc = om.apply_bc_matrix(om.assemble_matrix(dt), [b[1] for b in bcs])
    assert np.array_equal(cs.rp, Abc.indptr.astype(np.int64))
    assert np.array_equal(cs.ci, Abc.indices.astype(np.int32))
    scale = np.abs(Abc.data).max()
    assert np.abs(cs.A - Abc.data).max() <= 1e-13 * scale
    up = np.random.default_rng(1).standard_normal(om.dm.N)
    b_ref = om.rhs_L(up, dt)
    assert np.abs(cs.rhs_prev(up) - b_ref).max() <= 1e-12 * np.abs(b_ref).max()
    md = om.network_modes(dt)
    blocks = om.preconditioner_blocks(dt, u_weight=om.mu + om.lmbda, modes=md)
    for M_c, M_py in zip([cs.Lu] + cs.Pk, blocks):
        M_py = M_py.tocsr()
        M_py.sort_indices()
        assert np.array_equal(M_c.indptr, M_py.indptr) and np.array_equal(M_c.indices, M_py.indices)
        assert np.abs(M_c.data - M_py.data).max() <= 1e-13 * np.abs(M_py.data).max()


@pytest.mark.parametrize("J", [2, 4])
def test_c_system_step_matches_superlu(J):
    """A solve_direct step of the C driver (C assembly, C MINRES with SA
    V-cycles aggregated in C) within 1e-8 of the oracle's SuperLU step."""
    _ensure_built()
    from oracle import cbaseline, krylov
    problem, dt = make_problem(4, J)
    om = make_oracle(problem, 1.0)
    data = oracle_data(J)
    x_ref = om.step(np.zeros(om.dm.N), 0.0, dt, data)
    cs = _csystem(problem, dt, 1.0)
    cs.build_hierarchies()
    # the C aggregation gives the Python aggregation's aggregates
    S = krylov.strength(cs.Pk[0], 0.1)
    a_c, n_c = cbaseline.aggregate(S)
    a_py, n_py = krylov.aggregate(S)
    assert n_c == n_py and np.array_equal(a_c, a_py)
    dofs, vals = om.dirichlet_values(dt, data)
    v = np.zeros(om.dm.N)
    for d_, v_ in zip(dofs, vals):
        v[d_] = v_
    x, it = cs.step(np.zeros(cs.N), v[cs.bc_dofs])
    assert it > 0
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
