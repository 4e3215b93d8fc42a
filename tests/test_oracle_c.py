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
    so = os.path.join(root, "oracle", "_build", "libcminres.so")
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
