"""Parity at the sizes of the benchmark configurations.

* 16^3 Kuhn cube, A = 2 (N = 117,637): the CSR pattern bit-exact against the
  numpy oracle's DOLFIN rule (nnz 12,440,857), the Dirichlet-row matrix
  within 1e-12, and 10 solve_direct steps of dt = 0.0125
  (src/mpet/mpet/mpetsolver.py:424-462) each within 1e-8 of the oracle's
  trajectory.  The oracle solves that trajectory with its FP64 C MINRES +
  SA V-cycles at rtol 1e-12 (oracle/cbaseline.CSystem), itself pinned to
  SuperLU on small cubes (tests/test_oracle_c.py): SuperLU's fill makes it
  unusable at this size (12^3 already takes 131 s and 2e8 factor entries).
* 64^3 Kuhn cube, A = 4 (N = 7,538,567): the GPU's pattern bit-exact against
  the C oracle's (nnz 1,026,610,225; blocks uu 547,739,145, u-p_a
  51,821,379, p_a-p_b 4,018,753), the assembled values within 1e-12, and the
  first solve_direct step within 1e-8 of the C oracle's.
* The jittered ellipsoidal shell with 8 radial layers (73,728 cells), A = 4,
  log-normal per-cell K: one step within 1e-8 of the C oracle's.
"""
import math

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ensure_oracle():
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if not os.path.exists(os.path.join(root, "oracle", "_build", "liboracle.so")):
        sys.path.insert(0, root)
        import __graft_entry__
        __graft_entry__.build_oracle()


def _csystem(problem, dt):
    from oracle.cbaseline import CSystem
    p = problem.params
    mu, lmbda = problem.lame()
    m = problem.mesh
    cs = CSystem(m.coordinates(), m.cells(), int(p["J"]), mu, lmbda, p["alpha"], p["c"], p["K"], p["S"], 1.0, dt,
                 m.boundary_facets())
    cs.build_hierarchies()
    return cs


def _bc_values(cs, J, t1):
    xb = cs.dm.x[cs.bc_vertices]
    return np.concatenate([np.zeros(cs.bc_u.shape[0])]
                          + [math.sin(2 * math.pi * t1) * xb[:, 0] * (a + 1) for a in range(J)])


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_config1_16cube_pattern_values_and_ten_steps(precision):
    _ensure_oracle()
    from waterscapes_gb300 import MPETSolver
    J = 2
    problem, dt = make_problem(16, J)
    s = MPETSolver(problem, dict(dt=dt, T=10 * dt, precision=precision, rtol=1e-12))
    assert s.N == 117637 and s.nnz == 12440857
    if precision == "mixed":
        om = make_oracle(problem)
        dofs, _ = om.dirichlet_values(0.0, oracle_data(J))
        Abc = om.apply_bc_matrix(om.assemble_matrix(dt), dofs)
        rp, ci = s.pattern()
        assert np.array_equal(rp, Abc.indptr.astype(np.int64))
        assert np.array_equal(ci, Abc.indices.astype(np.int32))
        s.ctx.call("mpet_assemble", dt, 1)
        v = s.matrix_values()
        assert np.abs(v - Abc.data).max() <= 1e-12 * np.abs(Abc.data).max()
        del om, Abc
    cs = _csystem(problem, dt)
    up_ref = np.zeros(cs.N)
    t = 0.0
    problem.time.assign(0.0)
    k = 0
    for up, t1 in s.solve_direct():
        up_ref, _ = cs.step(up_ref, _bc_values(cs, J, t + dt), rtol=1e-12)
        t += dt
        assert abs(t1 - t) < 1e-12
        assert _rel(up.vector().cpu().numpy(), up_ref) <= 1e-8, "step %d" % k
        k += 1
    assert k == 10


def test_config2_64cube_pattern_values_and_first_step():
    _ensure_oracle()
    from waterscapes_gb300 import MPETSolver
    J = 4
    problem, dt = make_problem(64, J)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="mixed", rtol=1e-10))
    assert s.N == 7538567 and s.nnz == 1026610225
    rp, ci = s.pattern()
    Nu, nv = s.Nu, s.nv
    # block counts from the GPU pattern: per row, the columns below Nu are displacement columns
    # per row, the number of displacement columns (every row is non-empty)
    nu_cols = np.add.reduceat((ci < Nu).view(np.uint8), rp[:-1].astype(np.intp), dtype=np.int64)
    row_len = np.diff(rp)
    uu = int(nu_cols[:Nu].sum())
    up_rows = row_len[:Nu] - nu_cols[:Nu]
    assert uu == 547739145
    assert int(up_rows.sum()) == J * 51821379
    pa_u = [int(nu_cols[Nu + a * nv:Nu + (a + 1) * nv].sum()) for a in range(J)]
    assert pa_u == [51821379] * J
    pp = int((row_len[Nu:] - nu_cols[Nu:]).sum())
    assert pp == J * J * 4018753
    del nu_cols
    cs = _csystem(problem, dt)
    assert np.array_equal(rp, cs.rp)
    assert np.array_equal(ci, cs.ci)
    del rp, ci
    s.ctx.call("mpet_assemble", dt, 1)
    v = s.matrix_values()
    assert np.abs(v - cs.A).max() <= 1e-12 * np.abs(cs.A).max()
    del v
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    x_ref, _ = cs.step(np.zeros(cs.N), _bc_values(cs, J, dt), rtol=1e-10)
    assert _rel(s.up.vector().cpu().numpy(), x_ref) <= 1e-8


def test_config3_shell_8_layers_one_step():
    _ensure_oracle()
    from waterscapes_gb300 import MPETSolver
    import bench
    J = 4
    problem, dt = bench.workload(8, J, "ellipsoid")
    assert problem.mesh.num_cells() == 73728
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="mixed", rtol=1e-11))
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    cs = _csystem(problem, dt)
    x_ref, _ = cs.step(np.zeros(cs.N), _bc_values(cs, J, dt), rtol=1e-12)
    assert _rel(s.up.vector().cpu().numpy(), x_ref) <= 1e-8
