"""The total-pressure oracle (oracle/totalpressure.py) against the reference's
own known answers: the convergence-rate thresholds of
src/mpet/test/test_convergence_totalpressuresolver.py:153-229 (UnitSquareMesh
8, 16, 32; theta = 0.5 with 4, 8, 16 steps and theta = 1 with 8, 32, 128 steps;
J = 2, c = alpha = K = 1, S = 1, E = 1, nu = 0.35; Dirichlet data except a
traction sigma n on x = 1), and the equivalence of the two formulations: the
total-pressure step reproduces the MPET oracle's displacement and network
pressures up to the discretisation of p0.
"""
import numpy as np
import pytest

import mms

TP_PARAMS = dict(J=2, c=(1.0, 1.0), alpha=(1.0, 1.0), K=(1.0, 1.0), S=((1.0, 1.0), (1.0, 1.0)), E=1.0, nu=0.35)


def _square_oracle(n, theta, params=TP_PARAMS):
    from oracle.totalpressure import OracleTotalPressure
    from waterscapes_gb300 import UnitSquareMesh
    m = UnitSquareMesh(n)
    bf = m.boundary_facets()
    xm = m.coordinates()[bf].mean(axis=1)
    mm = np.where(np.abs(xm[:, 0] - 1.0) < 1e-12, 1, 0)
    cm = [np.zeros(bf.shape[0], dtype=np.int64) for _ in range(params["J"])]
    return OracleTotalPressure(m.coordinates(), m.cells(), bf, m.boundary_facet_cells(), params, theta, mm, cm)


def _rates(theta, ms):
    data, exact = mms.exact_solutions(TP_PARAMS, 2)
    ex = dict(exact, p=[exact["p0"]] + list(exact["p"]),
              dp=[lambda xx, tt: np.zeros((xx.shape[0], 2))] + list(exact["dp"]))
    errs = {k: [] for k in ("uL2", "uH1", "p1L2", "p2L2", "p1H1", "p2H1")}
    hs = []
    for n, M in zip((8, 16, 32), ms):
        om = _square_oracle(n, theta)
        up = np.zeros(om.dm.N)
        for up, t in om.solve_direct(up, 0.0, 1.0, 1.0 / M, data):
            pass
        e = mms.errornorms(om, up, t, ex)
        errs["uL2"].append(e["uL2"])
        errs["uH1"].append(e["uH1"])
        for a in (1, 2):
            errs["p%dL2" % a].append(e["pL2"][a])
            errs["p%dH1" % a].append(e["pH1"][a])
        hs.append(np.sqrt(2.0) / n)
    return {k: mms.rates(v, hs) for k, v in errs.items()}


@pytest.mark.parametrize("theta,ms", [(0.5, (4, 8, 16)), (1.0, (8, 32, 128))])
def test_reference_rate_thresholds(theta, ms):
    """test_convergence_totalpressuresolver.py:223-228."""
    r = _rates(theta, ms)
    assert r["uL2"][-1] > 1.70
    assert r["uH1"][-1] > 1.70
    assert r["p1L2"][-1] > 1.85
    assert r["p2L2"][-1] > 1.87
    assert r["p1H1"][-1] > 0.95
    assert r["p2H1"][-1] > 0.95


def test_symmetric_and_same_sparsity_as_mpet_with_one_more_field():
    om = _square_oracle(3, 0.5)
    A = om.assemble_matrix(0.1).tocsr()
    assert abs(A - A.T).max() < 1e-13 * abs(A).max()
    from oracle.mpet import OracleMPET
    from oracle.totalpressure import expand_params
    ref = OracleMPET(om.dm.x, om.dm.cells, om.bfacets, om.bfacet_cells, expand_params(TP_PARAMS), 0.5)
    B = ref.assemble_matrix(0.1).tocsr()
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def test_engine_field_view_matches_oracle_expansion():
    """The host side of MPETTotalPressureSolver presents p0 as pressure field 0 with the
    same expanded parameters as the oracle, and reads through to the problem."""
    from oracle.totalpressure import expand_params as oracle_expand
    from waterscapes_gb300 import Constant, MPETProblem, UnitSquareMesh
    from waterscapes_gb300.totalpressure import _FieldView, expand_params
    params = dict(TP_PARAMS, S=((0.0, 0.7), (0.7, 0.0)))
    a, b = expand_params(params), oracle_expand(params)
    for key in ("J", "alpha", "c"):
        assert tuple(np.atleast_1d(a[key])) == tuple(np.atleast_1d(b[key]))
    assert np.array_equal(np.asarray(a["S"], dtype=float), np.asarray(b["S"], dtype=float))
    assert np.array_equal(np.asarray(a["K"], dtype=float), np.asarray(b["K"], dtype=float))
    problem = MPETProblem(UnitSquareMesh(2), Constant(0.0), params=params)
    view = _FieldView(problem)
    assert view.params["J"] == 3 and view.g[0] is None and len(view.continuity_boundary_markers) == 3
    assert (view.continuity_boundary_markers[0].as_int32() == -1).all()
    problem.p_bar = ["a", "b"]
    assert view.p_bar == [None, "a", "b"]
    view.u_has_nullspace = True
    assert problem.u_has_nullspace is True
