"""Smoothed-aggregation set-up on the GPU against the host set-up.

Both follow one recipe (amg_setup.cpp, amg_device.cu): the same strength
graph, the same greedy aggregates, the same smoothed prolongators and
Galerkin products, summed in the same order and rounded the same way; only
the spectral-radius estimates (Lanczos with reductions in another order) may
differ in their last bits.  So every level must have the same size and the
same pattern (the aggregates are then the same), the values must agree to
1e-12 relative, and a step with the device hierarchy is the oracle's step.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _levels(s, block):
    from waterscapes_gb300 import _lib
    levels = ctypes.c_int32()
    s.ctx.call("mpet_get_amg_info", block, ctypes.byref(levels), None, None)
    out = []
    for k in range(levels.value):
        mats = []
        for which in (0, 1):
            if which == 1 and k + 1 == levels.value:
                break
            n, m, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
            s.ctx.call("mpet_get_amg_matrix", block, k, which, ctypes.byref(n), ctypes.byref(m), ctypes.byref(nnz),
                       None, None, None)
            rp = np.empty(n.value + 1, np.int64)
            ci = np.empty(max(nnz.value, 1), np.int32)
            v = np.empty(max(nnz.value, 1))
            s.ctx.call("mpet_get_amg_matrix", block, k, which, None, None, None, _lib._ptr(rp), _lib._ptr(ci),
                       _lib._ptr(v))
            mats.append((n.value, m.value, rp, ci[:nnz.value], v[:nnz.value]))
        out.append(mats)
    return out


def _square(n):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem, UnitSquareMesh
    params = dict(J=2, c=(0.3, 0.4), alpha=(0.4, 0.6), K=(0.2, 0.3), S=((0.0, 1.5), (1.5, 0.0)), E=520.0, nu=0.47)
    problem = MPETProblem(UnitSquareMesh(n), Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(2):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    return problem, 0.1


def _hierarchies(problem, dt, precision, where):
    from waterscapes_gb300 import MPETSolver
    # a small coarsest size, so that these small meshes get several aggregation levels
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision=precision, rtol=1e-11, amg_coarse_size=40,
                                 prec_u_order="natural"))
    s.ctx.call("mpet_set_amg_setup", where)
    s.ctx.call("mpet_assemble", dt, 1)
    s.ctx.call("mpet_setup_preconditioner", dt)
    J = int(problem.params["J"])
    return s, [_levels(s, b) for b in range(J + 1)]


@pytest.mark.parametrize("case,precision", [("cube", "fp64"), ("cube", "mixed"), ("square", "fp64")])
def test_device_hierarchies_match_host(case, precision):
    problem, dt = make_problem(6, 2) if case == "cube" else _square(12)
    _, host = _hierarchies(problem, dt, precision, 0)
    s, dev = _hierarchies(problem, dt, precision, 1)
    for b, (hh, dd) in enumerate(zip(host, dev)):
        assert len(hh) == len(dd), "block %d: %d host levels, %d device levels" % (b, len(hh), len(dd))
        assert len(dd) >= 2
        for k, (hl, dl) in enumerate(zip(hh, dd)):
            assert len(hl) == len(dl)
            for (n0, m0, rp0, ci0, v0), (n1, m1, rp1, ci1, v1) in zip(hl, dl):
                assert (n0, m0) == (n1, m1), (b, k)
                assert np.array_equal(rp0, rp1), (b, k)
                assert np.array_equal(ci0, ci1), (b, k)
                scale = np.abs(v0).max() if v0.size else 1.0
                assert np.abs(v0 - v1).max() <= 1e-12 * scale, (b, k)
    # a step with the device hierarchy
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    if case == "cube":
        om = make_oracle(problem)
        x_ref = om.step(np.zeros(om.dm.N), 0.0, dt, oracle_data(2))
        x = s.up.vector().cpu().numpy()
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_device_setup_rebuilds_after_permeability_change():
    """A second set-up after a K change (the adjoint's finite-difference path)
    rebuilds the pressure hierarchies on the device, frees the previous ones,
    and still matches the host set-up of the new blocks."""
    from waterscapes_gb300 import MPETSolver
    problem, dt = make_problem(5, 2)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="fp64", rtol=1e-11, amg_coarse_size=40,
                                 prec_u_order="natural"))
    s.ctx.call("mpet_assemble", dt, 1)
    s.ctx.call("mpet_setup_preconditioner", dt)
    free0 = torch.cuda.mem_get_info()[0]
    nc = problem.mesh.num_cells()
    rng = np.random.default_rng(3)
    for rep in range(3):
        K = torch.tensor(np.stack([10.0 ** rng.uniform(-2, 0, nc) for _ in range(2)]), dtype=torch.float64,
                         device=s.device)
        s.set_cell_permeability(K)
        s.ctx.call("mpet_assemble", dt, 1)
        s.ctx.call("mpet_setup_preconditioner", dt)
    torch.cuda.synchronize()
    # three rebuilds leave the device memory where one left it (within 64 MiB of allocator slack)
    assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)
    dev = [_levels(s, b) for b in range(3)]
    s.ctx.call("mpet_set_amg_setup", 0)
    s.ctx.call("mpet_setup_preconditioner", dt)
    host = [_levels(s, b) for b in range(3)]
    for hh, dd in zip(host, dev):
        assert len(hh) == len(dd)
        for hl, dl in zip(hh, dd):
            for (n0, m0, rp0, ci0, v0), (n1, m1, rp1, ci1, v1) in zip(hl, dl):
                assert np.array_equal(rp0, rp1) and np.array_equal(ci0, ci1)
                assert np.abs(v0 - v1).max() <= 1e-12 * max(np.abs(v0).max(), 1e-300)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_spatial_first_level_is_the_same_preconditioner(precision):
    """The first displacement level in a spatial (Morton) order is the same
    operator with its rows and columns permuted (and the embedding's rows with
    them): one preconditioner application equals the node-order one up to the
    rounding of sums taken in another order, and a step matches the oracle."""
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = make_problem(6, 2)
    zs = []
    for order in ("natural", "spatial"):
        s = MPETSolver(problem, dict(dt=dt, T=dt, precision=precision, rtol=1e-11, amg_coarse_size=40,
                                     prec_u_order=order))
        s.ctx.call("mpet_assemble", dt, 1)
        s.ctx.call("mpet_setup_preconditioner", dt)
        dtype = torch.float32 if precision == "mixed" else torch.float64
        r = torch.tensor(np.random.default_rng(6).standard_normal(s.N), dtype=dtype, device=s.device)
        z = torch.empty_like(r)
        s.ctx.call("mpet_apply_preconditioner", 1 if precision == "mixed" else 0, _lib._ptr(r), _lib._ptr(z))
        torch.cuda.synchronize()
        zs.append(z.double().cpu().numpy())
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.linalg.norm(zs[1] - zs[0]) <= tol * np.linalg.norm(zs[0])
    problem.time.assign(0.0)
    s._prec_dt = float(dt)
    assert s.step(dt).status == 0
    om = make_oracle(problem)
    x_ref = om.step(np.zeros(om.dm.N), 0.0, dt, oracle_data(2))
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
