"""Benchmark: MPET time steps per second on one GB300 (64^3 Kuhn cube, A=4).

Workload (default): unit cube, 64^3 hexahedra x 6 tetrahedra (1,572,864
cells), P2 displacement + 4 P1 pressures (N = 7,538,567 DOFs, nnz =
1,026,610,225), mu=1e3, lambda=1e4, alpha=0.25, c=1e-4, K=(1e-4..1e-1),
S off-diagonals 1e-2, dt=0.01, u=0 and p_a = sin(2 pi t) x0 a on the
boundary, zero initial state.  Synthetic by construction (generated mesh).

A "step" is one pass of the solve_direct time loop (mpetsolver.py:424-462):
right-hand side assembly + block-AMG-preconditioned MINRES solve to a 1e-10
relative preconditioned residual, with the matrix and the AMG hierarchy built
once before the loop (the reference assembles A and factorises once there).
``value`` is the mixed-precision (FP32 inner / FP64 refinement) rate with
the state resident in HBM; the FP64 path, the relative error between the
two, the FP32/FP64 SpMV bandwidth, the step() rate with per-step matrix
assembly and an end-to-end rate through the public API with host buffers
are reported alongside.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--n 64] [--impl reference]
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MPET steps/s at 64³ A=4, mixed vs FP64 GPU at 1e-8 rel err; SpMV HBM GB/s"

# The system SpMV kernel the autotuner picked, and its DRAM bytes per launch
# as a multiple of its algorithmic bytes (ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one launch on the 24^3 A=4 case, scaled by the
# entries of a launch here; the summaries are under profiles/).
ROOFLINE_KERNEL = {"csr": "k_spmv_sell<1,8,EpiMinres> (SELL-32)", "node-block": "k_spmv_nb<4,EpiMinres> (node blocks)"}
TRAFFIC_RATIO = {"node-block": 248650752 / 245547052}
TRAFFIC_SOURCE = {"node-block": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_spmv_nb launch on the "
                                "24^3 A=4 case (248,650,752 B vs 245,547,052 algorithmic), scaled to this launch"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(n, J, shape="cube"):
    """Kuhn cube n^3 x 6 (the 16^3 A=2 and 64^3 A=4 cases), or the jittered
    ellipsoidal shell (semi-axes 1, 0.8, 0.7, inner ratio 0.3, n radial layers,
    144 n^3 cells) with log-normal per-cell K_a (log10 mean -3 + a, sigma 0.5,
    seed 0)."""
    from waterscapes_gb300 import (CompiledSubDomain, Constant, EllipsoidShellMesh, Expression, MPETProblem,
                                   UnitCubeMesh, convert_to_E_nu)
    mesh = UnitCubeMesh(n) if shape == "cube" else EllipsoidShellMesh(n, seed=0)
    if J == 4:
        S = np.full((4, 4), 1e-2)
        np.fill_diagonal(S, 0.0)
        K = (1e-4, 1e-3, 1e-2, 1e-1)
        if shape != "cube":
            rng = np.random.default_rng(0)
            K = tuple(10.0 ** rng.normal(-3.0 + a, 0.5, size=mesh.num_cells()) for a in range(4))
        mat = dict(alpha=(0.25,) * 4, c=(1e-4,) * 4, K=K, S=tuple(map(tuple, S)))
        dt = 0.01
    else:
        mat = dict(alpha=(0.5, 0.5), c=(1e-4, 1e-4), K=(1e-3, 1e-2), S=((0.0, 0.1), (0.1, 0.0)))
        dt = 0.0125
    E, nu = convert_to_E_nu(1.0e3, 1.0e4)
    time_c = Constant(0.0)
    problem = MPETProblem(mesh, time_c, params=dict(J=J, E=E, nu=nu, **mat))
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 0)
    for a in range(J):
        CompiledSubDomain.on_boundary().mark(problem.continuity_boundary_markers[a], 0)
    problem.p_bar = [Expression((lambda a: (lambda x, t: math.sin(2 * math.pi * t) * x[:, 0] * (a + 1)))(a))
                     for a in range(J)]
    return problem, dt


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def spmv_alg_bytes(solver, sv):
    """Algorithmic bytes of one system SpMV with the variant chosen for its
    precision: every stored nonzero value once, one column id per nonzero
    (CSR / SELL) or per block (node-block copy), row pointers (CSR), x and y
    once each."""
    import ctypes
    N, nnz = solver.N, solver.nnz
    ch = ctypes.c_int32()
    solver.ctx.call("mpet_get_spmv_tuning" if sv == 4 else "mpet_get_spmv_tuning_fp64", None, ctypes.byref(ch))
    if ch.value in (8, 9):
        nb = ctypes.c_int64()
        solver.ctx.call("mpet_get_node_block_info", ctypes.byref(nb), None)
        return nnz * sv + nb.value * 4 + 2 * N * sv, "node-block"
    return nnz * (sv + 4) + (N + 1) * 8 + 2 * N * sv, "csr"


def time_spmv(solver, torch, lib, reps=20):
    """FP32 and FP64 SpMV with the assembled matrix, CUDA events on the engine's stream."""
    N, nnz = solver.N, solver.nnz
    out = {}
    stream = solver._stream
    for prec, dtype, sv in ((1, torch.float32, 4), (0, torch.float64, 8)):
        if prec == 1 and solver.params["precision"] != "mixed":
            continue
        x = torch.randn(N, dtype=dtype, device=solver.device)
        y = torch.empty(N, dtype=dtype, device=solver.device)
        for _ in range(3):
            solver.ctx.call("mpet_spmv", prec, lib._ptr(x), lib._ptr(y))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            solver.ctx.call("mpet_spmv", prec, lib._ptr(x), lib._ptr(y))
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        bytes_, layout = spmv_alg_bytes(solver, sv)
        out["fp32" if prec == 1 else "fp64"] = {"ms": ms, "alg_bytes": bytes_, "gbs": bytes_ / ms / 1e6,
                                                "layout": layout}
    return out


def run_steps(solver, torch, steps, warmup, dt):
    """solve_direct steps with the state on the device; returns (ms total, iterations, states)."""
    problem = solver.problem
    problem.time.assign(0.0)
    solver.up_.vector().zero_()
    gen = solver.solve_direct()
    for _ in range(warmup):
        next(gen)
    torch.cuda.synchronize()
    stream = solver._stream
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    it0 = len(solver.solver_monitor["niter"])
    before = solve_counters(solver)
    e0.record(stream)
    for _ in range(steps):
        next(gen)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    its = solver.solver_monitor["niter"][it0:]
    return ms, its, solver.up.vector().clone(), loop_split(solver, before, steps)


def time_precond(solver, torch, lib, reps=10):
    """One block-diagonal AMG preconditioner application (CUDA events)."""
    mixed = solver.params["precision"] == "mixed"
    dtype = torch.float32 if mixed else torch.float64
    r = torch.randn(solver.N, dtype=dtype, device=solver.device)
    z = torch.empty_like(r)
    prec = 1 if mixed else 0
    for _ in range(2):
        solver.ctx.call("mpet_apply_preconditioner", prec, lib._ptr(r), lib._ptr(z))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(solver._stream)
    for _ in range(reps):
        solver.ctx.call("mpet_apply_preconditioner", prec, lib._ptr(r), lib._ptr(z))
    e1.record(solver._stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def replica_rate(ms_local, steps):
    """Whole-job steps/s of independent replicas: every rank ran ``steps`` steps in
    ``ms_local`` ms; the job time is the slowest rank (max over ranks, gloo)."""
    import torch
    world = 1
    ms = float(ms_local)
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        world = torch.distributed.get_world_size()
        t = torch.tensor([ms], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return world * steps / (ms / 1e3), ms


def prec_form(solver):
    """Displacement block the preconditioner runs (elasticity AMG or vector Laplacian,
    with a matrix-free or CSR first level and the autotuner's timings of both)."""
    import ctypes
    v = ctypes.c_int32()
    solver.ctx.call("mpet_get_prec_info", ctypes.byref(v))
    if v.value:
        return "elasticity AMG (rigid-body modes)"
    used = ctypes.c_int32()
    ms = (ctypes.c_float * 2)()
    solver.ctx.call("mpet_get_prec_matrix_free", ctypes.byref(used), ms)
    return "vector Laplacian AMG, %s first level (Chebyshev product: CSR %.4f ms, matrix-free %.4f ms)" % (
        "matrix-free" if used.value else "CSR", ms[0], ms[1])


def spmv_tuning(solver, fp64=False):
    import ctypes
    ms = np.zeros(7)
    ch = ctypes.c_int32()
    solver.ctx.call("mpet_get_spmv_tuning_fp64" if fp64 else "mpet_get_spmv_tuning",
                    ms.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ch))
    slots = ["register/4", "register/8", "staged/4", "staged/8", "sell32/4", "sell32/8", "node-block"]
    variants = {0: "register/4", 1: "register/8", 2: "staged/4", 3: "staged/8", 4: "sell32/4", 5: "sell32/8",
                6: "sell32-late/4", 7: "sell32-late/8", 8: "node-block", 9: "node-block/64 registers",
                32: "sell32-fp16"}
    return {"ms": {slots[v]: round(float(ms[v]), 4) for v in range(7) if ms[v] > 0},
            "chosen": variants.get(ch.value, str(ch.value))}


def level_variants(solver):
    """SpMV variant the set-up autotuner chose for each level's operator, per
    hierarchy (displacement, then each network): 4/5 SELL-32, 6/7 SELL late,
    0-3 CSR register/staged, 8 node blocks, 16 matrix-free, 32 SELL FP16."""
    from waterscapes_gb300 import _lib
    out = {}
    for blk in range(solver.J + 1):
        sizes, _ = solver.amg_info(blk)
        va = np.zeros(max(len(sizes), 1), np.int32)
        solver.ctx.call("mpet_get_amg_variants", blk, _lib._ptr(va), None, None)
        out["displacement" if blk == 0 else "pressure %d" % blk] = [int(v) for v in va[:len(sizes)]]
    return out


def prec_setup_ms(solver):
    """Split of the last preconditioner set-up (ms): GPU block assembly, block
    downloads (host set-up only), the hierarchies (built on the GPU, or by
    concurrent host threads), FP32 copies + SpMV layouts + uploads + autotuning."""
    import ctypes
    ms = np.zeros(4)
    solver.ctx.call("mpet_get_setup_timing", ms.ctypes.data_as(ctypes.c_void_p))
    out = {"where": solver.params.get("amg_setup", "device"), "blocks_gpu": round(ms[0], 1),
           "downloads": round(ms[1], 1), "hierarchies": round(ms[2], 1), "layouts_autotune": round(ms[3], 1)}
    if out["where"] == "device":
        ph = np.zeros(8)
        solver.ctx.call("mpet_get_amg_setup_phases", ph.ctypes.data_as(ctypes.c_void_p))
        names = ["copy", "diag_rho", "strength_aggregate", "prolongator", "transpose", "galerkin", "coarsest",
                 "layouts_autotune"]
        out["device_phases"] = {k: round(float(v), 1) for k, v in zip(names, ph)}
    return out


def launches(solver):
    import ctypes
    n = ctypes.c_int64()
    solver.ctx.call("mpet_get_timing", None, None, None, ctypes.byref(n))
    return n.value


def solve_counters(solver):
    """(ms in MINRES graph replays, their iterations, ms in whole solves) so far."""
    import ctypes
    a, b, c = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
    solver.ctx.call("mpet_get_timing", ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), None)
    return a.value, b.value, c.value


def loop_split(solver, before, steps):
    """Where the timed steps went: inner MINRES (per iteration) vs the rest of
    each solve (refinement residuals, preconditioner set-up per sweep)."""
    a0, b0, c0 = before
    a1, b1, c1 = solve_counters(solver)
    its = max(1, b1 - b0)
    return {"inner_ms_per_iteration": (a1 - a0) / its, "solve_ms_per_step": (c1 - c0) / steps,
            "outside_inner_ms_per_step": ((c1 - c0) - (a1 - a0)) / steps}


def cpu_full_run(n, J, shape, warmup, steps, budget_s=180.0):
    """The oracle's CPU path on the FULL workload: the system, previous-state
    operator and preconditioner blocks assembled by the C restatement
    (oracle/cassemble.c), SA hierarchies built by the Python oracle
    (aggregation in C), then solve_direct steps (right-hand side B up_,
    Dirichlet values, MINRES with the block V-cycles in C on every host
    thread) from a zero state at t = 0.  ``warmup`` untimed steps, then up to
    ``steps`` timed steps, stopping early once ``budget_s`` seconds of timed
    steps have run (at least one).  Returns a dict with the rate and what ran."""
    from oracle import cbaseline
    cbaseline.load()
    problem, dt = workload(n, J, shape)
    m = problem.mesh
    p = problem.params
    mu, lmbda = problem.lame()
    t0 = time.perf_counter()
    cs = cbaseline.CSystem(m.coordinates(), m.cells(), J, mu, lmbda, p["alpha"], p["c"], p["K"], p["S"], 1.0, dt,
                           m.boundary_facets())
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    cs.build_hierarchies()
    t_hier = time.perf_counter() - t0
    xb = cs.dm.x[cs.bc_vertices]
    zero_u = np.zeros(cs.bc_u.shape[0])

    def bc_values(t1):
        return np.concatenate([zero_u] + [math.sin(2 * math.pi * t1) * xb[:, 0] * (a + 1) for a in range(J)])

    up = np.zeros(cs.N)
    t = 0.0
    its = []
    for _ in range(warmup):
        up, it = cs.step(up, bc_values(t + dt))
        t += dt
    times = []
    while len(times) < max(1, steps):
        ts = time.perf_counter()
        up, it = cs.step(up, bc_values(t + dt))
        times.append(time.perf_counter() - ts)
        its.append(it)
        t += dt
        if sum(times) >= budget_s:
            break
    sec = sum(times)
    return {"value": len(times) / sec, "steps": len(times), "warmup": warmup, "seconds": sec,
            "iterations": its, "N": cs.N, "nnz": cs.nnz, "assemble_s": t_asm, "hierarchies_s": t_hier,
            "cores": host_cores()}


def host_cores():
    """Threads OpenMP will use: OMP_NUM_THREADS, else the CPU affinity set."""
    v = os.environ.get("OMP_NUM_THREADS")
    if v and v.isdigit():
        return int(v)
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def profile_case(args):
    """Set-up, assembly and one time step capped at --maxit Krylov iterations."""
    import torch
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = workload(args.n, args.networks, args.workload)
    # (--inner-loop host: the inner iterations replay a graph without conditional
    # nodes, whose kernels a profiler can list one by one)
    sol = MPETSolver(problem, dict(dt=dt, T=1e9, precision="mixed", maxit=args.maxit, rtol=1e-10,
                                   inner_loop=args.inner_loop or "device",
                                   prec_u_order=args.prec_u_order or "natural"))
    sol._assemble(dt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("step")
    try:
        sol.advance(dt)
    except _lib.MpetError as e:
        if e.code != -4:
            raise
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"profile_case": args.n, "networks": args.networks, "maxit": args.maxit, "N": sol.N,
                      "nnz": sol.nnz, "step_s": time.perf_counter() - t0}))


def estimator_run(args):
    """Error indicators (AdaptiveMPETSolver) after one solve_direct step of the
    --n cube: time per indicator evaluation (cell + interior-facet kernels, the
    gather and the R4p sum) with CUDA events, against one step's time."""
    import torch
    from waterscapes_gb300 import AdaptiveMPETSolver, Constant, Expression
    problem, dt = workload(args.n, args.networks)
    problem.f = Expression(lambda x, t: torch.stack([torch.sin(x[:, 0] + t), x[:, 1] * t, x[:, 2]], 1))
    params = AdaptiveMPETSolver.default_params()
    params["MPETSolver"].update(dt=dt, T=1e9, theta=1.0, rtol=1e-10, precision="mixed")
    f_ = Expression(problem.f.fn, t=Constant(0.0))
    t0 = time.perf_counter()
    ad = AdaptiveMPETSolver(problem, f_, params)
    t_setup = time.perf_counter() - t0
    s = ad.inner_solver
    gen = s.solve_direct()
    next(gen)
    torch.cuda.synchronize()
    stream = s._stream
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        ad.indicators()
    torch.cuda.synchronize()
    reps = 5
    e0.record(stream)
    for _ in range(reps):
        out = ad.indicators()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    e0.record(stream)
    next(gen)
    e1.record(stream)
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1)
    print(json.dumps({"estimators": "AdaptiveMPETSolver indicators", "workload": "Kuhn cube %d^3, A=%d" % (
        args.n, args.networks), "cells": problem.mesh.num_cells(), "interior_facets": ad._nfi,
        "indicators_ms": ms, "step_ms": step_ms, "facet_tables_plus_solver_setup_s": t_setup,
        "eta_u_sum": float(out[1].sum()), "r4p": out[3]}))


def adjoint_check(args):
    """Gradient of the final-pressure misfit w.r.t. per-cell K by the discrete
    adjoint: A=2 on the Kuhn n^3 cube (default 32^3), 20 steps of dt = 0.025,
    a checkpoint every 5 steps; the target is the final pressure field of a
    seeded log-normal "true" K (log10 K_a ~ N(log10 K_a0, 0.5)), the gradient is
    taken at a second seeded field.  Checked against central differences
    (h = 1e-6 along K-relative Gaussian directions) and against the FP64-path
    adjoint.  Prints one JSON line."""
    import torch
    from waterscapes_gb300 import MPETSolver
    from waterscapes_gb300.adjoint import MisfitAdjoint
    n, J, nsteps, dt, every = args.n, 2, 20, 0.025, 5
    problem, _ = workload(n, J, "cube")
    nc = problem.mesh.num_cells()
    K0 = np.asarray(problem.params["K"], dtype=np.float64)
    rng = np.random.default_rng(0)
    K_true = np.stack([K0[a] * 10.0 ** rng.normal(0.0, 0.5, nc) for a in range(J)])
    K_eval = np.stack([K0[a] * 10.0 ** rng.normal(0.0, 0.5, nc) for a in range(J)])
    dev = torch.device("cuda", 0)
    f64 = dict(dtype=torch.float64, device=dev)
    where = args.amg_setup or "device"
    solvers = {p: MPETSolver(problem, dict(dt=dt, T=1e9, theta=1.0, rtol=1e-12, precision=p, amg_setup=where))
               for p in ("mixed", "fp64")}
    # finite-difference solves start from the unperturbed state of their step
    # and reduce that O(h) residual by 1e-6 (far below h itself)
    solvers["fd"] = MPETSolver(problem, dict(dt=dt, T=1e9, theta=1.0, rtol=1e-6, precision="mixed",
                                             amg_setup=where))
    zero = torch.zeros(solvers["mixed"].N, **f64)

    def driver(p, target):
        problem.time.assign(0.0)
        return MisfitAdjoint(solvers[p], target, nsteps, checkpoint_every=every, t0=0.0, up0=zero)

    # target: final pressures of the "true" field
    d = driver("mixed", torch.zeros(J, solvers["mixed"].nv, **f64))
    d.forward(torch.as_tensor(K_true, **f64))
    s = solvers["mixed"]
    target = d.x_final[s.Nu:].reshape(J, s.nv).clone()
    out = {"metric": "discrete-adjoint gradient of the final-pressure misfit w.r.t. per-cell K",
           "config": {"workload": "Kuhn cube %d^3 x 6 tets (%d cells), A=2, %d steps of dt=%g, checkpoint every %d"
                      % (n, nc, nsteps, dt, every), "N": s.N, "rtol": 1e-12}}
    for p in ("mixed", "fp64"):
        d = driver(p, target)
        Kt = torch.as_tensor(K_eval, **f64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss = d.forward(Kt)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g = d.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out[p] = {"loss": loss, "forward_s": t1 - t0, "backward_s": t2 - t1,
                  "forward_iterations": sum(d.stats["forward_iterations"][:nsteps]),
                  "adjoint_iterations": sum(d.stats["adjoint_iterations"])}
        if p == "mixed":
            g_mixed, d_mixed = g.clone(), d
        else:
            g64 = g
    out["rel_diff_mixed_vs_fp64_gradient"] = float(torch.linalg.norm(g_mixed - g64) / torch.linalg.norm(g64))
    # central differences on the mixed path.  Every perturbed solve starts
    # from the unperturbed state of its step (solved to 1e-12), so its
    # relative tolerance applies to the O(h) difference only.
    rng = np.random.default_rng(2)
    h = 1e-6
    errs = []
    Ke = torch.as_tensor(K_eval, **f64)
    d_ref = driver("mixed", target)
    d_ref.forward(Ke, keep_states=True)
    ref_states = d_ref.states
    d_fd = driver("fd", target)
    t0 = time.perf_counter()
    for _ in range(args.fd_dirs):
        dK = torch.as_tensor(K_eval * rng.standard_normal(K_eval.shape), **f64)
        lp = d_fd.forward(Ke + h * dK, guesses=ref_states)
        lm = d_fd.forward(Ke - h * dK, guesses=ref_states)
        fd = (lp - lm) / (2.0 * h)
        ad = float(torch.sum(g_mixed * dK))
        errs.append(abs(fd - ad) / abs(ad))
    out["central_differences"] = {"directions": args.fd_dirs, "h": h, "max_rel_err": max(errs),
                                  "median_rel_err": statistics.median(errs), "seconds": time.perf_counter() - t0,
                                  "amg_setup": where, "last_setup_ms": prec_setup_ms(solvers["fd"]),
                                  "path": "mixed precision with FP64 refinement; each perturbed solve starts "
                                          "from the unperturbed state (solved to 1e-12) and reduces the residual "
                                          "of the perturbation by 1e-6"}
    print(json.dumps(out))


def batch_problems(count, n_lo, n_hi, seed=0):
    """Independent A=2 instances: Kuhn cubes n^3 x 6 with n uniform in
    [n_lo, n_hi], K_a in log-uniform[1e-5, 1e-1], c_a in log-uniform[1e-5, 1e-3],
    S12 in log-uniform[1e-3, 1] (seeded); mu = 1e3, lambda = 1e4, alpha = 0.5;
    u = 0 and p_a = sin(2 pi t) x0 (a + 1) on the boundary."""
    from waterscapes_gb300 import (CompiledSubDomain, Constant, Expression, MPETProblem, UnitCubeMesh,
                                   convert_to_E_nu)
    rng = np.random.default_rng(seed)
    E, nu = convert_to_E_nu(1.0e3, 1.0e4)
    lu = lambda lo, hi: 10.0 ** rng.uniform(np.log10(lo), np.log10(hi))  # noqa: E731
    out = []
    for _ in range(count):
        n = int(rng.integers(n_lo, n_hi + 1))
        K = (lu(1e-5, 1e-1), lu(1e-5, 1e-1))
        c = (lu(1e-5, 1e-3), lu(1e-5, 1e-3))
        s12 = lu(1e-3, 1.0)
        p = MPETProblem(UnitCubeMesh(n), Constant(0.0),
                        params=dict(J=2, E=E, nu=nu, alpha=(0.5, 0.5), c=c, K=K, S=((0.0, s12), (s12, 0.0))))
        CompiledSubDomain.on_boundary().mark(p.momentum_boundary_markers, 0)
        for a in range(2):
            CompiledSubDomain.on_boundary().mark(p.continuity_boundary_markers[a], 0)
        p.p_bar = [Expression((lambda a: (lambda x, t: math.sin(2 * math.pi * t) * x[:, 0] * (a + 1)))(a))
                   for a in range(2)]
        out.append(p)
    return out


def batch_run(args):
    """Many independent instances advanced together (one launch per kernel for
    all of them): instance-steps/s of the mixed path over --steps steps of
    dt = 0.02 after --warmup steps, each instance converged to 1e-10 on its
    own; the final states of a few instances are checked against the same
    instances solved alone on the FP64 path.  Prints one JSON line."""
    import torch
    from waterscapes_gb300 import MPETBatchSolver, MPETSolver
    dt = 0.02
    t0 = time.perf_counter()
    problems = batch_problems(args.instances, args.n_min, args.n_max)
    t_mesh = time.perf_counter() - t0
    nsteps = args.warmup + args.steps
    params = dict(dt=dt, T=nsteps * dt, theta=1.0, rtol=1e-10, precision="mixed")
    t0 = time.perf_counter()
    bs = MPETBatchSolver(problems, params)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    bs._assemble(dt)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    gen = bs.solve_direct()
    for _ in range(args.warmup):
        next(gen)
    torch.cuda.synchronize()
    worst = 0.0
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    its0 = len(bs.solver_monitor["niter"])
    e0.record(bs._stream)
    for _ in range(args.steps):
        next(gen)
        worst = max(worst, float(bs.batch_relres().max()))
    e1.record(bs._stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    its = bs.solver_monitor["niter"][its0:]
    # a few instances solved alone on the FP64 path
    check = sorted(set(np.linspace(0, bs.ninst - 1, min(4, bs.ninst)).astype(int).tolist()))
    errs = []
    finals = {i: bs.instance_vector(i).clone() for i in check}
    del gen
    for i in check:
        p = problems[i]
        p.time.assign(0.0)
        s = MPETSolver(p, dict(params, precision="fp64"))
        for up, t in s.solve_direct():
            pass
        ref = up.vector()
        errs.append(float(torch.linalg.norm(finals[i] - ref) / torch.linalg.norm(ref)))
        s.ctx.close()
        del s, up
    sizes = [p.mesh.num_cells() // 6 for p in problems]
    ninst, bN, bnnz, tuning = bs.ninst, bs.N, bs.nnz, spmv_tuning(bs)
    bs.ctx.close()  # the device memory goes now, not when the collector breaks the solver's cycles
    del bs
    gc.collect()
    seq = None
    if args.sequential_steps > 0:
        # the same instances solved one after another (each its own solver, matrix and AMG
        # built before its timed steps), mixed path: one untimed step, then the timed ones
        t_solve = 0.0
        its_seq = []
        try:
            for p in problems:
                p.time.assign(0.0)
                s = MPETSolver(p, dict(params, T=1e9))
                g = s.solve_direct()
                next(g)
                torch.cuda.synchronize()
                e0.record(s._stream)
                for _ in range(args.sequential_steps):
                    next(g)
                e1.record(s._stream)
                torch.cuda.synchronize()
                t_solve += e0.elapsed_time(e1) / 1e3
                its_seq.append(s.solver_monitor["niter"][-1])
                del g
                s.ctx.close()
                del s
            seq = {"value": len(problems) * args.sequential_steps / t_solve, "unit": "instance-steps/s",
                   "steps_per_instance": args.sequential_steps, "after_untimed_steps": 1,
                   "iterations_last_step": {"min": int(min(its_seq)), "median": float(np.median(its_seq)),
                                            "max": int(max(its_seq))}}
        except Exception as e:  # the batched figure stands on its own
            seq = {"error": str(e), "instances_done": len(its_seq)}
    out = {"metric": "batched MPET instance-steps/s (A=2 instances in one union mesh)",
           "value": ninst * args.steps / (ms / 1e3), "unit": "instance-steps/s",
           "ms_per_step": ms / args.steps, "steps": args.steps, "warmup": args.warmup,
           "config": {"workload": "%d Kuhn cubes n^3 x 6 tets, n in [%d, %d] (seeded), A=2, dt=0.02"
                      % (ninst, args.n_min, args.n_max), "N": bN, "nnz": bnnz,
                      "cells": int(sum(p.mesh.num_cells() for p in problems)),
                      "n_mean": float(np.mean(sizes) ** (1 / 3.0))},
           "iterations_per_step": its, "worst_instance_relres": worst,
           "fp64_single_instance_check": {"instances": check, "rel_err": errs},
           "setup_s": {"meshes": t_mesh, "union_and_pattern": t_setup, "assemble_plus_amg": t_asm},
           "sequential": seq,
           "spmv_tuning": tuning}
    print(json.dumps(out))


def vcycle_profile(args):
    """Per-level cost of the block preconditioner on the --n cube (mixed
    precision): for every hierarchy (displacement, each pressure block) the
    rows and nonzeros of each level, its own time (V-cycle from level k minus
    V-cycle from level k+1, medians over L2-flushed launches), its algorithmic
    bytes and their rate against the measured HBM peak; plus one whole
    preconditioner application (the pressure V-cycles run concurrently with the
    displacement V-cycle).  Prints one JSON line."""
    import ctypes
    import torch
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = workload(args.n, args.networks, args.workload)
    base = dict(dt=dt, T=1e9, theta=1.0, rtol=1e-10, precision="mixed", amg_setup=args.amg_setup or "device",
                prec_u_order=args.prec_u_order or "natural")
    if args.cheb_degree is not None:
        base["amg_cheb_degree"] = args.cheb_degree
    if args.cheb_degree_coarse is not None:
        base["amg_cheb_degree_coarse"] = args.cheb_degree_coarse
    if args.cheb_coarse_level is not None:
        base["amg_cheb_coarse_level"] = args.cheb_coarse_level
    sol = MPETSolver(problem, base)
    sol._assemble(dt)
    torch.cuda.synchronize()
    hbm, kind = peaks()
    out = {"vcycle_profile": "Kuhn cube %d^3, A=%d" % (args.n, args.networks), "peak_gbs": hbm, "peak_kind": kind,
           "setup_ms": prec_setup_ms(sol), "blocks": []}
    for blk in range(args.networks + 1):
        sizes, nnz = sol.amg_info(blk)
        va, vp, vr = (np.zeros(16, np.int32) for _ in range(3))
        sol.ctx.call("mpet_get_amg_variants", blk, _lib._ptr(va), _lib._ptr(vp), _lib._ptr(vr))
        nl = ctypes.c_int32()
        ms = np.zeros(16)
        by = np.zeros(16)
        sol.ctx.call("mpet_profile_vcycle", blk, 7, ctypes.byref(nl), _lib._ptr(ms), _lib._ptr(by))
        L = nl.value
        levels = []
        for k in range(L):
            own = ms[k] - (ms[k + 1] if k + 1 < L else 0.0)
            levels.append({"rows": sizes[k], "nnz": nnz[k], "variants_a_p_r": [int(va[k]), int(vp[k]), int(vr[k])],
                           "own_ms": round(own, 5), "vcycle_from_here_ms":
                           round(ms[k], 5), "alg_bytes": int(by[k]),
                           "gbs": round(by[k] / own / 1e6, 1) if own > 0 else None,
                           "frac": round(by[k] / own / 1e6 / hbm, 3) if own > 0 else None})
        out["blocks"].append({"block": "displacement" if blk == 0 else "pressure %d" % blk, "levels": levels,
                              "vcycle_ms": round(ms[0], 5), "alg_bytes": int(by[:L].sum())})
    out["preconditioner_ms"] = time_precond(sol, torch, _lib)
    out["preconditioner_alg_bytes"] = int(sum(b["alg_bytes"] for b in out["blocks"]))
    out["preconditioner_gbs"] = out["preconditioner_alg_bytes"] / out["preconditioner_ms"] / 1e6
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--networks", type=int, default=4)
    ap.add_argument("--workload", default="cube", choices=["cube", "ellipsoid"],
                    help="cube: Kuhn n^3 cube; ellipsoid: jittered shell, n radial layers, per-cell K")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--per-step-error", action="store_true",
                    help="also run both precisions in lockstep and report the relative error after every step")
    ap.add_argument("--profile", action="store_true",
                    help="one step with at most --maxit MINRES iterations (small launch count for ncu)")
    ap.add_argument("--maxit", type=int, default=12)
    ap.add_argument("--adjoint", action="store_true",
                    help="discrete-adjoint gradient check (A=2 on the --n cube, 20 steps) instead of the bench")
    ap.add_argument("--fd-dirs", type=int, default=64)
    ap.add_argument("--batch", action="store_true",
                    help="batch of independent A=2 instances (--instances, n in [--n-min, --n-max]) instead of the bench")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--n-min", type=int, default=8)
    ap.add_argument("--n-max", type=int, default=32)
    ap.add_argument("--sequential-steps", type=int, default=3,
                    help="batch mode: also time this many steps of every instance solved alone (0: skip)")
    ap.add_argument("--cheb-degree", type=int, default=None, help="override amg_cheb_degree")
    ap.add_argument("--coarse-size", type=int, default=None, help="override amg_coarse_size")
    ap.add_argument("--cheb-degree-fine", type=int, default=None,
                    help="override amg_cheb_degree_fine (the finest level of every hierarchy)")
    ap.add_argument("--cheb-degree-coarse", type=int, default=None,
                    help="override amg_cheb_degree_coarse (levels 2, 3, ... of every hierarchy)")
    ap.add_argument("--cheb-coarse-level", type=int, default=None,
                    help="override amg_cheb_coarse_level (first level with the coarse degree)")
    ap.add_argument("--prec-u-order", default=None, choices=["spatial", "natural"],
                    help="row order of the first displacement level (default: natural)")
    ap.add_argument("--amg-setup", default=None, choices=["device", "host"],
                    help="where the smoothed-aggregation hierarchies are built (default: device)")
    ap.add_argument("--inner-loop", default=None, choices=["device", "host"],
                    help="inner Krylov loop: one graph launch with a device-side loop, or host-checked replays")
    ap.add_argument("--prec-u-form", default=None, choices=["elasticity", "laplacian"],
                    help="override the displacement block of the preconditioner")
    ap.add_argument("--inner-rtol", type=float, default=None, help="override inner_rtol")
    ap.add_argument("--vcycle-profile", action="store_true",
                    help="per-level time and algorithmic bytes of the block preconditioner instead of the bench")
    ap.add_argument("--estimators", action="store_true",
                    help="time the AdaptiveMPETSolver error indicators on the --n cube instead of the bench")
    ap.add_argument("--formulation", default="mpet", choices=["mpet", "total-pressure"],
                    help="total-pressure: MPETTotalPressureSolver (u, p0, networks) on the same workload")
    args = ap.parse_args()
    if args.batch:
        return batch_run(args)
    if args.profile:
        return profile_case(args)
    if args.adjoint:
        return adjoint_check(args)
    if args.estimators:
        return estimator_run(args)
    if args.vcycle_profile:
        return vcycle_profile(args)
    n, J = args.n, args.networks
    tp = args.formulation == "total-pressure"
    N_full = 3 * (2 * n + 1) ** 3 + (J + int(tp)) * (n + 1) ** 3
    workload_name = "Kuhn cube %d^3 x 6 tets, A=%d networks, P2/P1 (N=%d)" % (n, J, N_full)
    if tp:
        workload_name += ", total-pressure form (u, p0, p_1..p_A)"
    if args.workload == "ellipsoid":
        workload_name = ("jittered ellipsoidal shell (1, 0.8, 0.7; inner 0.3), %d radial layers, %d tets, A=%d, "
                         "log-normal per-cell K" % (n, 144 * n ** 3, J))

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        if tp or args.workload != "cube":
            print(json.dumps({"impl": "reference", "unavailable": "the CPU arm runs the MPET form on the Kuhn cube "
                                                                  "workloads only"}))
            return
        r = cpu_full_run(n, J, args.workload, warmup=min(args.warmup, 1), steps=args.steps)
        sample = ("oracle C restatement (OpenMP MINRES + block SA V-cycles, C assembly) on %d host threads: the full "
                  "%s; %d untimed warm-up step(s), then %d timed solve_direct step(s) of the %d requested (timed "
                  "steps stop after 180 s); MINRES iterations %s; set-up %.1f s assembly + %.1f s hierarchies "
                  "(untimed). FEniCS/PETSc (the reference's own path) is not installable here"
                  % (r["cores"], workload_name, r["warmup"], r["steps"], args.steps, r["iterations"],
                     r["assemble_s"], r["hierarchies_s"]))
        line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": "steps/s", "n_gpus": 0,
                "steps": r["steps"], "warmup": r["warmup"], "ms_per_step": 1e3 / r["value"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": workload_name, "nnz": r["nnz"], "dt": 0.01 if J == 4 else 0.0125,
                           "rtol": 1e-10, "requested_steps": args.steps, "requested_warmup": args.warmup,
                           "semantics": "solve_direct step: rhs + MINRES/block-SA-AMG solve (matrix and AMG "
                                        "built once)"},
                "cpu_baseline": {"value": r["value"], "unit": "steps/s", "cores": r["cores"], "kind": "port",
                                 "sample": sample},
                "e2e": {"value": r["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local_rank)
    from waterscapes_gb300 import MPETSolver, MPETTotalPressureSolver, _lib
    lib = _lib
    Solver = MPETTotalPressureSolver if tp else MPETSolver
    hbm, peak_kind = peaks()

    problem, dt = workload(n, J, args.workload)
    base = dict(dt=dt, T=1e9, theta=1.0, rtol=1e-10, device=local_rank)
    if args.cheb_degree is not None:
        base["amg_cheb_degree"] = args.cheb_degree
    if args.inner_rtol is not None:
        base["inner_rtol"] = args.inner_rtol
    if args.coarse_size is not None:
        base["amg_coarse_size"] = args.coarse_size
    if args.cheb_degree_fine is not None:
        base["amg_cheb_degree_fine"] = args.cheb_degree_fine
    if args.cheb_degree_coarse is not None:
        base["amg_cheb_degree_coarse"] = args.cheb_degree_coarse
    if args.inner_loop is not None:
        base["inner_loop"] = args.inner_loop
    if args.amg_setup is not None:
        base["amg_setup"] = args.amg_setup
    if args.prec_u_order is not None:
        base["prec_u_order"] = args.prec_u_order
    if args.prec_u_form is not None:
        base["prec_u_form"] = args.prec_u_form
    t0 = time.perf_counter()
    sol = Solver(problem, dict(base, precision="mixed"))
    t_setup = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sol._assemble(dt)
    torch.cuda.synchronize()
    t_asm_amg = time.perf_counter() - t0
    # matrix assembly alone (step() semantics re-assemble every step)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(sol._stream)
    sol.ctx.call("mpet_assemble", dt, 1)
    e1.record(sol._stream)
    torch.cuda.synchronize()
    asm_ms = e0.elapsed_time(e1)
    spmv = time_spmv(sol, torch, lib)
    precond_ms = time_precond(sol, torch, lib)

    clk = ClockSampler(local_rank)
    if world > 1:
        torch.distributed.barrier()
    L0 = launches(sol)
    clk.start()
    ms_mixed, its_mixed, x_mixed, split = run_steps(sol, torch, args.steps, args.warmup, dt)
    clocks = clk.stop()
    L1 = launches(sol)
    value, ms_max = replica_rate(ms_mixed, args.steps)

    # end to end through the public API with host buffers (pinned), copies timed
    problem.time.assign(0.0)
    host_prev = torch.zeros(sol.N, dtype=torch.float64).pin_memory()
    host_out = torch.empty(sol.N, dtype=torch.float64).pin_memory()
    for _ in range(2):
        sol.up_.vector().copy_(host_prev, non_blocking=True)
        sol.step(dt)
        host_out.copy_(sol.up.vector(), non_blocking=True)
    torch.cuda.synchronize()
    problem.time.assign(0.0)
    host_prev.zero_()
    e0.record(sol._stream)
    ke = max(2, min(args.steps, 5))
    for _ in range(ke):
        sol.up_.vector().copy_(host_prev, non_blocking=True)
        sol.advance(dt)
        host_out.copy_(sol.up.vector(), non_blocking=True)
        torch.cuda.current_stream().synchronize()
        host_prev.copy_(host_out)
    e1.record(sol._stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / ke

    # step() semantics: assemble every step
    step_ms = asm_ms + ms_mixed / args.steps

    res = {"mixed": {"ms_per_step": ms_mixed / args.steps, "iterations": its_mixed}}
    rel_err = None
    if not args.no_fp64:
        sol64 = Solver(problem, dict(base, precision="fp64"))
        sol64._assemble(dt)
        spmv64 = time_spmv(sol64, torch, lib)
        spmv["fp64_only_ctx"] = spmv64.get("fp64")
        precond64_ms = time_precond(sol64, torch, lib)
        ms64, its64, x64, split64 = run_steps(sol64, torch, args.steps, args.warmup, dt)
        rel_err = float(torch.linalg.norm(x_mixed - x64) / torch.linalg.norm(x64))
        res["fp64"] = {"ms_per_step": ms64 / args.steps, "iterations": its64,
                       "iteration_breakdown_ms": dict(split64, spmv_fp64=spmv64["fp64"]["ms"],
                                                      preconditioner=precond64_ms)}
        if args.per_step_error:
            # the two paths in lockstep from the zero state: relative error of the
            # mixed-precision state against the FP64 one after every step
            errs = []
            problem.time.assign(0.0)
            sol.up_.vector().zero_()
            sol64.up_.vector().zero_()
            g32, g64 = sol.solve_direct(), sol64.solve_direct()
            for _ in range(args.warmup + args.steps):
                t_now = float(problem.time)
                up32, _ = next(g32)
                problem.time.assign(t_now)
                up64, _ = next(g64)
                v64 = up64.vector()
                errs.append(float(torch.linalg.norm(up32.vector() - v64) / torch.linalg.norm(v64)))
            res["per_step_rel_err"] = errs
            del g32, g64
        del sol64

    cpu = None
    if rank == 0 and not args.no_cpu and not tp and args.workload == "cube":
        r = cpu_full_run(n, J, args.workload, warmup=0, steps=1)
        cpu = {"value": r["value"], "unit": "steps/s", "cores": r["cores"], "kind": "port",
               "sample": "oracle C restatement (OpenMP MINRES + block SA V-cycles, C assembly) on %d host threads: "
                         "one solve_direct step (%d MINRES iterations, %.1f s) of the full workload (N=%d) from the "
                         "zero state, after an untimed set-up (%.1f s assembly, %.1f s hierarchies)"
                         % (r["cores"], r["iterations"][0], r["seconds"], r["N"], r["assemble_s"],
                            r["hierarchies_s"])}

    if rank != 0:
        return
    sp32 = spmv.get("fp32") or spmv.get("fp64")
    headline = args.workload == "cube" and n == 64 and J == 4 and not tp
    tuning = spmv_tuning(sol)
    line = {
        "metric": METRIC if headline else "MPET steps/s, mixed vs FP64 GPU at 1e-8 rel err; SpMV HBM GB/s",
        "value": value,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 inner + f64 refinement",
        "data": "synthetic",
        "config": {"workload": workload_name, "nnz": sol.nnz, "dt": dt, "rtol": 1e-10,
                   "semantics": "solve_direct step: rhs + MINRES/block-SA-AMG solve (matrix and AMG built once)",
                   "l2": "inputs larger than L2 (CSR %.1f GB)" % (sol.nnz * 16 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64_steps_per_s": (1e3 / res["fp64"]["ms_per_step"]) if "fp64" in res else None,
        "mixed_over_fp64": (res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"]) if "fp64" in res else None,
        "rel_err_mixed_vs_fp64": rel_err,
        "rel_err_mixed_vs_fp64_per_step": res.get("per_step_rel_err"),
        "iterations_per_step": {"mixed": its_mixed, "fp64": res.get("fp64", {}).get("iterations")},
        "step_semantics": {"ms_per_step": step_ms, "assemble_ms": asm_ms},
        "setup_s": {"mesh_dofmap_pattern": t_setup, "assemble_plus_amg": t_asm_amg,
                    "preconditioner_ms": prec_setup_ms(sol)},
        "spmv": spmv,
        "spmv_tuning": tuning,
        "spmv_tuning_fp64_residual": spmv_tuning(sol, fp64=True),
        "preconditioner_u_block": prec_form(sol),
        "preconditioner_level_variants": level_variants(sol),
        "iteration_breakdown_ms": dict(split, spmv_fp32=(spmv.get("fp32") or spmv["fp64"])["ms"],
                                       preconditioner=precond_ms),
        "fp64_iteration_breakdown_ms": res.get("fp64", {}).get("iteration_breakdown_ms"),
        "roofline": {"kernel": ROOFLINE_KERNEL[sp32["layout"]] + (" FP32" if "fp32" in spmv else " FP64")
                     + (", 64-register kernel" if tuning.get("chosen") == "node-block/64 registers" else ""),
                     "bound": "hbm", "achieved": sp32["gbs"], "peak": hbm, "unit": "GB/s",
                     "frac": sp32["gbs"] / hbm, "peak_kind": peak_kind,
                     "alg_bytes_per_launch": sp32["alg_bytes"],
                     "traffic": (sp32["alg_bytes"] * TRAFFIC_RATIO[sp32["layout"]]
                                 if sp32["layout"] in TRAFFIC_RATIO else None),
                     "traffic_source": TRAFFIC_SOURCE.get(sp32["layout"])},
        "cpu_baseline": cpu,
        "e2e": {"value": 1e3 / e2e_ms, "unit": "steps/s", "h2d_bytes_per_step": sol.N * 8,
                "d2h_bytes_per_step": sol.N * 8},
        "clocks": clocks,
        "gpu_launches": (L1 - L0),
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
