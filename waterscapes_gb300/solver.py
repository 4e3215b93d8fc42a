"""MPETSolver drop-in: the reference's API over the GB300 engine.

Mirrors src/mpet/mpet/mpetsolver.py: constructor ``MPETSolver(problem,
params)``, ``default_params`` (:86-98, plus engine keys the reference does
not read), ``step(dt)`` (:317-379), ``solve()`` (:300-309) and
``solve_direct()`` (:382-462) generators yielding ``(up, t)``, the fields
``up`` / ``up_`` with ``vector()``, ``split()`` and ``assign()``, ``dt`` as a
mutable Constant and ``solver_monitor`` with the Krylov iteration counts.

Every numerical operation runs in libmpetgpu on the GPU (element kernels,
CSR assembly, Dirichlet rows, right-hand side, MINRES + AMG); this module
only moves parameters, evaluates the user's boundary/source expressions at
DOF coordinates, and orders the calls as the reference does.
"""
from __future__ import annotations

import ctypes
import math
import warnings

import numpy as np

from . import _lib
from .problem import Constant, Expression, is_zero

DIRICHLET_MARKER = 0
NEUMANN_MARKER = 1
ROBIN_MARKER = 2


def _torch():
    import torch
    return torch


class Function:
    """State vector in the global block-natural DOF order (float64, on the GPU)."""

    def __init__(self, solver, data):
        self._solver = solver
        self._v = data

    def vector(self):
        return self._v

    def function_space(self):
        return self._solver

    def split(self, deepcopy=False):
        s = self._solver
        v = self._v.clone() if deepcopy else self._v
        u = v[:s.Nu].view(s.nnodes, s.dim)
        ps = [v[s.Nu + a * s.nv: s.Nu + (a + 1) * s.nv] for a in range(s.J)]
        extra = []
        if getattr(s, "nrigid", 0):
            # the rigid-motion multipliers r (the R-space part of the reference's mixed function)
            extra = [s._rigid_r.clone() if deepcopy else s._rigid_r]
        for k in range(getattr(s, "nq", 0)):
            # one multiplier per constant-pressure constraint, in network order
            q = s._p_null[k:k + 1]
            extra.append(q.clone() if deepcopy else q)
        return tuple([u] + ps + extra)

    def assign(self, other):
        src = other.vector() if isinstance(other, Function) else other
        if not hasattr(src, "data_ptr"):
            src = _torch().as_tensor(np.asarray(src, dtype=np.float64))
        self._v.copy_(src.to(self._v.device, dtype=self._v.dtype))

    def __len__(self):
        return self._v.shape[0]


class MPETSolver:
    """Backward-Euler / theta-scheme MPET solver on one GB300."""

    def __init__(self, problem, params=None):
        torch = _torch()
        self.problem = problem
        self.params = self.default_params()
        if params is not None:
            self.params.update(params)
        self.solver_monitor = {"niter": [], "relres": []}
        mesh = problem.mesh
        if mesh.gdim not in (2, 3) or mesh.tdim != mesh.gdim:
            raise NotImplementedError("the GPU engine assembles triangle (2D) and tetrahedral (3D) meshes")
        self.dim = mesh.gdim
        pp = problem.params
        self.J = int(pp["J"])
        self._check_facet_data()
        dev = int(self.params["device"])
        self.device = torch.device("cuda", dev)
        torch.cuda.set_device(self.device)
        self._ctx = _lib.Context(dev)
        self._stream = torch.cuda.current_stream(self.device)
        self._ctx.call("mpet_set_stream", ctypes.c_void_p(self._stream.cuda_stream))
        # mesh and markers (coordinates as nv x 3, z = 0 in 2D)
        x = np.zeros((mesh.num_vertices(), 3), dtype=np.float64)
        x[:, :self.dim] = mesh.coordinates()
        cells = np.ascontiguousarray(mesh.cells(), dtype=np.int32)
        bf = np.ascontiguousarray(mesh.boundary_facets(), dtype=np.int32)
        markers = np.ascontiguousarray(np.stack(
            [problem.momentum_boundary_markers.as_int32()]
            + [problem.continuity_boundary_markers[a].as_int32() for a in range(self.J)], 0), dtype=np.int32)
        self._ctx.call("mpet_mesh_upload_dim", self.dim, x.shape[0], _lib._ptr(x), cells.shape[0], _lib._ptr(cells),
                       bf.shape[0], _lib._ptr(bf), _lib._ptr(markers), self.J)
        self._prm = self._make_params()
        self._ctx.call("mpet_setup", ctypes.byref(self._prm))
        # smoothed-aggregation set-up on the GPU ("device") or on host threads ("host")
        self._ctx.call("mpet_set_amg_setup", {"host": 0, "device": 1}[self.params.get("amg_setup", "device")])
        # per-cell permeability fields (K_a given as an array with one value per cell)
        Ks = [np.asarray(k, dtype=np.float64) for k in pp["K"]]
        self._K_cells = None
        if any(k.ndim > 0 for k in Ks):
            nc = mesh.num_cells()
            Kc = np.stack([np.broadcast_to(k, (nc,)) for k in Ks]).astype(np.float64)
            self._K_cells = torch.as_tensor(np.ascontiguousarray(Kc), device=self.device)
            self._ctx.call("mpet_set_cell_permeability", _lib._ptr(self._K_cells))
        N, nnz, nn, ne = (ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64())
        self._ctx.call("mpet_get_sizes", ctypes.byref(N), ctypes.byref(nnz), ctypes.byref(nn), ctypes.byref(ne))
        self.N, self.nnz, self.nnodes, self.ne = N.value, nnz.value, nn.value, ne.value
        self.nv = mesh.num_vertices()
        self.Nu = self.dim * self.nnodes
        f64 = dict(dtype=torch.float64, device=self.device)
        self.up_ = Function(self, torch.zeros(self.N, **f64))
        self.up = Function(self, torch.zeros(self.N, **f64))
        self.dt = Constant(float(self.params["dt"]))
        self._bcs = self.create_dirichlet_bcs()
        self._node_x = None
        # rigid-motion modes of a displacement without Dirichlet conditions
        # (the R-space multipliers of mpetsolver.py:115-124, 204-207)
        self.nrigid = 0
        self._rigid_r = None
        if problem.u_has_nullspace:
            from .nullspace import rigid_motions
            Z = rigid_motions(mesh, self._node_coordinates().cpu().numpy())
            self.nrigid = Z.shape[0]
            self._rigid_Z = torch.as_tensor(np.ascontiguousarray(Z.reshape(self.nrigid, -1)), device=self.device)
            self._ctx.call("mpet_set_rigid_modes", self.nrigid, _lib._ptr(self._rigid_Z))
            self._rigid_r = torch.zeros(self.nrigid, dtype=torch.float64, device=self.device)
        # constant-pressure constraints with multipliers (mpetsolver.py:120-124, 209-215)
        nets = [a for a, f in enumerate(problem.p_has_nullspace) if f]
        self.nq = len(nets)
        self._p_null = None
        if nets:
            arr = np.ascontiguousarray(nets, dtype=np.int32)
            self._ctx.call("mpet_set_pressure_constraints", self.nq, _lib._ptr(arr))
            self._p_null = torch.zeros(self.nq, dtype=torch.float64, device=self.device)
        self._assembled_dt = None
        self._prec_dt = None
        self._f = None
        self._g = None

    # --- parameters --------------------------------------------------------------
    @staticmethod
    def default_params():
        """mpetsolver.py:86-98 plus engine keys (ignored by the reference)."""
        return {"dt": 0.1, "t": 0.0, "T": 1.0, "theta": 1.0, "u_degree": 2, "p_degree": 1,
                "direct_solver": True,
                "precision": "mixed", "rtol": 1e-10, "inner_rtol": 3e-4, "maxit": 20000,
                "max_outer": 40, "amg_theta": 0.1, "amg_cheb_degree": 4, "amg_coarse_size": 500,
                "amg_p2_to_p1": True, "prec_u_weight": "mu+lmbda", "prec_network_modes": True,
                "prec_u_form": "laplacian", "krylov": "auto", "gmres_restart": 30,
                "amg_cheb_degree_fine": 0, "amg_cheb_degree_coarse": 3, "amg_cheb_coarse_level": 2,
                "inner_loop": "device",
                "amg_setup": "device", "prec_u_order": "natural",
                "check_every": 4, "device": 0}

    def _make_params(self):
        pp = self.problem.params
        mu, lmbda = self.problem.lame()
        prm = _lib.MpetParams()
        prm.num_networks = self.J
        prm.precision = _lib.PRECISION[self.params["precision"]]
        prm.mu, prm.lmbda = mu, lmbda
        for a in range(self.J):
            prm.alpha[a] = float(pp["alpha"][a])
            prm.c[a] = float(pp["c"][a])
            # a per-cell (DG0) permeability is uploaded separately; the scalar slot holds its mean
            prm.K[a] = float(np.mean(np.asarray(pp["K"][a], dtype=np.float64)))
            for b in range(self.J):
                prm.S[a * _lib.MAX_NETWORKS + b] = float(pp["S"][a][b])
        prm.theta = float(self.params["theta"])
        if int(self.params["u_degree"]) != 2 or int(self.params["p_degree"]) != 1:
            raise NotImplementedError("the GPU engine implements the P2 x P1 pair (u_degree=2, p_degree=1)")
        prm.rtol = float(self.params["rtol"])
        prm.inner_rtol = float(self.params["inner_rtol"])
        prm.maxit = int(self.params["maxit"])
        prm.max_outer = int(self.params["max_outer"])
        prm.amg_theta = float(self.params["amg_theta"])
        prm.amg_cheb_degree = int(self.params["amg_cheb_degree"])
        prm.amg_coarse_size = int(self.params["amg_coarse_size"])
        prm.check_every = int(self.params["check_every"])
        prm.amg_p2_to_p1 = 1 if self.params["amg_p2_to_p1"] else 0
        w = self.params["prec_u_weight"]
        prm.prec_u_weight = {"mu+lmbda": mu + lmbda, "mu": mu, "2mu": 2.0 * mu}[w] if isinstance(w, str) else float(w)
        prm.prec_network_modes = 1 if self.params["prec_network_modes"] else 0
        prm.prec_u_form = {"laplacian": 0, "elasticity": 1}[self.params.get("prec_u_form", "laplacian")]
        # MINRES for a symmetric system; GMRES (auto: when S is not symmetric)
        prm.krylov = _lib.KRYLOV[self.params.get("krylov", "auto")]
        prm.gmres_restart = int(self.params.get("gmres_restart", 30))
        prm.amg_cheb_degree_fine = int(self.params.get("amg_cheb_degree_fine", 0))
        prm.amg_cheb_degree_coarse = int(self.params.get("amg_cheb_degree_coarse", 3))
        prm.amg_cheb_coarse_level = int(self.params.get("amg_cheb_coarse_level", 2))
        prm.prec_u_order = {"natural": 0, "spatial": 1}[self.params.get("prec_u_order", "natural")]
        prm.inner_loop = {"device": 0, "host": 1}[self.params.get("inner_loop", "device")]
        if self.problem.u_has_nullspace:
            # mass shift of the displacement preconditioner block at the scale of the
            # lowest elastic mode: (mu + lambda) / diam^2
            xs = np.asarray(self.problem.mesh.coordinates())
            diam = float(np.linalg.norm(xs.max(0) - xs.min(0)))
            prm.prec_u_shift = (mu + lmbda) / diam ** 2
        return prm

    def _check_facet_data(self):
        """Which boundary-facet terms are active (mpetsolver.py:231-254)."""
        p = self.problem
        J = int(p.params["J"])
        mm = p.momentum_boundary_markers.array()
        self._traction_on = bool((mm == NEUMANN_MARKER).any() and not is_zero(p.s))
        cm = [p.continuity_boundary_markers[a].array() for a in range(J)]
        self._flux_on = any((cm[a] == NEUMANN_MARKER).any() and not is_zero(p.I[a]) for a in range(J))
        self._robin_on = any((cm[a] == ROBIN_MARKER).any() for a in range(J))

    # --- boundary conditions -------------------------------------------------------
    def create_dirichlet_bcs(self):
        """DOFs and coordinates of the topological Dirichlet conditions (mpetsolver.py:63-84)."""
        torch = _torch()
        bcs = []
        for field in range(1 + self.J):
            cnt = ctypes.c_int64()
            self._ctx.call("mpet_get_bc_count", field, ctypes.byref(cnt))
            n = cnt.value
            dofs = torch.empty(max(n, 1), dtype=torch.int32, device=self.device)
            coords = torch.empty(max(n, 1), 3, dtype=torch.float64, device=self.device)
            self._ctx.call("mpet_get_bc", field, _lib._ptr(dofs), _lib._ptr(coords))
            bcs.append({"field": field, "n": n, "dofs": dofs[:n], "coords": coords[:n]})
        self.bcs = [[bcs[0]], bcs[1:]]
        return bcs

    def _eval(self, expr, x, t, vector):
        """Values of a data term at points x (n x 3 tensor; z = 0 in 2D): (n, dim)
        for vector data, (n,) for scalar data."""
        torch = _torch()
        n = x.shape[0]
        d = self.dim
        if expr is None:
            v = torch.zeros((n, d) if vector else (n,), dtype=torch.float64, device=self.device)
            return v
        if isinstance(expr, Constant) or isinstance(expr, (int, float, tuple, list)):
            val = expr.values() if isinstance(expr, Constant) else expr
            if vector:
                val = tuple(float(a) for a in (val if isinstance(val, (tuple, list)) else (val,) * d))
                return torch.tensor(val, dtype=torch.float64, device=self.device).expand(n, d).contiguous()
            return torch.full((n,), float(val), dtype=torch.float64, device=self.device)
        v = expr(x, t)
        v = torch.as_tensor(v, dtype=torch.float64, device=self.device)
        if vector:
            v = v.reshape(n, d) if v.numel() == d * n else v.expand(n, d)
        else:
            v = v.reshape(n) if v.numel() == n else v.expand(n)
        return v.contiguous()

    def _set_bc_values(self, t):
        p = self.problem
        b0 = self._bcs[0]
        if b0["n"]:
            xn = b0["coords"][0::self.dim]
            vals = self._eval(p.u_bar, xn, t, True).reshape(-1).contiguous()
            self._bcv0 = vals
            self._ctx.call("mpet_set_bc_values", 0, _lib._ptr(vals))
        self._bcvp = []
        for a in range(self.J):
            ba = self._bcs[1 + a]
            if ba["n"]:
                vals = self._eval(p.p_bar[a], ba["coords"], t, False)
                self._bcvp.append(vals)
                self._ctx.call("mpet_set_bc_values", 1 + a, _lib._ptr(vals))

    def _node_coordinates(self):
        torch = _torch()
        if self._node_x is None:
            edges = np.empty((self.ne, 2), dtype=np.int64)
            self._ctx.call("mpet_get_edges", _lib._ptr(edges))
            x = np.zeros((self.nv, 3))
            x[:, :self.dim] = self.problem.mesh.coordinates()                 # z = 0 in 2D
            nx = np.concatenate([x, 0.5 * (x[edges[:, 0]] + x[edges[:, 1]])], 0)
            self._node_x = torch.as_tensor(nx, dtype=torch.float64, device=self.device)
        return self._node_x

    def _set_sources(self, t_theta, t1):
        p = self.problem
        f = None
        if not is_zero(p.f):
            f = self._eval(p.f, self._node_coordinates(), t1, True).reshape(-1).contiguous()
        g = None
        if any(not is_zero(gi) for gi in p.g):
            xv = self._node_coordinates()[:self.nv]
            g = _torch().stack([self._eval(gi, xv, t_theta, False) for gi in p.g], 0).contiguous()
        self._f, self._g = f, g
        self._ctx.call("mpet_set_sources", _lib._ptr(f), _lib._ptr(g))

    # --- boundary facets ------------------------------------------------------------
    def _facet_geometry(self):
        torch = _torch()
        if getattr(self, "_fgeo", None) is None:
            nf = self.problem.mesh.num_boundary_facets()
            fn = torch.empty(max(nf, 1), 6, dtype=torch.int32, device=self.device)
            geo = torch.empty(max(nf, 1), 4, dtype=torch.float64, device=self.device)
            self._ctx.call("mpet_get_facet_data", _lib._ptr(fn), _lib._ptr(geo))
            self._fnodes, self._fgeo = fn[:nf], geo[:nf]
            fn_count = 6 if self.dim == 3 else 3                                # P2 nodes of a facet
            self._fx = self._node_coordinates()[self._fnodes[:, :fn_count].long()]  # (nf, FN, 3)
            p = self.problem
            mk = lambda m: torch.as_tensor(m, device=self.device)
            self._fmask_u = mk(p.momentum_boundary_markers.array() == NEUMANN_MARKER)
            self._fmask_c = [(mk(p.continuity_boundary_markers[a].array() == NEUMANN_MARKER),
                              mk(p.continuity_boundary_markers[a].array() == ROBIN_MARKER)) for a in range(self.J)]
        return self._fx, self._fgeo

    def _eval_traction(self, expr, x, t, n):
        torch = _torch()
        if isinstance(expr, Expression):
            try:
                v = expr.fn(x, t, n)
            except TypeError:
                v = expr.fn(x, t)
            v = torch.as_tensor(v, dtype=torch.float64, device=self.device)
            d = self.dim
            return v.expand(x.shape[0], d) if v.numel() != d * x.shape[0] else v.reshape(x.shape[0], d)
        return self._eval(expr, x, t, True)

    def _per_network_vertex_data(self, fields, t, mask_index):
        torch = _torch()
        fx, _ = self._facet_geometry()
        fv = self.dim                                                      # vertices of a facet
        xv = fx[:, :fv, :].reshape(-1, 3)
        nf = fx.shape[0]
        out = torch.zeros(self.J, nf, fv, dtype=torch.float64, device=self.device)
        for a in range(self.J):
            mask = self._fmask_c[a][mask_index]
            if fields[a] is None or not bool(mask.any()):
                continue
            v = self._eval(fields[a], xv, t, False).reshape(nf, fv)
            out[a] = v * mask[:, None]
        return out.contiguous()

    def _set_facet_sources(self, t_theta, t1):
        """Traction (at t1), flux and Robin data (at t0 + theta dt) at facet nodes."""
        p = self.problem
        if self._traction_on:
            fx, geo = self._facet_geometry()
            nf, fn = fx.shape[0], fx.shape[1]
            n = geo[:, 1:1 + self.dim].repeat_interleave(fn, dim=0)
            s = self._eval_traction(p.s, fx.reshape(-1, 3), t1, n).reshape(nf, fn, self.dim)
            self._f_s = (s * self._fmask_u[:, None, None]).contiguous()
            self._ctx.call("mpet_set_facet_data", 0, _lib._ptr(self._f_s))
        if self._flux_on:
            self._f_I = self._per_network_vertex_data(p.I, t_theta, 0)
            self._ctx.call("mpet_set_facet_data", 1, _lib._ptr(self._f_I))
        if self._robin_on:
            self._f_b = self._per_network_vertex_data(p.beta, t_theta, 1)
            self._f_pr = self._per_network_vertex_data(p.p_robin, t_theta, 1)
            self._ctx.call("mpet_set_facet_data", 2, _lib._ptr(self._f_b))
            self._ctx.call("mpet_set_facet_data", 3, _lib._ptr(self._f_pr))

    # --- assembly / solve -------------------------------------------------------------
    def _assemble(self, dt):
        if self._robin_on:
            # lhs(F2a) is assembled with the data at the current time (mpetsolver.py:336-338)
            self._f_bm = self._per_network_vertex_data(self.problem.beta, float(self.problem.time), 1)
            self._ctx.call("mpet_set_facet_data", 4, _lib._ptr(self._f_bm))
        self._ctx.call("mpet_assemble", float(dt), 1)
        self._assembled_dt = float(dt)
        if self._prec_dt != float(dt):
            self._ctx.call("mpet_setup_preconditioner", float(dt))
            self._prec_dt = float(dt)

    def advance(self, dt=None):
        """One pass of the solve_direct loop body from ``up_`` at the current time
        with the matrix already assembled: time-dependent data at t0 + theta dt
        and t1, right-hand side, solve into ``up``; updates ``time`` but not ``up_``.
        Assembles first if no matrix for this dt exists."""
        dt = float(self.params["dt"] if dt is None else dt)
        if self._assembled_dt != dt:
            self._assemble(dt)
        return self._advance(dt, float(self.problem.time))

    def _advance(self, dt, t0, guess=None):
        theta = float(self.params["theta"])
        time = self.problem.time
        t_theta = t0 + theta * dt
        t1 = t0 + dt
        time.assign(t_theta)
        g_t = t_theta
        time.assign(t1)
        self._set_sources(g_t, t1)
        self._set_facet_sources(g_t, t1)
        self._set_bc_values(t1)
        st = _lib.MpetStats()
        if guess is None:
            self._ctx.call("mpet_step", float(dt), _lib._ptr(self.up_.vector()), _lib._ptr(self.up.vector()),
                           ctypes.byref(st))
        else:
            # the same step with a caller-chosen initial guess (rhs, then solve from the guess)
            if getattr(self, "_b", None) is None:
                self._b = _torch().empty(self.N, dtype=_torch().float64, device=self.device)
            self._ctx.call("mpet_rhs", float(dt), _lib._ptr(self.up_.vector()), _lib._ptr(self._b))
            self.up.vector().copy_(guess)
            self._ctx.call("mpet_solve", _lib._ptr(self._b), _lib._ptr(self.up.vector()), ctypes.byref(st))
        self.solver_monitor["niter"].append(st.iterations)
        self.solver_monitor["relres"].append(st.relres)
        self.last_stats = st.as_dict()
        if self.nrigid:
            r = np.zeros(self.nrigid)
            self._ctx.call("mpet_get_rigid_multipliers", _lib._ptr(r))
            self._rigid_r.copy_(_torch().as_tensor(r))
        if self.nq:
            q = np.zeros(self.nq)
            self._ctx.call("mpet_get_pressure_multipliers", _lib._ptr(q))
            self._p_null.copy_(_torch().as_tensor(q))
        return st

    def step(self, dt=None, up_=None):
        """One time step t -> t + dt (mpetsolver.py:317-379): assemble, BCs, solve.

        Like the reference, updates ``up`` and ``time`` but not ``up_``.
        """
        self.params["dt"] = float(dt)
        self.dt.assign(dt)
        if up_ is not None:
            self.up_.assign(up_)
        t0 = float(self.problem.time)
        self._assemble(float(dt))
        return self._advance(float(dt), t0)

    def solve(self):
        """mpetsolver.py:300-309: always the direct-solve time loop."""
        warnings.warn("Solving using direct solver, ignoring solver type.")
        return self.solve_direct()

    def solve_direct(self):
        """Generator of (up, t) over [t, T) (mpetsolver.py:382-462).

        The matrix is assembled once before the loop; each step assembles the
        right-hand side and solves.
        """
        dt = float(self.params["dt"])
        T = float(self.params["T"])
        time = self.problem.time
        self._bcs = self.create_dirichlet_bcs()
        self._assemble(dt)
        while float(time) < (T - 1.0e-9):
            t0 = float(time)
            self._advance(dt, t0)
            yield self.up, float(time)
            self.up_.assign(self.up)

    def set_cell_permeability(self, K):
        """Replace the permeability by per-cell (DG0) fields K (J x num_cells);
        the matrix and the preconditioner are rebuilt at the next step."""
        torch = _torch()
        K = torch.as_tensor(K, dtype=torch.float64, device=self.device).contiguous()
        if K.shape != (self.J, self.problem.mesh.num_cells()):
            raise ValueError("K must have shape (J, num_cells) = (%d, %d)" % (self.J, self.problem.mesh.num_cells()))
        self._K_cells = K
        self._ctx.call("mpet_set_cell_permeability", _lib._ptr(K))
        self._assembled_dt = None
        self._prec_dt = None

    # --- engine access used by tests and the bench --------------------------------------
    @property
    def ctx(self):
        return self._ctx

    def pattern(self):
        rp = np.empty(self.N + 1, dtype=np.int64)
        ci = np.empty(self.nnz, dtype=np.int32)
        self._ctx.call("mpet_get_pattern", _lib._ptr(rp), _lib._ptr(ci))
        return rp, ci

    def matrix_values(self):
        v = np.empty(self.nnz, dtype=np.float64)
        self._ctx.call("mpet_get_values", _lib._ptr(v))
        return v

    def edges(self):
        e = np.empty((self.ne, 2), dtype=np.int64)
        self._ctx.call("mpet_get_edges", _lib._ptr(e))
        return e

    def amg_info(self, block):
        lv = ctypes.c_int32()
        sizes = np.zeros(16, dtype=np.int64)
        nnz = np.zeros(16, dtype=np.int64)
        self._ctx.call("mpet_get_amg_info", block, ctypes.byref(lv), _lib._ptr(sizes), _lib._ptr(nnz))
        return sizes[:lv.value].tolist(), nnz[:lv.value].tolist()
