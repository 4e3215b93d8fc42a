"""ctypes driver of the oracle's C restatements (test infrastructure and CPU
baseline): oracle/cminres.c and oracle/cassemble.c, compiled together into
oracle/_build/liboracle.so.

* ``minres`` / ``minres_raw`` run krylov.minres with
  krylov.block_preconditioner's V-cycles in C on all host threads; the
  hierarchies (krylov.SAHierarchy) are built by the Python oracle and passed
  as CSR arrays.
* ``CSystem`` assembles the MPET system, the previous-state operator and the
  preconditioner blocks of a mesh of any size in C (OracleMPET's matrices
  without its per-cell dense arrays) and runs solve_direct steps
  (src/mpet/mpet/mpetsolver.py:382-462) with the C MINRES: the CPU baseline
  on the full 64^3 workload.
* ``aggregate`` is krylov.aggregate in C (same aggregates, faster).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_build", "liboracle.so")
_P, _I64, _D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double


class OCsr(ctypes.Structure):
    _fields_ = [("n", _I64), ("m", _I64), ("rp", _P), ("ci", _P), ("v", _P)]


class OLevel(ctypes.Structure):
    _fields_ = [("A", OCsr), ("P", OCsr), ("R", OCsr), ("dinv", _P), ("rho", _D)]


class OHier(ctypes.Structure):
    _fields_ = [("nlev", ctypes.c_int), ("lev", ctypes.POINTER(OLevel)), ("ncoarse", _I64), ("cinv", _P),
                ("cheb", ctypes.c_int), ("work", _P)]


class OPrec(ctypes.Structure):
    _fields_ = [("Nu", _I64), ("nv", _I64), ("nnodes", _I64), ("dim", ctypes.c_int), ("J", ctypes.c_int),
                ("hu", ctypes.POINTER(OHier)), ("hp", ctypes.POINTER(OHier)), ("Q", _P), ("scratch", _P)]


class OAsm(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("J", ctypes.c_int), ("nc", _I64), ("nv", _I64), ("nnodes", _I64),
                ("x", _P), ("cells", _P), ("cn", _P), ("mu", _D), ("lmbda", _D), ("theta", _D), ("dt", _D),
                ("alpha", _P), ("c", _P), ("K", _P), ("S", _P), ("u_weight", _D), ("lam", _P), ("kk", _P)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("oracle C checker not built (%s)" % LIB)
        _lib = ctypes.CDLL(LIB)
        _lib.oracle_minres.restype = ctypes.c_int
        _lib.oracle_minres.argtypes = [ctypes.POINTER(OCsr), _P, _P, ctypes.POINTER(OPrec), _D, ctypes.c_int,
                                       ctypes.POINTER(_D)]
        _lib.oracle_hier_work.restype = _I64
        _lib.oracle_hier_work.argtypes = [ctypes.c_int, _P]
        _lib.oracle_node_adjacency.restype = ctypes.c_int
        _lib.oracle_node_adjacency.argtypes = [_I64, ctypes.c_int, _P, _I64, _I64, _P, _P, _P]
        _lib.oracle_system_pattern.restype = None
        _lib.oracle_system_pattern.argtypes = [ctypes.c_int, ctypes.c_int, _I64, _I64, _P, _P, _P, _P, _P]
        _lib.oracle_colour_cells.restype = ctypes.c_int
        _lib.oracle_colour_cells.argtypes = [_I64, ctypes.c_int, _P, _I64, _P]
        _lib.oracle_assemble.restype = ctypes.c_int
        _lib.oracle_assemble.argtypes = [ctypes.POINTER(OAsm), ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                         _P]
        _lib.oracle_dirichlet_rows.restype = None
        _lib.oracle_dirichlet_rows.argtypes = [_I64, _P, _P, _P, _P]
        _lib.oracle_rhs_prev.restype = None
        _lib.oracle_rhs_prev.argtypes = [_I64, _I64, _P, _P, _P, _P, _P]
        _lib.oracle_aggregate.restype = _I64
        _lib.oracle_aggregate.argtypes = [_I64, _P, _P, _P]
    return _lib


class _Keep:
    """Holds the arrays the C structures point to."""

    def __init__(self):
        self.arrays = []

    def arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.arrays.append(a)
        return a

    def csr(self, M):
        if M is None:
            return OCsr(0, 0, None, None, None)
        M = sp.csr_matrix(M)
        M.sort_indices()
        rp = self.arr(M.indptr, np.int64)
        ci = self.arr(M.indices, np.int32)
        v = self.arr(M.data, np.float64)
        return OCsr(M.shape[0], M.shape[1], rp.ctypes.data, ci.ctypes.data, v.ctypes.data)

    def hier(self, H):
        levs = (OLevel * len(H.levels))()
        for k, L in enumerate(H.levels):
            d = self.arr(L["Dinv"], np.float64)
            levs[k] = OLevel(self.csr(L["A"]), self.csr(L.get("P")), self.csr(L.get("R")), d.ctypes.data,
                             float(L["rho"]))
        self.arrays.append(levs)
        Ac = H.levels[-1]["A"].toarray()
        cinv = self.arr(np.linalg.inv(Ac), np.float64)
        sizes = self.arr([L["A"].shape[0] for L in H.levels], np.int64)
        nwork = load().oracle_hier_work(len(H.levels), sizes.ctypes.data)
        work = self.arr(np.zeros(max(nwork, 1)), np.float64)
        return OHier(len(H.levels), levs, Ac.shape[0], cinv.ctypes.data, int(H.cheb_degree), work.ctypes.data)


def minres(A, b, hu, hp, dim, Nu, nv, Q=None, x0=None, rtol=1e-10, maxiter=5000):
    """x = x0 + MINRES(A, b - A x0) preconditioned like krylov.block_preconditioner;
    returns (x, iterations, final phibar / beta1)."""
    lib = load()
    k = _Keep()
    Ac = k.csr(A)
    hu_s = k.hier(hu)
    hp_s = (OHier * len(hp))(*[k.hier(h) for h in hp])
    nnodes = Nu // dim
    J = len(hp)
    q = k.arr(Q, np.float64).ctypes.data if Q is not None else None
    scratch = k.arr(np.zeros(2 * max(nnodes, J * nv)), np.float64)
    M = OPrec(Nu, nv, nnodes, dim, J, ctypes.pointer(hu_s), hp_s, q, scratch.ctypes.data)
    x = np.zeros(A.shape[0]) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    bb = k.arr(b, np.float64)
    rel = _D()
    it = lib.oracle_minres(ctypes.byref(Ac), bb.ctypes.data, x.ctypes.data, ctypes.byref(M), rtol, maxiter,
                           ctypes.byref(rel))
    if it < 0:
        raise MemoryError("oracle MINRES could not allocate its vectors")
    return x, it, rel.value


def aggregate(S):
    """krylov.aggregate restated in C (oracle_aggregate): the same three greedy
    passes in the same order, hence the same aggregates."""
    S = sp.csr_matrix(S)
    ptr = np.ascontiguousarray(S.indptr, dtype=np.int64)
    idx = np.ascontiguousarray(S.indices, dtype=np.int32)
    n = S.shape[0]
    agg = np.empty(max(n, 1), dtype=np.int64)
    nagg = load().oracle_aggregate(n, ptr.ctypes.data, idx.ctypes.data, agg.ctypes.data)
    if nagg < 0:
        raise MemoryError("oracle_aggregate")
    return agg[:n], int(nagg)


def minres_raw(rp, ci, v, b, x, hu, hp, dim, Nu, nv, Q=None, rtol=1e-10, maxiter=5000):
    """x += MINRES(A, b - A x) in place, A given by CSR arrays (int64 rp, int32
    ci, float64 v; used without copies); preconditioned like
    krylov.block_preconditioner.  Returns (iterations, final phibar / beta1)."""
    lib = load()
    k = _Keep()
    n = rp.shape[0] - 1
    for a, dt_ in ((rp, np.int64), (ci, np.int32), (v, np.float64), (x, np.float64)):
        if a.dtype != dt_ or not a.flags.c_contiguous:
            raise TypeError("minres_raw needs contiguous int64 rp, int32 ci, float64 values and x")
    Ac = OCsr(n, n, rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
    hu_s = k.hier(hu)
    hp_s = (OHier * len(hp))(*[k.hier(h) for h in hp])
    nnodes = Nu // dim
    J = len(hp)
    q = k.arr(Q, np.float64).ctypes.data if Q is not None else None
    scratch = k.arr(np.zeros(2 * max(nnodes, J * nv)), np.float64)
    M = OPrec(Nu, nv, nnodes, dim, J, ctypes.pointer(hu_s), hp_s, q, scratch.ctypes.data)
    bb = k.arr(b, np.float64)
    rel = _D()
    it = lib.oracle_minres(ctypes.byref(Ac), bb.ctypes.data, x.ctypes.data, ctypes.byref(M), rtol, maxiter,
                           ctypes.byref(rel))
    if it < 0:
        raise MemoryError("oracle MINRES could not allocate its vectors")
    return it, rel.value


def _zero_rows_columns(M, nodes):
    """MatZeroRowsColumns with unit diagonal (OracleMPET.zero_rows_columns without
    a right-hand side), vectorised, in place on a CSR matrix."""
    isbc = np.zeros(M.shape[0], dtype=bool)
    isbc[np.asarray(nodes, dtype=np.int64)] = True
    rows = np.repeat(np.arange(M.shape[0], dtype=np.int64), np.diff(M.indptr))
    M.data[isbc[rows] | isbc[M.indices]] = 0.0
    diag = np.nonzero((M.indices == rows) & isbc[rows])[0]
    M.data[diag] = 1.0
    return M


class CSystem:
    """The MPET system of one mesh assembled by oracle/cassemble.c.

    Holds, in the oracle's block-natural DOF order (fem.DofMap):
    the Dirichlet-row system A (CSR: ``rp``, ``ci``, ``A``), the pressure rows
    of the previous-state operator ``B`` (b = B up_ is OracleMPET.rhs_L without
    data terms), the Dirichlet DOFs of every field and the preconditioner's
    blocks (P2 block w (grad u, grad v), J pressure blocks, both with their
    Dirichlet DOFs eliminated symmetrically) as scipy CSR matrices.

    ``K`` is J constants or a (J, nc) per-cell array; ``bc_facets`` are the
    boundary facets (vertex ids) on which u and every p_a are prescribed
    (DirichletBC on marker 0 for every field).
    """

    def __init__(self, x, cells, J, mu, lmbda, alpha, c, K, S, theta, dt, bc_facets, u_weight=None,
                 modes="auto"):
        from . import fem
        from .mpet import network_modes
        lib = load()
        self.dm = dm = fem.DofMap(x, cells, J)
        d = dm.d
        self.d, self.J, self.theta, self.dt = d, int(J), float(theta), float(dt)
        nc, nv, nn = dm.cells.shape[0], dm.nv, dm.nnodes
        self.N, self.Nu, self.nv = dm.N, dm.Nu, nv
        n2 = dm.nloc2
        cn = np.ascontiguousarray(dm.cell_nodes, dtype=np.int64)
        cl = np.ascontiguousarray(dm.cells, dtype=np.int64)
        xx = np.ascontiguousarray(dm.x, dtype=np.float64)
        # node adjacency (two passes: counts, then ids)
        adj_ptr = np.zeros(nn + 1, dtype=np.int64)
        degv = np.zeros(nn, dtype=np.int32)
        if lib.oracle_node_adjacency(nc, n2, cn.ctypes.data, nn, nv, adj_ptr.ctypes.data, degv.ctypes.data, None):
            raise MemoryError("oracle_node_adjacency")
        adj = np.empty(int(adj_ptr[-1]), dtype=np.int32)
        lib.oracle_node_adjacency(nc, n2, cn.ctypes.data, nn, nv, adj_ptr.ctypes.data, degv.ctypes.data,
                                  adj.ctypes.data)
        # system pattern
        rp = np.empty(self.N + 1, dtype=np.int64)
        lib.oracle_system_pattern(d, J, nn, nv, adj_ptr.ctypes.data, degv.ctypes.data, adj.ctypes.data,
                                  rp.ctypes.data, None)
        ci = np.empty(int(rp[-1]), dtype=np.int32)
        lib.oracle_system_pattern(d, J, nn, nv, adj_ptr.ctypes.data, degv.ctypes.data, adj.ctypes.data,
                                  rp.ctypes.data, ci.ctypes.data)
        self.rp, self.ci, self.nnz = rp, ci, int(rp[-1])
        # vertex pattern of the pressure blocks: the vertex prefix of adj(v)
        vp = np.zeros(nv + 1, dtype=np.int64)
        np.cumsum(degv[:nv], out=vp[1:])
        vrows = np.repeat(np.arange(nv, dtype=np.int64), degv[:nv])
        voff = np.arange(vp[-1], dtype=np.int64) - vp[vrows]
        vci = adj[adj_ptr[vrows] + voff]
        # colouring
        colour = np.empty(nc, dtype=np.int32)
        ncol = lib.oracle_colour_cells(nc, d + 1, cl.ctypes.data, nv, colour.ctypes.data)
        if ncol < 0:
            raise RuntimeError("cell colouring needs more than 256 colours")
        # coefficients
        Kc = np.stack([np.broadcast_to(np.asarray(k, dtype=np.float64), (nc,)) for k in K]).astype(np.float64)
        Kc = np.ascontiguousarray(Kc)
        Sm = np.ascontiguousarray(np.asarray(S, dtype=np.float64).reshape(J, J))
        al = np.ascontiguousarray(alpha, dtype=np.float64)
        cc = np.ascontiguousarray(c, dtype=np.float64)
        Q, lam = network_modes(J, theta, Sm, cc, Kc.mean(axis=1), dt, modes)
        self.Q = None if np.allclose(Q, np.eye(J)) else Q
        kk = np.ascontiguousarray(sum(np.outer(Q[b_] ** 2, Kc[b_]) for b_ in range(J)))
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        w = float(mu + lmbda if u_weight is None else u_weight)
        P = OAsm(d, J, nc, nv, nn, xx.ctypes.data, cl.ctypes.data, cn.ctypes.data, float(mu), float(lmbda),
                 float(theta), float(dt), al.ctypes.data, cc.ctypes.data, Kc.ctypes.data, Sm.ctypes.data, w,
                 lam.ctypes.data, kk.ctypes.data)
        self.A = np.zeros(self.nnz, dtype=np.float64)
        self.B = np.zeros(self.nnz - int(rp[self.Nu]), dtype=np.float64)
        Lu = np.zeros(adj.shape[0], dtype=np.float64)
        Pk = np.zeros(J * int(vp[-1]), dtype=np.float64)
        lib.oracle_assemble(ctypes.byref(P), ncol, colour.ctypes.data, adj_ptr.ctypes.data, degv.ctypes.data,
                            adj.ctypes.data, rp.ctypes.data, vp.ctypes.data, self.A.ctypes.data, self.B.ctypes.data,
                            Lu.ctypes.data, Pk.ctypes.data)
        self.ncolours = ncol
        # Dirichlet DOFs: P2 nodes of the marked facets (vertices and edges) for u,
        # their vertices for every p_a
        f = np.sort(np.asarray(bc_facets, dtype=np.int64), axis=1)
        ekey = dm.edges[:, 0] * nv + dm.edges[:, 1]
        fe = []
        for (a, b_) in fem.local_edges(d - 1):
            kf = f[:, a] * nv + f[:, b_]
            fe.append(nv + np.searchsorted(ekey, kf))
        self.bc_nodes = np.unique(np.concatenate([f.ravel()] + fe))
        self.bc_vertices = np.unique(f.ravel())
        self.bc_u = (d * self.bc_nodes[:, None] + np.arange(d)[None, :]).ravel()
        self.bc_dofs = np.concatenate([self.bc_u] + [self.Nu + a * nv + self.bc_vertices for a in range(J)])
        lib.oracle_dirichlet_rows(self.bc_dofs.shape[0], self.bc_dofs.ctypes.data, rp.ctypes.data, ci.ctypes.data,
                                  self.A.ctypes.data)
        self.Lu = _zero_rows_columns(sp.csr_matrix((Lu, adj, adj_ptr), shape=(nn, nn)), self.bc_nodes)
        self.Pk = [_zero_rows_columns(sp.csr_matrix((Pk[k * vp[-1]:(k + 1) * vp[-1]].copy(), vci, vp),
                                                    shape=(nv, nv)), self.bc_vertices) for k in range(J)]
        self.hu = self.hp = None

    def matrix(self):
        """A as a scipy CSR matrix (shares the arrays)."""
        return sp.csr_matrix((self.A, self.ci, self.rp), shape=(self.N, self.N))

    def rhs_prev(self, up_prev):
        """b = B up_ (zero displacement rows)."""
        y = np.empty(self.N)
        load().oracle_rhs_prev(self.N, self.Nu, self.rp.ctypes.data, self.ci.ctypes.data, self.B.ctypes.data,
                               np.ascontiguousarray(up_prev, dtype=np.float64).ctypes.data, y.ctypes.data)
        return y

    def build_hierarchies(self, theta=0.1, cheb_degree=4):
        """The SA hierarchies of the block preconditioner (P2 block through the
        P1-in-P2 embedding, one per pressure block), aggregation in C."""
        from . import krylov
        P0 = krylov.p1_in_p2_embedding(self.dm, self.bc_nodes)
        self.hu = krylov.SAHierarchy(self.Lu, theta=theta, cheb_degree=cheb_degree, P0=P0, aggregate_fn=aggregate)
        self.hp = [krylov.SAHierarchy(B, theta=theta, cheb_degree=cheb_degree, aggregate_fn=aggregate)
                   for B in self.Pk]

    def step(self, up_prev, bc_values, rtol=1e-10, maxiter=5000):
        """One solve_direct step: b = B up_ with the Dirichlet values
        ``bc_values`` (aligned with ``bc_dofs``) in its Dirichlet rows, solved
        by MINRES from up_ with those values set.  Returns (up, iterations)."""
        b = self.rhs_prev(up_prev)
        b[self.bc_dofs] = bc_values
        x = np.array(up_prev, dtype=np.float64, copy=True)
        x[self.bc_dofs] = bc_values
        it, rel = minres_raw(self.rp, self.ci, self.A, b, x, self.hu, self.hp, self.d, self.Nu, self.nv, Q=self.Q,
                             rtol=rtol, maxiter=maxiter)
        if not rel <= rtol:
            raise RuntimeError("oracle MINRES stopped at relative residual %.3e after %d iterations" % (rel, it))
        return x, it
