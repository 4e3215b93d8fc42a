"""ctypes driver of oracle/cminres.c (test infrastructure and CPU baseline).

Runs krylov.minres with krylov.block_preconditioner's V-cycles in C on all
host threads; the hierarchies (krylov.SAHierarchy) are built by the Python
oracle and passed as CSR arrays.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_build", "libcminres.so")
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
