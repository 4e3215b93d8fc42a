"""ctypes binding of libmpetgpu (the C ABI in include/mpet_gpu.h).

The shared object is built in-tree by ``waterscapes_gb300.build``.  There is
no fallback: if the library is missing or the device is unavailable every
call raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmpetgpu.so")

MPET_OK = 0
ERRORS = {
    -1: "MPET_ERR_INVALID",
    -2: "MPET_ERR_NOMEM",
    -3: "MPET_ERR_CUDA",
    -4: "MPET_ERR_MAXIT",
    -5: "MPET_ERR_BREAKDOWN",
    -6: "MPET_ERR_TIMEOUT",
    -7: "MPET_ERR_STATE",
}
PRECISION = {"fp64": 0, "mixed": 1}
FORMULATION = {"mpet": 0, "total_pressure": 1}
KRYLOV = {"auto": 0, "minres": 1, "gmres": 2}
MAX_NETWORKS = 8


class MpetParams(ctypes.Structure):
    _fields_ = [
        ("num_networks", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("mu", ctypes.c_double),
        ("lmbda", ctypes.c_double),
        ("alpha", ctypes.c_double * MAX_NETWORKS),
        ("c", ctypes.c_double * MAX_NETWORKS),
        ("K", ctypes.c_double * MAX_NETWORKS),
        ("S", ctypes.c_double * (MAX_NETWORKS * MAX_NETWORKS)),
        ("theta", ctypes.c_double),
        ("rtol", ctypes.c_double),
        ("inner_rtol", ctypes.c_double),
        ("maxit", ctypes.c_int32),
        ("max_outer", ctypes.c_int32),
        ("amg_theta", ctypes.c_double),
        ("amg_cheb_degree", ctypes.c_int32),
        ("amg_coarse_size", ctypes.c_int32),
        ("check_every", ctypes.c_int32),
        ("amg_p2_to_p1", ctypes.c_int32),
        ("prec_network_modes", ctypes.c_int32),
        ("prec_u_weight", ctypes.c_double),
        ("prec_u_shift", ctypes.c_double),
        ("formulation", ctypes.c_int32),
        ("prec_u_form", ctypes.c_int32),
        ("prec_p0_weight", ctypes.c_double),
        ("krylov", ctypes.c_int32),
        ("gmres_restart", ctypes.c_int32),
        ("amg_cheb_degree_fine", ctypes.c_int32),
        ("inner_loop", ctypes.c_int32),
        ("amg_cheb_degree_coarse", ctypes.c_int32),
        ("amg_cheb_coarse_level", ctypes.c_int32),
        ("prec_u_order", ctypes.c_int32),
    ]


class MpetStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32),
        ("outer", ctypes.c_int32),
        ("status", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("relres", ctypes.c_double),
        ("relres_true", ctypes.c_double),
    ]

    def as_dict(self):
        return {"iterations": self.iterations, "outer": self.outer, "status": self.status,
                "relres": self.relres, "relres_true": self.relres_true}


class MpetError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


_lib = None
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_D = ctypes.c_double

SIGNATURES = {
    "mpet_ctx_create": [ctypes.c_int, ctypes.POINTER(_P)],
    "mpet_ctx_destroy": [_P],
    "mpet_last_error": [_P],
    "mpet_set_stream": [_P, _P],
    "mpet_synchronize": [_P],
    "mpet_mesh_upload": [_P, _I64, _P, _I64, _P, _I64, _P, _P, _I32],
    "mpet_mesh_upload_dim": [_P, _I32, _I64, _P, _I64, _P, _I64, _P, _P, _I32],
    "mpet_setup": [_P, ctypes.POINTER(MpetParams)],
    "mpet_update_params": [_P, ctypes.POINTER(MpetParams)],
    "mpet_get_sizes": [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
    "mpet_get_pattern": [_P, _P, _P],
    "mpet_get_edges": [_P, _P],
    "mpet_assemble": [_P, _D, _I32],
    "mpet_get_values": [_P, _P],
    "mpet_get_bc_count": [_P, _I32, ctypes.POINTER(_I64)],
    "mpet_get_bc": [_P, _I32, _P, _P],
    "mpet_set_bc_values": [_P, _I32, _P],
    "mpet_set_sources": [_P, _P, _P],
    "mpet_set_cell_permeability": [_P, _P],
    "mpet_set_cell_coefficients": [_P, _P, _P],
    "mpet_set_rigid_modes": [_P, _I32, _P],
    "mpet_get_rigid_multipliers": [_P, _P],
    "mpet_set_pressure_constraints": [_P, _I32, _P],
    "mpet_get_pressure_multipliers": [_P, _P],
    "mpet_set_batch": [_P, _I32, _P],
    "mpet_get_batch_relres": [_P, _P],
    "mpet_get_facet_data": [_P, _P, _P],
    "mpet_set_facet_data": [_P, _I32, _P],
    "mpet_rhs": [_P, _D, _P, _P],
    "mpet_setup_preconditioner": [_P, _D],
    "mpet_get_amg_info": [_P, _I32, ctypes.POINTER(_I32), _P, _P],
    "mpet_profile_vcycle": [_P, _I32, _I32, ctypes.POINTER(_I32), _P, _P],
    "mpet_solve": [_P, _P, _P, ctypes.POINTER(MpetStats)],
    "mpet_get_prec_info": [_P, ctypes.POINTER(_I32)],
    "mpet_get_setup_timing": [_P, _P],
    "mpet_step": [_P, _D, _P, _P, ctypes.POINTER(MpetStats)],
    "mpet_apply_preconditioner": [_P, _I32, _P, _P],
    "mpet_residual": [_P, _P, _P, _P, _P],
    "mpet_residual_noalloc": [_P, _P, _P, _P, _P],
    "mpet_spmv": [_P, _I32, _P, _P],
    "mpet_apply_symmetric": [_P, _P, _P],
    "mpet_get_spmv_tuning": [_P, _P, ctypes.POINTER(_I32)],
    "mpet_get_spmv_tuning_fp64": [_P, _P, ctypes.POINTER(_I32)],
    "mpet_set_spmv_variant": [_P, _I32],
    "mpet_set_hierarchy_spmv_variant": [_P, _I32],
    "mpet_set_wait_limit": [_P, _I32],
    "mpet_set_batch_skip": [_P, _I32],
    "mpet_set_amg_setup": [_P, _I32],
    "mpet_get_amg_setup_phases": [_P, _P],
    "mpet_get_amg_variants": [_P, _I32, _P, _P, _P],
    "mpet_get_amg_matrix": [_P, _I32, _I32, _I32, _P, _P, _P, _P, _P, _P],
    "mpet_set_element_kernel": [_P, _I32],
    "mpet_set_prec_matrix_free": [_P, _I32],
    "mpet_get_prec_matrix_free": [_P, ctypes.POINTER(_I32), _P],
    "mpet_get_node_block_info": [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
    "mpet_get_timing": [_P, ctypes.POINTER(_D), ctypes.POINTER(_I64), ctypes.POINTER(_D), ctypes.POINTER(_I64)],
    "mpet_pressure_misfit": [_P, _P, _P, ctypes.POINTER(_D), _P],
    "mpet_error_indicators": [_P, _D, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P, ctypes.POINTER(_D)],
    "mpet_adjoint_rhs": [_P, _D, _P, _P],
    "mpet_adjoint_step": [_P, _D, _P, _P, _P, _P, _P, ctypes.POINTER(MpetStats)],
}


def load(path=LIB_PATH):
    """Load libmpetgpu.so and declare argument types; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libmpetgpu.so not built at %s; run waterscapes_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name == "mpet_last_error" else ctypes.c_int
    _lib = lib
    return lib


def _ptr(a):
    """Raw address of a torch tensor, numpy array or None."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    if hasattr(a, "ctypes"):
        return ctypes.c_void_p(a.ctypes.data)
    return ctypes.c_void_p(int(a))


class Context:
    """Owning handle of one ``mpet_ctx``."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.mpet_ctx_create(int(device), ctypes.byref(h))
        if rc != MPET_OK:
            raise MpetError(rc, "mpet_ctx_create failed (no CUDA device %d?)" % device)
        self.h = h

    def check(self, rc):
        if rc != MPET_OK:
            msg = self.lib.mpet_last_error(self.h)
            raise MpetError(rc, msg.decode() if msg else "")
        return rc

    def call(self, name, *args):
        return self.check(getattr(self.lib, name)(self.h, *args))

    def close(self):
        if getattr(self, "h", None):
            self.lib.mpet_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
