"""ctypes binding of libnslgpu.so (the C ABI declared in include/nsl_gb300.h).

The library is built in-tree by ``nsl_gb300.build`` (``__graft_entry__.build()``). There is no CPU fallback: if the
library or a CUDA device is missing, every operation raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnslgpu.so")

# status codes (nslg_status)
OK, ERR_ARG, ERR_SHAPE, ERR_OOM, ERR_CUDA, NOT_CONVERGED, ERR_UNSUPPORTED, ERR_STATE = 0, 1, 2, 3, 4, 5, 7, 8
# operators (MatrixCombination order)
OP_M, OP_MDAGGER, OP_MMDAGGER, OP_MDAGGERM = 0, 1, 2, 3
PARTICLE, HOLE = 0, 1
FM_EXP, FM_DIAG = 0, 1
PREC_FP64, PREC_FP32, PREC_TF32X3, PREC_BF16_SPLIT = 0, 1, 2, 3
CG_SHARED, CG_PER_RHS = 0, 1
TERM_GAUGE, TERM_FERMION = 1, 2
STOP_RECURRENCE, STOP_TRUE_RESIDUAL, STOP_TRUE_RESIDUAL_DD = 0, 1, 2
NOALLOC_MAX_ELEMS = 2097152  # scratch of nslg_fm_apply_noalloc, complex128 values
TB_NCHANNELS = 12  # nslg_twobody_channel


class c128(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]

    @staticmethod
    def of(z) -> "c128":
        z = complex(z)
        return c128(z.real, z.imag)


class CgStats(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("reliable_updates", C.c_int64), ("converged", C.c_int64),
                ("systems", C.c_int64), ("recurrence_residual", C.c_double), ("true_residual", C.c_double),
                ("escalated", C.c_int64), ("dd_rebases", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class NslgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"nslg error {code}: {msg}")
        self.code = code


_P = C.c_void_p
_I64 = C.c_int64

# name: (restype, argtypes)
SIGNATURES = {
    "nslg_version": (C.c_int, []),
    "nslg_last_error": (C.c_char_p, []),
    "nslg_kernel_launches": (C.c_uint64, []),
    "nslg_ctx_create": (C.c_int, [C.c_int, _P, C.POINTER(_P)]),
    "nslg_ctx_destroy": (C.c_int, [_P]),
    "nslg_ctx_synchronize": (C.c_int, [_P]),
    "nslg_ctx_stream": (_P, [_P]),
    "nslg_fm_create": (C.c_int, [_P, _I64, _I64, _P, c128, c128, C.c_int, C.POINTER(_P)]),
    "nslg_fm_create_kind": (C.c_int, [_P, C.c_int, _I64, _I64, _P, c128, c128, C.c_int, C.POINTER(_P)]),
    "nslg_fm_destroy": (C.c_int, [_P]),
    "nslg_fm_set_exp_hopping": (C.c_int, [_P, c128, _P]),
    "nslg_fm_get_exp_hopping": (C.c_int, [_P, c128, _P]),
    "nslg_fm_populate": (C.c_int, [_P, _P, C.c_int]),
    "nslg_fm_get_phases": (C.c_int, [_P, _P]),
    "nslg_fm_apply": (C.c_int, [_P, C.c_int, _P, _P, _I64, C.c_int]),
    "nslg_fm_apply_noalloc": (C.c_int, [_P, C.c_int, _P, _P, _I64, C.c_int]),
    "nslg_fm_apply_dd": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _I64]),
    "nslg_fm_set_force_precision": (C.c_int, [_P, C.c_int]),
    "nslg_fm_set_stabilisation": (C.c_int, [_P, C.c_int]),
    "nslg_fm_logdet": (C.c_int, [_P, C.POINTER(c128)]),
    "nslg_fm_grad_logdet": (C.c_int, [_P, _P]),
    "nslg_hubbard_eval": (C.c_int, [_P, _P, c128, C.c_int, C.POINTER(c128)]),
    "nslg_hubbard_force": (C.c_int, [_P, _P, c128, C.c_int, C.c_int, _P]),
    "nslg_leapfrog": (C.c_int, [_P, _P, _P, _P, _P, c128, C.c_double, _I64, C.c_int, C.c_int, C.c_int]),
    "nslg_kinetic": (C.c_int, [_P, _P, C.POINTER(c128)]),
    "nslg_leapfrog_batch": (C.c_int, [_P, _I64, _P, _P, _P, _P, c128, C.c_double, _I64, C.c_int, C.c_int, C.c_int]),
    "nslg_hubbard_eval_batch": (C.c_int, [_P, _I64, _P, c128, C.c_int, _P]),
    "nslg_hubbard_eval_batch_u": (C.c_int, [_P, _I64, _P, _P, C.c_int, _P]),
    "nslg_leapfrog_group": (C.c_int, [C.c_int, _P, _P, _P, _P, _P, _P, _P, C.c_double, _I64, C.c_int, C.c_int,
                                      C.c_int]),
    "nslg_kinetic_batch": (C.c_int, [_P, _I64, _P, _P]),
    "nslg_accept_batch": (C.c_int, [_P, _I64, _P, _P, _P]),
    "nslg_cg_solve": (C.c_int, [_P, C.c_int, _P, _P, _P, _I64, C.c_double, _I64, C.c_int, C.c_int, C.c_int,
                                C.POINTER(CgStats)]),
    "nslg_cg_solve_dd": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _I64, C.c_double, _I64, C.c_int, C.c_int,
                                   C.POINTER(CgStats)]),
    "nslg_cg_solve_group": (C.c_int, [C.c_int, _P, C.c_int, _P, _P, _P, _P, _P, _P, _I64, C.c_int, C.c_int, _P]),
    "nslg_twobody_measure": (C.c_int, [_P, _P, _P, _I64, _I64, _P, _I64, _I64, C.c_double, _I64, C.c_int, _P,
                                       C.POINTER(CgStats)]),
}

_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Loads libnslgpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(f"libnslgpu.so is not built ({path}); run __graft_entry__.build()")
            lib = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
    return _lib


def check(code: int, allow=(OK,)):
    if code not in allow:
        msg = load().nslg_last_error()
        raise NslgError(code, msg.decode() if msg else "")
    return code
