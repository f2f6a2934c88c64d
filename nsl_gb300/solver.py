"""CG on the fermion operators, on the GPU.

Mirror of NSL::LinAlg::CG (src/NSL/LinAlg/Solver/Impl/CG.{hpp,tpp}): CG(M, matrixCombination=M, eps=1e-12,
maxIter=10000) and __call__(b[, x0]) -> x. The defaults reproduce the reference exactly: x0 = b, the recurrence
stopping rule |r|^2 <= eps^2, alpha/beta shared by the whole batch (mode="shared"), FP64, and on exhaustion the last
iterate is returned after an error is logged (CG.tpp:90-93). mode="per_rhs" solves every right-hand side as its own
system. stop="true_residual" recomputes r = b - A x in FP64 whenever the recurrence residual has dropped below its
running maximum by 1e4 (FP64-class operators) or 100 (FP32-class operators) (reliable updates) and stops on
|b - A x| <= eps; precision="fp32" evaluates the operator in FP32 (vectors stay FP64) and always uses that rule.
stop="true_residual_dd" goes below FP64's floor (~1e-16 |A| |x|): the solution is a double-double pair x + x_lo,
rebased with double-double residuals b - A (x + x_lo) (nslg_cg_solve_dd); the call returns x and keeps the low part
in `x_lo_`.
"""
from __future__ import annotations

import ctypes as C
import logging

from . import _lib
from . import tensor as T
from .fermion_matrix import HubbardExp, MatrixCombination, precision_code

log = logging.getLogger("nsl_gb300")

_MODES = {"shared": _lib.CG_SHARED, "per_rhs": _lib.CG_PER_RHS}
_STOPS = {"recurrence": _lib.STOP_RECURRENCE, "true_residual": _lib.STOP_TRUE_RESIDUAL,
          "true_residual_dd": _lib.STOP_TRUE_RESIDUAL_DD}


class CG:
    def __init__(self, M: HubbardExp, matrixCombination: MatrixCombination = MatrixCombination.M,
                 eps: float = 1e-12, maxIter: int = 10000, *, mode: str = "shared", precision="fp64",
                 stop: str | None = None):
        if not isinstance(M, HubbardExp):
            raise TypeError("CG on the GPU takes a HubbardExp fermion matrix (operators given as Python callables "
                            "have no device implementation)")
        if mode not in _MODES:
            raise ValueError(f"mode must be one of {sorted(_MODES)}")
        self.M_ = M
        self.op = int(MatrixCombination(matrixCombination))
        self.eps = float(eps)
        self.maxIter = int(maxIter)
        self.mode = mode
        self.precision = precision_code(precision)
        if stop is None:
            stop = "recurrence" if self.precision == _lib.PREC_FP64 else "true_residual"
        if stop not in _STOPS:
            raise ValueError(f"stop must be one of {sorted(_STOPS)}")
        self.stop = stop
        self.stats = None

    def __call__(self, b, x0=None):
        M = self.M_
        b = T.as_c128(b)
        shape = tuple(b.shape)
        if len(shape) < 2 or shape[-2:] != (M.Nt, M.Nx):
            raise ValueError(f"b must have shape (..., Nt, Nx) = (..., {M.Nt}, {M.Nx}), got {shape}")
        nbatch = T.numel(shape[:-2])
        x = T.empty_like(b)
        x0p = None
        if x0 is not None:
            x0 = T.as_c128(x0)
            if tuple(x0.shape) != shape:
                raise ValueError("x0 must have the shape of b")
            x0p = T.ptr(x0)
        st = _lib.CgStats()
        if self.stop == "true_residual_dd":
            self.x_lo_ = T.empty_like(b)
            with T.stream_order(M.ctx, b, x, self.x_lo_, *([x0] if x0 is not None else [])):
                rc = _lib.load().nslg_cg_solve_dd(M.handle, self.op, T.ptr(b), x0p, T.ptr(x), T.ptr(self.x_lo_),
                                                  nbatch, self.eps, self.maxIter, _MODES[self.mode], self.precision,
                                                  C.byref(st))
        else:
            with T.stream_order(M.ctx, b, x, *([x0] if x0 is not None else [])):
                rc = _lib.load().nslg_cg_solve(M.handle, self.op, T.ptr(b), x0p, T.ptr(x), nbatch, self.eps,
                                               self.maxIter, _MODES[self.mode], self.precision, _STOPS[self.stop],
                                               C.byref(st))
        _lib.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
        self.stats = st.as_dict()
        if rc == _lib.NOT_CONVERGED:
            log.error("Error CG did not converge within %d iterations! |r| = %g", self.maxIter,
                      st.recurrence_residual)
        else:
            log.info("CG Converged with precision: %g < %g after %d steps", st.recurrence_residual, self.eps,
                     st.iterations)
        return x


def cg_group(items, matrixCombination: MatrixCombination = MatrixCombination.MMdagger, eps=1e-12, maxIter=10000,
             precision="fp64", stop="true_residual"):
    """Independent CG solves on several fermion matrices of different sizes at once (nslg_cg_solve_group): every
    right-hand side of every instance is its own system; the iteration's vector kernels run once for all of them.

    items: a list of (HubbardExp, b) or (HubbardExp, b, x0), b of shape (..., Nt, Nx) for its matrix; eps: an absolute
    tolerance per item (a list) or one for all. Returns (xs, x_los, stats): the solutions in the kind of each b, the
    low parts under stop="true_residual_dd" (else None) and each instance's statistics. No counterpart in the
    reference (one CG per object, CG.tpp:15-113)."""
    lib = _lib.load()
    n = len(items)
    if n == 0:
        return [], [], []
    eps = list(eps) if isinstance(eps, (list, tuple)) else [float(eps)] * n
    fms, bs, x0s, xs, los, nb = [], [], [], [], [], []
    for it in items:
        M, b = it[0], T.as_c128(it[1])
        x0 = T.as_c128(it[2]) if len(it) > 2 and it[2] is not None else None
        shape = tuple(b.shape)
        if len(shape) < 2 or shape[-2:] != (M.Nt, M.Nx):
            raise ValueError(f"b must have shape (..., Nt, Nx) = (..., {M.Nt}, {M.Nx}), got {shape}")
        fms.append(M)
        bs.append(b)
        x0s.append(x0)
        xs.append(T.empty_like(b))
        los.append(T.empty_like(b) if stop == "true_residual_dd" else None)
        nb.append(T.numel(shape[:-2]))
    P = C.c_void_p * n
    st = (_lib.CgStats * n)()
    tensors = [t for t in bs + xs + los + x0s if t is not None]
    with T.stream_order(fms[0].ctx, *tensors):
        rc = lib.nslg_cg_solve_group(
            n, P(*[m.handle.value for m in fms]), int(MatrixCombination(matrixCombination)),
            P(*[T.ptr(b) for b in bs]), P(*[T.ptr(x) if x is not None else None for x in x0s]),
            P(*[T.ptr(x) for x in xs]), P(*[T.ptr(x) if x is not None else None for x in los]),
            (C.c_int64 * n)(*nb), (C.c_double * n)(*[float(e) for e in eps]), int(maxIter), precision_code(precision),
            _STOPS[stop], st)
    _lib.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
    stats = [st[i].as_dict() for i in range(n)]
    if rc == _lib.NOT_CONVERGED:
        log.error("Error CG (group) did not converge within %d iterations", maxIter)
    return xs, (los if stop == "true_residual_dd" else None), stats
