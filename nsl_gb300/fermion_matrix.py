"""HubbardExp: the exponential-discretisation fermion matrix on the GPU.

Python mirror of NSL::FermionMatrix::HubbardExp (src/NSL/FermionMatrix/Impl/hubbardExp.{hpp,tpp}) over the C ABI:
same constructor arguments (lattice, Nt, beta, mu[, species]), populate(phi[, species]), M / Mdagger / MMdagger /
MdaggerM on vectors of shape (..., Nt, Nx) (leading batch dims allowed, hubbardExp.hpp:148-170), species().
Every application runs in libnslgpu; there is no host fallback.
"""
from __future__ import annotations

import ctypes as C
import sys
import enum

import numpy as np

from . import _lib
from . import tensor as T
from .context import Context, default_context


class Species(enum.IntEnum):
    """NSL::Hubbard::Species (src/NSL/Action/Implementations/hubbard.tpp:7)."""

    Particle = 0
    Hole = 1


class MatrixCombination(enum.IntEnum):
    """NSL::FermionMatrix::MatrixCombination (src/NSL/LinAlg/Solver/applicationType.tpp:18)."""

    M = 0
    Mdagger = 1
    MMdagger = 2
    MdaggerM = 3


_PREC = {"fp64": _lib.PREC_FP64, "fp32": _lib.PREC_FP32, "tf32x3": _lib.PREC_TF32X3,
         "bf16split": _lib.PREC_BF16_SPLIT}


def precision_code(p) -> int:
    if isinstance(p, int):
        return p
    try:
        return _PREC[p]
    except KeyError:
        raise ValueError(f"unknown precision {p!r}; expected one of {sorted(_PREC)}") from None


class HubbardExp:
    """M_{tx,iy} = delta_ti delta_xy - [exp(delta K)]_xy exp(i phi_iy) B_t delta_{t,i+1}, B_0 = -1."""

    _kind = 0  # nslg_fm_kind: NSLG_FM_EXP

    def __init__(self, lattice, Nt: int, beta: complex = 1.0, mu: complex = 0.0,
                 species: Species = Species.Particle, ctx: Context | None = None):
        self.Lat = lattice
        self.Nt = int(Nt)
        self.Nx = int(lattice.sites())
        self.beta = complex(beta)
        self.mu = complex(mu)
        self.delta = self.beta / self.Nt
        self.ctx = ctx or default_context()
        self._species = Species(species)
        lib = _lib.load()
        h = C.c_void_p()
        hops = np.ascontiguousarray(lattice.hopping_matrix(1.0), dtype=np.complex128)
        _lib.check(lib.nslg_fm_create_kind(self.ctx.handle, self._kind, self.Nx, self.Nt, hops.ctypes.data,
                                           _lib.c128.of(self.beta), _lib.c128.of(self.mu), int(self._species),
                                           C.byref(h)))
        self.handle = h
        # exp(delta K) entries the lattice already holds (e.g. installed from the reference memo) are reused
        if self._kind == _lib.FM_EXP:
            for d, E in getattr(lattice, "_exp_memo", {}).items():
                self.set_exp_hopping_matrix(d, E)
        self.phi_ = None

    @classmethod
    def from_params(cls, lattice, params: dict, species: Species = Species.Particle, ctx=None):
        """HubbardExp(lattice, params) / HubbardExp(species, lattice, params) (hubbardExp.hpp:78-84)."""
        return cls(lattice, int(params["Nt"]), params.get("beta", 1.0), params.get("mu", 0.0), species, ctx)

    def __del__(self):
        if sys.is_finalizing():  # the CUDA runtime may already be torn down; the OS reclaims everything
            return
        try:
            if getattr(self, "handle", None):
                _lib.load().nslg_fm_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    # ---- lattice data -----------------------------------------------------------------------------------------
    def exp_hopping_matrix(self, delta: complex) -> np.ndarray:
        out = np.empty((self.Nx, self.Nx), dtype=np.complex128)
        _lib.check(_lib.load().nslg_fm_get_exp_hopping(self.handle, _lib.c128.of(delta), out.ctypes.data))
        return out

    def set_exp_hopping_matrix(self, delta: complex, expK):
        E = T.as_c128(expK)
        with T.stream_order(self.ctx, E):
            _lib.check(_lib.load().nslg_fm_set_exp_hopping(self.handle, _lib.c128.of(delta), T.ptr(E)))

    # ---- configuration ----------------------------------------------------------------------------------------
    def species(self) -> Species:
        return self._species

    def populate(self, phi, species: Species | None = None):
        """hubbardExp.hpp:103-128: phiExp = exp(i sgn phi + sgn mu_tilde) on the device."""
        phi = T.as_c128(phi)
        if tuple(phi.shape) != (self.Nt, self.Nx):
            raise ValueError(f"phi must have shape (Nt, Nx) = {(self.Nt, self.Nx)}, got {tuple(phi.shape)}")
        if species is not None:
            self._species = Species(species)
        with T.stream_order(self.ctx, phi):
            _lib.check(_lib.load().nslg_fm_populate(self.handle, T.ptr(phi), -1 if species is None
                                                    else int(self._species)))
        self.phi_ = phi

    def phases(self) -> np.ndarray:
        """phiExp (Nt, Nx) of the populated configuration, as the device holds it (nslg_fm_get_phases)."""
        out = np.empty((self.Nt, self.Nx), dtype=np.complex128)
        _lib.check(_lib.load().nslg_fm_get_phases(self.handle, out.ctypes.data))
        return out

    # ---- operators --------------------------------------------------------------------------------------------
    def _apply(self, op: int, psi, precision="fp64"):
        psi = T.as_c128(psi)
        shape = tuple(psi.shape)
        if len(shape) < 2 or shape[-2:] != (self.Nt, self.Nx):
            raise ValueError(f"psi must have shape (..., Nt, Nx) = (..., {self.Nt}, {self.Nx}), got {shape}")
        nbatch = T.numel(shape[:-2])
        out = T.empty_like(psi)
        with T.stream_order(self.ctx, psi, out):
            _lib.check(_lib.load().nslg_fm_apply(self.handle, op, T.ptr(psi), T.ptr(out), nbatch,
                                                 precision_code(precision)))
        return out

    def M(self, psi, precision="fp64"):
        """hubbardExp.tpp:39-41."""
        return self._apply(_lib.OP_M, psi, precision)

    def Mdagger(self, psi, precision="fp64"):
        """hubbardExp.tpp:44-75."""
        return self._apply(_lib.OP_MDAGGER, psi, precision)

    def MMdagger(self, psi, precision="fp64"):
        """hubbardExp.tpp:78-104, evaluated as M (M^dagger psi): two fused products instead of four."""
        return self._apply(_lib.OP_MMDAGGER, psi, precision)

    def MdaggerM(self, psi, precision="fp64"):
        """hubbardExp.tpp:107-125, evaluated as M^dagger (M psi)."""
        return self._apply(_lib.OP_MDAGGERM, psi, precision)

    def apply(self, combination: MatrixCombination, psi, precision="fp64"):
        return self._apply(int(combination), psi, precision)

    def apply_dd(self, combination: MatrixCombination, psi_hi, psi_lo=None):
        """(hi, lo) = combination (psi_hi + psi_lo) in double-double arithmetic (nslg_fm_apply_dd), the residual
        evaluation behind CG's "true_residual_dd" rule."""
        psi_hi = T.as_c128(psi_hi)
        shape = tuple(psi_hi.shape)
        if len(shape) < 2 or shape[-2:] != (self.Nt, self.Nx):
            raise ValueError(f"psi must have shape (..., Nt, Nx) = (..., {self.Nt}, {self.Nx}), got {shape}")
        lo = None if psi_lo is None else T.as_c128(psi_lo)
        oh, ol = T.empty_like(psi_hi), T.empty_like(psi_hi)
        tensors = [psi_hi, oh, ol] + ([lo] if lo is not None else [])
        with T.stream_order(self.ctx, *tensors):
            _lib.check(_lib.load().nslg_fm_apply_dd(self.handle, int(combination), T.ptr(psi_hi),
                                                    None if lo is None else T.ptr(lo), T.ptr(oh), T.ptr(ol),
                                                    T.numel(shape[:-2])))
        return oh, ol

    def set_force_precision(self, precision="fp64"):
        """Arithmetic of gradLogDetM (and so of the action force and leapfrog): "fp64" (default) or "bf16split"
        (the two matrix chains on the tensor cores, FP64-class; the LU and logDetM stay FP64)."""
        _lib.check(_lib.load().nslg_fm_set_force_precision(self.handle, precision_code(precision)))
        self.force_precision = precision

    _STAB = {"auto": 0, "plain": 1, "stratified": 2}

    def set_stabilisation(self, mode="auto"):
        """Form of logDetM / gradLogDetM: "plain" (the reference's single product of the time slices), "stratified"
        (U D T factorised chunk products, stable at any beta) or "auto" (stratified when beta * rho > 14, rho the
        largest |eigenvalue| bound of K)."""
        if mode not in self._STAB:
            raise ValueError(f"stabilisation must be one of {sorted(self._STAB)}")
        _lib.check(_lib.load().nslg_fm_set_stabilisation(self.handle, self._STAB[mode]))
        self.stabilisation = mode

    # ---- determinant ------------------------------------------------------------------------------------------
    def logDetM(self) -> complex:
        """hubbardExp.tpp:129-150 (principal branch; finite where the reference's det overflows)."""
        out = _lib.c128()
        _lib.check(_lib.load().nslg_fm_logdet(self.handle, C.byref(out)))
        return complex(out.re, out.im)

    def gradLogDetM(self):
        """hubbardExp.tpp:153-211: d log det M / d phi, shape (Nt, Nx), in the kind of the populated phi."""
        ref = self.phi_ if self.phi_ is not None else np.empty(0)
        out = T.empty_like(ref, (self.Nt, self.Nx))
        with T.stream_order(self.ctx, out):
            _lib.check(_lib.load().nslg_fm_grad_logdet(self.handle, T.ptr(out)))
        return out


class HubbardDiag(HubbardExp):
    """NSL::FermionMatrix::HubbardDiag (src/NSL/FermionMatrix/Impl/hubbardDiag.{hpp,tpp}), the diagonal
    discretisation: (M psi)_t = psi_t - sgn delta K psi_t - B_t exp(i sgn phi_{t-1} + sgn mu~) psi_{t-1}, B_0 = -1.

    Same constructor and methods as HubbardExp. Operators run in FP64 or FP32 ("fp64" / "fp32"); MMdagger and
    MdaggerM are the compositions M (M^dagger psi) and M^dagger (M psi) (equal to the reference's expanded forms);
    logDetM = i sgn sum(phi) + log det(1 + fk_0 ... fk_{Nt-1}), fk_t = (1 - sgn delta K) diag(phiExpInv[t+1]),
    with the second term on the principal branch and the first added as is (hubbardDiag.tpp:169-193). The reference
    writes its operators for one (Nt, Nx) vector; leading batch dimensions here are independent vectors.
    """

    _kind = 1  # nslg_fm_kind: NSLG_FM_DIAG

    def M(self, psi, precision="fp64"):
        """hubbardDiag.tpp:10-37."""
        return self._apply(_lib.OP_M, psi, precision)

    def Mdagger(self, psi, precision="fp64"):
        """hubbardDiag.tpp:40-71."""
        return self._apply(_lib.OP_MDAGGER, psi, precision)

    def MMdagger(self, psi, precision="fp64"):
        """hubbardDiag.tpp:74-118, evaluated as M (M^dagger psi)."""
        return self._apply(_lib.OP_MMDAGGER, psi, precision)

    def MdaggerM(self, psi, precision="fp64"):
        """hubbardDiag.tpp:121-165, evaluated as M^dagger (M psi)."""
        return self._apply(_lib.OP_MDAGGERM, psi, precision)

    def logDetM(self) -> complex:
        """hubbardDiag.tpp:169-193."""
        return super().logDetM()

    def gradLogDetM(self):
        """hubbardDiag.tpp:197-250."""
        return super().gradLogDetM()
