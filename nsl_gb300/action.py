"""Hubbard actions on the GPU.

Mirrors NSL::Action: HubbardGaugeAction (src/NSL/Action/Implementations/hubbardGaugeAction.tpp), HubbardFermionAction
(hubbardFermiAction.tpp) and the term sum Action<...> built with + (src/NSL/Action/action.tpp:72-167). eval / grad /
force take a Configuration ({"phi": phi}) or the field itself and run in libnslgpu.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import tensor as T
from .configuration import Configuration
from .fermion_matrix import HubbardExp


def tilde(params: dict, key: str) -> complex:
    """NSL::Hubbard::tilde (hubbard.tpp:9-19): delta * params[key], delta = beta / Nt."""
    delta = params.get("delta", complex(params["beta"]) / int(params["Nt"]))
    return complex(delta) * complex(params[key])


class _Term:
    terms = 0

    def __init__(self, params: dict, fieldName: str = "phi"):
        self.params = dict(params)
        self.configKey_ = fieldName
        self.Utilde = tilde(self.params, "U") if "U" in self.params else 1.0

    def _field(self, x):
        return x[self.configKey_] if isinstance(x, dict) else x

    def __add__(self, other):
        return Action(self) + other

    def eval(self, phi):
        return Action(self).eval(phi)

    def force(self, phi):
        return Action(self).force(phi)

    def grad(self, phi):
        return Action(self).grad(phi)

    __call__ = eval


class HubbardGaugeAction(_Term):
    """S = sum phi^2 / (2 U~), force = -phi / U~ (hubbardGaugeAction.tpp:55-67)."""

    terms = _lib.TERM_GAUGE


class HubbardFermionAction(_Term):
    """S = -(log det M_P + log det M_H), force = -(grad_P - grad_H) (hubbardFermiAction.tpp:68-113).

    FermionMatrixType is the reference's template argument (hubbardFermiAction.tpp:26-29): HubbardExp (default) or
    HubbardDiag."""

    terms = _lib.TERM_FERMION

    def __init__(self, lattice, params: dict, fieldName: str = "phi", ctx=None, FermionMatrixType=HubbardExp,
                 force_precision: str = "fp64", stabilisation: str = "auto"):
        super().__init__(params, fieldName)
        self.hfm_ = FermionMatrixType(lattice, int(params["Nt"]), params.get("beta", 1.0), params.get("mu", 0.0),
                                      ctx=ctx)
        if force_precision != "fp64":  # "bf16split": the log-det gradient on the tensor cores (action value FP64)
            self.hfm_.set_force_precision(force_precision)
        if stabilisation != "auto":  # "plain" / "stratified" form of log det and its gradient
            self.hfm_.set_stabilisation(stabilisation)


class Action:
    """Sum of Hubbard action terms acting on one field (action.tpp:72-143)."""

    def __init__(self, *summands):
        self.summands_ = list(summands)

    def __add__(self, other):
        return Action(*(self.summands_ + (other.summands_ if isinstance(other, Action) else [other])))

    @property
    def _key(self):
        return self.summands_[0].configKey_

    def _mask_and_fm(self):
        mask = 0
        fm = None
        ut = None
        for s in self.summands_:
            if not isinstance(s, (HubbardGaugeAction, HubbardFermionAction)):
                raise TypeError(f"unsupported action term {type(s).__name__}")
            if s.terms & mask:
                raise ValueError("each Hubbard term may appear once")
            mask |= s.terms
            if isinstance(s, HubbardFermionAction):
                fm = s.hfm_
            if isinstance(s, HubbardGaugeAction):
                ut = s.Utilde
        return mask, fm, (ut if ut is not None else 1.0)

    def eval(self, config) -> complex:
        phi = T.as_c128(config[self._key] if isinstance(config, dict) else config)
        mask, fm, ut = self._mask_and_fm()
        fm = self._fm_for(fm, phi)
        out = _lib.c128()
        with T.stream_order(fm.ctx, phi):
            _lib.check(_lib.load().nslg_hubbard_eval(fm.handle, T.ptr(phi), _lib.c128.of(ut), mask, C.byref(out)))
        return complex(out.re, out.im)

    __call__ = eval

    def eval_batch(self, configs) -> np.ndarray:
        """The action of every configuration of a batch phi (nconf, Nt, Nx) in one call (nslg_hubbard_eval_batch:
        one reduction and one batched log det for all configurations and both species)."""
        phi = T.as_c128(configs[self._key] if isinstance(configs, dict) else configs)
        mask, fm, ut = self._mask_and_fm()
        fm = self._fm_for(fm, phi)
        nconf = int(phi.shape[0]) if phi.ndim == 3 else 1
        out = (_lib.c128 * nconf)()
        with T.stream_order(fm.ctx, phi):
            _lib.check(_lib.load().nslg_hubbard_eval_batch(fm.handle, nconf, T.ptr(phi), _lib.c128.of(ut), mask, out))
        return np.array([complex(v.re, v.im) for v in out])

    def force(self, config, real_force: bool = False) -> Configuration:
        phi = T.as_c128(config[self._key] if isinstance(config, dict) else config)
        mask, fm, ut = self._mask_and_fm()
        fm = self._fm_for(fm, phi)
        out = T.empty_like(phi)
        with T.stream_order(fm.ctx, phi, out):
            _lib.check(_lib.load().nslg_hubbard_force(fm.handle, T.ptr(phi), _lib.c128.of(ut), mask,
                                                      int(real_force), T.ptr(out)))
        return Configuration({self._key: out})

    def grad(self, config) -> Configuration:
        f = self.force(config)
        return Configuration({k: -v for k, v in f.items()})

    def _fm_for(self, fm, phi):
        """The handle that evaluates the terms on a field of phi's shape. A gauge-only action has no fermion matrix;
        it gets a device handle over an empty lattice of the field's shape (only its buffers are used)."""
        if fm is None:
            from .lattice import SpatialLattice

            key = tuple(phi.shape[-2:])
            cached = getattr(self, "_gauge_fm", None)
            if cached is None or (cached.Nt, cached.Nx) != key:
                g = self.summands_[0]
                lat = SpatialLattice("gauge-only", np.zeros((key[1], key[1])), np.zeros((key[1], 1)))
                cached = HubbardExp(lat, key[0], g.params.get("beta", 1.0))
                self._gauge_fm = cached
            return cached
        if tuple(phi.shape[-2:]) != (fm.Nt, fm.Nx) or phi.ndim not in (2, 3):
            raise ValueError(f"field must have shape {(fm.Nt, fm.Nx)} or (nconf, {fm.Nt}, {fm.Nx}), "
                             f"got {tuple(phi.shape)}")
        return fm
