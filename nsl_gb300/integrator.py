"""Leapfrog integrators on the GPU (src/NSL/Integrator/Impl/leapfrog.tpp, leapfrogRealForce.tpp).

Leapfrog(action, trajectoryLength, numberSteps, backward=False)(q, p) -> (q', p'): eps = trajectoryLength/numberSteps
(negated when backward); half kick, numberSteps drifts, numberSteps-1 full kicks, half kick (numberSteps + 1 force
evaluations). The whole trajectory runs in libnslgpu (nslg_leapfrog) with fused kick/drift kernels. A field with a
leading batch dimension (nconf, Nt, Nx) advances nconf independent configurations together (nslg_leapfrog_batch:
their gradients share every launch), each exactly as a single call would.
"""
from __future__ import annotations

from . import _lib
from . import tensor as T
from .configuration import Configuration


class Leapfrog:
    real_force = False

    def __init__(self, action, trajectoryLength: float, numberSteps: int, backward: bool = False):
        from .action import Action

        self.action_ = action if isinstance(action, Action) else Action(action)
        self.trajLength_ = float(trajectoryLength)
        self.numSteps_ = int(numberSteps)
        self.backward = bool(backward)
        self.stepSize_ = self.trajLength_ / self.numSteps_ * (-1 if backward else 1)

    def __call__(self, q, p):
        key = self.action_._key
        q0 = T.as_c128(q[key] if isinstance(q, dict) else q)
        p0 = T.as_c128(p[key] if isinstance(p, dict) else p)
        mask, fm, ut = self.action_._mask_and_fm()
        fm = self.action_._fm_for(fm, q0)
        q1, p1 = T.empty_like(q0), T.empty_like(p0)
        if tuple(p0.shape) != tuple(q0.shape):
            raise ValueError(f"q and p shapes differ: {tuple(q0.shape)} vs {tuple(p0.shape)}")
        with T.stream_order(fm.ctx, q0, p0, q1, p1):
            if q0.ndim == 3:
                _lib.check(_lib.load().nslg_leapfrog_batch(fm.handle, int(q0.shape[0]), T.ptr(q0), T.ptr(p0),
                                                           T.ptr(q1), T.ptr(p1), _lib.c128.of(ut), self.trajLength_,
                                                           self.numSteps_, int(self.backward), int(self.real_force),
                                                           mask))
            else:
                _lib.check(_lib.load().nslg_leapfrog(fm.handle, T.ptr(q0), T.ptr(p0), T.ptr(q1), T.ptr(p1),
                                                     _lib.c128.of(ut), self.trajLength_, self.numSteps_,
                                                     int(self.backward), int(self.real_force), mask))
        return Configuration({key: q1}), Configuration({key: p1})


class LeapfrogRealForce(Leapfrog):
    """Leapfrog on Re F (leapfrogRealForce.tpp:44-70)."""

    real_force = True
