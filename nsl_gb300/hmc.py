"""Hybrid Monte Carlo over the GPU leapfrog (src/NSL/MarkovChain/HMC.tpp, markovState.tpp).

HMC(integrator, action, seed).generate_(state) follows HMC.tpp:186-241: momenta p ~ N(0, 1) (real), proposal
(q', p') from the integrator, S(q') from the action, H = S + 1/2 sum p^2, acceptance probability
exp(Re(H0 - H1)), accept when a uniform draw is <= it. The action, the trajectory and the kinetic sums run in
libnslgpu (FP64); only the random draws and the accept decision are host logic. Random numbers come from a seeded
numpy Generator (the reference draws from torch's global generator, so chains agree in distribution, not bitwise).
generate(state_or_config, Nconf, saveFrequency, chain="all"|"last") mirrors HMC.tpp:57-155 without the HDF5 output.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import tensor as T
from .configuration import Configuration


@dataclasses.dataclass
class MarkovState:
    """src/NSL/MarkovChain/markovState.tpp:13-85."""

    configuration: Configuration
    actionValue: complex
    acceptanceProbability: float = 1.0
    markovTime: int = 1
    accepted: bool = True
    weights: dict = dataclasses.field(default_factory=dict)


def getAcceptanceRate(chain) -> float:
    """markovState.tpp:88-96."""
    return float(sum(1.0 for s in chain if s.accepted)) / max(len(chain), 1)


class HMC:
    def __init__(self, integrator, action, seed: int | None = None):
        self.integrator_ = integrator
        self.action_ = action
        self.rng = np.random.default_rng(seed)
        self.last_deltaH = None

    def _kinetic(self, p) -> complex:
        # 1/2 sum p^2 on the device (nslg_kinetic) through the action's handle
        from . import _lib

        mask, fm, ut = self.action_._mask_and_fm()
        p = T.as_c128(p)
        fm = self.action_._fm_for(fm, p)
        out = _lib.c128()
        import ctypes as C

        with T.stream_order(fm.ctx, p):
            _lib.check(_lib.load().nslg_kinetic(fm.handle, T.ptr(p), C.byref(out)))
        return complex(out.re, out.im)

    def generate_(self, state: MarkovState) -> MarkovState:
        """HMC.tpp:186-241."""
        key = self.action_._key
        q0 = state.configuration[key]
        shape = tuple(q0.shape)
        p0 = self.rng.standard_normal(shape) + 0j
        if T.is_torch(q0):
            import torch

            p0 = torch.from_numpy(p0).to(q0.device)
        q1, p1 = self.integrator_(Configuration({key: q0}), Configuration({key: p0}))
        S1 = self.action_(q1)
        H0 = state.actionValue + self._kinetic(p0)
        H1 = S1 + self._kinetic(p1[key])
        dH = H1 - H0
        self.last_deltaH = dH
        acc = float(np.exp(min(700.0, (H0 - H1).real)))
        if self.rng.random() <= acc:
            return MarkovState(q1, S1, acc, state.markovTime + 1, True)
        return MarkovState(state.configuration, state.actionValue, acc, state.markovTime + 1, False)

    def generate(self, start, Nconf: int, saveFrequency: int = 1, chain: str = "all"):
        """HMC.tpp:57-180 (chain="all": Nconf states, saveFrequency-1 skipped between them; "last": final state)."""
        if not isinstance(start, MarkovState):
            cfg = Configuration(start)
            start = MarkovState(cfg, self.action_(cfg), 1.0, 1, True)
        saveFrequency = max(1, int(saveFrequency))
        if chain == "last":
            s = start
            for _ in range(1, Nconf * saveFrequency):
                s = self.generate_(s)
            return s
        mc = [start]
        for _ in range(1, Nconf):
            s = mc[-1]
            for _ in range(saveFrequency - 1):
                s = self.generate_(s)
            mc.append(self.generate_(s))
        return mc
