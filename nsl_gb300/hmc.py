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


class HMCChains:
    """nconf independent HMC chains advanced together: one batched trajectory (nslg_leapfrog_batch), one batched
    action evaluation (nslg_hubbard_eval_batch) and one batched kinetic sum (nslg_kinetic_batch) per step for all
    chains; the accept/reject of HMC.tpp:204-226 draws per chain on the host and the accepted fields are selected
    on the device (nslg_accept_batch). No counterpart in the reference, which runs one chain per HMC object; every chain follows
    the same rule as HMC.generate_ (its own momenta, its own uniform draw)."""

    def __init__(self, integrator, action, seed: int | None = None):
        self.integrator_ = integrator
        self.action_ = action
        self.rng = np.random.default_rng(seed)
        self.deltaH = []
        self.accepted = None

    def _handle(self, q):
        mask, fm, ut = self.action_._mask_and_fm()
        return self.action_._fm_for(fm, q)

    def _kinetic(self, p) -> np.ndarray:
        """1/2 sum p^2 (complex square) per chain, on the device (nslg_kinetic_batch)."""
        import ctypes as C

        from . import _lib

        p = T.as_c128(p)
        fm = self._handle(p)
        nconf = int(p.shape[0])
        out = (_lib.c128 * nconf)()
        with T.stream_order(fm.ctx, p):
            _lib.check(_lib.load().nslg_kinetic_batch(fm.handle, nconf, T.ptr(p), out))
        return np.array([complex(v.re, v.im) for v in out])

    def _select(self, acc: np.ndarray, q1, q):
        """q[b] = q1[b] for the accepted chains (nslg_accept_batch on the device; numpy fields on the host)."""
        from . import _lib

        if not T.is_torch(q):
            return np.where(acc[:, None, None], q1, q)
        q = q.clone()
        flags = np.ascontiguousarray(acc, dtype=np.int32)
        fm = self._handle(q)
        with T.stream_order(fm.ctx, q1, q):
            _lib.check(_lib.load().nslg_accept_batch(fm.handle, int(q.shape[0]), flags.ctypes.data, T.ptr(q1),
                                                     T.ptr(q)))
        return q

    def generate(self, phi0, Ntraj: int):
        """Runs Ntraj trajectories on every chain from phi0 (nconf, Nt, Nx); returns the final fields (nconf, Nt, Nx)
        and the per-chain acceptance rates. self.deltaH holds H1 - H0 per step (nconf values each)."""
        key = self.action_._key
        q = T.as_c128(phi0)
        nconf = int(q.shape[0])
        S = self.action_.eval_batch(q)
        acc_count = np.zeros(nconf)
        for _ in range(int(Ntraj)):
            p0 = self.rng.standard_normal(tuple(q.shape)) + 0j
            if T.is_torch(q):
                import torch

                p0 = torch.from_numpy(p0).to(q.device)
            q1c, p1c = self.integrator_(Configuration({key: q}), Configuration({key: p0}))
            q1, p1 = q1c[key], p1c[key]
            S1 = self.action_.eval_batch(q1)
            H0 = S + self._kinetic(p0)
            H1 = S1 + self._kinetic(p1)
            self.deltaH.append(H1 - H0)
            prob = np.exp(np.minimum(700.0, (H0 - H1).real))
            acc = self.rng.random(nconf) <= prob
            acc_count += acc
            q = self._select(acc, q1, q)
            S = np.where(acc, S1, S)
        self.accepted = acc_count
        return q, acc_count / max(int(Ntraj), 1)
