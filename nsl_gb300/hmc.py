"""Hybrid Monte Carlo over the GPU leapfrog (src/NSL/MarkovChain/HMC.tpp, markovState.tpp).

HMC(integrator, action, seed).generate_(state) follows HMC.tpp:186-241: momenta p ~ N(0, 1) (real), proposal
(q', p') from the integrator, S(q') from the action, H = S + 1/2 sum p^2, acceptance probability
exp(Re(H0 - H1)), accept when a uniform draw is <= it. The action, the trajectory and the kinetic sums run in
libnslgpu (FP64); only the random draws and the accept decision are host logic. Random numbers come from a seeded
numpy Generator (the reference draws from torch's global generator, so chains agree in distribution, not bitwise).
generate(state_or_config, Nconf, saveFrequency, chain="all"|"last", store) mirrors HMC.tpp:57-155; with a store
(markov_io.MarkovChainFile) it writes and resumes chains in NSL's H5IO node layout, without HDF5.
"""
from __future__ import annotations

import ctypes as C
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

    def generate(self, start, Nconf: int, saveFrequency: int = 1, chain: str = "all", store=None,
                 baseNode: str = "markovChain"):
        """HMC.tpp:57-180 (chain="all": Nconf states, saveFrequency-1 skipped between them; "last": final state).

        With a store (markov_io.MarkovChainFile, NSL's H5IO node layout) chain="all" follows HMC.tpp:78-120: it
        resumes from the highest-numbered state under baseNode (a state that cannot be read is deleted and the one
        before it is read instead), or writes the start state as state 0, and writes every new state as
        baseNode/n. The returned list has Nconf entries; those before the resumed state are None (the reference
        leaves them default-constructed)."""
        if not isinstance(start, MarkovState):
            cfg = Configuration(start)
            start = MarkovState(cfg, self.action_(cfg), 1.0, 1, True)
        saveFrequency = max(1, int(saveFrequency))
        if chain == "last":
            s = start
            for _ in range(1, Nconf * saveFrequency):
                s = self.generate_(s)
            return s
        mc = [None] * Nconf
        nstart = 0
        if store is not None and store.exist(baseNode):
            try:
                nstart = store.getMinMaxConfigs(baseNode)[1]
            except FileNotFoundError:  # the group exists but holds no state
                nstart = 0
            if nstart >= Nconf:
                raise ValueError(f"{baseNode} already holds state {nstart}, beyond Nconf = {Nconf}")
        resumed = False
        if store is not None and store.exist(f"{baseNode}/{nstart}"):
            try:
                mc[nstart] = _resumed(store, start, baseNode, None)
                resumed = True
            except Exception:  # the most recent state is incomplete: drop it and take the one before
                store.deleteData(f"{baseNode}/{nstart}")
                nstart -= 1
                if nstart >= 0:
                    mc[nstart] = _resumed(store, start, baseNode, nstart)
                    resumed = True
                else:  # the only state was state 0: start over
                    nstart = 0
        if not resumed:
            mc[nstart] = start
            if store is not None:
                store.write(start, f"{baseNode}/{nstart}")
        for n in range(nstart + 1, Nconf):
            s = mc[n - 1]
            for _ in range(saveFrequency - 1):
                s = self.generate_(s)
            mc[n] = self.generate_(s)
            if store is not None:
                store.write(mc[n], f"{baseNode}/{n}")
        return mc


def _resumed(store, template: MarkovState, baseNode: str, markovTime):
    """A Markov state read from the store with the template's field names and weight keys; each field comes back as
    the kind of array the template holds (a torch tensor on the template's device, or numpy)."""
    st = MarkovState(Configuration(template.configuration), template.actionValue, template.acceptanceProbability,
                     template.markovTime, template.accepted, dict(template.weights))
    store.read(st, baseNode, markovTime)
    cfg = Configuration()
    for k, v in st.configuration.items():
        ref = template.configuration[k]
        if T.is_torch(ref):
            import torch

            cfg[k] = torch.from_numpy(np.ascontiguousarray(v)).to(ref.device)
        else:
            cfg[k] = v
    st.configuration = cfg
    return st


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


class ChainEnsemble:
    """Independent HMC chains on lattices of different shapes and couplings, advanced together (no counterpart in the
    reference, which runs one chain per HMC object; every chain follows HMC.tpp:186-241 as HMC.generate_ does: its own
    momenta, its own uniform draw, FP64 Delta H).

    groups: one dict per lattice shape {"lattice", "Nt", "beta", "U": per-chain couplings (nconf values)[, "mu"]}.
    Per HMC step: the LeapfrogRealForce (real_force=True) or Leapfrog trajectories of every chain of every group are
    ONE nslg_leapfrog_group call (from the third step on, one CUDA-graph launch whose branches are the groups' batched
    trajectories), then per group one batched action (nslg_hubbard_eval_batch_u: one batched log det of all its
    chains and both species), one batched kinetic sum and the device-side selection of the accepted fields. Fields
    are CUDA tensors of shape (nconf_g, Nt_g, Nx_g) per group (numpy arrays are accepted and returned as numpy)."""

    def __init__(self, groups, trajectoryLength: float = 1.0, numberSteps: int = 10, seed: int | None = None,
                 real_force: bool = True, ctx=None, stabilisation: str = "auto"):
        from .context import Context
        from .fermion_matrix import HubbardExp

        self.ctx = ctx if ctx is not None else Context()
        self.groups = [dict(g) for g in groups]
        self.fms, self.Ut = [], []
        for g in self.groups:
            fm = HubbardExp(g["lattice"], int(g["Nt"]), g["beta"], g.get("mu", 0.0), ctx=self.ctx)
            if stabilisation != "auto":
                fm.set_stabilisation(stabilisation)
            self.fms.append(fm)
            delta = complex(g["beta"]) / int(g["Nt"])
            U = np.atleast_1d(np.asarray(g["U"], dtype=np.complex128))
            self.Ut.append(np.ascontiguousarray(delta * U))  # U~ = delta U (hubbard.tpp:9-19)
        self.traj = float(trajectoryLength)
        self.nmd = int(numberSteps)
        self.real_force = bool(real_force)
        self.rng = np.random.default_rng(seed)
        self.deltaH = []  # per step: list (per group) of nconf_g values H1 - H0
        self.accepted = None

    @property
    def nconf(self):
        return [len(u) for u in self.Ut]

    def _ptrs(self, xs):
        return (C.c_void_p * len(xs))(*[T.ptr(x) for x in xs])

    def leapfrog(self, qs, ps):
        """(q1, p1) per group after one trajectory of every chain (nslg_leapfrog_group)."""
        from . import _lib

        qs = [T.as_c128(q) for q in qs]
        ps = [T.as_c128(p) for p in ps]
        for k, (q, p, fm, n) in enumerate(zip(qs, ps, self.fms, self.nconf)):
            if tuple(q.shape) != (n, fm.Nt, fm.Nx) or tuple(p.shape) != tuple(q.shape):
                raise ValueError(f"group {k}: fields must have shape {(n, fm.Nt, fm.Nx)}, got {tuple(q.shape)} and "
                                 f"{tuple(p.shape)}")
        q1 = [T.empty_like(q) for q in qs]
        p1 = [T.empty_like(p) for p in ps]
        ng = len(self.fms)
        handles = (C.c_void_p * ng)(*[fm.handle for fm in self.fms])
        nconf = (C.c_int64 * ng)(*self.nconf)
        uts = [np.ascontiguousarray(u) for u in self.Ut]
        utp = (C.c_void_p * ng)(*[u.ctypes.data for u in uts])
        with T.stream_order(self.ctx, *qs, *ps, *q1, *p1):
            _lib.check(_lib.load().nslg_leapfrog_group(ng, handles, nconf, self._ptrs(qs), self._ptrs(ps),
                                                       self._ptrs(q1), self._ptrs(p1), utp, self.traj, self.nmd, 0,
                                                       int(self.real_force), _lib.TERM_GAUGE | _lib.TERM_FERMION))
        return q1, p1

    def action(self, qs):
        """S per chain, per group (gauge + fermion terms, FP64)."""
        from . import _lib

        out = []
        for q, fm, u in zip(qs, self.fms, self.Ut):
            q = T.as_c128(q)
            n = int(q.shape[0])
            S = (_lib.c128 * n)()
            with T.stream_order(self.ctx, q):
                _lib.check(_lib.load().nslg_hubbard_eval_batch_u(fm.handle, n, T.ptr(q), u.ctypes.data,
                                                                 _lib.TERM_GAUGE | _lib.TERM_FERMION, S))
            out.append(np.array([complex(v.re, v.im) for v in S]))
        return out

    def _kinetic(self, p, fm) -> np.ndarray:
        from . import _lib

        n = int(p.shape[0])
        out = (_lib.c128 * n)()
        with T.stream_order(self.ctx, p):
            _lib.check(_lib.load().nslg_kinetic_batch(fm.handle, n, T.ptr(p), out))
        return np.array([complex(v.re, v.im) for v in out])

    def _select(self, acc, q1, q, fm):
        from . import _lib

        if not T.is_torch(q):
            return np.where(acc[:, None, None], q1, q)
        q = q.clone()
        flags = np.ascontiguousarray(acc, dtype=np.int32)
        with T.stream_order(self.ctx, q1, q):
            _lib.check(_lib.load().nslg_accept_batch(fm.handle, int(q.shape[0]), flags.ctypes.data, T.ptr(q1),
                                                     T.ptr(q)))
        return q

    def momenta(self, qs):
        """Real Gaussian momenta per group, drawn from this ensemble's generator, in the kind and device of qs."""
        ps = []
        for q in qs:
            p = self.rng.standard_normal(tuple(q.shape)) + 0j
            if T.is_torch(q):
                import torch

                p = torch.from_numpy(p).to(q.device)
            ps.append(p)
        return ps

    def generate(self, phi0s, Ntraj: int):
        """Ntraj HMC steps of every chain from phi0s (one field batch per group); returns the final fields and the
        per-chain acceptance rates (per group)."""
        qs = [T.as_c128(q) for q in phi0s]
        S = self.action(qs)
        acc_count = [np.zeros(n) for n in self.nconf]
        for _ in range(int(Ntraj)):
            p0 = self.momenta(qs)
            q1, p1 = self.leapfrog(qs, p0)
            S1 = self.action(q1)
            step_dh = []
            for g, fm in enumerate(self.fms):
                H0 = S[g] + self._kinetic(T.as_c128(p0[g]), fm)
                H1 = S1[g] + self._kinetic(p1[g], fm)
                step_dh.append(H1 - H0)
                prob = np.exp(np.minimum(700.0, (H0 - H1).real))
                acc = self.rng.random(len(prob)) <= prob
                acc_count[g] += acc
                qs[g] = self._select(acc, q1[g], qs[g], fm)
                S[g] = np.where(acc, S1[g], S[g])
            self.deltaH.append(step_dh)
        self.accepted = acc_count
        return qs, [a / max(int(Ntraj), 1) for a in acc_count]
