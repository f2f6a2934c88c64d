"""Correlator-measurement service: continuous batching of point-source solves of mixed lattice sizes.

A request is a stored auxiliary field phi on a lattice (Nx sites, Nt slices, beta) plus the source times of
TwoPointCorrelator::measure (src/NSL/Measurements/Hubbard/twoPointCorrelationFunction.tpp:116-162): Nx point sources
per source time, solved with CG on MM^dagger and multiplied by M^dagger. The server keeps the lattice data resident
(one fermion-matrix handle per lattice and slot: exp(delta K), its digit planes, workspaces) and runs requests on
`slots` concurrent CUDA streams: a request is admitted when a slot is free and its device-memory estimate fits the
remaining HBM budget, so requests arriving while others are on the GPU start as soon as capacity frees up and their
kernels overlap with the running ones. Every request's result is independent of what runs beside it (the kernels
are deterministic and a request never shares buffers), so a result is the same alone and in the mix.
Latency is measured from submission to completion.
"""
from __future__ import annotations

import dataclasses
import queue
import threading
import time

import numpy as np

from .context import Context
from .fermion_matrix import HubbardExp, Species
from .measurement import TwoPointCorrelator


@dataclasses.dataclass
class CorrelatorRequest:
    lattice: object
    Nt: int
    beta: float
    phi: np.ndarray
    n_time_sources: int = 1
    species: Species = Species.Particle
    tag: object = None
    # filled by the server
    submitted: float = 0.0
    started: float = 0.0
    finished: float = 0.0
    result: np.ndarray | None = None
    stats: dict | None = None
    error: str | None = None
    done: threading.Event = dataclasses.field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.finished - self.submitted

    def device_bytes(self, digits: int = 7) -> int:
        """Device memory a request needs beyond the resident lattice data: the solver's FP64 vectors and the
        operand digit planes for its Nx right-hand sides per source time."""
        Nx = self.lattice.sites()
        step = max(1, self.Nt // max(1, self.n_time_sources))
        rhs = Nx * len(range(0, self.Nt, step))
        n = rhs * self.Nt * Nx
        ld = -(-Nx // 32) * 32
        return int(n * 16 * 9 + digits * 2 * rhs * self.Nt * ld * 2)


class CorrelatorServer:
    def __init__(self, slots: int = 4, hbm_budget_bytes: int = 64 << 30, precision: str = "bf16split",
                 eps: float = 1e-10, device: int = 0, max_iter: int = 100_000):
        self.slots = int(slots)
        self.budget = int(hbm_budget_bytes)
        self.in_use = 0
        self.precision = precision
        self.eps = eps
        self.max_iter = int(max_iter)
        self.device = device
        self._q: queue.Queue = queue.Queue()
        self._cv = threading.Condition()
        self._stop = False
        self._handles = [dict() for _ in range(self.slots)]
        self._ctx = [Context(device) for _ in range(self.slots)]
        self._threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(self.slots)]
        for t in self._threads:
            t.start()

    # ---- client side --------------------------------------------------------------------------------------------
    def submit(self, req: CorrelatorRequest) -> CorrelatorRequest:
        need = req.device_bytes()
        if need > self.budget:
            req.error = f"request needs {need} bytes, more than the HBM budget of {self.budget}"
            req.done.set()
            return req
        req.submitted = time.perf_counter()
        self._q.put(req)
        return req

    def close(self):
        self._stop = True
        for _ in self._threads:
            self._q.put(None)
        for t in self._threads:
            t.join(timeout=60)
        # release the resident lattice data now (fermion matrices before their contexts) instead of leaving it to
        # the cyclic garbage collector (the worker threads reference the server)
        self._threads = []
        self._handles = [dict() for _ in range(self.slots)]
        self._ctx = []

    # ---- server side --------------------------------------------------------------------------------------------
    def _admit(self, need: int):
        with self._cv:
            while self.in_use + need > self.budget:
                self._cv.wait(timeout=0.05)
            self.in_use += need

    def _release(self, need: int):
        with self._cv:
            self.in_use -= need
            self._cv.notify_all()

    def _handle(self, slot: int, req: CorrelatorRequest) -> HubbardExp:
        key = (id(req.lattice), req.Nt, float(req.beta))
        h = self._handles[slot].get(key)
        if h is None:
            h = HubbardExp(req.lattice, req.Nt, req.beta, ctx=self._ctx[slot])
            self._handles[slot][key] = h
        return h

    def _worker(self, slot: int):
        import torch

        torch.cuda.set_device(self.device)
        while True:
            req = self._q.get()
            if req is None:
                return
            need = req.device_bytes()
            self._admit(need)
            try:
                req.started = time.perf_counter()
                hfm = self._handle(slot, req)
                corr = TwoPointCorrelator(hfm, req.species, eps=self.eps, maxIter=self.max_iter,
                                          precision=self.precision)
                req.result = corr.measure(req.phi, req.n_time_sources)
                req.stats = corr.stats
            except Exception as e:  # reported on the request; the server keeps running
                req.error = f"{type(e).__name__}: {e}"
            finally:
                req.finished = time.perf_counter()
                self._release(need)
                req.done.set()


def latency_summary(reqs) -> dict:
    lat = np.array([r.latency for r in reqs if r.error is None])
    if lat.size == 0:
        return {"count": 0}
    return {"count": int(lat.size), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean())}
