"""Correlator-measurement service: continuous batching of point-source solves of mixed lattice sizes.

A request is a stored auxiliary field phi on a lattice (Nx sites, Nt slices, beta) plus the source times of
TwoPointCorrelator::measure (src/NSL/Measurements/Hubbard/twoPointCorrelationFunction.tpp:116-162): Nx point sources
per source time, solved with CG on MM^dagger and multiplied by M^dagger.

Scheduling. `slots` worker threads each own a CUDA stream (a context). A worker that is free takes every queued
request that fits (the HBM budget still available, a cap on the systems of one batch, and work per iteration within
a factor of the oldest request's) and solves all of them as ONE grouped CG (nslg_cg_solve_group): the point sources of requests of different shapes are independent systems of
one launch sequence, each masked out as it converges. Requests that arrive while batches run join the next batch of
the first worker that frees up, and the batches of different workers overlap on the device. Lattice data
(exp(delta K), its digit planes) stay resident per worker and shape; every request of a batch gets a handle of its
own (its own phi) from a per-shape pool that is reused across batches.

Accuracy. The default rule is the double-double one (stop="true_residual_dd"): every point-source solve meets
|b - MM^dagger (x + x_lo)| <= eps |b| certified in double-double arithmetic, and M^{-1} b = M^dagger (x + x_lo) is
applied in double-double too. A request's result depends only on its own data up to rounding: the group's
reductions are split according to the batch's composition, so a result alone and in a mix agree to the solver's
tolerance (not bitwise).

Failures are reported on the request (error, done set), never raised in a worker: a phi with NaN/Inf or of the wrong
shape is rejected at submission, before anything is queued or launched; a request whose memory estimate exceeds the
whole budget is rejected at submission; cancel() removes a queued request (a request cancelled while its batch runs
has its result discarded); systems that do not converge in max_iter are reported in the request's stats.
Latency is measured from submission to completion.
"""
from __future__ import annotations

import dataclasses
import threading
import time

import numpy as np

from .context import Context
from .fermion_matrix import HubbardExp, MatrixCombination, Species
from .measurement import TwoPointCorrelator
from .solver import cg_group


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
    cancelled: bool = False
    batch_size: int = 0
    done: threading.Event = dataclasses.field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.finished - self.submitted

    def source_count(self) -> int:
        step = max(1, self.Nt // max(1, self.n_time_sources))
        return self.lattice.sites() * len(range(0, self.Nt, step))

    def work(self) -> int:
        """Work of one CG iteration of the request, in units of one time slice's site-to-site product (Nx^2)."""
        return self.source_count() * self.Nt * self.lattice.sites() ** 2

    def device_bytes(self, digits: int = 6) -> int:
        """Device memory a request needs beyond the resident lattice data: the grouped solver's packed FP64 vectors
        (right-hand sides, iterate, residual, direction, products, double-double pair and residual: ~20 vectors) and
        the operand digit planes of its right-hand sides."""
        Nx = self.lattice.sites()
        rhs = self.source_count()
        n = rhs * self.Nt * Nx
        ld = -(-Nx // 32) * 32
        return int(n * 16 * 20 + digits * 2 * rhs * self.Nt * ld * 2)


class CorrelatorServer:
    def __init__(self, slots: int = 2, hbm_budget_bytes: int = 64 << 30, precision: str = "bf16split",
                 eps: float = 1e-10, device: int = 0, max_iter: int = 100_000, stop: str = "true_residual_dd",
                 max_batch_systems: int = 16384, cost_ratio: float = 8.0):
        self.slots = int(slots)
        self.budget = int(hbm_budget_bytes)
        self.in_use = 0
        self.precision = precision
        self.eps = eps
        self.stop = stop
        self.max_iter = int(max_iter)
        self.max_batch_systems = int(max_batch_systems)
        self.cost_ratio = float(cost_ratio)
        self.device = device
        self._queue: list[CorrelatorRequest] = []
        self._cv = threading.Condition()
        self._stop = False
        self._pools = [dict() for _ in range(self.slots)]  # per worker: shape key -> list of idle handles
        self._ctx = [Context(device) for _ in range(self.slots)]
        self.batches: list[int] = []  # requests per batch, in order of completion
        self._threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(self.slots)]
        for t in self._threads:
            t.start()

    # ---- client side --------------------------------------------------------------------------------------------
    def submit(self, req: CorrelatorRequest) -> CorrelatorRequest:
        req.submitted = time.perf_counter()
        phi = np.asarray(req.phi)
        Nx = req.lattice.sites()
        why = None
        if phi.shape != (req.Nt, Nx):
            why = f"phi must have shape (Nt, Nx) = {(req.Nt, Nx)}, got {phi.shape}"
        elif not np.all(np.isfinite(phi)):
            why = "phi contains NaN or Inf"
        elif req.device_bytes() > self.budget:
            why = f"request needs {req.device_bytes()} bytes, more than the HBM budget of {self.budget}"
        elif req.source_count() > self.max_batch_systems:
            why = f"request has {req.source_count()} sources, more than a batch holds ({self.max_batch_systems})"
        if why is not None:
            req.error = why
            req.finished = time.perf_counter()
            req.done.set()
            return req
        with self._cv:
            self._queue.append(req)
            self._cv.notify()
        return req

    def cancel(self, req: CorrelatorRequest) -> bool:
        """Removes a queued request (True); a running one is marked and its result discarded (False)."""
        with self._cv:
            req.cancelled = True
            if req in self._queue:
                self._queue.remove(req)
                req.error = "cancelled"
                req.finished = time.perf_counter()
                req.done.set()
                return True
        return False

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join(timeout=600)
        # release the resident lattice data now (fermion matrices before their contexts) instead of leaving it to
        # the cyclic garbage collector (the worker threads reference the server)
        self._threads = []
        self._pools = [dict() for _ in range(self.slots)]
        self._ctx = []

    # ---- server side --------------------------------------------------------------------------------------------
    def _take_batch(self):
        """Under the lock: the queued requests that fit, oldest first; their memory estimate is added to in_use. A
        batch runs until its slowest system is final, so it takes only requests whose work per iteration is within
        cost_ratio of its oldest one's: a large request does not hold up small ones (they go to the next batch of
        the other worker) and small ones do not wait for a large one."""
        batch, need, systems = [], 0, 0
        rest = []
        first = None
        for req in self._queue:
            nb = req.device_bytes()
            ns = req.source_count()
            w = req.work()
            similar = first is None or (w <= self.cost_ratio * first and first <= self.cost_ratio * w)
            if similar and self.in_use + need + nb <= self.budget and systems + ns <= self.max_batch_systems:
                batch.append(req)
                need += nb
                systems += ns
                first = w if first is None else first
            else:
                rest.append(req)
        self._queue = rest
        self.in_use += need
        return batch, need

    def _handle(self, slot: int, req: CorrelatorRequest, taken: list) -> HubbardExp:
        key = (id(req.lattice), req.Nt, float(req.beta))
        pool = self._pools[slot].setdefault(key, [])
        h = pool.pop() if pool else HubbardExp(req.lattice, req.Nt, req.beta, ctx=self._ctx[slot])
        taken.append((key, h))
        return h

    def _worker(self, slot: int):
        import torch

        torch.cuda.set_device(self.device)
        while True:
            with self._cv:
                while not self._stop and not self._queue:
                    self._cv.wait()
                if self._stop and not self._queue:
                    return
                batch, need = self._take_batch()
                if not batch:  # the budget is held by running batches: wait for a release
                    self._cv.wait(timeout=0.05)
                    continue
            self._run_batch(slot, batch, need)

    def _run_batch(self, slot: int, batch, need: int):
        import torch

        taken = []
        now = time.perf_counter()
        try:
            items, jobs = [], []
            for req in batch:
                req.started = now
                req.batch_size = len(batch)
                h = self._handle(slot, req, taken)
                corr = TwoPointCorrelator(h, req.species, eps=self.eps, maxIter=self.max_iter,
                                          precision=self.precision)
                h.populate(req.phi, req.species)
                tsrcs = corr.source_times(req.n_time_sources)
                b = torch.from_numpy(corr.sources(tsrcs)).cuda(self.device)
                items.append((h, b))
                jobs.append((req, h, corr, tsrcs))
            # point sources have |b| = 1: the tolerance is absolute
            xs, los, stats = cg_group(items, MatrixCombination.MMdagger, self.eps, self.max_iter,
                                      precision=self.precision, stop=self.stop)
            for k, (req, h, corr, tsrcs) in enumerate(jobs):
                if los is not None:  # M^{-1} b = M^dagger (x + x_lo), in double-double
                    hi, lo = h.apply_dd(MatrixCombination.Mdagger, xs[k], los[k])
                    invM = (hi + lo).cpu().numpy()
                else:
                    invM = h.Mdagger(xs[k]).cpu().numpy()
                if not req.cancelled:
                    req.result = corr.accumulate(invM, tsrcs, req.n_time_sources)
                    req.stats = stats[k]
        except Exception as e:  # reported on the requests; the server keeps running
            for req in batch:
                req.error = f"{type(e).__name__}: {e}"
        finally:
            for key, h in taken:
                self._pools[slot][key].append(h)
            end = time.perf_counter()
            with self._cv:  # the batch's memory is released before its requests are reported done
                self.batches.append(len(batch))
                self.in_use -= need
                self._cv.notify_all()
            for req in batch:
                if req.cancelled and req.error is None:
                    req.error = "cancelled"
                    req.result = None
                req.finished = end
                req.done.set()


def latency_summary(reqs) -> dict:
    lat = np.array([r.latency for r in reqs if r.error is None])
    if lat.size == 0:
        return {"count": 0}
    return {"count": int(lat.size), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean())}
