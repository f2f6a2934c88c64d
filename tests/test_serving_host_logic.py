"""Host-side failure handling of the correlator service, without GPU work: invalid fields are rejected at
submission (nothing queued or launched), a queued request can be cancelled, and admission respects the HBM budget
and the batch size. The tests use a server subclass with the scheduling state only (no contexts, no worker threads).
"""
import threading

import numpy as np

from nsl_gb300.lattice import Honeycomb
from nsl_gb300.serving import CorrelatorRequest, CorrelatorServer


class HostOnlyServer(CorrelatorServer):
    """The scheduling state of CorrelatorServer without contexts or worker threads."""

    def __init__(self, budget, max_batch_systems=16384, cost_ratio=8.0):
        self.slots = 0
        self.budget = budget
        self.in_use = 0
        self.max_batch_systems = max_batch_systems
        self.cost_ratio = cost_ratio
        self._queue = []
        self._cv = threading.Condition()
        self._stop = False
        self.batches = []


def _req(L=(2, 2), Nt=8, ntsrc=1, phi=None):
    lat = Honeycomb(L)
    if phi is None:
        phi = np.zeros((Nt, lat.sites()), dtype=complex)
    return CorrelatorRequest(lat, Nt, 1.0, phi, n_time_sources=ntsrc)


def test_nan_inf_and_shape_rejected_before_queueing():
    srv = HostOnlyServer(1 << 40)
    for bad in (np.nan, np.inf):
        phi = np.zeros((8, 8), dtype=complex)
        phi[2, 3] = bad
        r = srv.submit(_req(phi=phi))
        assert r.done.is_set() and "NaN or Inf" in r.error
    r = srv.submit(_req(phi=np.zeros((7, 8), dtype=complex)))
    assert r.done.is_set() and "shape" in r.error
    assert srv._queue == []


def test_cancel_queued_request():
    srv = HostOnlyServer(1 << 40)
    a, b = srv.submit(_req()), srv.submit(_req())
    assert srv.cancel(a)
    assert a.done.is_set() and a.error == "cancelled"
    assert srv._queue == [b] and not b.done.is_set()


def test_admission_by_budget_and_batch_size():
    one = _req().device_bytes()
    srv = HostOnlyServer(2 * one + one // 2)
    reqs = [srv.submit(_req()) for _ in range(4)]
    batch, need = srv._take_batch()
    assert batch == reqs[:2] and need == 2 * one and srv.in_use == 2 * one
    batch2, _ = srv._take_batch()  # the budget is held by the running batch
    assert batch2 == []
    srv.in_use -= need  # the batch finished
    batch3, _ = srv._take_batch()
    assert batch3 == reqs[2:]
    # a cap on the systems of one batch
    srv = HostOnlyServer(1 << 40, max_batch_systems=8)
    reqs = [srv.submit(_req()) for _ in range(3)]  # 8 sources each
    assert srv._take_batch()[0] == reqs[:1]


def test_oversized_request_rejected_at_submission():
    srv = HostOnlyServer(1000)
    r = srv.submit(_req())
    assert r.done.is_set() and "HBM budget" in r.error
    srv = HostOnlyServer(1 << 40, max_batch_systems=4)
    r = srv.submit(_req())
    assert r.done.is_set() and "sources" in r.error


def test_batches_group_requests_of_similar_work():
    """A batch takes the oldest request and the queued ones whose work per iteration is within cost_ratio of it: a
    large request (honeycomb 6x6, Nt 32: 2,916x the work of a 2x2, Nt 8 one) neither joins nor blocks small ones."""
    srv = HostOnlyServer(1 << 40)
    small = [srv.submit(_req()) for _ in range(2)]
    big = srv.submit(_req(L=(6, 6), Nt=32))
    small.append(srv.submit(_req(Nt=16)))  # 2x the work of the first: same batch
    batch, _ = srv._take_batch()
    assert batch == small
    batch, _ = srv._take_batch()
    assert batch == [big]
    assert big.work() > srv.cost_ratio * small[0].work()
