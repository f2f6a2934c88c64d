"""Continuous-batching correlator service: results are the same alone and in a concurrent mix; HBM admission."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_requests():
    import nsl_gb300 as N
    from nsl_gb300.serving import CorrelatorRequest

    rng = np.random.default_rng(31)
    reqs = []
    for L, Nt, beta in (((2, 2), 8, 1.0), ((3, 3), 16, 2.0), ((2, 3), 12, 1.5), ((3, 3), 8, 1.0), ((4, 4), 16, 2.0)):
        lat = N.Honeycomb(L)
        phi = rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * 2.0) + 0j
        reqs.append(CorrelatorRequest(lat, Nt, beta, phi, n_time_sources=2))
    return reqs


def test_results_alone_equal_results_in_the_mix():
    from nsl_gb300.serving import CorrelatorServer, latency_summary

    alone = []
    srv = CorrelatorServer(slots=1, precision="bf16split")
    for r in make_requests():
        srv.submit(r)
        r.done.wait(120)
        assert r.error is None, r.error
        alone.append(r.result)
    srv.close()

    srv = CorrelatorServer(slots=3, precision="bf16split")
    mixed = make_requests()
    for r in mixed:
        srv.submit(r)
    for r in mixed:
        assert r.done.wait(120)
        assert r.error is None, r.error
    srv.close()
    for a, m in zip(alone, mixed):
        assert np.array_equal(a, m.result)
    s = latency_summary(mixed)
    assert s["count"] == 5 and s["p99_s"] >= s["p50_s"] > 0


def test_correlator_matches_oracle_inverse():
    from nsl_gb300.serving import CorrelatorServer
    from oracle import nsl_oracle as O

    srv = CorrelatorServer(slots=2, precision="bf16split")
    reqs = make_requests()[:2]
    for r in reqs:
        srv.submit(r)
    for r in reqs:
        r.done.wait(120)
        h = O.HubbardExp(r.lattice.hopping_matrix(), r.Nt, r.beta)
        ref = O.two_point_correlator(h, r.phi, O.PARTICLE, r.n_time_sources)
        assert np.abs(r.result - ref).max() < 1e-8 * np.abs(ref).max()
    srv.close()


def test_admission_rejects_oversized_request():
    import nsl_gb300 as N
    from nsl_gb300.serving import CorrelatorRequest, CorrelatorServer

    srv = CorrelatorServer(slots=1, hbm_budget_bytes=1 << 20)
    lat = N.Honeycomb((4, 4))
    r = srv.submit(CorrelatorRequest(lat, 16, 2.0, np.zeros((16, 32), dtype=complex), 4))
    assert r.done.is_set() and "HBM budget" in r.error
    srv.close()
