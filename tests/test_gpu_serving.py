"""Continuous-batching correlator service: requests of mixed shapes batched into grouped solves; results the same
alone and in the mix (to the solver's tolerance); agreement with the oracle's dense inverse; HBM admission."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_requests(U=2.0, seed=31, shapes=None):
    import nsl_gb300 as N
    from nsl_gb300.serving import CorrelatorRequest

    rng = np.random.default_rng(seed)
    reqs = []
    for L, Nt, beta in shapes or (((2, 2), 8, 1.0), ((3, 3), 16, 2.0), ((2, 3), 12, 1.5), ((3, 3), 8, 1.0),
                                  ((4, 4), 16, 2.0)):
        lat = N.Honeycomb(L)
        phi = rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * U) + 0j
        reqs.append(CorrelatorRequest(lat, Nt, beta, phi, n_time_sources=2))
    return reqs


@pytest.mark.parametrize("precision", ["bf16split", "fp64"])
def test_results_alone_equal_results_in_the_mix(precision):
    """One request at a time on one worker, then all five submitted at once to two workers (batched into grouped
    solves of mixed shapes): each correlator agrees to 1e-9 relative (the solves certify 1e-10 per point source)."""
    from nsl_gb300.serving import CorrelatorServer, latency_summary

    alone = []
    srv = CorrelatorServer(slots=1, precision=precision)
    for r in make_requests():
        srv.submit(r)
        assert r.done.wait(300)
        assert r.error is None, r.error
        assert r.batch_size == 1
        alone.append(r.result)
    srv.close()

    srv = CorrelatorServer(slots=2, precision=precision)
    mixed = make_requests()
    for r in mixed:
        srv.submit(r)
    for r in mixed:
        assert r.done.wait(300)
        assert r.error is None, r.error
        assert r.stats["converged"] == r.stats["systems"]
    batches = list(srv.batches)
    srv.close()
    assert max(batches) >= 2  # some requests shared a grouped solve
    for a, m in zip(alone, mixed):
        assert np.abs(a - m.result).max() <= 1e-9 * np.abs(a).max()
    s = latency_summary(mixed)
    assert s["count"] == 5 and s["p99_s"] >= s["p50_s"] > 0


def test_correlator_matches_oracle_inverse():
    from nsl_gb300.serving import CorrelatorServer
    from oracle import nsl_oracle as O

    srv = CorrelatorServer(slots=2, precision="bf16split")
    reqs = make_requests()[:3]
    for r in reqs:
        srv.submit(r)
    for r in reqs:
        assert r.done.wait(300) and r.error is None, r.error
        h = O.HubbardExp(r.lattice.hopping_matrix(), r.Nt, r.beta)
        ref = O.two_point_correlator(h, r.phi, O.PARTICLE, r.n_time_sources)
        assert np.abs(r.result - ref).max() < 1e-8 * np.abs(ref).max()
    srv.close()


def test_admission_rejects_oversized_request_and_bad_fields():
    import nsl_gb300 as N
    from nsl_gb300.serving import CorrelatorRequest, CorrelatorServer

    srv = CorrelatorServer(slots=1, hbm_budget_bytes=1 << 20)
    lat = N.Honeycomb((4, 4))
    r = srv.submit(CorrelatorRequest(lat, 16, 2.0, np.zeros((16, 32), dtype=complex), 4))
    assert r.done.is_set() and "HBM budget" in r.error
    bad = np.zeros((16, 32), dtype=complex)
    bad[3, 4] = np.nan
    r = srv.submit(CorrelatorRequest(lat, 16, 2.0, bad, 1))
    assert r.done.is_set() and "NaN" in r.error
    srv.close()


def test_budget_limits_what_runs_at_once():
    """With a budget that holds one request at a time, three requests complete one after the other (batches of one)
    and the in-flight estimate returns to zero."""
    from nsl_gb300.serving import CorrelatorServer

    reqs = make_requests(shapes=(((2, 2), 8, 1.0), ((2, 2), 8, 1.0), ((2, 2), 8, 1.0)))
    srv = CorrelatorServer(slots=2, hbm_budget_bytes=reqs[0].device_bytes())
    for r in reqs:
        srv.submit(r)
    for r in reqs:
        assert r.done.wait(300) and r.error is None, r.error
    assert srv.in_use == 0 and max(srv.batches) == 1
    srv.close()
