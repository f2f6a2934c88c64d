"""Host-side logic of the HMC drivers (momenta draws, H, the Metropolis decision, per-chain bookkeeping) with a
fake integrator and action, on CPU (HMC.tpp:186-241, markovState.tpp:88-96)."""
import numpy as np

from nsl_gb300.configuration import Configuration
from nsl_gb300.hmc import HMC, HMCChains, MarkovState, getAcceptanceRate


class FakeAction:
    """S(phi) = sum phi^2 / 2 per configuration (complex square), field key "phi"."""

    _key = "phi"

    def eval_batch(self, phi):
        return 0.5 * (np.asarray(phi) ** 2).sum(axis=(1, 2))

    def __call__(self, cfg):
        phi = cfg["phi"] if isinstance(cfg, dict) else cfg
        return complex(0.5 * (np.asarray(phi) ** 2).sum())


class FakeIntegrator:
    """A fixed map (q, p) -> (q + shift, p * scale): enough to check the bookkeeping around it."""

    def __init__(self, shift, scale):
        self.shift, self.scale = shift, scale

    def __call__(self, q, p):
        return Configuration({"phi": q["phi"] + self.shift}), Configuration({"phi": p["phi"] * self.scale})


def test_chains_metropolis_per_chain():
    nconf, shape = 6, (3, 4)
    rng0 = np.random.default_rng(1)
    phi0 = rng0.standard_normal((nconf,) + shape) + 0j
    # chain-dependent shifts: some proposals raise H a lot (rejected), some lower it (accepted)
    shift = np.array([0.0, 0.01, -0.5, 2.0, 5.0, -0.1])[:, None, None]
    ch = HMCChains(FakeIntegrator(shift, 1.0), FakeAction(), seed=5)
    ch._kinetic = lambda p: 0.5 * (np.asarray(p) ** 2).sum(axis=(1, 2))  # host stand-in for nslg_kinetic_batch
    q, rate = ch.generate(phi0, 1)
    # the same draws by hand: p ~ N(0, 1) for every chain, then one uniform per chain
    rng = np.random.default_rng(5)
    p0 = rng.standard_normal((nconf,) + shape)
    u = rng.random(nconf)
    S0 = 0.5 * (phi0 ** 2).sum(axis=(1, 2))
    q1 = phi0 + shift
    S1 = 0.5 * (q1 ** 2).sum(axis=(1, 2))
    K = 0.5 * (p0 ** 2).sum(axis=(1, 2))
    dH = (S1 + K) - (S0 + K)
    assert np.allclose(ch.deltaH[0], dH)
    acc = u <= np.exp(np.minimum(700.0, -dH.real))
    assert np.array_equal(rate == 1.0, acc)
    assert np.allclose(q, np.where(acc[:, None, None], q1, phi0))


def test_single_chain_generate_and_acceptance_rate():
    hmc = HMC(FakeIntegrator(0.0, 1.0), FakeAction(), seed=3)
    hmc._kinetic = lambda p: complex(0.5 * (np.asarray(p) ** 2).sum())  # host stand-in for nslg_kinetic
    cfg = Configuration({"phi": np.zeros((2, 2)) + 0j})
    st = MarkovState(cfg, hmc.action_(cfg))
    chain = [st]
    for _ in range(5):
        chain.append(hmc.generate_(chain[-1]))
    # q' = q and p' = p: Delta H = 0, every proposal accepted with probability 1
    assert all(s.accepted and s.acceptanceProbability == 1.0 for s in chain[1:])
    assert [s.markovTime for s in chain] == [1, 2, 3, 4, 5, 6]
    assert getAcceptanceRate(chain) == 1.0
    chain[2].accepted = False
    assert getAcceptanceRate(chain) == 5 / 6


def test_configuration_arithmetic():
    """Configuration +, -, +=, -=, scalar * (Configuration.tpp:38-158): shared fields combine, fields of one side
    only are appended (negated for -), and + / - / * leave their operands untouched."""
    a = Configuration({"phi": np.ones((2, 2)) + 0j, "chi": np.full((2,), 2.0 + 0j)})
    b = Configuration({"phi": np.full((2, 2), 3.0 + 0j), "eta": np.full((3,), 5.0 + 0j)})
    c = a + b
    assert np.all(c["phi"] == 4) and np.all(c["chi"] == 2) and np.all(c["eta"] == 5)
    d = a - b
    assert np.all(d["phi"] == -2) and np.all(d["eta"] == -5)
    c["chi"][0] = 99  # a deep copy: the operand is untouched
    assert a["chi"][0] == 2
    e = 2.0 * a
    assert np.all(e["phi"] == 2) and np.all(a["phi"] == 1)
    a += b
    assert np.all(a["phi"] == 4) and np.all(a["eta"] == 5)
    a["eta"][0] = 7
    assert b["eta"][0] == 5
    a -= Configuration({"zeta": np.ones(1) + 0j})
    assert a["zeta"][0] == -1


def test_serving_latency_summary_and_admission_estimate():
    """The serving loop's host-side bookkeeping: p50/p99 over the completed requests (failed ones excluded) and the
    device-memory estimate that admission compares with the HBM budget (grows with the sources and the lattice)."""
    from nsl_gb300.lattice import Honeycomb
    from nsl_gb300.serving import CorrelatorRequest, latency_summary

    reqs = []
    for i in range(101):
        r = CorrelatorRequest(Honeycomb((3, 3)), 16, 1.0, np.zeros((16, 18)))
        r.submitted, r.finished = 10.0, 10.0 + 0.01 * i
        reqs.append(r)
    reqs[-1].error = "failed"
    s = latency_summary(reqs)
    assert s["count"] == 100
    assert abs(s["p50_s"] - 0.495) < 1e-12 and abs(s["p99_s"] - 0.9801) < 1e-12
    assert latency_summary([reqs[-1]]) == {"count": 0}
    small = CorrelatorRequest(Honeycomb((3, 3)), 16, 1.0, np.zeros((16, 18)))
    two = CorrelatorRequest(Honeycomb((3, 3)), 16, 1.0, np.zeros((16, 18)), n_time_sources=2)
    big = CorrelatorRequest(Honeycomb((6, 6)), 16, 1.0, np.zeros((16, 72)))
    assert small.device_bytes() < two.device_bytes() < big.device_bytes()
    assert two.device_bytes() == 2 * small.device_bytes()


def test_buffer_plumbing():
    """tensor.py: inputs become contiguous complex128 of their own kind (numpy stays numpy, torch stays torch),
    outputs are allocated like the input, and the data pointer is the buffer's."""
    import torch

    from nsl_gb300 import tensor as T

    a = np.arange(12, dtype=np.float64).reshape(3, 4)[:, ::2]  # float, non-contiguous
    c = T.as_c128(a)
    assert isinstance(c, np.ndarray) and c.dtype == np.complex128 and c.flags["C_CONTIGUOUS"]
    assert np.array_equal(c.real, a)
    t = T.as_c128(torch.ones(2, 3, dtype=torch.float32).t())
    assert T.is_torch(t) and t.dtype == torch.complex128 and t.is_contiguous() and not T.is_cuda(t)
    assert T.ptr(c) == c.ctypes.data and T.ptr(t) == t.data_ptr()
    e = T.empty_like(c, (5, 2))
    assert isinstance(e, np.ndarray) and e.shape == (5, 2) and e.dtype == np.complex128
    assert T.empty_like(t).shape == t.shape and T.numel((3, 4, 5)) == 60
