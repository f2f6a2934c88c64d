"""HMC step (kinetic term, Delta H, Metropolis) and the two-point correlator on the GPU."""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def test_hmc_deltaH_matches_oracle():
    """H = S + 1/2 sum p^2 and the acceptance exp(Re(H0 - H1)) (HMC.tpp:186-241) against the oracle, same p."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.hmc import HMC, MarkovState
    from nsl_gb300.integrator import LeapfrogRealForce
    from oracle import nsl_oracle as O

    g = load_golden("honey3x3_nt16")
    lat = N.Honeycomb((3, 3))
    p = {"Nt": g["Nt"], "beta": g["beta"], "mu": 0.0, "U": g["U"]}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    hmc = HMC(LeapfrogRealForce(S, 1.0, 10), S, seed=3)
    q0 = {"phi": g["phi"]}
    st = MarkovState(q0, S(q0))
    rng = np.random.default_rng(3)  # the same stream HMC draws p from
    p0 = rng.standard_normal(g["phi"].shape) + 0j
    new = hmc.generate_(st)
    A = O.HubbardAction(g["hops"], g["Nt"], g["beta"], g["U"])
    q1, p1 = O.leapfrog(A, g["phi"], p0, 1.0, 10, real_force=True)
    H0 = O.hamiltonian(A.eval(g["phi"]), p0)
    H1 = O.hamiltonian(A.eval(q1), p1)
    assert abs(hmc.last_deltaH - (H1 - H0)) < 1e-9 * max(1.0, abs(H0))
    assert abs(new.acceptanceProbability - O.metropolis_prob(H0, H1)) < 1e-9 * max(1.0, new.acceptanceProbability)


def test_hmc_chain_runs_and_accepts():
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.hmc import HMC, getAcceptanceRate
    from nsl_gb300.integrator import LeapfrogRealForce

    lat = N.Honeycomb((2, 2))
    p = {"Nt": 8, "beta": 2.0, "mu": 0.0, "U": 2.0}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    rng = np.random.default_rng(0)
    phi = rng.standard_normal((8, 8)) * np.sqrt(2.0 / 8 * 2.0) + 0j
    chain = HMC(LeapfrogRealForce(S, 1.0, 8), S, seed=1).generate({"phi": phi}, 12)
    assert len(chain) == 12
    assert getAcceptanceRate(chain) > 0.5
    assert all(np.all(np.isfinite(s.configuration["phi"])) for s in chain)


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_two_point_correlator(precision):
    """measure(Ntsrc) (twoPointCorrelationFunction.tpp:116-162) against the exact dense inverse."""
    import nsl_gb300 as N
    from nsl_gb300.measurement import TwoPointCorrelator
    from oracle import nsl_oracle as O

    lat = N.Ring(6)
    Nt, beta = 8, 2.0
    rng = np.random.default_rng(21)
    phi = rng.standard_normal((Nt, 6)) * 0.4 + 0j
    hfm = N.HubbardExp(lat, Nt, beta)
    corr = TwoPointCorrelator(hfm, N.Species.Particle, eps=1e-11, precision=precision).measure(phi, 4)
    ref = O.two_point_correlator(O.HubbardExp(lat.hopping_matrix(), Nt, beta), phi, O.PARTICLE, 4)
    assert rel_err(corr, ref) < 1e-9
