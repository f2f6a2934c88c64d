"""HMC step (kinetic term, Delta H, Metropolis) and the two-point correlator on the GPU."""
import numpy as np
import pytest

from conftest import TWOPOINT_CASES, load_golden, load_twopoint, rel_err

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


@pytest.mark.parametrize("name", TWOPOINT_CASES)
@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_two_point_correlators_vs_reference(name, precision):
    """measure(nts) and measureK(k, nts) of both species against the reference's TwoPointCorrelator outputs
    (twoPointCorrelationFunction.tpp:116-233, golden fixtures); the reference's CG stops at |r| <= 1e-12 over the
    whole source batch, the per-source solves here at a relative true residual of 1e-11."""
    import nsl_gb300 as N
    from nsl_gb300.measurement import TwoPointCorrelator

    g = load_twopoint(name)
    hfm = N.HubbardExp(N.Honeycomb(g["L"]), g["Nt"], g["beta"], g["mu"])
    for sp, tag in ((N.Species.Particle, "P"), (N.Species.Hole, "H")):
        tp = TwoPointCorrelator(hfm, sp, eps=1e-11, precision=precision, wallSources=g["wall"])
        assert rel_err(tp.measure(g["phi"], g["nts"]), g["corr_" + tag]) < 1e-9
        assert tp.stats["converged"] == tp.stats["systems"]
        blocks = tp.measureK_blocks(g["phi"], g["nts"])
        assert rel_err(blocks, g["block_" + tag]) < 1e-9
        assert rel_err(tp.measureK(g["phi"], 1, g["nts"]), g["block_" + tag][1]) < 1e-9


@pytest.mark.parametrize("L,Nt,nconf,real_force", [((3, 3), 16, 5, True), ((2, 2), 6, 3, False), ((6, 6), 8, 2, True)])
def test_leapfrog_batch_equals_single(L, Nt, nconf, real_force):
    """nconf configurations in one batched trajectory (eager, then captured and replayed) each follow the trajectory
    the single-configuration call gives them (to rounding: a single small-lattice call forms the force's matrix
    products as scans, a batch as chains), and the batched action equals the single evaluation; the first
    configuration also against the oracle's leapfrog."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import Leapfrog, LeapfrogRealForce
    from oracle import nsl_oracle as O

    lat = N.Honeycomb(L)
    beta, U = 4.0, 2.0
    p = {"Nt": Nt, "beta": beta, "mu": 0.1, "U": U}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    LF = LeapfrogRealForce if real_force else Leapfrog
    lf = LF(S, 1.0, 6)
    rng = np.random.default_rng(41)
    q = rng.standard_normal((nconf, Nt, lat.sites())) * np.sqrt(beta / Nt * U) + 0j
    pm = rng.standard_normal((nconf, Nt, lat.sites())) + 0j
    for _ in range(3):  # eager, capture, replay
        qb, pb = lf({"phi": q}, {"phi": pm})
    for b in range(nconf):
        qs, ps = lf({"phi": q[b]}, {"phi": pm[b]})
        assert rel_err(qb["phi"][b], qs["phi"]) < 1e-10
        assert rel_err(pb["phi"][b], ps["phi"]) < 1e-10
    A = O.HubbardAction(lat.hopping_matrix(), Nt, beta, U, mu=0.1)
    q1, p1 = O.leapfrog(A, q[0], pm[0], 1.0, 6, real_force=real_force)
    # honeycomb 6x6 at delta = 0.5: a 1e-15 relative change of phi moves this trajectory's end point by 1.2e-11
    # (oracle against itself), so rounding-level differences in the force show up at ~1e-9 there
    bar = 1e-8 if lat.sites() > 18 else 1e-10
    assert rel_err(qb["phi"][0], q1) < bar
    assert rel_err(pb["phi"][0], p1) < bar
    Sb = S.eval_batch(qb["phi"])
    for b in range(nconf):
        assert abs(Sb[b] - S(qb["phi"][b])) < 1e-10 * max(1.0, abs(Sb[b]))


def test_hmc_chains_match_single_chain_rule():
    """HMCChains: every chain's Delta H equals the oracle's for the same momenta; acceptance in (0, 1]."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.hmc import HMCChains
    from nsl_gb300.integrator import LeapfrogRealForce
    from oracle import nsl_oracle as O

    g = load_golden("honey3x3_nt16")
    lat = N.Honeycomb((3, 3))
    p = {"Nt": g["Nt"], "beta": g["beta"], "mu": 0.0, "U": g["U"]}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    nconf = 4
    rng = np.random.default_rng(5)
    phi0 = rng.standard_normal((nconf, g["Nt"], g["Nx"])) * np.sqrt(g["beta"] / g["Nt"] * g["U"]) + 0j
    ch = HMCChains(LeapfrogRealForce(S, 1.0, 10), S, seed=9)
    q, rate = ch.generate(phi0, 1)
    pr = np.random.default_rng(9).standard_normal(phi0.shape) + 0j  # the momenta of the first step
    A = O.HubbardAction(g["hops"], g["Nt"], g["beta"], g["U"])
    for b in range(nconf):
        q1, p1 = O.leapfrog(A, phi0[b], pr[b], 1.0, 10, real_force=True)
        dH = O.hamiltonian(A.eval(q1), p1) - O.hamiltonian(A.eval(phi0[b]), pr[b])
        assert abs(ch.deltaH[0][b] - dH) < 1e-8 * max(1.0, abs(A.eval(phi0[b])))
    q, rate = ch.generate(q, 5)
    assert rate.shape == (nconf,) and (rate >= 0).all() and (rate <= 1).all()


def test_leapfrog_batch_diag_discretisation():
    """Batched trajectories with FermionMatrixType = HubbardDiag: each configuration as in a single call (to
    rounding), and the batched action (evaluated configuration by configuration for this discretisation) equals the
    single one."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import LeapfrogRealForce

    lat = N.Honeycomb((2, 2))
    Nt, beta, U, nconf = 6, 1.5, 2.0, 3
    p = {"Nt": Nt, "beta": beta, "mu": 0.2, "U": U}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p, FermionMatrixType=N.HubbardDiag)
    lf = LeapfrogRealForce(S, 0.5, 4)
    rng = np.random.default_rng(43)
    q = rng.standard_normal((nconf, Nt, lat.sites())) * np.sqrt(beta / Nt * U) + 0j
    pm = rng.standard_normal((nconf, Nt, lat.sites())) + 0j
    for _ in range(3):
        qb, pb = lf({"phi": q}, {"phi": pm})
    Sb = S.eval_batch(qb["phi"])
    for b in range(nconf):
        qs, ps = lf({"phi": q[b]}, {"phi": pm[b]})
        assert rel_err(qb["phi"][b], qs["phi"]) < 1e-10
        assert rel_err(pb["phi"][b], ps["phi"]) < 1e-10
        assert abs(Sb[b] - S(qb["phi"][b])) < 1e-10 * max(1.0, abs(Sb[b]))


def test_density_and_double_occupancy():
    """n(x) and d(x) from both species' equal-time propagators on the GPU against the oracle's dense inverse, the
    free theory's half filling, and a short fixed-seed chain's averages (mu = 0: <n> = 1 within its error)."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.hmc import HMCChains
    from nsl_gb300.integrator import LeapfrogRealForce
    from nsl_gb300.observables import chain_observables, density_and_double_occupancy
    from oracle import nsl_oracle as O

    g = load_golden("honey2x2_nt6_mu")
    lat = N.Honeycomb((2, 2))
    hfm = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    n, d = density_and_double_occupancy(hfm, g["phi"], 2)
    n_o, d_o = O.density_double_occupancy(O.HubbardExp(g["hops"], g["Nt"], g["beta"], g["mu"]), g["phi"], 2)
    assert rel_err(n, n_o) < 1e-9 and rel_err(d, d_o) < 1e-9
    free = N.HubbardExp(lat, 8, 2.0, 0.0)
    n0, d0 = density_and_double_occupancy(free, np.zeros((8, lat.sites()), dtype=np.complex128))
    assert np.abs(n0 - 1).max() < 1e-9 and np.abs(d0 - 0.25).max() < 1e-9
    # a fixed-seed chain at mu = 0, U = 1: 8 chains x 4 trajectories, observables on the last configurations
    p = {"Nt": 8, "beta": 2.0, "mu": 0.0, "U": 1.0}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    rng = np.random.default_rng(17)
    phi0 = rng.standard_normal((8, 8, lat.sites())) * np.sqrt(2.0 / 8 * 1.0) + 0j
    q, rate = HMCChains(LeapfrogRealForce(S, 1.0, 8), S, seed=17).generate(phi0, 4)
    assert rate.mean() > 0.5
    obs, _ = chain_observables(N.HubbardExp(lat, 8, 2.0, 0.0), list(q), maxIter=5000)
    assert obs["unconverged"] == 0
    assert abs(obs["n"].real - 1.0) < 5 * obs["n_err"] + 1e-6
    assert 0.0 < obs["d"].real < 0.25 + 5 * obs["d_err"]


def test_fixed_seed_chains_match_the_oracle_chain():
    """A fixed-seed run of HMCChains (4 chains, 3 trajectories, honeycomb 2x2, Nt = 8) against the same Markov
    process run by the oracle with the same random stream (momenta for all chains, then one uniform per chain):
    the same accept decisions, the same fields to 1e-9, and the same density and double occupancy."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.hmc import HMCChains
    from nsl_gb300.integrator import LeapfrogRealForce
    from nsl_gb300.observables import density_and_double_occupancy
    from oracle import nsl_oracle as O

    lat = N.Honeycomb((2, 2))
    Nt, beta, U, nmd, nconf, ntraj, seed = 8, 2.0, 1.0, 8, 4, 3, 23
    p = {"Nt": Nt, "beta": beta, "mu": 0.0, "U": U}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    phi0 = np.random.default_rng(3).standard_normal((nconf, Nt, lat.sites())) * np.sqrt(beta / Nt * U) + 0j
    ch = HMCChains(LeapfrogRealForce(S, 1.0, nmd), S, seed=seed)
    q_gpu, rate = ch.generate(phi0, ntraj)

    A = O.HubbardAction(lat.hopping_matrix(), Nt, beta, U)
    rng = np.random.default_rng(seed)
    q = phi0.copy()
    Sq = np.array([A.eval(x) for x in q])
    acc_count = np.zeros(nconf)
    for _ in range(ntraj):
        p0 = rng.standard_normal(q.shape) + 0j
        u = rng.random(nconf)
        for b in range(nconf):
            q1, p1 = O.leapfrog(A, q[b], p0[b], 1.0, nmd, real_force=True)
            S1 = A.eval(q1)
            H0, H1 = O.hamiltonian(Sq[b], p0[b]), O.hamiltonian(S1, p1)
            if u[b] <= O.metropolis_prob(H0, H1):
                q[b], Sq[b] = q1, S1
                acc_count[b] += 1
    assert np.array_equal(rate, acc_count / ntraj)
    assert rel_err(q_gpu, q) < 1e-9
    hfm = N.HubbardExp(lat, Nt, beta, 0.0)
    hor = O.HubbardExp(lat.hopping_matrix(), Nt, beta, 0.0)
    for b in range(nconf):
        n, d = density_and_double_occupancy(hfm, q_gpu[b])
        n_o, d_o = O.density_double_occupancy(hor, q[b])
        assert rel_err(n, n_o) < 1e-8 and rel_err(d, d_o) < 1e-8


def test_cpu_runnable_configuration_chain_observables():
    """The CPU-runnable HMC configuration (honeycomb 3x3, Nt = 16, beta = 4, U = 2, Nmd = 10, trajectory length 1):
    1000 trajectories as 8 chains of 125 on the GPU (HMCChains) and the same Markov process run by the oracle from
    the same random stream. The acceptance rates agree, and <n> and the double occupancy over every fifth
    configuration (measured on the GPU and by the oracle's dense inverse respectively) agree within their statistical
    errors; at mu = 0 on the bipartite lattice <n> = 1."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.hmc import HMCChains
    from nsl_gb300.integrator import LeapfrogRealForce
    from nsl_gb300.observables import density_and_double_occupancy
    from oracle import nsl_oracle as O

    lat = N.Honeycomb((3, 3))
    Nt, beta, U, nmd, nconf, ntraj, seed = 16, 4.0, 2.0, 10, 8, 125, 41
    Nx = lat.sites()
    p = {"Nt": Nt, "beta": beta, "mu": 0.0, "U": U}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    phi0 = np.random.default_rng(4).standard_normal((nconf, Nt, Nx)) * np.sqrt(beta / Nt * U) + 0j
    ch = HMCChains(LeapfrogRealForce(S, 1.0, nmd), S, seed=seed)
    q = phi0.copy()
    gpu_cfgs = []
    acc_gpu = 0.0
    for _ in range(ntraj // 5):  # five trajectories, then keep the configurations
        q, rate = ch.generate(q, 5)
        acc_gpu += rate.sum() * 5
        gpu_cfgs.extend(list(np.asarray(q)))
    # the oracle's chain on the same random stream (momenta for all chains, one uniform per chain per trajectory)
    A = O.HubbardAction(lat.hopping_matrix(), Nt, beta, U)
    rng = np.random.default_rng(seed)
    qo = phi0.copy()
    So = np.array([A.eval(x) for x in qo])
    acc_o = 0
    ora_cfgs = []
    for k in range(ntraj):
        p0 = rng.standard_normal(qo.shape) + 0j
        u = rng.random(nconf)
        for b in range(nconf):
            q1, p1 = O.leapfrog(A, qo[b], p0[b], 1.0, nmd, real_force=True)
            S1 = A.eval(q1)
            if u[b] <= O.metropolis_prob(O.hamiltonian(So[b], p0[b]), O.hamiltonian(S1, p1)):
                qo[b], So[b] = q1, S1
                acc_o += 1
        if (k + 1) % 5 == 0:
            ora_cfgs.extend(list(qo.copy()))
    total = nconf * ntraj
    assert abs(acc_gpu / total - acc_o / total) < 0.02, (acc_gpu / total, acc_o / total)
    hfm = N.HubbardExp(lat, Nt, beta, 0.0)
    hor = O.HubbardExp(lat.hopping_matrix(), Nt, beta, 0.0)
    stats = []
    nd = [density_and_double_occupancy(hfm, c, stats=stats) for c in gpu_cfgs]
    ng = np.array([np.mean(n) for n, _ in nd])
    dg = np.array([np.mean(d) for _, d in nd])
    no, do = zip(*[(np.mean(a), np.mean(b)) for a, b in (O.density_double_occupancy(hor, c) for c in ora_cfgs)])
    no, do = np.array(no), np.array(do)

    def err(v):
        return v.std(ddof=1) / np.sqrt(len(v))

    assert all(s["converged"] == s["systems"] for s in stats)
    assert abs(ng.mean().real - 1.0) < 5 * err(ng.real) + 1e-9
    assert abs(ng.mean() - no.mean()) < 5 * np.hypot(err(ng.real), err(no.real)) + 1e-9
    assert abs(dg.mean() - do.mean()) < 5 * np.hypot(err(dg.real), err(do.real)) + 1e-9
