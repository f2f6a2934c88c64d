"""Chains of different lattice shapes and couplings in one launch (nslg_leapfrog_group, nsl_gb300.hmc.ChainEnsemble).

Every chain must follow the trajectory that a single-configuration nslg_leapfrog with its own U~ gives it (to the
rounding difference between a batched and a single force: 1e-10), whether its group runs eagerly, while being
captured, or as a branch of the group's one graph launch (those three bitwise equal), and the oracle's leapfrog and
action (hubbardGaugeAction.tpp, hubbardFermiAction.tpp, leapfrog.tpp) for the same field and U.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

# (lattice, Nt, beta, couplings of the group's chains): honeycomb and ring graphs, different Nx and Nt, U in [1, 4]
GROUPS = [(("honeycomb", (2, 2)), 8, 2.0, [1.0, 2.5, 4.0]), (("ring", 6), 12, 3.0, [3.0]),
          (("honeycomb", (3, 3)), 16, 4.0, [2.0, 1.5, 3.5, 1.2]), (("ring", 10), 4, 1.0, [2.2, 3.3])]


def _lattice(spec):
    import nsl_gb300 as N

    kind, L = spec
    return N.Honeycomb(L) if kind == "honeycomb" else N.Ring(L)


def _setup(seed=5, real_force=True, nmd=5):
    from nsl_gb300.hmc import ChainEnsemble

    groups = [{"lattice": _lattice(s), "Nt": Nt, "beta": beta, "U": U} for s, Nt, beta, U in GROUPS]
    ens = ChainEnsemble(groups, 1.0, nmd, seed=seed, real_force=real_force)
    rng = np.random.default_rng(seed)
    qs, ps = [], []
    for g in groups:
        Nx = g["lattice"].sites()
        n = len(g["U"])
        scale = np.sqrt(g["beta"] / g["Nt"] * np.asarray(g["U"]))[:, None, None]
        qs.append(rng.standard_normal((n, g["Nt"], Nx)) * scale + 0j)
        ps.append(rng.standard_normal((n, g["Nt"], Nx)) + 0j)
    return ens, groups, qs, ps


def _single(g, U, q, p, real_force, nmd):
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import Leapfrog, LeapfrogRealForce

    prm = {"Nt": g["Nt"], "beta": g["beta"], "mu": 0.0, "U": U}
    S = HubbardGaugeAction(prm) + HubbardFermionAction(g["lattice"], prm)
    lf = (LeapfrogRealForce if real_force else Leapfrog)(S, 1.0, nmd)
    q1, p1 = lf({"phi": q}, {"phi": p})
    return S, np.asarray(q1["phi"]), np.asarray(p1["phi"])


@pytest.mark.parametrize("real_force", [True, False])
def test_group_trajectories_equal_single_chains(real_force):
    nmd = 5
    ens, groups, qs, ps = _setup(real_force=real_force, nmd=nmd)
    runs = [ens.leapfrog(qs, ps) for _ in range(4)]  # eager, captured per group, one graph launch, replay
    for k in range(1, 4):
        for g in range(len(groups)):
            assert np.array_equal(runs[k][0][g], runs[0][0][g]) and np.array_equal(runs[k][1][g], runs[0][1][g])
    q1, p1 = runs[-1]
    for g, grp in enumerate(groups):
        for b, U in enumerate(grp["U"]):
            S, qs1, ps1 = _single(grp, U, qs[g][b], ps[g][b], real_force, nmd)
            assert rel_err(q1[g][b], qs1) < 1e-10, (g, b)
            assert rel_err(p1[g][b], ps1) < 1e-10, (g, b)


def test_group_against_oracle_and_actions():
    """One chain per group against the oracle's leapfrog with its U; the per-chain actions (nslg_hubbard_eval_batch_u)
    against the oracle's S = sum phi^2 / (2 U~) - log det M_P - log det M_H."""
    from oracle import nsl_oracle as O

    nmd = 5
    ens, groups, qs, ps = _setup(seed=8, nmd=nmd)
    for _ in range(3):
        q1, p1 = ens.leapfrog(qs, ps)
    S1 = ens.action(q1)
    for g, grp in enumerate(groups):
        K = grp["lattice"].hopping_matrix()
        for b in (0, len(grp["U"]) - 1):
            A = O.HubbardAction(K, grp["Nt"], grp["beta"], grp["U"][b])
            qo, po = O.leapfrog(A, qs[g][b], ps[g][b], 1.0, nmd, real_force=True)
            assert rel_err(q1[g][b], qo) < 1e-10, (g, b)
            assert rel_err(p1[g][b], po) < 1e-10, (g, b)
            So = A.eval(q1[g][b])
            assert abs(S1[g][b] - So) < 1e-10 * max(1.0, abs(So)), (g, b, S1[g][b], So)


def test_ensemble_delta_h_and_acceptance():
    """Three HMC steps of the whole ensemble from the same fields with fresh momenta (Nmd = 10): each step's Delta H
    per chain equals the oracle's Hamiltonian difference between the same two phase-space points (the chain's start
    and the GPU trajectory's end, its own U; 1e-10 relative to max(1, |H|)) and the oracle's own trajectory's Delta H
    (1e-6 relative: where a trajectory ends near a singular M, Delta H reaches 1e3..1e4 and the 1e-10 agreement of the
    two trajectories' end points moves it by up to 1e-8 relative); the acceptance rates of a short generate() are in
    [0, 1]. (Proposals are not chained, so the fields stay well inside the sampled region.)"""
    import torch

    from oracle import nsl_oracle as O

    nmd = 10
    ens, groups, qs, _ = _setup(seed=11, nmd=nmd)
    q = [torch.from_numpy(x).cuda() for x in qs]
    S = ens.action(q)
    for _ in range(3):
        p0 = ens.momenta(q)
        q1, p1 = ens.leapfrog(q, p0)
        S1 = ens.action(q1)
        for g, grp in enumerate(groups):
            K = grp["lattice"].hopping_matrix()
            for b, U in enumerate(grp["U"]):
                A = O.HubbardAction(K, grp["Nt"], grp["beta"], U)
                qn, pn = q[g][b].cpu().numpy(), p0[g][b].cpu().numpy()
                qo, po = O.leapfrog(A, qn, pn, 1.0, nmd, real_force=True)
                q1n, p1n = q1[g][b].cpu().numpy(), p1[g][b].cpu().numpy()
                H0o = O.hamiltonian(A.eval(qn), pn)
                H1o = O.hamiltonian(A.eval(q1n), p1n)  # the oracle at the GPU trajectory's end point
                dHo = O.hamiltonian(A.eval(qo), po) - H0o
                H0 = S[g][b] + 0.5 * np.sum(pn ** 2)
                H1 = S1[g][b] + 0.5 * np.sum(p1n ** 2)
                scale = max(1.0, abs(H0o), abs(H1o))
                assert abs(H0 - H0o) < 1e-10 * scale and abs(H1 - H1o) < 1e-10 * scale, (g, b, H0 - H0o, H1 - H1o)
                assert abs((H1 - H0) - dHo) < 1e-6 * max(1.0, abs(dHo)), (g, b, H1 - H0, dHo)
    qf, rates = ens.generate(q, 2)
    assert len(qf) == len(groups) and all(tuple(a.shape) == tuple(b.shape) for a, b in zip(qf, q))
    for r in rates:
        assert np.all((r >= 0) & (r <= 1))


def test_group_argument_checks():
    """Handles of different contexts, a handle listed twice and a zero coupling are NSLG_ERR_ARG, before any launch."""
    import ctypes as C

    import nsl_gb300 as N
    from nsl_gb300 import _lib

    lat = N.Honeycomb((2, 2))
    a = N.HubbardExp(lat, 4, 1.0)
    b = N.HubbardExp(lat, 4, 1.0, ctx=N.Context(0))
    q = np.zeros((1, 4, 8), dtype=np.complex128)
    u = np.array([0.5 + 0j])
    uz = np.array([0j])

    def call(fms, U):
        ng = len(fms)
        P = C.c_void_p * ng
        return _lib.load().nslg_leapfrog_group(ng, P(*[f.handle for f in fms]), (C.c_int64 * ng)(*([1] * ng)),
                                               P(*([q.ctypes.data] * ng)), P(*([q.ctypes.data] * ng)),
                                               P(*([q.ctypes.data] * ng)), P(*([q.ctypes.data] * ng)),
                                               P(*([U.ctypes.data] * ng)), 1.0, 2, 0, 1, 3)

    assert call([a, b], u) == _lib.ERR_ARG
    assert call([a, a], u) == _lib.ERR_ARG
    assert call([a], uz) == _lib.ERR_ARG
