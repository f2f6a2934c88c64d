"""GPU log det M, its gradient, the Hubbard actions, forces and leapfrog trajectories vs the reference.

Bars (FP64): log det to 1e-10 relative modulo 2 pi i (the reference's value is the principal branch of
log(det(.))); gradient and force to 1e-10 max-norm relative on the golden cases (the products they involve are
ill-conditioned at beta >= 4, so the bar sits above the 1e-12 of the operators); leapfrog q, p to 1e-9.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, rel_err

pytestmark = pytest.mark.gpu


def make(g):
    import nsl_gb300 as N

    spec = g["lattice_spec"]
    lat = N.Ring(int(spec[1])) if spec[0] == "ring" else N.Honeycomb((int(spec[1]), int(spec[2])))
    return N, lat


def params(g):
    return {"Nt": g["Nt"], "beta": g["beta"], "mu": g["mu"], "U": g["U"]}


def mod2pi(z):
    return complex(z.real, (z.imag + np.pi) % (2 * np.pi) - np.pi)


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_logdet_and_grad(name, species, tag):
    g = load_golden(name)
    N, lat = make(g)
    hfm = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    hfm.populate(g["phi"], N.Species(species))
    ref = complex(g[f"logdet_{tag}"])
    ld = hfm.logDetM()
    assert abs(mod2pi(ld - ref)) <= 1e-10 * max(1.0, abs(ref)), (ld, ref)
    assert -np.pi < ld.imag <= np.pi
    # the reference's own oracle-vs-libtorch spread is 5.6e-10 at beta = 8 (products of exp(+-delta K) with
    # condition ~e^{3 beta}); below beta = 8 both agree to 1e-12
    assert rel_err(hfm.gradLogDetM(), g[f"grad_{tag}"]) < (1e-10 if g["beta"] < 8 else 2e-9)


@pytest.mark.parametrize("name", [n for n in GOLDEN_CASES if "lf_q" in np.load(f"tests/golden/{n}.npz").files])
def test_action_force_leapfrog(name):
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import Leapfrog, LeapfrogRealForce

    g = load_golden(name)
    N, lat = make(g)
    S = HubbardGaugeAction(params(g)) + HubbardFermionAction(lat, params(g))
    q = {"phi": g["phi"]}
    assert abs(S(q) - complex(g["S"])) <= 1e-10 * abs(complex(g["S"]))
    assert rel_err(S.force(q)["phi"], g["force"]) < 1e-10
    for cls, qk, pk in ((Leapfrog, "lf_q", "lf_p"), (LeapfrogRealForce, "lfr_q", "lfr_p")):
        q1, p1 = cls(S, float(g["traj"]), int(g["nmd"]))(q, {"phi": g["p"]})
        assert rel_err(q1["phi"], g[qk]) < 1e-9, cls.__name__
        assert rel_err(p1["phi"], g[pk]) < 1e-9, cls.__name__


def test_force_is_real_for_real_phi():
    """Tests/Action/test_force.cpp:72: Im(force) == 0 for real phi (mu = 0)."""
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction

    g = load_golden("honey3x3_nt16")
    N, lat = make(g)
    S = HubbardGaugeAction(params(g)) + HubbardFermionAction(lat, params(g))
    F = S.force({"phi": g["phi"]})["phi"]
    assert np.abs(F.imag).max() < 1e-10 * np.abs(F).max()


def test_force_finite_differences():
    """Tests/Action/test_force.cpp:24-100: grad S against finite differences of S (ring Nx=2, Nt=8, beta=2, U=3)."""
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction

    N = __import__("nsl_gb300")
    lat = N.Ring(2)
    p = {"Nt": 8, "beta": 2.0, "mu": 0.0, "U": 3.0}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    rng = np.random.default_rng(4)
    phi = rng.standard_normal((8, 2)) * (2.0 / 8 * 3.0) + 0j
    grad = S.grad({"phi": phi})["phi"]
    eps = 1e-6
    S0 = S({"phi": phi})
    for t in range(8):
        for x in range(2):
            e = phi.copy()
            e[t, x] += eps
            fd = (S({"phi": e}) - S0) / eps
            assert abs(fd - grad[t, x]) < 1e-4


def test_leapfrog_reversible_and_energy():
    """Tests/Integrator/test_leapfrog.cpp:61-128 (gauge action): forward then backward returns (q, p); the energy
    violation falls like eps^2."""
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import Leapfrog

    N = __import__("nsl_gb300")
    lat = N.Honeycomb((2, 2))
    p = {"Nt": 8, "beta": 2.0, "mu": 0.0, "U": 2.0}
    S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p)
    rng = np.random.default_rng(8)
    q0 = rng.standard_normal((8, 8)) * 0.5 + 0j
    p0 = rng.standard_normal((8, 8)) + 0j
    q1, p1 = Leapfrog(S, 1.0, 10)({"phi": q0}, {"phi": p0})
    q2, p2 = Leapfrog(S, 1.0, 10, backward=True)(q1, p1)
    assert rel_err(q2["phi"], q0) < 1e-11 and rel_err(p2["phi"], p0) < 1e-11
    dH = []
    for nmd in (10, 20, 40):
        qa, pa = Leapfrog(S, 1.0, nmd)({"phi": q0}, {"phi": p0})
        H0 = S({"phi": q0}) + 0.5 * np.sum(p0 * p0)
        H1 = S(qa) + 0.5 * np.sum(pa["phi"] * pa["phi"])
        dH.append(abs((H1 - H0).real))
    assert dH[1] < dH[0] / 3 and dH[2] < dH[1] / 3


def test_gauge_only_leapfrog():
    from nsl_gb300.action import HubbardGaugeAction
    from nsl_gb300.integrator import Leapfrog
    from oracle import nsl_oracle as O

    p = {"Nt": 4, "beta": 1.0, "U": 2.0}
    S = HubbardGaugeAction(p)
    rng = np.random.default_rng(1)
    q0 = rng.standard_normal((4, 3)) + 0j
    p0 = rng.standard_normal((4, 3)) + 0j
    q1, p1 = Leapfrog(S, 1.0, 7)({"phi": q0}, {"phi": p0})

    class G:
        Ut = O.utilde(1.0, 4, 2.0)

        def force(self, x):
            return O.gauge_force(x, self.Ut)

    qo, po = O.leapfrog(G(), q0, p0, 1.0, 7)
    assert rel_err(q1["phi"], qo) < 1e-13 and rel_err(p1["phi"], po) < 1e-13


@pytest.mark.parametrize("name", ["honey3x3_nt16", "honey6x6_nt32_beta8"])
def test_leapfrog_graph_replay_matches_eager(name):
    """The first trajectory of a shape runs eagerly, the second is captured into a CUDA graph, later ones replay it:
    all give the reference's trajectory and are bitwise equal to one another (and the species state after a
    replayed trajectory is the one an eager trajectory leaves, so ordinary calls work after it)."""
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import LeapfrogRealForce

    g = load_golden(name)
    N, lat = make(g)
    fa = HubbardFermionAction(lat, params(g))
    S = HubbardGaugeAction(params(g)) + fa
    q = {"phi": g["phi"]}
    lf = LeapfrogRealForce(S, float(g["traj"]) if "traj" in g else 1.0, int(g["nmd"]) if "nmd" in g else 5)
    outs = [lf(q, {"phi": g["p"] if "p" in g else np.ones_like(g["phi"])}) for _ in range(4)]
    for q1, p1 in outs[1:]:
        assert np.array_equal(q1["phi"], outs[0][0]["phi"]) and np.array_equal(p1["phi"], outs[0][1]["phi"])
    if "lfr_q" in g:
        assert rel_err(outs[-1][0]["phi"], g["lfr_q"]) < 1e-9
        assert rel_err(outs[-1][1]["phi"], g["lfr_p"]) < 1e-9
    if "S" in g:  # the handle stays usable for ordinary calls after replays
        assert abs(S(q) - complex(g["S"])) <= 1e-10 * abs(complex(g["S"]))


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_tensor_core_gradient(name, species, tag):
    """gradLogDetM with its two matrix chains as split-BF16 tensor-core products (force precision "bf16split")
    against the reference's FP64 gradient: FP64-class, bar 1e-8 (5e-8 at beta = 8, where the 2 (Nt - 1) chained
    products of the ill-conditioned slices compound the ~1e-13 error of each product; measured 2.2e-8 there). The
    FP64 path meets 1e-10 (2e-9 at beta = 8)."""
    g = load_golden(name)
    N, lat = make(g)
    hfm = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    hfm.set_force_precision("bf16split")
    hfm.set_stabilisation("plain")  # the split-BF16 chains belong to the direct-product form
    hfm.populate(g["phi"], N.Species(species))
    assert rel_err(hfm.gradLogDetM(), g[f"grad_{tag}"]) < (5e-8 if g["beta"] >= 8 else 1e-8)
    hfm.set_force_precision("fp64")
    bar = 2e-9 if g["beta"] >= 8 else 1e-10
    assert rel_err(hfm.gradLogDetM(), g[f"grad_{tag}"]) < bar


def test_tensor_core_force_leapfrog():
    """A leapfrog trajectory with the tensor-core force stays within 1e-8 of the reference's FP64 trajectory; the
    action value (Delta H) is FP64 either way."""
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import LeapfrogRealForce

    g = load_golden("honey3x3_nt16")
    N, lat = make(g)
    S = HubbardGaugeAction(params(g)) + HubbardFermionAction(lat, params(g), force_precision="bf16split")
    q = {"phi": g["phi"]}
    for _ in range(3):  # eager, captured, replayed
        q1, p1 = LeapfrogRealForce(S, float(g["traj"]), int(g["nmd"]))(q, {"phi": g["p"]})
        assert rel_err(q1["phi"], g["lfr_q"]) < 1e-8
        assert rel_err(p1["phi"], g["lfr_p"]) < 1e-8
    assert abs(S(q) - complex(g["S"])) <= 1e-10 * abs(complex(g["S"]))


@pytest.mark.parametrize("name", ["honey3x3_nt16", "honey6x6_nt32_beta8"])
def test_tensor_core_force_pair_equals_species_gradients(name):
    """The split-BF16 force evaluates both species as a pair (one batched LU, the hole chains on a side stream): it
    equals -(grad_P - grad_H) of the one-species tensor-core gradients and differs from the FP64 force at the
    split-BF16 level. Lattices of at most 32 sites take the FP64 pair force at either precision."""
    from nsl_gb300.action import HubbardFermionAction

    g = load_golden(name)
    N, lat = make(g)
    F = {}
    for fp in ("fp64", "bf16split"):
        S = HubbardFermionAction(lat, params(g), force_precision=fp, stabilisation="plain")
        F[fp] = np.asarray(S.force({"phi": g["phi"]})["phi"])
    hfm = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    hfm.set_force_precision("bf16split")
    hfm.set_stabilisation("plain")
    gr = []
    for sp in (N.Species.Particle, N.Species.Hole):
        hfm.populate(g["phi"], sp)
        gr.append(np.asarray(hfm.gradLogDetM()))
    if g["Nx"] <= 32:
        assert rel_err(F["bf16split"], F["fp64"]) == 0.0
        assert rel_err(F["bf16split"], -(gr[0] - gr[1])) < 1e-8
        return
    assert rel_err(F["bf16split"], -(gr[0] - gr[1])) < 1e-12
    d = rel_err(F["bf16split"], F["fp64"])
    assert 0 < d < (5e-8 if g["beta"] >= 8 else 1e-8), d


@pytest.mark.parametrize("L,Nt", [((5, 5), 8), ((4, 4), 6)])
def test_logdet_gradient_mid_sizes(L, Nt):
    """Lattices between the small-matrix forms (<= 32 sites: Gauss-Jordan inverse, scans) and the 8-column LU
    (> 64 sites): 50 sites factor in two 32-column panels; log det, its gradient (both species) and the force
    against the oracle."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction
    from oracle import nsl_oracle as O

    lat = N.Honeycomb(L)
    Nx = lat.sites()
    beta, mu = 2.0, 0.1
    rng = np.random.default_rng(29)
    phi = rng.standard_normal((Nt, Nx)) * 0.4 + 0j
    hfm = N.HubbardExp(lat, Nt, beta, mu)
    ho = O.HubbardExp(lat.hopping_matrix(), Nt, beta, mu)
    grads = []
    for sp, osp in ((N.Species.Particle, O.PARTICLE), (N.Species.Hole, O.HOLE)):
        hfm.populate(phi, sp)
        ho.populate(phi, osp)
        ld, ld_o = hfm.logDetM(), ho.logDetM()
        assert abs(ld - ld_o) <= 1e-10 * max(1.0, abs(ld_o))
        g_o = ho.gradLogDetM()
        assert rel_err(hfm.gradLogDetM(), g_o) < 1e-10
        grads.append(g_o)
    F = np.asarray(HubbardFermionAction(lat, {"Nt": Nt, "beta": beta, "mu": mu}).force({"phi": phi})["phi"])
    assert rel_err(F, -(grads[0] - grads[1])) < 1e-10
