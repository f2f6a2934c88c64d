"""Pins the CPU oracle (oracle/nsl_oracle.py) to the reference NSL implementation.

The fixtures in tests/golden/ were produced by the reference's own code (tests/golden/make_golden.py drives
oracle/ref_harness/golden_harness.cpp). Bar: the reference's own tolerances where it states them
(Tests/FermionMatrix/test_fermionMatrixHubbardExp.cpp uses digits10 = 1e-14 relative for M), relaxed to what two
correct FP64 evaluations of an ill-conditioned product can agree on for logdet / gradient / CG.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, TWOBODY_CASES, TWOPOINT_CASES, load_golden, load_twobody, load_twopoint, rel_err
from oracle import nsl_oracle as O


def lattice_hops(g):
    spec = g["lattice_spec"]
    return O.ring_hops(int(spec[1])) if spec[0] == "ring" else O.honeycomb_hops(int(spec[1]), int(spec[2]))


def mod2pi(z):
    return complex(z.real, (z.imag + np.pi) % (2 * np.pi) - np.pi)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_lattice_and_expK(name):
    g = load_golden(name)
    K = lattice_hops(g)
    assert np.array_equal(K, g["hops"])
    d = g["beta"] / g["Nt"]
    assert rel_err(O.exp_hopping_matrix(K, d), g["expK_pos"]) < 1e-14
    assert rel_err(O.exp_hopping_matrix(K, -d), g["expK_neg"]) < 1e-14


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(O.PARTICLE, "P"), (O.HOLE, "H")])
def test_operators(name, species, tag):
    g = load_golden(name)
    h = O.HubbardExp(lattice_hops(g), g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], species)
    for fn, key in (("M", "M"), ("Mdagger", "Mdag"), ("MMdagger", "MMdag"), ("MdaggerM", "MdagM")):
        assert rel_err(getattr(h, fn)(g["psi"]), g[f"{key}_{tag}"]) < 1e-14, fn


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(O.PARTICLE, "P"), (O.HOLE, "H")])
def test_logdet_and_grad(name, species, tag):
    g = load_golden(name)
    h = O.HubbardExp(lattice_hops(g), g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], species)
    ref = complex(g[f"logdet_{tag}"])
    assert abs(h.logDetM() - ref) <= 1e-11 * max(1.0, abs(ref))
    # LU log-sum and the stratified product agree with the reference modulo 2 pi i
    for alt in (h.logDetM_lu(), h.logDetM_stable()):
        assert abs(mod2pi(alt - ref)) <= 1e-9 * max(1.0, abs(ref))
    assert rel_err(h.gradLogDetM(), g[f"grad_{tag}"]) < 1e-8


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(O.PARTICLE, "P"), (O.HOLE, "H")])
def test_diag_discretisation(name, species, tag):
    """HubbardDiag (hubbardDiag.tpp): operators (the reference's expanded MM^dagger / M^dagger M, and their
    equality with the compositions), log det (not folded to the principal branch: i sgn sum(phi) is added as is)
    and its gradient."""
    g = load_golden(name)
    h = O.HubbardDiag(lattice_hops(g), g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], species)
    for fn, key in (("M", "M"), ("Mdagger", "Mdag"), ("MMdagger", "MMdag"), ("MdaggerM", "MdagM")):
        assert rel_err(getattr(h, fn)(g["psi"]), g[f"diag_{key}_{tag}"]) < 1e-14, fn
    assert rel_err(h.M(h.Mdagger(g["psi"])), g[f"diag_MMdag_{tag}"]) < 1e-14
    assert rel_err(h.Mdagger(h.M(g["psi"])), g[f"diag_MdagM_{tag}"]) < 1e-14
    ref = complex(g[f"diag_logdet_{tag}"])
    assert abs(h.logDetM() - ref) <= 1e-11 * max(1.0, abs(ref))
    assert rel_err(h.gradLogDetM(), g[f"diag_grad_{tag}"]) < 1e-10


@pytest.mark.parametrize("name", [n for n in GOLDEN_CASES if "cg_x" in np.load(f"tests/golden/{n}.npz").files])
def test_cg_matches_reference(name):
    g = load_golden(name)
    h = O.HubbardExp(lattice_hops(g), g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], O.PARTICLE)
    x, iters, conv = O.cg(h.MMdagger, g["b"], float(g["cg_eps"]), 100000)
    assert conv
    assert abs(iters - int(g["cg_iters"])) <= max(2, int(0.02 * int(g["cg_iters"])))
    assert rel_err(x, g["cg_x"]) < 1e-9
    bn = np.linalg.norm(g["b"])
    assert np.linalg.norm(g["b"] - h.MMdagger(x)) / bn < 1e-10


@pytest.mark.parametrize("name", [n for n in GOLDEN_CASES if "lf_q" in np.load(f"tests/golden/{n}.npz").files])
def test_action_force_leapfrog(name):
    g = load_golden(name)
    A = O.HubbardAction(lattice_hops(g), g["Nt"], g["beta"], g["U"], g["mu"])
    assert abs(A.eval(g["phi"]) - complex(g["S"])) <= 1e-11 * abs(complex(g["S"]))
    assert rel_err(A.force(g["phi"]), g["force"]) < 1e-10
    for real_force, qk, pk in ((False, "lf_q", "lf_p"), (True, "lfr_q", "lfr_p")):
        q, p = O.leapfrog(A, g["phi"], g["p"], float(g["traj"]), int(g["nmd"]), real_force=real_force)
        assert rel_err(q, g[qk]) < 1e-10
        assert rel_err(p, g[pk]) < 1e-10


def test_m_dense_and_identities():
    """The reference's self-consistency identities on a small ring (test_fermionMatrixHubbardExp.cpp:184-356)."""
    rng = np.random.default_rng(5)
    K = O.ring_hops(4)
    h = O.HubbardExp(K, 6, 2.0)
    phi = rng.random((6, 4)) + 1j * rng.random((6, 4))
    psi = rng.random((6, 4)) + 1j * rng.random((6, 4))
    h.populate(phi)
    D = h.M_dense().reshape(24, 24)
    assert rel_err((D @ psi.reshape(-1)).reshape(6, 4), h.M(psi)) < 1e-14
    assert rel_err((D.conj().T @ psi.reshape(-1)).reshape(6, 4), h.Mdagger(psi)) < 1e-14
    assert rel_err(h.MMdagger(psi), h.M(h.Mdagger(psi))) < 1e-13
    assert rel_err(h.MdaggerM(psi), h.Mdagger(h.M(psi))) < 1e-13
    # logdet M of the dense matrix equals log det(1 + prod B) (exact identity of the block-cyclic structure)
    s, l = np.linalg.slogdet(D)
    ld = h.logDetM()
    assert abs(mod2pi(complex(l + np.log(s)) - ld)) < 1e-12 * max(1, abs(ld))


@pytest.mark.parametrize("name", TWOBODY_CASES)
def test_two_body_correlator_vs_reference(name):
    """The oracle's two-body correlator (exact inverses) against the reference's TwoBodyCorrelator::measure
    (its own CG at eps 1e-12): the momentum keys it allocated and all twelve channels."""
    g = load_twobody(name)
    assert np.array_equal(O.twobody_tuples(g["momenta"]), g["tuples"])
    mom, W = O.honeycomb_wall_sources(*g["L"])
    # the fixture's wall sources are a subset of the lattice momenta
    idx = [int(np.argmin(np.abs(mom - k).sum(axis=1))) for k in g["momenta"]]
    assert rel_err(W[idx], g["wall"]) < 1e-15
    h = O.HubbardExp(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
    out = O.two_body_correlator(h, g["phi"], g["wall"], g["tuples"], g["nts"])
    assert rel_err(out, g["out"]) < 5e-12


@pytest.mark.parametrize("name", TWOPOINT_CASES)
@pytest.mark.parametrize("species,tag", [(O.PARTICLE, "P"), (O.HOLE, "H")])
def test_two_point_correlator_vs_reference(name, species, tag):
    """The oracle's two-point correlators (exact inverses) against the reference's TwoPointCorrelator (its own CG at
    eps 1e-12 over the source batch): measure(nts) with point sources and measureK(k, nts) for every wall source.
    On the reference's own outputs the momentum block is the point-source correlator projected on the wall sources,
    block[k] = W[k]^* corr W[k]^T."""
    g = load_twopoint(name)
    h = O.HubbardExp(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
    corr = O.two_point_correlator(h, g["phi"], species, g["nts"])
    assert rel_err(corr, g["corr_" + tag]) < 5e-12
    W = g["wall"]
    block = np.stack([O.two_point_correlator_k(h, g["phi"], species, W, k, g["nts"]) for k in range(W.shape[0])])
    assert rel_err(block, g["block_" + tag]) < 5e-12
    proj = np.einsum("kay,tyx,kbx->ktab", np.conj(W), g["corr_" + tag], W)
    assert rel_err(proj, g["block_" + tag]) < 5e-12


def test_eq_mod_bz():
    """eq_modBZ_ (twoBodyCorrelationFunction.tpp:101-135): reciprocal-lattice shifts are equal, others not."""
    C = np.array([4 * np.pi / 3, 0.0])
    D = np.array([-2 * np.pi / 3, 2 * np.pi / np.sqrt(3.0)])
    k = np.array([0.3, -0.7])
    assert O.eq_modBZ(k, k + 2 * C - 3 * D)
    assert not O.eq_modBZ(k, k + 0.5 * C)
    assert not O.eq_modBZ(k, k + np.array([1e-6, 0.0]))


def test_free_density_and_particle_hole_symmetry():
    """The equal-time observables' definitions on the free theory (phi = 0): half filling n = 1 at mu = 0 on a
    bipartite lattice, n(mu) + n(-mu) = 2, and d = n_up n_down = (n / 2)^2 at mu = 0 (both spins half filled)."""
    K = O.honeycomb_hops(2, 2)
    zero = np.zeros((8, 8), dtype=np.complex128)
    n0, d0 = O.density_double_occupancy(O.HubbardExp(K, 8, 2.0, 0.0), zero)
    assert np.abs(n0 - 1.0).max() < 1e-13
    assert np.abs(d0 - 0.25).max() < 1e-13
    n_p, _ = O.density_double_occupancy(O.HubbardExp(K, 8, 2.0, 0.3), zero)
    n_m, _ = O.density_double_occupancy(O.HubbardExp(K, 8, 2.0, -0.3), zero)
    assert np.abs(n_p + n_m - 2.0).max() < 1e-13
    assert n_p.real.min() > 1.0
