"""Host logic of the two-point correlator (source placement, source-time shifts with the anti-periodic sign, averaging
and the momentum projection of measureK) on the CPU: the batched solve is replaced by a fake that inverts the oracle's
dense M M^dagger, so the glue around the device solve is checked against the reference's own outputs (golden fixtures
from TwoPointCorrelator::measure and measureK, twoPointCorrelationFunction.tpp:116-233)."""
import numpy as np
import pytest

from conftest import TWOPOINT_CASES, load_twopoint, rel_err
from oracle import nsl_oracle as O


class FakeFermionMatrix:
    """populate / Mdagger / Nt / Nx of the product's fermion matrix, evaluated by the oracle."""

    def __init__(self, g):
        self.o = O.HubbardExp(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
        self.Nt, self.Nx = g["Nt"], g["Nx"]
        self.populated = []

    def populate(self, phi, species):
        self.populated.append(int(species))
        self.o.populate(np.asarray(phi), int(species))

    def Mdagger(self, x):
        return self.o.Mdagger(x)


class FakeCG:
    """x = (M M^dagger)^{-1} b for every stacked right-hand side, from the dense matrix."""

    calls = []

    def __init__(self, hfm, combination, eps, maxIter, **kw):
        self.hfm = hfm
        self.stats = {"converged": 0}

    def __call__(self, b):
        FakeCG.calls.append(b.shape)
        n = self.hfm.Nt * self.hfm.Nx
        M = self.hfm.o.M_dense().reshape(n, n)
        x = np.linalg.solve(M @ M.conj().T, b.reshape(b.shape[0], n).T).T
        self.stats = {"converged": b.shape[0], "systems": b.shape[0]}
        return x.reshape(b.shape)


@pytest.fixture
def fake_solver(monkeypatch):
    from nsl_gb300 import measurement

    FakeCG.calls = []
    monkeypatch.setattr(measurement, "CG", FakeCG)
    return FakeCG


@pytest.mark.parametrize("name", TWOPOINT_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_measure_and_measureK_host_logic(fake_solver, name, species, tag):
    from nsl_gb300.fermion_matrix import Species
    from nsl_gb300.measurement import TwoPointCorrelator

    assert int(Species.Particle) == O.PARTICLE and int(Species.Hole) == O.HOLE
    g = load_twopoint(name)
    hfm = FakeFermionMatrix(g)
    tp = TwoPointCorrelator(hfm, Species(species), wallSources=g["wall"])
    corr = tp.measure(g["phi"], g["nts"])
    assert rel_err(corr, g["corr_" + tag]) < 5e-12
    nk, nb = g["wall"].shape[:2]
    ntsrc = len(tp.source_times(g["nts"]))
    # one batched solve of Nx point sources per source time
    assert fake_solver.calls[-1] == (ntsrc * g["Nx"], g["Nt"], g["Nx"])
    blocks = tp.measureK_blocks(g["phi"], g["nts"])
    assert blocks.shape == (nk, g["Nt"], nb, nb)
    assert rel_err(blocks, g["block_" + tag]) < 5e-12
    # every momentum and source time in one solve
    assert fake_solver.calls[-1] == (nk * ntsrc * nb, g["Nt"], g["Nx"])
    one = tp.measureK(g["phi"], nk - 1, g["nts"])
    assert rel_err(one, g["block_" + tag][nk - 1]) < 5e-12
    assert fake_solver.calls[-1] == (ntsrc * nb, g["Nt"], g["Nx"])
    assert set(hfm.populated) == {species}


def test_source_times_follow_the_reference_loop(fake_solver):
    """tsrcStep = Nt / NumberTimeSources (integer), tsrc = 0, step, ... < Nt; the average divides by
    NumberTimeSources even where the loop visits more source times (Nt = 8, 3 sources: 0, 2, 4, 6)."""
    from nsl_gb300.measurement import TwoPointCorrelator

    g = load_twopoint("twopoint_honey3x3_nt8")
    hfm = FakeFermionMatrix(g)
    tp = TwoPointCorrelator(hfm, wallSources=g["wall"])
    assert tp.source_times(4) == [0, 2, 4, 6]
    assert tp.source_times(3) == [0, 2, 4, 6]
    assert tp.source_times(8) == list(range(8))
    assert tp.source_times(16) == list(range(8))
    h = O.HubbardExp(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
    want = O.two_point_correlator(h, g["phi"], O.PARTICLE, 3)
    assert rel_err(tp.measure(g["phi"], 3), want) < 1e-12
    want_k = O.two_point_correlator_k(h, g["phi"], O.PARTICLE, g["wall"], 1, 3)
    assert rel_err(tp.measureK(g["phi"], 1, 3), want_k) < 1e-12


def test_wall_source_placement_and_errors():
    from nsl_gb300.measurement import TwoPointCorrelator

    g = load_twopoint("twopoint_honey2x2_nt6_mu")
    hfm = FakeFermionMatrix(g)
    tp = TwoPointCorrelator(hfm, wallSources=g["wall"])
    b = tp.wall_sources([2, 0], [0, 3])
    nb = g["wall"].shape[1]
    assert b.shape == (2 * 2 * nb, g["Nt"], g["Nx"])
    b = b.reshape(2, 2, nb, g["Nt"], g["Nx"])
    assert np.array_equal(b[0, 1, :, 3], g["wall"][2])
    assert np.array_equal(b[1, 0, :, 0], g["wall"][0])
    assert np.count_nonzero(np.abs(b).sum(axis=-1)) == 2 * 2 * nb  # one time slice per source
    with pytest.raises(ValueError):
        TwoPointCorrelator(hfm, wallSources=g["wall"][:, :, :-1])
    with pytest.raises(ValueError):
        TwoPointCorrelator(hfm).measureK(g["phi"], 0, 1)


def test_non_interacting_defaults(fake_solver):
    """measure() and measureK_blocks() without a configuration: phi = 0 and one source time (the reference's
    NonInteracting nodes); a configuration without NumberTimeSources is an error."""
    from nsl_gb300.fermion_matrix import Species
    from nsl_gb300.measurement import TwoPointCorrelator

    g = load_twopoint("twopoint_honey2x2_nt6_mu")
    hfm = FakeFermionMatrix(g)
    tp = TwoPointCorrelator(hfm, Species.Hole, wallSources=g["wall"])
    h = O.HubbardExp(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
    zero = np.zeros((g["Nt"], g["Nx"]), dtype=np.complex128)
    assert rel_err(tp.measure(), O.two_point_correlator(h, zero, O.HOLE, 1)) < 1e-12
    assert fake_solver.calls[-1] == (g["Nx"], g["Nt"], g["Nx"])
    want = np.stack([O.two_point_correlator_k(h, zero, O.HOLE, g["wall"], k, 1) for k in range(g["wall"].shape[0])])
    assert rel_err(tp.measureK_blocks(), want) < 1e-12
    with pytest.raises(TypeError):
        tp.measure(g["phi"])
