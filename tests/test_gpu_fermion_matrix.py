"""GPU parity of the fermion-matrix applications against the reference (golden fixtures) and the oracle.

FP64 bar: 1e-12 max-norm relative error (the reference's own M tests use digits10, test_fermionMatrixHubbardExp.cpp).
FP32 inner operator bar: 1e-5 relative (single-precision products over Nx terms).
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, rel_err

pytestmark = pytest.mark.gpu

OPS = (("M", "M"), ("Mdagger", "Mdag"), ("MMdagger", "MMdag"), ("MdaggerM", "MdagM"))


def make_lattice(g):
    from nsl_gb300.lattice import Honeycomb, Ring

    spec = g["lattice_spec"]
    return Ring(int(spec[1])) if spec[0] == "ring" else Honeycomb((int(spec[1]), int(spec[2])))


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_operators_vs_reference(name, species, tag):
    import nsl_gb300 as N

    g = load_golden(name)
    hfm = N.HubbardExp(make_lattice(g), g["Nt"], g["beta"], g["mu"])
    hfm.populate(g["phi"], N.Species(species))
    for fn, key in OPS:
        out = getattr(hfm, fn)(g["psi"])
        assert rel_err(out, g[f"{key}_{tag}"]) < 1e-12, fn


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_exp_hopping_matrix_vs_reference(name):
    import nsl_gb300 as N

    g = load_golden(name)
    hfm = N.HubbardExp(make_lattice(g), g["Nt"], g["beta"], g["mu"])
    d = g["beta"] / g["Nt"]
    assert rel_err(hfm.exp_hopping_matrix(d), g["expK_pos"]) < 1e-13
    assert rel_err(hfm.exp_hopping_matrix(-d), g["expK_neg"]) < 1e-13


def test_installed_reference_exp_matches():
    """With the reference's own exp(delta K) installed (its memo entry), results agree to rounding."""
    import nsl_gb300 as N

    g = load_golden("honey3x3_nt16")
    lat = make_lattice(g)
    d = g["beta"] / g["Nt"]
    lat.set_exp_hopping_matrix(d, g["expK_pos"])
    hfm = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    hfm.populate(g["phi"])
    assert rel_err(hfm.M(g["psi"]), g["M_P"]) < 1e-14


def test_torch_cuda_tensors_and_batch_dims():
    import torch

    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    g = load_golden("honey6x6_nt32_beta8")
    hfm = N.HubbardExp(make_lattice(g), g["Nt"], g["beta"])
    phi = torch.from_numpy(g["phi"]).cuda()
    hfm.populate(phi)
    rng = np.random.default_rng(3)
    psi = rng.standard_normal((2, 3, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((2, 3, g["Nt"], g["Nx"]))
    out = hfm.MMdagger(torch.from_numpy(psi).cuda())
    assert out.is_cuda and tuple(out.shape) == psi.shape
    h = O.HubbardExp(g["hops"], g["Nt"], g["beta"])
    h.populate(g["phi"])
    assert rel_err(out.cpu().numpy(), h.MMdagger(psi)) < 1e-12


@pytest.mark.parametrize("L,Nt,beta,R", [((12, 12), 64, 8.0, 4), ((8, 8), 16, 2.0, 7), ((5, 5), 33, 3.0, 3),
                                         ((24, 24), 128, 12.0, 1)])
def test_operators_vs_oracle_larger(L, Nt, beta, R):
    """Larger and ragged shapes (Nx, Nt*R not multiples of the tile) against the oracle, up to the honeycomb 24x24,
    Nt = 128, beta = 12 configuration (Nx = 1152)."""
    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    lat = N.Honeycomb(L)
    rng = np.random.default_rng(7)
    Nx = lat.sites()
    phi = rng.standard_normal((Nt, Nx)) * np.sqrt(beta / Nt * 3.0) + 0j
    psi = rng.standard_normal((R, Nt, Nx)) + 1j * rng.standard_normal((R, Nt, Nx))
    hfm = N.HubbardExp(lat, Nt, beta)
    hfm.populate(phi)
    h = O.HubbardExp(lat.hopping_matrix(), Nt, beta)
    h.populate(phi)
    for fn, _ in OPS:
        assert rel_err(getattr(hfm, fn)(psi), getattr(h, fn)(psi)) < 1e-12, fn
        assert rel_err(getattr(hfm, fn)(psi, precision="fp32"), getattr(h, fn)(psi)) < 2e-5, fn


def test_complex_hopping_matrix():
    """Complex kappa (ring with a twist) -> complex exp(delta K): the complex-by-complex product path."""
    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    lat = N.Ring(10, kappa=np.exp(0.3j))
    rng = np.random.default_rng(9)
    phi = rng.random((12, 10)) + 1j * rng.random((12, 10))
    psi = rng.standard_normal((2, 12, 10)) + 1j * rng.standard_normal((2, 12, 10))
    hfm = N.HubbardExp(lat, 12, 1.5, 0.1)
    hfm.populate(phi)
    h = O.HubbardExp(lat.hopping_matrix(), 12, 1.5, 0.1)
    h.populate(phi)
    for fn, _ in OPS:
        assert rel_err(getattr(hfm, fn)(psi), getattr(h, fn)(psi)) < 1e-12, fn


def test_batched_equals_single():
    """test_fermionMatrixHubbardExp.cpp:362-468: a batch equals its slices applied one by one."""
    import nsl_gb300 as N

    lat = N.Ring(8)
    rng = np.random.default_rng(11)
    phi = rng.random((10, 8)) + 0j
    psi = rng.random((10, 10, 8)) + 1j * rng.random((10, 10, 8))
    hfm = N.HubbardExp(lat, 10, 2.0)
    hfm.populate(phi)
    for fn, _ in OPS:
        full = getattr(hfm, fn)(psi)
        for n in range(10):
            assert np.array_equal(full[n], getattr(hfm, fn)(psi[n])), fn


def test_errors_are_reported():
    import nsl_gb300 as N
    from nsl_gb300._lib import NslgError

    lat = N.Ring(4)
    hfm = N.HubbardExp(lat, 4, 1.0)
    with pytest.raises(NslgError):
        hfm.M(np.zeros((4, 4), dtype=np.complex128))  # not populated
    hfm.populate(np.zeros((4, 4)))
    with pytest.raises(ValueError):
        hfm.M(np.zeros((3, 4), dtype=np.complex128))
    empty = hfm.M(np.zeros((0, 4, 4), dtype=np.complex128))
    assert empty.shape == (0, 4, 4)


@pytest.mark.parametrize("L,Nt,R", [((12, 12), 64, 4), ((3, 3), 16, 3), ((5, 5), 33, 2), ((2, 2), 8, 5),
                                    ((24, 24), 16, 1), ((8, 8), 12, 3)])
def test_split_bf16_operator(L, Nt, R):
    """Exact-accumulation split-BF16 tensor-core operator: FP64-class. Six balanced 9-bit digits carry 53 bits per
    operand, rounded to nearest, so the product's error is that of an FP64 product (~1e-15 of the output's maximum;
    bar 2e-14 against the oracle and against the device's FP64 operator, vs 2e-5 for the FP32-class operators);
    ragged tiles and K > 1024 (Nx = 1152) included."""
    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    beta = 4.0
    lat = N.Honeycomb(L)
    Nx = lat.sites()
    rng = np.random.default_rng(23)
    phi = rng.standard_normal((Nt, Nx)) * np.sqrt(beta / Nt * 3.0) + 0j
    psi = rng.standard_normal((R, Nt, Nx)) + 1j * rng.standard_normal((R, Nt, Nx))
    hfm = N.HubbardExp(lat, Nt, beta)
    hfm.populate(phi)
    h = O.HubbardExp(lat.hopping_matrix(), Nt, beta)
    h.populate(phi)
    for fn, _ in OPS:
        got = getattr(hfm, fn)(psi, precision="bf16split")
        assert rel_err(got, getattr(h, fn)(psi)) < 2e-14, fn
        assert rel_err(got, getattr(hfm, fn)(psi, precision="fp64")) < 2e-14, fn


def test_split_bf16_digit_bound_refuses_delocalised_exp():
    """exp(delta K) at delta = 4 on honeycomb 12x12 is delocalised: its digit sums can exceed FP32's exact range for
    some operand, so the split-BF16 operator reports an error instead of an inexact result (the FP64 operator still
    runs)."""
    import nsl_gb300 as N

    lat = N.Honeycomb((12, 12))
    Nt, beta = 2, 8.0
    Nx = lat.sites()
    rng = np.random.default_rng(5)
    hfm = N.HubbardExp(lat, Nt, beta)
    hfm.populate(rng.standard_normal((Nt, Nx)) * 0.1 + 0j)
    psi = rng.standard_normal((1, Nt, Nx)) + 0j
    with pytest.raises(RuntimeError, match="delocalised"):
        hfm.M(psi, precision="bf16split")
    hfm.M(psi, precision="fp64")
