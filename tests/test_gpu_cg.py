"""GPU CG against the reference's CG (golden fixtures) and the oracle.

Reference semantics (shared alpha/beta over the batch, recurrence stopping rule |r|^2 <= eps^2, x0 = b): the
solution matches the reference's to 1e-9 max-norm relative and the FP64 true residual is <= 1e-10 relative.
Per-RHS and mixed precision are checked on the true residual, which is what they guarantee.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def setup(name):
    import nsl_gb300 as N
    from nsl_gb300.lattice import Honeycomb, Ring

    g = load_golden(name)
    spec = g["lattice_spec"]
    lat = Ring(int(spec[1])) if spec[0] == "ring" else Honeycomb((int(spec[1]), int(spec[2])))
    hfm = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    hfm.populate(g["phi"], N.Species.Particle)
    return g, hfm


def true_res(hfm, b, x):
    r = b - hfm.MMdagger(x)
    return np.linalg.norm(r.reshape(r.shape[0], -1), axis=1) / np.linalg.norm(b.reshape(b.shape[0], -1), axis=1)


@pytest.mark.parametrize("name", ["ring2_nt8", "ring4_nt8", "honey2x2_nt6_mu", "honey3x3_nt16"])
def test_cg_reference_semantics(name):
    import nsl_gb300 as N

    g, hfm = setup(name)
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, float(g["cg_eps"]), 100000)
    x = cg(g["b"])
    assert cg.stats["converged"] == 1
    assert abs(cg.stats["iterations"] - int(g["cg_iters"])) <= max(2, int(0.02 * int(g["cg_iters"])))
    assert rel_err(x, g["cg_x"]) < 1e-9
    assert true_res(hfm, g["b"], x).max() < 1e-10


@pytest.mark.parametrize("precision,stop", [("fp64", "recurrence"), ("fp64", "true_residual"),
                                            ("fp32", "true_residual")])
def test_cg_per_rhs(precision, stop):
    import nsl_gb300 as N

    g, hfm = setup("honey3x3_nt16")
    b = g["b"]
    eps = 1e-10 * np.linalg.norm(b[0])
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, eps, 100000, mode="per_rhs", precision=precision, stop=stop)
    x = cg(b)
    assert cg.stats["converged"] == b.shape[0]
    assert true_res(hfm, b, x).max() < 2e-10
    assert rel_err(x, g["cg_x"]) < 1e-6


def test_cg_mixed_larger():
    """Honeycomb 6x6, Nt=32, beta=8: mixed precision reaches the 1e-10 relative true residual."""
    import nsl_gb300 as N

    g, hfm = setup("honey6x6_nt32_beta8")
    rng = np.random.default_rng(2)
    b = rng.standard_normal((3, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((3, g["Nt"], g["Nx"]))
    eps = 1e-10 * np.linalg.norm(b[0])
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, eps, 200000, mode="per_rhs", precision="fp32")
    x = cg(b)
    assert cg.stats["converged"] == 3
    assert cg.stats["reliable_updates"] >= 1
    assert true_res(hfm, b, x).max() < 1.5e-10


def test_cg_not_converged_returns_iterate():
    import nsl_gb300 as N

    g, hfm = setup("honey3x3_nt16")
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, 1e-14, 5)
    x = cg(g["b"])
    assert cg.stats["converged"] == 0 and cg.stats["iterations"] == 5
    assert np.all(np.isfinite(x))


def test_cg_zero_iterations_and_exact_guess():
    import nsl_gb300 as N

    g, hfm = setup("ring4_nt8")
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, 1e-12, 100000)
    x = cg(g["b"], g["cg_x"])  # a converged guess needs (almost) no iterations
    assert cg.stats["iterations"] <= 2
    assert rel_err(x, g["cg_x"]) < 1e-9


@pytest.mark.parametrize("op", ["M", "Mdagger", "MdaggerM"])
def test_cg_other_combinations(op):
    """CG on M^dagger M is a valid Hermitian solve; on M / M^dagger it follows the reference recurrence."""
    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    g, hfm = setup("ring2_nt8")
    comb = N.MatrixCombination[op]
    cg = N.CG(hfm, comb, 1e-12, 2000)
    x = cg(g["b"])
    h = O.HubbardExp(g["hops"], g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], O.PARTICLE)
    xo, it, conv = O.cg(getattr(h, op), g["b"], 1e-12, 2000)
    assert cg.stats["converged"] == int(conv)
    if conv:
        assert rel_err(x, xo) < 1e-8


def test_cg_tensor_core_mixed():
    """Mixed precision with the tcgen05 operator reaches the same FP64 true residual."""
    import nsl_gb300 as N

    g, hfm = setup("honey6x6_nt32_beta8")
    rng = np.random.default_rng(5)
    b = rng.standard_normal((4, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((4, g["Nt"], g["Nx"]))
    eps = 1e-10 * np.linalg.norm(b.reshape(4, -1), axis=1).min()
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, eps, 200000, mode="per_rhs", precision="tf32x3")
    x = cg(b)
    assert cg.stats["converged"] == 4
    assert true_res(hfm, b, x).max() < 1.5e-10


def test_cg_split_bf16_reaches_fp64_accuracy():
    """The FP64-class tensor-core operator converges like FP64 (no stall) on the beta = 8 golden lattice."""
    import nsl_gb300 as N

    g, hfm = setup("honey6x6_nt32_beta8")
    rng = np.random.default_rng(6)
    b = rng.standard_normal((4, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((4, g["Nt"], g["Nx"]))
    eps = 1e-10 * np.linalg.norm(b.reshape(4, -1), axis=1).min()
    cg = N.CG(hfm, N.MatrixCombination.MMdagger, eps, 200000, mode="per_rhs", precision="bf16split")
    x = cg(b)
    cg64 = N.CG(hfm, N.MatrixCombination.MMdagger, eps, 200000, mode="per_rhs", precision="fp64",
                stop="true_residual")
    cg64(b)
    assert cg.stats["converged"] == 4 and cg.stats["escalated"] == 0
    assert true_res(hfm, b, x).max() < 1.5e-10
    # seven digits (~1e-13 operator precision) stay close to the FP64 iteration count on this lattice
    assert cg.stats["iterations"] <= 2.0 * cg64.stats["iterations"]


def true_res_op(op, b, x):
    r = b - op(x)
    return np.linalg.norm(r.reshape(r.shape[0], -1), axis=1) / np.linalg.norm(b.reshape(b.shape[0], -1), axis=1)


@pytest.mark.parametrize("name,comb,mode", [("honey6x6_nt32_beta8", "MdaggerM", "per_rhs"),
                                            ("honey6x6_nt32_beta8", "MMdagger", "shared"),
                                            ("honey3x3_nt16", "MMdagger", "per_rhs"),
                                            ("ring6_nt4_complexphi_mu", "MdaggerM", "per_rhs")])
def test_cg_split_bf16_fused_forms(monkeypatch, name, comb, mode):
    """The split-BF16 CG with its dot products and updates fused into the operator epilogues: both two-factor
    operators, one shared system over the batch, and lattices whose Nx is not a multiple of the 32-site tile (the
    small ones would run in the resident kernel, which is switched off here)."""
    import nsl_gb300 as N

    monkeypatch.setenv("NSLG_CG_RESIDENT", "0")
    g, hfm = setup(name)
    rng = np.random.default_rng(7)
    b = rng.standard_normal((3, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((3, g["Nt"], g["Nx"]))
    norms = np.linalg.norm(b.reshape(3, -1), axis=1)
    eps = 1e-10 * (norms.min() if mode == "per_rhs" else np.linalg.norm(b))
    cg = N.CG(hfm, N.MatrixCombination[comb], eps, 200000, mode=mode, precision="bf16split")
    x = cg(b)
    op = getattr(hfm, comb)
    if mode == "per_rhs":
        assert cg.stats["converged"] == 3
        assert true_res_op(op, b, x).max() < 1.5e-10
    else:
        assert cg.stats["converged"] == 1
        assert np.linalg.norm(b - op(x)) / np.linalg.norm(b) < 1.5e-10


@pytest.mark.parametrize("precision,resident", [("fp64", "0"), ("bf16split", "0"), ("bf16split", "1")])
def test_cg_species_switch_on_one_handle(monkeypatch, precision, resident):
    """The captured CG iteration (and the resident kernel) reads the species' exp(+-delta K): a solve after
    populate(phi, Hole) on the handle and batch size a particle solve used converges to the hole system's solution."""
    import nsl_gb300 as N

    monkeypatch.setenv("NSLG_CG_RESIDENT", resident)
    g, hfm = setup("honey3x3_nt16")
    rng = np.random.default_rng(31)
    b = rng.standard_normal((4, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((4, g["Nt"], g["Nx"]))
    for sp in (N.Species.Particle, N.Species.Hole, N.Species.Particle):
        hfm.populate(g["phi"], sp)
        cg = N.CG(hfm, N.MatrixCombination.MMdagger, 1e-10 * np.linalg.norm(b[0]), 20000, mode="per_rhs",
                  precision=precision, stop="true_residual")
        x = cg(b)
        assert cg.stats["converged"] == 4, (sp, cg.stats)
        assert true_res(hfm, b, x).max() < 2e-10
