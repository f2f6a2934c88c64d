"""HubbardDiag (the diagonal discretisation) on the GPU against the reference's own outputs (golden fixtures) and the
oracle: operators, log det, its gradient, CG on MM^dagger and the action force."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, rel_err

pytestmark = pytest.mark.gpu


def setup(name, species=0):
    import nsl_gb300 as N
    from nsl_gb300.lattice import Honeycomb, Ring

    g = load_golden(name)
    spec = g["lattice_spec"]
    lat = Ring(int(spec[1])) if spec[0] == "ring" else Honeycomb((int(spec[1]), int(spec[2])))
    hfd = N.HubbardDiag(lat, g["Nt"], g["beta"], g["mu"])
    hfd.populate(g["phi"], N.Species(species))
    return g, lat, hfd


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_diag_operators_vs_reference(name, species, tag):
    g, _, hfd = setup(name, species)
    for fn, key in (("M", "M"), ("Mdagger", "Mdag"), ("MMdagger", "MMdag"), ("MdaggerM", "MdagM")):
        ref = g[f"diag_{key}_{tag}"]
        assert rel_err(getattr(hfd, fn)(g["psi"]), ref) < 1e-12, fn
        assert rel_err(getattr(hfd, fn)(g["psi"], precision="fp32"), ref) < 2e-5, fn


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_diag_logdet_and_grad_vs_reference(name, species, tag):
    g, _, hfd = setup(name, species)
    ref = complex(g[f"diag_logdet_{tag}"])
    assert abs(hfd.logDetM() - ref) <= 1e-10 * max(1.0, abs(ref))
    bar = 2e-9 if g["beta"] >= 8 else 1e-10
    assert rel_err(hfd.gradLogDetM(), g[f"diag_grad_{tag}"]) < bar


def test_diag_tensor_core_precisions_are_refused():
    from nsl_gb300 import _lib

    g, _, hfd = setup("honey3x3_nt16")
    for prec in ("bf16split", "tf32x3"):
        with pytest.raises(_lib.NslgError) as e:
            hfd.M(g["psi"], precision=prec)
        assert e.value.code == _lib.ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_diag_cg(precision):
    """CG on the diagonal discretisation's MM^dagger (per right-hand side, FP64 true residual)."""
    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    g, _, hfd = setup("honey3x3_nt16")
    rng = np.random.default_rng(9)
    b = rng.standard_normal((3, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((3, g["Nt"], g["Nx"]))
    eps = 1e-11 * np.linalg.norm(b.reshape(3, -1), axis=1).min()
    cg = N.CG(hfd, N.MatrixCombination.MMdagger, eps, 100000, mode="per_rhs", precision=precision,
              stop="true_residual")
    x = cg(b)
    assert cg.stats["converged"] == 3
    h = O.HubbardDiag(g["hops"], g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], O.PARTICLE)
    r = b - h.MMdagger(x)
    assert (np.linalg.norm(r.reshape(3, -1), axis=1) / np.linalg.norm(b.reshape(3, -1), axis=1)).max() < 2e-11


def test_diag_fermion_action_force_is_minus_gradient():
    """The fermion action with FermionMatrixType = HubbardDiag: force = -(grad_P - grad_H) (hubbardFermiAction.tpp),
    checked against the oracle's gradients and against central differences of the action."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction
    from oracle import nsl_oracle as O

    g, lat, _ = setup("honey2x2_nt6_mu")
    params = {"Nt": int(g["Nt"]), "beta": complex(g["beta"]), "mu": complex(g["mu"]), "U": 2.0}
    S = HubbardFermionAction(lat, params, FermionMatrixType=N.HubbardDiag)
    phi = np.real(g["phi"]) + 0j
    F = np.asarray(S.force({"phi": phi})["phi"])
    grads = []
    for sp in (O.PARTICLE, O.HOLE):
        h = O.HubbardDiag(g["hops"], g["Nt"], g["beta"], g["mu"])
        h.populate(phi, sp)
        grads.append(h.gradLogDetM())
    assert rel_err(F, -(grads[0] - grads[1])) < 1e-10
    # d S / d phi_{t x} by central differences on the real part
    eps = 1e-6
    for (t, x) in ((0, 0), (2, 3), (int(g["Nt"]) - 1, 1)):
        dp = np.zeros_like(phi)
        dp[t, x] = eps
        dS = (S.eval({"phi": phi + dp}) - S.eval({"phi": phi - dp})) / (2 * eps)
        assert abs(dS.real + F[t, x].real) < 1e-5 * max(1.0, abs(F[t, x]))
