"""The resident CG kernel (nsl_gb300/csrc/cg_resident.cuh): systems of at most 2048 elements on lattices of at most
64 sites with a mixed-precision request are solved whole in one CTA each (float-float iteration operator, FP64
vectors, FP64 reliable updates and, under the double-double rule, double-double rebases in the same kernel).

Checks: the residual guarantee of each stopping rule against the oracle (FP64 |b - A x| or the oracle's
double-double residual of x + x_lo), agreement with the launch-per-step solver on the same systems
(NSLG_CG_RESIDENT=0), both two-factor operators, the reference's shared mode (one system over the batch), a group
that mixes resident and launch-per-step instances, and exhaustion.
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import nsl_oracle as O
from test_gpu_cg import setup
from test_gpu_cg_dd import _same_operator

pytestmark = pytest.mark.gpu


def _solve(monkeypatch, hfm, comb, b, eps, precision, stop, mode="per_rhs", resident=True, max_iter=200000):
    import nsl_gb300 as N

    monkeypatch.setenv("NSLG_CG_RESIDENT", "1" if resident else "0")
    cg = N.CG(hfm, N.MatrixCombination[comb], eps, max_iter, mode=mode, precision=precision, stop=stop)
    x = np.asarray(cg(b))
    lo = np.asarray(cg.x_lo_) if stop == "true_residual_dd" else np.zeros_like(x)
    return x, lo, dict(cg.stats)


def _residuals(hfm, phi, comb, b, x, lo, dd):
    if dd:
        ho = _same_operator(hfm, phi)
        return np.array([np.linalg.norm(O.residual_dd(ho, comb, b[i], x[i], lo[i])) for i in range(b.shape[0])])
    r = b - getattr(hfm, comb)(x)
    return np.linalg.norm(r.reshape(r.shape[0], -1), axis=1)


@pytest.mark.parametrize("name,comb", [("honey3x3_nt16", "MMdagger"), ("honey3x3_nt16", "MdaggerM"),
                                       ("ring6_nt4_complexphi_mu", "MMdagger"), ("honey2x2_nt6_mu", "MdaggerM")])
@pytest.mark.parametrize("precision,stop", [("bf16split", "true_residual"), ("fp32", "true_residual_dd"),
                                            ("bf16split", "true_residual_dd")])
def test_resident_meets_tolerance_and_agrees(monkeypatch, name, comb, precision, stop):
    g, hfm = setup(name)
    rng = np.random.default_rng(17)
    b = rng.standard_normal((5, g["Nt"], g["Nx"])) + 1j * rng.standard_normal((5, g["Nt"], g["Nx"]))
    nb = np.linalg.norm(b.reshape(5, -1), axis=1)
    eps = (1e-13 if stop == "true_residual_dd" else 1e-10) * nb.min()
    x, lo, st = _solve(monkeypatch, hfm, comb, b, eps, precision, stop)
    assert st["converged"] == 5, st
    res = _residuals(hfm, g["phi"], comb, b, x, lo, stop == "true_residual_dd")
    assert res.max() <= eps * (1.01 if stop == "true_residual_dd" else 1.5), (res, eps)
    x0, lo0, st0 = _solve(monkeypatch, hfm, comb, b, eps, precision, stop, resident=False)
    assert st0["converged"] == 5
    # two solutions within eps of the same system: they differ by at most ~cond(A) eps / |A|
    assert rel_err(x + lo, x0 + lo0) < 1e-6


def test_resident_shared_mode_reference_batch(monkeypatch):
    """The reference's batch semantics (one system over all right-hand sides, 3 x 16 x 18 = 864 elements) in the
    resident kernel, with the reference's golden right-hand side and solution."""
    g, hfm = setup("honey3x3_nt16")
    b = g["b"]
    eps = 1e-11 * np.linalg.norm(b)
    x, _, st = _solve(monkeypatch, hfm, "MMdagger", b, eps, "bf16split", "true_residual", mode="shared")
    assert st["systems"] == 1 and st["converged"] == 1
    assert np.linalg.norm(b - hfm.MMdagger(x)) <= 1.5 * eps
    assert rel_err(x, g["cg_x"]) < 1e-6


def test_resident_low_temperature_dd(monkeypatch):
    """Honeycomb 3x3, Nt = 32, beta = 12 (|A| |x| / |b| ~ 1e8): the iteration needs reliable updates and
    double-double rebases to reach 1e-12 |b|; every pair meets it by the oracle's double-double residual."""
    import nsl_gb300 as N

    lat = N.Honeycomb((3, 3))
    Nt, beta, U = 32, 12.0, 3.0
    rng = np.random.default_rng(23)
    phi = rng.standard_normal((Nt, 18)) * np.sqrt(beta / Nt * U) + 0j
    hfm = N.HubbardExp(lat, Nt, beta)
    hfm.populate(phi)
    b = rng.standard_normal((4, Nt, 18)) + 1j * rng.standard_normal((4, Nt, 18))
    eps = 1e-12 * np.linalg.norm(b.reshape(4, -1), axis=1).min()
    x, lo, st = _solve(monkeypatch, hfm, "MMdagger", b, eps, "bf16split", "true_residual_dd")
    assert st["converged"] == 4 and st["reliable_updates"] >= 1 and st["dd_rebases"] >= 1, st
    res = _residuals(hfm, phi, "MMdagger", b, x, lo, True)
    assert res.max() <= eps * 1.01


def test_resident_exhaustion_reports_unconverged(monkeypatch):
    g, hfm = setup("honey3x3_nt16")
    b = g["b"][:1].repeat(2, axis=0)
    x, _, st = _solve(monkeypatch, hfm, "MMdagger", b, 1e-14, "fp32", "true_residual", max_iter=7)
    assert st["converged"] == 0 and st["iterations"] <= 8
    assert np.all(np.isfinite(x))


def test_group_mixes_resident_and_launch_per_step(monkeypatch):
    """cg_group over honeycomb 2x2 (Nt = 8), honeycomb 3x3 (Nt = 16) and honeycomb 6x6 (Nt = 32, 72 sites: too large
    for the resident kernel): the small instances run resident beside the large one's launch-per-step loop; every
    instance meets its double-double tolerance and equals its solve alone."""
    import nsl_gb300 as N

    monkeypatch.setenv("NSLG_CG_RESIDENT", "1")
    rng = np.random.default_rng(29)
    items, phis = [], []
    for L, Nt, beta in (((2, 2), 8, 2.0), ((3, 3), 16, 4.0), ((6, 6), 32, 4.0)):
        lat = N.Honeycomb(L)
        phi = rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * 3.0) + 0j
        h = N.HubbardExp(lat, Nt, beta)
        h.populate(phi)
        b = rng.standard_normal((3, Nt, lat.sites())) + 1j * rng.standard_normal((3, Nt, lat.sites()))
        items.append((h, b))
        phis.append(phi)
    eps = 1e-12
    xs, los, stats = N.cg_group(items, N.MatrixCombination.MMdagger, eps, 200000, precision="bf16split",
                                stop="true_residual_dd")
    for (h, b), phi, x, lo, st in zip(items, phis, xs, los, stats):
        assert st["converged"] == 3, st
        res = _residuals(h, phi, "MMdagger", b, np.asarray(x), np.asarray(lo), True)
        assert res.max() <= eps * 1.01
        xa, loa, _ = _solve(monkeypatch, h, "MMdagger", b, eps, "bf16split", "true_residual_dd")
        assert rel_err(np.asarray(x) + np.asarray(lo), xa + loa) < 1e-6
