"""The stratified log det M and gradient on the GPU (nsl_gb300/csrc/stable.cu) against the oracle.

Small lattices: against i diag(M^{-1}) and the dense log-determinant of M (M is well conditioned, so a dense inverse
is exact to ~1e-14 where the time-slice product is not). Honeycomb 12x12, Nt = 64, beta = 8 and 24x24, Nt = 128,
beta = 12: against the oracle's stratified forms on selected slices (tests/golden/stable_cfg*.npz, made by
tests/golden/make_stable_golden.py), and, on every slice, the similarity invariant tr G(s) (the sum over sites of a
gradient row is the same for every time slice). Bars: 1e-12 relative (max-norm over the compared rows) for the
gradient and the force (5e-12 at beta = 12 on 24x24, where two stratified evaluations with different chunkings, QR
methods and wraps agree to 2e-12..4e-12, measured: the conditioning of G itself), 1e-12 relative (modulo 2 pi i) for
log det.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden, rel_err
from oracle import nsl_oracle as O

pytestmark = pytest.mark.gpu


def mod2pi(z):
    return complex(z.real, (z.imag + np.pi) % (2 * np.pi) - np.pi)


def _field(Nx, Nt, beta, seed, U=3.0, mu=0.0, complex_phi=False):
    rng = np.random.default_rng(seed)
    phi = rng.standard_normal((Nt, Nx)) * np.sqrt(beta / Nt * U) + 0j
    if complex_phi:
        phi = phi + 0.2j * rng.standard_normal(phi.shape)
    return phi


def _lat(L):
    import nsl_gb300 as N

    return N.Honeycomb(L) if isinstance(L, tuple) else N.Ring(L)


SMALL = [((2, 2), 32, 12.0, 0, 0.0, False), ((3, 3), 32, 12.0, 1, 0.0, False), ((2, 2), 16, 8.0, 0, 0.3, True),
         (6, 24, 10.0, 1, 0.0, False), ((3, 3), 16, 4.0, 0, 0.0, False), ((4, 4), 13, 9.0, 1, 0.0, False)]


@pytest.mark.parametrize("L,Nt,beta,species,mu,cphi", SMALL)
def test_stratified_vs_dense_inverse(L, Nt, beta, species, mu, cphi):
    import nsl_gb300 as N

    lat = _lat(L)
    phi = _field(lat.sites(), Nt, beta, 7, mu=mu, complex_phi=cphi)
    h = N.HubbardExp(lat, Nt, beta, mu, N.Species(species))
    h.set_stabilisation("stratified")
    h.populate(phi)
    ho = O.HubbardExp(lat.hopping_matrix(), Nt, beta, mu, species)
    ho.populate(phi)
    n = Nt * lat.sites()
    Md = ho.M_dense().reshape(n, n)
    want = 1j * np.diag(np.linalg.inv(Md)).reshape(Nt, lat.sites())
    assert rel_err(np.asarray(h.gradLogDetM()), want) < 1e-12
    s, l = np.linalg.slogdet(Md)
    ld = h.logDetM()
    ref = complex(l, np.angle(s))
    assert abs(mod2pi(ld - ref)) <= 1e-12 * max(1.0, abs(ref)), (ld, ref)
    assert -np.pi < ld.imag <= np.pi


def test_auto_selects_the_form_by_temperature():
    """AUTO takes the direct product where it is accurate (beta rho <= 14) and the stratified form beyond."""
    import nsl_gb300 as N

    for L, Nt, beta, stratified in (((3, 3), 16, 2.0, False), ((3, 3), 32, 12.0, True)):
        lat = _lat(L)
        phi = _field(lat.sites(), Nt, beta, 3)
        g = {}
        for mode in ("auto", "plain", "stratified"):
            h = N.HubbardExp(lat, Nt, beta)
            h.set_stabilisation(mode)
            h.populate(phi)
            g[mode] = np.asarray(h.gradLogDetM())
        assert np.array_equal(g["auto"], g["stratified" if stratified else "plain"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("species,tag", [(0, "P"), (1, "H")])
def test_stratified_vs_reference_fixtures(name, species, tag):
    """Within the reference's own rounding (~1e-15 at beta <= 2, 2e-12 at beta = 4, 3e-10 at beta = 8)."""
    from test_gpu_action import make

    g = load_golden(name)
    N, lat = make(g)
    h = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
    h.set_stabilisation("stratified")
    h.populate(g["phi"], N.Species(species))
    bar = 1e-13 if g["beta"] <= 2 else (5e-12 if g["beta"] <= 4 else 1e-9)
    assert rel_err(np.asarray(h.gradLogDetM()), g[f"grad_{tag}"]) < bar
    ref = complex(g[f"logdet_{tag}"])
    assert abs(mod2pi(h.logDetM() - ref)) <= max(bar, 1e-12) * max(1.0, abs(ref))


def _big(name):
    z = np.load(os.path.join(ROOT, "tests", "golden", f"stable_{name}.npz"))
    d = {k: z[k] for k in z.files}
    L1, L2, Nt, beta, U, seed = d["params"]
    d.update(L=(int(L1), int(L2)), Nt=int(Nt), beta=float(beta), U=float(U))
    return d


@pytest.mark.parametrize("name", ["cfg2", "cfg3"])
def test_stratified_low_temperature_configurations(name):
    """Honeycomb 12x12, Nt = 64, beta = 8 and 24x24, Nt = 128, beta = 12 (AUTO selects the stratified form): log det
    and the gradient of both species against the oracle's stratified forms; tr G(s) the same on every slice; the
    fermion force -(grad_P - grad_H) on the compared slices."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction

    d = _big(name)
    lat = N.Honeycomb(d["L"])
    h = N.HubbardExp(lat, d["Nt"], d["beta"])
    sl = d["slices"]
    grads = {}
    for sp, tag in ((N.Species.Particle, "P"), (N.Species.Hole, "H")):
        h.populate(d["phi"], sp)
        ref = complex(d[f"logdet_{tag}"])
        ld = h.logDetM()
        assert abs(mod2pi(ld - ref)) <= 1e-12 * abs(ref), (ld, ref)
        gr = np.asarray(h.gradLogDetM())
        assert rel_err(gr[sl], d[f"grad_{tag}"]) < (5e-12 if d["beta"] > 8 else 1e-12)
        rows = gr.sum(axis=1)  # i (Nx - tr G(t+1)): a similarity invariant
        assert np.abs(rows - rows[0]).max() <= 1e-11 * np.abs(rows[0])
        grads[tag] = gr
    F = np.asarray(HubbardFermionAction(lat, {"Nt": d["Nt"], "beta": d["beta"], "mu": 0.0}).force(
        {"phi": d["phi"]})["phi"])
    assert rel_err(F, -(grads["P"] - grads["H"])) < 1e-13
    assert rel_err(F[sl], -(d["grad_P"] - d["grad_H"])) < (5e-12 if d["beta"] > 8 else 1e-12)


def test_stratified_leapfrog_and_delta_h():
    """A LeapfrogRealForce trajectory at beta = 12 (honeycomb 3x3, Nt = 32, Nmd = 6) with the stratified force and
    action against the oracle's trajectory on its stratified forms: fields and momenta to 1e-10, Delta H to 1e-9."""
    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import LeapfrogRealForce

    lat = N.Honeycomb((3, 3))
    Nt, beta, U, nmd = 32, 12.0, 3.0, 6
    phi = _field(lat.sites(), Nt, beta, 21, U=U)
    p0 = np.random.default_rng(22).standard_normal(phi.shape) + 0j
    params = {"Nt": Nt, "beta": beta, "mu": 0.0, "U": U}
    S = HubbardGaugeAction(params) + HubbardFermionAction(lat, params)
    SO = O.HubbardAction(lat.hopping_matrix(), Nt, beta, U, stable=True)
    for _ in range(3):  # eager, captured, replayed
        q1, p1 = LeapfrogRealForce(S, 1.0, nmd)({"phi": phi}, {"phi": p0})
    qo, po = O.leapfrog(SO, phi, p0, 1.0, nmd, real_force=True)
    assert rel_err(np.asarray(q1["phi"]), qo) < 1e-10
    assert rel_err(np.asarray(p1["phi"]), po) < 1e-10
    dH = (S(q1) + 0.5 * np.sum(np.asarray(p1["phi"]) ** 2)) - (S({"phi": phi}) + 0.5 * np.sum(p0 ** 2))
    dHo = O.hamiltonian(SO.eval(qo), po) - O.hamiltonian(SO.eval(phi), p0)
    assert abs(dH - dHo) < 1e-9 * max(1.0, abs(dHo)), (dH, dHo)


def test_split_force_keeps_direct_product_to_beta_rho_28():
    """Under AUTO the split-BF16 force setting keeps the direct product while beta rho <= 28 (honeycomb 6x6, Nt = 32,
    beta = 8: beta rho = 24), within 1e-7 of the stratified FP64 gradient the FP64 setting takes there; at
    beta rho = 36 it takes the stratified form like the FP64 setting."""
    from test_gpu_action import make

    g = load_golden("honey6x6_nt32_beta8")
    N, lat = make(g)
    grads = {}
    for fp, stab in (("bf16split", "auto"), ("bf16split", "plain"), ("fp64", "auto")):
        h = N.HubbardExp(lat, g["Nt"], g["beta"], g["mu"])
        h.set_force_precision(fp)
        h.set_stabilisation(stab)
        h.populate(g["phi"])
        grads[(fp, stab)] = np.asarray(h.gradLogDetM())
    assert np.array_equal(grads[("bf16split", "auto")], grads[("bf16split", "plain")])
    assert rel_err(grads[("bf16split", "auto")], grads[("fp64", "auto")]) < 1e-7
    lat3 = N.Honeycomb((3, 3))
    phi = _field(18, 32, 12.0, 5)
    out = {}
    for fp in ("bf16split", "fp64"):
        h = N.HubbardExp(lat3, 32, 12.0)
        h.set_force_precision(fp)
        h.populate(phi)
        out[fp] = np.asarray(h.gradLogDetM())
    assert np.array_equal(out["bf16split"], out["fp64"])
