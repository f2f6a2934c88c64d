"""CG with the double-double rule (nslg_cg_solve_dd, NSLG_STOP_TRUE_RESIDUAL_DD) against the oracle.

The solution pair x + x_lo is checked with the oracle's own double-double residual (oracle/nsl_oracle.py:
residual_dd, pinned to a 50-digit evaluation in tests/test_oracle_dd.py), at tolerances below what the FP64 x alone
can meet: the rounding of x to FP64 moves b - A x by ~1e-16 |A| |x|, which at beta = 8 is 1e-13..1e-9 |b|.
"""
import numpy as np
import pytest

from oracle import nsl_oracle as O

pytestmark = pytest.mark.gpu


def _case(L, Nt, beta, nrhs, seed, U=3.0):
    import nsl_gb300 as N

    lat = N.Honeycomb(L)
    Nx = lat.sites()
    rng = np.random.default_rng(seed)
    phi = rng.standard_normal((Nt, Nx)) * np.sqrt(beta / Nt * U) + 0j
    b = rng.standard_normal((nrhs, Nt, Nx)) + 1j * rng.standard_normal((nrhs, Nt, Nx))
    h = N.HubbardExp(lat, Nt, beta)
    h.populate(phi)
    return N, h, _same_operator(h, phi), b


def _same_operator(h, phi):
    """The oracle's HubbardExp on the device's FP64 exp(delta K) and phases: with |A| |x| / |b| up to 1e8, the last bit
    of a transcendental function's rounding moves b - A x by more than the tolerances checked here, so the oracle
    must evaluate the same FP64 matrix."""
    ho = O.HubbardExp(h.Lat.hopping_matrix(), h.Nt, h.beta, h.mu)
    ho.populate(phi)
    for d in {h.delta, np.conj(h.delta)}:
        ho.set_expK(d, h.exp_hopping_matrix(d))
    ho.set_phases(h.phases())
    return ho


def _dd_residuals(ho, op, b, x, xl):
    return np.array([np.linalg.norm(O.residual_dd(ho, op, b[i], x[i], xl[i])) for i in range(b.shape[0])])


@pytest.mark.parametrize("precision", ["fp64", "bf16split"])
@pytest.mark.parametrize("op", ["MMdagger", "MdaggerM"])
def test_dd_solve_below_fp64_floor(precision, op):
    """Honeycomb 3x3, Nt = 16, beta = 8, 4 right-hand sides, per-RHS, eps = 1e-14 |b|: every pair meets eps by the
    oracle's double-double residual, the x alone of at least one system does not, and the reported true residual is
    the pair's."""
    N, h, ho, b = _case((3, 3), 16, 8.0, 4, 31)
    nb = np.linalg.norm(b.reshape(4, -1), axis=1)
    eps = 1e-14 * nb.min()
    cg = N.CG(h, getattr(N.MatrixCombination, op), eps, 200000, mode="per_rhs", precision=precision,
              stop="true_residual_dd")
    x = np.asarray(cg(b))
    xl = np.asarray(cg.x_lo_)
    st = cg.stats
    assert st["converged"] == 4 and st["dd_rebases"] >= 1, st
    res = _dd_residuals(ho, op, b, x, xl)
    assert res.max() <= eps * 1.01, (res, eps)
    assert _dd_residuals(ho, op, b, x, 0 * x).max() > eps
    assert st["true_residual"] <= 1.01e-14
    # the pair is the solution: against the FP64 CG to its own accuracy
    cg64 = N.CG(h, getattr(N.MatrixCombination, op), 1e-11 * nb.min(), 200000, mode="per_rhs",
                stop="true_residual")
    x64 = np.asarray(cg64(b))
    assert np.abs(x - x64).max() <= 1e-6 * np.abs(x).max()


def test_dd_solve_honeycomb6x6_beta8_1e10():
    """Honeycomb 6x6 (Nx = 72), Nt = 32, beta = 8, 8 right-hand sides with the split-BF16 operator to 1e-10 relative
    true residual (the bench's rule at a smaller size)."""
    N, h, ho, b = _case((6, 6), 32, 8.0, 8, 32)
    nb = np.linalg.norm(b.reshape(8, -1), axis=1)
    eps = 1e-10 * nb.min()
    cg = N.CG(h, N.MatrixCombination.MMdagger, eps, 200000, mode="per_rhs", precision="bf16split",
              stop="true_residual_dd")
    x = np.asarray(cg(b))
    res = _dd_residuals(ho, "MMdagger", b, x, np.asarray(cg.x_lo_))
    assert cg.stats["converged"] == 8
    assert res.max() <= eps * 1.01


def test_dd_solve_shared_mode_and_x0():
    """The reference's batch semantics (one system over all right-hand sides) under the double-double rule, from a
    caller-given starting vector."""
    N, h, ho, b = _case((2, 2), 8, 4.0, 3, 33)
    eps = 1e-14 * np.linalg.norm(b)
    x0 = 0.5 * b
    cg = N.CG(h, N.MatrixCombination.MMdagger, eps, 100000, mode="shared", stop="true_residual_dd")
    x = np.asarray(cg(b, x0))
    r = O.residual_dd(ho, "MMdagger", b, x, np.asarray(cg.x_lo_))
    assert np.linalg.norm(r) <= eps * 1.01
    assert cg.stats["systems"] == 1 and cg.stats["converged"] == 1


@pytest.mark.parametrize("op", ["M", "Mdagger", "MMdagger", "MdaggerM"])
@pytest.mark.parametrize("complex_phi", [False, True])
def test_apply_dd_against_oracle(op, complex_phi):
    """nslg_fm_apply_dd against the oracle's double-double operator (itself pinned to 50 digits): the pairs agree to
    1e-28 of the result's size (a complex phi and mu != 0 make exp(delta K)'s phases complex)."""
    import nsl_gb300 as N

    lat = N.Honeycomb((3, 3))
    Nt, beta, mu = 8, 4.0, (0.2 if complex_phi else 0.0)
    rng = np.random.default_rng(41)
    phi = rng.standard_normal((Nt, 18)) * 0.8 + (0.3j * rng.standard_normal((Nt, 18)) if complex_phi else 0j)
    h = N.HubbardExp(lat, Nt, beta, mu)
    h.populate(phi)
    ho = _same_operator(h, phi)
    xh = rng.standard_normal((3, Nt, 18)) + 1j * rng.standard_normal((3, Nt, 18))
    xl = xh * 1e-17 * rng.standard_normal(xh.shape)
    gh, gl = h.apply_dd(getattr(N.MatrixCombination, op), xh, xl)
    oh, ol = O.apply_dd(ho, op, xh, xl)
    # compare the pairs: (gh - oh) + (gl - ol), each difference exact in FP64 at this size
    d = (np.asarray(gh) - oh) + (np.asarray(gl) - ol)
    assert np.abs(d).max() <= 1e-28 * np.abs(oh).max()


def test_dd_solve_plain_fp64_configuration_1e10():
    """The 64-RHS workload's lattice and field (honeycomb 12x12, Nt = 64, beta = 8, U = 3, seed 2026), two of its
    right-hand sides through the bench's rule (split-BF16 operator, double-double, 1e-10 relative): the oracle's
    double-double residual certifies both pairs."""
    import nsl_gb300 as N

    lat = N.Honeycomb((12, 12))
    Nt, beta, U = 64, 8.0, 3.0
    rng = np.random.default_rng(2026)
    phi = rng.standard_normal((Nt, 288)) * np.sqrt(beta / Nt * U) + 0j
    b = (rng.standard_normal((64, Nt, 288)) + 1j * rng.standard_normal((64, Nt, 288)))[:2]
    h = N.HubbardExp(lat, Nt, beta)
    h.populate(phi)
    ho = _same_operator(h, phi)
    nb = np.linalg.norm(b.reshape(2, -1), axis=1)
    eps = 1e-10 * nb.min()
    cg = N.CG(h, N.MatrixCombination.MMdagger, eps, 400000, mode="per_rhs", precision="bf16split",
              stop="true_residual_dd")
    x = np.asarray(cg(b))
    assert cg.stats["converged"] == 2, cg.stats
    res = _dd_residuals(ho, "MMdagger", b, x, np.asarray(cg.x_lo_))
    assert res.max() <= eps * 1.01, (res, eps)
