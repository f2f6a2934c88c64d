"""The oracle's double-double operator and certified CG (oracle/nsl_oracle.py: apply_dd, residual_dd, cg_certified).

apply_dd is checked against a 50-digit evaluation (mpmath) of the same operator with the same FP64 exp(delta K) and
phases; cg_certified must reach true residuals below what FP64 can represent (its x + x_lo pair is certified by
residual_dd).
"""
import numpy as np
import pytest

from oracle import nsl_oracle as O


def _h(L=(2, 2), Nt=6, beta=3.0, mu=0.0, species=O.PARTICLE, seed=1):
    K = O.honeycomb_hops(*L)
    h = O.HubbardExp(K, Nt, beta, mu, species)
    rng = np.random.default_rng(seed)
    h.populate(rng.standard_normal((Nt, K.shape[0])) * 0.7 + 0.1j * rng.standard_normal((Nt, K.shape[0])))
    return h, rng


def _mp_apply(h, op, xh, xl):
    mp = pytest.importorskip("mpmath").mp
    mp.dps = 50
    C = lambda z: mp.mpc(float(np.real(z)), float(np.imag(z)))  # noqa: E731
    Nt, Nx = h.Nt, h.Nx

    def M(v, dag):
        E = h.expK(h.sgn * (np.conj(h.delta) if dag else h.delta))
        out = np.empty(v.shape, dtype=object)
        for r in range(v.shape[0]):
            for t in range(Nt):
                src = (t + 1) % Nt if dag else (t - 1) % Nt
                s = -1 if (t == Nt - 1 if dag else t == 0) else 1
                for x in range(Nx):
                    acc = mp.mpc(0)
                    for y in range(Nx):
                        w = v[r, src, y] if dag else v[r, src, y] * C(h.phiExp[src, y])
                        acc += C(E[x, y]) * w
                    if dag:
                        acc = acc * C(np.conj(h.phiExp[t, x]))
                    out[r, t, x] = v[r, t, x] - s * acc
        return out

    v = np.empty(xh.shape, dtype=object)
    for i in np.ndindex(xh.shape):
        v[i] = C(xh[i]) + C(xl[i])
    seq = {"M": [False], "Mdagger": [True], "MMdagger": [True, False], "MdaggerM": [False, True]}[op]
    for dag in seq:
        v = M(v, dag)
    return v


@pytest.mark.parametrize("op", ["M", "Mdagger", "MMdagger", "MdaggerM"])
@pytest.mark.parametrize("species,mu", [(O.PARTICLE, 0.0), (O.HOLE, 0.2)])
def test_apply_dd_against_50_digits(op, species, mu):
    h, rng = _h(mu=mu, species=species)
    xh = rng.standard_normal((2, h.Nt, h.Nx)) + 1j * rng.standard_normal((2, h.Nt, h.Nx))
    xl = xh * 1e-17 * rng.standard_normal(xh.shape)
    ref = _mp_apply(h, op, xh, xl)
    hi, lo = O.apply_dd(h, op, xh, xl)
    mp = pytest.importorskip("mpmath").mp
    err = max(abs(mp.mpc(float(hi[i].real), float(hi[i].imag)) + mp.mpc(float(lo[i].real), float(lo[i].imag))
                  - ref[i]) for i in np.ndindex(xh.shape))
    scale = max(abs(v) for v in ref.flat)
    assert float(err) < 1e-29 * float(scale)


def test_certified_cg_goes_below_fp64_floor():
    """Honeycomb 3x3, Nt = 16, beta = 8 (|x| / |b| ~ 750): the certified CG reaches 1e-14 relative true residual of
    the pair x + x_lo, while x alone (the pair rounded to FP64) sits at its rounding floor, ~5e-13."""
    K = O.honeycomb_hops(3, 3)
    h = O.HubbardExp(K, 16, 8.0)
    rng = np.random.default_rng(5)
    h.populate(rng.standard_normal((16, 18)) * np.sqrt(8.0 / 16 * 3.0) + 0j)
    b = rng.standard_normal((16, 18)) + 1j * rng.standard_normal((16, 18))
    nb = np.linalg.norm(b)
    xh, xl, it, rebases, res = O.cg_certified(h, "MMdagger", b, 1e-14 * nb)
    assert res <= 1e-14 * nb
    assert np.linalg.norm(O.residual_dd(h, "MMdagger", b, xh, xl)) <= 1e-14 * nb
    assert np.linalg.norm(O.residual_dd(h, "MMdagger", b, xh, 0 * xh)) > 1e-14 * nb
    assert rebases >= 2
