"""Two-body correlators on the GPU (nslg_twobody_measure) against the reference's own outputs (golden fixtures) and
the oracle: all twelve channels, both solver precisions, the non-interacting case, HubbardDiag as the fermion
matrix, chunked source times and device-resident inputs."""
import numpy as np
import pytest

from conftest import TWOBODY_CASES, load_twobody, rel_err

pytestmark = pytest.mark.gpu


def make(g, FermionMatrixType=None, **kw):
    import nsl_gb300 as N
    from nsl_gb300.measurement import TwoBodyCorrelator

    lat = N.Honeycomb(g["L"])
    params = {"Nt": g["Nt"], "beta": g["beta"], "mu": g["mu"], "wallSources": g["wall"], "momenta": g["momenta"]}
    if FermionMatrixType is not None:
        kw["FermionMatrixType"] = FermionMatrixType
    return lat, TwoBodyCorrelator(lat, params, **kw)


@pytest.mark.parametrize("name", TWOBODY_CASES)
@pytest.mark.parametrize("precision", ["fp64", "bf16split"])
def test_twobody_vs_reference(name, precision):
    g = load_twobody(name)
    _, tb = make(g, eps=1e-12, precision=precision)
    assert np.array_equal(tb.tuples, g["tuples"])
    out = tb.measure_array(g["phi"], g["nts"])
    assert tb.stats["converged"] == tb.stats["systems"]
    # the reference's CG stops at |r| <= 1e-12 over the whole batch; the channels are quadratic in the solutions
    assert rel_err(out, g["out"]) < 1e-10
    # the dictionary form keyed like the reference's maps
    res = tb.measure(g["phi"], g["nts"])
    w, x, P, Q = (int(v) for v in g["tuples"][7])
    assert np.array_equal(res["I1S0Izn1Sz0"][(w, x, P, Q)], out[11, 7])


def test_twobody_noninteracting_and_chunked():
    """measure() with no configuration is the free theory with one source time; Nt source times processed one per
    chunk (NSLG_TB_CHUNK=1) agree with the single batched solve."""
    import os

    from oracle import nsl_oracle as O

    g = load_twobody("twobody_honey3x3_nt8")
    _, tb = make(g)
    free = tb.measure()
    h = O.HubbardExp(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
    want = O.two_body_correlator(h, np.zeros((g["Nt"], g["Nx"]), dtype=np.complex128), g["wall"], g["tuples"], 1)
    got = np.stack([np.stack([free[ch][tuple(int(v) for v in t)] for t in g["tuples"]]) for ch in tb.CHANNELS])
    assert rel_err(got, want) < 1e-10
    full = tb.measure_array(g["phi"], g["Nt"])
    os.environ["NSLG_TB_CHUNK"] = "1"
    try:
        chunked = tb.measure_array(g["phi"], g["Nt"])
    finally:
        del os.environ["NSLG_TB_CHUNK"]
    assert rel_err(chunked, full) < 1e-10  # same systems; batch-dependent reduction order only
    want = O.two_body_correlator(h, g["phi"], g["wall"], g["tuples"], g["Nt"])
    assert rel_err(full, want) < 1e-10


def test_twobody_diag_discretisation_and_device_inputs():
    """FermionMatrixType = HubbardDiag against the oracle's HubbardDiag; a CUDA phi gives a CUDA result."""
    import torch

    import nsl_gb300 as N
    from oracle import nsl_oracle as O

    g = load_twobody("twobody_honey2x2_nt6_mu")
    _, tb = make(g, FermionMatrixType=N.HubbardDiag)
    out = tb.measure_array(g["phi"], g["nts"])
    h = O.HubbardDiag(O.honeycomb_hops(*g["L"]), g["Nt"], g["beta"], g["mu"])
    want = O.two_body_correlator(h, g["phi"], g["wall"], g["tuples"], g["nts"])
    assert rel_err(out, want) < 1e-10
    dev = tb.measure_array(torch.from_numpy(g["phi"]).cuda(), g["nts"])
    assert dev.is_cuda
    assert rel_err(dev.cpu().numpy(), out) < 1e-13


def test_twobody_argument_errors():
    from nsl_gb300 import _lib

    g = load_twobody("twobody_honey2x2_nt6_mu")
    _, tb = make(g)
    with pytest.raises(_lib.NslgError) as e:
        tb.measure_array(g["phi"], g["Nt"] + 1)
    assert e.value.code == _lib.ERR_ARG
    tb.tuples = np.array([[0, 0, 0, 9]], dtype=np.int64)
    with pytest.raises(_lib.NslgError) as e:
        tb.measure_array(g["phi"], 1)
    assert e.value.code == _lib.ERR_ARG
