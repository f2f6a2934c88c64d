"""nslg_cg_solve_group: fermion matrices of different Nx, Nt, beta, phi (and species) solved in one launch sequence.

Each instance's solution must be the one its own solve gives (same rule; the reductions are split differently, so
to the tolerance, not bitwise), each system's true residual must meet its own eps (checked with the oracle on the
device's FP64 operator), and per-instance statistics must describe each instance.
"""
import numpy as np
import pytest

from oracle import nsl_oracle as O

pytestmark = pytest.mark.gpu


def _instances(seed=51):
    import nsl_gb300 as N

    rng = np.random.default_rng(seed)
    out = []
    for lat, Nt, beta, sp, nrhs in ((N.Honeycomb((2, 2)), 8, 2.0, 0, 3), (N.Ring(6), 16, 3.0, 1, 2),
                                    (N.Honeycomb((3, 3)), 12, 4.0, 0, 4), (N.Honeycomb((4, 4)), 6, 1.5, 1, 1)):
        Nx = lat.sites()
        phi = rng.standard_normal((Nt, Nx)) * np.sqrt(beta / Nt * 2.0) + 0j
        h = N.HubbardExp(lat, Nt, beta, 0.0, N.Species(sp))
        h.populate(phi)
        b = rng.standard_normal((nrhs, Nt, Nx)) + 1j * rng.standard_normal((nrhs, Nt, Nx))
        out.append((h, phi, b))
    return out


def _oracle(h, phi):
    ho = O.HubbardExp(h.Lat.hopping_matrix(), h.Nt, h.beta, h.mu, int(h.species()))
    ho.populate(phi)
    for d in {h.delta, np.conj(h.delta), -h.delta, -np.conj(h.delta)}:
        ho.set_expK(d, h.exp_hopping_matrix(d))
    ho.set_phases(h.phases())
    return ho


@pytest.mark.parametrize("precision,stop,rel", [("fp64", "true_residual", 1e-10), ("bf16split", "true_residual", 1e-10),
                                                ("fp32", "true_residual", 1e-9), ("fp64", "true_residual_dd", 1e-13)])
def test_group_equals_individual_solves(precision, stop, rel):
    import nsl_gb300 as N

    inst = _instances()
    eps = [rel * np.linalg.norm(b.reshape(b.shape[0], -1), axis=1).min() for _, _, b in inst]
    xs, los, stats = N.cg_group([(h, b) for h, _, b in inst], N.MatrixCombination.MMdagger, eps, 100000,
                                precision=precision, stop=stop)
    for i, (h, phi, b) in enumerate(inst):
        assert stats[i]["systems"] == b.shape[0] and stats[i]["converged"] == b.shape[0], stats[i]
        cg = N.CG(h, N.MatrixCombination.MMdagger, eps[i], 100000, mode="per_rhs", precision=precision, stop=stop)
        xi = np.asarray(cg(b))
        x = np.asarray(xs[i])
        assert np.abs(x - xi).max() <= 1e-6 * np.abs(xi).max()
        ho = _oracle(h, phi)
        for r in range(b.shape[0]):
            if stop == "true_residual_dd":
                res = np.linalg.norm(O.residual_dd(ho, "MMdagger", b[r], x[r], np.asarray(los[i])[r]))
            else:
                res = np.linalg.norm(b[r] - ho.MMdagger(x[r]))
            assert res <= eps[i] * 1.05, (i, r, res, eps[i])


def test_group_on_device_buffers_and_x0():
    import torch

    import nsl_gb300 as N

    inst = _instances(seed=52)
    items = [(h, torch.from_numpy(b).cuda(), torch.from_numpy(0.25 * b).cuda()) for h, _, b in inst]
    eps = 1e-9
    xs, _, stats = N.cg_group(items, N.MatrixCombination.MdaggerM, eps, 100000, precision="fp64")
    for (h, phi, b), x, st in zip(inst, xs, stats):
        assert x.is_cuda
        ho = _oracle(h, phi)
        assert st["converged"] == b.shape[0]
        r = b - ho.MdaggerM(x.cpu().numpy())
        assert np.linalg.norm(r.reshape(b.shape[0], -1), axis=1).max() <= eps * 1.05


def test_group_rejects_mixed_contexts_and_bad_sizes():
    import ctypes as C

    import nsl_gb300 as N
    from nsl_gb300 import _lib

    h1 = N.HubbardExp(N.Ring(4), 4, 1.0, ctx=N.Context(0))
    h2 = N.HubbardExp(N.Ring(4), 4, 1.0, ctx=N.Context(0))
    phi = np.zeros((4, 4)) + 0j
    h1.populate(phi)
    h2.populate(phi)
    b = np.ones((1, 4, 4), dtype=np.complex128)
    x = np.empty_like(b)
    P = C.c_void_p * 2
    lib = _lib.load()
    rc = lib.nslg_cg_solve_group(2, P(h1.handle.value, h2.handle.value), _lib.OP_MMDAGGER, P(b.ctypes.data, b.ctypes.data),
                                 None, P(x.ctypes.data, x.ctypes.data), None, (C.c_int64 * 2)(1, 1),
                                 (C.c_double * 2)(1e-8, 1e-8), 100, _lib.PREC_FP64, _lib.STOP_TRUE_RESIDUAL, None)
    assert rc == _lib.ERR_ARG
    rc = lib.nslg_cg_solve_group(1, P(h1.handle.value, None), _lib.OP_MMDAGGER, P(b.ctypes.data, None), None,
                                 P(x.ctypes.data, None), None, (C.c_int64 * 1)(0), (C.c_double * 1)(1e-8), 100,
                                 _lib.PREC_FP64, _lib.STOP_TRUE_RESIDUAL, None)
    assert rc == _lib.ERR_SHAPE


@pytest.mark.parametrize("precision,stop", [("bf16split", "true_residual_dd"), ("bf16split", "true_residual"),
                                            ("fp32", "true_residual")])
def test_group_of_one_instance(precision, stop):
    """A group of a single fermion matrix (what a batch of one request is): the packed plan, not the single-matrix
    fused iteration, runs it, and the result equals the matrix's own solve."""
    import nsl_gb300 as N

    h, phi, b = _instances(seed=53)[2]
    eps = 1e-10 * np.linalg.norm(b.reshape(b.shape[0], -1), axis=1).min()
    xs, los, stats = N.cg_group([(h, b)], N.MatrixCombination.MMdagger, eps, 100000, precision=precision, stop=stop)
    assert stats[0]["converged"] == b.shape[0]
    cg = N.CG(h, N.MatrixCombination.MMdagger, eps, 100000, mode="per_rhs", precision=precision, stop=stop)
    xi = np.asarray(cg(b))
    assert np.abs(np.asarray(xs[0]) - xi).max() <= 1e-6 * np.abs(xi).max()
    ho = _oracle(h, phi)
    for r in range(b.shape[0]):
        if stop == "true_residual_dd":
            res = np.linalg.norm(O.residual_dd(ho, "MMdagger", b[r], np.asarray(xs[0])[r], np.asarray(los[0])[r]))
        else:
            res = np.linalg.norm(b[r] - ho.MMdagger(np.asarray(xs[0])[r]))
        assert res <= eps * 1.05
