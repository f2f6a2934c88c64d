"""nslg_fm_apply_noalloc: the allocation-free operator entry point agrees with nslg_fm_apply.

Collected last (file name) so that it runs after the other GPU tests as well as alone in a fresh process.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(L=(3, 3), Nt=16, beta=4.0, nbatch=3, seed=5, kind="exp", species=0):
    import torch

    import nsl_gb300 as N

    lat = N.Honeycomb(L)
    rng = np.random.default_rng(seed)
    phi = rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * 2.0) + 0j
    psi = rng.standard_normal((nbatch, Nt, lat.sites())) + 1j * rng.standard_normal((nbatch, Nt, lat.sites()))
    h = (N.HubbardExp if kind == "exp" else N.HubbardDiag)(lat, Nt, beta)
    h.populate(phi, N.Species(species))
    return h, torch.from_numpy(psi).cuda()


def _noalloc(h, op, psi, precision):
    import torch

    from nsl_gb300 import _lib
    from nsl_gb300 import tensor as T
    from nsl_gb300.fermion_matrix import precision_code

    out = torch.empty_like(psi)
    with T.stream_order(h.ctx, psi, out):
        code = _lib.load().nslg_fm_apply_noalloc(h.handle, op, T.ptr(psi), T.ptr(out), psi.shape[0],
                                                 precision_code(precision))
    torch.cuda.synchronize()
    return code, out


@pytest.mark.parametrize("kind,species", [("exp", 0), ("exp", 1), ("diag", 0)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-14), ("fp32", 1e-6)])
def test_noalloc_matches_apply_twice(precision, tol, kind, species):
    """Both species of HubbardExp and HubbardDiag: the factor matrices made resident by the allocating calls are
    the ones the allocation-free call reads."""
    from nsl_gb300 import _lib

    h, psi = _setup(kind=kind, species=species)
    ops = [_lib.OP_M, _lib.OP_MDAGGER, _lib.OP_MMDAGGER, _lib.OP_MDAGGERM]
    refs = {op: h._apply(op, psi, precision).cpu().numpy() for op in ops}  # allocating entry point
    for _ in range(2):  # two calls in a row reuse the same scratch
        for op in ops:
            code, out = _noalloc(h, op, psi, precision)
            assert code == _lib.OK, _lib.load().nslg_last_error()
            ref = refs[op]
            assert np.abs(out.cpu().numpy() - ref).max() <= tol * np.abs(ref).max()


def test_noalloc_limits():
    import torch

    from nsl_gb300 import _lib
    from nsl_gb300 import tensor as T

    h, psi = _setup()
    lib = _lib.load()
    # exp(delta K) not resident yet on a fresh handle -> ERR_STATE (it would have to be computed, i.e. allocated)
    code, _ = _noalloc(h, _lib.OP_M, psi, "fp64")
    assert code == _lib.ERR_STATE
    h.M(psi)
    h.Mdagger(psi)
    # host buffers need staging -> ERR_ARG
    host = psi.cpu().numpy()
    out_h = np.empty_like(host)
    assert lib.nslg_fm_apply_noalloc(h.handle, _lib.OP_M, host.ctypes.data, out_h.ctypes.data, host.shape[0],
                                     _lib.PREC_FP64) == _lib.ERR_ARG
    # tensor-core precisions need workspaces -> ERR_ARG
    code, _ = _noalloc(h, _lib.OP_M, psi, "bf16split")
    assert code == _lib.ERR_ARG
    # a two-factor operator beyond the scratch -> ERR_SHAPE (the buffers are never touched: no kernel runs)
    per = h.Nt * h.Nx
    nbig = _lib.NOALLOC_MAX_ELEMS // per + 1
    big = torch.zeros((nbig, h.Nt, h.Nx), dtype=torch.complex128, device="cuda")
    out = torch.empty_like(big)
    with T.stream_order(h.ctx, big, out):
        assert lib.nslg_fm_apply_noalloc(h.handle, _lib.OP_MMDAGGER, T.ptr(big), T.ptr(out), nbig,
                                         _lib.PREC_FP64) == _lib.ERR_SHAPE
    # the single-factor operators have no scratch and no limit
    with T.stream_order(h.ctx, big, out):
        assert lib.nslg_fm_apply_noalloc(h.handle, _lib.OP_M, T.ptr(big), T.ptr(out), nbig, _lib.PREC_FP64) == _lib.OK
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0


def test_noalloc_allocates_nothing():
    """The entry point's contract: no device allocation. Free device memory (cudaMemGetInfo through torch) is
    sampled after the scratch lookup and the output buffers exist, and again after a loop of calls of every
    operator; it must not move."""
    import torch

    from nsl_gb300 import _lib
    from nsl_gb300 import tensor as T

    h, psi = _setup(nbatch=4)
    lib = _lib.load()
    ops = [_lib.OP_M, _lib.OP_MDAGGER, _lib.OP_MMDAGGER, _lib.OP_MDAGGERM]
    for op in ops:  # factor matrices resident (allocating calls)
        h._apply(op, psi, "fp64")
    outs = [torch.empty_like(psi) for _ in ops]
    torch.cuda.synchronize()
    # the first call looks the scratch array up (the runtime may load the module then)
    with T.stream_order(h.ctx, psi, outs[0]):
        assert lib.nslg_fm_apply_noalloc(h.handle, _lib.OP_MMDAGGER, T.ptr(psi), T.ptr(outs[0]), psi.shape[0],
                                         _lib.PREC_FP64) == _lib.OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        for op, out in zip(ops, outs):
            for prec in (_lib.PREC_FP64, _lib.PREC_FP32):
                with T.stream_order(h.ctx, psi, out):
                    assert lib.nslg_fm_apply_noalloc(h.handle, op, T.ptr(psi), T.ptr(out), psi.shape[0],
                                                     prec) == _lib.OK, lib.nslg_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
