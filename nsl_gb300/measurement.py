"""Correlators: the two-point correlator from point sources (src/NSL/Measurements/Hubbard/
twoPointCorrelationFunction.tpp:116-162) and the two-body correlators from momentum wall sources (TwoBodyCorrelator,
twoBodyCorrelationFunction.tpp; evaluated on the device by nslg_twobody_measure, see the class below).

TwoPointCorrelator.measure(phi, NumberTimeSources): for every source time tsrc = 0, Nt/Ntsrc, ... the point sources
src[x, tsrc, x] = 1 (one right-hand side per site x) are solved with CG on MM^dagger, multiplied by M^dagger to give
the columns of M^{-1}, shifted t -> t - tsrc with the anti-periodic sign on the wrapped slices and accumulated as
corr[t, y, x]; the sum is divided by NumberTimeSources. Here every source time's Nx right-hand sides go into one
batched solve (independent systems, mixed precision by default) instead of one CG per source time.

TwoPointCorrelator.measureK(phi, k, NumberTimeSources) (twoPointCorrelationFunction.tpp:169-233): the same with the
nb momentum wall sources W[k, s] of params["wallSources"] on the source slice in place of the Nx point sources,
projected onto the wall sources, block[t, s1, s2] = <W[k, s1], corrK[s2, t]>. measureK_blocks batches every momentum
and source time into one solve. (On the same configuration and source times the block equals
W[k]^* corr W[k]^T of measure's corr.)
"""
from __future__ import annotations

import math

import numpy as np

from . import tensor as T
from .fermion_matrix import HubbardExp, MatrixCombination, Species
from .solver import CG


class TwoPointCorrelator:
    def __init__(self, hfm: HubbardExp, species: Species = Species.Particle, *, eps: float = 1e-10,
                 maxIter: int = 1_000_000, precision="tf32x3", device=None, wallSources=None):
        self.hfm_ = hfm
        self.species_ = Species(species)
        self.eps = float(eps)  # relative true residual per right-hand side (|b| = 1 for a point source)
        self.maxIter = int(maxIter)
        self.precision = precision
        self.device = device
        # params["wallSources"] of the reference: (nk, nb, Nx) momentum wall sources, used by measureK
        self.wallSources = None
        if wallSources is not None:
            W = np.ascontiguousarray(np.asarray(wallSources, dtype=np.complex128))
            if W.ndim != 3 or W.shape[2] != hfm.Nx:
                raise ValueError(f"wallSources must be (nk, nb, Nx={hfm.Nx}), got {W.shape}")
            self.wallSources = W
        self.stats = None

    def source_times(self, NumberTimeSources: int):
        """tsrc = 0, Nt/Ntsrc, 2 Nt/Ntsrc, ... < Nt (integer step, as the reference's loop)."""
        Nt = self.hfm_.Nt
        return list(range(0, Nt, max(1, Nt // int(NumberTimeSources))))

    def sources(self, tsrcs):
        """src[k * Nx + x, tsrc_k, x] = 1 (the reference's srcVec_ for each source time, stacked)."""
        Nt, Nx = self.hfm_.Nt, self.hfm_.Nx
        b = np.zeros((len(tsrcs) * Nx, Nt, Nx), dtype=np.complex128)
        for k, t in enumerate(tsrcs):
            b[k * Nx + np.arange(Nx), t, np.arange(Nx)] = 1.0
        return b

    def _solve(self, phi, b):
        """M^{-1} b = M^dagger (M M^dagger)^{-1} b for every stacked source (one batched per-RHS solve), on the host."""
        hfm = self.hfm_
        if T.is_cuda(phi) or self.device is not None:
            import torch

            b = torch.from_numpy(b).to(phi.device if T.is_cuda(phi) else self.device)
        cg = CG(hfm, MatrixCombination.MMdagger, self.eps, self.maxIter, mode="per_rhs",
                precision=self.precision, stop="true_residual")
        x = cg(b)
        self.stats = cg.stats
        invM = hfm.Mdagger(x)
        if T.is_torch(invM):
            invM = invM.cpu().numpy()
        return invM

    @staticmethod
    def _shift_back(blk, tsrc: int):
        """invM.shift(-tsrc, -2, -1) of the reference: t -> t - tsrc along the time axis (second to last), the
        slices that wrap around picking up the anti-periodic sign."""
        Nt = blk.shape[-2]
        blk = np.roll(blk, -tsrc, axis=-2)
        if tsrc > 0:
            blk[..., Nt - tsrc:, :] *= -1.0
        return blk

    def _free_if_none(self, phi, NumberTimeSources):
        """No configuration: the reference's non-interacting correlators (U = 0 <=> phi = 0, one source time,
        twoPointCorrelationFunction.tpp:255-266 and :340-350)."""
        if phi is None:
            return np.zeros((self.hfm_.Nt, self.hfm_.Nx), dtype=np.complex128), 1
        if NumberTimeSources is None:
            raise TypeError("NumberTimeSources is required with a configuration")
        return phi, NumberTimeSources

    def measure(self, phi=None, NumberTimeSources: int | None = None):
        phi, NumberTimeSources = self._free_if_none(phi, NumberTimeSources)
        self.hfm_.populate(phi, self.species_)
        tsrcs = self.source_times(NumberTimeSources)
        invM = self._solve(phi, self.sources(tsrcs))  # (Ntsrc * Nx, Nt, Nx): columns of M^{-1}
        return self.accumulate(invM, tsrcs, NumberTimeSources)

    def accumulate(self, invM, tsrcs, NumberTimeSources: int):
        """corr[t, y, x] from the columns of M^{-1} of every source time (the shift to the source time with the
        anti-periodic sign and the average over source times of twoPointCorrelationFunction.tpp:139-162)."""
        Nt, Nx = self.hfm_.Nt, self.hfm_.Nx
        corr = np.zeros((Nt, Nx, Nx), dtype=np.complex128)
        for k, t in enumerate(tsrcs):
            blk = self._shift_back(invM[k * Nx:(k + 1) * Nx], t)  # (x_src, t, y)
            corr += np.transpose(blk, (1, 2, 0))  # (t, y, x_src)
        return corr / float(NumberTimeSources)

    def wall_sources(self, ks, tsrcs):
        """src[(i * Ntsrc + j) * nb + s, tsrc_j, :] = W[ks[i], s, :] (the reference's srcVecK_, stacked over the
        momenta and source times)."""
        W = self.wallSources[list(ks)]  # (nk', nb, Nx)
        nk, nb, Nx = W.shape
        b = np.zeros((nk, len(tsrcs), nb, self.hfm_.Nt, Nx), dtype=np.complex128)
        for j, t in enumerate(tsrcs):
            b[:, j, :, t, :] = W
        return b.reshape(nk * len(tsrcs) * nb, self.hfm_.Nt, Nx)

    def measureK_blocks(self, phi=None, NumberTimeSources: int | None = None, ks=None):
        """measureK for several momenta at once: all momenta's and source times' wall sources in one batched solve.
        Returns block[i, t, s1, s2] = sum_x conj(W[ks[i], s1, x]) corrK[s2, t, x], corrK the wall-source propagator
        shifted to the source time and averaged (divided by NumberTimeSources, as the reference). Without a
        configuration: the non-interacting blocks of every momentum, as the reference's measureK() writes first."""
        if self.wallSources is None:
            raise ValueError("measureK needs wallSources (nk, nb, Nx)")
        phi, NumberTimeSources = self._free_if_none(phi, NumberTimeSources)
        ks = list(range(self.wallSources.shape[0])) if ks is None else [int(k) for k in ks]
        hfm = self.hfm_
        Nt, Nx = hfm.Nt, hfm.Nx
        nb = self.wallSources.shape[1]
        hfm.populate(phi, self.species_)
        tsrcs = self.source_times(NumberTimeSources)
        invM = self._solve(phi, self.wall_sources(ks, tsrcs)).reshape(len(ks), len(tsrcs), nb, Nt, Nx)
        corrK = np.zeros((len(ks), nb, Nt, Nx), dtype=np.complex128)
        for j, t in enumerate(tsrcs):
            corrK += self._shift_back(invM[:, j].copy(), t)
        corrK /= float(NumberTimeSources)
        return np.einsum("kax,kbtx->ktab", np.conj(self.wallSources[ks]), corrK)

    def measureK(self, phi, k: int, NumberTimeSources: int):
        """twoPointCorrelationFunction.tpp:169-233: the (Nt, nb, nb) momentum block of wall source k."""
        return self.measureK_blocks(phi, NumberTimeSources, [k])[0]


# ----------------------------------------------------------------------------------------------------------------
# Two-body correlators
# ----------------------------------------------------------------------------------------------------------------
TWOBODY_CHANNELS = ("I1S1Iz1Sz1", "I1S1Iz1Sz0", "I1S1Iz1Szn1", "I1S1Iz0Sz1", "I1S1Iz0Szn1", "I1S1Izn1Sz1",
                    "I1S1Izn1Sz0", "I1S1Izn1Szn1", "I0S1Iz0Sz1", "I0S1Iz0Szn1", "I1S0Iz1Sz0", "I1S0Izn1Sz0")


def eq_modBZ(k, q, eps: float = 2e-12) -> bool:
    """k == q modulo the honeycomb reciprocal lattice (twoBodyCorrelationFunction.tpp:101-135): k - q = m C + n D with
    integer m, n for C = (4 pi/3, 0), D = (-2 pi/3, 2 pi/sqrt 3)."""
    d0, d1 = float(k[0]) - float(q[0]), float(k[1]) - float(q[1])
    c0, c1 = 4 * math.pi / 3, 0.0
    e0, e1 = -2 * math.pi / 3, 2 * math.pi / math.sqrt(3.0)
    den = c1 * e0 - c0 * e1
    m = (d1 * e0 - d0 * e1) / den
    n = (d0 * c1 - d1 * c0) / den
    return abs(round(m) - m) < eps and abs(round(n) - n) < eps


def momentum_tuples(momenta) -> np.ndarray:
    """The correlator keys (w, x, P, Q) with k_w + k_x == k_P + k_Q mod BZ, in lexicographic order: the entries the
    reference allocates as map[w][x][P][Q] (twoBodyCorrelationFunction.tpp:196-226) and writes to "w-x-P-Q"."""
    k = np.asarray(momenta, dtype=np.float64).reshape(-1, 2)
    nk = k.shape[0]
    s = (k[:, None, :] + k[None, :, :]).reshape(nk * nk, 2)  # k_w + k_x for (w, x) row-major
    d0 = s[:, None, 0] - s[None, :, 0]  # the test of eq_modBZ on every pair of pair sums at once
    d1 = s[:, None, 1] - s[None, :, 1]
    c0, c1 = 4 * math.pi / 3, 0.0
    e0, e1 = -2 * math.pi / 3, 2 * math.pi / math.sqrt(3.0)
    den = c1 * e0 - c0 * e1
    m = (d1 * e0 - d0 * e1) / den
    n = (d0 * c1 - d1 * c0) / den
    ok = (np.abs(np.round(m) - m) < 2e-12) & (np.abs(np.round(n) - n) < 2e-12)
    wx, pq = np.nonzero(ok)  # lexicographic in (w, x, P, Q)
    return np.stack([wx // nk, wx % nk, pq // nk, pq % nk], axis=1).astype(np.int64).reshape(-1, 4)


def honeycomb_wall_sources(lattice, ks=None):
    """Sublattice plane waves on a Honeycomb: momenta k = m1 b1 / L1 + m2 b2 / L2 (reciprocal vectors of
    honeycomb.tpp:81-84) and W[k, s, x] = exp(i k . r_x) / sqrt(L1 L2) on sublattice s (A = even, B = odd sites).
    The reference reads momenta and wall sources from its YAML input; these are one common choice."""
    L1, L2 = lattice.L
    b = np.array([[2 * math.pi / 3, 2 * math.pi / math.sqrt(3.0)], [2 * math.pi / 3, -2 * math.pi / math.sqrt(3.0)]])
    allk = [(m1, m2) for m2 in range(L2) for m1 in range(L1)]
    idx = range(len(allk)) if ks is None else ks
    mom = np.array([allk[i][0] * b[0] / L1 + allk[i][1] * b[1] / L2 for i in idx])
    sites = np.asarray(lattice.sites_, dtype=np.float64)
    ph = np.exp(1j * mom @ sites.T) / math.sqrt(L1 * L2)
    W = np.zeros((len(mom), 2, sites.shape[0]), dtype=np.complex128)
    W[:, 0, 0::2] = ph[:, 0::2]
    W[:, 1, 1::2] = ph[:, 1::2]
    return mom, W


class TwoBodyCorrelator:
    """TwoBodyCorrelator<Type, LatticeType, FermionMatrixType>(lattice, params)
    (src/NSL/Measurements/Hubbard/twoBodyCorrelationFunction.tpp:12-180) without its HDF5 layer.

    params: "Nt", "beta", "mu" (default 0), "wallSources" (nk, nb, Nx) and "momenta" (nk, 2), as the reference reads
    them. measure(phi, NumberTimeSources) evaluates one configuration on the GPU (nslg_twobody_measure: batched CG
    solves of every source time, projections and the twelve channel contractions on the device) and returns
    {channel: {(w, x, P, Q): (Nt, nb^2, nb^2)}} like the reference's map4D members; measure() with no configuration
    is the reference's non-interacting case (phi = 0, one source time, :319-328). The solves use the true-residual
    rule |b - A x| <= eps per source vector (the reference's CG defaults eps = 1e-12, maxIter = 10000,
    CG.hpp:31-40)."""

    CHANNELS = TWOBODY_CHANNELS

    def __init__(self, lattice, params: dict, *, FermionMatrixType=HubbardExp, eps: float = 1e-12,
                 maxIter: int = 10000, precision="fp64", ctx=None):
        self.params_ = params
        self.Nt = int(params["Nt"])
        self.hfm_ = FermionMatrixType(lattice, self.Nt, complex(params["beta"]), complex(params.get("mu", 0.0)),
                                      ctx=ctx)
        self.Nx = self.hfm_.Nx
        self.wall = np.ascontiguousarray(np.asarray(params["wallSources"], dtype=np.complex128))
        if self.wall.ndim != 3 or self.wall.shape[2] != self.Nx:
            raise ValueError(f"wallSources must be (nk, nb, Nx={self.Nx}), got {self.wall.shape}")
        self.nk, self.nb = int(self.wall.shape[0]), int(self.wall.shape[1])
        self.momenta = np.asarray(params["momenta"], dtype=np.float64).reshape(self.nk, 2)
        self.tuples = momentum_tuples(self.momenta)
        self.eps = float(eps)
        self.maxIter = int(maxIter)
        self.precision = precision
        self.stats = None

    def measure_array(self, phi, NumberTimeSources: int):
        """out[channel, tuple, t, i nb + j, l nb + k] for the tuples in self.tuples (numpy, or a CUDA tensor when
        phi is one)."""
        import ctypes as C

        from . import _lib
        from .fermion_matrix import precision_code

        lib = _lib.load()
        phi = T.as_c128(phi)
        shape = (_lib.TB_NCHANNELS, len(self.tuples), self.Nt, self.nb * self.nb, self.nb * self.nb)
        out = T.empty_like(phi, shape)
        tuples = np.ascontiguousarray(self.tuples, dtype=np.int64)
        st = _lib.CgStats()
        with T.stream_order(self.hfm_.ctx, phi, out):
            rc = lib.nslg_twobody_measure(self.hfm_.handle, T.ptr(phi), self.wall.ctypes.data, self.nk, self.nb,
                                          tuples.ctypes.data if len(tuples) else None, len(tuples),
                                          int(NumberTimeSources), self.eps, self.maxIter,
                                          precision_code(self.precision), T.ptr(out), C.byref(st))
        _lib.check(rc, allow=(_lib.OK, _lib.NOT_CONVERGED))
        self.stats = st.as_dict()
        if rc == _lib.NOT_CONVERGED:
            import warnings

            warnings.warn(f"TwoBodyCorrelator: {st.systems - st.converged} of {st.systems} solves did not converge "
                          f"within {self.maxIter} iterations", RuntimeWarning)
        self.hfm_.phi_ = phi
        return out

    def measure(self, phi=None, NumberTimeSources: int | None = None):
        if phi is None:  # the non-interacting correlators: U = 0 <=> phi = 0, one source time
            phi = np.zeros((self.Nt, self.Nx), dtype=np.complex128)
            NumberTimeSources = 1
        if NumberTimeSources is None:
            NumberTimeSources = int(self.params_.get("Number Time Sources", 1))
        arr = self.measure_array(phi, NumberTimeSources)
        if T.is_torch(arr):
            arr = arr.cpu().numpy()
        keys = [tuple(int(v) for v in t) for t in self.tuples]
        return {ch: {k: arr[c, u] for u, k in enumerate(keys)} for c, ch in enumerate(self.CHANNELS)}
