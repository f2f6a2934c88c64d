"""Two-point correlator from point sources (src/NSL/Measurements/Hubbard/twoPointCorrelationFunction.tpp:116-162).

measure(phi, NumberTimeSources): for every source time tsrc = 0, Nt/Ntsrc, ... the point sources
src[x, tsrc, x] = 1 (one right-hand side per site x) are solved with CG on MM^dagger, multiplied by M^dagger to give
the columns of M^{-1}, shifted t -> t - tsrc with the anti-periodic sign on the wrapped slices and accumulated as
corr[t, y, x]; the sum is divided by NumberTimeSources. Here every source time's Nx right-hand sides go into one
batched solve (independent systems, mixed precision by default) instead of one CG per source time.
"""
from __future__ import annotations

import numpy as np

from . import tensor as T
from .fermion_matrix import HubbardExp, MatrixCombination, Species
from .solver import CG


class TwoPointCorrelator:
    def __init__(self, hfm: HubbardExp, species: Species = Species.Particle, *, eps: float = 1e-10,
                 maxIter: int = 1_000_000, precision="tf32x3", device=None):
        self.hfm_ = hfm
        self.species_ = Species(species)
        self.eps = float(eps)  # relative true residual per right-hand side (|b| = 1 for a point source)
        self.maxIter = int(maxIter)
        self.precision = precision
        self.device = device
        self.stats = None

    def sources(self, tsrcs):
        """src[k * Nx + x, tsrc_k, x] = 1 (the reference's srcVec_ for each source time, stacked)."""
        Nt, Nx = self.hfm_.Nt, self.hfm_.Nx
        b = np.zeros((len(tsrcs) * Nx, Nt, Nx), dtype=np.complex128)
        for k, t in enumerate(tsrcs):
            b[k * Nx + np.arange(Nx), t, np.arange(Nx)] = 1.0
        return b

    def measure(self, phi, NumberTimeSources: int):
        hfm = self.hfm_
        Nt, Nx = hfm.Nt, hfm.Nx
        hfm.populate(phi, self.species_)
        step = max(1, Nt // int(NumberTimeSources))
        tsrcs = list(range(0, Nt, step))
        b = self.sources(tsrcs)
        if T.is_cuda(phi) or self.device is not None:
            import torch

            b = torch.from_numpy(b).to(phi.device if T.is_cuda(phi) else self.device)
        cg = CG(hfm, MatrixCombination.MMdagger, self.eps, self.maxIter, mode="per_rhs",
                precision=self.precision, stop="true_residual")
        x = cg(b)
        self.stats = cg.stats
        invM = hfm.Mdagger(x)  # (Ntsrc * Nx, Nt, Nx): columns of M^{-1}
        if T.is_torch(invM):
            invM = invM.cpu().numpy()
        corr = np.zeros((Nt, Nx, Nx), dtype=np.complex128)
        for k, t in enumerate(tsrcs):
            blk = invM[k * Nx:(k + 1) * Nx]  # (x_src, t, y)
            blk = np.roll(blk, -t, axis=1)
            if t > 0:
                blk[:, Nt - t:, :] *= -1.0
            corr += np.transpose(blk, (1, 2, 0))  # (t, y, x_src)
        return corr / float(NumberTimeSources)
