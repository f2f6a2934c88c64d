"""Equal-time observables of a configuration: the electron density and the double occupancy per site.

The reference's HMC chains do not compute these (it measures correlators only); they are defined here from the
equal-time propagators the TwoPointCorrelator measures (src/NSL/Measurements/Hubbard/twoPointCorrelationFunction.tpp:
116-162): with particles p (spin up) and holes h (spin-down electrons after the particle-hole transformation),
    G_P(x) = <p_x p_x^dagger> = corr_P[t = 0, x, x],   G_H(x) = <h_x h_x^dagger> = corr_H[t = 0, x, x]
(averaged over the source times), so for one configuration
    n_up(x) = 1 - G_P(x),   n_down(x) = 1 - <h_x^dagger h_x> ... = G_H(x),
    n(x) = n_up(x) + n_down(x) = 1 - G_P(x) + G_H(x),
    d(x) = <n_up(x) n_down(x)> = (1 - G_P(x)) G_H(x)
(particles and holes are independent for a fixed auxiliary field, so the equal-time expectation factorises). For
phi = 0 this is the free theory: G = (1 + B)^{-1} with B the product of the time-slice matrices, and at mu = 0 on a
bipartite lattice n(x) = 1 exactly. Ensemble values are averages over the chain's configurations (real weights at
mu = 0 on bipartite lattices).
"""
from __future__ import annotations

import numpy as np

from .fermion_matrix import Species
from .measurement import TwoPointCorrelator


def equal_time_propagators(hfm, phi, NumberTimeSources: int = 1, *, eps: float = 1e-10, precision="fp64",
                           maxIter: int = 20000, stats: list | None = None):
    """(G_P, G_H): the equal-time diagonal of M^{-1} for both species, each (Nx,), averaged over source times.
    The solves' statistics are appended to `stats` when given (a configuration near a zero of det M makes MM^dagger
    too ill-conditioned for CG; its solves then report fewer converged systems than they ran)."""
    out = []
    for sp in (Species.Particle, Species.Hole):
        tp = TwoPointCorrelator(hfm, sp, eps=eps, maxIter=maxIter, precision=precision)
        corr = tp.measure(phi, NumberTimeSources)
        if stats is not None:
            stats.append(tp.stats)
        out.append(np.diagonal(np.asarray(corr[0])).astype(np.complex128))
    return out[0], out[1]


def density_and_double_occupancy(hfm, phi, NumberTimeSources: int = 1, **kw):
    """(n(x), d(x)) for one configuration phi (see the module docstring for the definitions)."""
    gp, gh = equal_time_propagators(hfm, phi, NumberTimeSources, **kw)
    return 1.0 - gp + gh, (1.0 - gp) * gh


def chain_observables(hfm, configs, NumberTimeSources: int = 1, **kw):
    """Averages of n and d over a chain's configurations (iterable of phi): ({"n": mean over sites and
    configurations, "d": ..., their standard errors, "unconverged": configurations whose solves did not all
    converge}, per-configuration site means)."""
    ns, ds = [], []
    unconverged = 0
    for phi in configs:
        st = []
        n, d = density_and_double_occupancy(hfm, phi, NumberTimeSources, stats=st, **kw)
        unconverged += any(s["converged"] != s["systems"] for s in st)
        ns.append(np.mean(n))
        ds.append(np.mean(d))
    ns, ds = np.array(ns), np.array(ds)
    return {"n": complex(ns.mean()), "d": complex(ds.mean()), "unconverged": unconverged,
            "n_err": float(ns.std(ddof=1) / np.sqrt(len(ns))) if len(ns) > 1 else 0.0,
            "d_err": float(ds.std(ddof=1) / np.sqrt(len(ds))) if len(ds) > 1 else 0.0}, (ns, ds)
