"""Generate tests/golden/stable_*.npz: the oracle's stratified log det M and gradient at the low-temperature
configurations, where the reference's own direct product is inaccurate (its log det is NaN at beta >= 8).

The oracle's stratified forms (oracle/nsl_oracle.py: logDetM_stable, gradLogDetM_stable) are pinned by
tests/test_oracle_stable.py against dense inverses of M, dense log-determinants, finite differences and the
reference's fixtures. Here they are evaluated once on the large configurations (too slow to recompute inside a
test), on selected time slices of the gradient, for both species:
  honeycomb 12x12 (Nx = 288), Nt = 64, beta = 8, U = 3 (phi ~ N(0, delta U), seed 11)
  honeycomb 24x24 (Nx = 1152), Nt = 128, beta = 12, U = 3 (phi ~ N(0, delta U), seed 12)
The field is regenerated from its seed (numpy's default_rng, identical on every platform) and stored as well.

Run from the repository root:  python tests/golden/make_stable_golden.py [cfg2|cfg3]
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nsl_gb300.lattice import Honeycomb  # noqa: E402  (vectorised neighbour search; same K as the reference's)
from oracle import nsl_oracle as O  # noqa: E402

CASES = {
    "cfg2": dict(L=(12, 12), Nt=64, beta=8.0, U=3.0, seed=11, slices=[0, 1, 20, 31, 62, 63]),
    "cfg3": dict(L=(24, 24), Nt=128, beta=12.0, U=3.0, seed=12, slices=[0, 63, 127]),
}


def field(c, Nx):
    rng = np.random.default_rng(c["seed"])
    return rng.standard_normal((c["Nt"], Nx)) * np.sqrt(c["beta"] / c["Nt"] * c["U"]) + 0j


def make(name):
    c = CASES[name]
    K = Honeycomb(c["L"]).hopping_matrix()
    Nx = K.shape[0]
    phi = field(c, Nx)
    out = {"phi": phi, "slices": np.array(c["slices"]),
           "params": np.array([c["L"][0], c["L"][1], c["Nt"], c["beta"], c["U"], c["seed"]], dtype=float)}
    for sp, tag in ((O.PARTICLE, "P"), (O.HOLE, "H")):
        h = O.HubbardExp(K, c["Nt"], c["beta"], 0.0, sp)
        h.populate(phi)
        t0 = time.time()
        out[f"logdet_{tag}"] = np.array(h.logDetM_stable())
        g = h.gradLogDetM_stable(slices=c["slices"])
        out[f"grad_{tag}"] = g[c["slices"]]
        print(f"{name} {tag}: {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", f"stable_{name}.npz"), **out)


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(CASES)):
        make(n)
