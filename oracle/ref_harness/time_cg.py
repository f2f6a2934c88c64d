"""Per-iteration time of the reference's own CG (CG.tpp:15-95 on libtorch, through the golden harness) against the
oracle's numpy restatement of the same iteration, on one host thread each: honeycomb 12x12 (Nx=288), Nt=64, beta=8,
U=3, one complex Gaussian right-hand side, a fixed number of iterations (eps far below reach).

Test infrastructure only (it runs the reference build in oracle/_ref/):
    make -C oracle/ref_harness REF=<reference checkout>
    python oracle/ref_harness/time_cg.py [iterations]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "golden_harness")
L, NT, BETA, U, SEED = (12, 12), 64, 8.0, 3.0, 2026
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def inputs():
    import numpy as np

    from nsl_gb300.lattice import Honeycomb

    lat = Honeycomb(L)
    Nx = lat.sites()
    rng = np.random.default_rng(SEED)
    phi = rng.standard_normal((NT, Nx)) * np.sqrt(BETA / NT * U) + 0j
    b = rng.standard_normal((1, NT, Nx)) + 1j * rng.standard_normal((1, NT, Nx))
    return lat, phi, b


def time_port(iters):
    """The oracle's CG (reference semantics) for `iters` iterations, numpy on one thread."""
    from oracle import nsl_oracle as O

    lat, phi, b = inputs()
    h = O.HubbardExp(lat.hopping_matrix(), NT, BETA)
    h.populate(phi)
    O.cg(h.MMdagger, b, eps=1e-300, max_iter=3)  # warm-up
    t0 = time.perf_counter()
    O.cg(h.MMdagger, b, eps=1e-300, max_iter=iters)
    return (time.perf_counter() - t0) / iters


def time_reference(iters):
    import numpy as np

    lat, phi, b = inputs()
    with tempfile.TemporaryDirectory() as d:
        phi.astype(np.complex128).tofile(os.path.join(d, "phi.bin"))
        b.astype(np.complex128).tofile(os.path.join(d, "psi.bin"))
        b.astype(np.complex128).tofile(os.path.join(d, "b.bin"))
        with open(os.path.join(d, "params.txt"), "w") as f:
            f.write(f"lattice honeycomb {L[0]} {L[1]}\nNt {NT}\nbeta {BETA!r}\nmu 0.0\nU {U!r}\nnrhs 1\n"
                    f"cg_eps 1e-300\ncg_maxiter {iters}\n")
        subprocess.run([HARNESS, d], check=True, capture_output=True)
        with open(os.path.join(d, "cg_seconds.txt")) as f:
            secs = float(f.read().split()[0])
        with open(os.path.join(d, "cg_iters.txt")) as f:
            done = int(f.readline().strip())
            msg = f.readline()
    if done < 0 and "did not converge within" in msg:  # exhausted (CG.tpp:90): every iteration ran
        done = iters
    return secs / max(done, 1), done


def main():
    iters = int(sys.argv[1]) if len(sys.argv) > 1 else 200
    if not os.path.exists(HARNESS):
        sys.exit(f"build the harness first: make -C oracle/ref_harness REF=<reference checkout> ({HARNESS} missing)")
    if os.environ.get("_TIME_CG_PORT"):
        print(json.dumps({"port_s_per_iter": time_port(iters)}))
        return
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1", _TIME_CG_PORT="1")
    port = json.loads(subprocess.run([sys.executable, __file__, str(iters)], env=env, check=True,
                                     capture_output=True, text=True).stdout)["port_s_per_iter"]
    ref, done = time_reference(iters)
    print(json.dumps({"workload": f"honeycomb {L[0]}x{L[1]} (Nx=288), Nt={NT}, beta={BETA}, U={U}, 1 RHS, "
                                  f"MMdag CG", "iterations": done, "threads": 1,
                      "reference_ms_per_iteration": ref * 1e3, "port_ms_per_iteration": port * 1e3,
                      "port_over_reference_time": port / ref}))


if __name__ == "__main__":
    main()
