import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libnslgpu.so")
    config.addinivalue_line("markers", "slow: longer CPU test")


def golden_path(name):
    return os.path.join(ROOT, "tests", "golden", name + ".npz")


GOLDEN_CASES = ["ring2_nt8", "ring6_nt4_complexphi_mu", "ring4_nt8", "honey2x2_nt6_mu", "honey3x3_nt16",
                "honey6x6_nt32_beta8"]


TWOBODY_CASES = ["twobody_honey3x3_nt8", "twobody_honey2x2_nt6_mu"]
TWOPOINT_CASES = ["twopoint_honey3x3_nt8", "twopoint_honey2x2_nt6_mu"]


def load_twobody(name):
    """A two-body correlator fixture: phi, wall, momenta, tuples, out (12, ntuple, Nt, nb^2, nb^2) and the lattice.
    Two-point fixtures load the same way: phi, wall, momenta, corr_P / corr_H (Nt, Nx, Nx) from measure(nts) and
    block_P / block_H (nk, Nt, nb, nb) from measureK(k, nts)."""
    import numpy as np

    z = np.load(golden_path(name))
    d = {k: z[k] for k in z.files}
    Nt, Nx, beta, mu, U, nts = d["params"]
    d.update(Nt=int(Nt), Nx=int(Nx), beta=float(beta), mu=float(mu), U=float(U), nts=int(nts))
    d["L"] = tuple(int(v) for v in str(d["lattice"]).split()[1:])
    return d


load_twopoint = load_twobody


def load_golden(name):
    import numpy as np

    z = np.load(golden_path(name))
    d = {k: z[k] for k in z.files}
    Nt, Nx, R, beta, mu, U = d["params"]
    d.update(Nt=int(Nt), Nx=int(Nx), R=int(R), beta=float(beta), mu=float(mu), U=float(U))
    d["lattice_spec"] = str(d["lattice"]).split()
    return d


def rel_err(a, b):
    """max |a - b| / max |b| (max-norm relative error)."""
    import numpy as np

    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def ensure_built():
    """Builds libnslgpu.so in-tree if it is missing (nvcc cross-compiles without a GPU)."""
    import os

    from nsl_gb300 import build as B

    if os.path.exists(B.CSRC) and B.nvcc_available():
        B.build()  # incremental: recompiles only what changed
    return B.LIB
