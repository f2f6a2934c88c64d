"""The C ABI from plain C: tests/cpp/abi_client.c is compiled with gcc against include/nsl_gb300.h, linked to
libnslgpu.so and run on a golden case; its outputs (M, CG solution, log det, gradient) must match the reference's."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, ensure_built, load_golden, rel_err

pytestmark = pytest.mark.gpu


def test_c_client_matches_reference(tmp_path):
    from oracle import nsl_oracle as O

    lib = ensure_built()
    exe = tmp_path / "abi_client"
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-std=c11", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "abi_client.c"), "-o", str(exe), "-L" + libdir,
                    "-l:libnslgpu.so", "-lm", "-Wl,-rpath," + libdir], check=True)
    g = load_golden("honey3x3_nt16")
    for k in ("hops", "phi", "psi"):
        np.ascontiguousarray(g[k], dtype=np.complex128).tofile(tmp_path / f"{k}.bin")
    (tmp_path / "params.txt").write_text(f"{g['Nx']} {g['Nt']} {g['R']} {g['beta']!r} {g['mu']!r}\n")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    shape = (g["R"], g["Nt"], g["Nx"])
    M = np.fromfile(tmp_path / "M.bin", dtype=np.complex128).reshape(shape)
    x = np.fromfile(tmp_path / "x.bin", dtype=np.complex128).reshape(shape)
    ld = np.fromfile(tmp_path / "logdet.bin", dtype=np.complex128)[0]
    grad = np.fromfile(tmp_path / "grad.bin", dtype=np.complex128).reshape(g["Nt"], g["Nx"])
    assert rel_err(M, g["M_P"]) < 1e-12
    assert abs(ld - complex(g["logdet_P"])) <= 1e-10 * max(1.0, abs(complex(g["logdet_P"])))
    assert rel_err(grad, g["grad_P"]) < 1e-10
    h = O.HubbardExp(g["hops"], g["Nt"], g["beta"], g["mu"])
    h.populate(g["phi"], O.PARTICLE)
    res = np.linalg.norm((g["psi"] - h.MMdagger(x)).reshape(g["R"], -1), axis=1)
    assert (res / np.linalg.norm(g["psi"].reshape(g["R"], -1), axis=1)).max() < 2e-10
    assert "converged 2/2" in r.stdout or f"converged {g['R']}/{g['R']}" in r.stdout
