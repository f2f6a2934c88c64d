"""The C++ drop-in header (include/nsl_gb300/nsl_dropin.hpp) compiles inside the reference's own templates.

Compile-only check against the reference NSL headers where the reference checkout is named by NSL_REFERENCE_DIR
(skipped when the variable is unset; GPU hosts have no checkout); the classes are exercised on the GPU through the same C ABI by the -m gpu tests. The two-point correlator's
host-side steps also run here, over a host stand-in of the library's entry points, against the reference's outputs.
"""
import os
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("NSL_REFERENCE_DIR", "")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "NSL")), reason="NSL_REFERENCE_DIR does not name the reference checkout")
def test_dropin_header_compiles_against_reference():
    torch = pytest.importorskip("torch")
    tdir = os.path.dirname(torch.__file__)
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-DFMT_HEADER_ONLY", "-w", f"-I{REF}/src/NSL", f"-I{REF}/src",
           f"-I{tdir}/include", f"-I{tdir}/include/torch/csrc/api/include",
           "-I" + os.path.join(ROOT, "oracle", "ref_harness"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_compile.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.fixture(scope="module")
def dropin_host_exe(tmp_path_factory):
    """tests/cpp/dropin_host.cpp built once against the reference headers and libtorch."""
    if not os.path.isdir(os.path.join(REF, "src", "NSL")):
        pytest.skip("NSL_REFERENCE_DIR does not name the reference checkout")
    torch = pytest.importorskip("torch")
    tdir = os.path.dirname(torch.__file__)
    exe = tmp_path_factory.mktemp("dropin") / "dropin_host"
    cmd = ["g++", "-std=c++20", "-O1", "-DFMT_HEADER_ONLY", "-D_GLIBCXX_USE_CXX11_ABI=1", "-w",
           f"-I{REF}/src/NSL", f"-I{REF}/src", f"-I{tdir}/include", f"-I{tdir}/include/torch/csrc/api/include",
           "-I" + os.path.join(ROOT, "oracle", "ref_harness"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_host.cpp"), "-o", str(exe),
           f"-L{tdir}/lib", f"-Wl,-rpath,{tdir}/lib", "-ltorch", "-ltorch_cpu", "-lc10"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("name", ["twopoint_honey3x3_nt8", "twopoint_honey2x2_nt6_mu"])
def test_dropin_two_point_host_logic(dropin_host_exe, tmp_path, name):
    """TwoPointCorrelatorGB300's own tensor steps (point and wall sources, shifts, averaging, projection) against the
    reference's TwoPointCorrelator outputs, with the library's entry points replaced by a host stand-in over the
    reference's HubbardExp and CG (tests/cpp/dropin_host.cpp)."""
    import numpy as np

    from conftest import load_twopoint, rel_err

    g = load_twopoint(name)
    nk, nb = g["wall"].shape[:2]
    (tmp_path / "params.txt").write_text(f"{g['L'][0]} {g['L'][1]} {g['Nt']} {g['beta']!r} {g['mu']!r} {nk} {nb} "
                                         f"{g['nts']}\n")
    g["phi"].astype(np.complex128).tofile(tmp_path / "phi.bin")
    g["wall"].astype(np.complex128).tofile(tmp_path / "wall.bin")
    r = subprocess.run([str(dropin_host_exe), str(tmp_path), "twopoint"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    for tag in "PH":
        corr = np.fromfile(tmp_path / f"corr_{tag}.bin", dtype=np.complex128).reshape(g["Nt"], g["Nx"], g["Nx"])
        assert rel_err(corr, g["corr_" + tag]) < 1e-10
        block = np.fromfile(tmp_path / f"block_{tag}.bin", dtype=np.complex128).reshape(nk, g["Nt"], nb, nb)
        assert rel_err(block, g["block_" + tag]) < 1e-10


@pytest.mark.parametrize("name", ["honey2x2_nt6_mu", "honey3x3_nt16"])
def test_dropin_fermion_matrix_in_reference_hmc_templates(dropin_host_exe, tmp_path, name):
    """HubbardExpGB300 inside the reference's HubbardFermionAction, Action sum, Leapfrog and LeapfrogRealForce (the
    drop-in's copies, populate order and result shapes at run time), over the host stand-in of the library's entry
    points: the action, force and both trajectories equal the reference's own outputs."""
    import numpy as np

    from conftest import load_golden, rel_err

    g = load_golden(name)
    L = tuple(int(v) for v in str(g["lattice"]).split()[1:])
    (tmp_path / "params.txt").write_text(f"{L[0]} {L[1]} {g['Nt']} {g['beta']!r} {g['mu']!r} {g['U']!r} "
                                         f"{int(g['nmd'])} {float(g['traj'])!r}\n")
    g["phi"].astype(np.complex128).tofile(tmp_path / "phi.bin")
    g["p"].astype(np.complex128).tofile(tmp_path / "p.bin")
    r = subprocess.run([str(dropin_host_exe), str(tmp_path), "action"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]

    def rd(fn, shape):
        return np.fromfile(tmp_path / fn, dtype=np.complex128).reshape(shape)

    shape = (g["Nt"], g["Nx"])
    assert abs(rd("S.bin", (1,))[0] - g["S"]) < 1e-12 * abs(g["S"])
    assert rel_err(rd("force.bin", shape), g["force"]) < 1e-12
    for k in ("lf_q", "lf_p", "lfr_q", "lfr_p"):
        assert rel_err(rd(k + ".bin", shape), g[k]) < 1e-12, k


@pytest.mark.parametrize("name", ["honey2x2_nt6_mu", "honey3x3_nt16"])
def test_dropin_cg_reference_semantics(dropin_host_exe, tmp_path, name):
    """CGGB300(hfm, MMdagger, eps, maxIter)(b) over the host stand-in (shared mode: the reference's own CG on the
    batch) equals the reference's CG solution in the fixture."""
    import numpy as np

    from conftest import load_golden, rel_err

    g = load_golden(name)
    L = tuple(int(v) for v in str(g["lattice"]).split()[1:])
    (tmp_path / "params.txt").write_text(f"{L[0]} {L[1]} {g['Nt']} {g['beta']!r} {g['mu']!r} "
                                         f"{float(g['cg_eps'])!r} 100000 {g['R']}\n")
    g["phi"].astype(np.complex128).tofile(tmp_path / "phi.bin")
    g["b"].astype(np.complex128).tofile(tmp_path / "b.bin")
    r = subprocess.run([str(dropin_host_exe), str(tmp_path), "cg"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    x = np.fromfile(tmp_path / "cg_x.bin", dtype=np.complex128).reshape(g["R"], g["Nt"], g["Nx"])
    assert rel_err(x, g["cg_x"]) < 1e-12
