"""The C++ drop-in classes (include/nsl_gb300/nsl_dropin.hpp) on the GPU through the real libnslgpu.so.

tests/cpp/dropin_host.cpp built with -DNSLG_DROPIN_DEVICE: HubbardExpGB300 inside the reference's own
HubbardFermionAction, Action sum, Leapfrog and LeapfrogRealForce templates, CGGB300 on MM^dagger and
TwoPointCorrelatorGB300, all reaching the library's CUDA kernels, against the reference's outputs in the golden
fixtures. Needs the reference's headers (NSL_REFERENCE_DIR names the checkout; skipped otherwise) and libtorch's C++
headers and libraries from the installed torch.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, ensure_built, load_golden, load_twopoint, rel_err

pytestmark = pytest.mark.gpu

REF = os.environ.get("NSL_REFERENCE_DIR", "")


@pytest.fixture(scope="module")
def dropin_device_exe(tmp_path_factory):
    if not os.path.isdir(os.path.join(REF, "src", "NSL")):
        pytest.skip("NSL_REFERENCE_DIR does not name the reference checkout")
    torch = pytest.importorskip("torch")
    tdir = os.path.dirname(torch.__file__)
    if not os.path.isdir(os.path.join(tdir, "include", "torch", "csrc", "api", "include")):
        pytest.skip("the installed torch has no C++ headers")
    lib = ensure_built()
    exe = tmp_path_factory.mktemp("dropin_dev") / "dropin_device"
    abi = "1" if torch.compiled_with_cxx11_abi() else "0"
    cmd = ["g++", "-std=c++20", "-O1", "-DFMT_HEADER_ONLY", f"-D_GLIBCXX_USE_CXX11_ABI={abi}", "-DNSLG_DROPIN_DEVICE",
           "-w", f"-I{REF}/src/NSL", f"-I{REF}/src", f"-I{tdir}/include", f"-I{tdir}/include/torch/csrc/api/include",
           "-I" + os.path.join(ROOT, "oracle", "ref_harness"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_host.cpp"), "-o", str(exe),
           f"-L{os.path.dirname(lib)}", f"-Wl,-rpath,{os.path.dirname(lib)}", "-lnslgpu",
           f"-L{tdir}/lib", f"-Wl,-rpath,{tdir}/lib", "-ltorch", "-ltorch_cpu", "-lc10"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run(exe, d, mode):
    r = subprocess.run([str(exe), str(d), mode], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])


@pytest.mark.parametrize("name", ["honey2x2_nt6_mu", "honey3x3_nt16"])
def test_dropin_action_and_trajectories_on_gpu(dropin_device_exe, tmp_path, name):
    """The reference's own HMC templates with HubbardExpGB300 on the GPU: action, force and both leapfrog trajectories
    against the reference's outputs (FP64; the bars of the library's own action and leapfrog tests)."""
    g = load_golden(name)
    L = tuple(int(v) for v in str(g["lattice"]).split()[1:])
    (tmp_path / "params.txt").write_text(f"{L[0]} {L[1]} {g['Nt']} {g['beta']!r} {g['mu']!r} {g['U']!r} "
                                         f"{int(g['nmd'])} {float(g['traj'])!r}\n")
    g["phi"].astype(np.complex128).tofile(tmp_path / "phi.bin")
    g["p"].astype(np.complex128).tofile(tmp_path / "p.bin")
    _run(dropin_device_exe, tmp_path, "action")

    def rd(fn, shape):
        return np.fromfile(tmp_path / fn, dtype=np.complex128).reshape(shape)

    shape = (g["Nt"], g["Nx"])
    assert abs(rd("S.bin", (1,))[0] - g["S"]) < 1e-10 * abs(g["S"])
    assert rel_err(rd("force.bin", shape), g["force"]) < 1e-10
    for k in ("lf_q", "lf_p", "lfr_q", "lfr_p"):
        assert rel_err(rd(k + ".bin", shape), g[k]) < 1e-9, k


@pytest.mark.parametrize("name", ["honey2x2_nt6_mu", "honey3x3_nt16"])
def test_dropin_cg_on_gpu(dropin_device_exe, tmp_path, name):
    """CGGB300(hfm, MMdagger, eps, maxIter)(b) on the GPU (the reference's batch semantics) against the reference's
    CG solution."""
    g = load_golden(name)
    L = tuple(int(v) for v in str(g["lattice"]).split()[1:])
    (tmp_path / "params.txt").write_text(f"{L[0]} {L[1]} {g['Nt']} {g['beta']!r} {g['mu']!r} "
                                         f"{float(g['cg_eps'])!r} 100000 {g['R']}\n")
    g["phi"].astype(np.complex128).tofile(tmp_path / "phi.bin")
    g["b"].astype(np.complex128).tofile(tmp_path / "b.bin")
    _run(dropin_device_exe, tmp_path, "cg")
    x = np.fromfile(tmp_path / "cg_x.bin", dtype=np.complex128).reshape(g["R"], g["Nt"], g["Nx"])
    assert rel_err(x, g["cg_x"]) < 1e-9


@pytest.mark.parametrize("name", ["twopoint_honey3x3_nt8", "twopoint_honey2x2_nt6_mu"])
def test_dropin_two_point_on_gpu(dropin_device_exe, tmp_path, name):
    """TwoPointCorrelatorGB300::measure / measureK on the GPU against the reference's correlators."""
    g = load_twopoint(name)
    nk, nb = g["wall"].shape[:2]
    (tmp_path / "params.txt").write_text(f"{g['L'][0]} {g['L'][1]} {g['Nt']} {g['beta']!r} {g['mu']!r} {nk} {nb} "
                                         f"{g['nts']}\n")
    g["phi"].astype(np.complex128).tofile(tmp_path / "phi.bin")
    g["wall"].astype(np.complex128).tofile(tmp_path / "wall.bin")
    _run(dropin_device_exe, tmp_path, "twopoint")
    for tag in "PH":
        corr = np.fromfile(tmp_path / f"corr_{tag}.bin", dtype=np.complex128).reshape(g["Nt"], g["Nx"], g["Nx"])
        assert rel_err(corr, g["corr_" + tag]) < 1e-9
        block = np.fromfile(tmp_path / f"block_{tag}.bin", dtype=np.complex128).reshape(nk, g["Nt"], nb, nb)
        assert rel_err(block, g["block_" + tag]) < 1e-9
