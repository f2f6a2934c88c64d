"""CPU checks of the C ABI library and the host-side logic (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, ensure_built, load_golden


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            names += re.findall(r"NSLG_API\s+[\w\s\*]+?\b(nslg_\w+)\s*\(", src)
    return names


def test_library_loads_and_exports_every_declared_symbol():
    lib = ctypes.CDLL(ensure_built())
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from nsl_gb300 import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES), set(declared_symbols()) - set(_lib.SIGNATURES)


def test_only_nslg_symbols_exported():
    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", ensure_built()], capture_output=True, text=True).stdout
    syms = [l.split()[-1] for l in out.splitlines() if l.split() and l.split()[-2] in ("T", "D", "B")]
    foreign = [s for s in syms if not s.startswith("nslg_") and not s.startswith("_")]
    assert not foreign, foreign[:20]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_lattices_match_reference(name):
    from nsl_gb300.lattice import Honeycomb, Ring

    g = load_golden(name)
    spec = g["lattice_spec"]
    lat = Ring(int(spec[1])) if spec[0] == "ring" else Honeycomb((int(spec[1]), int(spec[2])))
    assert lat.sites() == g["Nx"]
    assert np.array_equal(lat.hopping_matrix(), g["hops"])


def test_honeycomb_properties():
    """Coordination 3 and Hermitian K (Tests/Lattice/test_honeycomb.cpp:17-87), bipartite."""
    from nsl_gb300.lattice import Honeycomb

    for L in ((3, 3), (4, 6), (12, 12)):
        lat = Honeycomb(L)
        K = lat.hopping_matrix()
        assert np.allclose(K, K.conj().T)
        assert np.all(lat.adjacency_matrix().sum(axis=1) == 3)
        assert lat.bipartite()


@pytest.mark.parametrize("name", ["twobody_honey3x3_nt8", "twobody_honey2x2_nt6_mu"])
def test_twobody_momentum_keys_match_reference(name):
    """The host-side key list of TwoBodyCorrelator equals the keys the reference allocated, and the package's
    honeycomb wall sources are the fixture's."""
    from conftest import load_twobody
    from nsl_gb300.lattice import Honeycomb
    from nsl_gb300.measurement import honeycomb_wall_sources, momentum_tuples

    g = load_twobody(name)
    assert np.array_equal(momentum_tuples(g["momenta"]), g["tuples"])
    mom, W = honeycomb_wall_sources(Honeycomb(g["L"]))
    idx = [int(np.argmin(np.abs(mom - k).sum(axis=1))) for k in g["momenta"]]
    assert np.abs(W[idx] - g["wall"]).max() < 1e-15
    assert np.abs(mom[idx] - g["momenta"]).max() < 1e-15


def test_python_binding_arity_matches_the_header():
    """Every ctypes signature has as many arguments as the header's declaration (a mismatch would pass arguments
    shifted into the wrong parameters)."""
    from nsl_gb300 import _lib

    src = "".join(open(os.path.join(ROOT, "include", f)).read() for f in sorted(os.listdir(os.path.join(ROOT, "include")))
                  if f.endswith(".h"))
    decls = re.findall(r"NSLG_API\s+[\w\s\*]+?\b(nslg_\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.S)
    assert len(decls) >= 20
    for name, params in decls:
        params = params.strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(_lib.SIGNATURES[name][1]) == n, (name, n, len(_lib.SIGNATURES[name][1]))


def test_c_client_builds_against_the_header_and_library(tmp_path):
    """The header is plain C11 and the library links from C (tests/cpp/abi_client.c; it runs in the -m gpu tests)."""
    import subprocess

    lib = ensure_built()
    libdir = os.path.dirname(lib)
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-O2", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "abi_client.c"), "-o", str(tmp_path / "abi_client"),
                        "-L" + libdir, "-l:libnslgpu.so", "-lm", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_pointer_rule_rejects_other_gpus_memory(tmp_path):
    """The rule every entry point applies to a caller buffer (nsl_gb300/csrc/ptr_class.h): device memory of the
    handle's GPU and managed memory are used in place, host memory is staged, and device memory of another GPU is
    refused (NSLG_ERR_ARG) before anything is launched. Compiled with the host C compiler: no GPU involved."""
    import subprocess

    src = tmp_path / "ptr_rule.c"
    src.write_text(r'''
#include <stdio.h>
#include "ptr_class.h"
int main(void) {
    int bad = 0;
    bad |= nslg_ptr_class(1, 0, 0, 0) != NSLG_PTR_DEVICE;   /* device memory of the handle's GPU */
    bad |= nslg_ptr_class(1, 0, 3, 3) != NSLG_PTR_DEVICE;
    bad |= nslg_ptr_class(1, 0, 1, 0) != NSLG_PTR_FOREIGN;  /* another GPU's memory: refused */
    bad |= nslg_ptr_class(1, 0, 0, 2) != NSLG_PTR_FOREIGN;
    bad |= nslg_ptr_class(0, 1, 1, 0) != NSLG_PTR_DEVICE;   /* managed: addressable everywhere */
    bad |= nslg_ptr_class(0, 0, -1, 0) != NSLG_PTR_HOST;    /* pageable or pinned host memory: staged */
    printf("%d\n", bad);
    return bad;
}
''')
    exe = tmp_path / "ptr_rule"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "nsl_gb300", "csrc"),
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)]).returncode == 0
