"""Generate the golden fixtures in this directory from the reference NSL implementation.

Test infrastructure only. For every case below this script writes seeded inputs (phi, psi, b, p) as raw complex128,
runs the reference harness (oracle/ref_harness/golden_harness.cpp, built by its Makefile into oracle/_ref/) on them
and packs inputs and reference outputs into ``<case>.npz``. The reference is evaluated by its own code
(src/NSL/FermionMatrix/Impl/hubbardExp.tpp, hubbardDiag.tpp, LinAlg/Solver/Impl/CG.tpp, Action/Implementations/*.tpp,
Integrator/Impl/leapfrog*.tpp, Measurements/Hubbard/twoBodyCorrelationFunction.tpp, twoPointCorrelationFunction.tpp) on libtorch's CPU complex128 path.

Run from the repository root, where the reference checkout is available:
    make -C oracle/ref_harness REF=<reference checkout>
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "golden_harness")


def honeycomb_sites(L1, L2):
    return 2 * L1 * L2


# name: lattice, Nt, beta, mu, U, nrhs, phi kind, extras
CASES = {
    # Ring lattice of the reference force test (Tests/Action/test_force.cpp:30-40): Nx=2, Nt=8, beta=2, U=3.
    "ring2_nt8": dict(lattice=("ring", 2), Nt=8, beta=2.0, mu=0.0, U=3.0, nrhs=3, phi="real",
                      logdet=True, cg=(1e-12, 100000), lf=(10, 1.0), seed=11),
    # Ring, general complex phi (the reference M tests draw phi.rand() complex, test_fermionMatrixHubbardExp.cpp:148-151).
    "ring6_nt4_complexphi_mu": dict(lattice=("ring", 6), Nt=4, beta=1.0, mu=0.3, U=2.0, nrhs=2, phi="complex",
                                    logdet=True, cg=None, lf=None, seed=12),
    "ring4_nt8": dict(lattice=("ring", 4), Nt=8, beta=2.0, mu=0.0, U=3.0, nrhs=3, phi="real",
                      logdet=True, cg=(1e-12, 100000), lf=(10, 1.0), seed=13),
    # Honeycomb 2x2 with a chemical potential.
    "honey2x2_nt6_mu": dict(lattice=("honeycomb", 2, 2), Nt=6, beta=1.5, mu=0.2, U=2.0, nrhs=2, phi="real",
                            logdet=True, cg=(1e-12, 100000), lf=(4, 0.5), seed=14),
    # Plain Hubbard HMC configuration: honeycomb 3x3 (Nx=18), Nt=16, beta=4, U=2.
    "honey3x3_nt16": dict(lattice=("honeycomb", 3, 3), Nt=16, beta=4.0, mu=0.0, U=2.0, nrhs=2, phi="real",
                          logdet=True, cg=(1e-12, 100000), lf=(10, 1.0), seed=1234),
    # Larger lattice at low temperature: honeycomb 6x6 (Nx=72), Nt=32, beta=8, U=3 (operator applications only).
    "honey6x6_nt32_beta8": dict(lattice=("honeycomb", 6, 6), Nt=32, beta=8.0, mu=0.0, U=3.0, nrhs=2, phi="real",
                                logdet=True, cg=None, lf=None, seed=15),
}


# Two-body correlator cases (TwoBodyCorrelator::measure(NumberTimeSources), twoBodyCorrelationFunction.tpp:188-306):
# honeycomb sublattice plane-wave wall sources for a subset of the lattice momenta (indices into the L1 x L2 grid).
TWOBODY_CASES = {
    "twobody_honey3x3_nt8": dict(lattice=("honeycomb", 3, 3), Nt=8, beta=2.0, mu=0.0, U=2.0, ks=(0, 1, 3, 4, 5),
                                 nts=2, seed=21),
    "twobody_honey2x2_nt6_mu": dict(lattice=("honeycomb", 2, 2), Nt=6, beta=1.5, mu=0.2, U=2.0, ks=(0, 1, 2, 3),
                                    nts=3, seed=22),
}
# Two-point correlator cases, both species: TwoPointCorrelator::measure(NumberTimeSources) with point sources
# (twoPointCorrelationFunction.tpp:116-162) and measureK(k, NumberTimeSources) with the wall sources above
# (:169-233), on the reference's HubbardExp and CG(MM^dagger) with its default eps 1e-12 over the whole source batch.
TWOPOINT_CASES = {
    "twopoint_honey3x3_nt8": dict(lattice=("honeycomb", 3, 3), Nt=8, beta=2.0, mu=0.0, U=2.0, ks=(0, 1, 4),
                                  nts=4, seed=31),
    "twopoint_honey2x2_nt6_mu": dict(lattice=("honeycomb", 2, 2), Nt=6, beta=1.5, mu=0.2, U=2.0, ks=(0, 1, 2, 3),
                                     nts=2, seed=32),
}
# Not a fixture: the reference's TwoBodyCorrelator with FermionMatrixType = HubbardDiag ("diag": True above, the
# harness's "twobody nk nb nts diag") applies HubbardDiag's single-vector operators to the (nk, nb, Nt, Nx) source
# batch, which shifts along the leading axis; its channels differ from the per-vector definition by ~100%.


def honeycomb_positions(L1, L2):
    """Site coordinates of the reference Honeycomb (honeycomb.tpp:73-95)."""
    a = np.array([[1.5, 0.8660254037844386], [1.5, -0.8660254037844386]])
    r = np.array([1.0, 0.0])
    sites = np.zeros((2 * L1 * L2, 2))
    for l1 in range(L1):
        for l2 in range(L2):
            i = l1 + L1 * l2
            sites[2 * i] = l1 * a[0] + l2 * a[1] + r / 2
            sites[2 * i + 1] = l1 * a[0] + l2 * a[1] - r / 2
    return sites


def wall_sources(L1, L2, ks):
    """Momenta m1 b1 / L1 + m2 b2 / L2 (honeycomb.tpp:81-84) and sublattice plane waves exp(i k.r) / sqrt(L1 L2)."""
    b = np.array([[2 * np.pi / 3, 2 * np.pi / np.sqrt(3.0)], [2 * np.pi / 3, -2 * np.pi / np.sqrt(3.0)]])
    allk = [(m1, m2) for m2 in range(L2) for m1 in range(L1)]
    mom = np.array([allk[i][0] * b[0] / L1 + allk[i][1] * b[1] / L2 for i in ks])
    sites = honeycomb_positions(L1, L2)
    ph = np.exp(1j * mom @ sites.T) / np.sqrt(L1 * L2)
    W = np.zeros((len(ks), 2, sites.shape[0]), dtype=np.complex128)
    W[:, 0, 0::2] = ph[:, 0::2]
    W[:, 1, 1::2] = ph[:, 1::2]
    return mom, W


def run_twobody_case(name, spec, workdir):
    d = os.path.join(workdir, name)
    os.makedirs(d, exist_ok=True)
    lat = spec["lattice"]
    Nt, Nx = spec["Nt"], nsites(lat)
    rng = np.random.default_rng(spec["seed"])
    phi = rng.standard_normal((Nt, Nx)) * np.sqrt(spec["beta"] / Nt * spec["U"]) + 0j
    mom, W = wall_sources(lat[1], lat[2], spec["ks"])
    phi.astype(np.complex128).tofile(os.path.join(d, "phi.bin"))
    W.astype(np.complex128).tofile(os.path.join(d, "wall.bin"))
    np.ascontiguousarray(mom, dtype=np.float64).tofile(os.path.join(d, "momenta.bin"))
    nk, nb = W.shape[0], W.shape[1]
    lines = ["lattice " + " ".join(str(x) for x in lat), f"Nt {Nt}", f"beta {spec['beta']!r}", f"mu {spec['mu']!r}",
             f"U {spec['U']!r}", "nrhs 1", f"twobody {nk} {nb} {spec['nts']}" + (" diag" if spec.get("diag") else "")]
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    subprocess.run([HARNESS, d], check=True)
    tuples = np.loadtxt(os.path.join(d, "tb_tuples.txt"), dtype=np.int64).reshape(-1, 4)
    out = np.fromfile(os.path.join(d, "tb_out.bin"), dtype=np.complex128).reshape(12, len(tuples), Nt, nb * nb,
                                                                                  nb * nb)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), phi=phi, wall=W, momenta=mom, tuples=tuples, out=out,
                        params=np.array([Nt, Nx, spec["beta"], spec["mu"], spec["U"], spec["nts"]], dtype=np.float64),
                        kind=np.array("diag" if spec.get("diag") else "exp"),
                        lattice=np.array(" ".join(str(x) for x in lat)))
    print(f"{name}: Nx={Nx} Nt={Nt} nk={nk} tuples={len(tuples)}")


def run_twopoint_case(name, spec, workdir):
    d = os.path.join(workdir, name)
    os.makedirs(d, exist_ok=True)
    lat = spec["lattice"]
    Nt, Nx = spec["Nt"], nsites(lat)
    rng = np.random.default_rng(spec["seed"])
    phi = rng.standard_normal((Nt, Nx)) * np.sqrt(spec["beta"] / Nt * spec["U"]) + 0j
    mom, W = wall_sources(lat[1], lat[2], spec["ks"])
    phi.astype(np.complex128).tofile(os.path.join(d, "phi.bin"))
    W.astype(np.complex128).tofile(os.path.join(d, "wall.bin"))
    nk, nb = W.shape[0], W.shape[1]
    lines = ["lattice " + " ".join(str(x) for x in lat), f"Nt {Nt}", f"beta {spec['beta']!r}", f"mu {spec['mu']!r}",
             f"U {spec['U']!r}", "nrhs 1", f"twopoint {nk} {nb} {spec['nts']}"]
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    subprocess.run([HARNESS, d], check=True)

    def rd(fn, shape):
        return np.fromfile(os.path.join(d, fn), dtype=np.complex128).reshape(shape)

    np.savez_compressed(os.path.join(HERE, name + ".npz"), phi=phi, wall=W, momenta=mom,
                        corr_P=rd("tp_corr_P.bin", (Nt, Nx, Nx)), corr_H=rd("tp_corr_H.bin", (Nt, Nx, Nx)),
                        block_P=rd("tpk_P.bin", (nk, Nt, nb, nb)), block_H=rd("tpk_H.bin", (nk, Nt, nb, nb)),
                        params=np.array([Nt, Nx, spec["beta"], spec["mu"], spec["U"], spec["nts"]], dtype=np.float64),
                        lattice=np.array(" ".join(str(x) for x in lat)))
    print(f"{name}: Nx={Nx} Nt={Nt} nk={nk} nts={spec['nts']}")


def nsites(lat):
    return lat[1] if lat[0] == "ring" else honeycomb_sites(lat[1], lat[2])


def make_inputs(spec):
    rng = np.random.default_rng(spec["seed"])
    Nt, Nx, R = spec["Nt"], nsites(spec["lattice"]), spec["nrhs"]
    delta = spec["beta"] / Nt
    if spec["phi"] == "real":
        phi = rng.standard_normal((Nt, Nx)) * np.sqrt(delta * spec["U"]) + 0j
    else:
        phi = rng.random((Nt, Nx)) + 1j * rng.random((Nt, Nx))
    psi = rng.standard_normal((R, Nt, Nx)) + 1j * rng.standard_normal((R, Nt, Nx))
    b = rng.standard_normal((R, Nt, Nx)) + 1j * rng.standard_normal((R, Nt, Nx))
    p = rng.standard_normal((Nt, Nx)) + 0j
    return dict(phi=phi, psi=psi, b=b, p=p)


def run_case(name, spec, workdir):
    d = os.path.join(workdir, name)
    os.makedirs(d, exist_ok=True)
    inp = make_inputs(spec)
    for k, v in inp.items():
        np.ascontiguousarray(v, dtype=np.complex128).tofile(os.path.join(d, k + ".bin"))
    lat = spec["lattice"]
    lines = ["lattice " + " ".join(str(x) for x in lat), f"Nt {spec['Nt']}", f"beta {spec['beta']!r}",
             f"mu {spec['mu']!r}", f"U {spec['U']!r}", f"nrhs {spec['nrhs']}"]
    if spec["logdet"]:
        lines.append("logdet 1")
    if spec["cg"]:
        lines += [f"cg_eps {spec['cg'][0]!r}", f"cg_maxiter {spec['cg'][1]}"]
    if spec["lf"]:
        lines += [f"nmd {spec['lf'][0]}", f"traj {spec['lf'][1]!r}"]
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    subprocess.run([HARNESS, d], check=True)

    Nt, Nx, R = spec["Nt"], nsites(lat), spec["nrhs"]
    out = dict(inp)
    out["params"] = np.array([Nt, Nx, R, spec["beta"], spec["mu"], spec["U"]], dtype=np.float64)
    out["lattice"] = np.array(" ".join(str(x) for x in lat))

    def rd(fn, shape):
        return np.fromfile(os.path.join(d, fn), dtype=np.complex128).reshape(shape)

    out["hops"] = rd("hops.bin", (Nx, Nx))
    out["expK_pos"] = rd("expK_pos.bin", (Nx, Nx))
    out["expK_neg"] = rd("expK_neg.bin", (Nx, Nx))
    for s in "PH":
        for op in ("M", "Mdag", "MMdag", "MdagM"):
            out[f"{op}_{s}"] = rd(f"{op}_{s}.bin", (R, Nt, Nx))
        if spec["logdet"]:
            out[f"logdet_{s}"] = rd(f"logdet_{s}.bin", (1,))[0]
            out[f"grad_{s}"] = rd(f"grad_{s}.bin", (Nt, Nx))
        # HubbardDiag (the diagonal discretisation) on the same inputs
        for op in ("M", "Mdag", "MMdag", "MdagM"):
            out[f"diag_{op}_{s}"] = rd(f"diag_{op}_{s}.bin", (R, Nt, Nx))
        if spec["logdet"]:
            out[f"diag_logdet_{s}"] = rd(f"diag_logdet_{s}.bin", (1,))[0]
            out[f"diag_grad_{s}"] = rd(f"diag_grad_{s}.bin", (Nt, Nx))
    if spec["cg"]:
        out["cg_eps"] = np.float64(spec["cg"][0])
        out["cg_x"] = rd("cg_x.bin", (R, Nt, Nx))
        with open(os.path.join(d, "cg_iters.txt")) as f:
            out["cg_iters"] = np.int64(int(f.readline().strip()))
    if spec["lf"]:
        out["nmd"] = np.int64(spec["lf"][0])
        out["traj"] = np.float64(spec["lf"][1])
        for k in ("S", "S_gauge", "S_fermion", "lf_S", "lfr_S"):
            out[k] = rd(k + ".bin", (1,))[0]
        for k in ("force", "force_fermion", "lf_q", "lf_p", "lfr_q", "lfr_p"):
            out[k] = rd(k + ".bin", (Nt, Nx))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: Nx={Nx} Nt={Nt} R={R}" + (f" cg_iters={int(out['cg_iters'])}" if spec["cg"] else ""))


def main(argv):
    if not os.path.exists(HARNESS):
        sys.exit(f"build the harness first: make -C oracle/ref_harness ({HARNESS} missing)")
    names = argv[1:] or list(CASES) + list(TWOBODY_CASES) + list(TWOPOINT_CASES)
    with tempfile.TemporaryDirectory() as work:
        for name in names:
            if name in TWOBODY_CASES:
                run_twobody_case(name, TWOBODY_CASES[name], work)
            elif name in TWOPOINT_CASES:
                run_twopoint_case(name, TWOPOINT_CASES[name], work)
            else:
                run_case(name, CASES[name], work)


if __name__ == "__main__":
    main(sys.argv)
