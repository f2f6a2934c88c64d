"""Benchmark: batched MM^dagger CG solves per second on one GB300 (N independent replicas under torchrun).

Workload (the plain-FP64 drop-in configuration): periodic honeycomb 12x12 (Nx=288), Nt=64, beta=8, U=3, mu=0; a real
auxiliary field phi ~ N(0, delta*U) from a fixed seed and 64 complex Gaussian right-hand sides. A step solves
MM^dagger x = b for all 64 right-hand sides (independent systems) to a relative true residual
|b - MM^dagger x| / |b| <= 1e-10 with the mixed-precision solver: FP64 vectors, the operator on the tensor cores
(split-BF16 digits with exact accumulation by default), FP64 reliable updates, and the double-double rule
(nslg_cg_solve_dd): at this temperature |A| |x| / |b| reaches 1e7..1e8, so an FP64 x cannot hold a 1e-10 residual
(its own rounding moves b - A x by 1e-9..1e-8 |b|); the solution is kept as a double-double pair x + x_lo and its
residual is certified in double-double arithmetic. The plain-FP64 GPU arm runs the same rule with the FP64 operator.

Every timed step is preceded by an L2 flush (a 256 MB device write on the solver's stream, outside the step's CUDA
events); within a step the solver's ~110-140 MB working set is re-read every iteration, as in any CG.

JSON line (rank 0): value = solves/s with inputs resident in HBM; e2e = the same through the public API from pinned
host buffers (H2D of b and D2H of x and x_lo inside the timed region); fp64_gpu = the plain-FP64 GPU path (FP64
operator, same rule) on the same solve; roofline = the dominant kernel (the operator application at the solver's
precision), timed live with CUDA events on the library's stream; cpu_baseline = whole certified CG solves of single
right-hand sides on the host cores (the oracle's restatement of the reference CG iteration with the same reliable
updates and double-double rebases, one right-hand side per worker process); hmc = leapfrog trajectories per second;
serving = p50/p99 latency of a Poisson stream of mixed-size correlator requests; precision_config = the honeycomb
24x24, Nt=128, beta=12 configuration.

--impl reference times the same certified CPU solves on all host cores (the oracle port: the reference's own CG stops
on its recurrence residual, whose true residual is 3.4e-7 here, and the reference C++ library needs libtorch C++
headers and its source checkout, which the GPU host does not have).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L, NT, BETA, U, NRHS, TOL, SEED = (12, 12), 64, 8.0, 3.0, 64, 1e-10, 2026
MAX_ITER = 400000
METRIC = "MMdag CG solves/s (mixed precision, 1e-10 true residual)"
UNIT = "solves/s"
FP64_NOMINAL_TFLOPS = 1.25  # GB300 nominal FP64 (non-tensor) rate
# DRAM bytes (read + write) of one M application on the 64 right-hand sides, from one ncu capture (cold caches) of the
# split-BF16 digit pre-pass (19.2 MB) and tensor-core kernel (48.4 MB) at honeycomb 12x12, Nt = 64, 64 right-hand sides
TRAFFIC_PER_APPLY = {"bf16split": 67.6e6}
SPLIT_DIGIT_PAIRS = 21  # digit products per 16-site step of the split-BF16 operator (6 digits, orders d < 6)


T_START = time.perf_counter()


def log(msg):
    print(f"[bench {time.perf_counter() - T_START:7.1f} s] {msg}", file=sys.stderr, flush=True)


def workload():
    from nsl_gb300.lattice import Honeycomb

    lat = Honeycomb(L)
    Nx = lat.sites()
    rng = np.random.default_rng(SEED)
    phi = rng.standard_normal((NT, Nx)) * np.sqrt(BETA / NT * U) + 0j
    b = rng.standard_normal((NRHS, NT, Nx)) + 1j * rng.standard_normal((NRHS, NT, Nx))
    return lat, phi, b


def config(precision):
    """The workload of every arm (the same dict in the reference arm's line)."""
    return {"workload": f"honeycomb {L[0]}x{L[1]} (Nx=288), Nt={NT}, beta={BETA}, U={U}, {NRHS} Gaussian RHS, "
                        f"MMdag CG to {TOL:g} relative true residual (double-double certified)",
            "Nx": 288, "Nt": NT, "beta": BETA, "U": U, "nrhs": NRHS, "tolerance": TOL, "cg_mode": "per_rhs",
            "stop_rule": "true_residual_dd",
            "cfg3_note": "the honeycomb 24x24, Nt=128, beta=12 configuration is measured in precision_config (per "
                         "iteration, gradient, log det and a full certified solve of a few right-hand sides); the "
                         "timed step stays on 12x12 because full 64-RHS solves at beta=12 do not fit the driver's steps",
            "l2": "flushed before every timed step (a 256 MB device write on the solver's stream, outside the "
                  "step's events); within a step the solver's ~110-140 MB working set is re-read every iteration"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) >= 7:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [v for v in (num(s[0]) for s in self.samples) if v is not None]
        mx = [v for v in (num(s[1]) for s in self.samples) if v is not None]
        pw = [v for v in (num(s[2]) for s in self.samples) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_median": statistics.median(pw) if pw else None, "reasons": reasons,
                "samples": len(self.samples)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def _cpu_solve(args):
    """One whole certified CG solve of right-hand side i on the host (worker process): the oracle's restatement of the
    reference CG iteration (CG.tpp:15-95, FP64, the reference's 4-product MM^dagger) with FP64 reliable updates and
    double-double rebases, to the bench tolerance."""
    K, phi, b_i, eps = args
    from oracle import nsl_oracle as O

    h = O.HubbardExp(K, NT, BETA)
    h.populate(phi)
    t0 = time.perf_counter()
    xh, xl, it, rebases, res = O.cg_certified(h, "MMdagger", b_i, eps, MAX_ITER)
    return {"seconds": time.perf_counter() - t0, "iterations": it, "rebases": rebases,
            "true_residual": res / float(np.linalg.norm(b_i))}


class CpuSolver:
    """A pool of single-threaded worker processes (spawned, so no CUDA state is inherited), one right-hand side each."""

    def __init__(self, workers=None):
        import multiprocessing as mp

        self.workers = workers or os.cpu_count() or 1
        for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
            os.environ[v] = "1"  # inherited by the spawned workers: one core each
        self.pool = mp.get_context("spawn").Pool(self.workers)

    def solve(self, lat, phi, b, eps, rhs):
        """Solves the right-hand sides `rhs` concurrently; returns (wall seconds, per-solve records)."""
        K = lat.hopping_matrix()
        t0 = time.perf_counter()
        recs = self.pool.map(_cpu_solve, [(K, phi, b[i], eps) for i in rhs], chunksize=1)
        return time.perf_counter() - t0, recs

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_record(wall, recs, workers, what):
    return {"value": len(recs) / wall, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{what}: {len(recs)} whole solves of single right-hand sides, {workers} single-threaded "
                      f"worker processes, {wall:.1f} s wall; iterations {min(r['iterations'] for r in recs)}.."
                      f"{max(r['iterations'] for r in recs)}, double-double rebases "
                      f"{max(r['rebases'] for r in recs)}, true residual <= "
                      f"{max(r['true_residual'] for r in recs):.2e}"}


def cpu_baseline(lat, phi, b, eps):
    """One round of certified CPU solves, one right-hand side per host core (bounded: each solve is a few tens of
    seconds of one core)."""
    solver = CpuSolver()
    try:
        wall, recs = solver.solve(lat, phi, b, eps, list(range(min(solver.workers, NRHS))))
    finally:
        solver.close()
    return cpu_record(wall, recs, solver.workers, "oracle certified CG (reference iteration, FP64 reliable updates, "
                                                  "double-double rebases)")


def run_reference(args, rank, world):
    """The reference arm: W warm-up and K timed certified solves (one right-hand side per step, the steps spread over
    all host cores) on the bench workload; value = K / wall time of the timed solves."""
    if rank != 0:
        return
    lat, phi, b = workload()
    eps = TOL * float(np.linalg.norm(b.reshape(NRHS, -1), axis=1).min())
    solver = CpuSolver()
    try:
        solver.solve(lat, phi, b, eps, [i % NRHS for i in range(args.warmup)])
        wall, recs = solver.solve(lat, phi, b, eps, [i % NRHS for i in range(args.warmup, args.warmup + args.steps)])
    finally:
        solver.close()
    cb = cpu_record(wall, recs, solver.workers, "oracle certified CG (reference iteration, FP64 reliable updates, "
                                                "double-double rebases), the timed steps")
    value = cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64) + double-double",
            "data": "synthetic (seeded)", "config": config(args.precision), "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_operator(hfm, psi, precision, stream, reps=50):
    """Average duration of one M application on device buffers (asynchronous calls, back to back on the library's
    stream, CUDA events on that stream): the row-scale/digit pre-pass plus the tensor-core kernel."""
    import torch

    out = torch.empty_like(psi)
    for _ in range(3):
        hfm.M(psi, precision=precision)
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for _ in range(reps):
        out = hfm.M(psi, precision=precision)
    k1.record(stream)
    torch.cuda.synchronize()
    return k0.elapsed_time(k1) * 1e-3 / reps


def time_dd_apply(hfm, xh, xl, stream, reps=5):
    """Average duration of one double-double MM^dagger application (the residual of a rebase) on device buffers."""
    import torch

    from nsl_gb300 import _lib

    lib = _lib.load()
    oh, ol = torch.empty_like(xh), torch.empty_like(xh)
    nb = xh.shape[0]

    def once():
        from nsl_gb300 import tensor as T

        with T.stream_order(hfm.ctx, xh, xl, oh, ol):
            _lib.check(lib.nslg_fm_apply_dd(hfm.handle, _lib.OP_MMDAGGER, T.ptr(xh), T.ptr(xl), T.ptr(oh), T.ptr(ol),
                                            nb))

    once()
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for _ in range(reps):
        once()
    k1.record(stream)
    torch.cuda.synchronize()
    return k0.elapsed_time(k1) / reps


def hmc_rate(ctx, stream):
    """Leapfrog trajectories per second: honeycomb 3x3, Nt=16, beta=4, U=2, Nmd=10 (the CPU-runnable HMC
    configuration) and one trajectory of the 12x12 configuration (Nmd=20)."""
    import torch

    import nsl_gb300 as N
    from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
    from nsl_gb300.integrator import LeapfrogRealForce

    out = {}
    for name, Lc, Nt, beta, Uc, nmd, reps in (("honeycomb3x3_Nt16_beta4_Nmd10", (3, 3), 16, 4.0, 2.0, 10, 10),
                                              ("honeycomb12x12_Nt64_beta8_Nmd20", (12, 12), 64, 8.0, 3.0, 20, 3)):
        lat = N.Honeycomb(Lc)
        p = {"Nt": Nt, "beta": beta, "mu": 0.0, "U": Uc}
        rng = np.random.default_rng(7)
        q = {"phi": rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * Uc) + 0j}
        pm = {"phi": rng.standard_normal((Nt, lat.sites())) + 0j}
        rec = {"dtype": "f64 action (Delta H) both ways; force f64 (traj_per_s: the stratified form at beta = 8 on "
                        "12x12, beta rho = 24 > 14) or split-BF16 direct product (traj_per_s_bf16split_force; lattices "
                        "of at most 32 sites take the FP64 force at either setting)"}
        forces = {}
        for fp in ("fp64", "bf16split"):
            S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p, ctx=ctx, force_precision=fp)
            lf = LeapfrogRealForce(S, 1.0, nmd)
            lf(q, pm)  # eager run (builds the workspaces), then the captured trajectory
            lf(q, pm)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                lf(q, pm)
            torch.cuda.synchronize()
            rec["traj_per_s" if fp == "fp64" else "traj_per_s_bf16split_force"] = reps / (time.perf_counter() - t0)
            forces[fp] = np.asarray(S.force(q)["phi"])
        rec["force_rel_err_bf16split_vs_fp64"] = float(np.abs(forces["bf16split"] - forces["fp64"]).max() /
                                                       np.abs(forces["fp64"]).max())
        rec["cpu_port_traj_per_s"] = cpu_trajectory_rate(lat, Nt, beta, Uc, nmd, q["phi"], pm["phi"])
        out[name] = rec
    # many independent chains of the small configuration in one batched trajectory (FP64 force)
    for name, Lc, Nt, beta, Uc, nmd, nconf, reps in (
            ("honeycomb3x3_Nt16_beta4_Nmd10_chains256", (3, 3), 16, 4.0, 2.0, 10, 256, 5),
            ("honeycomb6x6_Nt32_beta4_Nmd10_chains32", (6, 6), 32, 4.0, 2.0, 10, 32, 3)):
        lat = N.Honeycomb(Lc)
        p = {"Nt": Nt, "beta": beta, "mu": 0.0, "U": Uc}
        rng = np.random.default_rng(8)
        q = {"phi": rng.standard_normal((nconf, Nt, lat.sites())) * np.sqrt(beta / Nt * Uc) + 0j}
        pm = {"phi": rng.standard_normal((nconf, Nt, lat.sites())) + 0j}
        S = HubbardGaugeAction(p) + HubbardFermionAction(lat, p, ctx=ctx)
        lf = LeapfrogRealForce(S, 1.0, nmd)
        lf(q, pm)
        lf(q, pm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            lf(q, pm)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / reps
        out[name] = {"dtype": "f64", "chains": nconf, "traj_per_s": nconf / dt, "seconds_per_batched_trajectory": dt,
                     "note": "all chains advance in one batched trajectory (nslg_leapfrog_batch); traj_per_s counts "
                             "trajectories of all chains"}
    out["chain_mix_256"] = chain_mix_rate(ctx)
    return out


# 256 chains of uneven size: (graph, sites parameter, Nt, chains). Honeycomb L x L has Nx = 2 L^2 (18, 50, 72, 128,
# 288), Ring(n) has Nx = n; beta = 4 for every group, U ~ U[1, 4] per chain. More chains on the cheap lattices:
# the FP64 force of one chain costs ~32 Nt Nx^3 flops.
CHAIN_MIX = (("honeycomb", 3, 16, 32), ("honeycomb", 3, 32, 32), ("honeycomb", 3, 64, 24), ("honeycomb", 3, 128, 16),
             ("ring", 18, 64, 16), ("honeycomb", 5, 16, 24), ("honeycomb", 5, 32, 16), ("honeycomb", 5, 64, 12),
             ("ring", 50, 32, 16), ("honeycomb", 6, 16, 16), ("honeycomb", 6, 32, 12), ("honeycomb", 6, 64, 8),
             ("honeycomb", 8, 16, 12), ("honeycomb", 8, 32, 8), ("ring", 128, 16, 8), ("honeycomb", 12, 16, 4))


def chain_mix_rate(ctx, nmd=10, reps=3):
    """HMC on 256 chains of uneven size (CHAIN_MIX: Nx in {18, 50, 72, 128, 288}, Nt in {16, 32, 64, 128},
    honeycomb and ring graphs, U ~ U[1, 4] per chain, LeapfrogRealForce with Nmd = 10 over length 1): every chain's
    trajectory in one nslg_leapfrog_group call (one CUDA-graph launch with one branch per lattice shape), then the
    per-group batched action, kinetic sums and accept step. Reports trajectories per second over all chains for the
    trajectory launch alone and for whole HMC steps, the groups' total graph kernels, and the acceptance rate."""
    import torch

    import nsl_gb300 as N
    from nsl_gb300.hmc import ChainEnsemble

    rng = np.random.default_rng(SEED + 9)
    groups, phis = [], []
    for kind, L, Nt, n in CHAIN_MIX:
        lat = N.Honeycomb((L, L)) if kind == "honeycomb" else N.Ring(L)
        U = rng.uniform(1.0, 4.0, n)
        beta = 4.0
        groups.append({"lattice": lat, "Nt": Nt, "beta": beta, "U": U})
        phi = rng.standard_normal((n, Nt, lat.sites())) * np.sqrt(beta / Nt * U)[:, None, None] + 0j
        phis.append(torch.from_numpy(phi).cuda())
    ens = ChainEnsemble(groups, 1.0, nmd, seed=SEED + 10, real_force=True, ctx=ctx)
    nchains = sum(ens.nconf)
    p = ens.momenta(phis)
    for _ in range(2):  # eager, then each group captured
        ens.leapfrog(phis, p)
    launches0 = N._lib.load().nslg_kernel_launches()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        ens.leapfrog(phis, p)
    torch.cuda.synchronize()
    t_traj = (time.perf_counter() - t0) / reps
    kernels = (N._lib.load().nslg_kernel_launches() - launches0) // reps
    ens.generate(phis, 1)  # warm the per-group action and selection paths
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, rates = ens.generate(phis, reps)
    torch.cuda.synchronize()
    t_step = (time.perf_counter() - t0) / reps
    return {"chains": nchains, "groups": len(groups),
            "shapes": [f"{k}{L}:Nx={g['lattice'].sites()},Nt={Nt},chains={n}" for (k, L, Nt, n), g in
                       zip(CHAIN_MIX, groups)],
            "traj_per_s_trajectory_launch": nchains / t_traj, "seconds_per_group_launch": t_traj,
            "traj_per_s_hmc_step": nchains / t_step, "seconds_per_hmc_step": t_step,
            "kernels_per_group_launch": int(kernels),
            "acceptance": float(np.mean(np.concatenate(rates))), "dtype": "f64 force, f64 action and Delta H",
            "note": "one nslg_leapfrog_group call per HMC step: a CUDA graph whose branches are the 16 shape groups' "
                    "batched trajectories; actions, kinetic sums and accept per group"}


def cpu_trajectory_rate(lat, Nt, beta, Uc, nmd, q, p, seconds=6.0):
    """The oracle's LeapfrogRealForce trajectory (numpy FP64, reference algorithm) on the host cores: whole
    trajectories when they fit in `seconds`, else the force evaluations timed and scaled to the Nmd + 1 a
    trajectory needs."""
    from oracle import nsl_oracle as O

    S = O.HubbardAction(lat.hopping_matrix(), Nt, beta, Uc)
    t0 = time.perf_counter()
    S.force(q)
    t_force = time.perf_counter() - t0
    if t_force * (nmd + 1) < seconds / 2:
        n = 0
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds or n < 1:
            O.leapfrog(S, q, p, 1.0, nmd, real_force=True)
            n += 1
        return n / (time.perf_counter() - t0)
    return 1.0 / (t_force * (nmd + 1))


# The serving mix spans the correlator configuration's range: honeycomb Nx = 18 .. 1152, Nt = 16 .. 256 with
# delta = beta / Nt = 1/16, U drawn from [1, 4] per request
SERVING_SHAPES = (((3, 3), 16), ((3, 3), 256), ((5, 5), 32), ((6, 6), 64), ((8, 8), 32), ((12, 12), 16),
                  ((12, 12), 64), ((24, 24), 16))
SERVING_MAX_ITER = 50000


def serving_load(n_requests=24, rate_hz=6.0, slots=2):
    """Correlator serving under a Poisson stream of mixed-size requests (honeycomb Nx = 18..1152, Nt = 16..256,
    beta = min(Nt/16, 8), U ~ U[1, 4], one source time: Nx point-source solves each, split-BF16 mixed CG to 1e-10 certified in
    double-double): p50/p99 latency from submission to completion, point-source solves per second over the stream, the
    batches the grouped solver formed, and the requests whose field puts a near-zero mode into M (not converged in
    SERVING_MAX_ITER iterations, reported)."""
    import nsl_gb300 as N
    from nsl_gb300.serving import CorrelatorRequest, CorrelatorServer, latency_summary

    rng = np.random.default_rng(SEED + 5)
    lats = {L: N.Honeycomb(L) for L, _ in SERVING_SHAPES}

    def request(k, U=None):
        L, Nt = SERVING_SHAPES[k % len(SERVING_SHAPES)]
        lat, beta = lats[L], min(Nt / 16.0, 8.0)
        Uc = rng.uniform(1.0, 4.0) if U is None else U
        phi = rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * Uc) + 0j
        return CorrelatorRequest(lat, Nt, beta, phi, n_time_sources=1, tag=(L, Nt, Uc))

    srv = CorrelatorServer(slots=slots, hbm_budget_bytes=96 << 30, precision="bf16split", eps=1e-10,
                           max_iter=SERVING_MAX_ITER, stop="true_residual_dd")
    warm = [srv.submit(request(k, U=1.0)) for k in range(slots * len(SERVING_SHAPES))]  # resident data per worker
    for r in warm:
        r.done.wait(1200)
    srv.batches.clear()
    order = rng.permutation(n_requests)
    reqs = []
    t0 = time.perf_counter()
    for k in order:
        time.sleep(rng.exponential(1.0 / rate_hz))
        reqs.append(srv.submit(request(int(k))))
    for r in reqs:
        r.done.wait(1200)
    t1 = time.perf_counter()
    batches = list(srv.batches)
    srv.close()
    errors = [r.error for r in reqs if r.error]
    summary = latency_summary(reqs)
    done = [r for r in reqs if r.error is None]
    rhs = sum(r.lattice.sites() * r.n_time_sources for r in done)
    unconverged = [{"Nx": r.lattice.sites(), "Nt": r.Nt, "U": round(r.tag[2], 3), "converged": r.stats["converged"],
                    "systems": r.stats["systems"]} for r in done if r.stats["converged"] != r.stats["systems"]]
    by_shape = {}
    for r in done:
        by_shape.setdefault(f"Nx{r.lattice.sites()}_Nt{r.Nt}", []).append(r)
    summary["by_shape"] = {k: {"requests": len(v), "p50_s": float(np.percentile([r.latency for r in v], 50)),
                               "iterations_max": max(int(r.stats.get("iterations", 0)) for r in v)}
                           for k, v in sorted(by_shape.items())}
    summary.update({"requests": n_requests, "arrival_rate_hz": rate_hz, "slots": slots,
                    "point_source_solves_per_s": rhs / (t1 - t0), "errors": len(errors),
                    "requests_converged": len(done) - len(unconverged), "not_converged": unconverged,
                    "batches": len(batches), "requests_per_batch_max": max(batches) if batches else 0,
                    "requests_per_batch_mean": float(np.mean(batches)) if batches else 0.0,
                    "max_iter": SERVING_MAX_ITER, "rule": "1e-10 per point source, double-double certified",
                    "mix": "honeycomb L in {3,5,6,8,12,24} (Nx 18..1152), Nt in {16,32,64,256}, beta = min(Nt/16, 8), "
                           "U ~ U[1,4], 1 source time"})
    return summary


def twobody_rate(ctx):
    """Two-body correlators from momentum wall sources (TwoBodyCorrelator::measure(NumberTimeSources)) on one
    configuration: every lattice momentum with both sublattice bands as wall sources, all channels for every
    momentum-conserving tuple. Seconds per configuration on the GPU for the FP64 and split-BF16 solvers (the
    result stays on the device), and the oracle (numpy, exact dense inverse in place of the solves) for one source
    time on the host, scaled to the source-time count, where it is small enough to run."""
    import torch

    import nsl_gb300 as N
    from nsl_gb300.measurement import TwoBodyCorrelator, honeycomb_wall_sources

    out = {}
    cases = (("honeycomb3x3_Nt16_beta4_all_momenta_16src", (3, 3), 16, 4.0, 2.0, 16, True),
             ("honeycomb6x6_Nt32_beta4_all_momenta_4src", (6, 6), 32, 4.0, 2.0, 4, False))
    for name, Lc, Nt, beta, Uc, nts, cpu in cases:
        lat = N.Honeycomb(Lc)
        mom, W = honeycomb_wall_sources(lat)
        rng = np.random.default_rng(SEED + 9)
        phi = rng.standard_normal((Nt, lat.sites())) * np.sqrt(beta / Nt * Uc) + 0j
        phi_d = torch.from_numpy(phi).cuda()
        params = {"Nt": Nt, "beta": beta, "mu": 0.0, "wallSources": W, "momenta": mom}
        rec = {"momenta": len(mom), "bands": 2, "time_sources": nts}
        for prec in ("fp64", "bf16split"):
            tb = TwoBodyCorrelator(lat, params, eps=1e-11, maxIter=20000, precision=prec, ctx=ctx)
            res = tb.measure_array(phi_d, nts)  # warm-up: workspaces, exp(delta K), planes
            torch.cuda.synchronize()
            reps = 3
            t0 = time.perf_counter()
            for _ in range(reps):
                res = tb.measure_array(phi_d, nts)
            torch.cuda.synchronize()
            rec[f"seconds_{prec}"] = (time.perf_counter() - t0) / reps
            rec[f"converged_{prec}"] = f"{tb.stats['converged']}/{tb.stats['systems']}"
            rec["tuples"] = len(tb.tuples)
            rec["solves_per_configuration"] = int(tb.stats["systems"])
            if prec == "fp64":
                ref = res
            else:
                rec["rel_diff_bf16split_vs_fp64"] = float((res - ref).abs().max() / ref.abs().max())
            del res
        if cpu:
            from oracle import nsl_oracle as O

            h = O.HubbardExp(lat.hopping_matrix(), Nt, beta)
            t0 = time.perf_counter()
            O.two_body_correlator(h, phi, W, tb.tuples, 1)  # one source time (tsrc = 0)
            rec["cpu_port_seconds"] = (time.perf_counter() - t0) * nts
            rec["cpu_port_note"] = ("oracle (numpy FP64, dense inverse per species in place of the solves), one source "
                                    "time timed on the host and scaled to the source-time count")
        out[name] = rec
        torch.cuda.empty_cache()
    return out


def precision_config(ctx, stream, nrhs=8, cg_iters=64, solve_rhs=2, fp64_solve=False):
    """The honeycomb 24x24 (Nx = 1152), Nt = 128, beta = 12, U = 3 configuration. The field is the one of the oracle's
    stratified fixture (tests/golden/stable_cfg3.npz, seed 12), so the errors of log det and its gradient are measured
    against the oracle's stratified forms (QR-stratified products, pinned to dense inverses of M on smaller
    lattices). Reported: the split-BF16 operator's error and time against FP64; CG time per iteration in both forms;
    log det M and gradLogDetM in the stratified FP64 form (the default at this temperature) and in the reference's
    direct-product form, each with its error; a full certified solve (double-double rule, 1e-10) of `solve_rhs`
    right-hand sides with the split-BF16 operator, and with fp64_solve (bench.py --cfg3-fp64-solve, ~10 minutes) the
    same solve with the FP64 operator."""
    import torch

    import nsl_gb300 as N

    z = np.load(os.path.join(ROOT, "tests", "golden", "stable_cfg3.npz"))
    Lc, Nt, beta, Uc = (24, 24), 128, 12.0, 3.0
    lat = N.Honeycomb(Lc)
    Nx = lat.sites()
    phi = z["phi"]
    sl = z["slices"]
    rng = np.random.default_rng(SEED + 7)
    h = N.HubbardExp(lat, Nt, beta, ctx=ctx)
    h.populate(phi)
    psi = torch.from_numpy(rng.standard_normal((nrhs, Nt, Nx)) + 1j * rng.standard_normal((nrhs, Nt, Nx))).cuda()
    out = {"workload": f"honeycomb 24x24 (Nx={Nx}), Nt={Nt}, beta={beta}, U={Uc}, phi of the oracle fixture "
                       f"(seed 12), {nrhs} RHS for the operator and per-iteration timings"}

    def timed(f, reps=3):
        f()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            r = f()
        torch.cuda.synchronize()
        return r, (time.perf_counter() - t0) / reps

    y64, t64 = timed(lambda: h.M(psi, precision="fp64"))
    ysp, tsp = timed(lambda: h.M(psi, precision="bf16split"))
    out["operator_M"] = {"fp64_ms": t64 * 1e3, "bf16split_ms": tsp * 1e3,
                         "bf16split_rel_err": float((ysp - y64).abs().max() / y64.abs().max())}
    cg_rate = {}
    for prec in ("fp64", "bf16split"):
        cg = N.CG(h, N.MatrixCombination.MMdagger, 1e-300, cg_iters, mode="per_rhs", precision=prec,
                  stop="true_residual")
        cg(psi)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cg(psi)
        torch.cuda.synchronize()
        cg_rate[prec] = (time.perf_counter() - t0) / max(cg.stats["iterations"], 1)
    out["cg_ms_per_iteration"] = {k: v * 1e3 for k, v in cg_rate.items()}
    out["cg_mixed_over_fp64_per_iteration"] = cg_rate["fp64"] / cg_rate["bf16split"]

    def mod2pi(v):
        return complex(v.real, (v.imag + np.pi) % (2 * np.pi) - np.pi)

    for mode in ("stratified", "plain"):
        h.set_stabilisation(mode)
        rec = {}
        for sp, tag in ((N.Species.Particle, "P"), (N.Species.Hole, "H")):
            h.populate(phi, sp)
            g, tg = timed(lambda: h.gradLogDetM(), reps=1)
            ld, tl = timed(lambda: h.logDetM(), reps=1)
            g = np.asarray(g)
            ref_g, ref_ld = z[f"grad_{tag}"], complex(z[f"logdet_{tag}"])
            rec[tag] = {"gradLogDetM_ms": tg * 1e3, "logDetM_ms": tl * 1e3, "logDetM": [ld.real, ld.imag],
                        "gradLogDetM_rel_err_vs_oracle": float(np.abs(g[sl] - ref_g).max() / np.abs(ref_g).max()),
                        "logDetM_rel_err_vs_oracle": abs(mod2pi(ld - ref_ld)) / abs(ref_ld)}
        out[f"logdet_grad_{mode}"] = rec
    h.set_stabilisation("auto")
    h.populate(phi, N.Species.Particle)
    out["logdet_grad_note"] = ("errors against the oracle's QR-stratified forms on time slices "
                               f"{[int(v) for v in sl]} (tests/golden/stable_cfg3.npz); 'plain' is the reference's "
                               "direct product of the 128 slices, 'stratified' the default at this temperature")

    # a full certified solve of a few right-hand sides
    b = torch.from_numpy(rng.standard_normal((solve_rhs, Nt, Nx)) + 1j * rng.standard_normal((solve_rhs, Nt, Nx)))
    b = b.cuda()
    eps = TOL * float(torch.linalg.vector_norm(b.reshape(solve_rhs, -1), dim=1).min())
    cg = N.CG(h, N.MatrixCombination.MMdagger, eps, MAX_ITER, mode="per_rhs", precision="bf16split",
              stop="true_residual_dd")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cg(b)
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    out["full_solve_bf16split"] = {"rhs": solve_rhs, "tolerance": TOL, "seconds": ts, **cg.stats}
    if fp64_solve:
        c64 = N.CG(h, N.MatrixCombination.MMdagger, eps, MAX_ITER, mode="per_rhs", precision="fp64",
                   stop="true_residual_dd")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c64(b)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        out["full_solve_fp64"] = {"rhs": solve_rhs, "tolerance": TOL, "seconds": t64, **c64.stats}
        out["full_solve_mixed_over_fp64"] = t64 / ts
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16split", choices=["bf16split", "tf32x3", "fp32", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the certified CPU solves (cpu_baseline)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain-FP64 comparison solve")
    ap.add_argument("--no-hmc", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the 24x24, Nt=128, beta=12 configuration")
    ap.add_argument("--cfg3-fp64-solve", action="store_true",
                    help="also run the full certified 24x24, Nt=128 solve with the FP64 operator (~10 minutes)")
    ap.add_argument("--no-twobody", action="store_true", help="skip the two-body correlator timing")
    ap.add_argument("--profile", action="store_true",
                    help="short fixed run for profilers: 2 operator applications per precision and 32 CG iterations")
    ap.add_argument("--profile-hmc", action="store_true",
                    help="short fixed run for profilers: the HMC force (both species) of the 12x12, Nt=64, beta=8 "
                         "configuration in FP64 and on the tensor cores, then three honeycomb 3x3 trajectories")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch

    import nsl_gb300 as N
    from nsl_gb300 import _lib
    from nsl_gb300.replicas import job_rate, max_over_ranks

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    lat, phi, b = workload()
    ctx = N.Context(local)
    stream = ctx.torch_stream()
    hfm = N.HubbardExp(lat, NT, BETA, ctx=ctx)
    hfm.populate(phi)
    bnorm = np.linalg.norm(b.reshape(NRHS, -1), axis=1)
    eps = TOL * float(bnorm.min())
    b_dev = torch.from_numpy(b).cuda()

    if args.profile_hmc:
        from nsl_gb300.action import HubbardFermionAction, HubbardGaugeAction
        from nsl_gb300.integrator import LeapfrogRealForce

        rng = np.random.default_rng(7)
        phi_h = rng.standard_normal((NT, lat.sites())) * np.sqrt(BETA / NT * U) + 0j
        pp = {"Nt": NT, "beta": BETA, "mu": 0.0, "U": U}
        for fp in ("fp64", "bf16split"):  # the HMC force (both species) of the 12x12 field
            HubbardFermionAction(lat, pp, ctx=ctx, force_precision=fp).force({"phi": phi_h})
        torch.cuda.synchronize()
        # one honeycomb 3x3, Nt=16, beta=4, Nmd=10 trajectory: eager, then captured and replayed
        lat3 = N.Honeycomb((3, 3))
        p3 = {"Nt": 16, "beta": 4.0, "mu": 0.0, "U": 2.0}
        q3 = {"phi": rng.standard_normal((16, 18)) * np.sqrt(0.25 * 2.0) + 0j}
        pm3 = {"phi": rng.standard_normal((16, 18)) + 0j}
        lf3 = LeapfrogRealForce(HubbardGaugeAction(p3) + HubbardFermionAction(lat3, p3, ctx=ctx), 1.0, 10)
        for _ in range(3):
            lf3(q3, pm3)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "done", "hmc_force": ["fp64", "bf16split"], "trajectory": "honeycomb3x3"}))
        return

    if args.profile:
        for prec in ("fp64", "fp32", "tf32x3", "bf16split"):
            for _ in range(2):
                hfm.M(b_dev, precision=prec)
        cgp = N.CG(hfm, N.MatrixCombination.MMdagger, eps, 32, mode="per_rhs", precision=args.precision,
                   stop="true_residual_dd")
        cgp(b_dev)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "done", "precision": args.precision}))
        return

    cg = N.CG(hfm, N.MatrixCombination.MMdagger, eps, MAX_ITER, mode="per_rhs", precision=args.precision,
              stop="true_residual_dd")
    for i in range(max(args.warmup, 3)):  # warm-up (also builds the operator planes and captures the CUDA graphs)
        t0 = time.perf_counter()
        x = cg(b_dev)
        log(f"warm-up {i}: {time.perf_counter() - t0:.2f} s, {cg.stats}")
    torch.cuda.synchronize()

    flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > the 126 MB L2

    def flush_l2():
        with torch.cuda.stream(stream):
            flush_buf.zero_()

    launches0 = _lib.load().nslg_kernel_launches()
    stats = []
    barrier()
    torch.cuda.synchronize()

    def timed_steps(fn, steps):
        """Seconds of `steps` calls of fn, each after an L2 flush: CUDA events on the solver's stream bracket each
        step (the flush before it is outside), summed."""
        marks = []
        for _ in range(steps):
            flush_l2()
            e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e_a.record(stream)
            fn()
            e_b.record(stream)
            marks.append((e_a, e_b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in marks) * 1e-3

    def step_dev():
        nonlocal x
        x = cg(b_dev)
        stats.append(dict(cg.stats))

    with ClockSampler(local) as clocks:
        t_local = timed_steps(step_dev, args.steps)
    barrier()
    launches = _lib.load().nslg_kernel_launches() - launches0
    t = max_over_ranks(t_local, dist, "cuda")
    value = world * NRHS * args.steps / t

    # end to end through the public API with pinned host buffers (H2D of b, D2H of x and x_lo inside the timed
    # region); fewer steps than the device-resident loop (each is a whole solve)
    e2e_steps = max(1, min(args.steps, 5))
    b_host = torch.from_numpy(b).pin_memory()
    barrier()
    torch.cuda.synchronize()
    e2e = job_rate(NRHS * e2e_steps, timed_steps(lambda: cg(b_host), e2e_steps), dist, "cuda")

    fp64 = None
    if not args.no_fp64:
        cg64 = N.CG(hfm, N.MatrixCombination.MMdagger, eps, MAX_ITER, mode="per_rhs", precision="fp64",
                    stop="true_residual_dd")
        log("FP64 comparison solve")
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush_l2()
        f0.record(stream)
        cg64(b_dev)
        f1.record(stream)
        torch.cuda.synchronize()
        t64 = f0.elapsed_time(f1) * 1e-3
        fp64 = {"value": NRHS / t64, "unit": UNIT, "seconds": t64, "iterations": cg64.stats["iterations"],
                "reliable_updates": cg64.stats["reliable_updates"], "dd_rebases": cg64.stats["dd_rebases"],
                "converged": cg64.stats["converged"], "true_residual_max": cg64.stats["true_residual"],
                "mixed_over_fp64": value / world / (NRHS / t64),
                "note": "same vectors, reliable updates and double-double rule, FP64 CUDA-core operator"}

    # the double-double residual of a rebase: MM^dagger on the 64 right-hand sides in double-double
    xl0 = torch.zeros_like(b_dev)
    dd_ms = time_dd_apply(hfm, b_dev, xl0, stream)

    # dominant kernel: the operator application at the solver's precision (M on the 64 right-hand sides)
    t_apply = time_operator(hfm, b_dev, args.precision, stream)
    t_apply64 = time_operator(hfm, b_dev, "fp64", stream, reps=10)
    Nx = lat.sites()
    # algorithmic: the complex (Nt*R, Nx) x real (Nx, Nx) product (exp(delta K) is real on the honeycomb lattice at
    # real beta): 4 real flops per term
    flops = 4.0 * NT * Nx * Nx * NRHS
    if fp64 is not None:
        fp64["operator_M_ms"] = t_apply64 * 1e3
        fp64["operator_M_tflops"] = flops / t_apply64 / 1e12
        fp64["operator_M_frac_of_fp64_nominal"] = flops / t_apply64 / 1e12 / FP64_NOMINAL_TFLOPS
    hbm, bf16, which = peaks()
    # split-BF16: 21 digit-pair BF16 products over the real and imaginary GEMM rows (2 Nt R rows, Nx x Nx)
    executed = {"bf16split": SPLIT_DIGIT_PAIRS * 2.0 * (2 * NT * NRHS) * Nx * Nx,
                "tf32x3": 3 * 2.0 * (2 * NT * NRHS) * Nx * Nx}.get(args.precision, flops)
    roofline = {"bound": "tensor", "achieved": flops / t_apply / 1e12, "peak": bf16, "unit": "TFLOP/s",
                "frac": flops / t_apply / 1e12 / bf16, "traffic": TRAFFIC_PER_APPLY.get(args.precision),
                "kernel": f"operator M on 64 RHS at precision {args.precision} (digit pre-pass + tensor-core kernel)",
                "launch_ms": t_apply * 1e3,
                "algorithmic_gflop_per_launch": flops / 1e9,
                "executed_tensor_tflops": executed / t_apply / 1e12,
                "executed_frac": executed / t_apply / 1e12 / bf16,
                "peak_source": f"{which} bf16 dense (MEASURED_PEAKS.json)",
                # the arithmetic the product replaces is FP64: the part's nominal FP64 rate, for scale
                "algorithmic_over_fp64_nominal": flops / t_apply / 1e12 / FP64_NOMINAL_TFLOPS}

    log("operator timing done; HMC")
    hmc = None if args.no_hmc else hmc_rate(ctx, stream)
    log("HMC done; serving load")
    serving = None if args.no_serving else serving_load()
    log("serving done; 24x24 precision configuration")
    precision = None if args.no_precision else precision_config(ctx, stream, fp64_solve=args.cfg3_fp64_solve)
    log("precision configuration done; two-body correlators")
    twobody = None if args.no_twobody else twobody_rate(ctx)
    log("two-body done; CPU baseline")
    cpu = None if args.no_cpu or rank != 0 else cpu_baseline(lat, phi, b, eps)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": f"c128 vectors, {args.precision} operator, f64 reliable updates, double-double rebases",
                "operator_precision": args.precision,
                "data": "synthetic (seeded)", "config": config(args.precision),
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(b.nbytes),
                        "d2h_bytes_per_step": int(2 * b.nbytes), "steps": e2e_steps},
                "gpu_launches": int(launches),
                "clocks": clocks.summary(),
                "roofline": roofline,
                "cpu_baseline": cpu,
                "fp64_gpu": fp64,
                "dd_residual_ms": dd_ms,
                "hmc": hmc,
                "serving": serving,
                "twobody": twobody,
                "precision_config": precision,
                "solver": {"iterations_max": max(s["iterations"] for s in stats),
                           "reliable_updates": stats[-1]["reliable_updates"], "dd_rebases": stats[-1]["dd_rebases"],
                           "escalated": stats[-1]["escalated"], "converged": stats[-1]["converged"],
                           "true_residual_max": stats[-1]["true_residual"],
                           "true_residual_rule": "double-double |b - A (x + x_lo)| / |b|, max over the 64 systems"}}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
