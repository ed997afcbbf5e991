#!/usr/bin/env python3
"""Throughput benchmark of the GB300 MD step engine.

Workload (default "lj1m"): 1,048,576 argon atoms on an FCC lattice of 64^3
cubic cells at reduced density 0.8442 in a periodic box (L = 366.0 A),
Maxwell-Boltzmann velocities at 94.4 K from a fixed seed with the momentum
zeroed, LJ cutoff 2.5 sigma, neighbour cells of 2.8 sigma (skin 0.3 sigma),
Gear 5th order with dt = 2 fs, precision form (FP32 pair arithmetic, FP64
Gear state and reductions).  One bench step is 100 MD steps, list rebuilds
included on the reference's schedule (cpu/cpumd/Host.cpp:289).  The state
(176 MB) plus the list (330 MB) exceed the 129 MB L2, so no L2 flush is
needed between steps.

The JSON line also carries the plain FP64 GPU path on the same workload (the
speedup of the chosen form is measured against it), the force RMS error and
energy drift of the chosen form, the roofline of the LJ force kernel and the
CPU oracle timed on the host cores.

--impl reference times the reference's CPU implementation of the step on the
host cores (the compiled reference where it exists, else its C restatement
in oracle/, with all host threads) on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIGMA = 3.405
EPS_K = 119.8
KB = 8.314e-7
EPS = EPS_K * KB
MD_PER_BENCH_STEP = 100
METRIC = "atom-steps/s on 1 GB300, chosen form vs plain FP64 GPU, at stated drift/RMS error"

WORKLOADS = {
    # name: (fcc cells per edge, temperature K, precision)
    "lj1m": (64, 94.4, "mixed"),
    "lj864": (6, 94.4, "mixed"),
    "lj256k": (40, 94.4, "mixed"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max over ranks (gloo on the host; the data path has no
    collective: the ranks run independent replicas)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def make_workload(name: str, seed: int = 2024):
    from moleculardynamics_gb300 import lattice as lat
    ncell, temp, prec = WORKLOADS[name]
    pos, vel, L = lat.make_system("fcc", ncell, temp, seed=seed)
    return pos, vel, L, prec


def engine_for(eng, n, L, precision, device, output=MD_PER_BENCH_STEP, lj_kernel=0, threads=0,
               row_loads=0, stage_cap=0):
    cfg = eng.make_config(n_lj=n, dt=2.0, lj_rs=2.8 * SIGMA, lj_rcut=2.5 * SIGMA, periodic=1,
                          box=L, precision=precision, species=eng.SPECIES_ARGON, device=device,
                          output_timesteps=output, lj_kernel=lj_kernel, cluster_threads=threads,
                          cluster_row_loads=row_loads, cluster_stage_cap=stage_cap)
    return eng.Engine(cfg)


def drift_per_1000(recs: np.ndarray, n: int, first_step: int) -> float:
    """(E_end - E_start) / N / eps per 1000 MD steps, E = KE + shifted LJ energy."""
    sel = recs[recs[:, 15] >= first_step]
    if len(sel) < 2:
        return float("nan")
    e = sel[:, 3] + sel[:, 12]
    steps = sel[-1, 15] - sel[0, 15]
    return float((e[-1] - e[0]) / n / EPS / steps * 1000.0)


# FP64 operations per atom of the fused Gear update: correct 6 per component
# (a = F/m, the difference, four FMAs), predict 10 per component (4 + 3 + 2 + 1
# FMAs), and the compensated force widened with one subtraction per component.
# Each takes one FP64 pipe slot (a warp-wide FP64 instruction per 64 cycles per
# scheduler at GB300's measured rate), so n x 51 / (FMA rate) is the launch's
# FP64 floor.
GEAR_FP64_OPS_PER_ATOM = 3 * (6 + 10 + 1)


def fp32_roofline(entries: int, launch_s: float, arith: dict) -> dict:
    """FP32 arithmetic of one LJ force evaluation against the FP32 rate
    measured on this device (md_measure_arith_peaks: FMA chains on every SM):
    8 flops per row entry (3 differences, r^2 as a product and two FMAs) and
    15 per pair inside the cutoff (reciprocal, the r^-6 chain and force
    scalar, three FMAs into the sums), FMA = 2 flops; the pairs inside the
    cutoff are (2.5 / 2.8)^3 of the entries (uniform density)."""
    inside = entries * (2.5 / 2.8) ** 3
    flops = 8.0 * entries + 15.0 * inside
    achieved = flops / launch_s / 1e12
    peak = arith["fp32_gflops"] / 1e3
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": "measured (FMA chains on this device)",
            "flops_alg_per_launch": flops}


def fp64_lj_roofline(entries: int, launch_s: float, arith: dict) -> dict:
    """The plain FP64 LJ kernel (k_lj_fp64) against the FP64 rate measured
    on this device.  Operations of the reference's formula as the kernel
    evaluates it (no FMA contraction, for bit-exact parity;
    cpu/common/LennardJones.h:12-30): per row entry 3 differences, r^2 (3
    products, 2 sums) and the cutoff test = 8; per pair inside the cutoff
    a square root, 4 divisions, 10 products and sums and 3 FMA-free updates
    of the sums (6) = 21, each counted as one flop.  Divisions and square
    roots take many FP64 pipe slots each, so this count sits well below
    the pipe's occupancy."""
    inside = entries * (2.5 / 2.8) ** 3
    flops = 8.0 * entries + 21.0 * inside
    achieved = flops / launch_s / 1e12
    peak = arith["fp64_gflops"] / 1e3
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": "measured (FMA chains on this device)",
            "flops_alg_per_launch": flops,
            "divisions_and_sqrt_per_launch": 5.0 * inside}


# FP32 flops of the bond-order force evaluation (k_mb_short + k_mb_pass1 +
# k_mb_pass2), counted from the kernels' FP32 expressions with FMA = 2 and a
# reciprocal, square root, exponential or tanh = 1: per pair within the cutoff
# (attractive, repulsive and van der Waals terms, the pair cutoff, the bond
# order from xi, the force) 75; per pass-1 triplet (i, j, m), both sides of
# the angle term with their derivatives, 110; per pass-2 triplet (k, i, j)
# 130.  The FP64 instantiation evaluates the reference's own expressions
# (more operations, divisions in place of products); the same counts are used
# for it, so its fraction is a lower bound.
MB_FLOPS_PAIR, MB_FLOPS_TRIPLET1, MB_FLOPS_TRIPLET2 = 75.0, 110.0, 130.0


def bond_order_counts(pos: np.ndarray, L: float, rcut: float = 3.0) -> dict:
    """Pairs and triplets the bond-order passes evaluate at these positions:
    c_i neighbours of atom i within rcut (minimum image); pass 1 takes every
    pair (i, j) with every other m of i's neighbours, pass 2 every (k, i) with
    every other j of i's neighbours (an upper bound: it keeps only j in k's
    candidate row)."""
    from scipy.spatial import cKDTree
    x = np.mod(pos[:, :3] + 0.5 * L, L)
    tree = cKDTree(x, boxsize=L)
    c = np.array([len(v) - 1 for v in tree.query_ball_point(x, rcut)], dtype=np.float64)
    pairs = float(c.sum())
    trip = float((c * (c - 1)).sum())
    return {"pairs": pairs, "triplets_pass1": trip, "triplets_pass2": trip,
            "mean_neighbours": float(c.mean())}


def bond_order_roofline(counts: dict, launch_s: float, arith: dict, fp64: bool) -> dict:
    flops = (MB_FLOPS_PAIR * counts["pairs"] + MB_FLOPS_TRIPLET1 * counts["triplets_pass1"]
             + MB_FLOPS_TRIPLET2 * counts["triplets_pass2"])
    achieved = flops / launch_s / 1e12
    peak = (arith["fp64_gflops"] if fp64 else arith["fp32_gflops"]) / 1e3
    return {"kernel": "k_mb_short + k_mb_pass1 + k_mb_pass2" + ("<double>" if fp64 else "<float>"),
            "bound": "fp64" if fp64 else "fp32", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "measured (FMA chains on this device)",
            "flops_alg_per_launch": flops, "avg_launch_ms": launch_s * 1e3, "counts": counts}


def roofline_traffic(workload: str, kernel: str = "lj_force"):
    """dram bytes per launch of the LJ kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline(pos, vel, L, steps: int, threads: int):
    """The CPU oracle on a bounded sample of the same workload (host cores)."""
    from oracle.oracle import load_oracle, load_reference
    O = load_oracle()
    p = dict(n_lj=len(pos), n_mb=0, timesteps=steps, use_lj=1, use_mb=0, output_timesteps=0,
             dt=2.0, lj_rs=2.8 * SIGMA, lj_rcut=2.5 * SIGMA, mb_rs=3.5, mb_rcut=3.0,
             energy_loss=1.0, vxcm=0.0, periodic=1, box=L, species=1, threads=threads)
    r = O.run(p, pos, vel)
    kind = "port"
    return r["elapsed_ms"], kind


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    from moleculardynamics_gb300 import lattice as lat  # noqa: F401
    from oracle.oracle import build_oracle
    build_oracle()
    pos, vel, L, _ = make_workload(args.workload)
    n = len(pos)
    threads = os.cpu_count() or 1
    per = args.ref_md_steps
    # warm-up run (list build + W bench steps), then the timed run
    cpu_baseline(pos, vel, L, per * args.warmup, threads)
    ms, kind = cpu_baseline(pos, vel, L, per * args.steps, threads)
    value = n * per * args.steps / (ms / 1e3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "atom-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {n} argon atoms FCC, periodic, dt 2 fs",
                   "md_steps_per_bench_step": per, "form": "reference CPU path (FP64)"},
        "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": kind,
                         "sample": f"{n} atoms, {per * args.steps} MD steps after the list build, "
                                   f"{threads} OpenMP threads of the C restatement of the "
                                   "reference step (oracle/mdoracle.c)"},
        "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def batched_form(eng, device, steps: int, loop_steps: int, seed: int = 4096) -> dict:
    """The batched form on the 256-replica ensemble (sizes log-uniform on
    [256, 32000], T uniform on [60, 150] K): all replicas in one context, one
    persistent launch per MD step replayed from CUDA graphs.  Compared with
    looping the plain FP64 path, and the single-system precision path,
    replica by replica over the same replicas."""
    from moleculardynamics_gb300 import lattice as lat
    pos, vel, natoms, boxes, temps = lat.make_batch(256, 256, 32000, 60.0, 150.0, seed=seed)
    n = int(natoms.sum())
    cfg = eng.make_config(dt=2.0, lj_rs=2.8 * SIGMA, lj_rcut=2.5 * SIGMA, periodic=1,
                          precision=eng.PREC_MIXED, species=eng.SPECIES_ARGON, device=device)
    b = eng.Batch(cfg, natoms, boxes)
    b.upload(pos, vel)
    b.begin(0.0)
    b.step(200)  # thermalise before tuning the tiles
    tune = b.autotune(2)
    b.step(100)
    b.synchronize()
    r0 = b.replica_records()
    s0 = b.stats()
    b.set_timing(True)
    b.step(steps)
    b.synchronize()
    ms, _ = b.kernel_time(eng.KERNEL_STEP)
    fu_ms, fu_n = b.kernel_time(eng.KERNEL_FUSED)
    s1 = b.stats()
    b.set_timing(False)
    r1 = b.replica_records()
    value = n * steps / (ms / 1e3)
    e0 = r0[:, 3] + r0[:, 12]
    e1 = r1[:, 3] + r1[:, 12]
    drift = np.abs(e1 - e0) / natoms / EPS / steps * 1000.0
    # force error against the FP64 path, replica by replica (a sample)
    bp, bv = b.download()
    fb, _ = b.compute_forces()
    b.close()
    off = np.concatenate([[0], np.cumsum(natoms)])
    rms = []
    for k in np.linspace(0, len(natoms) - 1, 8).astype(int):
        p, v = bp[off[k]:off[k + 1]], bv[off[k]:off[k + 1]]
        e = engine_for(eng, len(p), float(boxes[k]), eng.PREC_FP64, device, output=0)
        e.upload(np.ascontiguousarray(p), np.ascontiguousarray(v))
        e.begin(0.0)
        fa, _ = e.compute_forces()
        e.close()
        fk = fb[off[k]:off[k + 1]]
        rms.append(float(np.sqrt(((fk - fa) ** 2).sum(1).mean()) / np.sqrt((fa ** 2).sum(1).mean())))

    def loop(precision):
        tot_ms = 0.0
        for k in range(len(natoms)):
            e = engine_for(eng, int(natoms[k]), float(boxes[k]), precision, device, output=0)
            e.upload(np.ascontiguousarray(pos[off[k]:off[k + 1]]),
                     np.ascontiguousarray(vel[off[k]:off[k + 1]]))
            e.begin(0.0)
            e.step(2)
            e.synchronize()
            e.set_timing(True)
            e.step(loop_steps)
            e.synchronize()
            tot_ms += e.kernel_time(eng.KERNEL_STEP)[0]
            e.close()
        return n * loop_steps / (tot_ms / 1e3)

    v64 = loop(eng.PREC_FP64)
    v32 = loop(eng.PREC_MIXED)
    return {
        "metric": "atom-steps/s of the whole ensemble on 1 GB300", "value": value,
        "unit": "atom-steps/s", "md_steps": steps,
        "config": {"replicas": len(natoms), "atoms": n, "sizes": [int(natoms.min()), int(natoms.max())],
                   "temperatures_K": [float(temps.min()), float(temps.max())],
                   "dt_fs": 2.0, "form": "precision pairs, FP64 Gear, one persistent launch "
                                         "per step, CUDA-graph windows of 6 steps",
                   "autotune": tune},
        "fused_kernel_ms": fu_ms / max(fu_n, 1),
        "list_builds": s1["list_builds"] - s0["list_builds"],
        "plain_fp64_loop": {"value": v64, "md_steps_per_replica": loop_steps},
        "precision_single_loop": {"value": v32, "md_steps_per_replica": loop_steps},
        "speedup_vs_plain_fp64_loop": value / v64,
        "speedup_vs_precision_loop": value / v32,
        "accuracy": {"force_rms_rel_vs_fp64_max": max(rms),
                     "energy_drift_eps_per_atom_per_1000_steps_max": float(drift.max()),
                     "energy_drift_eps_per_atom_per_1000_steps_mean": float(drift.mean())},
    }


# surrogate training data: temperatures of the exact trajectories and the MD
# steps at which they are sampled (denser early, where the lattice's first
# transient is); held-out states along a further trajectory
SUR_TEMPS = (300.0, 600.0, 900.0, 1200.0, 1500.0)
SUR_MARKS = (25, 50, 75, 100, 150, 200, 300, 400, 500, 700, 1000, 1500, 2000, 3000, 4000, 5000,
             6500, 8000, 10000)
SUR_HELDOUT = (5, 100, 400, 1000, 3000, 6000, 10000)
# learning-rate schedule (fraction of the Adam steps, rate) of each model kind
SUR_LR = {0: ((0.25, 2e-3), (0.25, 1e-3), (0.25, 3e-4), (0.25, 1e-4)),
          1: ((0.25, 1e-3), (0.25, 5e-4), (0.25, 2e-4), (0.25, 5e-5))}
# thresholds tried for the best accepted one (relative RMS force error)
SUR_LADDER = (1e-4, 3e-4, 1e-3, 3e-3, 1e-2, 0.02, 0.03, 0.05, 0.07, 0.1, 0.15, 0.2, 0.3, 0.5, 1.0)


def surrogate_form(eng, device, train_steps: int, run_steps: int, fp64_steps: int,
                   arith: dict, sweep: bool = False, seed: int = 5) -> dict:
    """The learned bond-order surrogate on the 32,768-atom nitrogen diamond
    (16^3 cells, nearest neighbour 1.5 A, 0.02 A noise).

    Training data: trajectories of the 32,768-atom system from 300, 600, 900,
    1200 and 1500 K, 10,000 steps each (the exact method in its precision
    form), sampled at the SUR_MARKS steps; at each sample the exact FP64
    bond-order forces are the labels: 95 snapshots = 3.1 M atomic
    environments.  Both model kinds are force-matched on them for
    `train_steps` Adam steps (one snapshot per step, four learning-rate stages):
      * the per-atom energy network 32-64-64-1 (BF16 tcgen05), forces from its
        gradient;
      * the direct-force head 32-H-H-32 (FP32), forces from its outputs.
    Their force error is taken at held-out states along a further 900 K
    trajectory.  With `sweep`, also the head at H = 32 and 128 and the head
    and the energy network on a quarter and a sixteenth of the snapshots:
    the error against model size and data.

    Then, with the model of the lower held-out error, NVE runs of the
    32,768-atom system from one 900 K state: the exact FP64 method
    (`fp64_steps`), the exact precision form and the surrogate at threshold
    1e-4 (`run_steps` each, exact-kernel check every 10 steps; the 1e-4 run
    reads the network's error at every check along what is then the exact
    trajectory), and the surrogate at the best accepted threshold: the
    smallest of SUR_LADDER that at least half of those checks pass.  Energy
    drift is that of kinetic + exact bond-order energy (the head has no
    energy of its own)."""
    from moleculardynamics_gb300 import lattice as lat
    a = 4 * 1.5 / np.sqrt(3.0)

    def system(T, sd, ncell=16):
        return lat.make_system("diamond", ncell, T, seed=sd, a=a, noise=0.02,
                               species=lat.SPECIES_N, mass_table="neon")

    def engine(pos, vel, L, precision=eng.PREC_FP64):
        cfg = eng.make_config(n_mb=len(pos), use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5,
                              periodic=1, box=L, species=eng.SPECIES_NEON, device=device,
                              precision=precision)
        e = eng.Engine(cfg)
        e.upload(pos, vel)
        e.begin(0.0)
        return e

    def rel(fa, fb):
        return float(np.sqrt(((fa - fb) ** 2).sum(1).mean() / (fb ** 2).sum(1).mean()))

    def states(T, sd, marks):
        pos, vel, L = system(T, sd)
        e = engine(pos, vel, L, eng.PREC_MIXED)
        out, done = [], 0
        for m in marks:
            e.step(m - done)
            done = m
            out.append(e.download() + (L, m))
        e.close()
        return out

    t0 = time.perf_counter()
    snaps = [x for k, T in enumerate(SUR_TEMPS) for x in states(T, seed + k, SUR_MARKS)]
    t_traj = time.perf_counter() - t0
    natoms = len(snaps[0][0])
    heldout = []
    for p, v, L, m in states(900.0, seed + 20, SUR_HELDOUT):
        ef = engine(p, v, L)
        heldout.append((m, ef, ef.compute_forces()[0]))

    def collect(keep):
        s = eng.Surrogate(seed=seed, cutoff=3.0, device=device)
        t0 = time.perf_counter()
        for j in keep:
            p, v, L, _ = snaps[j]
            e = engine(p, v, L)
            s.collect(e)
            e.close()
        return s, time.perf_counter() - t0

    def train(s, kind, hidden, nsnap, t_collect):
        if kind == 1:
            s.set_model(1, hidden)
        else:
            s.set_model(0)
        t0 = time.perf_counter()
        le = lf = None
        for frac, lr in SUR_LR[kind]:
            le, lf = s.train_forces(max(1, int(round(train_steps * frac))), lr=lr,
                                    w_energy=0.1 if kind == 0 else 0.0, w_force=1.0)
        t_train = time.perf_counter() - t0
        errs = {m: rel(s.forces(ef)[0], fx) for m, ef, fx in heldout}
        name = "energy network 32-64-64-1 (BF16 tcgen05)" if kind == 0 else \
            f"direct-force head 32-{hidden}-{hidden}-32 (FP32)"
        return {"model": name, "kind": kind, "hidden": 64 if kind == 0 else hidden,
                "parameters": s.nparams if kind == 0 else len(s.head_params()),
                "snapshots": nsnap, "environments": nsnap * natoms, "adam_steps": train_steps,
                "loss_force": lf, "loss_energy": le if kind == 0 else None,
                "heldout_force_rms_rel_by_step": errs,
                "heldout_force_rms_rel_mean": float(np.mean(list(errs.values()))),
                "collect_s": t_collect, "train_s": t_train}

    full = list(range(len(snaps)))
    s, t_collect = collect(full)
    plan = [(0, 64), (1, 64)] + ([(1, 32), (1, 128)] if sweep else [])
    models, chosen, saved = [], None, None
    for kind, hidden in plan:
        rec = train(s, kind, hidden, len(full), t_collect)
        models.append(rec)
        if chosen is None or rec["heldout_force_rms_rel_mean"] < \
                chosen["heldout_force_rms_rel_mean"]:
            chosen = rec
            saved = (s.head_params(), s.head_scale()) if kind == 1 else None
    # the chosen model back in place
    if chosen["kind"] == 0:
        s.set_model(0)
    else:
        s.set_model(1, chosen["hidden"])
        s.head_params(saved[0])
        s.head_scale(saved[1])
    if sweep:
        for stride in (4, 16):
            keep = full[::stride]
            sub, tc = collect(keep)
            for kind in (0, 1):
                models.append(train(sub, kind, 64, len(keep), tc))
            sub.close()
    for _, ef, _ in heldout:
        ef.close()
    pos, vel, L = system(900.0, seed + 10)
    n = len(pos)

    def run(threshold, steps, precision=eng.PREC_FP64, series=False):
        e = engine(pos, vel, L, precision)
        if threshold is not None:
            s.attach(e, threshold, 10)
        e.step(5)
        e.synchronize()
        th0 = e.thermo_now()
        ex0 = e.compute_forces()[1][3]
        es0 = s.forces(e)[1]
        errs = []
        e.set_timing(True)
        if series:  # the check error after every check (one per 10 steps);
            # a check declined for descriptors outside the training range fails
            declined = 0
            for _ in range(steps // 10):
                e.step(10)
                rep = eng.Surrogate.report(e)
                errs.append(np.inf if rep["declined_steps"] > declined else rep["last_error"])
                declined = rep["declined_steps"]
        else:
            e.step(steps)
        e.synchronize()
        ms, _ = e.kernel_time(eng.KERNEL_STEP)
        mb_ms, mb_n = e.kernel_time(eng.KERNEL_MB)
        e.set_timing(False)
        th1 = e.thermo_now()
        fk, en = e.compute_forces()
        fs, es1 = s.forces(e)
        rep = eng.Surrogate.report(e) if threshold is not None else None
        p1, v1 = e.download()
        e.close()
        # the exact FP64 forces at the final positions are the reference for every variant
        e64 = engine(p1, v1, L)
        fx, _ = e64.compute_forces()
        e64.close()
        used = threshold is not None and rep and rep["surrogate_steps"] > 0
        # the same precision with lists built at the final positions, as the
        # FP64 reference's are: the arithmetic's own error, without the list state
        same = None
        if precision != eng.PREC_FP64 and threshold is None:
            ef = engine(p1, v1, L, precision)
            same = rel(ef.compute_forces()[0], fx)
            ef.close()
        per = 1000.0 / n / steps
        out = {"md_steps": steps, "ms_per_step": ms / steps, "value": n * steps / (ms / 1e3),
               "force_rms_rel_vs_exact": rel(fs if used else fk, fx),
               "force_rms_rel_vs_exact_same_lists": same,
               "network_force_rms_rel_vs_exact": rel(fs, fx),
               "energy_drift_per_atom_per_1000_steps": ((th1["ek"] + en[3]) -
                                                        (th0["ek"] + ex0)) * per,
               "surrogate": rep}
        if used and np.isfinite(es0):  # the energy network's own energy
            out["network_energy_drift_per_atom_per_1000_steps"] = \
                ((th1["ek"] + es1) - (th0["ek"] + es0)) * per
        if threshold is None and mb_n:
            out["roofline"] = bond_order_roofline(bond_order_counts(p1, L), mb_ms / mb_n / 1e3,
                                                  arith, precision == eng.PREC_FP64)
        return out, np.array(errs)

    exact, _ = run(None, fp64_steps)
    exact32, _ = run(None, run_steps, eng.PREC_MIXED)
    # the surrogate runs beside the precision form: its error check and fallback
    # is the exact kernel of the context (FP32 pairs, FP64 Gear)
    strict, errs = run(1e-4, run_steps, eng.PREC_MIXED, series=True)
    accept = {str(t): float((errs <= t).mean()) for t in SUR_LADDER}
    tau = next((t for t in SUR_LADDER if accept[str(t)] >= 0.5), SUR_LADDER[-1])
    fin = errs[np.isfinite(errs)]
    strict["check_error_along_exact_trajectory"] = {
        "declined_checks": int((~np.isfinite(errs)).sum()),
        "min": float(fin.min()) if len(fin) else None,
        "median": float(np.median(errs)), "max": float(fin.max()) if len(fin) else None,
        "by_1000_steps": [float(np.median(errs[k:k + 100])) for k in range(0, len(errs), 100)]}
    at_best, _ = run(tau, run_steps, eng.PREC_MIXED)
    at_best["threshold"] = tau
    # the surrogate's own step: every check accepted
    every, _ = run(1.0, 1000, eng.PREC_MIXED)
    # the other model kind at the same threshold: the energy network's forces
    # are a gradient (conservative), the head's are not
    other = None
    if chosen["kind"] == 1:
        s.set_model(0)
        other, _ = run(tau, run_steps, eng.PREC_MIXED)
        other["model"] = next(m["model"] for m in models if m["kind"] == 0)
        other["threshold"] = tau
    s.close()
    return {
        "metric": "atom-steps/s of the bond-order system on 1 GB300", "unit": "atom-steps/s",
        "config": {"atoms": n, "lattice": "N diamond 16^3 cells, 1.5 A bonds, 0.02 A noise",
                   "training": f"{len(snaps)} snapshots of {natoms}-atom trajectories from "
                               f"{', '.join('%g' % t for t in SUR_TEMPS)} K over 10,000 steps "
                               f"= {len(snaps) * natoms} atomic environments, exact FP64 "
                               f"bond-order forces as labels; force matching, {train_steps} "
                               "Adam steps; held-out states along a 900 K trajectory",
                   "run": f"NVE at 900 K (dt 0.5 fs), FP64 Gear; surrogate runs {run_steps} "
                          f"steps, exact FP64 {fp64_steps} steps",
                   "threshold_policy": "exact-kernel check every 10 steps (the context's "
                                       "precision: FP32 pairs for the surrogate runs); a "
                                       "step with any atom's descriptors outside the training "
                                       "range (widened by a tenth) takes the exact forces"},
        "trajectories_s": t_traj,
        "models": models,
        "chosen_model": chosen["model"],
        "acceptance_along_exact_trajectory": accept,
        "best_accepted_threshold": tau,
        "exact": exact,
        "exact_precision_form": exact32,
        "surrogate_threshold_1e-4": strict,
        "surrogate_best_threshold": at_best,
        "surrogate_every_step_1000_steps": every,
        "surrogate_best_threshold_energy_network": other,
        "speedup_best_threshold_vs_exact": exact["ms_per_step"] / at_best["ms_per_step"],
        "speedup_threshold_1e-4_vs_exact": exact["ms_per_step"] / strict["ms_per_step"],
        "speedup_precision_form_vs_exact": exact["ms_per_step"] / exact32["ms_per_step"],
        "speedup_best_threshold_vs_precision_form":
            exact32["ms_per_step"] / at_best["ms_per_step"],
        "speedup_surrogate_step_vs_precision_form":
            exact32["ms_per_step"] / every["ms_per_step"],
    }


def run_gb300(args, rank, world):
    from moleculardynamics_gb300 import build as b
    from moleculardynamics_gb300 import engine as eng
    if rank == 0:
        b.build()
    dist = Dist(world)
    dist.barrier()
    b.build()
    eng.load()
    device = int(os.environ.get("LOCAL_RANK", "0"))
    # FP64 and FP32 rates of this device (FMA chains), the denominators of
    # the FP64 and FP32 rooflines below
    arith = eng.measure_arith_peaks(device)
    arith["sms"] = eng.device_sm_count(device)
    pos, vel, L, prec_name = make_workload(args.workload)
    n = len(pos)
    precision = eng.PREC_MIXED if prec_name == "mixed" else eng.PREC_FP64
    lj_kernel = {"auto": eng.LJ_AUTO, "rows": eng.LJ_ROWS, "cluster": eng.LJ_CLUSTER}[args.lj_kernel]
    e = engine_for(eng, n, L, precision, device, lj_kernel=lj_kernel, threads=args.threads,
                   row_loads=args.row_loads, stage_cap=args.stage_cap)
    e.upload(pos, vel)
    e.begin(0.0)
    # tiles are tuned on the thermalised state (on the initial lattice every
    # row has the same length, which favours other tilings), then warmed again
    for _ in range(args.warmup):
        e.step(MD_PER_BENCH_STEP)
    tune = e.autotune(3) if not args.no_tune else None
    e.step(MD_PER_BENCH_STEP)
    warm_steps = (args.warmup + 1) * MD_PER_BENCH_STEP
    e.synchronize()
    e.set_timing(True)
    s0 = e.stats()
    clocks = Clocks(device)
    dist.barrier()
    clocks.start()
    for _ in range(args.steps):
        e.step(MD_PER_BENCH_STEP)
    e.synchronize()
    ck = clocks.stop()
    dist.barrier()
    step_ms, _ = e.kernel_time(eng.KERNEL_STEP)
    lj_ms, lj_n = e.kernel_time(eng.KERNEL_LJ)
    pr_ms, pr_n = e.kernel_time(eng.KERNEL_PREDICT)
    co_ms, co_n = e.kernel_time(eng.KERNEL_CORRECT)
    li_ms, li_n = e.kernel_time(eng.KERNEL_LIST)
    fu_ms, fu_n = e.kernel_time(eng.KERNEL_FUSED)
    fc_ms, fc_n = e.kernel_time(eng.KERNEL_FUSED_CORRECT)
    s1 = e.stats()
    e.set_timing(False)
    t_max = dist.max(step_ms)
    md_steps = args.steps * MD_PER_BENCH_STEP
    value = world * n * md_steps / (t_max / 1e3)
    recs = e.records()
    drift = drift_per_1000(recs, n, warm_steps)
    # energy drift over the full run length of the workload (10,000 MD steps),
    # continued from the timed state; records every 100 steps
    t_drift0 = int(recs[-1, 15]) if len(recs) else 0
    for _ in range(max(args.drift_steps, 0) // MD_PER_BENCH_STEP):
        e.step(MD_PER_BENCH_STEP)
    e.synchronize()
    drift_long = drift_per_1000(e.records(), n, t_drift0) if args.drift_steps > 0 else None

    # end to end through the C ABI: the caller owns the Gear state in pinned
    # host memory; every bench step copies it in, runs, and copies it back
    hp = eng.pinned((n, 4))
    hv = eng.pinned((n, 3))
    ha, hb, hc = (eng.pinned((n, 3)) for _ in range(3))
    p0, v0 = e.download()
    st = e.download_state()
    hp[:], hv[:], ha[:], hb[:], hc[:] = p0, v0, st["acc"], st["b"], st["c"]

    def e2e_step():
        e.upload_state(hp, hv, ha, hb, hc)
        e.step(MD_PER_BENCH_STEP)
        e.lib.md_download(e.h, hp, hv)
        e.lib.md_download_state(e.h, ha.ctypes.data, hb.ctypes.data, hc.ctypes.data, None)

    for _ in range(args.warmup):  # untimed, as for the device-timed loop
        e2e_step()
    e.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e.synchronize()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = world * n * md_steps / e2e_s
    h2d = n * (32 + 24 + 3 * 24)   # pos4, vel3, acc3, b3, c3 in
    d2h = n * (32 + 24 + 3 * 24)   # the same out

    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if precision == eng.PREC_MIXED else "f64",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {n} argon atoms, FCC {WORKLOADS[args.workload][0]}^3 "
                               f"cells at rho*=0.8442, periodic L={L:.1f} A, T=94.4 K, rc=2.5 sigma, "
                               "skin 0.3 sigma, dt=2 fs, Gear 5th order",
                   "form": "precision: FP32 pairs, compensated FP32 sums, FP64 Gear state "
                           "and reductions" if precision == eng.PREC_MIXED else "plain FP64",
                   "md_steps_per_bench_step": MD_PER_BENCH_STEP, "atoms": n,
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "lj_kernel": "cluster" if s1["lj_cluster"] else "rows",
                   "autotune": tune,
                   "l2": "inputs larger than L2 (Gear state 176 MB + list >= 160 MB), no flush"},
        "gpu_launches": s1["launches"] - s0["launches"],
        "clocks": ck,
        "e2e": {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "list": {"builds_in_timed_region": s1["list_builds"] - s0["list_builds"],
                 "skin_trips": s1["list_trips"], "mean_compact_row": s1["lj_list_entries"] / n,
                 "cells_per_edge": s1["lj_cells"], "tma": s1["lj_tma"],
                 "cluster_segments": s1["cluster_segments"],
                 "cluster_max_staged": s1["cluster_max_staged"]},
        "kernel_ms_per_md_step": {
            "lj_force": lj_ms / max(lj_n, 1), "predict": pr_ms / max(pr_n, 1),
            "correct": co_ms / max(co_n, 1),
            "fused_force_gear": fu_ms / max(fu_n, 1),
            "fused_force_correct": fc_ms / max(fc_n, 1),
            "list_build_amortised": li_ms / md_steps},
        "kernel_launches": {"lj_force": lj_n, "predict": pr_n, "correct": co_n,
                            "fused_force_gear": fu_n, "fused_force_correct": fc_n,
                            "list_build": li_n},
        "accuracy": {"energy_drift_eps_per_atom_per_1000_steps": drift,
                     "energy_drift_eps_per_atom_per_1000_steps_long": drift_long,
                     "drift_leg_md_steps": args.drift_steps},
        "arith_peaks": dict(arith, how="md_measure_arith_peaks: 8 dependent FMA chains per "
                                        "thread, 2048 threads per SM, best of 3, FMA = 2 flops"),
    }
    peaks = measured_peaks()
    if fu_n:
        # the fused kernel: float4 position, 16-bit row length and entries,
        # FP64 position in and out, float4 next position out, vel/acc/b/c in
        # and out (FP64), float4 build position in
        entries = s1["lj_list_entries"]
        bytes_alg = n * (16 + 2 + 32 + 32 + 16 + 96 + 96 + 16) + 2 * entries
        avg_s = fu_ms / fu_n / 1e3
        achieved = bytes_alg / avg_s / 1e9
        peak = peaks.get("hbm_gbs")
        kname = ("k_lj_lean<1> (force + Gear, fused)" if (tune or {}).get("row_loads") == 2
                 or args.row_loads == 2 else "k_lj_cl<fused Gear>")
        line["roofline"] = {"kernel": kname, "bound": "hbm", "achieved": achieved,
                            "peak": peak if peak else 6800.0, "unit": "GB/s",
                            "frac": achieved / (peak if peak else 6800.0),
                            "peak_source": "measured" if peak else "fallback",
                            "traffic": roofline_traffic(args.workload, "lj_cluster_fused"),
                            "bytes_alg_per_launch": bytes_alg,
                            "avg_launch_ms": fu_ms / fu_n}
        line["roofline_fp32"] = fp32_roofline(entries, avg_s, arith)
        # the FP64 pipe's share: the Gear update alone at the measured FP64 rate
        floor_ms = n * GEAR_FP64_OPS_PER_ATOM / (arith["fp64_gflops"] * 1e9 / 2.0) * 1e3
        line["roofline"]["fp64_gear_floor_ms"] = floor_ms
        line["roofline"]["fp64_gear_ops_per_atom"] = GEAR_FP64_OPS_PER_ATOM
        line["roofline"]["fp64_gear_floor_share_of_launch"] = floor_ms / (fu_ms / fu_n)
        line["roofline"]["launch_ms_at_60pct_hbm"] = bytes_alg / (0.6 * line["roofline"]["peak"]
                                                                  * 1e9) * 1e3
    elif lj_n:
        entries = s1["lj_list_entries"]
        if s1["lj_cluster"]:
            # float4 position, 16-bit row length and entries, FP64 force out
            bytes_alg = n * (16 + 2 + 24) + 2 * entries
            kname = "k_lj_cl"
            traffic = roofline_traffic(args.workload, "lj_cluster")
        else:
            pos_b = 16 if precision == eng.PREC_MIXED else 32
            bytes_alg = n * (pos_b + 4 + 24) + 4 * entries
            kname = "k_lj_tma" if precision == eng.PREC_MIXED else "k_lj_fp64"
            traffic = roofline_traffic(args.workload)
        avg_s = lj_ms / lj_n / 1e3
        achieved = bytes_alg / avg_s / 1e9
        peak = peaks.get("hbm_gbs")
        line["roofline"] = {"kernel": kname,
                            "bound": "hbm", "achieved": achieved,
                            "peak": peak if peak else 6800.0, "unit": "GB/s",
                            "frac": achieved / (peak if peak else 6800.0),
                            "peak_source": "measured" if peak else "fallback",
                            "traffic": traffic,
                            "bytes_alg_per_launch": bytes_alg,
                            "avg_launch_ms": lj_ms / lj_n}
        if precision == eng.PREC_MIXED:
            line["roofline_fp32"] = fp32_roofline(entries, avg_s, arith)

    if rank == 0 and not args.no_compare:
        # plain FP64 GPU path on the same workload (fewer steps: it is slow)
        f64 = engine_for(eng, n, L, eng.PREC_FP64, device)
        f64.upload(pos, vel)
        f64.begin(0.0)
        f64.step(20)
        f64.synchronize()
        f64.set_timing(True)
        k64 = max(1, args.fp64_steps)
        f64.step(k64)
        f64.synchronize()
        ms64, _ = f64.kernel_time(eng.KERNEL_STEP)
        lj64_ms, lj64_n = f64.kernel_time(eng.KERNEL_LJ)
        ent64 = f64.stats()["lj_list_entries"]
        v64 = n * k64 / (ms64 / 1e3)
        # force error of the chosen form at the same positions
        pnow, vnow = e.download()
        f64.upload(pnow, vnow)
        f64.begin(0.0)
        fa, _ = f64.compute_forces()
        fb, _ = e.compute_forces()
        f64.close()
        rms = float(np.sqrt(((fb - fa) ** 2).sum(1).mean()) / np.sqrt((fa ** 2).sum(1).mean()))
        line["plain_fp64"] = {"value": v64, "unit": "atom-steps/s", "md_steps": k64,
                              "lj_force_ms": lj64_ms / max(lj64_n, 1),
                              "roofline": dict(fp64_lj_roofline(ent64, lj64_ms / max(lj64_n, 1)
                                                                / 1e3, arith),
                                               kernel="k_lj_fp64",
                                               avg_launch_ms=lj64_ms / max(lj64_n, 1))}
        line["speedup_vs_plain_fp64"] = value / world / v64
        line["accuracy"]["force_rms_rel_vs_fp64"] = rms
    if rank == 0 and not args.no_forms:
        line["forms"] = {"batched": batched_form(eng, device, args.batch_steps,
                                                  args.batch_loop_steps),
                         "surrogate": surrogate_form(eng, device, args.sur_train_steps,
                                                     args.sur_run_steps, args.sur_fp64_steps,
                                                     arith, args.sur_sweep)}
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        csteps = args.cpu_md_steps
        ms, kind = cpu_baseline(pos, vel, L, csteps, threads)
        line["cpu_baseline"] = {"value": n * csteps / (ms / 1e3), "unit": "atom-steps/s",
                                "cores": threads, "kind": kind,
                                "sample": f"{n} atoms, {csteps} MD steps after the list build, "
                                          f"{threads} OpenMP threads, C restatement of the "
                                          "reference step (oracle/mdoracle.c)"}
        # the reference as shipped runs on one core
        ms1, kind1 = cpu_baseline(pos, vel, L, args.cpu_1t_steps, 1)
        line["cpu_baseline_1thread"] = {
            "value": n * args.cpu_1t_steps / (ms1 / 1e3), "unit": "atom-steps/s", "cores": 1,
            "kind": kind1,
            "sample": f"{n} atoms, {args.cpu_1t_steps} MD step(s) after the list build, one "
                      "thread, C restatement of the reference step (oracle/mdoracle.c)"}
    e.close()
    dist.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def bond_order_lattice(eng, T: float, seed: int, precision, device: int = 0, ncell: int = 16):
    """Nitrogen on an ncell^3 diamond lattice (nearest neighbour 1.5 A, 0.02 A
    noise) in its periodic box, bond order only (rs 3.5 A, rcut 3.0 A, dt
    0.5 fs); returns a begun engine."""
    from moleculardynamics_gb300 import lattice as lat
    a = 4 * 1.5 / np.sqrt(3.0)
    pos, vel, L = lat.make_system("diamond", ncell, T, seed=seed, a=a, noise=0.02,
                                  species=lat.SPECIES_N, mass_table="neon")
    cfg = eng.make_config(n_mb=len(pos), use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5,
                          periodic=1, box=L, species=eng.SPECIES_NEON, device=device,
                          precision=precision)
    e = eng.Engine(cfg)
    e.upload(pos, vel)
    e.begin(0.0)
    return e


def run_case(args) -> int:
    """Profiling cases (one process, one GPU, no JSON contract line)."""
    from moleculardynamics_gb300 import build as b
    from moleculardynamics_gb300 import engine as eng
    b.build()
    eng.load()
    if args.case in ("bo32k", "bo32k64"):
        prec = eng.PREC_MIXED if args.case == "bo32k" else eng.PREC_FP64
        e = bond_order_lattice(eng, 900.0, 15, prec)
        e.set_timing(True)
        e.step(args.steps)
        e.synchronize()
        ms, _ = e.kernel_time(eng.KERNEL_STEP)
        e.close()
        print(json.dumps({"case": args.case, "atoms": 32768, "md_steps": args.steps,
                          "ms_per_step": ms / max(args.steps, 1)}))
    if args.case == "batch":
        # the batched form's ensemble (256 replicas, 1,868,538 atoms), tuned
        # after 300 steps, then --steps MD steps inside a profiler range with
        # the step split into its kernels and the list builds and skin trips
        import ctypes
        from moleculardynamics_gb300 import lattice as lat
        pos, vel, natoms, boxes, _ = lat.make_batch(256, 256, 32000, 60.0, 150.0, seed=4096)
        cfg = eng.make_config(dt=2.0, lj_rs=2.8 * SIGMA, lj_rcut=2.5 * SIGMA, periodic=1,
                              precision=eng.PREC_MIXED, species=eng.SPECIES_ARGON)
        b = eng.Batch(cfg, natoms, boxes)
        b.upload(pos, vel)
        b.begin(0.0)
        b.step(200)
        tune = b.autotune(2)
        b.step(100)
        b.synchronize()
        s0 = b.stats()
        drv = ctypes.CDLL("libcuda.so.1")
        drv.cuProfilerStart()
        b.set_timing(True)
        b.step(args.steps)
        b.synchronize()
        drv.cuProfilerStop()
        s1 = b.stats()
        split = {}
        for name, k in (("step", eng.KERNEL_STEP), ("fused", eng.KERNEL_FUSED),
                        ("fused_correct", eng.KERNEL_FUSED_CORRECT), ("predict", eng.KERNEL_PREDICT),
                        ("list", eng.KERNEL_LIST)):
            ms, cnt = b.kernel_time(k)
            split[name] = {"ms": ms, "launches": cnt}
        b.close()
        print(json.dumps({"case": "batch", "atoms": int(natoms.sum()), "md_steps": args.steps,
                          "ms_per_step": split["step"]["ms"] / max(args.steps, 1),
                          "kernels": split, "autotune": tune,
                          "list_builds": s1["list_builds"] - s0["list_builds"],
                          "skin_trips": s1["list_trips"] - s0["list_trips"],
                          "segments": s1["cluster_segments"], "max_staged": s1["cluster_max_staged"]}))
    if args.case == "sur32k":
        # a briefly trained surrogate (two FP64 snapshots, 300 Adam steps; the
        # model kind of --sur-kind) driving the 32,768-atom lattice: --steps MD
        # steps inside a profiler range (ncu --profile-from-start off)
        import ctypes
        s = eng.Surrogate(seed=5, cutoff=3.0)
        e = bond_order_lattice(eng, 900.0, 15, eng.PREC_FP64)
        for _ in range(2):
            e.step(20)
            s.collect(e)
        e.close()
        if args.sur_kind == 1:
            s.set_model(1, 64)
        s.train_forces(300, lr=1e-3, w_energy=0.1, w_force=1.0)
        e = bond_order_lattice(eng, 900.0, 15, eng.PREC_MIXED)
        s.attach(e, 1.0, 10)
        e.step(20)
        e.synchronize()
        drv = ctypes.CDLL("libcuda.so.1")
        drv.cuProfilerStart()
        e.set_timing(True)
        e.step(args.steps)
        e.synchronize()
        drv.cuProfilerStop()
        ms, _ = e.kernel_time(eng.KERNEL_STEP)
        rep = eng.Surrogate.report(e)
        e.close()
        s.close()
        print(json.dumps({"case": "sur32k", "atoms": 32768, "kind": args.sur_kind,
                          "md_steps": args.steps, "ms_per_step": ms / max(args.steps, 1),
                          "surrogate": rep}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="lj1m", choices=sorted(WORKLOADS))
    ap.add_argument("--no-compare", action="store_true", help="skip the plain FP64 leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--fp64-steps", type=int, default=100)
    ap.add_argument("--cpu-md-steps", type=int, default=5)
    ap.add_argument("--cpu-1t-steps", type=int, default=1)
    ap.add_argument("--drift-steps", type=int, default=10000,
                    help="MD steps of the energy-drift leg after the timed loop")
    ap.add_argument("--ref-md-steps", type=int, default=2)
    ap.add_argument("--lj-kernel", default="auto", choices=["auto", "rows", "cluster"])
    ap.add_argument("--no-tune", action="store_true", help="skip the cluster autotuner")
    ap.add_argument("--threads", type=int, default=0,
                    help="cluster segment threads (0: the autotuner chooses)")
    ap.add_argument("--row-loads", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="cluster row scheme: 1 block TMA tiles, 2 register prefetch, "
                         "3 per-warp TMA tiles, 4 block TMA tiles three deep "
                         "(0: the autotuner chooses)")
    ap.add_argument("--stage-cap", type=int, default=0,
                    help="cluster staged atoms per segment (0: the autotuner chooses)")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched/surrogate forms")
    ap.add_argument("--batch-steps", type=int, default=5000)
    ap.add_argument("--batch-loop-steps", type=int, default=10)
    ap.add_argument("--sur-train-steps", type=int, default=20000)
    ap.add_argument("--sur-run-steps", type=int, default=10000)
    ap.add_argument("--sur-fp64-steps", type=int, default=400)
    ap.add_argument("--sur-sweep", action="store_true",
                    help="also train the head at H = 32, 128 and both kinds on less data")
    ap.add_argument("--case", default=None, choices=["bo32k", "bo32k64", "sur32k", "batch"],
                    help="a profiling case instead of the benchmark: bo32k runs the "
                         "32,768-atom bond-order lattice in the precision form for --steps "
                         "MD steps and prints its step time (bo32k64: the plain FP64 path); "
                         "sur32k the same lattice driven by a briefly trained surrogate, the "
                         "steps inside a profiler range; batch the batched form's 256-replica "
                         "ensemble, the steps inside a profiler range")
    ap.add_argument("--sur-kind", type=int, default=1, choices=[0, 1],
                    help="sur32k: 0 the energy network, 1 the direct-force head (H = 64)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.case:
        return run_case(args)
    rank, world, _ = dist_env()
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    return run_gb300(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
