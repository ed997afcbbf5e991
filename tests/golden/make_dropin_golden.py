#!/usr/bin/env python3
"""Generates tests/golden/dropin/: the files the reference's own cpumd writes
for one run, to be compared byte for byte with what mdgb_run writes.

Run where the reference sources exist: oracle/build_ref.sh builds the
unmodified cpumd program (cpu/cpumd/Main.cpp + Host.cpp and the common
files, argon in the NG slot) as oracle/_ref/cpumd_argon.  The run:
  864 argon atoms, FCC 6^3 at rho* = 0.8442, Maxwell-Boltzmann at 94.4 K
  (seeded), LJ rs 2.8 sigma / rcut 2.5 sigma, dt 2 fs, 200 steps, records
  every 50 steps, animation frames every 50 steps, vxcm 0 and 0.001 (two
  passes of the sweep, cpu/cpumd/Host.cpp:75), walls as the reference has
  them (no periodic box).
Committed: the configuration file, the input state (dropin_input.npz; the
Input text file is written from it by input_text below), the .dat/.txt
pair of every pass, and SHA-256 digests of the Output file and of the .anm
animation of every pass (manifest.json).
With --bond-order: the bond-order and mixed cases of tests/golden/dropin_bo/
and tests/golden/dropin_mixed/ (main_bond_order below).
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "dropin")
sys.path.insert(0, ROOT)

CONFIG = "dropin.cfg"
VXCM = ("0", "0.001")


def input_text(pos4: np.ndarray, vel3: np.ndarray) -> str:
    """The Input file (common/Loader.cpp:125-155: x y z type vx vy vz per
    atom, whitespace separated), every double written with 17 significant
    digits so that it reads back exactly."""
    rows = np.concatenate([pos4, vel3], axis=1)
    return "".join(" ".join("%.17g" % v for v in r) + "\n" for r in rows)


def sha256(path: str) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def outputs(run_dir: str):
    """(name -> bytes of the .dat/.txt files, name -> digest of Output/.anm)"""
    files, digests = {}, {}
    for v in VXCM:
        for ext in ("dat", "txt"):
            name = f"results(vxcm-{v}).{ext}"
            with open(os.path.join(run_dir, name), "rb") as f:
                files[name] = f.read()
        name = f"anim(vxcm-{v}).anm"
        digests[name] = sha256(os.path.join(run_dir, name))
    digests["output.txt"] = sha256(os.path.join(run_dir, "output.txt"))
    return files, digests


def main():
    from moleculardynamics_gb300 import lattice as lat
    from oracle.oracle import REF_DIR
    exe = os.path.join(REF_DIR, "cpumd_argon")
    if not os.path.exists(exe):
        sys.exit("oracle/_ref/cpumd_argon not built (run oracle/build_ref.sh)")
    os.makedirs(OUT, exist_ok=True)
    pos, vel, _ = lat.make_system("fcc", 6, 94.4, seed=864)
    np.savez(os.path.join(OUT, "dropin_input.npz"), pos=pos, vel=vel)
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(os.path.join(OUT, CONFIG), d)
        with open(os.path.join(d, "input.txt"), "w") as f:
            f.write(input_text(pos, vel))
        r = subprocess.run([exe, CONFIG], cwd=d, capture_output=True, text=True)
        if r.returncode != 0:
            sys.exit(r.stdout + r.stderr)
        files, digests = outputs(d)
    for name, data in files.items():
        with open(os.path.join(OUT, name), "wb") as f:
            f.write(data)
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump({"config": CONFIG, "vxcm": list(VXCM), "files": sorted(files),
                   "sha256": digests}, f, indent=1, sort_keys=True)
    print("wrote", OUT)


def bond_order_case(name: str, cfg: str, pos, vel):
    """tests/golden/<name>/: the unmodified cpumd with the reference's own
    constants (oracle/_ref/cpumd_neon) on cfg.  The bond-order forces use exp
    and tanh, whose CUDA and libm results differ in the last bits, so the
    comparison is numerical: the run's Output, .dat and .txt are committed
    whole."""
    from oracle.oracle import REF_DIR
    exe = os.path.join(REF_DIR, "cpumd_neon")
    if not os.path.exists(exe):
        sys.exit("oracle/_ref/cpumd_neon not built (run oracle/build_ref.sh)")
    out = os.path.join(HERE, name)
    np.savez(os.path.join(out, "dropin_input.npz"), pos=pos, vel=vel)
    names = ["results(vxcm-0).dat", "results(vxcm-0).txt", "output.txt"]
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(os.path.join(out, cfg), d)
        with open(os.path.join(d, "input.txt"), "w") as f:
            f.write(input_text(pos, vel))
        r = subprocess.run([exe, cfg], cwd=d, capture_output=True, text=True)
        if r.returncode != 0:
            sys.exit(r.stdout + r.stderr)
        for fname in names:
            shutil.copy(os.path.join(d, fname), os.path.join(out, fname))
    with open(os.path.join(out, "manifest.json"), "w") as f:
        json.dump({"config": cfg, "files": names}, f, indent=1, sort_keys=True)
    print("wrote", out)


def main_bond_order():
    """dropin_bo: 64 N and O atoms alternating on a 2^3 diamond (1.5 A bonds,
    0.02 A noise, 300 K); dropin_mixed: the same block beside 108 neon atoms
    (FCC 3^3 at 6.0 A, 100 K, 22 A away), LJ and bond order together."""
    from moleculardynamics_gb300 import lattice as lat
    a = 4 * 1.5 / np.sqrt(3.0)
    pos, vel, _ = lat.make_system("diamond", 2, 300.0, seed=64, a=a, noise=0.02,
                                  species=lat.SPECIES_N, mass_table="neon")
    pos[::2, 3] = lat.SPECIES_O
    bond_order_case("dropin_bo", "dropin_bo.cfg", pos, vel)
    p2, v2, _ = lat.make_system("fcc", 3, 100.0, seed=65, a=6.0, species=lat.SPECIES_NG,
                                mass_table="neon")
    p2[:, :3] += np.array([22.0, 0.0, 0.0])
    bond_order_case("dropin_mixed", "dropin_mixed.cfg",
                    np.ascontiguousarray(np.concatenate([pos, p2])),
                    np.ascontiguousarray(np.concatenate([vel, v2])))


if __name__ == "__main__":
    if "--bond-order" in sys.argv:
        main_bond_order()
    else:
        main()
