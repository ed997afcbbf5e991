#!/usr/bin/env python3
"""Generates tests/golden/ from the reference engine compiled in place.

Run where the reference sources exist (oracle/build_ref.sh builds
oracle/_ref/libmdref_{neon,argon}.so from them); the outputs are committed so
that the tests can pin the oracle on machines without the reference.

Every fixture is the reference's own output on a seeded input:
  lj_neon     108 NG atoms (reference constants), FCC 3^3, no periodic box:
              neighbour rows, LJ forces, calculatePotentional,
              PerformCalculations, 60 steps of the hostMain loop
  lj_argon    256 argon atoms (NG slot re-parameterised), FCC 4^3, 60 steps
  bo_no       64 bond-order atoms (N and O) on a diamond lattice: rows,
              manyBodyForces, calculatePotentional, 12 steps
  mixed       64 bond-order + 108 NG atoms, 12 steps of LJ + bond order
  walls       32 NG atoms thrown at the walls (vxcm 0.9, energy loss 0.5)
  quirk       an atom at +max|x| in cell `cells` (NeighborList.cpp:53,81,147)
  configs/    configuration files and the values readConfiguration returns
              (alone: make_golden.py --configs-only)
  results     a .dat/.txt pair written by writeResults/tailResults
"""
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from moleculardynamics_gb300 import lattice as lat  # noqa: E402
from oracle.oracle import build_reference, load_reference  # noqa: E402


def params(**kw):
    d = dict(n_lj=0, n_mb=0, timesteps=0, use_lj=1, use_mb=0, output_timesteps=20, dt=2.0,
             lj_rs=7.0, lj_rcut=6.5, mb_rs=3.5, mb_rcut=3.0, energy_loss=1.0, vxcm=0.0,
             periodic=0, box=0.0, species=0, threads=0)
    d.update(kw)
    return d


def lj_case(R, pos, vel, rs, rc, steps, species_name):
    vmax, box = R.ready_list(pos, vel)
    nl = R.build_neighbor_list(pos, rs, rc, box)
    rcsq = R.settings(rs, rc)[2]
    f = R.lj_forces(pos, nl, rcsq)
    vlj, vmb = R.calculate_potential(pos)
    th = R.perform_calculations(pos, vel)
    run = R.run(params(n_lj=len(pos), timesteps=steps, lj_rs=rs, lj_rcut=rc), pos, vel, 10)
    return dict(pos=pos, vel=vel, rs=rs, rc=rc, box=box, rows=nl.rows, nlistsize=nl.nlistsize,
                nlargest=nl.nlargest, force=f, vib_lj=vlj, vib_mb=vmb, thermo=th,
                steps=steps, run_pos=run["pos"], run_vel=run["vel"], run_acc=run["acc"],
                run_b=run["b"], run_c=run["c"], run_force=run["force"],
                run_thermo=run["thermo"], run_builds=run["builds"], species=species_name)


def write_configs(R):
    """Configuration files (common/ConfigParser.cpp semantics) and the values
    the reference's readConfiguration returns for them."""
    cfgdir = os.path.join(HERE, "configs")
    os.makedirs(cfgdir, exist_ok=True)
    base = {"Lennard Jones Particles": "864", "Many Body Particles": "0", "Timesteps": "1000",
            "DT": "2", "Temperature": "94.4", "LennardJonesRS": "9.534",
            "LennardJonesRCUT": "8.5125", "ManyBodyRS": "3.5", "ManyBodyRCUT": "3",
            "Input": "input.txt", "Output": "output.txt", "Filename": "results",
            "CUDA Blocks": "64", "Use Cuda": "0", "UseLennardJones": "1", "UseManyBody": "0",
            "LennardJonesBPP": "0", "ManyBodyBPP": "0", "OutputTimesteps": "100", "Debug": "0",
            "Fallback": "1", "VXCMFROM": "0", "VXCMTO": "0", "VXCMSTEP": "1", "EnergyLoss": "1",
            "AnimationTimesteps": "-1", "AnimationData": "anim"}
    cases = {
        "plain": "".join(f"{k}={v}\n" for k, v in base.items()),
        "comments_case_blanks": "// header comment\n\n" + "".join(
            f"{k.lower() if i % 2 else k.upper()}={v}   // note\n" if k != "Input" else
            f"{k}={v}\t \n" for i, (k, v) in enumerate(base.items())),
        "duplicate_first_wins": "".join(f"{k}={v}\n" for k, v in base.items()) + "Timesteps=5\n",
        "single_char_value_kept_blanks": "".join(
            f"{k}={v}{'  ' if k == 'Debug' else ''}\n" for k, v in base.items()),
        # "//" cut at its last occurrence again and again: "output.txt///c" -> "output.txt/"
        "triple_slash_comment": "".join(
            f"{k}={v}{'///c' if k == 'Output' else ''}\n" for k, v in base.items()),
        # a value of blanks only keeps them
        "blank_only_value": "".join(
            f"{k}={'   ' if k == 'AnimationData' else v}\n" for k, v in base.items()),
        # the last line has no newline
        "last_line_without_newline": "\n".join(f"{k}={v}" for k, v in base.items()),
    }
    expect = {}
    for name, text in cases.items():
        path = os.path.join(cfgdir, name + ".cfg")
        with open(path, "w") as fh:
            fh.write(text)
        ints = np.zeros(13, np.int32)
        floats = np.zeros(10, np.float32)
        import ctypes as C
        strs = C.create_string_buffer(1024)
        R.lib.ref_read_configuration(path.encode(), ints, floats, strs)
        raw = strs.raw
        expect[name] = dict(ints=ints.tolist(), floats=[float(x) for x in floats],
                            strings=[raw[256 * k:256 * (k + 1)].split(b"\0")[0].decode()
                                     for k in range(4)])
    # files the reference rejects (missing key; line without '=')
    with open(os.path.join(cfgdir, "bad_missing_key.cfg"), "w") as fh:
        fh.write("".join(f"{k}={v}\n" for k, v in base.items() if k != "EnergyLoss"))
    with open(os.path.join(cfgdir, "bad_no_equals.cfg"), "w") as fh:
        fh.write("".join(f"{k}={v}\n" for k, v in base.items()) + "garbage line\n")
    # keys are not trimmed: "Timesteps =5" is another key, and Timesteps is missing
    with open(os.path.join(cfgdir, "bad_key_with_blank.cfg"), "w") as fh:
        fh.write("".join(f"{k}{' ' if k == 'Timesteps' else ''}={v}\n"
                         for k, v in base.items()))
    with open(os.path.join(cfgdir, "expected.json"), "w") as fh:
        json.dump(expect, fh, indent=1)


def main():
    build_reference()
    R = load_reference("neon")
    RA = load_reference("argon")
    if R is None or RA is None:
        sys.exit("reference not built (sources missing?)")
    if "--configs-only" in sys.argv:
        write_configs(R)
        return
    out = {}
    pos, vel, _ = lat.make_system("fcc", 3, 100.0, seed=11, a=4.3, species=2,
                                  mass_table="neon", noise=0.05)
    out["lj_neon"] = lj_case(R, pos, vel, 7.0, 6.5, 60, "neon")
    pos, vel, _ = lat.make_system("fcc", 4, 94.4, seed=12, noise=0.05)
    out["lj_argon"] = lj_case(RA, pos, vel, 9.534, 8.5125, 60, "argon")

    # bond order: 64 atoms, N and O, diamond with nearest neighbour 1.5 A
    a = 4 * 1.5 / np.sqrt(3)
    pos, vel, _ = lat.make_system("diamond", 2, 300.0, seed=13, a=a, noise=0.02, species=0,
                                  mass_table="neon")
    pos[::2, 3] = 1
    vmax, box = R.ready_list(pos, vel)
    nl = R.build_neighbor_list(pos, 3.5, 3.0, box)
    rcsq = R.settings(3.5, 3.0)[2]
    f = R.mb_forces(pos, nl, len(pos), rcsq)
    vlj, vmb = R.calculate_potential(pos)
    run = R.run(params(n_mb=len(pos), use_lj=0, use_mb=1, timesteps=12, dt=0.5,
                       output_timesteps=4), pos, vel, 10)
    out["bo_no"] = dict(pos=pos, vel=vel, box=box, rows=nl.rows, nlistsize=nl.nlistsize,
                        nlargest=nl.nlargest, force=f, vib_lj=vlj, vib_mb=vmb,
                        run_pos=run["pos"], run_vel=run["vel"], run_force=run["force"],
                        run_thermo=run["thermo"], run_builds=run["builds"])

    # mixed: bond-order block plus a neon block beside it
    p1 = pos.copy()
    v1 = vel.copy()
    p2, v2, _ = lat.make_system("fcc", 3, 100.0, seed=14, a=6.0, species=2, mass_table="neon")
    p2[:, :3] += np.array([22.0, 0.0, 0.0])
    mp = np.ascontiguousarray(np.concatenate([p1, p2]))
    mv = np.ascontiguousarray(np.concatenate([v1, v2]))
    run = R.run(params(n_lj=len(p2), n_mb=len(p1), use_lj=1, use_mb=1, timesteps=12, dt=0.5,
                       lj_rs=9.0, lj_rcut=8.0, output_timesteps=4), mp, mv, 10)
    out["mixed"] = dict(pos=mp, vel=mv, n_mb=len(p1), n_lj=len(p2), run_pos=run["pos"],
                        run_vel=run["vel"], run_thermo=run["thermo"],
                        run_builds=run["builds"])

    # walls: a small cluster thrown at the walls
    pos, vel, _ = lat.make_system("fcc", 2, 300.0, seed=5, a=5.0, species=2, mass_table="neon")
    run = R.run(params(n_lj=len(pos), timesteps=400, lj_rs=9.0, lj_rcut=8.0, vxcm=0.9,
                       energy_loss=0.5, output_timesteps=100), pos, vel, 10)
    out["walls"] = dict(pos=pos, vel=vel, run_pos=run["pos"], run_vel=run["vel"],
                        run_builds=run["builds"])

    # the edge quirk: box 8, rs 2, one atom at x = +4 in cell 4 == cells
    rng = np.random.default_rng(7)
    qp = np.zeros((200, 4))
    qp[:, :3] = rng.uniform(-3.9, 3.9, (200, 3))
    qp[0, :3] = [4.0, 1.0, -2.0]
    qp[1, :3] = [-4.0, 3.9, 3.9]
    qp[:, 3] = 2
    nl = R.build_neighbor_list(qp, 2.0, 1.5, 8.0)
    out["quirk"] = dict(pos=qp, rows=nl.rows, nlistsize=nl.nlistsize, nlargest=nl.nlargest)

    flat = {}
    for case, d in out.items():
        for k, v in d.items():
            flat[f"{case}/{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "reference_fixtures.npz"), **flat)

    write_configs(R)

    # results writer
    rng = np.random.default_rng(21)
    recs = rng.standard_normal((3, 11))
    recs[:, 0] = [0.0, 200.0, 400.0]
    rp = out["bo_no"]["pos"]
    tmp = tempfile.mkdtemp()
    stem = os.path.join(tmp, "res")
    R.lib.ref_write_results(stem.encode(), 0, len(rp), 200, 2.0, 0, 9.0, 8.0, 1, 3.5, 3.0,
                            0.5, 123.0, np.ascontiguousarray(recs), 3, np.ascontiguousarray(rp))
    shutil.copy(stem + "(vxcm-0.5).dat", os.path.join(HERE, "results_vxcm-0.5.dat"))
    shutil.copy(stem + "(vxcm-0.5).txt", os.path.join(HERE, "results_vxcm-0.5.txt"))
    np.save(os.path.join(HERE, "results_records.npy"), recs)
    shutil.rmtree(tmp)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
