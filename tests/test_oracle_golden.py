"""The CPU oracle against golden fixtures written by the reference itself
(tests/golden/make_golden.py).  Everything here is bit-exact: the oracle is a
restatement of the reference's own arithmetic built with -ffp-contract=off."""
import os

import numpy as np
import pytest

from conftest import run_params

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_fixtures.npz"))


def g(case, key):
    return GOLD[f"{case}/{key}"]


@pytest.mark.parametrize("case,species", [("lj_neon", 0), ("lj_argon", 1)])
def test_lj_rows_forces_energy_thermo(oracle, case, species):
    pos = np.ascontiguousarray(g(case, "pos"))
    vel = np.ascontiguousarray(g(case, "vel"))
    rs, rc = float(g(case, "rs")), float(g(case, "rc"))
    vmax, box = oracle.ready_list(pos, vel)
    assert box == float(g(case, "box"))
    nl = oracle.build_list(pos.copy(), rs, box)
    assert nl.nlistsize == int(g(case, "nlistsize")) and nl.nlargest == int(g(case, "nlargest"))
    assert np.array_equal(nl.rows, g(case, "rows"))
    f = oracle.lj_forces(pos, nl, oracle.settings(rs, rc)[2], species=species)
    oracle.free_list(nl)
    assert np.array_equal(f, g(case, "force"))
    assert oracle.calculate_potential(pos, species) == (float(g(case, "vib_lj")),
                                                        float(g(case, "vib_mb")))
    assert np.array_equal(oracle.perform_calculations(pos, vel, species), g(case, "thermo"))


@pytest.mark.parametrize("case,species", [("lj_neon", 0), ("lj_argon", 1)])
def test_lj_trajectory(oracle, case, species):
    pos, vel = g(case, "pos"), g(case, "vel")
    r = oracle.run(run_params(n_lj=len(pos), timesteps=int(g(case, "steps")),
                              lj_rs=float(g(case, "rs")), lj_rcut=float(g(case, "rc")),
                              output_timesteps=20, species=species), pos, vel, 10)
    for k in ("pos", "vel", "acc", "b", "c", "force"):
        assert np.array_equal(r[k], g(case, "run_" + k)), k
    assert r["builds"] == int(g(case, "run_builds"))
    assert np.array_equal(r["thermo"][:, :8], g(case, "run_thermo"))


def test_bond_order_rows_forces_energy(oracle):
    pos, vel = np.ascontiguousarray(g("bo_no", "pos")), g("bo_no", "vel")
    box = float(g("bo_no", "box"))
    nl = oracle.build_list(pos.copy(), 3.5, box)
    assert np.array_equal(nl.rows, g("bo_no", "rows"))
    f, miss = oracle.mb_forces(pos, nl, len(pos), oracle.settings(3.5, 3.0)[2])
    oracle.free_list(nl)
    assert miss == 0
    assert np.array_equal(f, g("bo_no", "force"))
    vlj, vmb = oracle.calculate_potential(pos)
    assert vmb == float(g("bo_no", "vib_mb"))


def test_bond_order_and_mixed_trajectories(oracle):
    pos, vel = g("bo_no", "pos"), g("bo_no", "vel")
    r = oracle.run(run_params(n_mb=len(pos), use_lj=0, use_mb=1, timesteps=12, dt=0.5,
                              output_timesteps=4, species=0), pos, vel, 10)
    assert np.array_equal(r["pos"], g("bo_no", "run_pos"))
    assert np.array_equal(r["vel"], g("bo_no", "run_vel"))
    assert np.array_equal(r["thermo"][:, :8], g("bo_no", "run_thermo"))
    nmb, nlj = int(g("mixed", "n_mb")), int(g("mixed", "n_lj"))
    r = oracle.run(run_params(n_lj=nlj, n_mb=nmb, use_lj=1, use_mb=1, timesteps=12, dt=0.5,
                              lj_rs=9.0, lj_rcut=8.0, output_timesteps=4, species=0),
                   g("mixed", "pos"), g("mixed", "vel"), 10)
    assert np.array_equal(r["pos"], g("mixed", "run_pos"))
    assert np.array_equal(r["vel"], g("mixed", "run_vel"))
    assert r["builds"] == int(g("mixed", "run_builds"))


def test_walls(oracle):
    pos, vel = g("walls", "pos"), g("walls", "vel")
    r = oracle.run(run_params(n_lj=len(pos), timesteps=400, lj_rs=9.0, lj_rcut=8.0, vxcm=0.9,
                              energy_loss=0.5, species=0), pos, vel)
    assert r["wall_hits"] > 0
    assert np.array_equal(r["pos"], g("walls", "run_pos"))
    assert np.array_equal(r["vel"], g("walls", "run_vel"))


def test_edge_cell_quirk(oracle):
    pos = np.ascontiguousarray(g("quirk", "pos"))
    nl = oracle.build_list(pos.copy(), 2.0, 8.0)
    assert nl.cells == 4 and nl.cell[0, 0] == 4  # the atom at +max sits in cell `cells`
    assert np.array_equal(nl.rows, g("quirk", "rows"))
    oracle.free_list(nl)


def test_empty_and_single_atom_lists(oracle):
    one = np.array([[0.0, 0.0, 0.0, 2.0]])
    nl = oracle.build_list(one.copy(), 2.0, 1.0)
    assert nl.nlistsize == 0 and nl.nlargest == 0
    oracle.free_list(nl)
    # box 2, rs 2: one cell; the atom at +max|x| lands in cell 1 == cells, so
    # atom 0 cannot see it while it sees atom 0 (NeighborList.cpp:53,81,147)
    two = np.array([[0.0, 0.0, 0.0, 2.0], [1.0, 0.0, 0.0, 2.0]])
    nl = oracle.build_list(two.copy(), 2.0, 2.0)
    assert nl.nlistsize == 1 and nl.rows.tolist() == [[-1], [0]]
    oracle.free_list(nl)


def test_oracle_is_thread_count_independent(oracle):
    pos, vel = g("lj_argon", "pos"), g("lj_argon", "vel")
    p = run_params(n_lj=len(pos), timesteps=30, output_timesteps=0, species=1)
    a = oracle.run(dict(p, threads=1), pos, vel)
    b = oracle.run(dict(p, threads=4), pos, vel)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
