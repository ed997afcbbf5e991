"""The CPU oracle against the reference engine compiled in place, on fresh
seeded inputs (bit-exact).  Skipped where the reference sources are absent."""
import numpy as np
import pytest

from conftest import run_params
from systems import argon_fcc, mixed_system, nitrogen_diamond


@pytest.mark.parametrize("seed", [101, 202])
def test_lists_and_lj_forces(oracle, reference, reference_argon, seed):
    pos, vel, L = argon_fcc(5, seed=seed, noise=0.1)
    for ref, sp in ((reference, 0), (reference_argon, 1)):
        vmax, box = oracle.ready_list(pos, vel)
        assert (vmax, box) == ref.ready_list(pos, vel)
        nl = oracle.build_list(pos.copy(), 9.534, box)
        rl = ref.build_neighbor_list(pos, 9.534, 8.5125, box)
        assert np.array_equal(nl.rows, rl.rows) and nl.nlargest == rl.nlargest
        rcsq = oracle.settings(9.534, 8.5125)[2]
        assert rcsq == ref.settings(9.534, 8.5125)[2]
        assert np.array_equal(oracle.lj_forces(pos, nl, rcsq, species=sp),
                              ref.lj_forces(pos, rl, rcsq))
        oracle.free_list(nl)


def test_bond_order_and_energy(oracle, reference):
    pos, vel, L = nitrogen_diamond(3, seed=303, mixed_o=True)
    box = oracle.ready_list(pos, vel)[1]
    nl = oracle.build_list(pos.copy(), 3.5, box)
    rl = reference.build_neighbor_list(pos, 3.5, 3.0, box)
    assert np.array_equal(nl.rows, rl.rows)
    rcsq = oracle.settings(3.5, 3.0)[2]
    f, miss = oracle.mb_forces(pos, nl, len(pos), rcsq)
    assert miss == 0
    assert np.array_equal(f, reference.mb_forces(pos, rl, len(pos), rcsq))
    oracle.free_list(nl)
    assert oracle.calculate_potential(pos) == reference.calculate_potential(pos)


def test_gear_and_thermo(oracle, reference):
    rng = np.random.default_rng(404)
    pos, vel, L = argon_fcc(3, seed=404)
    n = len(pos)
    st = [pos.copy(), vel.copy()] + [rng.standard_normal((n, 3)) * 1e-4 for _ in range(3)]
    so = [x.copy() for x in st]
    oracle.predict(*st, 1.5)
    reference.predict(*so, 1.5)
    assert all(np.array_equal(a, b) for a, b in zip(st, so))
    f = rng.standard_normal((n, 3)) * 1e-3
    fl1 = oracle.correct(st[0], st[1], f, st[2], st[3], st[4], 1.5, 3.0, 0.8)
    fl2 = reference.correct(so[0], so[1], f, so[2], so[3], so[4], 1.5, 3.0, 0.8)
    assert fl1 == fl2 == 1  # a 3 A wall half-width: atoms hit it
    assert all(np.array_equal(a, b) for a, b in zip(st, so))
    assert np.array_equal(oracle.accelerations(pos, f), reference.accelerations(pos, f))
    assert np.array_equal(oracle.perform_calculations(pos, vel), reference.perform_calculations(pos, vel))


def test_step_loops(oracle, reference, reference_argon):
    pos, vel, L = argon_fcc(4, seed=505, noise=0.05)
    p = run_params(n_lj=len(pos), timesteps=120, output_timesteps=30)
    a = oracle.run(p, pos, vel, 10)
    b = reference_argon.run(p, pos, vel, 10)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    assert np.array_equal(a["thermo"][:, :8], b["thermo"]) and a["builds"] == b["builds"]
    mpos, mvel, nmb, nlj = mixed_system(seed=606)
    p = run_params(n_lj=nlj, n_mb=nmb, use_mb=1, timesteps=10, dt=0.5, lj_rs=9.0, lj_rcut=8.0,
                   species=0)
    a = oracle.run(p, mpos, mvel)
    b = reference.run(p, mpos, mvel)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
