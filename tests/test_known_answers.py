"""Known answers the reference itself never tested, checked on the CPU oracle
(the same arithmetic the GPU engine is held to)."""
import numpy as np
import pytest

from moleculardynamics_gb300 import lattice as lat

SIG, EPS = 3.405, 9.960172e-5


def pair(r):
    pos = np.array([[0.0, 0.0, 0.0, 2.0], [r, 0.0, 0.0, 2.0]])
    return pos


def test_two_argon_atoms(oracle):
    """f = r_ij 24 eps / sigma^2 (2 (sigma/r)^14 - (sigma/r)^8): zero at the LJ
    minimum 2^(1/6) sigma, 24 eps / sigma (repulsive) at r = sigma."""
    for r, expect in ((2 ** (1 / 6) * SIG, 0.0), (SIG, 24 * EPS / SIG)):
        pos = pair(r)
        nl = oracle.build_list(pos.copy(), 9.0, 2 * r)
        f = oracle.lj_forces(pos, nl, 8.5 ** 2, species=1)
        oracle.free_list(nl)
        fx = -f[0, 0]  # force on atom 0 points away from atom 1 when repulsive
        assert abs(fx - expect) <= 1e-6 * 24 * EPS / SIG
        assert np.array_equal(f[0], -f[1])


def _energy_lj(oracle, pos, rs, rc):
    nl = oracle.build_list(pos.copy(), rs, oracle.ready_list(pos, np.zeros((len(pos), 3)))[1])
    f, e = oracle.lj_forces(pos, nl, oracle.settings(rs, rc)[2], species=1, energy=True)
    oracle.free_list(nl)
    return f, e[0]


def test_lj_forces_are_the_gradient_of_the_list_energy(oracle):
    """F_i = -dE/dr_i by central differences (E over the same pairs)."""
    pos, _, _ = lat.make_system("fcc", 2, 0.0, seed=1, noise=0.2)
    pos = np.ascontiguousarray(pos)
    f, _ = _energy_lj(oracle, pos, 12.0, 11.0)
    h = 1e-5
    rng = np.random.default_rng(0)
    for i in rng.choice(len(pos), 6, replace=False):
        for d in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[i, d] += h
            p2[i, d] -= h
            fd = -(_energy_lj(oracle, p1, 12.0, 11.0)[1] - _energy_lj(oracle, p2, 12.0, 11.0)[1]) / (2 * h)
            assert abs(fd - f[i, d]) <= 1e-6 * np.abs(f).max()


def test_bond_order_force_versus_gradient(oracle):
    """The reference's bond-order force is not the exact gradient of its pair
    energy (BondOrderFuncs.h: xi_ji is summed over i's neighbours, and the
    third-body pass keeps only j in k's row).  Recorded bound: the force
    agrees with -dE/dr to 30% RMS on a compact N2-like cluster, and the
    two-atom case (no third body) is exact."""
    pos = np.array([[0.0, 0.0, 0.0, 0.0], [1.2, 0.1, -0.05, 0.0]])
    nl = oracle.build_list(pos.copy(), 3.5, 2.5)
    f, miss, e = oracle.mb_forces(pos, nl, 2, oracle.settings(3.5, 3.0)[2], energy=True)
    h = 1e-6
    p1, p2 = pos.copy(), pos.copy()
    p1[1, 0] += h
    p2[1, 0] -= h
    e1 = oracle.mb_forces(p1, nl, 2, oracle.settings(3.5, 3.0)[2], energy=True)[2][0]
    e2 = oracle.mb_forces(p2, nl, 2, oracle.settings(3.5, 3.0)[2], energy=True)[2][0]
    oracle.free_list(nl)
    # E counts each ordered pair once with a factor 1/2: dE/dx_1 = F_1 for two atoms
    assert abs(-(e1 - e2) / (2 * h) - f[1, 0]) <= 1e-6 * abs(f[1, 0])


def test_gear_harmonic_oscillator(oracle):
    """Gear predictor-corrector on x'' = -w^2 x against cos(w t)."""
    m = 39.948
    k = 1e-3
    w = np.sqrt(k / m)
    dt = 2.0
    r = np.array([[1.0, 0.0, 0.0, 2.0]])
    v = np.zeros((1, 3))
    a = np.array([[-k * 1.0 / m, 0.0, 0.0]])
    b = np.zeros((1, 3))
    c = np.zeros((1, 3))
    steps = 2000
    for _ in range(steps):
        oracle.predict(r, v, a, b, c, dt)
        f = np.array([[-k * r[0, 0], 0.0, 0.0]])
        oracle.correct(r, v, f, a, b, c, dt, 1e9, 1.0, walls=False, species=1)
    exact = np.cos(w * dt * steps)
    assert abs(r[0, 0] - exact) < 2e-3


def test_thermo_identities(oracle):
    pos, vel, _ = lat.make_system("fcc", 3, 94.4, seed=9)
    out = oracle.perform_calculations(pos, vel, species=1)
    m = float(np.float32(39.948))  # the reference's masses are float literals
    assert abs(out[3] - 0.5 * m * (vel ** 2).sum()) <= 1e-12 * out[3]
    assert np.all(np.abs(out[4:7]) < 1e-12 * m * np.abs(vel).sum())   # momentum zeroed
    assert abs(out[7] - 94.4) < 1e-6 * 94.4                          # temperature rescaled
