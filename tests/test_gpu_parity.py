"""GPU engine against the CPU oracle, through the C ABI (include/mdgb.h).

Bars: neighbour rows (and periodic images) bit-exact; LJ forces, Gear steps
and LJ trajectories bit-exact (same roundings as the reference); bond-order
forces within 1e-10 relative RMS (CUDA's exp/tanh differ from libm in the
last bit); energies, virial and thermo within 1e-12 relative (summation
order); the mixed-precision form within 1e-4 relative RMS of the FP64 path.
"""
import numpy as np
import pytest

from conftest import rel_rms, run_params
from systems import argon_fcc, mixed_system, nitrogen_diamond

pytestmark = pytest.mark.gpu

RS, RC = 9.534, 8.5125          # 2.8 and 2.5 sigma of argon
MB_RS, MB_RC = 3.5, 3.0


def _engine(eng, n_lj=0, n_mb=0, **kw):
    cfg = eng.make_config(n_lj=n_lj, n_mb=n_mb, **kw)
    return eng.Engine(cfg)


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("periodic", [0, 1])
def test_lj_rows_forces_energy(eng, oracle, periodic):
    pos, vel, L = argon_fcc(6)
    n = len(pos)
    with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=periodic, box=L) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest, img = e.neighbor_list(0, images=True)
        f, en = e.compute_forces()
        gpos, _ = e.download()
    p = pos.copy()
    box = L if periodic else oracle.ready_list(pos, vel)[1]
    nl = oracle.build_list(p, RS, box, periodic=bool(periodic))
    assert (nls, nlargest) == (nl.nlistsize, nl.nlargest)
    assert np.array_equal(rows, nl.rows)
    assert np.array_equal(img, nl.code)
    assert np.array_equal(gpos, p)  # periodic wrap is bit-identical too
    rcsq = oracle.settings(RS, RC)[2]
    fo, eo = oracle.lj_forces(p, nl, rcsq, species=1, energy=True)
    oracle.free_list(nl)
    assert np.array_equal(f, fo)
    for k in range(3):
        assert _rel(en[k], eo[k]) < 1e-12


def test_single_cell_periodic_box(eng, oracle):
    """A 256-atom box is under 3 cells wide: rows are all atoms, minimum image."""
    pos, vel, L = argon_fcc(4)
    n = len(pos)
    with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=1, box=L) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest, img = e.neighbor_list(0, images=True)
        f, _ = e.compute_forces()
    p = pos.copy()
    nl = oracle.build_list(p, RS, L, periodic=True)
    assert nl.cells == 1
    assert np.array_equal(rows, nl.rows) and np.array_equal(img, nl.code)
    fo = oracle.lj_forces(p, nl, oracle.settings(RS, RC)[2], species=1)
    oracle.free_list(nl)
    assert np.array_equal(f, fo)


def test_quirk_cell_at_box_edge(eng, oracle):
    """An atom at +max|x| lands in cell `cells` and loses its own cell
    (common/NeighborList.cpp:53,81,147)."""
    rng = np.random.default_rng(7)
    n = 200
    pos = np.zeros((n, 4))
    pos[:, :3] = rng.uniform(-3.9, 3.9, (n, 3))
    pos[0, :3] = [4.0, 1.0, -2.0]      # box = 8, rs = 2: cells = 4, this atom in cell 4
    pos[1, :3] = [-4.0, 3.9, 3.9]
    pos[:, 3] = 2
    vel = np.zeros((n, 3))
    vel[:, 0] = 1e-3
    with _engine(eng, n_lj=n, lj_rs=2.0, lj_rcut=1.5, species=0) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest = e.neighbor_list(0)
    nl = oracle.build_list(pos.copy(), 2.0, 8.0)
    assert nl.cells == 4 and nl.cell[0, 0] == 4
    assert np.array_equal(rows, nl.rows) and (nls, nlargest) == (nl.nlistsize, nl.nlargest)
    oracle.free_list(nl)


@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_systems(eng, oracle, n):
    pos, vel, L = argon_fcc(2)
    pos, vel = np.ascontiguousarray(pos[:n]), np.ascontiguousarray(vel[:n])
    with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest = e.neighbor_list(0)
        f, _ = e.compute_forces()
        e.step(5)
    nl = oracle.build_list(pos.copy(), RS, oracle.ready_list(pos, vel)[1])
    assert nls == nl.nlistsize and nlargest == nl.nlargest
    assert np.array_equal(rows, nl.rows)
    assert np.array_equal(f, oracle.lj_forces(pos, nl, oracle.settings(RS, RC)[2], species=1))
    oracle.free_list(nl)


@pytest.mark.parametrize("periodic", [0, 1])
def test_bond_order_forces(eng, oracle, periodic):
    pos, vel, L = nitrogen_diamond(4 if periodic else 3, mixed_o=True)
    n = len(pos)
    with _engine(eng, n_mb=n, use_lj=0, use_mb=1, mb_rs=MB_RS, mb_rcut=MB_RC, dt=0.5,
                 periodic=periodic, box=L, species=0) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest = e.neighbor_list(1)
        f, en = e.compute_forces()
        st = e.stats()
    p = pos.copy()
    box = L if periodic else oracle.ready_list(pos, vel)[1]
    nl = oracle.build_list(p, MB_RS, box, periodic=bool(periodic))
    assert np.array_equal(rows, nl.rows)
    fo, miss, eo = oracle.mb_forces(p, nl, n, oracle.settings(MB_RS, MB_RC)[2], energy=True)
    oracle.free_list(nl)
    assert miss == 0 and st["missing_xi"] == 0
    assert rel_rms(f, fo) < 1e-10
    assert _rel(en[3], eo[0]) < 1e-10
    if not periodic:
        assert _rel(en[4], eo[1]) < 1e-9


def test_mixed_lj_and_bond_order(eng, oracle):
    pos, vel, nmb, nlj = mixed_system()
    with _engine(eng, n_lj=nlj, n_mb=nmb, use_lj=1, use_mb=1, lj_rs=9.0, lj_rcut=8.0,
                 mb_rs=MB_RS, mb_rcut=MB_RC, dt=0.5, species=0) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        f, _ = e.compute_forces()
    box = oracle.ready_list(pos, vel)[1]
    lj = oracle.build_list(pos.copy(), 9.0, box)
    mb = oracle.build_list(pos.copy(), MB_RS, box, n=nmb)
    fo = oracle.lj_forces(pos, lj, oracle.settings(9.0, 8.0)[2], species=0)
    fo, miss = oracle.mb_forces(pos, mb, nmb, oracle.settings(MB_RS, MB_RC)[2], f_init=fo,
                                ljexist=True)
    oracle.free_list(lj)
    oracle.free_list(mb)
    assert np.array_equal(f[nmb:], fo[nmb:])  # pure LJ atoms: bit-exact
    assert rel_rms(f, fo) < 1e-10


@pytest.mark.parametrize("periodic", [0, 1])
def test_lj_trajectory_bit_exact(eng, oracle, periodic):
    """The first workload at its stated length: 864 argon atoms (FCC 6^3,
    rho* = 0.8442, 94.4 K), 1000 NVE steps of 2 fs in FP64, list rebuilds
    included, equal to the bit; records every 100 steps, their energies
    (and so the energy drift over the run) as the oracle's."""
    pos, vel, L = argon_fcc(6)
    n = len(pos)
    with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=periodic, box=L,
                 output_timesteps=100) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(1000)
        gp, gv = e.download()
        recs = e.records()
        st = e.stats()
    ref = oracle.run(run_params(n_lj=n, timesteps=1000, output_timesteps=100, periodic=periodic,
                                box=L, threads=oracle.max_threads()), pos, vel,
                     thermo_records=20)
    assert st["list_builds"] == ref["builds"]
    assert np.array_equal(gp, ref["pos"]) and np.array_equal(gv, ref["vel"])
    th = ref["thermo"]
    assert len(recs) == len(th) == 10   # t = 0, 100, ..., 900
    for r, o in zip(recs, th):
        assert _rel(r[1], o[7]) < 1e-12          # temperature
        assert _rel(r[3], o[3]) < 1e-12          # kinetic energy
        assert _rel(r[11], o[8]) < 1e-12         # E_lj
        assert _rel(r[14], o[11]) < 1e-12        # virial


def test_wall_reflections(eng, oracle):
    """The reference's walls (cpu/common/Device.cpp:86-118) with energy loss."""
    from moleculardynamics_gb300 import lattice as lat
    pos, vel, L = lat.make_system("fcc", 2, 300.0, seed=5, a=5.0, species=2, mass_table="neon")
    n = len(pos)
    with _engine(eng, n_lj=n, lj_rs=9.0, lj_rcut=8.0, species=0, energy_loss=0.5) as e:
        e.upload(pos, vel)
        e.begin(0.9)
        e.step(400)
        gp, gv = e.download()
        st = e.stats()
    ref = oracle.run(run_params(n_lj=n, timesteps=400, lj_rs=9.0, lj_rcut=8.0, species=0,
                                vxcm=0.9, energy_loss=0.5), pos, vel)
    assert st["wall_hits"] == ref["wall_hits"] > 0
    assert np.array_equal(gp, ref["pos"]) and np.array_equal(gv, ref["vel"])


def test_bond_order_trajectory(eng, oracle):
    pos, vel, L = nitrogen_diamond(3)
    n = len(pos)
    with _engine(eng, n_mb=n, use_lj=0, use_mb=1, mb_rs=MB_RS, mb_rcut=MB_RC, dt=0.5,
                 species=0) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(20)
        gp, gv = e.download()
    ref = oracle.run(run_params(n_mb=n, use_lj=0, use_mb=1, timesteps=20, dt=0.5, species=0),
                     pos, vel)
    assert rel_rms(gp[:, :3], ref["pos"][:, :3]) < 1e-12
    assert rel_rms(gv, ref["vel"]) < 1e-8


def test_periodic_bond_order_needs_three_cells(eng):
    pos, vel, L = nitrogen_diamond(3)
    with pytest.raises(eng.EngineError):
        _engine(eng, n_mb=len(pos), use_lj=0, use_mb=1, periodic=1, box=L, dt=0.5)


def test_thermo_and_reference_potential(eng, oracle):
    pos, vel, nmb, nlj = mixed_system()
    with _engine(eng, n_lj=nlj, n_mb=nmb, use_lj=1, use_mb=1, lj_rs=9.0, lj_rcut=8.0,
                 mb_rs=MB_RS, mb_rcut=MB_RC, dt=0.5, species=0) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        th = e.thermo_now()
        vlj, vmb = e.reference_potential()
    tho = oracle.perform_calculations(pos, vel)
    for k, name in enumerate(["com_x", "com_y", "com_z", "ek", "momentum_x", "momentum_y",
                              "momentum_z", "temperature"]):
        assert abs(th[name] - tho[k]) <= 1e-12 * max(abs(tho[k]), 1e-9), name
    olj, omb = oracle.calculate_potential(pos)
    assert _rel(vlj, olj) < 1e-12 and _rel(vmb, omb) < 1e-11


@pytest.mark.parametrize("ncell", [6, 16])
def test_precision_form_forces(eng, oracle, ncell):
    """FP32 pairs with compensated sums vs the FP64 path at the same positions
    (lattice with 0.1 A noise, about the thermal amplitude at 94.4 K)."""
    pos, vel, L = argon_fcc(ncell, noise=0.1)
    n = len(pos)
    out = {}
    for prec in (eng.PREC_FP64, eng.PREC_MIXED):
        with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=1, box=L, precision=prec) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[prec] = e.compute_forces()
    err = rel_rms(out[eng.PREC_MIXED][0], out[eng.PREC_FP64][0])
    assert err < 1e-4, err
    assert _rel(out[eng.PREC_MIXED][1][0], out[eng.PREC_FP64][1][0]) < 1e-5


def test_precision_form_bond_order(eng):
    pos, vel, L = nitrogen_diamond(3)
    n = len(pos)
    out = {}
    for prec in (eng.PREC_FP64, eng.PREC_MIXED):
        with _engine(eng, n_mb=n, use_lj=0, use_mb=1, mb_rs=MB_RS, mb_rcut=MB_RC, dt=0.5,
                     precision=prec, species=0) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[prec] = e.compute_forces()[0]
    assert rel_rms(out[eng.PREC_MIXED], out[eng.PREC_FP64]) < 1e-4


@pytest.mark.parametrize("mixed_o,steps", [(False, 0), (True, 0), (False, 300)])
def test_precision_form_bond_order_periodic(eng, mixed_o, steps):
    """The FP32 bond-order passes against FP64 at the same positions, lists built
    at those positions: periodic diamond (N, or N and O), on the lattice and
    after 300 FP64 steps at 900 K, when the structure has left the lattice."""
    pos, vel, L = nitrogen_diamond(4, temperature=900.0, seed=31, mixed_o=mixed_o)
    n = len(pos)
    kw = dict(n_mb=n, use_lj=0, use_mb=1, mb_rs=MB_RS, mb_rcut=MB_RC, dt=0.5, periodic=1,
              box=L, species=0)
    if steps:
        with _engine(eng, precision=eng.PREC_FP64, **kw) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            e.step(steps)
            pos, vel = e.download()
    out, miss = {}, {}
    for prec in (eng.PREC_FP64, eng.PREC_MIXED):
        with _engine(eng, precision=prec, **kw) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[prec] = e.compute_forces()[0]
            miss[prec] = e.stats()["missing_xi"]
    assert rel_rms(out[eng.PREC_MIXED], out[eng.PREC_FP64]) < 1e-4
    assert miss[eng.PREC_MIXED] == miss[eng.PREC_FP64]


def test_reference_signature_layer(eng, oracle):
    """mdgb_* (the functions a drop-in Device.cpp forwards to) against the oracle."""
    sh = eng.Shim(species=eng.SPECIES_NEON)
    pos, vel, L = argon_fcc(5)
    pos[:, 3] = 2
    n = len(pos)
    box = oracle.ready_list(pos, vel)[1]
    rows, nls, nlargest = sh.build_neighbor_list(pos, RS, RC, box)
    nl = oracle.build_list(pos.copy(), RS, box)
    assert np.array_equal(rows, nl.rows) and nlargest == nl.nlargest
    rcsq = oracle.settings(RS, RC)[2]
    f = sh.lennard_jones_forces(pos, rows, nlargest, rcsq)
    fo = oracle.lj_forces(pos, nl, rcsq, species=0)
    oracle.free_list(nl)
    assert np.array_equal(f, fo)
    rng = np.random.default_rng(11)
    st = [pos.copy(), vel.copy()] + [rng.standard_normal((n, 3)) * 1e-5 for _ in range(3)]
    so = [x.copy() for x in st]
    sh.predict(*st, 2.0)
    oracle.predict(*so, 2.0)
    assert all(np.array_equal(a, b) for a, b in zip(st, so))
    fl = sh.correct(st[0], st[1], fo, st[2], st[3], st[4], 2.0, 9.0, 0.7)
    flo = oracle.correct(so[0], so[1], fo, so[2], so[3], so[4], 2.0, 9.0, 0.7)
    assert fl == flo
    assert all(np.array_equal(a, b) for a, b in zip(st, so))
    assert np.array_equal(sh.calculate_accelerations(pos, fo), oracle.accelerations(pos, fo))
    mb_pos, mb_vel, _ = nitrogen_diamond(2)
    mbox = oracle.ready_list(mb_pos, mb_vel)[1]
    r2, nls2, nl2 = sh.build_neighbor_list(mb_pos, MB_RS, MB_RC, mbox)
    onl = oracle.build_list(mb_pos.copy(), MB_RS, mbox)
    fm = sh.many_body_forces(mb_pos, r2, nl2, len(mb_pos), oracle.settings(MB_RS, MB_RC)[2])
    fmo, _ = oracle.mb_forces(mb_pos, onl, len(mb_pos), oracle.settings(MB_RS, MB_RC)[2])
    oracle.free_list(onl)
    assert rel_rms(fm, fmo) < 1e-10
    th = sh.perform_calculations(pos, vel)
    tho = oracle.perform_calculations(pos, vel)
    # momenta cancel to ~1e-16: compare them on the scale of sum m|v|
    mscale = (20.1797 * np.abs(vel)).sum()
    assert np.allclose(th, tho, rtol=1e-12, atol=1e-13 * mscale)
    vlj, vmb = sh.calculate_potential(mb_pos)
    olj, omb = oracle.calculate_potential(mb_pos)
    assert _rel(vmb, omb) < 1e-11


def test_large_list_checksum(eng, oracle):
    """32,000 argon atoms (partially filled FCC 20^3), periodic: rows equal."""
    pos, vel, L = argon_fcc(20, natoms=32000)
    n = len(pos)
    with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=1, box=L) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest, img = e.neighbor_list(0, images=True)
    nl = oracle.build_list(pos.copy(), RS, L, periodic=True)
    assert np.array_equal(rows, nl.rows) and np.array_equal(img, nl.code)
    oracle.free_list(nl)


def test_skin_trip_refresh_keeps_trajectory_exact(eng, oracle):
    """Atoms at 1 K on a lattice with 0.5 A noise: the largest speed at the
    build is tiny, so the reference's schedule (Host.cpp:289) waits long, while
    the noise accelerates atoms past the list's skin.  The engine then walks
    the full candidate rows and refreshes the compact rows; the trajectory must
    still equal the oracle's, which always walks the full rows."""
    pos, vel, L = argon_fcc(6, temperature=1.0, seed=4, noise=0.5)
    n = len(pos)
    rs, rc = RS, RC
    with _engine(eng, n_lj=n, lj_rs=rs, lj_rcut=rc, periodic=1, box=L) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(200)
        gp, gv = e.download()
        st = e.stats()
    ref = oracle.run(run_params(n_lj=n, timesteps=200, lj_rs=rs, lj_rcut=rc, periodic=1, box=L),
                     pos, vel)
    assert st["list_trips"] > 0
    assert st["list_builds"] == ref["builds"]
    assert np.array_equal(gp, ref["pos"]) and np.array_equal(gv, ref["vel"])


def test_precision_form_trips_and_tma_path(eng):
    """Precision form through the TMA kernel, with skin trips: forces stay
    within 1e-4 of the FP64 path at the same positions."""
    pos, vel, L = argon_fcc(10, temperature=300.0, seed=6, noise=0.1)
    n = len(pos)
    rs, rc = 8.7, 8.5125
    with _engine(eng, n_lj=n, lj_rs=rs, lj_rcut=rc, periodic=1, box=L,
                 precision=eng.PREC_MIXED) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(150)
        st = e.stats()
        p, v = e.download()
        fm, _ = e.compute_forces()
    with _engine(eng, n_lj=n, lj_rs=rs, lj_rcut=rc, periodic=1, box=L) as e:
        e.upload(p, v)
        e.begin(0.0)
        f64, _ = e.compute_forces()
    assert st["list_trips"] > 0
    assert rel_rms(fm, f64) < 1e-4
