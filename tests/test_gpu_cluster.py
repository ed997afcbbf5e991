"""The cluster kernel of the precision form (periodic, LJ only) through the C ABI.

Bars: candidate rows and images bit-exact against the oracle (the state is
stored in cell order on the device; rows come back in the caller's
numbering); forces within 1e-4 relative RMS of the FP64 path at the same
positions; forces bit-identical across segment lengths and block sizes (the
per-atom pair order and arithmetic do not depend on them); downloads return
the caller's numbering.
"""
import numpy as np
import pytest

from conftest import rel_rms
from systems import argon_fcc

pytestmark = pytest.mark.gpu

RS, RC = 9.534, 8.5125


def _engine(eng, n, L, **kw):
    kw.setdefault("precision", eng.PREC_MIXED)
    cfg = eng.make_config(n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=1, box=L, **kw)
    return eng.Engine(cfg)


@pytest.mark.parametrize("ncell,natoms", [(4, None), (6, None), (8, None), (20, 32000)])
def test_cluster_rows_bit_exact(eng, oracle, ncell, natoms):
    pos, vel, L = argon_fcc(ncell, natoms=natoms, noise=0.2)
    n = len(pos)
    with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest, img = e.neighbor_list(0, images=True)
        gpos, gvel = e.download()
        st = e.stats()
    assert st["lj_cluster"] == 1
    p = pos.copy()
    nl = oracle.build_list(p, RS, L, periodic=True)
    assert (nls, nlargest) == (nl.nlistsize, nl.nlargest)
    assert np.array_equal(rows, nl.rows)
    assert np.array_equal(img, nl.code)
    oracle.free_list(nl)
    assert np.array_equal(gpos, p)      # wrapped positions, caller's numbering
    assert np.array_equal(gvel, vel)


@pytest.mark.parametrize("ncell", [4, 8, 16])
def test_cluster_forces_vs_fp64(eng, ncell):
    pos, vel, L = argon_fcc(ncell, noise=0.1)
    n = len(pos)
    out = {}
    for kind in ("fp64", "cluster"):
        kw = dict(precision=eng.PREC_FP64) if kind == "fp64" else dict(lj_kernel=eng.LJ_CLUSTER)
        with _engine(eng, n, L, **kw) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[kind] = e.compute_forces()
    err = rel_rms(out["cluster"][0], out["fp64"][0])
    assert err < 1e-4, err
    for k in range(3):   # E, E_shifted, W
        assert abs(out["cluster"][1][k] - out["fp64"][1][k]) < 1e-5 * abs(out["fp64"][1][k])


def test_cluster_matches_rows_kernel(eng):
    """Cluster and row-list kernels evaluate the same pairs in FP32."""
    pos, vel, L = argon_fcc(10, noise=0.1)
    n = len(pos)
    out = {}
    for k in (eng.LJ_ROWS, eng.LJ_CLUSTER):
        with _engine(eng, n, L, lj_kernel=k) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[k] = e.compute_forces()[0]
    assert rel_rms(out[eng.LJ_CLUSTER], out[eng.LJ_ROWS]) < 1e-6


def test_cluster_independent_of_tiling(eng):
    pos, vel, L = argon_fcc(12, noise=0.1)
    n = len(pos)
    ref = None
    for cells, threads, loads, cap in [(0, 0, 1, 0), (1, 32, 2, 0), (3, 224, 1, 0),
                                       (64, 64, 2, 0), (0, 0, 2, 0), (0, 0, 3, 0),
                                       (2, 224, 3, 0), (0, 32, 3, 0), (0, 0, 4, 0),
                                       (2, 224, 4, 0), (1, 32, 4, 0), (0, 128, 1, 64),
                                       (0, 96, 2, 1152)]:
        with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER, cluster_cells=cells,
                     cluster_threads=threads, cluster_row_loads=loads,
                     cluster_stage_cap=cap) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            e.step(20)
            p, v = e.download()
            f, en = e.compute_forces()
        if ref is None:
            ref = (p, v, f)
        else:
            assert np.array_equal(p, ref[0]) and np.array_equal(v, ref[1])
            assert np.array_equal(f, ref[2])


def test_cluster_trips_and_refresh(eng):
    """Skin trips refresh the 16-bit rows from shared memory; after 150 steps
    the forces still agree with the FP64 path at the same positions."""
    pos, vel, L = argon_fcc(10, temperature=300.0, seed=6, noise=0.1)
    n = len(pos)
    rs = 8.7
    cfg = eng.make_config(n_lj=n, lj_rs=rs, lj_rcut=RC, periodic=1, box=L,
                          precision=eng.PREC_MIXED, lj_kernel=eng.LJ_CLUSTER)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(150)
        st = e.stats()
        p, v = e.download()
        fm, _ = e.compute_forces()
    cfg = eng.make_config(n_lj=n, lj_rs=rs, lj_rcut=RC, periodic=1, box=L)
    with eng.Engine(cfg) as e:
        e.upload(p, v)
        e.begin(0.0)
        f64, _ = e.compute_forces()
    assert st["list_trips"] > 0
    assert rel_rms(fm, f64) < 1e-4


def test_cluster_mixed_species(eng):
    """N and O atoms among the argon: the type-selecting pair path."""
    pos, vel, L = argon_fcc(8, noise=0.1)
    pos[::7, 3] = 0
    pos[3::11, 3] = 1
    n = len(pos)
    out = {}
    for kind in ("fp64", "cluster"):
        kw = dict(precision=eng.PREC_FP64) if kind == "fp64" else dict(lj_kernel=eng.LJ_CLUSTER)
        with _engine(eng, n, L, species=0, **kw) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[kind] = e.compute_forces()[0]
    assert rel_rms(out["cluster"], out["fp64"]) < 1e-4


def test_cluster_state_round_trip(eng):
    """Upload after a permuting build maps through the caller's numbering."""
    pos, vel, L = argon_fcc(8, noise=0.1)
    n = len(pos)
    rng = np.random.default_rng(5)
    a3, b3, c3 = (rng.standard_normal((n, 3)) for _ in range(3))
    with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        p0, _ = e.download()
        e.upload_state(p0, vel, a3, b3, c3)
        p1, v1 = e.download()
        st = e.download_state()
    assert np.array_equal(p1, p0) and np.array_equal(v1, vel)
    assert np.array_equal(st["acc"], a3) and np.array_equal(st["b"], b3)
    assert np.array_equal(st["c"], c3)


def test_cluster_pinned_transfers(eng):
    """Pinned caller arrays are read and written by the device in place (no
    staging copy); the result equals the staged path's, and the species
    check done on the device keeps the all-argon fast path."""
    pos, vel, L = argon_fcc(8, noise=0.1)
    n = len(pos)
    rng = np.random.default_rng(6)
    a3, b3, c3 = (rng.standard_normal((n, 3)) for _ in range(3))
    hp, hv = eng.pinned((n, 4)), eng.pinned((n, 3))
    ha, hb, hc = (eng.pinned((n, 3)) for _ in range(3))
    with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(7)
        p0, v0 = e.download()
        s0 = e.download_state()
        # device -> pinned
        e.lib.md_download(e.h, hp, hv)
        e.lib.md_download_state(e.h, ha.ctypes.data, hb.ctypes.data, hc.ctypes.data, None)
        assert np.array_equal(hp, p0) and np.array_equal(hv, v0)
        assert np.array_equal(ha, s0["acc"]) and np.array_equal(hb, s0["b"])
        assert np.array_equal(hc, s0["c"])
        # pinned -> device
        hp[:], hv[:], ha[:], hb[:], hc[:] = pos, vel, a3, b3, c3
        e.upload_state(hp, hv, ha, hb, hc)
        p1, v1 = e.download()
        s1 = e.download_state()
        f1, _ = e.compute_forces()
        e.upload_state(pos, vel, a3, b3, c3)
        f2, _ = e.compute_forces()
    assert np.array_equal(p1, pos) and np.array_equal(v1, vel)
    assert np.array_equal(s1["acc"], a3) and np.array_equal(s1["b"], b3)
    assert np.array_equal(s1["c"], c3)
    assert np.array_equal(f1, f2)


def test_cluster_energy_conservation(eng):
    pos, vel, L = argon_fcc(8, seed=9)
    n = len(pos)
    with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER, output_timesteps=100) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(1000)
        rec = e.records()
    etot = rec[:, 3] + rec[:, 12]          # ek + shifted LJ energy
    eps = 9.960172e-5
    drift = abs(etot[-1] - etot[0]) / n / eps
    assert drift < 1e-4, drift


def test_records_leave_the_trajectory_unchanged(eng):
    """A record after every step makes every step a correct-only launch
    followed by the energy launch and a separate predict; the trajectory is
    that of the fused steps, bit for bit, across list builds, and the last
    record's energy is that of an energy evaluation at the final state."""
    pos, vel, L = argon_fcc(8, noise=0.1, seed=4)
    n = len(pos)
    out = {}
    for every in (0, 1):
        with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER, output_timesteps=every) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            e.step(120)
            out[every] = e.download()
            st = e.stats()
            if every:
                rec = e.records()
                assert len(rec) >= 120
                _, en = e.compute_forces()
                # the last record holds the final state's shifted LJ energy
                assert abs(rec[-1, 12] - en[1]) <= 1e-6 * abs(en[1])
        assert st["list_builds"] > 2
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_autotune_keeps_forces(eng):
    """The autotuner only changes tiling: forces stay bit-identical."""
    pos, vel, L = argon_fcc(12, noise=0.1)
    n = len(pos)
    with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        f0, _ = e.compute_forces()
        r = e.autotune(2)
        f1, _ = e.compute_forces()
        e.step(10)
    assert r["candidates"] >= 1 and r["threads"] in (64, 96, 128, 160, 192)
    assert r["row_loads"] in (1, 2, 3, 4)
    assert np.array_equal(f0, f1)


def test_dense_neighbourhood_falls_back_to_rows(eng):
    """12,167 argon atoms 1.2 A apart in a 27.6 A box (one cell with minimum
    images): more atoms than a segment can stage.  AUTO hands the system to the
    row-list kernel (the state is mapped back to the caller's numbering) and
    runs as LJ_ROWS does, bit for bit; LJ_CLUSTER reports the limit."""
    m, a = 23, 1.2
    L = m * a
    g = (np.arange(m) + 0.5) * a - L / 2
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    n = m ** 3
    rng = np.random.default_rng(3)
    pos = np.zeros((n, 4))
    pos[:, 0], pos[:, 1], pos[:, 2] = x.ravel(), y.ravel(), z.ravel()
    pos[:, :3] += rng.uniform(-0.01, 0.01, (n, 3))
    pos[:, 3] = 2
    vel = rng.normal(0.0, 1e-4, (n, 3))
    out = {}
    for k in (eng.LJ_ROWS, eng.LJ_AUTO):
        with _engine(eng, n, L, lj_kernel=k, dt=0.01) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            f0 = e.compute_forces()[0]
            e.step(4)
            p, v = e.download()
            st = e.stats()
        assert st["lj_cluster"] == 0
        assert np.isfinite(p).all() and np.isfinite(f0).all()
        out[k] = (f0, p, v)
    for a_, b_ in zip(out[eng.LJ_ROWS], out[eng.LJ_AUTO]):
        assert np.array_equal(a_, b_)
    with _engine(eng, n, L, lj_kernel=eng.LJ_CLUSTER, dt=0.01) as e:
        e.upload(pos, vel)
        with pytest.raises(eng.EngineError, match="shared-memory stage"):
            e.begin(0.0)
