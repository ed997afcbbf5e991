"""The batched form: independent periodic replicas of uneven sizes in one
context (md_batch_create), one persistent launch per step, CUDA graphs.

Bars: each replica's trajectory equals the same replica run alone through the
single-system precision path (the replicas share no pairs; list builds, and
with them the periodic wraps, may come at other steps, so positions agree to
rounding, 1e-8 A, velocities to 1e-10 A/fs); graphs on and
off give bit-identical trajectories; per-replica records equal the
single-system ones; the autotuner leaves forces bit-identical.
"""
import numpy as np
import pytest

from conftest import rel_rms
from moleculardynamics_gb300 import lattice as lat

pytestmark = pytest.mark.gpu

RS, RC = 9.534, 8.5125


def _batch_system(seed=11):
    return lat.make_batch(nrep=5, nmin=256, nmax=3000, seed=seed)


def _cfg(eng, **kw):
    return eng.make_config(dt=2.0, lj_rs=RS, lj_rcut=RC, periodic=1,
                           precision=eng.PREC_MIXED, species=eng.SPECIES_ARGON, **kw)


def _split(a, natoms):
    return np.split(a, np.cumsum(natoms)[:-1])


def test_batch_matches_single_replicas(eng):
    pos, vel, natoms, boxes, _ = _batch_system()
    with eng.Batch(_cfg(eng), natoms, boxes) as b:
        b.upload(pos, vel)
        b.begin(0.0)
        b.step(60)
        bp, bv = b.download()
        st = b.stats()
    assert st["lj_cluster"] == 1
    for k, (p, v) in enumerate(zip(_split(pos, natoms), _split(vel, natoms))):
        cfg = _cfg(eng, n_lj=len(p), box=float(boxes[k]))
        with eng.Engine(cfg) as e:
            e.upload(np.ascontiguousarray(p), np.ascontiguousarray(v))
            e.begin(0.0)
            e.step(60)
            sp, sv = e.download()
        gp = _split(bp, natoms)[k]
        gv = _split(bv, natoms)[k]
        assert np.allclose(gp[:, :3], sp[:, :3], rtol=0, atol=1e-8), k
        assert np.allclose(gv, sv, rtol=0, atol=1e-10), k
        assert np.array_equal(gp[:, 3], sp[:, 3])


def test_batch_graphs_bit_identical(eng):
    pos, vel, natoms, boxes, _ = _batch_system(seed=12)
    out = []
    for graphs in (True, False):
        with eng.Batch(_cfg(eng), natoms, boxes) as b:
            b.set_graphs(graphs)
            b.upload(pos, vel)
            b.begin(0.0)
            b.step(50)
            b.step(23)
            out.append(b.download())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_batch_records_per_replica(eng):
    pos, vel, natoms, boxes, temps = _batch_system(seed=13)
    with eng.Batch(_cfg(eng), natoms, boxes) as b:
        b.upload(pos, vel)
        b.begin(0.0)
        rec = b.replica_records()
    assert rec.shape == (len(natoms), 16)
    # the generator rescales to T with FP64 masses; the species table holds
    # them as float literals, as common/Constants.h does
    assert np.allclose(rec[:, 1], temps, rtol=1e-6)
    for k, (p, v) in enumerate(zip(_split(pos, natoms), _split(vel, natoms))):
        cfg = _cfg(eng, n_lj=len(p), box=float(boxes[k]))
        with eng.Engine(cfg) as e:
            e.upload(np.ascontiguousarray(p), np.ascontiguousarray(v))
            e.begin(0.0)
            th = e.thermo_now()
            _, en = e.compute_forces()
        assert abs(rec[k, 3] - th["ek"]) <= 1e-12 * abs(th["ek"])
        assert abs(rec[k, 11] - en[0]) <= 1e-9 * abs(en[0])
        assert abs(rec[k, 12] - en[1]) <= 1e-9 * abs(en[1])


def test_batch_energy_conservation(eng):
    pos, vel, natoms, boxes, _ = _batch_system(seed=14)
    eps = 9.960172e-5
    with eng.Batch(_cfg(eng), natoms, boxes) as b:
        b.upload(pos, vel)
        b.begin(0.0)
        r0 = b.replica_records()
        b.step(500)
        r1 = b.replica_records()
    e0 = r0[:, 3] + r0[:, 12]
    e1 = r1[:, 3] + r1[:, 12]
    drift = np.abs(e1 - e0) / natoms / eps
    assert drift.max() < 1e-4, drift


def test_batch_autotune_keeps_forces(eng):
    pos, vel, natoms, boxes, _ = _batch_system(seed=15)
    with eng.Batch(_cfg(eng), natoms, boxes) as b:
        b.upload(pos, vel)
        b.begin(0.0)
        f0, _ = b.compute_forces()
        r = b.autotune(2)
        f1, _ = b.compute_forces()
    assert r["candidates"] >= 1
    assert np.array_equal(f0, f1)


def test_batch_forces_vs_fp64(eng):
    pos, vel, natoms, boxes, _ = _batch_system(seed=16)
    with eng.Batch(_cfg(eng), natoms, boxes) as b:
        b.upload(pos, vel)
        b.begin(0.0)
        fb, _ = b.compute_forces()
    for k, (p, v) in enumerate(zip(_split(pos, natoms), _split(vel, natoms))):
        cfg = eng.make_config(n_lj=len(p), dt=2.0, lj_rs=RS, lj_rcut=RC, periodic=1,
                              box=float(boxes[k]), species=eng.SPECIES_ARGON)
        with eng.Engine(cfg) as e:
            e.upload(np.ascontiguousarray(p), np.ascontiguousarray(v))
            e.begin(0.0)
            f64, _ = e.compute_forces()
        assert rel_rms(_split(fb, natoms)[k], f64) < 1e-4, k


def test_batch_rejects_bad_input(eng):
    with pytest.raises(eng.EngineError):
        eng.Batch(_cfg(eng), [300, 300], [30.0, 15.0])          # box under 2 rs
    cfg = eng.make_config(dt=2.0, lj_rs=RS, lj_rcut=RC, periodic=1)   # FP64: not batched
    with pytest.raises(eng.EngineError):
        eng.Batch(cfg, [300], [30.0])
