"""The GPU engine against outputs of the reference itself (tests/golden/),
through the C ABI: neighbour rows and LJ forces bit-exact, LJ trajectories
(60 steps, list rebuilds and wall hits included) bit-exact, bond-order
forces and trajectories within 1e-10 relative RMS."""
import os

import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_fixtures.npz"))


def g(case, key):
    a = GOLD[f"{case}/{key}"]
    return np.ascontiguousarray(a) if a.ndim else a


@pytest.mark.parametrize("case,species", [("lj_neon", 0), ("lj_argon", 1)])
def test_lj_against_reference_outputs(eng, case, species):
    pos, vel = g(case, "pos"), g(case, "vel")
    rs, rc = float(g(case, "rs")), float(g(case, "rc"))
    cfg = eng.make_config(n_lj=len(pos), lj_rs=rs, lj_rcut=rc, species=species,
                          output_timesteps=20)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nl = e.neighbor_list(0)
        assert (nls, nl) == (int(g(case, "nlistsize")), int(g(case, "nlargest")))
        assert np.array_equal(rows, g(case, "rows"))
        f, _ = e.compute_forces()
        assert np.array_equal(f, g(case, "force"))
        vlj, vmb = e.reference_potential()
        assert abs(vlj - float(g(case, "vib_lj"))) <= 1e-12 * abs(float(g(case, "vib_lj")))
        e.step(int(g(case, "steps")))
        p, v = e.download()
        st = e.download_state()
        recs = e.records()
    assert np.array_equal(p, g(case, "run_pos")) and np.array_equal(v, g(case, "run_vel"))
    for k in ("acc", "b", "c"):
        assert np.array_equal(st[k], g(case, "run_" + k)), k
    th = g(case, "run_thermo")
    assert len(recs) == len(th)
    assert np.allclose(recs[:, 1], th[:, 7], rtol=1e-12)   # temperature
    assert np.allclose(recs[:, 3], th[:, 3], rtol=1e-12)   # kinetic energy


def test_bond_order_against_reference_outputs(eng):
    pos, vel = g("bo_no", "pos"), g("bo_no", "vel")
    cfg = eng.make_config(n_mb=len(pos), use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5,
                          species=0)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nl = e.neighbor_list(1)
        assert np.array_equal(rows, g("bo_no", "rows"))
        f, _ = e.compute_forces()
        assert rel_rms(f, g("bo_no", "force")) < 1e-10
        vlj, vmb = e.reference_potential()
        assert abs(vmb - float(g("bo_no", "vib_mb"))) <= 1e-11 * abs(float(g("bo_no", "vib_mb")))
        e.step(12)
        p, v = e.download()
    assert rel_rms(p[:, :3], g("bo_no", "run_pos")[:, :3]) < 1e-12
    assert rel_rms(v, g("bo_no", "run_vel")) < 1e-8


def test_mixed_and_walls_against_reference_outputs(eng):
    nmb, nlj = int(g("mixed", "n_mb")), int(g("mixed", "n_lj"))
    cfg = eng.make_config(n_lj=nlj, n_mb=nmb, use_lj=1, use_mb=1, lj_rs=9.0, lj_rcut=8.0,
                          mb_rs=3.5, mb_rcut=3.0, dt=0.5, species=0)
    with eng.Engine(cfg) as e:
        e.upload(g("mixed", "pos"), g("mixed", "vel"))
        e.begin(0.0)
        e.step(12)
        p, v = e.download()
        st = e.stats()
    assert st["list_builds"] == int(g("mixed", "run_builds"))
    assert rel_rms(v, g("mixed", "run_vel")) < 1e-8
    pos, vel = g("walls", "pos"), g("walls", "vel")
    cfg = eng.make_config(n_lj=len(pos), lj_rs=9.0, lj_rcut=8.0, species=0, energy_loss=0.5)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.9)
        e.step(400)
        p, v = e.download()
        st = e.stats()
    assert st["wall_hits"] > 0
    assert np.array_equal(p, g("walls", "run_pos")) and np.array_equal(v, g("walls", "run_vel"))


def test_edge_cell_quirk_against_reference(eng):
    pos = g("quirk", "pos")
    vel = np.zeros((len(pos), 3))
    vel[:, 0] = 1e-3
    cfg = eng.make_config(n_lj=len(pos), lj_rs=2.0, lj_rcut=1.5, species=0)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nl = e.neighbor_list(0)
    assert np.array_equal(rows, g("quirk", "rows"))
