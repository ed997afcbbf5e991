"""Edge cases through the C ABI against the oracle: no atoms, one atom, two
LJ atoms, a lone bond-order pair, and the precision form on a periodic box
under three cells wide (minimum images)."""
import numpy as np
import pytest

from conftest import rel_rms, run_params
from systems import argon_fcc

pytestmark = pytest.mark.gpu

RS, RC = 9.534, 8.5125


def _engine(eng, **kw):
    return eng.Engine(eng.make_config(**kw))


@pytest.mark.parametrize("n_lj,n_mb", [(0, 0), (-1, 2), (2, -1)])
def test_no_atoms_is_a_config_error(eng, n_lj, n_mb):
    with pytest.raises(eng.EngineError) as ei:
        _engine(eng, n_lj=n_lj, n_mb=n_mb)
    assert ei.value.status == 1  # MD_BAD_CONFIG


def _trajectory(eng, oracle, pos, vel, steps, **kw):
    with _engine(eng, **kw) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(steps)
        gp, gv = e.download()
        st = e.stats()
    p = {k: v for k, v in kw.items() if k in run_params()}
    ref = oracle.run(run_params(timesteps=steps, **p), pos, vel)
    return gp, gv, st, ref


def test_one_atom_moves_in_a_straight_line(eng, oracle):
    """No neighbour: zero force, the Gear steps of a free particle, bit for bit."""
    pos = np.array([[0.0, 0.0, 0.0, 2.0]])
    vel = np.array([[1e-3, -2e-3, 5e-4]])
    gp, gv, st, ref = _trajectory(eng, oracle, pos, vel, 50, n_lj=1, lj_rs=RS, lj_rcut=RC,
                                  species=1)
    assert np.array_equal(gp, ref["pos"]) and np.array_equal(gv, ref["vel"])
    assert np.array_equal(gv, vel)
    assert st["list_builds"] == ref["builds"]


def test_two_argon_atoms(eng, oracle):
    """One pair approaching through the minimum of the potential, 200 steps, bit for bit."""
    pos = np.array([[0.0, 0.0, 0.0, 2.0], [3.9, 0.3, -0.2, 2.0]])
    vel = np.array([[1e-3, 0.0, 0.0], [-1e-3, 0.0, 0.0]])
    gp, gv, st, ref = _trajectory(eng, oracle, pos, vel, 200, n_lj=2, lj_rs=RS, lj_rcut=RC,
                                  species=1)
    assert np.array_equal(gp, ref["pos"]) and np.array_equal(gv, ref["vel"])
    assert st["list_builds"] == ref["builds"]


def test_lone_bond_order_pair(eng, oracle):
    """An N-O pair at 1.5 A with no third body: forces and a 100-step
    trajectory within the bond-order bar (1e-10)."""
    pos = np.array([[0.0, 0.0, 0.0, 0.0], [1.5, 0.1, 0.0, 1.0]])
    vel = np.zeros((2, 3))
    kw = dict(n_mb=2, use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5, species=0)
    with _engine(eng, **kw) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        f, _ = e.compute_forces()
    p = pos.copy()
    nl = oracle.build_list(p, 3.5, oracle.ready_list(pos, vel)[1])
    fo, miss = oracle.mb_forces(p, nl, 2, oracle.settings(3.5, 3.0)[2])
    oracle.free_list(nl)
    assert miss == 0 and rel_rms(f, fo) < 1e-10
    assert np.allclose(f[0], -f[1], rtol=1e-12, atol=0.0)  # a pair: equal and opposite
    gp, gv, st, ref = _trajectory(eng, oracle, pos, vel, 100, **kw)
    assert rel_rms(gp[:, :3], ref["pos"][:, :3]) < 1e-10
    assert rel_rms(gv, ref["vel"]) < 1e-8


def test_precision_form_on_a_box_under_three_cells(eng):
    """256 argon atoms, periodic L = 21.0 A < 3 r_list: the precision form's
    minimum-image path against the FP64 path at the same positions."""
    pos, vel, L = argon_fcc(4, noise=0.1)
    n = len(pos)
    out = {}
    for prec in (eng.PREC_FP64, eng.PREC_MIXED):
        with _engine(eng, n_lj=n, lj_rs=RS, lj_rcut=RC, periodic=1, box=L,
                     precision=prec, species=1) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            out[prec] = e.compute_forces()[0]
            e.step(50)
    assert rel_rms(out[eng.PREC_MIXED], out[eng.PREC_FP64]) < 1e-4
