"""Failure detection on the GPU, made on the host: every failure here comes
from an input or a setting, never from a fault of the GPU.

The reference ends the process on any error (common/Global.h:116-117
TC/CPPSAFE_CALL); the engine returns a status instead and leaves the device
usable.  Each test checks the status the call returns, then that the same
GPU still runs a correct step afterwards.
  * bounded waits: md_set_wait_limit(0) makes the first mbarrier wait of the
    LJ kernels give up; the kernel records the timeout, lets its copies in
    flight land and returns, and md_step reports MD_TIMEOUT;
  * non-finite input: a NaN position or velocity, or two atoms on the same
    site (an infinite pair force), gives MD_NONFINITE;
  * the cell grid: a position far outside the box handed to the
    reference-signature list build gives MD_CELL_OVERFLOW (the reference
    would index outside its bucket table, common/NeighborList.cpp:99-112)."""
import numpy as np
import pytest

from systems import argon_fcc

pytestmark = pytest.mark.gpu

MD_NONFINITE, MD_TIMEOUT, MD_CELL_OVERFLOW = 3, 4, 9
RS, RC = 9.534, 8.5125


def _cfg(eng, n, L=None, kernel=None, prec=None):
    kw = dict(n_lj=n, dt=2.0, lj_rs=RS, lj_rcut=RC, species=eng.SPECIES_ARGON)
    if L is not None:
        kw.update(periodic=1, box=L)
    if prec is not None:
        kw.update(precision=prec)
    if kernel is not None:
        kw.update(lj_kernel=kernel)
    return eng.make_config(**kw)


def _run(eng, cfg, pos, vel, steps):
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(steps)
        return e.download()


def _status_of(fn):
    from moleculardynamics_gb300.engine import EngineError
    with pytest.raises(EngineError) as ei:
        fn()
    return ei.value.status


@pytest.mark.parametrize("kernel", ["cluster", "rows"])
def test_wait_limit_zero_times_out_and_the_gpu_answers(eng, kernel):
    pos, vel, L = argon_fcc(6, seed=5, noise=0.1)
    k = eng.LJ_CLUSTER if kernel == "cluster" else eng.LJ_ROWS
    cfg = _cfg(eng, len(pos), L, k, eng.PREC_MIXED)
    want = _run(eng, cfg, pos, vel, 12)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        used = e.stats()["lj_cluster" if kernel == "cluster" else "lj_tma"]
        assert used == 1, f"the {kernel} kernel did not run"
        e.set_wait_limit(0)
        assert _status_of(lambda: e.step(6)) == MD_TIMEOUT
        # the same context goes on after a fresh upload with the default limit
        e.set_wait_limit(1 << 20)
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(12)
        got = e.download()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("form", ["fp64", "cluster"])
@pytest.mark.parametrize("what", ["position", "velocity", "same_site"])
def test_nonfinite_input_is_reported(eng, form, what):
    pos, vel, L = argon_fcc(6, seed=6, noise=0.1)
    if form == "fp64":
        cfg = _cfg(eng, len(pos))
    else:
        cfg = _cfg(eng, len(pos), L, eng.LJ_CLUSTER, eng.PREC_MIXED)
    bad_p, bad_v = pos.copy(), vel.copy()
    if what == "position":
        bad_p[17, 1] = np.nan
    elif what == "velocity":
        bad_v[17, 2] = np.nan
    else:
        bad_p[17, :3] = bad_p[18, :3]  # zero distance: infinite force

    def go():
        with eng.Engine(cfg) as e:
            e.upload(bad_p, bad_v)
            e.begin(0.0)
            e.step(4)

    assert _status_of(go) == MD_NONFINITE
    # the device still runs the clean system
    p, v = _run(eng, cfg, pos, vel, 4)
    assert np.isfinite(p).all() and np.isfinite(v).all()


def test_position_outside_the_cell_grid_is_reported(eng):
    sh = eng.Shim(species=eng.SPECIES_ARGON)
    pos, vel, L = argon_fcc(3, seed=7, noise=0.1)
    pos = np.ascontiguousarray(pos)
    far = pos.copy()
    far[5, 0] = 1e12  # beyond the 2^21 cells per axis the build addresses
    assert _status_of(lambda: sh.build_neighbor_list(far, RS, RC, L)) == MD_CELL_OVERFLOW
    nan = pos.copy()
    nan[5, 2] = np.nan
    assert _status_of(lambda: sh.build_neighbor_list(nan, RS, RC, L)) == MD_NONFINITE
    rows, nls, nlargest = sh.build_neighbor_list(pos, RS, RC, L)
    assert nls > 0 and (rows[:, 0] >= 0).all()
