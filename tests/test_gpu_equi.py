"""equi's initial velocities on the device (md_choose_velocities) against the
C restatement of the reference (oracle/mdoracle.c orc_choose_velocities,
bit-exact to the reference compiled in place: tests/test_equi_pinned.py), fed
the device generator's uniforms (oracle/equi_ref.py):

* argon systems in both precisions (the cluster path stores atoms in cell
  order; the draws follow the caller's numbering): velocities within 1e-12
  relative.  The device runs the reference's inverf step for step (its own
  erf/erfc series, no FMA contraction); what differs is CUDA's exp, log and
  sqrt against the host's, and parallel against sequential momentum sums;
* a many-body + LJ system: the N-O pairs share one draw, the momentum sums
  count a pair once, and the result matches the restatement;
* pure many-body systems: O-N pairs only match the restatement; O-N and
  N-O pairs in turn, where the reference's removal loop never ends: an
  error, not a hang;
* equi's schedule (new velocities after every 50th step) as the same calls
  made by hand, bit-identical, and the temperature right after a
  reassignment.
"""
import numpy as np
import pytest

from oracle import equi_ref
from systems import argon_fcc, mixed_system, nitrogen_diamond

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def _close(a, b):
    scale = np.abs(b).max()
    return np.abs(a - b).max() <= 1e-12 * scale


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_argon_velocities_match_the_restatement(eng, precision):
    pos, vel, L = argon_fcc(6, noise=0.05)
    prec = eng.PREC_FP64 if precision == "fp64" else eng.PREC_MIXED
    cfg = eng.make_config(n_lj=len(pos), dt=2.0, lj_rs=9.534, lj_rcut=8.5125, periodic=1, box=L,
                          species=eng.SPECIES_ARGON, precision=prec)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        e.choose_velocities(94.4, SEED)
        _, v = e.download()
    ref, shifts = equi_ref.choose_velocities(pos, 0, 94.4, SEED, "argon")
    assert ref is not None and shifts <= 3
    assert _close(v, ref)
    m = equi_ref.masses("argon")[2]
    assert np.abs((m * v).sum(0)).max() < 1e-13 * m * np.abs(v).sum()
    t = m * (v * v).sum() / (3 * len(v))
    assert abs(t - 94.4 * equi_ref.RB) < 1e-12 * t


def test_many_body_pairs_share_a_draw(eng):
    pos, vel, n_mb, n_lj = mixed_system(seed=9)
    cfg = eng.make_config(n_lj=n_lj, n_mb=n_mb, dt=0.5, use_lj=1, use_mb=1, lj_rs=9.0,
                          lj_rcut=8.0, mb_rs=3.5, mb_rcut=3.0, species=eng.SPECIES_NEON)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.choose_velocities(300.0, SEED + 1)
        _, v = e.download()
    ref, shifts = equi_ref.choose_velocities(pos, n_mb, 300.0, SEED + 1, "neon")
    assert ref is not None and shifts > 3  # the pairs' masses slow the removal down
    assert np.array_equal(v[0:n_mb:2], v[1:n_mb:2])
    assert _close(v, ref)


def test_pure_many_body_systems(eng):
    """O-N pairs only: the first shift removes the momentum (every pair has
    the same masses).  Pairs O-N and N-O in turn: after the first shift each
    further one overshoots by exactly as much as it corrects, and the
    reference's loop never ends; the device version reports it."""
    for pattern in ("same", "alternating"):
        pos, vel, _ = nitrogen_diamond(3, mixed_o=True)
        if pattern == "alternating":
            pos[:, 3] = np.tile([1, 0, 0, 1], len(pos) // 4)
        n = len(pos)
        ref, shifts = equi_ref.choose_velocities(pos, n, 300.0, SEED, "neon")
        cfg = eng.make_config(n_mb=n, use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5)
        with eng.Engine(cfg) as e:
            e.upload(pos, vel)
            if pattern == "same":
                assert ref is not None
                e.choose_velocities(300.0, SEED)
                _, v = e.download()
                assert np.array_equal(v[0::2], v[1::2])
                assert _close(v, ref)
            else:
                assert ref is None
                with pytest.raises(eng.EngineError):
                    e.choose_velocities(300.0, SEED)


def test_equilibration_schedule(eng):
    pos, vel, L = argon_fcc(6, noise=0.05)
    cfg = eng.make_config(n_lj=len(pos), dt=2.0, lj_rs=9.534, lj_rcut=8.5125, periodic=1, box=L,
                          species=eng.SPECIES_ARGON, precision=eng.PREC_MIXED)
    gamma = 0x632BE59BD9B4E019
    with eng.Engine(cfg) as a:
        a.upload(pos, vel)
        a.begin(0.0)
        a.set_equilibration(60.0, SEED, 50)
        a.step(51)  # new velocities after steps 0 and 50
        th = a.thermo_now()
        pa, va = a.download()
    with eng.Engine(cfg) as b:
        b.upload(pos, vel)
        b.begin(0.0)
        b.step(1)
        b.choose_velocities(60.0, (SEED + gamma) % (1 << 64))
        b.step(50)
        b.choose_velocities(60.0, (SEED + 2 * gamma) % (1 << 64))
        pb, vb = b.download()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    # the reference's temperature (float kB) of the rescaled velocities
    assert abs(th["temperature"] - 60.0) < 1e-6 * 60.0
