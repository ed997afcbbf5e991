"""Run outputs on the device (common/Results.cpp):

* tailResults: the many-body pair list computed on the GPU equals the one in
  the reference's own result file for the same positions (golden fixture),
  and the result files written from it are byte-identical to the reference's;
* animation frames (pushAnim / writeAnimationBinaryData): each frame is the
  float conversion of the state at its step, frames follow the reference's
  schedule (the state before the first step, then every `every` steps; a
  second frame at step 0 for every = 0), the .anm file has the reference's
  layout, and capturing frames leaves the trajectory bit-identical.
"""
import os
import struct

import numpy as np
import pytest

from moleculardynamics_gb300 import lattice as lat
from systems import argon_fcc

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_pairs(txt: str) -> np.ndarray:
    tail = txt.split("ManyBody Pairs:\n", 1)[1]
    amount, rest = tail.split("\n", 1)
    n = int(amount.split(":")[1])
    items = [s for s in rest.strip().split("] ") if s]
    pairs = np.array([[int(v) for v in s.strip("[] ").split(",")] for s in items], np.int32)
    assert len(pairs) == n
    return pairs.reshape(-1, 2)


def test_tail_pairs_match_the_reference_file(eng, tmp_path):
    import ctypes as C
    gold = np.load(os.path.join(GOLD, "reference_fixtures.npz"))
    pos = np.ascontiguousarray(gold["bo_no/pos"])
    n = len(pos)
    cfg = eng.make_config(n_lj=0, n_mb=n, dt=2.0, timesteps=200, lj_rs=9.0, lj_rcut=8.0,
                          use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0)
    with eng.Engine(cfg) as e:
        e.upload(pos, np.zeros((n, 3)))
        pairs = e.tail_pairs()
    ref_txt = open(os.path.join(GOLD, "results_vxcm-0.5.txt")).read()
    assert np.array_equal(pairs, _golden_pairs(ref_txt))
    recs = np.load(os.path.join(GOLD, "results_records.npy"))
    th = np.zeros((3, 16))
    th[:, :11] = recs
    th = np.ascontiguousarray(th)
    flat = np.ascontiguousarray(pairs.ravel())
    stem = str(tmp_path / "res")
    L = eng.load()
    s = L.md_write_results_pairs(stem.encode(), C.byref(cfg), 0.5, 123.0, th.ctypes.data, 3,
                                 flat.ctypes.data, len(pairs))
    assert s == 0
    for ext in ("dat", "txt"):
        mine = open(f"{stem}(vxcm-0.5).{ext}", "rb").read()
        ref = open(os.path.join(GOLD, f"results_vxcm-0.5.{ext}"), "rb").read()
        assert mine == ref, ext


def test_tail_pairs_larger_system_against_numpy(eng):
    """4,096 atoms of alternating N and O on a diamond lattice (1.5 A bonds):
    the GPU pair list equals a numpy restatement of tailResults."""
    pos, vel, _ = lat.make_system("diamond", 8, 300.0, seed=5, a=4 * 1.5 / np.sqrt(3),
                                  noise=0.05, species=lat.SPECIES_N, mass_table="neon")
    pos[::2, 3] = lat.SPECIES_O
    n = len(pos)
    cfg = eng.make_config(n_mb=n, use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        pairs = e.tail_pairs()
    ref = []
    x = pos[:, :3]
    t = pos[:, 3].astype(int)
    lim = float(np.float32(2) * np.float32(1.15))
    for i in range(n - 1):
        d = x[i] - x[i + 1:]
        dist = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        js = np.nonzero((dist < lim) & (t[i + 1:] != t[i]))[0] + i + 1
        ref.extend((i, j) for j in js)
    ref = np.array(ref, np.int32).reshape(-1, 2)
    assert len(ref) > n // 2  # many bonded neighbours of the other species
    assert np.array_equal(pairs, ref)


def _argon(eng, n_cells=6, **kw):
    pos, vel, L = argon_fcc(n_cells, noise=0.05)
    cfg = eng.make_config(n_lj=len(pos), dt=2.0, lj_rs=9.534, lj_rcut=8.5125, periodic=1,
                          box=L, species=eng.SPECIES_ARGON, **kw)
    return pos, vel, cfg


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_animation_frames_are_the_state(eng, precision):
    prec = eng.PREC_FP64 if precision == "fp64" else eng.PREC_MIXED
    pos, vel, cfg = _argon(eng, precision=prec)
    with eng.Engine(cfg) as e:
        e.set_animation(5, 8)
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(20)
        frames = [e.animation_frame(k) for k in range(e.animation_count())]
    # the state before the first step, then after the steps 5, 10 and 15
    assert len(frames) == 4
    for k, done in enumerate([0, 6, 11, 16]):
        with eng.Engine(cfg) as e:
            e.upload(pos, vel)
            e.begin(0.0)
            if done:
                e.step(done)
            p, v = e.download()
        assert np.array_equal(frames[k][0], p.astype(np.float32)), k
        assert np.array_equal(frames[k][1], v.astype(np.float32)), k


def test_animation_every_zero_and_off(eng):
    pos, vel, cfg = _argon(eng, precision=eng.PREC_MIXED)
    with eng.Engine(cfg) as e:
        e.set_animation(0)
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(12)
        assert e.animation_count() == 2  # cpu/cpumd/Host.cpp:126 and :188 at step 0
        e.set_animation(-1)
        e.begin(0.0)
        e.step(5)
        assert e.animation_count() == 0


def test_animation_leaves_the_trajectory_unchanged(eng):
    pos, vel, cfg = _argon(eng, precision=eng.PREC_MIXED)
    out = []
    for every in (-1, 7):
        with eng.Engine(cfg) as e:
            if every >= 0:
                e.set_animation(every, 2)  # outgrows the first pinned block
            e.upload(pos, vel)
            e.begin(0.0)
            e.step(60)
            out.append(e.download())
            if every >= 0:
                assert e.animation_count() == 1 + 60 // 7
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_animation_file_layout(eng, tmp_path):
    """common/Results.cpp:51-86: atoms, animation steps, frames; every
    frame's positions (4 floats per atom), then every frame's velocities."""
    pos, vel, cfg = _argon(eng, n_cells=4, precision=eng.PREC_FP64)
    stem = str(tmp_path / "anim")
    with eng.Engine(cfg) as e:
        e.set_animation(3)
        e.upload(pos, vel)
        e.begin(0.0)
        e.step(10)
        frames = [e.animation_frame(k) for k in range(e.animation_count())]
        e.write_animation(stem, 0.25)
    n = len(pos)
    want = struct.pack("<3i", n, 3, len(frames))
    want += b"".join(f[0].astype("<f4").tobytes() for f in frames)
    want += b"".join(f[1].astype("<f4").tobytes() for f in frames)
    assert open(f"{stem}(vxcm-0.25).anm", "rb").read() == want
