"""The drop-in end to end: mdgb_run (cpumd's main + hostMain with the step
loop on the GPU engine, moleculardynamics_gb300/csrc/mdgb_run.cpp) on the
configuration and Input that the reference's own cpumd ran
(tests/golden/make_dropin_golden.py: cpu/cpumd/Main.cpp + Host.cpp compiled
unmodified, argon in the NG slot), writes the same files byte for byte:

* the Output text file (common/Loader.cpp:88-120) after the last pass;
* the Filename(vxcm-V).dat/.txt results of both vxcm passes
  (common/Results.cpp:120-229), the .txt with its "Time took" line masked
  (wall-clock time);
* the AnimationData(vxcm-V).anm frames of both passes
  (common/Results.cpp:51-86).

The records are computed with ReferenceEnergy = 2: the reference's all-pairs
energy (common/DebugCalculations.cpp:129-270) with every sum in the
reference's order on the device, so their doubles are the reference's."""
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "dropin")


def _mask_time(b: bytes) -> bytes:
    return b"\n".join(b"VXCM <masked>" if b": Time took: " in line else line
                      for line in b.split(b"\n"))


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def test_mdgb_run_writes_the_reference_files(eng, tmp_path):
    from moleculardynamics_gb300 import build
    from golden.make_dropin_golden import input_text
    with open(os.path.join(GOLD, "manifest.json")) as f:
        man = json.load(f)
    data = np.load(os.path.join(GOLD, "dropin_input.npz"))
    shutil.copy(os.path.join(GOLD, man["config"]), tmp_path)
    (tmp_path / "input.txt").write_text(input_text(data["pos"], data["vel"]))
    r = subprocess.run([build.RUN, man["config"]], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    for name in man["files"]:
        with open(os.path.join(GOLD, name), "rb") as f:
            want = f.read()
        got = (tmp_path / name).read_bytes()
        if name.endswith(".txt"):
            want, got = _mask_time(want), _mask_time(got)
        assert got == want, name
    for name, digest in man["sha256"].items():
        assert _sha(tmp_path / name) == digest, name


def _tokens_close(want: str, got: str, rtol: float = 2e-7):
    """Equal token by token: numbers within rtol (the last printed digit),
    everything else exactly."""
    tw, tg = want.split(), got.split()
    assert len(tw) == len(tg)
    for a, b in zip(tw, tg):
        try:
            x, y = float(a), float(b)
        except ValueError:
            assert a == b
            continue
        assert abs(x - y) <= rtol * max(abs(x), 1e-30) or a == b, (a, b)


@pytest.mark.parametrize("case", ["dropin_bo", "dropin_mixed"])
def test_mdgb_run_bond_order_matches_the_reference(eng, tmp_path, case):
    """The bond-order half, alone (dropin_bo: 64 N and O atoms) and beside
    108 neon atoms with LJ on (dropin_mixed), in the reference's walls for 200
    steps; fixtures made by the unmodified cpumd with the reference's
    constants.  The reference's exp and tanh (libm) and CUDA's differ in the
    last bits, so the records' doubles (.dat) are compared within 1e-10
    (measured 3e-13 for dropin_bo); the .dat header, the printed records, the
    N-O pair list and the final state (.txt, Output) match to their printed
    digits."""
    from moleculardynamics_gb300 import build
    from golden.make_dropin_golden import input_text
    gold = os.path.join(HERE, "golden", case)
    with open(os.path.join(gold, "manifest.json")) as f:
        man = json.load(f)
    data = np.load(os.path.join(gold, "dropin_input.npz"))
    shutil.copy(os.path.join(gold, man["config"]), tmp_path)
    (tmp_path / "input.txt").write_text(input_text(data["pos"], data["vel"]))
    r = subprocess.run([build.RUN, man["config"]], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    # .dat: the header (particles, steps, dt, two flags each with rs and rcut
    # when set, vxcm) exact, then records of 11 doubles
    want = open(os.path.join(gold, "results(vxcm-0).dat"), "rb").read()
    got = (tmp_path / "results(vxcm-0).dat").read_bytes()
    head = len(want) - 88 * ((len(want) - 14) // 88)
    assert got[:head] == want[:head] and len(got) == len(want)
    rw = np.frombuffer(want[head:], np.float64).reshape(-1, 11)
    rg = np.frombuffer(got[head:], np.float64).reshape(-1, 11)
    assert np.all(np.abs(rg - rw) <= 1e-10 * np.maximum(np.abs(rw), 1e-12))
    _tokens_close(_mask_time(open(os.path.join(gold, "results(vxcm-0).txt"), "rb").read()).decode(),
                  _mask_time((tmp_path / "results(vxcm-0).txt").read_bytes()).decode())
    _tokens_close(open(os.path.join(gold, "output.txt")).read(),
                  (tmp_path / "output.txt").read_text())
