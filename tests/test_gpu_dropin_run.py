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
