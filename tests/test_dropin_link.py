"""The reference's cpumd program, unmodified, linked against the GPU engine.

cpu/cpumd/Host.cpp and Main.cpp plus the reference's config, loader,
results and energy files are compiled in place (same shims as
oracle/build_ref.sh); cpu/common/Device.cpp and common/NeighborList.cpp are
replaced by moleculardynamics_gb300/refshim/cpumd_device_gb300.cpp, which
forwards to libmdgb.so.  The program must link (running it needs a GPU and
the reference sources, which only exist on different machines)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"
SHIM = os.path.join(ROOT, "oracle", "_ref", "shim")


def test_cpumd_links_against_the_engine(eng, reference, tmp_path):
    if not os.path.isdir(SHIM):
        pytest.skip("oracle/_ref/shim not built")
    flags = ["-O1", "-std=gnu++14", "-w", "-DEQUI", "-I", SHIM, "-include",
             os.path.join(SHIM, "prelude.h"), "-I", os.path.join(ROOT, "include"),
             "-I", os.path.join(REF, "cpu", "common"), "-I", os.path.join(REF, "common")]
    srcs = [os.path.join(REF, p) for p in ("cpu/cpumd/Host.cpp", "cpu/cpumd/Main.cpp",
                                           "common/Loader.cpp", "common/ConfigParser.cpp",
                                           "common/Results.cpp", "common/DebugCalculations.cpp")]
    srcs.append(os.path.join(ROOT, "moleculardynamics_gb300", "refshim",
                             "cpumd_device_gb300.cpp"))
    exe = str(tmp_path / "cpumd_gb300")
    lib = os.path.dirname(eng.LIB_PATH)
    r = subprocess.run(["g++"] + flags + srcs + ["-o", exe, "-L", lib, "-lmdgb",
                                                 f"-Wl,-rpath,{lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    syms = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    for s in ("mdgb_predict", "mdgb_correct", "mdgb_lennard_jones_forces",
              "mdgb_many_body_forces", "mdgb_build_neighbor_list"):
        assert s in syms
