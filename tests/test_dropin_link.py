"""The reference's cpumd program, unmodified, linked against the GPU engine.

cpu/cpumd/Host.cpp and Main.cpp plus the reference's config, loader,
results and energy files are compiled in place (same shims as
oracle/build_ref.sh); cpu/common/Device.cpp and common/NeighborList.cpp are
replaced by moleculardynamics_gb300/refshim/cpumd_device_gb300.cpp, which
forwards to libmdgb.so.  The program must link (running it needs a GPU and
the reference sources, which only exist on different machines)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import reference_source_root

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "oracle", "_ref", "shim")
ADAPTER = os.path.join(ROOT, "moleculardynamics_gb300", "refshim", "cpumd_device_gb300.cpp")


def _ref_root():
    ref = reference_source_root()
    if not os.path.isdir(SHIM) or not ref or not os.path.isdir(ref):
        pytest.skip("reference sources or oracle/_ref/shim not present")
    return ref


def _flags(REF):
    return ["-O1", "-std=gnu++14", "-w", "-DEQUI", "-I", SHIM, "-include",
            os.path.join(SHIM, "prelude.h"), "-I", os.path.join(ROOT, "include"),
            "-I", os.path.join(REF, "cpu", "common"), "-I", os.path.join(REF, "common")]


def test_cpumd_links_against_the_engine(eng, reference, tmp_path):
    REF = _ref_root()
    flags = _flags(REF)
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


class Int3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


def test_adapter_compute_bucket_is_the_reference_function(eng, reference, tmp_path):
    """The adapter's computeBucket (first hash, second hash on a collision,
    linear probe; common/NeighborList.cpp:161-207) against the reference's
    own, compiled in oracle/_ref: the same buckets for the same sequence of
    claims and look-ups, collisions included."""
    REF = _ref_root()
    so = str(tmp_path / "adapter.so")
    lib = os.path.dirname(eng.LIB_PATH)
    r = subprocess.run(["g++"] + _flags(REF) + ["-fPIC", "-shared", ADAPTER, "-o", so,
                                                "-L", lib, "-lmdgb", f"-Wl,-rpath,{lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    sym = "_Z13computeBucketiiiP4int3ib"
    ours = getattr(C.CDLL(so), sym)
    theirs = getattr(reference.lib, sym)
    for f in (ours, theirs):
        f.restype = C.c_int
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(Int3), C.c_int, C.c_bool]
    rng = np.random.default_rng(11)
    for buckets in (7, 61, 3 * 864):
        tab = [(Int3 * buckets)(), (Int3 * buckets)()]
        for t in tab:
            for b in t:
                b.x = b.y = b.z = -1
        # up to half the table in distinct cells: collisions on the small
        # tables, and an empty bucket always left (the reference's probe loop
        # only ends at an empty bucket or the cell itself); negative and large
        # coordinates exercise the wrapping products
        cells = rng.integers(-40, 400, size=(min(buckets // 2, 200), 3))
        cells[::7] *= 100000
        cells = np.unique(cells, axis=0)
        for c in cells:
            for pop in (False, True):
                a = ours(int(c[0]), int(c[1]), int(c[2]), tab[0], buckets, pop)
                b = theirs(int(c[0]), int(c[1]), int(c[2]), tab[1], buckets, pop)
                assert a == b, (buckets, c, pop)
        # look-ups of cells never claimed
        for c in rng.integers(1000, 2000, size=(50, 3)):
            a = ours(int(c[0]), int(c[1]), int(c[2]), tab[0], buckets, True)
            b = theirs(int(c[0]), int(c[1]), int(c[2]), tab[1], buckets, True)
            assert a == b
        assert [(q.x, q.y, q.z) for q in tab[0]] == [(q.x, q.y, q.z) for q in tab[1]]
