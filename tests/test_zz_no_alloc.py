"""mdgb_many_body_forces_static: bond-order forces for callers that may not
allocate GPU memory (a host application that owns all device memory through
its own pool, or a loop that cannot take an allocation's synchronisation).

The test plays such a caller: it brings its own device arrays for the inputs
and the output (allocated here by the test, as the host application would
have), calls the entry point through the C ABI twice in a row on two
different systems, on a stream the caller created, and compares each result
with the regular entry point mdgb_many_body_forces (same tolerance as the
other bond-order tests).  It also checks what the entry point exists for:
the device's free memory does not drop across the second call (the first
may load the library's code onto the device).  With ljexist = 0 the
output array starts as NaN garbage, which the call must overwrite.  This
file is collected last so that a failure here stops a -x run only after
every other test ran; it passes alone in a fresh process too."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_rms
from systems import nitrogen_diamond

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            rt = None
    assert rt is not None, "CUDA runtime not found"
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaDeviceSynchronize.argtypes = []
    rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
    rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
    rt.cudaStreamDestroy.argtypes = [C.c_void_p]
    return rt


def _free_bytes(rt):
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


class DeviceArray:
    """Device memory owned by the calling application (not by the library)."""

    def __init__(self, rt, host: np.ndarray):
        self.rt = rt
        self.nbytes = host.nbytes
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), max(self.nbytes, 1)) == 0
        assert rt.cudaMemcpy(self.ptr, host.ctypes.data, self.nbytes, 1) == 0  # host->device

    def get(self, like: np.ndarray) -> np.ndarray:
        out = np.empty_like(like)
        assert self.rt.cudaMemcpy(out.ctypes.data, self.ptr, self.nbytes, 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def _system(ncell, seed, mixed_o):
    pos, vel, _ = nitrogen_diamond(ncell, seed=seed, mixed_o=mixed_o)
    return np.ascontiguousarray(pos), vel


def test_static_scratch_entry_point_matches_the_regular_one(eng, oracle):
    lib = eng.load()
    sh = eng.Shim(species=eng.SPECIES_NEON)
    rt = _cudart()
    rcsq = oracle.settings(3.5, 3.0)[2]
    err = C.create_string_buffer(256)
    stream = C.c_void_p()
    assert rt.cudaStreamCreate(C.byref(stream)) == 0
    d_miss = DeviceArray(rt, np.full(1, -1, np.int32))
    for call, (ncell, seed, mixed_o, ljexist) in enumerate([(2, 31, True, 0), (3, 32, False, 1)]):
        pos, vel = _system(ncell, seed, mixed_o)
        n = len(pos)
        box = oracle.ready_list(pos, vel)[1]
        rows, nls, nlargest = sh.build_neighbor_list(pos, 3.5, 3.0, box)
        f0 = np.random.default_rng(seed).standard_normal((n, 3)) * 1e-3 if ljexist else None
        expect = sh.many_body_forces(pos, rows, nlargest, n, rcsq, f_init=f0,
                                     ljexist=bool(ljexist))
        d_pos = DeviceArray(rt, pos)
        d_rows = DeviceArray(rt, np.ascontiguousarray(rows, np.int32))
        # ljexist = 0 overwrites: start from garbage
        f_init = f0 if ljexist else np.full((n, 3), np.nan)
        d_f = DeviceArray(rt, np.ascontiguousarray(f_init))
        assert rt.cudaDeviceSynchronize() == 0
        free0 = _free_bytes(rt)
        s = lib.mdgb_many_body_forces_static(d_pos.ptr, d_f.ptr, n, nlargest, nls, d_rows.ptr,
                                             rcsq, ljexist, d_miss.ptr, stream, err, 256)
        assert s == 0, (call, s, err.value)
        assert rt.cudaStreamSynchronize(stream) == 0
        if call > 0:  # the first call may load the library's code on this device
            assert _free_bytes(rt) >= free0, "the call allocated device memory"
        got = d_f.get(f_init)
        missing = d_miss.get(np.zeros(1, np.int32))[0]
        for d in (d_pos, d_rows, d_f):
            d.free()
        assert np.isfinite(got).all(), call
        assert rel_rms(got, expect) < 1e-10, call
        assert missing == 0, (call, missing)
    d_miss.free()
    assert rt.cudaStreamDestroy(stream) == 0


def test_static_scratch_rejects_oversized_problems(eng):
    lib = eng.load()
    err = C.create_string_buffer(256)
    rt = _cudart()
    d = DeviceArray(rt, np.zeros(8))
    s = lib.mdgb_many_body_forces_static(d.ptr, d.ptr, 20000, 1, 1, d.ptr, 9.0, 0, None, None,
                                         err, 256)
    d.free()
    assert s == 6 and b"too large" in err.value  # MD_BAD_ARGUMENT with a message
