"""Python binding of the engine's C ABI (include/mdgb.h) over ctypes.

This mirrors the two C layers for tests and benchmarks:

* ``Engine``: the device-resident step engine (md_create / md_upload /
  md_begin / md_step / md_download ...), the drop-in for the step loop of
  cpu/cpumd/Host.cpp;
* ``Shim``: the reference-signature functions (mdgb_predict, mdgb_correct,
  mdgb_lennard_jones_forces, ...) with the reference's arguments.

There is no CPU fallback: loading fails with an error when libmdgb.so has
not been built (``moleculardynamics_gb300.build.build()``), and every call
that fails on the device raises ``EngineError``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libmdgb.so")

PREC_FP64, PREC_MIXED = 0, 1
LJ_AUTO, LJ_ROWS, LJ_CLUSTER = 0, 1, 2
SPECIES_NEON, SPECIES_ARGON = 0, 1
(KERNEL_LJ, KERNEL_MB, KERNEL_PREDICT, KERNEL_CORRECT, KERNEL_LIST, KERNEL_STEP,
 KERNEL_FUSED, KERNEL_FUSED_CORRECT) = range(8)


class EngineError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (md_status {status})")
        self.status = status


class MdConfig(C.Structure):
    _fields_ = [("n_lj", C.c_int), ("n_mb", C.c_int), ("dt", C.c_float), ("timesteps", C.c_int),
                ("lj_rs", C.c_float), ("lj_rcut", C.c_float), ("mb_rs", C.c_float),
                ("mb_rcut", C.c_float), ("use_lj", C.c_int), ("use_mb", C.c_int),
                ("output_timesteps", C.c_int), ("energy_loss", C.c_float), ("periodic", C.c_int),
                ("box", C.c_double), ("precision", C.c_int), ("species", C.c_int),
                ("device", C.c_int), ("reference_energy", C.c_int), ("lj_kernel", C.c_int),
                ("cluster_cells", C.c_int), ("cluster_threads", C.c_int),
                ("cluster_row_loads", C.c_int), ("cluster_stage_cap", C.c_int)]


THERMO_FIELDS = ["time", "temperature", "e", "ek", "eu", "com_x", "com_y", "com_z",
                 "momentum_x", "momentum_y", "momentum_z", "e_lj", "e_lj_shifted", "e_mb",
                 "virial", "step"]


class MdThermo(C.Structure):
    _fields_ = [(k, C.c_double) for k in THERMO_FIELDS]


class MdStats(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("list_builds", C.c_longlong),
                ("list_trips", C.c_longlong), ("wall_hits", C.c_longlong),
                ("missing_xi", C.c_longlong), ("launches", C.c_longlong),
                ("lj_max_row", C.c_int), ("lj_nlargest", C.c_int), ("mb_nlargest", C.c_int),
                ("lj_cells", C.c_int), ("mb_cells", C.c_int), ("lj_list_entries", C.c_longlong),
                ("lj_tma", C.c_int), ("lj_cluster", C.c_int), ("cluster_segments", C.c_int),
                ("cluster_max_staged", C.c_int)]


class MdTuneResult(C.Structure):
    _fields_ = [("threads", C.c_int), ("stage_cap", C.c_int), ("row_loads", C.c_int),
                ("candidates", C.c_int), ("best_ms", C.c_double)]


class MdSurrogateStats(C.Structure):
    _fields_ = [("surrogate_steps", C.c_longlong), ("exact_steps", C.c_longlong),
                ("checks", C.c_longlong), ("rejected_checks", C.c_longlong),
                ("last_error", C.c_double), ("max_error", C.c_double),
                ("declined_steps", C.c_longlong)]


class ListSettings(C.Structure):
    _fields_ = [("maxnlmove", C.c_float), ("maxnlmovesq", C.c_float), ("rcut", C.c_float),
                ("rs", C.c_float), ("rcutsq", C.c_float), ("nlistsize", C.c_int),
                ("nlargestsize", C.c_int)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_lib = None

# every exported symbol of include/mdgb.h
EXPORTS = ["md_create", "md_destroy", "md_status_string", "md_last_error", "md_upload",
           "md_upload_state", "md_download", "md_download_state", "md_begin", "md_step",
           "md_record_count", "md_get_records", "md_thermo_now", "md_reference_potential",
           "md_compute_forces", "md_neighbor_list", "md_get_stats", "md_set_timing",
           "md_kernel_time", "md_synchronize", "mdgb_predict", "mdgb_correct",
           "mdgb_lennard_jones_forces", "mdgb_many_body_forces", "mdgb_calculate_accelerations",
           "mdgb_build_neighbor_list", "mdgb_free", "mdgb_perform_calculations",
           "mdgb_calculate_potential", "mdgb_set_species", "mdgb_last_status", "md_read_config",
           "md_write_results", "md_write_results_pairs", "md_host_alloc", "md_host_free",
           "md_set_animation", "md_animation_count", "md_get_animation_frame",
           "md_write_animation", "md_tail_pairs", "md_choose_velocities",
           "md_set_equilibration",
           "mdgb_many_body_forces_static", "md_autotune", "md_set_graphs", "md_batch_create",
           "md_batch_size", "md_batch_records", "mdgb_tc_selftest", "mdgb_conv_selftest",
           "md_surrogate_create",
           "md_surrogate_destroy", "md_surrogate_param_count", "md_surrogate_collect",
           "md_surrogate_samples", "md_surrogate_train", "md_surrogate_attach",
           "md_surrogate_report", "md_surrogate_forces", "md_surrogate_descriptors",
           "md_surrogate_params", "md_surrogate_normalisation", "md_surrogate_loss_grad",
           "md_surrogate_net", "md_surrogate_train_forces", "md_surrogate_force_grad",
           "md_surrogate_desc_directional", "md_set_wait_limit", "md_measure_arith_peaks",
           "md_device_sm_count", "md_surrogate_set_model", "md_surrogate_head_param_count",
           "md_surrogate_head_params", "md_surrogate_head_grad", "md_surrogate_head_scale",
           "md_surrogate_range"]


def load(path: str | None = None) -> C.CDLL:
    """Loads libmdgb.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} not built: run moleculardynamics_gb300.build.build()")
    L = C.CDLL(p)
    P = C.POINTER
    L.md_create.argtypes = [P(MdConfig), P(C.c_void_p)]
    L.md_destroy.argtypes = [C.c_void_p]
    L.md_status_string.restype = C.c_char_p
    L.md_status_string.argtypes = [C.c_int]
    L.md_last_error.restype = C.c_char_p
    L.md_last_error.argtypes = [C.c_void_p]
    L.md_upload.argtypes = [C.c_void_p, _dp, _dp]
    L.md_upload_state.argtypes = [C.c_void_p] + [C.c_void_p] * 5
    L.md_download.argtypes = [C.c_void_p, _dp, _dp]
    L.md_download_state.argtypes = [C.c_void_p] + [C.c_void_p] * 4
    L.md_begin.argtypes = [C.c_void_p, C.c_float]
    L.md_step.argtypes = [C.c_void_p, C.c_int]
    L.md_record_count.argtypes = [C.c_void_p]
    L.md_get_records.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.md_thermo_now.argtypes = [C.c_void_p, P(MdThermo)]
    L.md_reference_potential.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
    L.md_compute_forces.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.md_neighbor_list.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_longlong,
                                   P(C.c_int), P(C.c_int)]
    L.md_get_stats.argtypes = [C.c_void_p, P(MdStats)]
    L.md_set_timing.argtypes = [C.c_void_p, C.c_int]
    L.md_kernel_time.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(C.c_longlong)]
    L.md_synchronize.argtypes = [C.c_void_p]
    L.md_autotune.argtypes = [C.c_void_p, C.c_int, P(MdTuneResult)]
    L.md_set_graphs.argtypes = [C.c_void_p, C.c_int]
    L.md_set_wait_limit.argtypes = [C.c_void_p, C.c_int]
    L.md_measure_arith_peaks.argtypes = [C.c_int, P(C.c_double), P(C.c_double)]
    L.md_device_sm_count.argtypes = [C.c_int, P(C.c_int)]
    L.mdgb_tc_selftest.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int]
    L.mdgb_conv_selftest.argtypes = [_fp, _dp, C.c_int, _dp, _dp, _fp, _fp]
    L.md_surrogate_create.argtypes = [C.c_int, C.c_ulonglong, C.c_float, P(C.c_void_p)]
    L.md_surrogate_destroy.argtypes = [C.c_void_p]
    L.md_surrogate_param_count.restype = C.c_int
    L.md_surrogate_collect.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, P(C.c_int)]
    L.md_surrogate_samples.argtypes = [C.c_void_p, P(C.c_int)]
    L.md_surrogate_train.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, P(C.c_double)]
    L.md_surrogate_attach.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int]
    L.md_surrogate_report.argtypes = [C.c_void_p, P(MdSurrogateStats)]
    L.md_surrogate_forces.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, P(C.c_double)]
    L.md_surrogate_descriptors.argtypes = [C.c_void_p, C.c_void_p, _fp, C.c_int]
    L.md_surrogate_desc_directional.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp]
    L.md_surrogate_params.argtypes = [C.c_void_p, _fp, C.c_int]
    L.md_surrogate_normalisation.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_int]
    L.md_surrogate_loss_grad.argtypes = [C.c_void_p, _fp, _fp, C.c_int, _fp, P(C.c_double)]
    L.md_surrogate_net.argtypes = [C.c_void_p, _fp, C.c_int, _fp, _fp]
    L.md_surrogate_train_forces.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float,
                                            C.c_float, P(C.c_double), P(C.c_double)]
    L.md_surrogate_force_grad.argtypes = [C.c_void_p, _fp, _fp, C.c_int, _fp]
    L.md_surrogate_set_model.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.md_surrogate_head_param_count.argtypes = [C.c_int]
    L.md_surrogate_head_params.argtypes = [C.c_void_p, _fp, C.c_int, C.c_int]
    L.md_surrogate_head_grad.argtypes = [C.c_void_p, _fp, _fp, C.c_int, _fp]
    L.md_surrogate_head_scale.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int]
    L.md_surrogate_range.argtypes = [C.c_void_p, _fp, _fp, C.c_int]
    L.md_batch_create.argtypes = [P(MdConfig), C.c_int, _ip, _dp, P(C.c_void_p)]
    L.md_batch_size.argtypes = [C.c_void_p]
    L.md_batch_records.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.md_host_alloc.restype = C.c_void_p
    L.md_host_alloc.argtypes = [C.c_size_t]
    L.md_host_free.argtypes = [C.c_void_p]
    L.mdgb_predict.argtypes = [_dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int]
    L.mdgb_correct.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_double,
                               P(C.c_int), C.c_float]
    L.mdgb_lennard_jones_forces.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, _ip, C.c_double]
    L.mdgb_many_body_forces.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, _ip, C.c_double,
                                        C.c_int]
    L.mdgb_calculate_accelerations.argtypes = [_dp, _dp, _dp, C.c_int]
    L.mdgb_build_neighbor_list.restype = P(C.c_int)
    L.mdgb_build_neighbor_list.argtypes = [_dp, P(ListSettings), C.c_double, C.c_int, C.c_int]
    L.mdgb_free.argtypes = [C.c_void_p]
    L.mdgb_perform_calculations.argtypes = [_dp, _dp, C.c_int] + [P(C.c_double)] * 8
    L.mdgb_calculate_potential.argtypes = [_dp, P(C.c_double), P(C.c_double), C.c_int]
    L.mdgb_set_species.argtypes = [C.c_int]
    L.mdgb_many_body_forces_static.restype = C.c_int
    L.mdgb_many_body_forces_static.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                               C.c_int, C.c_void_p, C.c_double, C.c_int,
                                               C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    L.mdgb_last_status.restype = C.c_int
    L.md_read_config.argtypes = [C.c_char_p, P(MdConfig), C.c_char_p, P(C.c_double),
                                 C.c_char_p, C.c_int]
    L.md_write_results.argtypes = [C.c_char_p, P(MdConfig), C.c_float, C.c_float,
                                   C.c_void_p, C.c_int, C.c_void_p]
    L.md_write_results_pairs.argtypes = [C.c_char_p, P(MdConfig), C.c_float, C.c_float,
                                         C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    L.md_set_animation.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.md_animation_count.restype = C.c_int
    L.md_animation_count.argtypes = [C.c_void_p]
    L.md_get_animation_frame.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.md_write_animation.argtypes = [C.c_void_p, C.c_char_p, C.c_float]
    L.md_tail_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_int, P(C.c_int)]
    L.md_choose_velocities.argtypes = [C.c_void_p, C.c_double, C.c_ulonglong]
    L.md_set_equilibration.argtypes = [C.c_void_p, C.c_double, C.c_ulonglong, C.c_int]
    if path is None:
        _lib = L
    return L


def make_config(n_lj=0, n_mb=0, dt=2.0, timesteps=0, lj_rs=9.534, lj_rcut=8.5125, mb_rs=3.5,
                mb_rcut=3.0, use_lj=1, use_mb=0, output_timesteps=0, energy_loss=1.0,
                periodic=0, box=0.0, precision=PREC_FP64, species=SPECIES_ARGON, device=0,
                reference_energy=0, lj_kernel=0, cluster_cells=0,
                cluster_threads=0, cluster_row_loads=0, cluster_stage_cap=0) -> MdConfig:
    return MdConfig(n_lj, n_mb, dt, timesteps, lj_rs, lj_rcut, mb_rs, mb_rcut, use_lj, use_mb,
                    output_timesteps, energy_loss, periodic, box, precision, species, device,
                    reference_energy, lj_kernel, cluster_cells, cluster_threads,
                    cluster_row_loads, cluster_stage_cap)


class Engine:
    """One md_ctx: a system on the GPU, stepped by the engine."""

    def __init__(self, cfg: MdConfig):
        self.lib = load()
        self.cfg = cfg
        self.n = cfg.n_lj + cfg.n_mb
        h = C.c_void_p()
        s = self.lib.md_create(C.byref(cfg), C.byref(h))
        if s != 0:
            raise EngineError(s, "md_create: " + self.lib.md_status_string(s).decode())
        self.h = h

    def _ck(self, s: int, what: str):
        if s != 0:
            raise EngineError(s, f"{what}: {self.lib.md_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.md_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, pos4: np.ndarray, vel3: np.ndarray):
        self._ck(self.lib.md_upload(self.h, np.ascontiguousarray(pos4, np.float64),
                                    np.ascontiguousarray(vel3, np.float64)), "md_upload")

    def upload_state(self, pos4, vel3, acc=None, b=None, c=None):
        keep = [np.ascontiguousarray(x, np.float64) if x is not None else None
                for x in (pos4, vel3, acc, b, c)]
        ptrs = [x.ctypes.data if x is not None else None for x in keep]
        self._ck(self.lib.md_upload_state(self.h, *ptrs), "md_upload_state")

    def download(self):
        pos = np.zeros((self.n, 4))
        vel = np.zeros((self.n, 3))
        self._ck(self.lib.md_download(self.h, pos, vel), "md_download")
        return pos, vel

    def download_state(self):
        arrs = [np.zeros((self.n, 3)) for _ in range(4)]
        self._ck(self.lib.md_download_state(self.h, *[a.ctypes.data for a in arrs]),
                 "md_download_state")
        return dict(acc=arrs[0], b=arrs[1], c=arrs[2], force=arrs[3])

    def begin(self, vxcm: float = 0.0):
        self._ck(self.lib.md_begin(self.h, vxcm), "md_begin")

    def step(self, nsteps: int):
        self._ck(self.lib.md_step(self.h, nsteps), "md_step")

    def records(self) -> np.ndarray:
        n = self.lib.md_record_count(self.h)
        out = (MdThermo * max(n, 1))()
        self._ck(self.lib.md_get_records(self.h, out, n), "md_get_records")
        return np.array([[getattr(r, k) for k in THERMO_FIELDS] for r in out[:n]]).reshape(n, 16)

    def thermo_now(self) -> dict:
        t = MdThermo()
        self._ck(self.lib.md_thermo_now(self.h, C.byref(t)), "md_thermo_now")
        return {k: getattr(t, k) for k in THERMO_FIELDS}

    def reference_potential(self):
        a, b = C.c_double(), C.c_double()
        self._ck(self.lib.md_reference_potential(self.h, C.byref(a), C.byref(b)),
                 "md_reference_potential")
        return a.value, b.value

    def compute_forces(self):
        f = np.zeros((self.n, 3))
        e = np.zeros(5)
        self._ck(self.lib.md_compute_forces(self.h, f.ctypes.data, e.ctypes.data),
                 "md_compute_forces")
        return f, e

    def neighbor_list(self, which: int = 0, images: bool = False):
        nls, nl = C.c_int(), C.c_int()
        self._ck(self.lib.md_neighbor_list(self.h, which, None, None, 0, C.byref(nls),
                                           C.byref(nl)), "md_neighbor_list")
        rows_n = self.cfg.n_mb if which == 1 else self.n
        rows = np.zeros((rows_n, nls.value), np.int32)
        img = np.zeros((rows_n, nls.value), np.int8) if images else None
        self._ck(self.lib.md_neighbor_list(self.h, which, rows.ctypes.data,
                                           img.ctypes.data if images else None, rows.size,
                                           C.byref(nls), C.byref(nl)), "md_neighbor_list")
        return (rows, nls.value, nl.value) + ((img,) if images else ())

    def stats(self) -> dict:
        s = MdStats()
        self._ck(self.lib.md_get_stats(self.h, C.byref(s)), "md_get_stats")
        return {k: getattr(s, k) for k, _ in MdStats._fields_}

    def autotune(self, evals: int = 3) -> dict:
        r = MdTuneResult()
        self._ck(self.lib.md_autotune(self.h, evals, C.byref(r)), "md_autotune")
        return {k: getattr(r, k) for k, _ in MdTuneResult._fields_}

    def set_timing(self, on: bool):
        self._ck(self.lib.md_set_timing(self.h, int(on)), "md_set_timing")

    def kernel_time(self, kernel: int):
        ms, n = C.c_double(), C.c_longlong()
        self._ck(self.lib.md_kernel_time(self.h, kernel, C.byref(ms), C.byref(n)),
                 "md_kernel_time")
        return ms.value, n.value

    def synchronize(self):
        self._ck(self.lib.md_synchronize(self.h), "md_synchronize")

    def set_wait_limit(self, tries: int):
        self._ck(self.lib.md_set_wait_limit(self.h, int(tries)), "md_set_wait_limit")

    def set_graphs(self, on: bool):
        self._ck(self.lib.md_set_graphs(self.h, int(on)), "md_set_graphs")

    def set_animation(self, every: int, frames_hint: int = 0):
        """Animation frames every `every` steps from md_begin on (-1: off)."""
        self._ck(self.lib.md_set_animation(self.h, every, frames_hint), "md_set_animation")

    def animation_count(self) -> int:
        return self.lib.md_animation_count(self.h)

    def animation_frame(self, k: int):
        """(positions n x 4 float32, velocities n x 3 float32) of frame k."""
        p = np.zeros((self.n, 4), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        self._ck(self.lib.md_get_animation_frame(self.h, k, p.ctypes.data, v.ctypes.data),
                 "md_get_animation_frame")
        return p, v

    def write_animation(self, anim_file: str, vxcm: float = 0.0):
        self._ck(self.lib.md_write_animation(self.h, anim_file.encode(), vxcm),
                 "md_write_animation")

    def choose_velocities(self, temperature: float, seed: int):
        """equi's chooseVelocities on the device state (kelvin)."""
        self._ck(self.lib.md_choose_velocities(self.h, temperature, seed),
                 "md_choose_velocities")

    def set_equilibration(self, temperature: float, seed: int, every: int = 50):
        self._ck(self.lib.md_set_equilibration(self.h, temperature, seed, every),
                 "md_set_equilibration")

    def tail_pairs(self) -> np.ndarray:
        """Many-body pairs closer than 2 reNO (k x 2, the reference's order)."""
        cnt = C.c_int(0)
        self._ck(self.lib.md_tail_pairs(self.h, None, 0, C.byref(cnt)), "md_tail_pairs")
        out = np.zeros((max(cnt.value, 1), 2), np.int32)
        if cnt.value:
            self._ck(self.lib.md_tail_pairs(self.h, out.ctypes.data, cnt.value, C.byref(cnt)),
                     "md_tail_pairs")
        return out[:cnt.value]


class Surrogate:
    """Learned surrogate of the bond-order term (md_surrogate_*)."""

    def __init__(self, seed: int = 1, cutoff: float = 3.0, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        s = self.lib.md_surrogate_create(device, seed, cutoff, C.byref(h))
        if s != 0:
            raise EngineError(s, "md_surrogate_create")
        self.h = h
        self.nparams = self.lib.md_surrogate_param_count()
        self.kind, self.hidden = 0, 64

    def close(self):
        if getattr(self, "h", None):
            self.lib.md_surrogate_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, s, what):
        if s != 0:
            raise EngineError(s, what)

    def collect(self, e: "Engine", stride: int = 1, offset: int = 0) -> int:
        n = C.c_int()
        s = self.lib.md_surrogate_collect(self.h, e.h, stride, offset, C.byref(n))
        if s != 0:
            raise EngineError(s, "md_surrogate_collect: " + self.lib.md_last_error(e.h).decode())
        return n.value

    def samples(self) -> int:
        n = C.c_int()
        self._ck(self.lib.md_surrogate_samples(self.h, C.byref(n)), "md_surrogate_samples")
        return n.value

    def train(self, steps: int, batch: int = 1024, lr: float = 1e-3) -> float:
        loss = C.c_double()
        self._ck(self.lib.md_surrogate_train(self.h, steps, batch, lr, C.byref(loss)),
                 "md_surrogate_train")
        return loss.value

    def train_forces(self, steps: int, lr: float = 1e-3, w_energy: float = 1.0,
                     w_force: float = 1.0):
        le, lf = C.c_double(), C.c_double()
        self._ck(self.lib.md_surrogate_train_forces(self.h, steps, lr, w_energy, w_force,
                                                    C.byref(le), C.byref(lf)),
                 "md_surrogate_train_forces")
        return le.value, lf.value

    def force_grad(self, x, v):
        x = np.ascontiguousarray(x, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        g = np.zeros(self.nparams, np.float32)
        self._ck(self.lib.md_surrogate_force_grad(self.h, x, v, len(x), g),
                 "md_surrogate_force_grad")
        return g

    def set_model(self, kind: int, hidden: int = 64):
        """0: the per-atom energy network (tensor cores); 1: the direct-force
        head with `hidden` units per hidden layer (32, 64 or 128)."""
        self._ck(self.lib.md_surrogate_set_model(self.h, kind, hidden), "md_surrogate_set_model")
        self.kind, self.hidden = kind, hidden

    def head_params(self, new=None) -> np.ndarray:
        n = self.lib.md_surrogate_head_param_count(self.hidden)
        p = np.zeros(n, np.float32) if new is None else np.ascontiguousarray(new, np.float32)
        self._ck(self.lib.md_surrogate_head_params(self.h, p, n, 0 if new is None else 1),
                 "md_surrogate_head_params")
        return p

    def head_scale(self, new: float | None = None) -> float:
        """s_out, the forces of one unit of head output (0 before training)."""
        v = C.c_double(0.0 if new is None else new)
        self._ck(self.lib.md_surrogate_head_scale(self.h, C.byref(v), 0 if new is None else 1),
                 "md_surrogate_head_scale")
        return v.value

    def descriptor_range(self, lo=None, hi=None):
        """The accepted descriptor range (32 lower, 32 upper bounds): read, or set."""
        if lo is None:
            lo, hi = np.zeros(32, np.float32), np.zeros(32, np.float32)
            self._ck(self.lib.md_surrogate_range(self.h, lo, hi, 0), "md_surrogate_range")
            return lo, hi
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        self._ck(self.lib.md_surrogate_range(self.h, lo, hi, 1), "md_surrogate_range")

    def head_grad(self, x, v):
        x = np.ascontiguousarray(x, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        g = np.zeros(self.lib.md_surrogate_head_param_count(self.hidden), np.float32)
        self._ck(self.lib.md_surrogate_head_grad(self.h, x, v, len(x), g),
                 "md_surrogate_head_grad")
        return g

    def attach(self, e: "Engine", threshold: float, check_every: int = 10):
        s = self.lib.md_surrogate_attach(e.h, self.h, threshold, check_every)
        if s != 0:
            raise EngineError(s, "md_surrogate_attach: " + self.lib.md_last_error(e.h).decode())

    @staticmethod
    def detach(e: "Engine"):
        e._ck(e.lib.md_surrogate_attach(e.h, None, 0.0, 1), "md_surrogate_attach")

    @staticmethod
    def report(e: "Engine") -> dict:
        r = MdSurrogateStats()
        e._ck(e.lib.md_surrogate_report(e.h, C.byref(r)), "md_surrogate_report")
        return {k: getattr(r, k) for k, _ in MdSurrogateStats._fields_}

    def forces(self, e: "Engine"):
        f = np.zeros((e.cfg.n_mb, 3))
        en = C.c_double()
        s = self.lib.md_surrogate_forces(self.h, e.h, f.ctypes.data, C.byref(en))
        if s != 0:
            raise EngineError(s, "md_surrogate_forces: " + self.lib.md_last_error(e.h).decode())
        return f, en.value

    def desc_directional(self, e: "Engine", e3: np.ndarray) -> np.ndarray:
        """sum_j (e_j - e_i) . dG_if/dd_j for the first n_mb atoms (n_mb x 32)."""
        n = e.cfg.n_mb
        e3 = np.ascontiguousarray(e3, np.float64).reshape(n, 3)
        q = np.zeros((n, 32))
        s = self.lib.md_surrogate_desc_directional(self.h, e.h, e3, q)
        if s != 0:
            raise EngineError(s, "md_surrogate_desc_directional: " +
                              self.lib.md_last_error(e.h).decode())
        return q

    def descriptors(self, e: "Engine", normalised: bool = False) -> np.ndarray:
        g = np.zeros((e.cfg.n_mb, 32), np.float32)
        s = self.lib.md_surrogate_descriptors(self.h, e.h, g, int(normalised))
        if s != 0:
            raise EngineError(s, "md_surrogate_descriptors: " +
                              self.lib.md_last_error(e.h).decode())
        return g

    def params(self, new=None) -> np.ndarray:
        if new is not None:
            p = np.ascontiguousarray(new, np.float32)
            self._ck(self.lib.md_surrogate_params(self.h, p, 1), "md_surrogate_params")
            return p
        p = np.zeros(self.nparams, np.float32)
        self._ck(self.lib.md_surrogate_params(self.h, p, 0), "md_surrogate_params")
        return p

    def normalisation(self, mean=None, istd=None, mu=0.0, sigma=1.0):
        if mean is not None:
            m = np.ascontiguousarray(mean, np.float32)
            i = np.ascontiguousarray(istd, np.float32)
            ms = np.array([mu, sigma], np.float64)
            self._ck(self.lib.md_surrogate_normalisation(self.h, m.ctypes.data, i.ctypes.data,
                                                         ms.ctypes.data, 1),
                     "md_surrogate_normalisation")
            return
        m = np.zeros(32, np.float32)
        i = np.zeros(32, np.float32)
        ms = np.zeros(2)
        self._ck(self.lib.md_surrogate_normalisation(self.h, m.ctypes.data, i.ctypes.data,
                                                     ms.ctypes.data, 0),
                 "md_surrogate_normalisation")
        return m, i, ms[0], ms[1]

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_double()
        self._ck(self.lib.md_surrogate_loss_grad(self.h, x, t, len(t), g, C.byref(loss)),
                 "md_surrogate_loss_grad")
        return loss.value, g

    def net(self, x):
        x = np.ascontiguousarray(x, np.float32)
        t = np.zeros(len(x), np.float32)
        d = np.zeros((len(x), 32), np.float32)
        self._ck(self.lib.md_surrogate_net(self.h, x, len(x), t, d), "md_surrogate_net")
        return t, d


class Batch(Engine):
    """Many independent periodic replicas in one md_ctx (md_batch_create):
    replica k holds natoms[k] atoms in a box of edge boxes[k]; arrays given to
    upload/download hold the replicas one after another."""

    def __init__(self, cfg: MdConfig, natoms, boxes):
        self.lib = load()
        na = np.ascontiguousarray(natoms, np.int32)
        bx = np.ascontiguousarray(boxes, np.float64)
        self.natoms = na
        self.boxes = bx
        cfg.n_lj = int(na.sum())
        cfg.n_mb = 0
        self.cfg = cfg
        self.n = int(na.sum())
        h = C.c_void_p()
        s = self.lib.md_batch_create(C.byref(cfg), len(na), na, bx, C.byref(h))
        if s != 0:
            raise EngineError(s, "md_batch_create: " + self.lib.md_status_string(s).decode())
        self.h = h

    def replica_records(self) -> np.ndarray:
        """(nrep, 16) records of the current state, md_thermo layout."""
        k = len(self.natoms)
        out = (MdThermo * k)()
        self._ck(self.lib.md_batch_records(self.h, out, k), "md_batch_records")
        return np.array([[getattr(r, f) for f in THERMO_FIELDS] for r in out]).reshape(k, 16)


class Shim:
    """The reference-signature functions (mdgb_*), host arrays in and out."""

    def __init__(self, species: int = SPECIES_NEON):
        self.lib = load()
        self.lib.mdgb_set_species(species)

    def _ck(self, what):
        s = self.lib.mdgb_last_status()
        if s != 0:
            raise EngineError(s, what)

    def predict(self, r4, v, a, b, c, dt):
        self.lib.mdgb_predict(r4, v, a, b, c, dt, len(r4))
        self._ck("mdgb_predict")

    def correct(self, r4, v, f, a, b, c, dt, npos, energy_loss=1.0):
        flag = C.c_int()
        self.lib.mdgb_correct(r4, v, f, a, b, c, dt, len(r4), npos, C.byref(flag), energy_loss)
        self._ck("mdgb_correct")
        return flag.value

    def lennard_jones_forces(self, pos4, rows, nlargest, rcutsq):
        f = np.zeros((len(pos4), 3))
        rows = np.ascontiguousarray(rows, np.int32)
        self.lib.mdgb_lennard_jones_forces(pos4, f, len(pos4), nlargest, rows.shape[1], rows,
                                           rcutsq)
        self._ck("mdgb_lennard_jones_forces")
        return f

    def many_body_forces(self, pos4, rows, nlargest, mbp, rcutsq, f_init=None, ljexist=False):
        f = np.zeros((len(pos4), 3)) if f_init is None else np.ascontiguousarray(f_init).copy()
        rows = np.ascontiguousarray(rows, np.int32)
        self.lib.mdgb_many_body_forces(pos4, f, mbp, nlargest, rows.shape[1], rows, rcutsq,
                                       int(ljexist))
        self._ck("mdgb_many_body_forces")
        return f

    def calculate_accelerations(self, pos4, f):
        a = np.zeros((len(pos4), 3))
        self.lib.mdgb_calculate_accelerations(pos4, a, np.ascontiguousarray(f), len(pos4))
        self._ck("mdgb_calculate_accelerations")
        return a

    def build_neighbor_list(self, pos4, rs, rcut, box, n=None):
        n = len(pos4) if n is None else n
        s = ListSettings(0, 0, rcut, rs, 0, 0, 0)
        p = self.lib.mdgb_build_neighbor_list(pos4, C.byref(s), box, 3 * len(pos4), n)
        self._ck("mdgb_build_neighbor_list")
        nls = s.nlistsize
        rows = np.ctypeslib.as_array(p, shape=(n * nls,)).reshape(n, nls).copy() if n * nls \
            else np.zeros((n, 0), np.int32)
        self.lib.mdgb_free(p)
        return rows, nls, s.nlargestsize

    def perform_calculations(self, pos4, vel3):
        vals = [C.c_double() for _ in range(8)]
        self.lib.mdgb_perform_calculations(pos4, vel3, len(pos4), *[C.byref(v) for v in vals])
        self._ck("mdgb_perform_calculations")
        return np.array([v.value for v in vals])

    def calculate_potential(self, pos4):
        a, b = C.c_double(), C.c_double()
        self.lib.mdgb_calculate_potential(pos4, C.byref(a), C.byref(b), len(pos4))
        self._ck("mdgb_calculate_potential")
        return a.value, b.value


def tc_selftest(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """C = A B^T on the tensor cores (tcgen05, BF16 operands, FP32 accumulate);
    A is 128 x K, B is N x K."""
    L = load()
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    Cm = np.zeros((128, B.shape[0]), np.float32)
    s = L.mdgb_tc_selftest(A, B, Cm, B.shape[0], A.shape[1])
    if s != 0:
        raise EngineError(s, "mdgb_tc_selftest")
    return Cm


def conv_selftest(f: np.ndarray, d: np.ndarray):
    """The fused Gear update's integer-operation conversions on the device,
    each beside the conversion instruction: (widen(f), (double)f,
    narrow(d), __double2float_rn(d)); f and d of equal length."""
    L = load()
    f = np.ascontiguousarray(f, np.float32)
    d = np.ascontiguousarray(d, np.float64)
    n = len(f)
    if len(d) != n:
        raise ValueError("f and d differ in length")
    w, wr = np.zeros(n), np.zeros(n)
    nr, nrr = np.zeros(n, np.float32), np.zeros(n, np.float32)
    s = L.mdgb_conv_selftest(f, d, n, w, wr, nr, nrr)
    if s != 0:
        raise EngineError(s, "mdgb_conv_selftest")
    return w, wr, nr, nrr


def pinned(shape, dtype=np.float64):
    """A numpy array over page-locked host memory (md_host_alloc); the memory
    lives as long as the returned array."""
    L = load()
    nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
    p = L.md_host_alloc(max(nbytes, 1))
    if not p:
        raise EngineError(8, "md_host_alloc failed")
    buf = (C.c_char * max(nbytes, 1)).from_address(p)
    arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    class _Owner:
        def __del__(self, p=p, L=L):
            L.md_host_free(p)
    arr_owner = _Owner()
    # keep the owner alive with the array
    out = arr.view(_PinnedArray)
    out._owner = arr_owner
    return out


class _PinnedArray(np.ndarray):
    pass


def read_config(path: str):
    """md_read_config: returns (MdConfig, strings dict, extras dict) or raises."""
    L = load()
    cfg = MdConfig()
    strs = C.create_string_buffer(2048)
    extra = (C.c_double * 6)()
    err = C.create_string_buffer(512)
    s = L.md_read_config(path.encode(), C.byref(cfg), strs, extra, err, 512)
    if s != 0:
        raise EngineError(s, err.value.decode())
    raw = strs.raw
    names = ["Input", "Output", "Filename", "AnimationData"]
    strings = {k: raw[512 * i:512 * (i + 1)].split(b"\0")[0].decode() for i, k in enumerate(names)}
    extras = dict(zip(["Temperature", "VXCMFROM", "VXCMTO", "VXCMSTEP", "CUDA Blocks",
                       "AnimationTimesteps"], list(extra)))
    return cfg, strings, extras


def measure_arith_peaks(device: int = 0) -> dict:
    """FP64 and FP32 FMA-chain rates of the device (GFLOP/s, FMA = 2)."""
    lib = load()
    f64, f32 = C.c_double(), C.c_double()
    s = lib.md_measure_arith_peaks(device, C.byref(f64), C.byref(f32))
    if s != 0:
        raise EngineError(s, "md_measure_arith_peaks")
    return {"fp64_gflops": f64.value, "fp32_gflops": f32.value}


def device_sm_count(device: int = 0) -> int:
    lib = load()
    n = C.c_int()
    s = lib.md_device_sm_count(device, C.byref(n))
    if s != 0:
        raise EngineError(s, "md_device_sm_count")
    return n.value
