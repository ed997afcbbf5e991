"""ctypes bindings of the CPU oracle (test infrastructure, not the product).

Two libraries are bound here:

* ``libmdoracle.so``: the C restatement in oracle/mdoracle.c, built by
  ``build_oracle()`` on any machine (here and on the GPU machine);
* ``_ref/libmdref_<variant>.so``: the reference engine of
  vakuras/moleculardynamics compiled in place by oracle/build_ref.sh.  It only
  exists where the reference sources are present, so callers must accept
  ``load_reference()`` returning None.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline arm may
import this module.  Arrays use the reference's host layouts: positions are
``real4`` (x, y, z, type as a float) and vectors ``real3``, with real = double
(common/Global.h:25-33, -DEQUI as cpumd is built).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libmdoracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

SPECIES_NEON = 0
SPECIES_ARGON = 1


def build_oracle(force: bool = False) -> str:
    """Compile oracle/mdoracle.c into oracle/libmdoracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "mdoracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(os.path.join(HERE, "mdoracle.h"))):
        return ORACLE_SO
    base = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
            "-shared", "-o", ORACLE_SO + ".tmp", src, "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True)
    os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def reference_source_root() -> str | None:
    """Where oracle/_ref was built from (recorded by build_ref.sh), or the
    MDGB_REFERENCE_SRC environment variable; None when neither is set."""
    env = os.environ.get("MDGB_REFERENCE_SRC")
    if env:
        return env
    rec = os.path.join(HERE, "_ref", "source_root")
    if os.path.isfile(rec):
        with open(rec) as f:
            return f.read().strip() or None
    return None


def build_reference(ref_root: str | None = None) -> bool:
    """Build oracle/_ref from the reference sources at ref_root (default: the
    MDGB_REFERENCE_SRC environment variable or the recorded tree); False when
    they are not present."""
    ref_root = ref_root or reference_source_root()
    if not ref_root or not os.path.isfile(os.path.join(ref_root, "common", "NeighborList.cpp")):
        return False
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), ref_root], check=True,
                   capture_output=True)
    return True


class OrcList(C.Structure):
    _fields_ = [("n", C.c_int), ("nlistsize", C.c_int), ("nlargest", C.c_int),
                ("cells", C.c_int), ("maxcell", C.c_int), ("periodic", C.c_int),
                ("box", C.c_double), ("rows", C.POINTER(C.c_int)),
                ("code", C.POINTER(C.c_byte)), ("cell", C.POINTER(C.c_int))]


class OrcSpecies(C.Structure):
    _fields_ = [(k, C.c_float) for k in ("sigNG", "sigNGN", "sigNGO", "epsNG", "epsNGN",
                                         "epsNGO", "mN", "mO", "mNG")]


class OrcRunParams(C.Structure):
    _fields_ = [("n_lj", C.c_int), ("n_mb", C.c_int), ("timesteps", C.c_int),
                ("use_lj", C.c_int), ("use_mb", C.c_int), ("output_timesteps", C.c_int),
                ("dt", C.c_float), ("lj_rs", C.c_float), ("lj_rcut", C.c_float),
                ("mb_rs", C.c_float), ("mb_rcut", C.c_float), ("energy_loss", C.c_float),
                ("vxcm", C.c_float), ("periodic", C.c_int), ("box", C.c_double),
                ("species", C.c_int), ("threads", C.c_int)]


@dataclass
class NeighborList:
    """A list in the reference layout: rows[i, k], -1 padded."""
    rows: np.ndarray
    code: np.ndarray | None
    nlistsize: int
    nlargest: int
    cells: int = 0
    cell: np.ndarray | None = None
    handle: object = None


class Oracle:
    """The C restatement (oracle/mdoracle.c)."""

    def __init__(self, path: str | None = None):
        self.lib = C.CDLL(path or build_oracle())
        L = self.lib
        L.orc_build_list.restype = C.POINTER(OrcList)
        L.orc_build_list.argtypes = [_dp, C.c_int, C.c_float, C.c_double, C.c_int]
        L.orc_free_list.argtypes = [C.POINTER(OrcList)]
        L.orc_lj_forces.argtypes = [_dp, _dp, C.c_int, C.POINTER(OrcList), C.c_double,
                                    C.POINTER(OrcSpecies), C.c_void_p]
        L.orc_mb_forces.argtypes = [_dp, _dp, C.c_int, C.POINTER(OrcList), C.c_double,
                                    C.c_int, C.POINTER(C.c_longlong), C.c_void_p]
        L.orc_predict.argtypes = [_dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int]
        L.orc_correct.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int,
                                  C.c_double, C.POINTER(C.c_int), C.c_float, C.c_int,
                                  C.POINTER(OrcSpecies)]
        L.orc_accelerations.argtypes = [_dp, _dp, _dp, C.c_int, C.POINTER(OrcSpecies)]
        L.orc_perform_calculations.argtypes = [_dp, _dp, C.c_int, _dp, C.POINTER(OrcSpecies)]
        L.orc_calculate_potential.argtypes = [_dp, C.c_int, C.POINTER(C.c_double),
                                              C.POINTER(C.c_double), C.POINTER(OrcSpecies)]
        L.orc_ready_list.argtypes = [_dp, _dp, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
        L.orc_next_build.argtypes = [C.c_float, C.c_double, C.c_double, C.c_int]
        L.orc_inverf.restype = C.c_double
        L.orc_inverf.argtypes = [C.c_double]
        L.orc_choose_velocities.restype = C.c_long
        L.orc_choose_velocities.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int,
                                            _dp, C.c_long, C.c_long, C.POINTER(C.c_long)]
        L.orc_next_build.restype = C.c_int
        L.orc_list_settings.argtypes = [C.c_float, C.c_float] + [C.POINTER(C.c_float)] * 3
        L.orc_run.argtypes = [C.POINTER(OrcRunParams), _dp, _dp, _dp, _dp, _dp, _dp,
                              C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
        L.orc_run.restype = C.c_int
        L.orc_max_threads.restype = C.c_int

    def species(self, which: int) -> OrcSpecies:
        sp = OrcSpecies()
        self.lib.orc_species_get(which, C.byref(sp))
        return sp

    @staticmethod
    def list_settings(lib, rs: float, rcut: float):
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        lib.orc_list_settings(rs, rcut, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def settings(self, rs, rcut):
        return self.list_settings(self.lib, rs, rcut)

    def ready_list(self, pos4, vel3):
        vm, bx = C.c_double(), C.c_double()
        self.lib.orc_ready_list(pos4, vel3, len(pos4), C.byref(vm), C.byref(bx))
        return vm.value, bx.value

    def next_build(self, maxnlmove, vmax, dt, t):
        return self.lib.orc_next_build(maxnlmove, vmax, dt, t)

    def build_list(self, pos4: np.ndarray, rs: float, box: float, periodic: bool = False,
                   n: int | None = None) -> NeighborList:
        """Builds the list; with periodic=True pos4 is wrapped in place."""
        n = len(pos4) if n is None else n
        h = self.lib.orc_build_list(pos4, n, rs, box, int(periodic))
        if not h:
            raise ValueError("oracle list build failed (periodic box smaller than 2 rs?)")
        l = h.contents
        nls = l.nlistsize
        rows = np.ctypeslib.as_array(l.rows, shape=(n * nls,)).reshape(n, nls).copy() if n * nls else np.zeros((n, 0), np.int32)
        code = np.ctypeslib.as_array(l.code, shape=(n * nls,)).reshape(n, nls).copy() if n * nls else np.zeros((n, 0), np.int8)
        cell = np.ctypeslib.as_array(l.cell, shape=(3 * n,)).reshape(n, 3).copy() if n else np.zeros((0, 3), np.int32)
        return NeighborList(rows, code, nls, l.nlargest, l.cells, cell, h)

    def free_list(self, nl: NeighborList):
        if nl.handle is not None:
            self.lib.orc_free_list(nl.handle)
            nl.handle = None

    def lj_forces(self, pos4, nl: NeighborList, rcutsq: float, species: int = SPECIES_NEON,
                  energy: bool = False):
        n = len(pos4)
        f = np.zeros((n, 3))
        e = np.zeros(3)
        sp = self.species(species)
        self.lib.orc_lj_forces(pos4, f, n, nl.handle, rcutsq, C.byref(sp),
                               e.ctypes.data if energy else None)
        return (f, e) if energy else f

    def mb_forces(self, pos4, nl: NeighborList, mbp: int, rcutsq: float, f_init=None,
                  ljexist: bool = False, energy: bool = False):
        f = np.zeros((len(pos4), 3)) if f_init is None else f_init.copy()
        miss = C.c_longlong()
        e = np.zeros(2)
        self.lib.orc_mb_forces(pos4, f, mbp, nl.handle, rcutsq, int(ljexist), C.byref(miss),
                               e.ctypes.data if energy else None)
        out = (f, miss.value)
        return out + (e,) if energy else out

    def predict(self, r4, v, a, b, c, dt):
        self.lib.orc_predict(r4, v, a, b, c, dt, len(r4))

    def correct(self, r4, v, f, a, b, c, dt, npos, energy_loss=1.0, walls=True,
                species=SPECIES_NEON):
        flag = C.c_int()
        sp = self.species(species)
        self.lib.orc_correct(r4, v, f, a, b, c, dt, len(r4), npos, C.byref(flag), energy_loss,
                             int(walls), C.byref(sp))
        return flag.value

    def accelerations(self, pos4, f, species=SPECIES_NEON):
        a = np.zeros((len(pos4), 3))
        sp = self.species(species)
        self.lib.orc_accelerations(pos4, a, f, len(pos4), C.byref(sp))
        return a

    def perform_calculations(self, pos4, vel3, species=SPECIES_NEON):
        out = np.zeros(8)
        sp = self.species(species)
        self.lib.orc_perform_calculations(pos4, vel3, len(pos4), out, C.byref(sp))
        return out

    def calculate_potential(self, pos4, species=SPECIES_NEON):
        a, b = C.c_double(), C.c_double()
        sp = self.species(species)
        self.lib.orc_calculate_potential(pos4, len(pos4), C.byref(a), C.byref(b), C.byref(sp))
        return a.value, b.value

    def run(self, p: dict, pos4, vel3, thermo_records: int = 0):
        """One vxcm pass of hostMain; returns dict of final state and stats."""
        prm = OrcRunParams(**p)
        n = len(pos4)
        pos = np.ascontiguousarray(pos4, dtype=np.float64).copy()
        vel = np.ascontiguousarray(vel3, dtype=np.float64).copy()
        a, b, c, f = (np.zeros((n, 3)) for _ in range(4))
        th = np.zeros((max(thermo_records, 1), 12))
        stats = (C.c_longlong * 3)()
        el = C.c_double()
        nrec = self.lib.orc_run(C.byref(prm), pos, vel, a, b, c, f,
                                th.ctypes.data if thermo_records else None, stats, C.byref(el))
        if nrec < 0:
            raise ValueError("oracle run failed")
        return dict(pos=pos, vel=vel, acc=a, b=b, c=c, force=f, thermo=th[:nrec],
                    builds=stats[0], wall_hits=stats[1], missing_xi=stats[2],
                    elapsed_ms=el.value)

    def max_threads(self) -> int:
        return self.lib.orc_max_threads()


def _oracle_inverf(self, z: float) -> float:
    """cpu/equi/Statistics.cpp:115-140 inverf (mdoracle.c restatement)."""
    return self.lib.orc_inverf(float(z))


def _oracle_choose_velocities(self, pos4, n_mb: int, temp: float, species: int, u,
                              max_shifts: int = 100000):
    """cpu/equi/Host.cpp:416-572 with the uniforms u given: (vel, uniforms
    used, shifts); vel is None where the momentum removal does not converge."""
    pos4 = np.ascontiguousarray(pos4, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    vel = np.zeros((len(pos4), 3))
    sh = C.c_long()
    k = self.lib.orc_choose_velocities(pos4, vel, len(pos4), n_mb, temp, species, u, len(u),
                                       max_shifts, C.byref(sh))
    return (None if k < 0 else vel), k, sh.value


Oracle.inverf = _oracle_inverf
Oracle.choose_velocities = _oracle_choose_velocities


class ReferenceEqui:
    """The reference's equi velocity draw compiled in place
    (oracle/_ref/libmdref_equi_<variant>.so), rand() replaying given draws."""

    def __init__(self, path: str):
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_equi_inverf.restype = C.c_double
        L.ref_equi_inverf.argtypes = [C.c_double]
        L.ref_equi_choose_velocities.restype = C.c_long
        L.ref_equi_choose_velocities.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, _ip,
                                                 C.c_long]

    def inverf(self, z: float) -> float:
        return self.lib.ref_equi_inverf(float(z))

    def choose_velocities(self, pos4, n_lj: int, n_mb: int, temp: float, draws):
        """(vel, draws used); draws are rand() values in [0, 0x7fff]."""
        pos4 = np.ascontiguousarray(pos4, np.float64)
        draws = np.ascontiguousarray(draws, np.int32)
        vel = np.zeros((len(pos4), 3))
        k = self.lib.ref_equi_choose_velocities(pos4, vel, n_lj, n_mb, temp, draws, len(draws))
        return vel, k


def load_reference_equi(variant: str = "argon") -> ReferenceEqui | None:
    path = os.path.join(REF_DIR, f"libmdref_equi_{variant}.so")
    if not os.path.exists(path):
        return None
    try:
        return ReferenceEqui(path)
    except OSError:
        return None


class Reference:
    """The reference engine compiled in place (oracle/_ref/libmdref_<variant>.so)."""

    def __init__(self, path: str):
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_real_size.restype = C.c_int
        L.ref_build_neighbor_list.restype = C.POINTER(C.c_int)
        L.ref_build_neighbor_list.argtypes = [_dp, C.c_int, C.c_float, C.c_float, C.c_double,
                                              C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_build_list.restype = C.POINTER(C.c_int)
        L.ref_build_list.argtypes = [_dp, C.c_float, C.c_float, C.c_double, C.c_int,
                                     C.c_double, C.c_int, C.c_int, C.c_double,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_free_list.argtypes = [C.POINTER(C.c_int)]
        L.ref_lj_forces.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, _ip, C.c_double]
        L.ref_mb_forces.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, _ip, C.c_double,
                                    C.c_int]
        L.ref_predict.argtypes = [_dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int]
        L.ref_correct.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int,
                                  C.c_double, C.POINTER(C.c_int), C.c_float]
        L.ref_accelerations.argtypes = [_dp, _dp, _dp, C.c_int]
        L.ref_perform_calculations.argtypes = [_dp, _dp, C.c_int, _dp]
        L.ref_calculate_potential.argtypes = [_dp, C.c_int, C.POINTER(C.c_double),
                                              C.POINTER(C.c_double)]
        L.ref_ready_list.argtypes = [_dp, _dp, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
        L.ref_list_settings.argtypes = [C.c_float, C.c_float] + [C.POINTER(C.c_float)] * 3
        L.ref_run.argtypes = [C.POINTER(OrcRunParams), _dp, _dp, _dp, _dp, _dp, _dp,
                              C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.ref_run.restype = C.c_int
        L.ref_read_configuration.argtypes = [C.c_char_p, _ip, np.ctypeslib.ndpointer(
            dtype=np.float32, flags="C_CONTIGUOUS"), C.c_char_p]
        L.ref_write_results.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_float,
                                        C.c_int, C.c_float, C.c_float, C.c_int, C.c_float,
                                        C.c_float, C.c_float, C.c_float, _dp, C.c_int, _dp]
        L.ref_write_output.argtypes = [C.c_char_p, C.c_int, _dp, _dp]
        L.ref_read_input.argtypes = [C.c_char_p, C.c_int, _dp, _dp]
        assert L.ref_real_size() == 8, "reference must be the double build (-DEQUI)"

    def settings(self, rs, rcut):
        return _ref_settings(self.lib, rs, rcut)

    def build_neighbor_list(self, pos4, rs, rcut, box, buckets=None, n=None) -> NeighborList:
        n = len(pos4) if n is None else n
        buckets = 3 * len(pos4) if buckets is None else buckets
        nls, nl = C.c_int(), C.c_int()
        p = self.lib.ref_build_neighbor_list(pos4, n, rs, rcut, box, buckets, C.byref(nls),
                                             C.byref(nl))
        rows = np.ctypeslib.as_array(p, shape=(n * nls.value,)).reshape(n, nls.value).copy() \
            if n * nls.value else np.zeros((n, 0), np.int32)
        self.lib.ref_free_list(p)
        return NeighborList(rows, None, nls.value, nl.value)

    def ready_list(self, pos4, vel3):
        vm, bx = C.c_double(), C.c_double()
        self.lib.ref_ready_list(pos4, vel3, len(pos4), C.byref(vm), C.byref(bx))
        return vm.value, bx.value

    def next_build(self, pos4, rs, rcut, box, vmax, n, t, dt):
        nb, nls, nl = C.c_int(), C.c_int(), C.c_int()
        p = self.lib.ref_build_list(pos4, rs, rcut, box, 3 * len(pos4), vmax, n, t, dt,
                                    C.byref(nb), C.byref(nls), C.byref(nl))
        self.lib.ref_free_list(p)
        return nb.value

    def lj_forces(self, pos4, nl: NeighborList, rcutsq):
        f = np.zeros((len(pos4), 3))
        rows = np.ascontiguousarray(nl.rows, dtype=np.int32)
        self.lib.ref_lj_forces(pos4, f, len(pos4), nl.nlargest, nl.nlistsize, rows, rcutsq)
        return f

    def mb_forces(self, pos4, nl: NeighborList, mbp, rcutsq, f_init=None, ljexist=False):
        f = np.zeros((len(pos4), 3)) if f_init is None else f_init.copy()
        rows = np.ascontiguousarray(nl.rows, dtype=np.int32)
        self.lib.ref_mb_forces(pos4, f, mbp, nl.nlargest, nl.nlistsize, rows, rcutsq,
                               int(ljexist))
        return f

    def predict(self, r4, v, a, b, c, dt):
        self.lib.ref_predict(r4, v, a, b, c, dt, len(r4))

    def correct(self, r4, v, f, a, b, c, dt, npos, energy_loss=1.0):
        flag = C.c_int()
        self.lib.ref_correct(r4, v, f, a, b, c, dt, len(r4), npos, C.byref(flag), energy_loss)
        return flag.value

    def accelerations(self, pos4, f):
        a = np.zeros((len(pos4), 3))
        self.lib.ref_accelerations(pos4, a, f, len(pos4))
        return a

    def perform_calculations(self, pos4, vel3):
        out = np.zeros(8)
        self.lib.ref_perform_calculations(pos4, vel3, len(pos4), out)
        return out

    def calculate_potential(self, pos4):
        a, b = C.c_double(), C.c_double()
        self.lib.ref_calculate_potential(pos4, len(pos4), C.byref(a), C.byref(b))
        return a.value, b.value

    def run(self, p: dict, pos4, vel3, thermo_records: int = 0):
        prm = OrcRunParams(**p)
        n = len(pos4)
        pos = np.ascontiguousarray(pos4, dtype=np.float64).copy()
        vel = np.ascontiguousarray(vel3, dtype=np.float64).copy()
        a, b, c, f = (np.zeros((n, 3)) for _ in range(4))
        th = np.zeros((max(thermo_records, 1), 8))
        nb = C.c_int()
        el = C.c_double()
        nrec = self.lib.ref_run(C.byref(prm), pos, vel, a, b, c, f,
                                th.ctypes.data if thermo_records else None, C.byref(nb),
                                C.byref(el))
        return dict(pos=pos, vel=vel, acc=a, b=b, c=c, force=f, thermo=th[:nrec],
                    builds=nb.value, elapsed_ms=el.value)


def _ref_settings(lib, rs, rcut):
    a, b, c = C.c_float(), C.c_float(), C.c_float()
    lib.ref_list_settings(rs, rcut, C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def load_oracle() -> Oracle:
    return Oracle()


def load_reference(variant: str = "neon") -> Reference | None:
    """The compiled reference, or None where it was not (or cannot be) built."""
    path = os.path.join(REF_DIR, f"libmdref_{variant}.so")
    if not os.path.exists(path):
        return None
    try:
        return Reference(path)
    except OSError:
        return None
