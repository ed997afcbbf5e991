"""Seeded synthetic inputs in the reference's input layout.

The reference reads positions and velocities from a text ``Input`` file with
seven numbers per atom, ``x y z type vx vy vz`` (common/Loader.cpp:125-155),
written by its ``equi`` generator.  There is no public dataset: every workload
here is a lattice built from a seed.  Units are the reference's: angstrom,
femtosecond, g/mol, energy in 1e7 J/mol, kB = 8.314e-7 per kelvin
(common/DebugCalculations.cpp:122).

Species indices: N = 0, O = 1, NG = 2 (common/Constants.h:13-15).  Argon
systems are NG atoms with the engine's argon species table.
"""
from __future__ import annotations

import numpy as np

KB = 8.314e-7
SPECIES_N, SPECIES_O, SPECIES_NG = 0, 1, 2
MASS = {"neon": {0: 14.00674, 1: 15.9994, 2: 20.1797},
        "argon": {0: 14.00674, 1: 15.9994, 2: 39.948}}
SIGMA_AR = 3.405
EPS_AR_K = 119.8

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
DIAMOND_BASIS = np.concatenate([FCC_BASIS, FCC_BASIS + 0.25])


def fcc_constant(rho_star: float = 0.8442, sigma: float = SIGMA_AR) -> float:
    """FCC cubic cell edge at reduced density rho* = rho sigma^3."""
    return sigma * (4.0 / rho_star) ** (1.0 / 3.0)


def lattice(ncell, a: float, basis: np.ndarray, natoms: int | None = None) -> np.ndarray:
    """Sites of an ncell^3 (or (nx,ny,nz)) cubic lattice, centred on the origin.

    Sites are ordered cell by cell (x slowest), basis atom fastest, and shifted
    by a/8 so that none sits exactly on the box edge.  ``natoms`` keeps the
    first sites only (a partially filled lattice)."""
    nx, ny, nz = (ncell, ncell, ncell) if np.isscalar(ncell) else ncell
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    sites = (g.reshape(-1, 1, 3) + basis[None]).reshape(-1, 3) * a
    sites += a / 8.0
    sites -= np.array([nx, ny, nz]) * a / 2.0
    return sites[:natoms] if natoms is not None else sites


def maxwell_boltzmann(rng: np.random.Generator, masses: np.ndarray, temperature: float,
                      zero_momentum: bool = True, rescale: bool = True) -> np.ndarray:
    """Velocities (angstrom/fs) drawn at ``temperature`` with total momentum zeroed.

    With ``rescale`` the result is scaled so that the reference's temperature
    (common/DebugCalculations.cpp:115-122: sum m (v - v_cm)^2 / (3 N kB))
    equals ``temperature`` exactly."""
    n = len(masses)
    v = rng.standard_normal((n, 3)) * np.sqrt(KB * temperature / masses)[:, None]
    if zero_momentum and n > 1:
        v -= (masses[:, None] * v).sum(0) / masses.sum()
    if rescale and n > 1 and temperature > 0:
        t = (masses[:, None] * v * v).sum() / (3.0 * n * KB)
        v *= np.sqrt(temperature / t)
    return v


def make_system(kind: str, ncell, temperature: float, seed: int, a: float | None = None,
                noise: float = 0.0, natoms: int | None = None, species: int = SPECIES_NG,
                mass_table: str = "argon"):
    """Positions (N,4: x,y,z,type) and velocities (N,3) of a seeded lattice.

    kind: "fcc" or "diamond".  noise: Gaussian position noise (angstrom).
    Returns (pos4, vel3, box_edge)."""
    rng = np.random.default_rng(seed)
    basis = FCC_BASIS if kind == "fcc" else DIAMOND_BASIS
    if a is None:
        a = fcc_constant()
    xyz = lattice(ncell, a, basis, natoms)
    if noise > 0:
        xyz = xyz + noise * rng.standard_normal(xyz.shape)
    n = len(xyz)
    pos4 = np.zeros((n, 4))
    pos4[:, :3] = xyz
    pos4[:, 3] = species
    masses = np.full(n, MASS[mass_table][species])
    vel3 = maxwell_boltzmann(rng, masses, temperature)
    nx = ncell if np.isscalar(ncell) else ncell[0]
    return np.ascontiguousarray(pos4), np.ascontiguousarray(vel3), nx * a


def write_input(path: str, pos4: np.ndarray, vel3: np.ndarray) -> None:
    """Writes the reference Input/Output text format (common/Loader.cpp:88-120)."""
    with open(path, "w") as fh:
        for p, v in zip(pos4, vel3):
            fh.write(" ".join(f"{x:e}" for x in (*p, *v)) + " \n")


def read_input(path: str, n: int):
    vals = np.loadtxt(path).reshape(-1)[: 7 * n].reshape(n, 7)
    return np.ascontiguousarray(vals[:, :4]), np.ascontiguousarray(vals[:, 4:])


def make_batch(nrep: int = 256, nmin: int = 256, nmax: int = 32000, tmin: float = 60.0,
               tmax: float = 150.0, seed: int = 4096, rho_star: float = 0.8442):
    """An ensemble of independent argon replicas of uneven sizes.

    Replica sizes are drawn log-uniform on [nmin, nmax]; replica k is the
    first N_k sites of a ceil((N_k / 4)^(1/3))^3 FCC lattice at density
    rho_star (so its box is that lattice's edge), with Maxwell-Boltzmann
    velocities at a temperature drawn uniform on [tmin, tmax].
    Returns (pos4, vel3, natoms, boxes, temperatures), the atoms of the
    replicas one after another."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), nrep))).astype(np.int64)
    temps = rng.uniform(tmin, tmax, nrep)
    seeds = rng.integers(0, 2**31 - 1, nrep)
    a = fcc_constant(rho_star)
    pos, vel, boxes = [], [], []
    for n_k, t_k, s_k in zip(sizes, temps, seeds):
        ncell = int(np.ceil((n_k / 4.0) ** (1.0 / 3.0) - 1e-9))
        p, v, L = make_system("fcc", ncell, float(t_k), seed=int(s_k), a=a, natoms=int(n_k))
        pos.append(p)
        vel.append(v)
        boxes.append(L)
    return (np.ascontiguousarray(np.concatenate(pos)), np.ascontiguousarray(np.concatenate(vel)),
            sizes.astype(np.int32), np.asarray(boxes, np.float64), temps)
