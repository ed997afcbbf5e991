"""Seeded test systems (lattices in the reference's input layout)."""
import numpy as np

from moleculardynamics_gb300 import lattice as lat

# Bond-order diamond spacing used by the tests: nearest neighbour 1.5 A.
DIAMOND_A = 4 * 1.5 / np.sqrt(3)


def argon_fcc(ncell=6, temperature=94.4, seed=1, natoms=None, noise=0.0):
    """Argon FCC at rho* = 0.8442.  A perfect lattice has zero net forces by
    symmetry; noise (angstrom) gives a thermal-like configuration."""
    return lat.make_system("fcc", ncell, temperature, seed=seed, natoms=natoms, noise=noise)


def nitrogen_diamond(ncell=3, temperature=300.0, seed=2, noise=0.02, mixed_o=False):
    pos, vel, L = lat.make_system("diamond", ncell, temperature, seed=seed, a=DIAMOND_A,
                                  noise=noise, species=lat.SPECIES_N, mass_table="neon")
    if mixed_o:
        pos[::2, 3] = lat.SPECIES_O
    return pos, vel, L


def mixed_system(seed=3):
    """64 bond-order atoms (N and O) plus 108 neon atoms placed beside them."""
    p1, v1, _ = nitrogen_diamond(2, seed=seed, mixed_o=True)
    p2, v2, _ = lat.make_system("fcc", 3, 100.0, seed=seed + 1, a=6.0, species=lat.SPECIES_NG,
                                mass_table="neon")
    p2[:, :3] += np.array([22.0, 0.0, 0.0])
    pos = np.ascontiguousarray(np.concatenate([p1, p2]))
    vel = np.ascontiguousarray(np.concatenate([v1, v2]))
    return pos, vel, len(p1), len(p2)
