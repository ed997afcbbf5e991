"""equi's chooseVelocities with the engine's generator, for the tests only.

Test infrastructure: nothing in the product imports this file.  The draws
come from the counter-based generator the GPU uses in place of rand()
(seeded from the clock in the reference, cpu/equi/Host.cpp:83): the
splitmix64 finaliser of seed + (3 atom + component + 1) * golden gamma,
whose top 32 bits u give (u + 1) / (2^32 + 1), on (0, 1) like
(rand() + 1) / (RAND_MAX + 2) (cpu/equi/Host.h:26).  The velocities are then
those of the C restatement of cpu/equi/Host.cpp:416-572 and of the
reference's inverf (cpu/equi/Statistics.cpp:115-140) in oracle/mdoracle.c,
which tests/test_equi_pinned.py holds bit-exact to the reference compiled in
place.  Kept from the reference: many-body atoms i, i + 1 (i even, i < n_mb)
share the draw of atom i, made with atom i's mass (:465-472); the momentum
sums before the removal count such a pair once with that mass, and so does
totalm (:474-478); the z draw applies inverf before the affine map
(:457-461).
"""
import numpy as np

MASK = (1 << 64) - 1
GAMMA = 0x9E3779B97F4A7C15
RB = 8.314e-7  # cpu/equi/Host.cpp:85


def mix64(x: int) -> int:
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & MASK
    return x ^ (x >> 31)


def uniform(seed: int, atom: int, comp: int) -> float:
    z = mix64((seed + (3 * atom + comp + 1) * GAMMA) & MASK)
    return ((z >> 32) + 1.0) / 4294967297.0


def masses(species: str):
    """common/Constants.h masses (float literals), NG slot neon or argon."""
    ng = 39.948 if species == "argon" else 20.1797
    return [float(np.float32(14.00674)), float(np.float32(15.9994)), float(np.float32(ng))]


def draws(pos4, n_mb: int, seed: int) -> np.ndarray:
    """The uniforms of one chooseVelocities call in the reference's order:
    x, y, z of every atom that draws (the second atom of a many-body pair
    takes its partner's draw)."""
    n = len(pos4)
    u = []
    i = 0
    while i < n:
        u += [uniform(seed, i, 0), uniform(seed, i, 1), uniform(seed, i, 2)]
        if i < n_mb:
            i += 1
        i += 1
    return np.array(u)


def choose_velocities(pos4, n_mb: int, temperature_k: float, seed: int, species="argon",
                      max_shifts=100000):
    """(velocities n x 3, shifts), or (None, shifts) where a shift of the
    removal loop after the second does not shrink the largest component
    (the reference loops forever there)."""
    from oracle.oracle import SPECIES_ARGON, SPECIES_NEON, load_oracle
    O = load_oracle()
    sp = SPECIES_ARGON if species == "argon" else SPECIES_NEON
    vel, _, shifts = O.choose_velocities(pos4, n_mb, temperature_k * RB, sp,
                                         draws(pos4, n_mb, seed), max_shifts)
    return vel, shifts
