"""CPU restatement of equi's chooseVelocities, for the tests only.

Test infrastructure: nothing in the product imports this file.  It follows
cpu/equi/Host.cpp:416-572 statement by statement (sequential sums in atom
order, the while loop of the momentum removal) with two replacements that
the GPU version makes too:

* rand() (seeded from the clock, :83) becomes a counter-based generator:
  the splitmix64 finaliser of seed + (3 atom + component + 1) * golden
  gamma, whose top 32 bits u give (u + 1) / (2^32 + 1), on (0, 1) like
  (rand() + 1) / (RAND_MAX + 2) (cpu/equi/Host.h:26);
* inverf (cpu/equi/Statistics.cpp:115-140) becomes scipy's erfinv (the GPU
  calls CUDA's erfinv; the two agree to a few ulps).

Kept from the reference: many-body atoms i, i + 1 (i even, i < n_mb) share
the draw of atom i, made with atom i's mass (:465-472); the momentum sums
before the removal count such a pair once with that mass, and so does totalm
(:474-478); the z draw applies inverf before the affine map (:457-461).
"""
import numpy as np
from scipy.special import erfinv

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


def choose_velocities(pos4, n_mb: int, temperature_k: float, seed: int, species="argon",
                      max_shifts=100000):
    """(velocities n x 3, shifts), or (None, shifts) where a shift of the
    removal loop does not shrink the largest component (the reference loops
    forever there)."""
    m_of = masses(species)
    temp = temperature_k * RB
    n = len(pos4)
    types = [int(w) for w in pos4[:, 3]]
    vel = np.zeros((n, 3))
    cm = [0.0, 0.0, 0.0]
    totalm = 0.0
    i = 0
    while i < n:
        mass = m_of[types[i]]
        sc = np.sqrt(2.0 * temp / mass)
        vx = erfinv(2.0 * uniform(seed, i, 0) - 1.0) * sc
        vy = erfinv(2.0 * uniform(seed, i, 1) - 1.0) * sc
        vz = (2.0 * erfinv(uniform(seed, i, 2)) - 1.0) * sc
        vel[i] = (vx, vy, vz)
        if i < n_mb and i + 1 < n:
            vel[i + 1] = vel[i]
            i += 1
        for k in range(3):
            cm[k] += mass * vel[i, k]
        totalm += mass
        i += 1
    cm = [c / totalm for c in cm]
    shifts = 0
    prev = 1e300
    while abs(cm[0]) > 1e-15 or abs(cm[1]) > 1e-15 or abs(cm[2]) > 1e-15:
        shifts += 1
        big = max(abs(c) for c in cm)
        if shifts > max_shifts or not big < prev:
            return None, shifts
        prev = big
        vel -= np.array(cm)
        cm = [0.0, 0.0, 0.0]
        for j in range(n):
            m = m_of[types[j]]
            for k in range(3):
                cm[k] += vel[j, k] * m
        cm = [c / totalm for c in cm]
    t = 0.0
    for j in range(n):
        v = vel[j]
        t += m_of[types[j]] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    t = t / (3.0 * n)
    return vel * np.sqrt(temp / t), shifts
