"""equi's velocity draw pinned to the reference compiled in place.

cpu/equi/Statistics.cpp (inverf with its own erf/erfc) and
cpu/equi/Host.cpp:416-572 (chooseVelocities) are built by oracle/build_ref.sh
with rand() replaying draws the test gives and RAND_MAX = 0x7fff, the value
of the platform the reference was written for.  The C restatement
(oracle/mdoracle.c orc_inverf, orc_choose_velocities) is fed the same draws
as uniforms y = (r + 1) / (RAND_MAX + 2) (cpu/equi/Host.h:26) and must return
the same bits, including the reference's inaccurate inverf for negative
arguments (its erf series stops after two terms when the sum is negative)."""
import numpy as np
import pytest

from systems import argon_fcc, mixed_system

RB = 8.314e-7  # cpu/equi/Host.cpp:85
RANDMAX2 = 0x7FFF + 2


@pytest.fixture(scope="module")
def ref_equi(reference):
    from oracle.oracle import load_reference_equi
    r = {v: load_reference_equi(v) for v in ("neon", "argon")}
    if r["neon"] is None or r["argon"] is None:
        pytest.skip("oracle/_ref/libmdref_equi_*.so not built")
    return r


def test_inverf_bit_exact(oracle, ref_equi):
    R = ref_equi["argon"]
    rng = np.random.default_rng(7)
    zs = np.concatenate([np.linspace(-0.99999, 0.99999, 4001), rng.uniform(-1, 1, 2000),
                         [0.0, -0.8125, 0.8125, np.nextafter(0.8125, 0), 1e-300, -1e-300,
                          1.0 - 2.0 ** -30, -1.0 + 2.0 ** -30]])
    for z in zs:
        assert oracle.inverf(z) == R.inverf(z), z
    # the reference's own quirk, kept: inaccurate for negative arguments
    from scipy.special import erfinv
    assert abs(R.inverf(-0.5) - erfinv(-0.5)) > 1e-4
    assert abs(R.inverf(0.5) - erfinv(0.5)) < 1e-12


@pytest.mark.parametrize("case", ["argon", "mixed"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_choose_velocities_bit_exact(oracle, ref_equi, case, seed):
    if case == "argon":
        pos, _, _ = argon_fcc(3, seed=seed)
        n_lj, n_mb, species, T = len(pos), 0, 1, 94.4
    else:
        pos, _, n_mb, n_lj = mixed_system(seed=seed)
        species, T = 0, 300.0
    rng = np.random.default_rng(100 + seed)
    draws = rng.integers(0, 0x7FFF + 1, size=3 * len(pos))
    u = (draws.astype(np.float64) + 1.0) / RANDMAX2
    vo, used, shifts = oracle.choose_velocities(pos, n_mb, T * RB, species, u)
    assert vo is not None, "the momentum removal must converge for this system"
    vr, used_r = ref_equi["argon" if species == 1 else "neon"].choose_velocities(
        pos, n_lj, n_mb, T * RB, draws)
    assert used == used_r
    assert np.array_equal(vo, vr)
