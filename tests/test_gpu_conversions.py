"""The fused Gear update's conversions by integer operations (widen: FP32 to
FP64, exact; narrow: FP64 to FP32, nearest-even) against the device's own
conversion instructions: bit-identical on normal numbers and exact ties;
subnormal FP32 inputs widen to signed zero; non-finite values stay
non-finite."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_widen_and_narrow_match_the_conversion_instructions(eng):
    rng = np.random.default_rng(7)
    n = 1 << 20
    f = (rng.standard_normal(n) * 10.0 ** rng.integers(-36, 37, n)).astype(np.float32)
    f[:6] = [0.0, -0.0, np.inf, -np.inf, np.nan, 1e-40]
    d = rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)
    # positions of a 366 A box, and exact halfway cases between FP32 neighbours
    m = n // 4
    d[:m] = rng.uniform(-400.0, 400.0, m)
    base = rng.uniform(1.0, 400.0, m).astype(np.float32)
    half = np.spacing(base).astype(np.float64) / 2
    d[m:2 * m] = base.astype(np.float64) + half * rng.choice([-1.0, 1.0], m)
    d[2 * m:2 * m + 4] = [0.0, -0.0, 1e300, np.nan]
    w, wr, nr, nrr = eng.conv_selftest(f, d)
    tiny = np.abs(f) < np.finfo(np.float32).tiny
    fin = np.isfinite(f)
    assert np.array_equal(w[fin & ~tiny].view(np.uint64), wr[fin & ~tiny].view(np.uint64))
    assert np.all(w[tiny & fin] == 0.0)
    assert np.all(~np.isfinite(w[~fin]))
    ok = np.isfinite(d)
    assert np.array_equal(nr[ok].view(np.uint32), nrr[ok].view(np.uint32))
    assert np.isnan(nr[2 * m + 3])
