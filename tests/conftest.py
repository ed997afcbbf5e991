import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine through the C ABI)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import build_oracle, load_oracle
    build_oracle()
    return load_oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference engine compiled in place; skipped where it cannot exist."""
    from oracle.oracle import build_reference, load_reference
    ref = load_reference("neon")
    if ref is None:
        try:
            build_reference()
        except Exception:
            pass
        ref = load_reference("neon")
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    return ref


@pytest.fixture(scope="session")
def reference_argon(reference):
    from oracle.oracle import load_reference
    return load_reference("argon")


@pytest.fixture(scope="session")
def eng():
    """The built engine module (libmdgb.so loaded)."""
    from moleculardynamics_gb300 import build, engine
    build.build()
    engine.load()
    return engine


def run_params(**kw):
    d = dict(n_lj=0, n_mb=0, timesteps=0, use_lj=1, use_mb=0, output_timesteps=0, dt=2.0,
             lj_rs=9.534, lj_rcut=8.5125, mb_rs=3.5, mb_rcut=3.0, energy_loss=1.0, vxcm=0.0,
             periodic=0, box=0.0, species=1, threads=0)
    d.update(kw)
    return d


def rel_rms(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.sqrt(((a - b) ** 2).sum(axis=-1).mean()) / np.sqrt((b ** 2).sum(axis=-1).mean()))
