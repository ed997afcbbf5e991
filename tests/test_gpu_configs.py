"""The second workload of the benchmark set as parity cases (the reference's
own non-periodic box, FP64 plain path), against the CPU oracle:

* bond order: 4,096 nitrogen atoms on an 8^3 diamond lattice (1.5 A bonds),
  0.02 A noise, 300 K, dt 0.5 fs: rows bit-exact, forces and energy within
  1e-10 relative; then 200 steps (of the workload's 2,000: the oracle takes
  about 0.2 s per step on 8 host threads, so 200 is what a test affords),
  positions within 1e-10 and velocities within 1e-8, and the forces,
  energy and virial at the end within 1e-10 of the oracle's at the same
  positions;
* LJ: 8,000 argon atoms (the first 8,000 sites of an FCC 13^3 lattice),
  dt 2 fs: rows, forces and the workload's 2,000 steps bit-exact.
"""
import numpy as np
import pytest

from conftest import rel_rms, run_params
from moleculardynamics_gb300 import lattice as lat
from systems import nitrogen_diamond

pytestmark = pytest.mark.gpu


def test_bond_order_4096(eng, oracle):
    pos, vel, _ = nitrogen_diamond(8, temperature=300.0, seed=31, noise=0.02)
    n = len(pos)
    assert n == 4096
    cfg = eng.make_config(n_mb=n, use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0, dt=0.5,
                          species=0)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest = e.neighbor_list(1)
        f, en = e.compute_forces()
        e.step(200)
        gp, gv = e.download()
    box = oracle.ready_list(pos, vel)[1]
    nl = oracle.build_list(pos.copy(), 3.5, box)
    assert np.array_equal(rows, nl.rows) and nlargest == nl.nlargest
    rcsq = oracle.settings(3.5, 3.0)[2]
    fo, miss, eo = oracle.mb_forces(pos, nl, n, rcsq, energy=True)
    oracle.free_list(nl)
    assert miss == 0
    assert rel_rms(f, fo) < 1e-10
    assert abs(en[3] - eo[0]) <= 1e-10 * abs(eo[0])
    ref = oracle.run(run_params(n_mb=n, timesteps=200, use_lj=0, use_mb=1, dt=0.5, species=0,
                                threads=oracle.max_threads()), pos, vel)
    assert rel_rms(gp[:, :3], ref["pos"][:, :3]) < 1e-10
    assert rel_rms(gv, ref["vel"]) < 1e-8
    # forces, energy and virial at the end, on the GPU's final positions
    with eng.Engine(cfg) as e:
        e.upload(gp, gv)
        e.begin(0.0)
        f2, en2 = e.compute_forces()
    box = oracle.ready_list(gp, gv)[1]
    nl = oracle.build_list(gp.copy(), 3.5, box)
    fo2, miss2, eo2 = oracle.mb_forces(gp, nl, n, rcsq, energy=True)
    oracle.free_list(nl)
    assert miss2 == 0
    assert rel_rms(f2, fo2) < 1e-10
    assert abs(en2[3] - eo2[0]) <= 1e-10 * abs(eo2[0])
    assert abs(en2[4] - eo2[1]) <= 1e-10 * abs(eo2[1])


def test_lj_8000(eng, oracle):
    pos, vel, _ = lat.make_system("fcc", 13, 94.4, seed=32, natoms=8000)
    n = len(pos)
    rs, rc = 9.534, 8.5125
    cfg = eng.make_config(n_lj=n, lj_rs=rs, lj_rcut=rc, dt=2.0)
    with eng.Engine(cfg) as e:
        e.upload(pos, vel)
        e.begin(0.0)
        rows, nls, nlargest = e.neighbor_list(0)
        f, _ = e.compute_forces()
        e.step(2000)
        gp, gv = e.download()
    box = oracle.ready_list(pos, vel)[1]
    nl = oracle.build_list(pos.copy(), rs, box)
    assert np.array_equal(rows, nl.rows) and nlargest == nl.nlargest
    fo = oracle.lj_forces(pos, nl, oracle.settings(rs, rc)[2], species=1)
    oracle.free_list(nl)
    assert np.array_equal(f, fo)
    ref = oracle.run(run_params(n_lj=n, timesteps=2000, threads=oracle.max_threads()), pos, vel)
    assert np.array_equal(gp, ref["pos"]) and np.array_equal(gv, ref["vel"])
