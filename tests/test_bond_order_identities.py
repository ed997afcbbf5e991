"""The FP32 bond-order kernels write the angle derivatives of
cpu/common/BondOrderFuncs.h in a shorter form (md_forces.cu, k_mb_pass1 and
k_mb_pass2 with T = float).  The reference writes each as one quotient per
component,

    ((2 r_ij d_ij + 2 r_im d_im) 2 r_ij r_im - (2 r_im d_ij + 2 r_ij d_im) num)
        / (4 r_ij^2 r_im^2),

which equals d_ij (1/r_im - cos/r_ij) + d_im (1/r_ij - cos/r_im) (d the unit
vectors).  The four angle terms of the two passes are checked here in FP64 on
random triangles against the reference's expressions."""
import numpy as np


def _unit(v):
    r = np.linalg.norm(v)
    return v / r, r


def test_angle_derivative_forms_equal_the_reference_quotients():
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(3000):
        pi, pj, pm = rng.normal(size=(3, 3)) * 1.5
        # pass 1: pair i-j, third body m (derivatives with respect to r_i)
        dij, rij = _unit(pi - pj)
        dim, rim = _unit(pi - pm)
        rjm = np.linalg.norm(pj - pm)
        num = rij**2 + rim**2 - rjm**2
        cos = num / (2 * rij * rim)
        ref = ((2 * rij * dij + 2 * rim * dim) * 2 * rij * rim
               - (2 * rim * dij + 2 * rij * dim) * num) / (4 * rij**2 * rim**2)
        new = dij * (1 / rim - cos / rij) + dim * (1 / rij - cos / rim)
        worst = max(worst, np.abs(ref - new).max() / np.abs(ref).max())
        num = rij**2 + rjm**2 - rim**2
        cos = num / (2 * rij * rjm)
        ref = ((2 * rij * dij - 2 * rim * dim) * 2 * rij * rjm
               - 2 * rjm * dij * num) / (4 * rij**2 * rjm**2)
        new = dij * (1 / rjm - cos / rij) - dim * (rim / (rij * rjm))
        worst = max(worst, np.abs(ref - new).max() / np.abs(ref).max())
        # pass 2: pair i-j, third body k (derivatives with respect to r_k)
        pk = pm
        dik, rik = _unit(pk - pi)
        djk, rjk = _unit(pk - pj)  # -(r_j - r_k) / r_jk
        num = rij**2 + rik**2 - rjk**2
        cos = num / (2 * rij * rik)
        ref = ((2 * rik * dik - 2 * rjk * djk) * 2 * rij * rik
               - (2 * rij * dik) * num) / (4 * rij**2 * rik**2)
        new = dik * (1 / rij - cos / rik) - djk * (rjk / (rij * rik))
        worst = max(worst, np.abs(ref - new).max() / np.abs(ref).max())
        num = rij**2 + rjk**2 - rik**2
        cos = num / (2 * rij * rjk)
        ref = ((2 * rjk * djk - 2 * rik * dik) * 2 * rij * rjk
               - (2 * rij * djk) * num) / (4 * rij**2 * rjk**2)
        new = djk * (1 / rij - cos / rjk) - dik * (rik / (rij * rjk))
        worst = max(worst, np.abs(ref - new).max() / np.abs(ref).max())
    assert worst < 1e-11, worst
