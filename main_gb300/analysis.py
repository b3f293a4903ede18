"""Observables derived from the dimer axes (host side, numpy).

``orientation_correlation`` restates the spatial orientation correlation of
collective_code/1D_Orientation_Correlation.py:30-53 (the same script sits in
rotational_code/linear_periodic_ci and linear_periodic_no_ci): for every frame,
the Legendre averages <P1(u)> and <P2(u)> of u = n_i . n_{i+j} over the motors
i, for motor separations j along the periodic motor index.  The frames are
the dimer axes that ``Engine.dimer_axes`` (mpcmd_dimer_axes) returns, stacked
in the layout of the reference's ``Dimer/nucvec`` dataset.
"""
import numpy as np


def orientation_correlation(nuc):
    """<P1>(t, j) and <P2>(t, j) of 1D_Orientation_Correlation.py:44-53.

    nuc: array [frames, 3, motors] (the reference's nucvec layout; one frame
    is ``Engine.dimer_axes(...)[0].T``).  Returns (P1, P2), each
    [frames, jmax]: jmax = motors / 2 + 1 for an even motor count and
    int(motors / 2) for an odd one (the script's :33-38 sizes, whose odd case
    drops the last separation).
    """
    nuc = np.asarray(nuc, dtype=np.float64)
    if nuc.ndim != 3 or nuc.shape[1] != 3:
        raise ValueError("nuc: [frames, 3, motors]")
    n = nuc.shape[2]
    jmax = int(0.5 * n) + 1 if n % 2 == 0 else int(0.5 * n)
    p1 = np.zeros((nuc.shape[0], jmax))
    p2 = np.zeros((nuc.shape[0], jmax))
    for j in range(jmax):
        # u[:, j, i] = n_i . n_{(i + j) mod N}; the script adds u[:, j, i] and
        # u[:, j, (i - j) mod N] for every i
        u = np.einsum("tci,tci->ti", nuc, np.roll(nuc, -j, axis=2))
        u_back = np.roll(u, j, axis=1)
        p1[:, j] = (u + u_back).sum(axis=1) / (2.0 * n)
        p2[:, j] = (0.5 * (3.0 * u ** 2 - 1) + 0.5 * (3.0 * u_back ** 2 - 1)).sum(axis=1) / (2.0 * n)
    return p1, p2
