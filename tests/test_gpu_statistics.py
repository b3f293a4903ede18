"""Ensemble statistics of the FP32 production build on the plain single-dimer
box at full size (30^3 periodic cells, 270,000 solvent, one dimer, kT = 1/6,
rotation angle 120 degrees, collision interval 0.5).

* Maxwell velocities (initial_mod.f95:274-345 draws them; the collision and
  the MD keep them): Kolmogorov-Smirnov test of every component against
  N(0, kT/m) after 20 collision periods, and the kinetic temperature.
* Momentum conservation: the total momentum (FP64 reduction of solvent and
  spheres) drifts by at most 1e-10 of sum |p_i| over 100 collision periods in
  the FP64 build.  The FP32 build's drift is a random walk: every collision
  rounds each stored velocity (half an ulp, about 1e-8 at v ~ 0.4) and each
  cell's FP32 sum (its mean is off by about sqrt(n) ulps, and the rotation
  turns that error), which over 100 periods of 270,000 particles in 27,000
  cells gives a standard deviation near 5e-10 of sum |p_i| per component;
  the cell sums are FP32 atomics in no fixed order, so the walk differs
  from run to run (the worst of 10 checkpoints x 3 components was seen
  between 1e-9 and 2.2e-9).  The bound is 1e-8.
* Solvent self-diffusion against the FP64 reference algorithm (the oracle) on
  independent seeds, within two standard errors of the difference (standard
  errors from the spread of the replicas), and both within 10 % of the
  molecular-chaos formula of
  rotational_code/linear_periodic_langevin/Code/derived_quantities_mod.f90:33,
  D = (kT tau / 2m) (3 n / ((n - 1 + e^-n)(1 - cos a)) - 1).  At this mean
  free path (0.2 cells) correlated collisions raise D above the formula by
  about 8 % (measured with the oracle: 0.0548 against 0.0509), so the formula
  is a bias check, not a 2-SE target.
* Dimer propulsion speed (the axial velocity of Output_SelkovDimer.f90:
  168-172) of FP32 and FP64 ensembles, within two standard errors.

The two-ensemble comparisons state their result in standard errors of the
difference (z in the assertion message).  The GPU runs are not
bit-reproducible (the FP32 and FP64 cell sums and sphere sums are atomics in
no fixed order, and the MD amplifies the last-bit differences), so every run
of these tests is a fresh draw: with 6 + 6 and 8 + 8 replicas a correct build
exceeds 2 SE in about 7 % of runs (Student t, 10 and 14 degrees of freedom).
The assertions therefore take 3 SE (about 1 % of correct runs); every run
recorded before this bound was set passed at 2 SE.
"""
import math
import os

import numpy as np
import pytest

from gpu_helpers import min_image
from main_gb300 import Engine, config
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
Z_BOUND = 3.0   # standard errors of the difference (see the module docstring)


def _engine(prec, seed=1):
    cfg = config.workload("c0", precision=prec, seed=seed)
    e = Engine(cfg)
    e.initial()
    e.prepare()
    return cfg, e


def test_maxwell_velocities_fp32():
    stats = pytest.importorskip("scipy.stats")
    cfg, e = _engine(32)
    e.run(20 * cfg["mpc_every"])
    st = e.download_state()
    sigma = math.sqrt(cfg["kT"] / cfg["mass"][0])
    v = np.concatenate([st["vx"], st["vy"], st["vz"]])
    T = float((v ** 2).mean()) * cfg["mass"][0]
    assert abs(T - cfg["kT"]) <= 5e-3 * cfg["kT"], T
    for k in ("vx", "vy", "vz"):
        res = stats.kstest(st[k] / sigma, "norm")
        assert res.pvalue > 1e-3, (k, res.statistic, res.pvalue)


def _abs_momentum(st, cfg):
    m = np.asarray(cfg["mass"])[st["flag"] & 3]
    p = m * (np.abs(st["vx"]) + np.abs(st["vy"]) + np.abs(st["vz"]))
    sm = np.array([cfg["mc"], cfg["mn"]])
    return float(p.sum() + (np.abs(st["dvel"]).sum(axis=1) * sm).sum())


@pytest.mark.parametrize("prec,bound", [(64, 1e-10), (32, 1e-8)])
def test_momentum_conservation(prec, bound):
    cfg, e = _engine(prec)
    p0 = e.observables()["momentum"]
    scale = _abs_momentum(e.download_state(), cfg)
    worst = 0.0
    for _ in range(10):
        e.run(10 * cfg["mpc_every"])
        p = e.observables()["momentum"]
        worst = max(worst, float(np.abs(p - p0).max()) / scale)
    assert worst <= bound, worst


def _msd_diffusion(get_state, run_period, cfg, periods, t1):
    """D from the slope of the mean squared displacement between collision
    periods t1 and `periods` (positions unwrapped by the minimum image of each
    period's displacement)."""
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)[:, None]
    st = get_state()
    prev = np.stack([st["x"], st["y"], st["z"]])
    disp = np.zeros_like(prev)
    msd = {}
    for k in range(1, periods + 1):
        run_period()
        st = get_state()
        cur = np.stack([st["x"], st["y"], st["z"]])
        d = cur - prev
        disp += d - L * np.round(d / L)
        prev = cur
        if k in (t1, periods):
            msd[k] = float((disp ** 2).sum(axis=0).mean())
    return (msd[periods] - msd[t1]) / (6.0 * (periods - t1) * cfg["mpc_dt"])


def test_solvent_diffusion_fp32_against_reference_algorithm():
    periods, t1, reps = 40, 15, 6
    d32, d64 = [], []
    for r in range(reps):
        cfg, e = _engine(32, seed=100 + r)
        S = cfg["mpc_every"]
        d32.append(_msd_diffusion(e.download_state, lambda: e.run(S), cfg, periods, t1))
        e.close()
        c64 = config.workload("c0", precision=64, seed=200 + r)
        o = Oracle(c64, threads=THREADS)
        o.initial()
        o.prepare()
        d64.append(_msd_diffusion(o.get_state, lambda: o.run(S), c64, periods, t1))
    m32, m64 = np.mean(d32), np.mean(d64)
    se = math.sqrt(np.var(d32, ddof=1) / reps + np.var(d64, ddof=1) / reps)
    z = abs(m32 - m64) / se
    assert z <= Z_BOUND, (m32, m64, se, z)
    n = 10.0
    a = cfg["rot_angle"]
    formula = cfg["kT"] * cfg["mpc_dt"] / (2.0 * cfg["mass"][0]) * (
        3.0 * n / ((n - 1.0 + math.exp(-n)) * (1.0 - math.cos(a))) - 1.0)
    for m in (m32, m64):
        assert abs(m - formula) <= 0.10 * formula, (m, formula)


def test_dimer_propulsion_speed_fp32_against_fp64():
    periods, skip, reps = 100, 10, 8
    speeds = {32: [], 64: []}
    for prec in (32, 64):
        for r in range(reps):
            cfg, e = _engine(prec, seed=300 + r)
            vs = []
            for k in range(periods):
                e.run(cfg["mpc_every"])
                if k >= skip:
                    vs.append(float(e.dimer_axes(normalize=1)[1][0]))
            speeds[prec].append(np.mean(vs))
            e.close()
    a, b = np.array(speeds[32]), np.array(speeds[64])
    se = math.sqrt(a.var(ddof=1) / reps + b.var(ddof=1) / reps)
    z = abs(a.mean() - b.mean()) / se
    assert z <= Z_BOUND, (a.mean(), b.mean(), se, z)
