"""Device output observables against the oracle: mpcmd_concentration
(output_mod.f95:482-575) and mpcmd_dimer_axes (output_mod.f95:826-846,
Output_SelkovDimer.f90:146-172).

* The concentration kernel bins the host view of the positions that
  mpcmd_download_state returns (inside-list members at the current step,
  outside particles at the last rebuild, free-flight members streamed): the
  oracle's binning of the downloaded state must give bit-identical fields.
  The runs stop between rebuilds, so deferred and free-flight particles are
  present.
* Against the FP64 oracle's own trajectory the counts agree up to the
  particles within the 1e-9 trajectory tolerance of a bin or slab face.
* Dimer axes: 1e-12 against numpy on the downloaded sphere state.
"""
import math

import numpy as np
import pytest

from gpu_helpers import CASES, pair
from main_gb300 import Engine, MpcmdError, config
from oracle import oracle as O

pytestmark = pytest.mark.gpu

KEYS = ("totals", "c1d_a", "c1d_b", "xy_a", "xy_b", "xz_a", "xz_b", "yz_a", "yz_b")


def conc_params(cfg):
    hw = cfg["rc"] * 2 ** (1.0 / 6.0)   # cutoffC, the reference's slab half thickness
    return (cfg["lx"] / 2 + 0.3, cfg["ly"] / 2 - 0.2, cfg["lz"] / 2 + 0.1, hw, 0.5, 0.5, 0.5)


def engine_fields(e, prm):
    return e.concentration(*prm)


def state_fields(st, cfg, prm):
    return O.concentration(st["x"], st["y"], st["z"], st["flag"], (cfg["lx"], cfg["ly"], cfg["lz"]), prm)


@pytest.mark.parametrize("case", ["c0", "c1", "c2"])
@pytest.mark.parametrize("prec", [64, 32])
def test_concentration_bins_the_download_view(case, prec):
    cfg = CASES[case](prec)
    e = Engine(cfg)
    e.initial()
    e.prepare()
    prm = conc_params(cfg)
    for chunk in (37, 40):      # mid-period, then past a collision step
        e.run(chunk)
        got = engine_fields(e, prm)
        ref = state_fields(e.download_state(), cfg, prm)
        for k in KEYS:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=(case, prec, k))
        assert got["totals"][0] + got["totals"][1] > 0


@pytest.mark.parametrize("case", ["c0", "c1", "c2"])
def test_concentration_follows_the_oracle_trajectory_fp64(case):
    cfg = CASES[case](64)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    o.run(60)
    e.run(60)
    prm = conc_params(cfg)
    got = engine_fields(e, prm)
    ref = state_fields(o.get_state(), cfg, prm)
    np.testing.assert_array_equal(got["totals"], ref["totals"])
    vols = {"c1d": prm[4] * cfg["ly"] * 2 * prm[3], "xy": prm[4] * prm[5] * 2 * prm[3],
            "xz": prm[4] * prm[6] * 2 * prm[3], "yz": prm[5] * prm[6] * 2 * prm[3]}
    for k in KEYS[1:]:
        dc = np.abs(np.rint((got[k] - ref[k]) * vols[k.split("_")[0]]))
        assert dc.sum() <= 2, (case, k, dc.sum())


def test_concentration_rejects_bad_parameters():
    cfg = CASES["c0"](64)
    e = Engine(cfg)
    e.initial()
    with pytest.raises(MpcmdError) as ex:
        e.concentration(1.0, 1.0, 1.0, 1.0, 0.0, 0.5, 0.5)
    assert ex.value.status == 1


@pytest.mark.parametrize("case", ["c0", "c1", "c2"])
def test_dimer_axes(case):
    cfg = CASES[case](64)
    e = Engine(cfg)
    e.initial()
    e.prepare()
    e.run(30)
    st = e.download_state()
    X, V = st["dpos"], st["dvel"]
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)
    d = X[0::2] - X[1::2]
    for c in range(3 if cfg["geometry"] == config.GEOM_PERIODIC else 2):
        d[:, c] = np.where(d[:, c] > 0.5 * L[c], d[:, c] - L[c], np.where(d[:, c] < -0.5 * L[c], d[:, c] + L[c], d[:, c]))
    ln = np.linalg.norm(d, axis=1)
    mc, mn = e.cfg["mc"], e.cfg["mn"]
    vcm = (mc * V[0::2] + mn * V[1::2]) / (mc + mn)
    nuc0, vd = e.dimer_axes(0)
    nuc1, _ = e.dimer_axes(1)
    np.testing.assert_allclose(nuc0, d / e.cfg["dcn"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(nuc1, d / ln[:, None], rtol=0, atol=1e-12)
    np.testing.assert_allclose(vd, (vcm * d / ln[:, None]).sum(axis=1), rtol=0, atol=1e-12)
    # the bond is held at Dcn by RATTLE, so both normalisations agree closely
    assert np.abs(ln - e.cfg["dcn"]).max() < 1e-5


@pytest.mark.parametrize("case", ["c0", "c1", "c2"])
@pytest.mark.parametrize("prec", [64, 32])
def test_observables_match_the_downloaded_state(case, prec):
    """mpcmd_observables' solvent sums (output_mod.f95:681-806) against FP64
    sums over the downloaded host state: species counts exact; momentum and
    kinetic energy within 1e-6 of the sum of the magnitudes (the FP32 build
    sums compensated FP32 terms per thread and reduces in FP64)."""
    cfg = CASES[case](prec)
    e = Engine(cfg)
    e.initial()
    e.prepare()
    e.run(37)
    st = e.download_state()
    obs = e.observables()
    m = np.asarray(cfg["mass"], float)[st["flag"]]
    v = np.stack([st["vx"], st["vy"], st["vz"]])
    p = (m * v).sum(axis=1)
    pabs = np.abs(m * v).sum(axis=1)
    ke = 0.5 * (m * (v * v).sum(axis=0)).sum()
    np.testing.assert_array_equal(obs["species_count"], np.bincount(st["flag"], minlength=4))
    assert np.all(np.abs(obs["solvent_momentum"] - p) <= 1e-6 * pabs + 1e-9), (obs["solvent_momentum"], p)
    assert abs(obs["kinetic_solvent"] - ke) <= 1e-6 * ke
