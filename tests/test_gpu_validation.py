"""Validation at the workloads' real sizes and horizons.

* The plain single-dimer box at full size (30^3 periodic cells, 270,000
  solvent, one dimer): the FP64 engine against the FP64 oracle over 100
  collision periods (5,000 MD steps), every 1,000 steps.  Positions,
  velocities and the dimer within 1e-5 relative (|d| <= 1e-5 max(1, |ref|));
  species flags and counts identical.  A perturbation of 1e-13 in the
  velocities of the oracle grows to about 1e-7 over the same horizon, so the
  bar leaves two orders of magnitude for the summation-order differences.
* The FP32 production build against the FP64 run over the same horizon,
  through observables (total energy, momentum, species counts).
* The collective quasi-2D box at its real geometry (128x128x16 cells with z
  walls and the reactive floor, 2,621,440 solvent, 64 dimers): FP64 engine
  against the oracle over 120 MD steps (two collision periods and a bit).
* The FP32 reaction stage given the oracle's tables (distribute counts and
  first members identical by construction of the input): relabels identical.

The ensemble statistics live in test_gpu_statistics.py.
"""
import os

import numpy as np
import pytest

from gpu_helpers import min_image
from main_gb300 import Engine, config
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
REL = 1e-5


def _pair_full(cfg):
    o = Oracle(cfg, threads=THREADS)
    o.initial()
    e = Engine(cfg)
    e.upload_state(o.get_state())
    o.set_cell_order(e.cell_order())
    return o, e


def _rel_close(se, so, cfg, rel):
    """Largest |engine - oracle| / max(1, |oracle|) over positions (minimum
    image), velocities and the dimer state."""
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)
    worst = {}
    for i, k in enumerate("xyz"):
        d = se[k] - so[k]
        if i < 2 or cfg["geometry"] == config.GEOM_PERIODIC:
            d = min_image(d, L[i])
        worst[k] = float((np.abs(d) / np.maximum(1.0, np.abs(so[k]))).max())
    for k in ("vx", "vy", "vz"):
        worst[k] = float((np.abs(se[k] - so[k]) / np.maximum(1.0, np.abs(so[k]))).max())
    if len(so["dpos"]):
        dd = se["dpos"] - so["dpos"]
        for c in range(2 if cfg["geometry"] == config.GEOM_WALLS else 3):
            dd[:, c] = min_image(dd[:, c], L[c])
        worst["dpos"] = float((np.abs(dd) / np.maximum(1.0, np.abs(so["dpos"]))).max())
        worst["dvel"] = float((np.abs(se["dvel"] - so["dvel"]) / np.maximum(1.0, np.abs(so["dvel"]))).max())
    for k, v in worst.items():
        assert v <= rel, (k, v, worst)
    return worst


def test_plain_dimer_full_size_100_collision_periods_fp64():
    cfg = config.workload("c0", precision=64)
    assert (cfg["lx"], cfg["n_solvent"], cfg["n_dimers"]) == (30, 270000, 1)
    o, e = _pair_full(cfg)
    o.prepare()
    e.prepare()
    S = cfg["mpc_every"]
    for block in range(5):
        o.run(20 * S)
        e.run(20 * S)
        se, so = e.download_state(), o.get_state()
        _rel_close(se, so, cfg, REL)
        assert np.array_equal(se["flag"], so["flag"]), block
    oo, oe = o.observables(), e.observables()
    assert oo["cstep"] == oe["cstep"] == 100 * S
    assert np.array_equal(oo["species_count"], oe["species_count"])
    # catalysis and the bulk reaction both fired (the comparison is not vacuous)
    assert 0 < oo["species_count"][1] < cfg["n_solvent"]
    e_o = oo["kinetic_solvent"] + oo["kinetic_dimer"] + oo["potential"]
    e_e = oe["kinetic_solvent"] + oe["kinetic_dimer"] + oe["potential"]
    assert abs(e_o - e_e) <= REL * abs(e_o)


def _observable_series(cfg, periods, every):
    e = Engine(cfg)
    e.initial()
    e.prepare()
    out = []
    for _ in range(periods // every):
        e.run(every * cfg["mpc_every"])
        ob = e.observables()
        _, vd = e.dimer_axes(normalize=1)
        out.append(dict(ob, energy=ob["kinetic_solvent"] + ob["kinetic_dimer"] + ob["potential"], vdot=vd.copy()))
    return out


def test_plain_dimer_fp32_against_fp64_observables():
    """FP32 and FP64 builds from the same seeded input over 100 collision
    periods.  Rounding differences grow chaotically, so the comparison is
    through conserved or slowly varying quantities: total energy (both builds
    conserve it to the integration error), total momentum (FP64 reductions of
    both), and the B count (catalysis minus bulk decay), which may differ by
    the particles whose trajectories near the C sphere diverged."""
    c64 = config.workload("c0", precision=64)
    c32 = config.workload("c0", precision=32)
    a = _observable_series(c64, 100, 10)
    b = _observable_series(c32, 100, 10)
    e0 = abs(a[0]["energy"])
    for ra, rb in zip(a, b):
        assert abs(ra["energy"] - rb["energy"]) <= 2e-4 * e0, (ra["energy"], rb["energy"])
        assert np.abs(ra["momentum"] - rb["momentum"]).max() <= 1e-3, (ra["momentum"], rb["momentum"])
        nb_a, nb_b = ra["species_count"][1], rb["species_count"][1]
        assert abs(nb_a - nb_b) <= 5.0 * np.sqrt(max(nb_a, 1)) + 20, (nb_a, nb_b)
        assert ra["species_count"].sum() == rb["species_count"].sum() == c64["n_solvent"]


def test_collective_quasi2d_real_geometry_fp64():
    cfg = config.workload("c1", precision=64)
    assert (cfg["lx"], cfg["ly"], cfg["lz"], cfg["n_dimers"]) == (128, 128, 16, 64)
    o, e = _pair_full(cfg)
    import oracle.oracle as O
    o.set_list_mode(O.LISTS_CELLS)
    o.prepare()
    e.prepare()
    for chunk in (1, 49, 70):
        o.run(chunk)
        e.run(chunk)
        se, so = e.download_state(), o.get_state()
        _rel_close(se, so, cfg, 1e-9)
        assert np.array_equal(se["flag"], so["flag"]), chunk
    assert np.array_equal(o.observables()["species_count"], e.observables()["species_count"])


def _snap_state(st, cfg, rng, margin=2e-3):
    """Redraw every particle within `margin` of a cell face, of an LJ cutoff or
    of a list radius (cutoff + skin) at a uniform bulk position, so that the
    FP32 cell-relative conversion bins, lists and excludes exactly as FP64
    does.  Redrawn particles land outside every list radius."""
    st = {k: np.array(v, copy=True) for k, v in st.items()}
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)
    cut = 2.0 ** (1.0 / 6.0)
    pos = np.stack([st["x"], st["y"], st["z"]], axis=1)
    radii = [((cfg["rc"] if s % 2 == 0 else cfg["rn"]) * cut) for s in range(len(st["dpos"]))]

    def dist(p):
        out = []
        for s, R in enumerate(radii):
            d = p - st["dpos"][s]
            d -= L * np.round(d / L)
            out.append((np.linalg.norm(d, axis=1), R))
        return out

    def bad(p, fresh):
        f = p - np.floor(p)
        b = ((f < margin) | (f > 1.0 - margin)).any(axis=1)
        for r, R in dist(p):
            b |= np.abs(r - R) < margin
            b |= np.abs(r - R - cfg["skin"]) < margin
            if fresh:
                b |= r < R + cfg["skin"] + margin
        return b

    todo = np.nonzero(bad(pos, False))[0]
    for _ in range(200):
        if not len(todo):
            break
        pos[todo] = rng.random((len(todo), 3)) * L
        todo = todo[bad(pos[todo], True)]
    assert not len(todo)
    st["x"], st["y"], st["z"] = pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy()
    return st


@pytest.mark.parametrize("case", ["c0", "c2"])
def test_fp32_reaction_relabels_bit_exact(case):
    """The FP32 reaction stage (float rate constants, 32-bit Philox words, the
    exact FP64 draw only inside the guard band) makes the oracle's decisions:
    with inputs binned identically in both precisions (checked: distribute
    counts, first members and excluded cells equal), the species after the
    stage are identical, over several collision steps' draws."""
    if case == "c0":
        cfg = config.workload("c0", precision=32, k=[0.05, 0, 0, 0, 0, 0])
    else:
        cfg = config.workload("c2", scale=0.25, precision=32, n_dimers=8)
    o = Oracle(cfg, threads=THREADS)
    o.initial()
    st = o.get_state()
    rng = np.random.default_rng(7)
    if case == "c0":
        # half of the solvent B, so the bulk B -> A reaction fires often
        st["flag"] = np.where(rng.random(cfg["n_solvent"]) < 0.5, 1, 0).astype(np.int32)
    st = _snap_state(st, cfg, rng)
    fired = 0
    for step in (50, 100, 150, 200, 250, 300):
        o.set_state(st)
        e = Engine(cfg)
        e.upload_state(st)
        o.set_cell_order(e.cell_order())
        o.set_cstep(0)   # prepare sorts at step 0 (main_pattern.f95:170-172), as the fresh engine does
        # the lists of prepare decide the inside/outside order of the
        # distribute lists (distribute_mod.f95:95-182)
        o.prepare()
        e.prepare()
        o.set_cstep(step)
        e.set_step(step)
        pre = o.get_state()["flag"]
        o.distribute()
        e.distribute()
        cnt_o, first_o = o.distribute_result()
        cnt_e, first_e = e.distribute_result()
        assert np.array_equal(cnt_o, cnt_e)
        assert np.array_equal(first_o, first_e)
        if cfg["exclusion"] == config.EXCL_CELLS:
            assert np.array_equal(o.affected(), e.affected())
        o.reaction()
        e.reaction()
        fo, fe = o.get_state()["flag"], e.download_state()["flag"]
        assert np.array_equal(fo, fe), (step, int((fo != fe).sum()))
        fired += int((fo != pre).sum())
        e.close()
    assert fired > 100, fired
