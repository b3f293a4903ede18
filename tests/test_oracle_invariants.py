"""Known answers and invariants of the oracle restatement (CPU).

The reference has no tests or golden outputs; these pin the oracle against
facts the reference code itself fixes:
  * the collision conserves each cell's momentum and kinetic energy
    (mpc_rotation_mod.f95:205-228 is a rotation about the cell centre of mass);
  * the Selkov RKMPC decision equals the nested branches of
    RMPC_SelkovDimer.f90:127-324 (restated literally below);
  * RATTLE holds the bond to the tolerances of evolve_mod.f95:105,116;
  * the reactive floor patterns of reactive_grid_mod.f95:8-99;
  * the sort follows hilbert.txt (sort_hilbert_mod.f95:57-77);
  * total momentum is conserved by the whole time step.
"""
import math

import numpy as np
import pytest

from conftest import hilbert_order
from main_gb300 import config
from oracle.oracle import Oracle


def small(name="c0", **kw):
    return config.workload(name, scale=0.55 if name == "c0" else 0.25, **kw)


def test_collision_conserves_cell_momentum_and_energy():
    cfg = small("c0", n_dimers=0)
    o = Oracle(cfg)
    o.initial()
    o.set_cstep(50)
    before = o.get_state()
    o.mpc_rotation()
    after = o.get_state()
    cells = o.new_cell()
    nc = o.cell_rotation()[2].size
    for v in ("vx", "vy", "vz"):
        pb = np.bincount(cells, weights=before[v], minlength=nc)
        pa = np.bincount(cells, weights=after[v], minlength=nc)
        assert np.max(np.abs(pa - pb)) < 1e-12
    kb = np.bincount(cells, weights=before["vx"] ** 2 + before["vy"] ** 2 + before["vz"] ** 2, minlength=nc)
    ka = np.bincount(cells, weights=after["vx"] ** 2 + after["vy"] ** 2 + after["vz"] ** 2, minlength=nc)
    assert np.max(np.abs(ka - kb)) < 1e-12


def test_collision_rotates_by_the_angle():
    cfg = small("c0", n_dimers=0, rot_angle=2 * math.pi / 3)
    o = Oracle(cfg)
    o.initial()
    o.set_cstep(100)
    b = o.get_state()
    o.mpc_rotation()
    a = o.get_state()
    cm, axis, _ = o.cell_rotation()
    c = o.new_cell()
    db = np.stack([b["vx"], b["vy"], b["vz"]], 1) - cm[c]
    da = np.stack([a["vx"], a["vy"], a["vz"]], 1) - cm[c]
    u = axis[c]
    # components along the axis are kept; the perpendicular parts turn by rotang
    assert np.allclose((db * u).sum(1), (da * u).sum(1), atol=1e-12)
    pb = db - (db * u).sum(1)[:, None] * u
    pa = da - (da * u).sum(1)[:, None] * u
    nb, na = np.linalg.norm(pb, axis=1), np.linalg.norm(pa, axis=1)
    ok = nb > 1e-6
    cosang = (pb[ok] * pa[ok]).sum(1) / (nb[ok] * na[ok])
    assert np.allclose(cosang, math.cos(cfg["rot_angle"]), atol=1e-9)


def _selkov_nested(k, tau, nF, nG, nI, x1, x2):
    """RMPC_SelkovDimer.f90:127-324 restated branch by branch.
    Returns (target species code, new code) or None."""
    a1 = k[0]; a2 = k[1] * nF; a5 = k[4] * nG; a6 = k[5]
    a3 = 0.0 if nG == 0 else k[2] * nF * nG * (nG - 1)
    a4 = 0.0 if nG <= 1 else k[3] * nG * (nG - 1) * (nG - 2)
    if nI == 0:
        a1 = 0.0; a6 = 0.0
    a00 = a1 + a2 + a3 + a4 + a5 + a6
    p = 1 - math.exp(-a00 * tau)
    r = a00 * x1
    if not (p > x2):
        return None
    I, F, G = (3,), (0,), (1,)
    if nI > 0:
        if nF == 0:
            if nG == 0:
                if r < a1: return (3, 0)
                if a1 <= r < a00: return (3, 1)
            elif 0 < nG <= 2:
                if r < a1: return (3, 0)
                if a1 <= r < a1 + a5: return (1, 3)
                if a1 + a5 <= r < a00: return (3, 1)
            else:
                if r < a1: return (3, 0)
                if a1 <= r < a1 + a4: return (1, 0)
                if a1 + a4 <= r < a1 + a4 + a5: return (1, 3)
                if a1 + a4 + a5 <= r < a00: return (3, 1)
        else:
            if nG == 0:
                if r < a1: return (3, 0)
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a00: return (3, 1)
            elif nG == 1:
                if r < a1: return (3, 0)
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a1 + a2 + a5: return (1, 3)
                if a1 + a2 + a5 <= r < a00: return (3, 1)
            elif nG == 2:
                if r < a1: return (3, 0)
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a1 + a2 + a3: return (0, 1)
                if a1 + a2 + a3 <= r < a1 + a2 + a3 + a5: return (1, 3)
                if a1 + a2 + a3 + a5 <= r < a00: return (3, 1)
            else:
                if r < a1: return (3, 0)
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a1 + a2 + a3: return (0, 1)
                if a1 + a2 + a3 <= r < a1 + a2 + a3 + a4: return (1, 0)
                if a1 + a2 + a3 + a4 <= r < a1 + a2 + a3 + a4 + a5: return (1, 3)
                if a1 + a2 + a3 + a4 + a5 <= r < a00: return (3, 1)
    else:
        if nF == 0:
            if nG == 0:
                return None
            elif 0 < nG <= 2:
                if a1 <= r < a00: return (1, 3)
            else:
                if a1 <= r < a1 + a4: return (1, 0)
                if a1 + a4 <= r < a00: return (1, 3)
        else:
            if nG == 0:
                if a1 <= r < a00: return (0, 3)
            elif nG == 1:
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a00: return (1, 3)
            elif nG == 2:
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a1 + a2 + a3: return (0, 1)
                if a1 + a2 + a3 <= r < a00: return (1, 3)
            else:
                if a1 <= r < a1 + a2: return (0, 3)
                if a1 + a2 <= r < a1 + a2 + a3: return (0, 1)
                if a1 + a2 + a3 <= r < a1 + a2 + a3 + a4: return (1, 0)
                if a1 + a2 + a3 + a4 <= r < a00: return (1, 3)
    return None


def test_selkov_cell_decision_matches_nested_branches():
    # a one-cell box: each particle sits in cell 0, counts chosen per trial
    rng = np.random.default_rng(7)
    ks = [[0.0009485, 0.0001, 0.0004, 0.0004, 0.001, 0.0001], [1.0, 0.1, 1.0, 0.0, 0.01, 0.0],
          [0.3, 0.2, 0.05, 0.02, 0.4, 0.1]]
    checked = 0
    for k in ks:
        for trial in range(60):
            nF, nG, nI = (int(v) for v in rng.integers(0, 6, 3))
            n = nF + nG + nI
            if n == 0:
                continue
            cfg = config.base_config(lx=1, ly=1, lz=1, geometry=config.GEOM_PERIODIC, n_dimers=0,
                                     kinetics=config.KIN_SELKOV, exclusion=config.EXCL_CELLS,
                                     rotation_sense=-1, n_solvent=n, init_count=[nF, nG, 0, nI],
                                     k=k, mpc_dt=0.5 if trial % 2 else 5.0, cell_capacity=200, seed=trial + 11)
            o = Oracle(cfg)
            flag = np.array([0] * nF + [1] * nG + [3] * nI, dtype=np.int32)
            z = np.full(n, 0.5)
            o.set_state(dict(x=z, y=z, z=z, vx=z * 0, vy=z * 0, vz=z * 0, flag=flag))
            o.set_cstep(trial * 50)
            o.distribute()
            o.reaction()
            after = o.get_state()["flag"]
            from oracle.oracle import contract_u01
            x1 = contract_u01(cfg["seed"], 3, 0, 0, trial * 50, 0)
            x2 = contract_u01(cfg["seed"], 3, 0, 0, trial * 50, 1)
            want = _selkov_nested(k, cfg["mpc_dt"], nF, nG, nI, x1, x2)
            exp = flag.copy()
            if want is not None:
                tgt, new = want
                idx = np.nonzero(flag == tgt)[0]
                exp[idx[0]] = new
            assert (after == exp).all(), (k, nF, nG, nI, want)
            checked += 1
    assert checked > 100


def test_rattle_holds_bond_and_momentum_conserved():
    cfg = small("c0")
    o = Oracle(cfg)
    o.initial()
    o.prepare()
    o.run(120)
    st = o.get_state()
    d = st["dpos"][0] - st["dpos"][1]
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)
    d -= L * np.round(d / L)
    assert abs(d @ d - cfg["dcn"] ** 2) < 1e-6                     # evolve_mod.f95:105
    dv = st["dvel"][0] - st["dvel"][1]
    assert abs(2 * dv @ d) < 1e-8                                  # evolve_mod.f95:116
    ob = o.observables()
    assert np.max(np.abs(ob["momentum"])) < 1e-9
    assert ob["species_count"][1] > 0                               # catalysis made B


@pytest.mark.parametrize("rtype", [1, 2, 3, 4, 5, 6, 7])
def test_reactive_grid_patterns(rtype):
    cfg = config.base_config(lx=64, ly=64, lz=8, geometry=config.GEOM_WALLS, n_dimers=0,
                             react_box_type=rtype, n_solvent=64)
    o = Oracle(cfg)
    o.prepare()
    t = o.reactive_grid().reshape(64, 64)
    covered = t.mean()
    expect = {1: 0.5, 2: 0.5, 6: 1.0, 7: 0.0}
    if rtype in expect:
        assert abs(covered - expect[rtype]) < 1e-9
    elif rtype == 3:
        assert 0.25 < covered < 0.35          # disc of radius 20 in a 64x64 floor
    elif rtype == 5:
        assert abs(covered - 8 / 64) < 1e-9   # strip of 8 columns
    else:
        assert covered < 0.05


def test_sort_follows_hilbert_fixture():
    order, box, sha = hilbert_order()
    import hashlib
    assert hashlib.sha256(order.tobytes()).digest() == sha
    assert sorted(order.tolist()) == list(range(box[0] * box[1] * box[2]))
    cfg = config.base_config(lx=box[0], ly=box[1], lz=box[2], geometry=config.GEOM_WALLS, n_dimers=0,
                             n_solvent=3 * box[0] * box[1] * box[2], sort_every=1)
    o = Oracle(cfg)
    o.initial()
    o.set_cell_order(order)
    before = o.get_state()
    o.sort()
    after = o.get_state()
    cid = (np.floor(after["x"]) + box[0] * (np.floor(after["y"]) + box[1] * np.floor(after["z"]))).astype(int)
    rank = np.empty(order.size, int)
    rank[order] = np.arange(order.size)
    assert (np.diff(rank[cid]) >= 0).all()           # cells in hilbert.txt order
    # stable: within a cell the old index order is kept
    cb = (np.floor(before["x"]) + box[0] * (np.floor(before["y"]) + box[1] * np.floor(before["z"]))).astype(int)
    perm = np.lexsort((np.arange(cb.size), rank[cb]))
    assert np.array_equal(after["x"], before["x"][perm])


def test_selkov_driver_matches_hybrid_driver():
    """Main_SelkovDimer.f90's full velocity-Verlet driver and the collective
    driver with the Selkov options are the same dynamics for one dimer whose
    shells do not overlap; short trajectories agree to FP64 round-off."""
    cfg = config.base_config(lx=14, ly=14, lz=14, geometry=config.GEOM_PERIODIC, n_dimers=1,
                             kinetics=config.KIN_SELKOV, exclusion=config.EXCL_CELLS,
                             catalysis=config.CAT_PROBABILISTIC, rotation_sense=-1, rc=2.0, rn=4.0, dcn=7.0,
                             rp_ab=1.0, rp_ba=0.0, cell_capacity=200, sort_every=0,
                             init_count=[0, 0, 0, 0], k=[0.0009485, 0.0001, 0.0004, 0.0004, 0.001, 0.0001],
                             mpc_dt=0.1, md_dt=0.005)
    n = cfg["n_solvent"]
    cfg["init_count"] = [n // 3, n // 12, 0, n - n // 3 - n // 12]
    a = Oracle(cfg)
    a.initial()
    st = a.get_state()
    b = Oracle(cfg)
    b.set_state(st)
    a.prepare()
    b.selkov_prepare()
    for _ in range(3):
        a.run(20)
        for _ in range(20):
            b.selkov_step()
    sa, sb = a.get_state(), b.get_state()
    for k in ("x", "y", "z"):
        d = np.abs(sa[k] - sb[k])
        d = np.minimum(d, cfg["lx"] - d)
        assert d.max() < 1e-9, k
    for k in ("vx", "vy", "vz"):
        assert np.max(np.abs(sa[k] - sb[k])) < 1e-9, k
    assert (sa["flag"] == sb["flag"]).mean() > 0.999
    assert np.max(np.abs(sa["dpos"] - sb["dpos"])) < 1e-9


@pytest.mark.parametrize("name", ["c0", "c1"])
def test_cell_list_search_gives_the_same_run(name):
    # the cell-binned pair search (a CPU baseline for comparison) finds the
    # same lists in the same order as neighbour_list_mod.f95's all-pairs loop
    import oracle.oracle as O
    cfg = small(name)
    a = Oracle(cfg, threads=4)
    a.initial()
    st = a.get_state()
    b = Oracle(cfg, threads=4)
    b.set_state(st)
    b.set_list_mode(O.LISTS_CELLS)
    a.prepare()
    b.prepare()
    a.run(60)
    b.run(60)
    sa, sb = a.get_state(), b.get_state()
    for k in ("x", "y", "z", "vx", "vy", "vz", "flag", "dpos", "dvel"):
        assert np.array_equal(sa[k], sb[k]), k


def test_catalysis_on_exit_converts_exactly_the_leavers():
    """MPCMD_CAT_ON_EXIT: an A inside the C cutoff at one step's force
    evaluation and outside it at the next becomes a B, and nothing else
    changes species (bulk reaction off)."""
    from main_gb300 import config
    cfg = config.workload("c0", scale=0.55, precision=64, catalysis=config.CAT_ON_EXIT, k=[0, 0, 0, 0, 0, 0])
    from oracle.oracle import Oracle
    o = Oracle(cfg, threads=2)
    o.initial()
    o.prepare()
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)
    cutC = cfg["rc"] * 2.0 ** (1.0 / 6.0)

    def inside(st):
        d = np.stack([st["x"], st["y"], st["z"]], axis=1) - st["dpos"][0]
        d -= L * np.round(d / L)
        return (d * d).sum(axis=1) <= cutC * cutC

    o.step()
    prev = o.get_state()
    converted = 0
    for _ in range(150):
        o.step()
        cur = o.get_state()
        leavers = inside(prev) & ~inside(cur) & (prev["flag"] == 0)
        expect = prev["flag"].copy()
        expect[leavers] = 1
        assert np.array_equal(cur["flag"], expect)
        converted += int(leavers.sum())
        prev = cur
    assert converted > 10, converted
