"""The rotor variant of the oracle (rotational_code/2d_array and
linear_periodic_ci) against known answers of the reference code (CPU):

  * the grid and line layouts of the initial placement
    (2d_array/initial_mod.f95:68-90, linear_periodic_ci/initial_mod.f95:72-88),
    restated here in numpy from the same draws;
  * RATTLE holds every rotor's midpoint at its anchor and the bond length to
    the tolerances of 2d_array/evolve_mod.f95:99-105 and the midpoint velocity
    to those of :116-122;
  * the harmonic tether of forces_mod.f95:177-201 is the only force on an
    isolated rotor's spheres besides the solvent (no motor-motor LJ, no 9-3
    wall);
  * the anchors survive set/get and follow the state exchange.
"""
import math
import os

import numpy as np
import pytest

from main_gb300 import config
from oracle import oracle as O

TAG_INIT_DIMER = 5


def rotor_cfg(name="rot", **kw):
    return config.workload(name, scale=0.5 if name == "rot" else 0.25, **kw)


def expected_layout(cfg):
    """Sphere positions of the layout, restated from the reference formulas."""
    cut = 2.0 ** (1.0 / 6.0)
    nd = cfg["n_dimers"]
    dcn, rc, sep = cfg["dcn"], cfg["rc"], cfg["layout_sep"]
    w = dcn + 2.0 * rc * cut
    out = np.zeros((2 * nd, 3))
    for i in range(nd):
        theta = 2.0 * math.pi * O.contract_u01(cfg["seed"], TAG_INIT_DIMER, i, 0, 0, 0)
        if cfg["layout"] == config.LAYOUT_GRID:
            rows, cols = cfg["layout_rows"], cfg["layout_cols"]
            j, k = i // cols, i % cols
            cx = 0.5 * (cfg["lx"] - w * cols - sep * (cols - 1)) + 0.5 * w + k * (w + sep)
            cy = 0.5 * (cfg["ly"] - (w + sep) * (rows - 1) - w) + 0.5 * w + j * (w + sep)
        else:
            cx = 0.5 * sep + 0.5 * w + i * (w + sep)
            cy = cfg["ly"] * 0.5
        out[2 * i] = (cx + 0.5 * dcn * math.cos(theta), cy + 0.5 * dcn * math.sin(theta), cfg["tether_z"])
        out[2 * i + 1] = (cx - 0.5 * dcn * math.cos(theta), cy - 0.5 * dcn * math.sin(theta), cfg["tether_z"])
    return out


@pytest.mark.parametrize("name", ["rot", "rot_line"])
def test_layout_matches_reference_formulas(name):
    cfg = rotor_cfg(name)
    o = O.Oracle(cfg, threads=4)
    o.initial()
    st = o.get_state()
    exp = expected_layout(cfg)
    assert np.abs(st["dpos"] - exp).max() <= 1e-12
    # anchors are the midpoints of the placed rotors, in the box plane z = zdimeq
    mid = 0.5 * (st["dpos"][0::2] + st["dpos"][1::2])
    assert np.array_equal(o.get_anchors(), mid)
    assert np.all(mid[:, 2] == cfg["tether_z"])
    # neighbouring motors are a pitch apart (sep = 0 for the grid workload)
    pitch = cfg["dcn"] + 2.0 * cfg["rc"] * 2.0 ** (1.0 / 6.0) + cfg["layout_sep"]
    assert abs((mid[1, 0] - mid[0, 0]) - pitch) <= 1e-12
    # no solvent particle starts inside a sphere's LJ range
    d = st["dpos"]
    for s in range(d.shape[0]):
        dx = st["x"] - d[s, 0]
        dy = st["y"] - d[s, 1]
        dx -= cfg["lx"] * np.round(dx / cfg["lx"])
        dy -= cfg["ly"] * np.round(dy / cfg["ly"])
        r2 = dx * dx + dy * dy + (st["z"] - d[s, 2]) ** 2
        assert r2.min() >= (cfg["rc"] * 2.0 ** (1.0 / 6.0)) ** 2


@pytest.mark.parametrize("name", ["rot", "rot_line"])
def test_rattle_holds_anchor_bond_and_midpoint_velocity(name):
    cfg = rotor_cfg(name)
    o = O.Oracle(cfg, threads=4)
    o.initial()
    anchors = o.get_anchors().copy()
    o.prepare()
    o.run(3 * cfg["mpc_every"])
    st = o.get_state()
    d = st["dpos"].reshape(-1, 2, 3)
    v = st["dvel"].reshape(-1, 2, 3)
    mid = 0.5 * (d[:, 0] + d[:, 1])
    assert np.abs(mid - anchors).max() < 1e-6
    bond2 = ((d[:, 0] - d[:, 1]) ** 2).sum(axis=1)
    assert np.abs(bond2 - cfg["dcn"] ** 2).max() < 1e-6
    assert np.abs(0.5 * (v[:, 0] + v[:, 1])).max() < 1e-8
    # the rotors turn (the solvent pushes them) and stay near the tether plane
    assert np.abs(v).max() > 0.0
    assert np.abs(d[:, :, 2] - cfg["tether_z"]).max() < 0.05
    assert o.status() == 0


def test_tether_and_no_motor_motor_forces():
    # two rotors whose spheres overlap in LJ range: with the rotor variant the
    # sphere forces are the solvent forces plus the tether only
    cfg = rotor_cfg("rot_line", n_dimers=2, layout=config.LAYOUT_LINE, layout_sep=-3.0, em=1.0,
                    n_solvent=4, init_count=[4, 0, 0, 0])
    o = O.Oracle(cfg, threads=1)
    st = {k: np.array([1.0, 2.0, 3.0, 4.0]) for k in ("x", "y")}
    st["z"] = np.full(4, cfg["lz"] - 0.5)
    for k in ("vx", "vy", "vz"):
        st[k] = np.zeros(4)
    st["flag"] = np.zeros(4, dtype=np.int32)
    dz = 0.01
    st["dpos"] = np.array([[20.0, 8.0, cfg["tether_z"] + dz], [25.0, 8.0, cfg["tether_z"] + dz],
                           [27.0, 8.0, cfg["tether_z"] - dz], [32.0, 8.0, cfg["tether_z"] - dz]])
    st["dvel"] = np.zeros((4, 3))
    o.set_state(st)
    o.prepare()
    o.run(1)
    got = o.get_state()
    f = got["dforce"]
    # the tether force -k (z - zeq) at the positions after the RATTLE step
    dzs = got["dpos"][:, 2] - cfg["tether_z"]
    assert np.allclose(f[:, 2], -cfg["tether_k"] * dzs, rtol=0, atol=1e-9)
    # sphere 1 of rotor 0 and sphere 0 of rotor 1 are 2 apart: a motor-motor
    # LJ force would be large; the rotor variant has none
    assert np.abs(f[:, 0]).max() == 0.0 and np.abs(f[:, 1]).max() == 0.0


def test_anchor_exchange():
    cfg = rotor_cfg("rot")
    o = O.Oracle(cfg, threads=2)
    o.initial()
    st = o.get_state()
    st["dpos"] = st["dpos"] + np.array([0.25, -0.5, 0.0])
    o.set_state(st)
    mid = 0.5 * (st["dpos"][0::2] + st["dpos"][1::2])
    assert np.array_equal(o.get_anchors(), mid)
    new = mid + 0.125
    o.set_anchors(new)
    assert np.array_equal(o.get_anchors(), new)
    with pytest.raises(ValueError):
        o.set_anchors(new[:-1])


def test_rotational_decks_parse():
    from conftest import reference_root
    if reference_root() is None:
        pytest.skip("MPCMD_REFERENCE_ROOT does not name a reference checkout")
    ref = os.path.join(reference_root(), "rotational_code")
    g = config.rotational_config(config.read_rotational_input(os.path.join(ref, "2d_array", "input.txt")))
    assert (g["lx"], g["ly"], g["lz"], g["n_dimers"], g["layout_rows"], g["layout_cols"]) == (64, 64, 32, 36, 6, 6)
    assert g["tether_k"] == 1000.0 and g["tether_z"] == 3.0 and g["mpc_every"] == 20
    assert g["n_solvent"] == math.floor(10.0 * 64 * 64 * 32)
    line = config.read_rotational_input(os.path.join(ref, "linear_periodic_ci", "input.txt"), config.LAYOUT_LINE)
    c = config.rotational_config(line, config.LAYOUT_LINE)
    assert (c["lx"], c["n_dimers"], c["layout"]) == (256, 26, config.LAYOUT_LINE)
    pitch = c["dcn"] + 2.0 * c["rc"] * 2.0 ** (1.0 / 6.0)
    assert abs(c["layout_sep"] - (256 - 26 * pitch) / 26) < 1e-12


def _two_rotor_state(cfg, placed):
    """Two rotors along x at the tether plane and solvent particles `placed`
    [(x, y, z, species, owner)], the rest far above the rotors."""
    n = cfg["n_solvent"]
    st = {k: np.zeros(n) for k in ("vx", "vy", "vz")}
    st["x"] = 1.0 + (np.arange(n) % 60).astype(float)
    st["y"] = 0.5 + (np.arange(n) // 60 % 15).astype(float)
    st["z"] = np.full(n, cfg["lz"] - 0.5)
    st["flag"] = np.zeros(n, dtype=np.int32)
    owner = np.zeros(n, dtype=np.int32)
    for i, (x, y, z, sp, ow) in enumerate(placed):
        st["x"][i], st["y"][i], st["z"][i], st["flag"][i], owner[i] = x, y, z, sp, ow
    zc = cfg["tether_z"]
    st["dpos"] = np.array([[10.0, 8.0, zc], [15.0, 8.0, zc], [40.0, 8.0, zc], [45.0, 8.0, zc]])
    st["dvel"] = np.zeros((4, 3))
    return st, owner


@pytest.mark.parametrize("tags", [0, 1])
def test_owner_tags_select_the_interaction(tags):
    # linear_periodic_no_ci/forces_mod.f95:79-121: a B of motor 1 near the N
    # sphere of motor 2 acts as an A there; a particle in the C cutoff of
    # motor 2 becomes a B of motor 2
    cfg = rotor_cfg("rot_owner", n_dimers=2, owner_tags=tags, n_solvent=64, init_count=[64, 0, 0, 0],
                    sort_every=0)
    o = O.Oracle(cfg, threads=1)
    st, owner = _two_rotor_state(cfg, [(45.0, 10.1, cfg["tether_z"], 1, 1),
                                       (40.0, 10.0, cfg["tether_z"], 1, 1)])
    o.set_state(st)
    o.set_owner(owner)
    o.prepare()
    o.run(1)
    got = o.get_state()
    f = got["dforce"]
    # the N sphere of motor 2 (sphere 3) feels only particle 0, along y
    if tags:
        assert np.array_equal(o.get_owner()[:2], [1, 2])
        f_tag = f[3, 1]
        ref = O.Oracle(dict(cfg, owner_tags=0), threads=1)
        ref.set_state(st)
        ref.prepare()
        ref.run(1)
        fb = ref.get_state()["dforce"][3, 1]
        assert f_tag != 0.0
        assert abs(f_tag / fb - cfg["eps_n"][0] / cfg["eps_n"][1]) < 1e-12
    else:
        assert np.array_equal(o.get_owner()[:2], [1, 1])   # untouched without tags
    assert np.array_equal(got["flag"][:2], [1, 1])


def test_owner_tags_follow_the_particles():
    # A particles carry no tag and every B one of a motor, through catalysis,
    # the B -> A reaction and the sort (sort_hilbert_mod.f95:75)
    cfg = rotor_cfg("rot_owner", sort_every=40, k=[0.5, 0, 0, 0, 0, 0])
    o = O.Oracle(cfg, threads=4)
    o.initial()
    assert not o.get_owner().any()
    o.prepare()
    o.run(6 * cfg["mpc_every"])
    st, own = o.get_state(), o.get_owner()
    assert np.all(own[st["flag"] == 0] == 0)
    b = st["flag"] == 1
    assert b.sum() > 0
    assert np.all((own[b] >= 1) & (own[b] <= cfg["n_dimers"]))
    # every motor has made some of them
    assert set(np.unique(own[b])) == set(range(1, cfg["n_dimers"] + 1))


def test_rotational_deck_mapping(tmp_path):
    # a deck in the layout of rotational_code/2d_array/input.txt (one value per
    # line, a comment after it) maps to the rotor configuration of
    # main_rotation.f95:53-110
    vals = ["6048421", "2000", "10.", "0.", "32.", "32.", "16.", "0", "2", "3", "1.0", "1.0", "2.0", "2.0",
            "5.0", "0.1", "0.1", "0.1", "1.0", "1000.0", "1.0", "1.0", "0.0", "0.2", "0.7", "1.0",
            "1.5707963267948966192", "0.005", "0.1", "10000", "0.001", "100", "100", "100", "100"]
    deck = tmp_path / "input.txt"
    deck.write_text("".join("%s\t\tvalue %d\n" % (v, i) for i, v in enumerate(vals)))
    c = config.rotational_config(config.read_rotational_input(str(deck)))
    assert (c["lx"], c["ly"], c["lz"], c["n_dimers"], c["layout_rows"], c["layout_cols"]) == (32, 32, 16, 6, 2, 3)
    assert c["variant"] == config.VARIANT_ROTOR and c["layout"] == config.LAYOUT_GRID
    assert c["tether_k"] == 1000.0 and c["tether_z"] == 3.0 and c["mpc_every"] == 20
    assert c["n_solvent"] == math.floor(10.0 * 32 * 32 * 16) and c["init_count"][1] == 0
    assert c["k"][0] == 0.001 and c["eps_n"][:2] == [0.1, 1.0] and c["react_box_type"] == 0
    # the oracle takes it: the layout lands in the box at the tether plane
    o = O.Oracle(dict(c, n_solvent=2048, init_count=[2048, 0, 0, 0]), threads=2)
    o.initial()
    d = o.get_state()["dpos"]
    assert np.all((d[:, 0] > 0) & (d[:, 0] < 32) & (d[:, 1] > 0) & (d[:, 1] < 32)) and np.all(d[:, 2] == 3.0)
