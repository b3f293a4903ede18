"""GPU engine vs the FP64 oracle on identical seeded inputs and identical
contract random draws (C ABI through main_gb300.Engine).

Tolerances: FP64 engine (compiled without FMA contraction) - integer results
bit-exact, floats <= 1e-9 absolute after 120 MD steps; FP32 engine
(cell-relative FP32 state) - floats <= 2e-4 (positions) / 2e-3 (velocities)
absolute after 100 MD steps, species flags >= 99.9 % identical (a flip needs a
particle within FP32 round-off of a cutoff or cell edge).
"""
import numpy as np
import pytest

from gpu_helpers import CASES, assert_close, pair, state_diff
from main_gb300 import Engine, MpcmdError, config
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

MODES = ["c0", "c1", "c2"]


@pytest.mark.parametrize("case", MODES)
@pytest.mark.parametrize("prec", [64, 32])
def test_collision_stage(case, prec):
    cfg = CASES[case](prec)
    o, e = pair(cfg)
    for step in (50, 100):
        o.set_cstep(step)
        e.set_step(step)
        o.mpc_rotation()
        e.mpc_rotation()
        assert np.array_equal(e.shift(), o.shift())
        kc_o, kc_e = o.new_cell(), e.new_cell()
        cm_o, ax_o, n_o = o.cell_rotation()
        cm_e, ax_e, n_e = e.cell_rotation()
        se, so = e.download_state(), o.get_state()
        if prec == 64:
            assert np.array_equal(kc_o, kc_e)
            assert np.array_equal(n_o, n_e)
            assert np.abs(cm_e - cm_o).max() < 1e-13
            assert np.abs(ax_e - ax_o).max() < 1e-13
            assert_close(se, so, cfg, pos=0.0, vel=1e-13)
        else:
            assert (kc_o != kc_e).mean() < 1e-4
            # FP32 axis: 32-bit draws and float trigonometry, about 1e-7
            assert np.abs(ax_e - ax_o).max() < 1e-6
            assert_close(se, so, cfg, pos=1e-6, vel=2e-5)


@pytest.mark.parametrize("case", MODES)
def test_neighbour_lists_fp64(case):
    cfg = CASES[case](64)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    assert np.array_equal(np.sort(o.inside()), e.inside())
    for s in range(2 * cfg["n_dimers"]):
        assert np.array_equal(np.sort(o.neighbours(s)), e.neighbours(s)), s


@pytest.mark.parametrize("case", MODES)
def test_distribute_and_reaction_stages_fp64(case):
    cfg = CASES[case](64)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    o.run(49)
    e.run(49)
    # step 50: the oracle runs the whole main-loop iteration, the engine the
    # stage calls one by one (main_pattern.f95:212-224)
    o.step()
    e.evolve()
    e.distribute()
    cnt_e, first_e = e.distribute_result()
    cnt_o, first_o = o.distribute_result()
    assert np.array_equal(cnt_e, cnt_o)
    assert np.array_equal(first_e, first_o)
    if cfg["exclusion"] == config.EXCL_CELLS:
        assert np.array_equal(e.affected(), o.affected())
    e.mpc_rotation()
    e.reaction()
    assert_close(e.download_state(), o.get_state(), cfg, pos=1e-11, vel=1e-11, flags=1.0, dimer=1e-11)


@pytest.mark.parametrize("case", MODES)
def test_trajectory_fp64(case):
    cfg = CASES[case](64)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    for chunk in (1, 48, 1, 70):
        o.run(chunk)
        e.run(chunk)
        d = assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    oo, oe = o.observables(), e.observables()
    assert np.array_equal(oo["species_count"], oe["species_count"])
    assert oo["time_penetrate"] == oe["time_penetrate"]
    assert abs(oo["potential"] - oe["potential"]) <= 1e-9 * max(1.0, abs(oo["potential"]))


@pytest.mark.parametrize("case", MODES)
def test_trajectory_fp32(case):
    cfg = CASES[case](32)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    o.run(100)
    e.run(100)
    assert_close(e.download_state(), o.get_state(), cfg, pos=2e-4, vel=2e-3, flags=0.999, dimer=1e-4)


@pytest.mark.parametrize("case", ["c0", "c2"])
def test_fused_step_equals_staged_calls(case):
    """mpcmd_run (fused collision step) == evolve + distribute + mpc_rotation +
    reaction called one by one, as main_pattern.f95:212-224 calls them."""
    cfg = CASES[case](64)
    o = Oracle(cfg)
    o.initial()
    st = o.get_state()
    a, b = Engine(cfg), Engine(cfg)
    for x in (a, b):
        x.upload_state(st)
        x.prepare()
    a.run(100)
    for step in range(1, 101):
        b.evolve()
        if step % cfg["mpc_every"] == 0:
            b.distribute()
            b.mpc_rotation()
            b.reaction()
    assert_close(a.download_state(), b.download_state(), cfg, pos=1e-12, vel=1e-12, flags=1.0, dimer=1e-12)


@pytest.mark.parametrize("case", MODES)
def test_initial_matches_oracle(case):
    cfg = CASES[case](64)
    o = Oracle(cfg)
    o.initial()
    e = Engine(cfg)
    e.initial()
    se, so = e.download_state(), o.get_state()
    assert np.array_equal(se["dpos"], so["dpos"])
    assert np.array_equal(se["flag"], so["flag"])
    assert_close(se, so, cfg, pos=0.0, vel=1e-13)


def test_sort_follows_hilbert_fixture():
    from conftest import hilbert_order
    order, box, _ = hilbert_order()
    cfg = config.base_config(lx=box[0], ly=box[1], lz=box[2], geometry=config.GEOM_WALLS, n_dimers=0,
                             n_solvent=2 * box[0] * box[1] * box[2], precision=64)
    o = Oracle(cfg)
    o.initial()
    o.set_cell_order(order)
    e = Engine(cfg)
    e.set_cell_order(order)
    e.upload_state(o.get_state())
    o.sort()
    e.sort()
    se, so = e.download_state(), o.get_state()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.array_equal(se[k], so[k]), k
    assert np.array_equal(se["flag"], so["flag"])


def test_checkpoint_roundtrip(tmp_path):
    cfg = CASES["c0"](32)
    o, e = pair(cfg)
    e.prepare()
    e.run(60)
    path = str(tmp_path / "ck.bin")
    e.checkpoint(path)
    f = Engine(cfg)
    f.restore(path)
    c1, c2 = e.counters(), f.counters()
    assert c1["cstep"] == c2["cstep"]
    # the file holds every particle at the checkpoint step; the restored
    # context, prepared as restart_mod.f95 does (forces of the state, no
    # kick), goes on as the original one; at the collision step 100 every
    # particle is at that step in both views
    f.prepare()
    e.run(40)
    f.run(40)
    # (an FP32 context: the two materializations of the lag round apart)
    assert_close(f.download_state(), e.download_state(), cfg, pos=2e-4, vel=2e-3, flags=0.999, dimer=1e-4)
    # a truncated file is refused
    data = open(path, "rb").read()
    open(path, "wb").write(data[: len(data) // 2])
    with pytest.raises(MpcmdError) as err:
        Engine(cfg).restore(path)
    assert err.value.status == 10


def test_cell_overflow_is_reported():
    cfg = CASES["c0"](32, cell_capacity=4)
    o, e = pair(cfg)
    e.prepare()
    with pytest.raises(MpcmdError) as err:
        e.run(50)
    assert err.value.status == 3


def test_displacement_rebuild_trigger_fp64():
    """evolve_mod.f95:465 rebuilds when a shell particle has moved more than
    half the skin; a particle pushed deep into a sphere's core triggers it.
    The engine replays the step after the rebuild exactly like the oracle."""
    cfg = CASES["c0"](64)
    o = Oracle(cfg)
    o.initial()
    st = o.get_state()
    c = st["dpos"][0]
    # put particle 0 at 0.65 sigma from the C sphere: a large LJ push (about
    # 0.3 cells per MD step afterwards, well below a box length)
    st["x"][0], st["y"][0], st["z"][0] = (c[0] + 0.65 * cfg["rc"]) % cfg["lx"], c[1], c[2]
    o2 = Oracle(cfg)
    o2.set_state(st)
    e = Engine(cfg)
    e.upload_state(st)
    o2.set_cell_order(e.cell_order())
    o2.prepare()
    e.prepare()
    o2.run(20)
    e.run(20)
    assert_close(e.download_state(), o2.get_state(), cfg, pos=1e-8, vel=1e-8, flags=1.0, dimer=1e-8)
    ob = o2.observables()
    c = e.counters()
    # the push shortens time_penetrate to about one step: rebuilds came from the
    # displacement test first and both codes agree on the schedule
    assert ob["time_penetrate"] == c["time_penetrate"] and c["time_penetrate"] < 5
    assert c["last_rebuild"] == ob["cstep"] - ob["time_count"]


@pytest.mark.parametrize("case", ["c1", "c2"])
def test_restart_continues_the_run_fp64(case):
    """mpcmd_checkpoint at step 60, mpcmd_restore and mpcmd_prepare (the
    restart forces of restart_mod.f95:415-528): the restored context and the
    uninterrupted one agree at the collision steps 100 and 150."""
    import tempfile, os
    cfg = CASES[case](64)
    o, e = pair(cfg)
    e.prepare()
    e.run(60)
    path = os.path.join(tempfile.mkdtemp(prefix="mpcmd_ck_"), "ck.bin")
    e.checkpoint(path)
    f = Engine(cfg)
    f.restore(path)
    f.prepare()
    steps = 100 - 60 if cfg["mpc_every"] == 50 else (-60) % cfg["mpc_every"] + cfg["mpc_every"]
    for chunk in (steps, cfg["mpc_every"]):
        e.run(chunk)
        f.run(chunk)
        assert_close(f.download_state(), e.download_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)


@pytest.mark.parametrize("case", ["c1", "c2"])
def test_prepare_restart_matches_oracle(case):
    """A mid-run state started with mpcmd_prepare_restart and with the
    oracle's prepare + restart_forces: forces of the state, then 60 steps."""
    cfg = CASES[case](64)
    o, e = pair(cfg)
    o.prepare()
    o.run(37)
    st = o.get_state()
    r = Oracle(cfg)
    r.set_state(st)
    r.set_cstep(37, 0)
    r.set_cell_order(e.cell_order())
    r.prepare()
    r.restart_forces()
    e.upload_state(st)
    e.set_step(37, 0)
    e.prepare_restart()
    se, so = e.download_state(), r.get_state()
    assert np.abs(se["dforce"] - so["dforce"]).max() <= 1e-9 * max(1.0, np.abs(so["dforce"]).max())
    assert np.array_equal(se["flag"], so["flag"])
    r.run(63)
    e.run(63)
    assert_close(e.download_state(), r.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)


@pytest.mark.parametrize("prec", [64, 32])
def test_catalysis_on_exit(prec):
    """A -> B on leaving the C interaction shell (MPCMD_CAT_ON_EXIT) against
    the oracle's restatement of the same rule, over 120 MD steps."""
    cfg = CASES["c0"](prec, catalysis=config.CAT_ON_EXIT)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    o.run(120)
    e.run(120)
    if prec == 64:
        assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
        assert np.array_equal(o.observables()["species_count"], e.observables()["species_count"])
    else:
        assert_close(e.download_state(), o.get_state(), cfg, pos=2e-4, vel=2e-3, flags=0.999, dimer=1e-4)
    assert o.observables()["species_count"][1] > 0
