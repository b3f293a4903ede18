"""Rotor variant (rotational_code/2d_array grid, linear_periodic_ci line) on
the GPU engine against the FP64 oracle on identical seeded inputs.

Tolerances as in test_gpu_parity: FP64 engine <= 1e-9 absolute after 120 MD
steps, FP32 engine <= 2e-4 (positions) / 2e-3 (velocities) after 100 MD
steps; the layouts of mpcmd_initial and the anchors are bit-exact.
"""
import numpy as np
import pytest

from gpu_helpers import assert_close, pair
from main_gb300 import Engine, MpcmdError, config
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "rot": lambda prec, **kw: config.workload("rot", scale=0.5, precision=prec, **kw),
    "rot_line": lambda prec, **kw: config.workload("rot_line", scale=0.25, precision=prec, **kw),
    # linear_periodic_no_ci: owner tags, a sort inside the run, a fast B -> A reaction
    "rot_owner": lambda prec, **kw: config.workload("rot_owner", scale=0.25, precision=prec, sort_every=40,
                                                    k=[0.5, 0, 0, 0, 0, 0], **kw),
}


@pytest.mark.parametrize("case", list(CASES))
def test_layout_and_anchors_match_oracle(case):
    cfg = CASES[case](64)
    o = Oracle(cfg)
    o.initial()
    e = Engine(cfg)
    e.initial()
    se, so = e.download_state(), o.get_state()
    assert np.array_equal(se["dpos"], so["dpos"])
    assert np.array_equal(e.get_anchors(), o.get_anchors())
    assert np.array_equal(se["flag"], so["flag"])
    assert_close(se, so, cfg, pos=0.0, vel=1e-13)


@pytest.mark.parametrize("case", list(CASES))
def test_rotor_trajectory_fp64(case):
    cfg = CASES[case](64)
    o, e = pair(cfg)
    assert np.array_equal(e.get_anchors(), o.get_anchors())
    o.prepare()
    e.prepare()
    for chunk in (1, 48, 1, 70):
        o.run(chunk)
        e.run(chunk)
        assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
        if cfg["owner_tags"]:
            assert np.array_equal(e.get_owner_tags(), o.get_owner())
    if cfg["owner_tags"]:
        assert e.get_owner_tags().any()
    oo, oe = o.observables(), e.observables()
    assert np.array_equal(oo["species_count"], oe["species_count"])
    assert abs(oo["potential"] - oe["potential"]) <= 1e-9 * max(1.0, abs(oo["potential"]))
    # the rotors stay on their anchors and turn
    st = e.download_state()
    mid = 0.5 * (st["dpos"][0::2] + st["dpos"][1::2])
    assert np.abs(mid - e.get_anchors()).max() < 1e-6
    assert np.abs(st["dvel"]).max() > 0.0


@pytest.mark.parametrize("case", list(CASES))
def test_rotor_trajectory_fp32(case):
    cfg = CASES[case](32)
    o, e = pair(cfg)
    o.prepare()
    e.prepare()
    o.run(100)
    e.run(100)
    assert_close(e.download_state(), o.get_state(), cfg, pos=2e-4, vel=2e-3, flags=0.999, dimer=1e-4)
    if cfg["owner_tags"]:
        assert (e.get_owner_tags() == o.get_owner()).mean() >= 0.999


def test_set_anchors_and_checkpoint(tmp_path):
    cfg = CASES["rot"](64)
    o, e = pair(cfg)
    # anchors moved off the midpoints: RATTLE pulls the rotors onto them
    new = e.get_anchors() + np.array([0.05, -0.05, 0.0])
    e.set_anchors(new)
    o.set_anchors(new)
    o.prepare()
    e.prepare()
    o.run(30)
    e.run(30)
    assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    st = e.download_state()
    mid = 0.5 * (st["dpos"][0::2] + st["dpos"][1::2])
    assert np.abs(mid - new).max() < 1e-6
    path = str(tmp_path / "rot.ck")
    e.checkpoint(path)
    f = Engine(cfg)
    f.restore(path)
    assert np.array_equal(f.get_anchors(), new)
    # the restored context (restart forces in its prepare) goes on as the
    # uninterrupted one: both agree at the collision step 60
    f.prepare()
    e.run(30)
    f.run(30)
    assert_close(f.download_state(), e.download_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)


def test_owner_tags_exchange_checkpoint_and_config(tmp_path):
    cfg = CASES["rot_owner"](64)
    o, e = pair(cfg)
    assert not e.get_owner_tags().any()
    tags = (np.arange(cfg["n_solvent"]) % (cfg["n_dimers"] + 1)).astype(np.int32)
    e.set_owner_tags(tags)
    assert np.array_equal(e.get_owner_tags(), tags)
    with pytest.raises(MpcmdError):
        e.set_owner_tags(np.full(cfg["n_solvent"], cfg["n_dimers"] + 1, dtype=np.int32))
    e.prepare()
    e.run(30)
    path = str(tmp_path / "owner.ck")
    e.checkpoint(path)
    f = Engine(cfg)
    f.restore(path)
    assert np.array_equal(f.get_owner_tags(), e.get_owner_tags())
    f.prepare()
    e.run(30)
    f.run(30)
    assert np.array_equal(f.get_owner_tags(), e.get_owner_tags())
    assert_close(f.download_state(), e.download_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    # a context without owner tags refuses the calls; owner tags need the
    # deterministic catalysis of the rotor codes
    plain = Engine(CASES["rot_line"](64))
    with pytest.raises(MpcmdError):
        plain.get_owner_tags()
    with pytest.raises(MpcmdError):
        Engine(dict(cfg, catalysis=config.CAT_PROBABILISTIC))
