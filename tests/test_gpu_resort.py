"""Order-only re-sorts (mpcmd_set_resort) change where particles live in
device memory, never what the run computes.

With a re-sort at every collision step the FP64 engine still follows the
FP64 oracle (whose arrays keep the reference's index order) within the
trajectory tolerance of test_gpu_parity (1e-9 after up to 220 MD steps),
with identical species: the first members of the species lists
(distribute_mod.f95:95-182), the probabilistic catalysis draws and the
on-exit record all go by main index, not by slot.  The cases cover the
deterministic and probabilistic catalysis, the Selkov reaction with affected
cells, walls with the reactive floor, catalysis on exit, and owner tags with
the reference's own sort inside the run (sort_hilbert_mod.f95:6-98 then
orders by main index the particles that re-sorts had moved).
"""
import numpy as np
import pytest

from gpu_helpers import CASES, assert_close, pair
from main_gb300 import MpcmdError, config

pytestmark = pytest.mark.gpu

RESORT_CASES = {
    "c0": lambda: CASES["c0"](64),
    "c1": lambda: CASES["c1"](64),
    "c2": lambda: CASES["c2"](64),
    "c0_on_exit": lambda: CASES["c0"](64, catalysis=config.CAT_ON_EXIT),
    "rot_owner": lambda: config.workload("rot_owner", scale=0.25, precision=64, sort_every=40,
                                         k=[0.5, 0, 0, 0, 0, 0]),
}


@pytest.mark.parametrize("case", list(RESORT_CASES))
def test_resort_every_collision_matches_oracle_fp64(case):
    cfg = RESORT_CASES[case]()
    o, e = pair(cfg)
    e.set_resort(cfg["mpc_every"])
    o.prepare()
    e.prepare()
    for chunk in (1, 48, 1, 70, 100):
        o.run(chunk)
        e.run(chunk)
        assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
        if cfg["owner_tags"]:
            assert np.array_equal(e.get_owner_tags(), o.get_owner())
    assert e.counters()["resorts"] >= 3
    oo, oe = o.observables(), e.observables()
    assert np.array_equal(oo["species_count"], oe["species_count"])
    assert oo["species_count"][1] > 0


def test_resorted_context_reports_main_indices():
    """After re-sorts the index-valued outputs (shell members, sphere pairs,
    distribute first members) and a checkpoint name the reference's indices."""
    import os
    import tempfile
    cfg = CASES["c0"](64)
    o, e = pair(cfg)
    e.set_resort(cfg["mpc_every"])
    o.prepare()
    e.prepare()
    o.run(150)
    e.run(150)
    assert e.counters()["resorts"] >= 2
    # staged collision step 200: distribute lists as the oracle builds them
    o.run(49)
    e.run(49)
    o.step()
    e.evolve()
    e.distribute()
    cnt_e, first_e = e.distribute_result()
    cnt_o, first_o = o.distribute_result()
    assert np.array_equal(cnt_e, cnt_o)
    assert np.array_equal(first_e, first_o)
    e.mpc_rotation()
    e.reaction()
    assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    # a fresh list pass on both sides: identical shell members and pairs
    o.prepare()
    e.prepare()
    assert np.array_equal(np.sort(o.inside()), e.inside())
    for s in range(2 * cfg["n_dimers"]):
        assert np.array_equal(np.sort(o.neighbours(s)), e.neighbours(s)), s
    # a checkpoint holds the particles in index order
    path = os.path.join(tempfile.mkdtemp(prefix="mpcmd_rs_"), "ck.bin")
    e.checkpoint(path)
    from main_gb300 import Engine
    f = Engine(cfg)
    f.restore(path)
    assert_close(f.download_state(), e.download_state(), cfg, pos=0.0, vel=0.0, flags=1.0, dimer=0.0)


def test_resort_interval_must_be_a_multiple_of_the_collision_interval():
    cfg = CASES["c0"](32)
    _, e = pair(cfg)
    with pytest.raises(MpcmdError):
        e.set_resort(cfg["mpc_every"] + 1)
    with pytest.raises(MpcmdError):
        e.set_resort(-cfg["mpc_every"])
    e.set_resort(0)
    e.prepare()
    e.run(2 * cfg["mpc_every"])
    assert e.counters()["resorts"] == 0


def test_resort_of_a_crowded_region_matches_oracle_fp64():
    """Particles crowded into one corner of the box (density 60 in an 8^3
    block, about 3 elsewhere): rank bins there hold more members than the
    re-sort's shared-memory counting sort takes, so those bins keep their
    bin order (the fallback path); the run still follows the oracle."""
    import numpy as np
    from main_gb300 import Engine
    from oracle.oracle import Oracle
    cfg = config.base_config(lx=16, ly=16, lz=16, n_dimers=0, n_solvent=40960, precision=64, cell_capacity=200)
    rng = np.random.default_rng(17)
    n_dense = 30720
    pos = np.empty((cfg["n_solvent"], 3))
    pos[:n_dense] = rng.random((n_dense, 3)) * 8.0
    rest = []
    while len(rest) < cfg["n_solvent"] - n_dense:
        p = rng.random(3) * 16.0
        if not (p < 8.0).all():
            rest.append(p)
    pos[n_dense:] = np.array(rest)
    v = rng.normal(scale=np.sqrt(cfg["kT"]), size=pos.shape)
    st = dict(x=pos[:, 0].copy(), y=pos[:, 1].copy(), z=pos[:, 2].copy(),
              vx=v[:, 0].copy(), vy=v[:, 1].copy(), vz=v[:, 2].copy(),
              flag=np.zeros(cfg["n_solvent"], np.int32),
              dpos=np.zeros((0, 3)), dvel=np.zeros((0, 3)), dforce=np.zeros((0, 3)))
    o = Oracle(cfg)
    o.set_state(st)
    e = Engine(cfg)
    e.upload_state(st)
    o.set_cell_order(e.cell_order())
    e.set_resort(cfg["mpc_every"])
    o.prepare()
    e.prepare()
    for chunk in (50, 70):
        o.run(chunk)
        e.run(chunk)
        assert_close(e.download_state(), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0)
    assert e.counters()["resorts"] == 2


@pytest.mark.parametrize("case", ["c0", "c2"])
def test_resort_every_collision_fp32_trajectory(case):
    """The FP32 production build with a re-sort at every collision step
    follows the oracle within the FP32 trajectory bar of test_gpu_parity."""
    cfg = CASES[case](32)
    o, e = pair(cfg)
    e.set_resort(cfg["mpc_every"])
    o.prepare()
    e.prepare()
    o.run(120)
    e.run(120)
    assert e.counters()["resorts"] == 2
    assert_close(e.download_state(), o.get_state(), cfg, pos=2e-4, vel=2e-3, flags=0.999, dimer=1e-4)
