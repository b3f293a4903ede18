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
