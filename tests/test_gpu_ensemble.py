"""Batched ensemble (mpcmd_ens_*) against single-context runs and the oracle.

Each replica of a batched ensemble follows the step sequence of an mpcmd
context of the same configuration with the same contract streams, so the FP64
ensemble equals, replica by replica, the FP64 single-context runs (1e-9 after
120 MD steps: two graph-replayed collision periods and 20 steps issued one by
one), and the oracle on small replicas.  The FP32 production build conserves
each replica's momentum and particle count; the autotuner picks a schedule
from its candidates and caches it per shape class.
"""
import math
import os

import numpy as np
import pytest

from gpu_helpers import assert_close
from main_gb300 import Engine, config
from main_gb300 import ensemble as E
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def uneven_replicas(n=8, seed=3):
    """Uneven small replicas: boxes 14..20 (non-cubic included), densities,
    sphere sizes, bonds, interactions and rates all different."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        rc = rng.uniform(2.0, 3.2)
        rn = rng.uniform(1.0, 2.0)
        dcn = rc + rn + rng.uniform(0.5, 1.5)
        L = int(rng.integers(14, 21))
        lz = L if i % 3 else L + 2
        out.append(E.replica(L, L, lz, density=rng.uniform(5.0, 15.0), seed=500 + 7 * i, rc=rc, rn=rn, dcn=dcn,
                             eps_n=(1.0, rng.uniform(0.05, 1.0), 1.0, 1.0), kT=rng.uniform(0.12, 0.22),
                             k1=10 ** rng.uniform(-3, -1)))
    return out


def test_initial_state_equals_single_context_initial():
    reps = uneven_replicas(4)
    ens = E.Ensemble(reps, precision=64)
    ens.initial()
    for r, rep in enumerate(reps):
        cfg = E.config_of_replica(rep, precision=64)
        e = Engine(cfg)
        e.initial()
        se, sb = e.download_state(), ens.download(r)
        for k in ("x", "y", "z"):
            assert np.array_equal(se[k], sb[k]), (r, k)
        assert np.array_equal(se["flag"], sb["flag"])
        assert np.array_equal(se["dpos"], sb["dpos"])
        for k in ("vx", "vy", "vz"):
            assert np.abs(se[k] - sb[k]).max() < 1e-13, (r, k)
        e.close()
    ens.close()


@pytest.mark.parametrize("sort_every", [10000, 100])
def test_replicas_equal_their_single_context_runs_fp64(sort_every):
    reps = uneven_replicas(8)
    ens = E.Ensemble(reps, precision=64, sort_every=sort_every)
    engines = []
    for r, rep in enumerate(reps):
        cfg = E.config_of_replica(rep, precision=64, sort_every=sort_every)
        e = Engine(cfg)
        e.initial()
        ens.upload(r, e.download_state())
        e.prepare()
        engines.append((cfg, e))
    ens.prepare()
    for chunk in (100, 20, 30):   # two graph periods; 20 steps one by one; the rest of the period
        ens.run(chunk)
        for r, (cfg, e) in enumerate(engines):
            e.run(chunk)
            assert_close(ens.download(r), e.download_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    obs_b = ens.observables()
    for r, (cfg, e) in enumerate(engines):
        oe = e.observables()
        assert np.array_equal(obs_b[r]["species_count"], oe["species_count"]), r
        assert abs(obs_b[r]["potential"] - oe["potential"]) <= 1e-9 * max(1.0, abs(oe["potential"]))
        assert np.abs(obs_b[r]["momentum"] - oe["momentum"]).max() <= 1e-9
    c = ens.counters()
    # a period with a sort step is issued launch by launch, not replayed
    assert c["graph_replays"] == (2 if sort_every == 10000 else 1)
    assert c["cstep"] == 150 and c["status"] == 0
    assert c["rebuilds"] > 3 * len(reps)   # collision steps and between-collision rebuilds
    ens.close()


def test_small_replicas_against_the_oracle():
    reps = uneven_replicas(3, seed=11)
    ens = E.Ensemble(reps, precision=64)
    ens.initial()
    oracles = []
    for r, rep in enumerate(reps):
        cfg = E.config_of_replica(rep, precision=64)
        o = Oracle(cfg)
        o.set_state(ens.download(r))
        o.set_cell_order(Engine(cfg).cell_order())
        o.prepare()
        oracles.append((cfg, o))
    ens.prepare()
    for chunk in (50, 70):
        ens.run(chunk)
        for r, (cfg, o) in enumerate(oracles):
            o.run(chunk)
            assert_close(ens.download(r), o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    for r, (cfg, o) in enumerate(oracles):
        assert np.array_equal(ens.observables()[r]["species_count"], o.observables()["species_count"])


def test_fp32_ensemble_conserves_and_autotunes(tmp_path):
    reps = E.sample_replicas(16, seed=5, edge=(16, 24))
    ens = E.Ensemble(reps, precision=32)
    ens.initial()
    ens.prepare()
    o0 = ens.observables()
    cache = str(tmp_path / "schedules.txt")
    sched = ens.autotune(cache, periods=1)
    assert sched[0] in (1024, 2048, 4096) and sched[1] in (128, 256) and sched[2] in (128, 256)
    assert os.path.exists(cache) and len(open(cache).read().split()) == 5
    # the tuner restored the state it timed from
    assert ens.counters()["cstep"] == 0
    assert np.array_equal(ens.observables()[0]["species_count"], o0[0]["species_count"])
    ens.reset_samples(history=8)
    ens.run(8 * ens.mpc_every)
    o1 = ens.observables()
    for r, rep in enumerate(reps):
        assert o1[r]["species_count"].sum() == rep["n_solvent"]
        p_scale = rep["n_solvent"] * math.sqrt(3 * rep["kT"])
        assert np.abs(o1[r]["momentum"] - o0[r]["momentum"]).max() <= 1e-6 * p_scale, r
        assert o1[r]["species_count"][1] > 0   # catalysis made B
    mean, cnt, axes = ens.samples()
    assert np.all(cnt == 8) and np.all(np.isfinite(mean))
    assert np.allclose(np.linalg.norm(axes, axis=2), 1.0, atol=1e-5)
    # a second ensemble of the same shape class takes the cached schedule
    ens2 = E.Ensemble(reps, precision=32)
    ens2.initial()
    ens2.prepare()
    assert ens2.autotune(cache) == sched
    ens.field_accumulate(nz=16, nr=8, zmax=6.0, rmax=6.0)
    counts, ns = ens.field_read()
    assert ns == 1 and counts.shape == (16, 16, 8) and counts.sum() > 0
    ens.close()
    ens2.close()


def test_fp32_ensemble_follows_fp64_ensemble():
    """The FP32 build (FP32 solvent, four lanes per replica in the dimer step)
    follows the FP64 build from the same state: after 120 MD steps (two or
    three collision steps) every replica's dimer positions and velocities
    and the propulsion-speed samples and axes agree to 1e-2, far inside what
    a wrong component or a lost sphere sum gives (O(0.1) and larger).  The
    two builds drift apart by roundings (about 1e-5 here), and now and then
    by a solvent particle that one build finds inside a cutoff and the other
    just outside (a catalytic conversion one step apart), which can move a
    dimer's velocity by about 1e-3; the bound leaves room for that."""
    reps = uneven_replicas(8, seed=11)
    e64 = E.Ensemble(reps, precision=64)
    e64.initial()
    e32 = E.Ensemble(reps, precision=32)
    for r in range(len(reps)):
        e32.upload(r, e64.download(r))
    for e in (e64, e32):
        e.prepare()
        e.reset_samples(history=4)
        e.run(120)
    for r in range(len(reps)):
        a, b = e32.download(r), e64.download(r)
        L = np.array([reps[r]["lx"], reps[r]["ly"], reps[r]["lz"]], float)
        dp = a["dpos"] - b["dpos"]
        dp -= L * np.round(dp / L)
        assert np.abs(dp).max() <= 1e-2, (r, np.abs(dp).max())
        assert np.abs(a["dvel"] - b["dvel"]).max() <= 1e-2, (r, np.abs(a["dvel"] - b["dvel"]).max())
    m32, c32, ax32 = e32.samples()
    m64, c64, ax64 = e64.samples()
    assert np.array_equal(c32, c64) and np.all(c32 >= 2), (c32, c64)
    assert np.abs(m32 - m64).max() <= 1e-2, np.abs(m32 - m64).max()
    assert np.abs(ax32 - ax64).max() <= 1e-2
    e32.close()
    e64.close()
