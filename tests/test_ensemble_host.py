"""Host logic of the batched ensemble (CPU only): the replica sampler of the
ensemble workload, the replica <-> single-context configuration mapping and
the rotational-diffusion estimate from axis samples."""
import math

import numpy as np

from main_gb300 import config
from main_gb300 import ensemble as E


def test_sampled_replicas_follow_the_workload_ranges():
    reps = E.sample_replicas(256, seed=1)
    assert len({r["seed"] for r in reps}) == 256
    for r in reps:
        L = r["lx"]
        assert r["lx"] == r["ly"] == r["lz"] and 16 <= L <= 48
        assert 2.0 <= r["rc"] <= 5.0 and 1.0 <= r["rn"] <= 3.0
        assert r["rc"] + r["rn"] + 0.5 <= r["dcn"] <= r["rc"] + r["rn"] + 1.5
        assert 1e-3 <= r["k1"] <= 1e-1
        rho = r["n_solvent"] / L ** 3
        assert 5.0 - 0.01 <= rho <= 20.0 + 0.01
        # unique minimum images of the bond and of the list radii
        assert r["dcn"] < L / 2 and r["rc"] * E.CUT + 1.5 < L / 2
    edges = np.array([r["lx"] for r in reps])
    assert edges.min() < 25 and edges.max() > 40   # spread over the range


def test_wide_sampler_varies_the_surrogate_inputs():
    reps = E.sample_replicas(64, seed=2, wide=True)
    x = E.surrogate_inputs(reps)
    assert x.shape == (64, 8)
    assert x[:, 3].std() > 0.1 and x[:, 6].std() > 0.01


def test_replica_and_single_context_config_agree():
    cfg = config.workload("c0", scale=0.55, precision=64, seed=9, k=[0.03, 0, 0, 0, 0, 0])
    rep = E.replica_of_config(cfg)
    back = E.config_of_replica(rep, precision=64)
    for k in ("lx", "ly", "lz", "n_solvent", "seed", "rc", "rn", "dcn", "kT", "mc", "mn", "mpc_every"):
        assert back[k] == cfg[k], k
    assert back["k"][0] == 0.03 and back["geometry"] == config.GEOM_PERIODIC


def test_rotational_diffusion_of_a_known_random_walk():
    rng = np.random.default_rng(4)
    R, K, dt, Dr = 6, 4000, 0.5, 0.01
    u = np.zeros((R, K, 3))
    u[:, 0] = [1.0, 0.0, 0.0]
    for k in range(1, K):
        # rotational Brownian step: a small random rotation of variance 2 Dr dt per axis
        w = rng.normal(0.0, math.sqrt(2 * Dr * dt), (R, 3))
        v = u[:, k - 1] + np.cross(w, u[:, k - 1])
        u[:, k] = v / np.linalg.norm(v, axis=1, keepdims=True)
    est = E.rotational_diffusion(u, dt, max_lag=40)
    assert np.all(np.abs(est - Dr) < 0.2 * Dr), est
