"""The learned surrogate trained on batched-ensemble replicas, and what it
gains over the method without it.

Small scale (replicas of 16 to 20 cells, 100 collision periods, 768 training
points): the test trains the network on simulated replicas only, evaluates it
on held-out replicas (new parameters, new seeds) simulated twice with
different seeds, and checks

* that the trained network explains the B concentration field and the
  rotational diffusion of held-out points better than the method without it:
  the training-mean prediction (R^2 <= 0 for the rotational diffusion; for
  the field it keeps the shape every replica shares, which the network has
  to beat by a margin) and the untrained network;
* that its propulsion-speed error against the held-out runs is no larger
  than the run-to-run scatter of the simulation itself (the second seed):
  at these run lengths the per-point speed is dominated by the dimer's
  thermal motion, and the network predicts the mean at least as well as a
  repeated simulation does;
* what it gains: the whole held-out set predicted in one call, far faster
  than simulating it.
"""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from main_gb300 import ensemble as E  # noqa: E402
from main_gb300 import surrogate as S  # noqa: E402
from main_gb300 import sweep as W  # noqa: E402

pytestmark = pytest.mark.gpu

PERIODS = 100


@pytest.fixture(scope="module")
def data():
    tr = E.sample_replicas(768, seed=21, base_seed=40_000, wide=True, edge=(16, 20))
    ho = E.sample_replicas(128, seed=22, base_seed=50_000, wide=True, edge=(16, 20))
    rep = [dict(r, seed=r["seed"] + 7_000_000) for r in ho]
    out = {}
    for name, reps in (("tr", tr), ("ho", ho), ("rep", rep)):
        sp, dr, fd, ps, secs = W.simulate(reps, PERIODS, batch=512)
        out[name] = dict(reps=reps, X=E.surrogate_inputs(reps), Y=S.targets(sp, dr, fd), secs=secs)
    return out


def test_trained_surrogate_explains_held_out_replicas(data):
    tr, ho, rep = data["tr"], data["ho"], data["rep"]
    net, sc, losses = W.fit(tr["X"], tr["Y"], epochs=60, seed=1)
    assert losses[-1] < 0.8 * losses[0]
    t0 = time.perf_counter()
    P = W.predict(net, sc, ho["X"])
    t_pred = time.perf_counter() - t0
    Y, Yr = ho["Y"], rep["Y"]
    field_r2 = W.r2(P[:, 2:].ravel(), Y[:, 2:].ravel())
    drot_r2 = W.r2(P[:, 1], Y[:, 1])
    assert field_r2 > 0.3, field_r2
    assert drot_r2 > 0.3, drot_r2
    # the method without the network: the training-mean field for every
    # parameter point (it already carries the field's shared spatial shape
    # around the sphere), and the same network untrained
    mean_pred = np.broadcast_to(tr["Y"].mean(axis=0), Y.shape)
    mean_r2 = W.r2(mean_pred[:, 2:].ravel(), Y[:, 2:].ravel())
    assert field_r2 > mean_r2 + 0.1, (field_r2, mean_r2)
    assert W.r2(mean_pred[:, 1], Y[:, 1]) <= 0.0 < drot_r2
    raw = S.Mlp(batch=256, max_rows=65536, seed=1)
    P0 = W.predict(raw, sc, ho["X"])
    assert W.r2(P0[:, 2:].ravel(), Y[:, 2:].ravel()) < field_r2 - 0.3
    # speed: no worse than a repeated simulation of the same points
    rmse_net = float(np.sqrt(((P[:, 0] - Y[:, 0]) ** 2).mean()))
    rmse_sim = float(np.sqrt(((Yr[:, 0] - Y[:, 0]) ** 2).mean()))
    assert rmse_net <= rmse_sim, (rmse_net, rmse_sim)
    # the gain: all held-out points predicted far faster than simulated
    assert t_pred * 20 < ho["secs"], (t_pred, ho["secs"])
    raw.close()
    net.close()
