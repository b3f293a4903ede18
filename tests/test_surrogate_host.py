"""Host-side logic of the learned surrogate (no GPU): the sweep screen that
decides which points go back to the plain simulation, the targets, the input
and target scaling, and the loss weights."""
import numpy as np

from main_gb300 import surrogate as S


def test_screen_keeps_the_fastest_and_the_uncertain_points():
    rng = np.random.default_rng(3)
    speed = rng.normal(size=1000)
    unc = rng.random(1000)
    sel = S.screen(speed, unc, keep_fraction=0.02, trust=0.99)
    top = set(np.argsort(-speed)[:20].tolist())
    flagged = set(np.nonzero(unc > 0.99)[0].tolist())
    assert set(sel.tolist()) == top | flagged
    assert np.all(np.diff(sel) > 0)          # sorted, no duplicates
    assert sel.dtype == np.int64


def test_screen_without_trust_and_tiny_fraction():
    speed = np.array([0.1, 0.5, -0.2, 0.4])
    assert S.screen(speed, np.zeros(4), keep_fraction=0.0).tolist() == [1]   # at least one point
    assert S.screen(speed, np.zeros(4), keep_fraction=0.5).tolist() == [1, 3]
    # every point above the trust level is sent back, whatever its speed
    assert S.screen(speed, np.array([0.0, 0.0, 2.0, 0.0]), keep_fraction=0.25, trust=1.0).tolist() == [1, 2]


def test_targets_layout_and_log_diffusion():
    speed = np.array([0.01, -0.02])
    drot = np.array([1e-3, 0.0])               # 0 is clipped to 1e-6 before the log
    field = np.arange(2 * S.FIELD_Z * S.FIELD_R, dtype=float).reshape(2, S.FIELD_Z, S.FIELD_R)
    Y = S.targets(speed, drot, field)
    assert Y.shape == (2, S.N_OUT)
    assert np.array_equal(Y[:, 0], speed)
    assert np.allclose(Y[:, 1], [-3.0, -6.0])
    assert np.array_equal(Y[1, 2:], field[1].ravel())


def test_scaler_round_trip_and_log_k2():
    rng = np.random.default_rng(5)
    X = rng.random((64, S.N_IN)) + 0.5
    X[:, 4] = 10 ** rng.uniform(-3, -1, 64)     # k2 enters on a log scale
    Y = rng.normal(size=(64, 5)) * [1.0, 2.0, 0.0, 3.0, 4.0]   # a constant column keeps unit scale
    sc = S.Scaler(X, Y)
    xn = sc.x(X)
    assert xn.dtype == np.float32
    assert np.allclose(xn.mean(axis=0), 0.0, atol=1e-5)
    assert np.allclose(xn.std(axis=0), 1.0, atol=1e-4)
    assert np.allclose(sc.y_inv(sc.y(Y)), Y, atol=1e-5)
    assert sc.ys[2] == 1.0


def test_output_weights_sum_to_one():
    w = S.output_weights()
    assert w.shape == (S.N_OUT,)
    assert abs(float(w.sum()) - 1.0) < 1e-5
    assert w[0] == np.float32(0.5) and w[1] == np.float32(0.1)
