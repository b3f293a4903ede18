"""The orientation correlation of main_gb300.analysis against a literal
transcription of the loops of 1D_Orientation_Correlation.py:30-53 (CPU)."""
import numpy as np
import pytest

from main_gb300.analysis import orientation_correlation


def literal(nuc):
    # the script's loops, transcribed statement by statement
    T, N = nuc.shape[0], nuc.shape[2]
    u = np.ones((T, N, N))
    if N % 2 == 0:
        P1 = np.zeros((T, int(0.5 * N + 1)))
        P2 = np.zeros((T, int(0.5 * N + 1)))
    else:
        P1 = np.zeros((T, int(0.5 * N)))
        P2 = np.zeros((T, int(0.5 * N)))
    for j in range(N):
        for i in range(N):
            u[:, j, i] = (nuc[:, 0, i] * nuc[:, 0, (i + j) % N] + nuc[:, 1, i] * nuc[:, 1, (i + j) % N]
                          + nuc[:, 2, i] * nuc[:, 2, (i + j) % N])
    for j in range(P1.shape[1]):
        for i in range(N):
            P1[:, j] = P1[:, j] + u[:, j, i] + u[:, j, (i - j) % N]
            P2[:, j] = P2[:, j] + 0.5 * (3. * u[:, j, i] ** 2 - 1) + 0.5 * (3. * u[:, j, (i - j) % N] ** 2 - 1)
        P1[:, j] = P1[:, j] / (2. * N)
        P2[:, j] = P2[:, j] / (2. * N)
    return P1, P2


@pytest.mark.parametrize("n", [2, 7, 26])
def test_matches_the_script(n):
    rng = np.random.default_rng(n)
    nuc = rng.normal(size=(5, 3, n))
    nuc /= np.linalg.norm(nuc, axis=1, keepdims=True)
    p1, p2 = orientation_correlation(nuc)
    q1, q2 = literal(nuc)
    assert p1.shape == q1.shape and p2.shape == q2.shape
    assert np.abs(p1 - q1).max() <= 1e-12 and np.abs(p2 - q2).max() <= 1e-12


def test_known_answers():
    # aligned motors: P1 = P2 = 1; alternating (antiparallel neighbours): P1 = (-1)^j, P2 = 1
    n = 6
    al = np.zeros((2, 3, n)); al[:, 0, :] = 1.0
    p1, p2 = orientation_correlation(al)
    assert np.allclose(p1, 1.0) and np.allclose(p2, 1.0)
    alt = al.copy(); alt[:, 0, 1::2] = -1.0
    p1, p2 = orientation_correlation(alt)
    assert np.allclose(p1, [(-1.0) ** j for j in range(p1.shape[1])]) and np.allclose(p2, 1.0)
    with pytest.raises(ValueError):
        orientation_correlation(np.zeros((2, 2, 3)))
    # one motor: no separation (the script's odd-count size int(N / 2) = 0)
    p1, p2 = orientation_correlation(al[:, :, :1])
    assert p1.shape == (2, 0) and p2.shape == (2, 0)
