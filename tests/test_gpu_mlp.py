"""The surrogate's own BF16 tensor-core kernels (mpcmd_mlp_*) against an FP64
numpy MLP.

The reference rounds to BF16 where the kernels hold BF16 (the inputs, the
weights, every hidden activation, the output gradient and every hidden
gradient) and computes everything else in FP64, so the comparison isolates
the kernels' FP32 accumulation and FP32 elementwise arithmetic: outputs
within 1e-2 of their scale, and every gradient tensor within 2e-2 relative
L2 error of the FP64 gradient (a BF16 rounding that flips between the two
changes a value by 2^-8).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from main_gb300.surrogate import Mlp  # noqa: E402

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def reference(layers, x, t=None, w=None):
    """FP64 forward (and backward when targets are given) with the kernels' BF16 points."""
    hs, zs = [bf16(x)], []
    for (W, b) in layers[:-1]:
        z = hs[-1] @ bf16(W).T + b
        zs.append(z)
        hs.append(bf16(silu(z)))
    W, b = layers[-1]
    y = hs[-1] @ bf16(W).T + b
    if t is None:
        return y
    B = x.shape[0]
    dy = bf16(2.0 * w[None, :] * (y - t) / B)
    loss = float((w[None, :] * (y - t) ** 2).sum() / B)
    grads = [None] * len(layers)
    g = dy
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        grads[l] = (g.T @ hs[l], g.sum(axis=0))
        if l == 0:
            break
        dh = g @ bf16(W)
        g = bf16(dh * dsilu(zs[l - 1]))
    return y, loss, grads


def relerr(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def net():
    m = Mlp(batch=128, max_rows=65536, seed=3)
    yield m
    m.close()


def test_forward_matches_fp64_reference(net):
    rng = np.random.default_rng(0)
    x = rng.normal(size=(300, 8)).astype(np.float32)   # not a multiple of 128 rows
    y = net.forward(x).cpu().numpy()
    ref = reference(net.unflatten(net.params().astype(np.float64)), x.astype(np.float64))
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() <= 1e-2 * scale, (np.abs(y - ref).max(), scale)


def test_gradients_match_fp64_reference(net):
    rng = np.random.default_rng(1)
    B = net.batch
    x = rng.normal(size=(B, 8)).astype(np.float32)
    t = rng.normal(size=(B, net.n_out)).astype(np.float32)
    w = np.full(net.n_out, 1.0 / net.n_out, dtype=np.float32)
    w[0] = 0.5
    g, loss = net.gradients(x, t, w)
    layers = net.unflatten(net.params().astype(np.float64))
    _, loss_ref, gref = reference(layers, x.astype(np.float64), t.astype(np.float64), w.astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref, (loss, loss_ref)
    got = net.unflatten(g.astype(np.float64))
    for l, ((gw, gb), (rw, rb)) in enumerate(zip(got, gref)):
        assert relerr(gw, rw) <= 2e-2, (l, "W", relerr(gw, rw))
        assert relerr(gb, rb) <= 2e-2, (l, "b", relerr(gb, rb))
        assert np.abs(rw).max() > 0   # the layer receives gradient (the check is not vacuous)


def test_inference_at_65536_rows_equals_small_batches(net):
    rng = np.random.default_rng(2)
    x = rng.normal(size=(65536, 8)).astype(np.float32)
    big = net.forward(x).cpu().numpy()
    for lo in (0, 32768, 65536 - 128):
        small = net.forward(x[lo:lo + 128]).cpu().numpy()
        assert np.array_equal(big[lo:lo + 128], small)


def test_adam_training_fits_a_smooth_map():
    m = Mlp(n_out=2 + 64 * 32, batch=256, max_rows=1024, seed=5, lr=1e-3)
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, size=(4096, 8)).astype(np.float32)
    # a smooth vector-valued target: two scalars and a field that varies with the inputs
    zz, rr = np.meshgrid(np.linspace(-1, 1, 64), np.linspace(0, 1, 32), indexing="ij")
    a = X[:, 0:1] + 0.5 * X[:, 1:2] * X[:, 2:3]
    field = np.tanh(a[:, :, None] * zz[None] + X[:, 3:4, None] * rr[None]).reshape(4096, -1)
    Y = np.concatenate([np.sin(2 * X[:, :1]) + X[:, 1:2] ** 2, X[:, 2:3] * X[:, 3:4], field], axis=1).astype(np.float32)
    w = np.full(Y.shape[1], 0.4 / (Y.shape[1] - 2), dtype=np.float32)
    w[0], w[1] = 0.5, 0.1
    Xt, Yt, Wt = (torch.as_tensor(a, device="cuda") for a in (X, Y, w))
    first = None
    for step in range(400):
        idx = torch.as_tensor(rng.integers(0, 4096, 256), device="cuda")
        loss = m.train_step(Xt[idx].contiguous(), Yt[idx].contiguous(), Wt)
        first = loss if first is None else first
    assert loss < 0.1 * first, (first, loss)
    pred = m.forward(X[:512]).cpu().numpy()
    assert np.abs(pred[:, 0] - Y[:512, 0]).mean() < 0.1
    m.close()
