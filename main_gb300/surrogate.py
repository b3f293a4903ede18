"""Learned surrogate of the batched ensemble (mpcmd_mlp_* in include/mpcmd.h).

``Mlp`` drives the library's own BF16 tensor-core training and inference
kernels (tcgen05.mma with TMA-staged operands and FP32 accumulation in tensor
memory, Adam on FP32 master weights).  PyTorch only holds the device buffers
that cross the C ABI.

The surrogate maps the eight replica parameters (sigma_C, sigma_N, bond
length, eps_B on N, k2, density, kT, box edge) to the propulsion speed
(Output_SelkovDimer.f90:168-172), the rotational diffusion (from the axis
autocorrelation of collective_code/1D_Orientation_Correlation.py:40-53) and
the axisymmetric B concentration around the dimer (64 x 32 (z, r) bins).
It is trained only on replicas that the batched ensemble simulates;
``screen`` ranks a parameter sweep with it and sends the points it flags back
to the plain simulation, which decides them.
"""
import ctypes as C
import math

import numpy as np

from . import MpcmdError, MpcmdMlpConfig, lib

N_IN = 8
FIELD_Z, FIELD_R = 64, 32
N_OUT = 2 + FIELD_Z * FIELD_R


class Mlp:
    """One network on the current CUDA device."""

    def __init__(self, n_in=N_IN, n_hidden=256, n_layers=4, n_out=N_OUT, batch=256, max_rows=65536, seed=1,
                 lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        import torch
        self.torch = torch
        self.cfg = MpcmdMlpConfig(n_in, n_hidden, n_layers, n_out, batch, max_rows, seed, lr, beta1, beta2, eps)
        h = C.c_void_p()
        st = lib().mpcmd_mlp_create(C.byref(self.cfg), C.byref(h))
        if st != 0:
            raise MpcmdError(st, "mlp_create")
        self.h = h
        self.n_in, self.n_hidden, self.n_layers, self.n_out, self.batch = n_in, n_hidden, n_layers, n_out, batch
        n = C.c_int64(0)
        lib().mpcmd_mlp_param_count(self.h, C.byref(n))
        self.n_params = n.value

    def close(self):
        if getattr(self, "h", None):
            lib().mpcmd_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, st, what):
        if st != 0:
            raise MpcmdError(st, what)

    def shapes(self):
        """(n_out_l, n_in_l) of every layer, input to output."""
        dims = [self.n_in] + [self.n_hidden] * self.n_layers + [self.n_out]
        return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]

    def unflatten(self, flat):
        out, off = [], 0
        for n, k in self.shapes():
            w = flat[off:off + n * k].reshape(n, k)
            off += n * k
            b = flat[off:off + n]
            off += n
            out.append((w, b))
        return out

    def params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        self._c(lib().mpcmd_mlp_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))), "mlp_get_params")
        return p

    def set_params(self, flat):
        p = np.ascontiguousarray(flat, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError("set_params: %d values, expected %d" % (p.size, self.n_params))
        self._c(lib().mpcmd_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))), "mlp_set_params")

    def _dev(self, a, shape):
        t = self.torch.as_tensor(a, dtype=self.torch.float32, device="cuda").contiguous()
        if tuple(t.shape) != tuple(shape):
            raise ValueError("expected shape %s, got %s" % (shape, tuple(t.shape)))
        return t

    def forward(self, x):
        """y [rows, n_out] for x [rows, n_in] (array or CUDA tensor); a CUDA tensor."""
        x = self._dev(x, (len(x), self.n_in))
        y = self.torch.empty((x.shape[0], self.n_out), dtype=self.torch.float32, device="cuda")
        self._c(lib().mpcmd_mlp_forward(self.h, x.data_ptr(), x.shape[0], y.data_ptr()), "mlp_forward")
        return y

    def gradients(self, x, t, w):
        """(flat FP32 gradients in the parameter layout, loss) of one batch."""
        B = self.batch
        x, t, w = self._dev(x, (B, self.n_in)), self._dev(t, (B, self.n_out)), self._dev(w, (self.n_out,))
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_double(0)
        self._c(lib().mpcmd_mlp_gradients(self.h, x.data_ptr(), t.data_ptr(), w.data_ptr(),
                                          g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)), "mlp_gradients")
        return g, loss.value

    def train_step(self, x, t, w, want_loss=True):
        """One Adam step on a batch of CUDA tensors; the loss before the step."""
        loss = C.c_double(0)
        self._c(lib().mpcmd_mlp_train_step(self.h, x.data_ptr(), t.data_ptr(), w.data_ptr(),
                                           C.byref(loss) if want_loss else None), "mlp_train_step")
        return loss.value if want_loss else None


# ------------------------------------------------------------ data ----
class Scaler:
    """Standardisation of the inputs (k2 on a log scale) and of the targets
    (speed, log rotational diffusion, field) so every output has unit scale."""

    def __init__(self, X, Y):
        self.xm, self.xs = self._fit(self.xform(X))
        self.ym, self.ys = self._fit(Y)

    @staticmethod
    def _fit(a):
        m = a.mean(axis=0)
        s = a.std(axis=0)
        s[s < 1e-12] = 1.0
        return m, s

    @staticmethod
    def xform(X):
        X = np.array(X, dtype=np.float64, copy=True)
        X[:, 4] = np.log10(X[:, 4])
        return X

    def x(self, X):
        return ((self.xform(X) - self.xm) / self.xs).astype(np.float32)

    def y(self, Y):
        return ((Y - self.ym) / self.ys).astype(np.float32)

    def y_inv(self, Yn):
        return Yn * self.ys + self.ym


def targets(speed, drot, field):
    """The network's targets of each replica: speed, log10 of the rotational
    diffusion, the flattened (z, r) B-concentration field."""
    d = np.log10(np.clip(np.asarray(drot, dtype=np.float64), 1e-6, None))
    return np.concatenate([np.asarray(speed, np.float64)[:, None], d[:, None],
                           np.asarray(field, np.float64).reshape(len(speed), -1)], axis=1)


def output_weights(n_field=FIELD_Z * FIELD_R, speed_weight=0.5):
    """Loss weights: the speed carries speed_weight of the loss, the rotational
    diffusion 0.1, the field the rest spread over its bins."""
    w = np.full(2 + n_field, (1.0 - speed_weight - 0.1) / n_field, dtype=np.float32)
    w[0] = speed_weight
    w[1] = 0.1
    return w


def train(net, Xn, Yn, w, epochs, seed=0, log_every=0):
    """Minibatch Adam over normalised data (device tensors are made here);
    returns the loss of every step."""
    import torch
    rng = np.random.default_rng(seed)
    X = torch.as_tensor(Xn, device="cuda")
    Y = torch.as_tensor(Yn, device="cuda")
    W = torch.as_tensor(w, device="cuda")
    B = net.batch
    n = X.shape[0]
    losses = []
    for ep in range(epochs):
        perm = torch.as_tensor(rng.permutation(n), device="cuda")
        for s in range(0, n - B + 1, B):
            idx = perm[s:s + B]
            xb = X[idx].contiguous()
            yb = Y[idx].contiguous()
            losses.append(net.train_step(xb, yb, W))
        if log_every and (ep + 1) % log_every == 0:
            print("epoch %d loss %.4g" % (ep + 1, losses[-1]))
    return losses


def screen(pred_speed, uncertainty, keep_fraction=0.05, trust=None):
    """Indices of the sweep points the plain simulation decides: the top
    keep_fraction by predicted speed, plus every point whose predicted
    uncertainty exceeds `trust` (when given)."""
    pred_speed = np.asarray(pred_speed)
    k = max(1, int(math.ceil(keep_fraction * len(pred_speed))))
    top = np.argsort(-pred_speed)[:k]
    sel = set(int(i) for i in top)
    if trust is not None:
        sel |= set(int(i) for i in np.nonzero(np.asarray(uncertainty) > trust)[0])
    return np.array(sorted(sel), dtype=np.int64)
