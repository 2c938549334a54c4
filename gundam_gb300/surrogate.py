"""Learned surrogate of the binned expected rates.

log rate_b(theta) ~= base_b(theta) + sigma_b * MLP(z(theta))_b

* base: an affine least-squares fit of the log rates on the standardised
  parameters (FP64 on the host), which carries the bulk of the response;
* MLP: dims[0] = n_params -> 512 -> 512 -> 512 -> n_bins, SiLU, BF16 weights
  with FP32 accumulation, trained and evaluated by the tcgen05 kernels of
  libgw (gwm_* in include/gw.h) on the standardised residual.

Training data are parameter draws from the prior with its covariance
inflated, reweighted exactly by the engine (``training_data``).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _err(net) -> str:
    buf = C.create_string_buffer(512)
    N.libgw().gwm_last_error(net, buf, len(buf))
    return buf.value.decode(errors="replace")


def _chk(rc, net=None):
    if rc != N.GW_OK:
        raise N.GwError(rc, _err(net))


class MLP:
    """The network on the GPU (FP32 master weights, BF16 compute)."""

    def __init__(self, dims, batch_max=4096, device=0):
        self.dims = [int(d) for d in dims]
        self.batch_max = int(batch_max)
        d = np.asarray(self.dims, dtype=np.int32)
        p = C.c_void_p()
        _chk(N.libgw().gwm_create(_p(d), len(dims) - 1, self.batch_max, device, C.byref(p)))
        self._n = p

    @property
    def n_layers(self):
        return len(self.dims) - 1

    def init(self, seed=0):
        rng = np.random.default_rng(seed)
        for l in range(self.n_layers):
            fan_in, fan_out = self.dims[l], self.dims[l + 1]
            lim = math.sqrt(6.0 / (fan_in + fan_out))
            w = rng.uniform(-lim, lim, (fan_out, fan_in)).astype(np.float32)
            self.set_layer(l, w, np.zeros(fan_out, np.float32))

    def set_layer(self, l, w, b):
        w = np.ascontiguousarray(w, dtype=np.float32)
        b = np.ascontiguousarray(b, dtype=np.float32)
        _chk(N.libgw().gwm_set_layer(self._n, l, _p(w), _p(b)), self._n)

    def get_layer(self, l):
        w = np.empty((self.dims[l + 1], self.dims[l]), np.float32)
        b = np.empty(self.dims[l + 1], np.float32)
        _chk(N.libgw().gwm_get_layer(self._n, l, _p(w), _p(b)), self._n)
        return w, b

    @staticmethod
    def _pad(x, mult=8):
        n = x.shape[0]
        m = ((n + mult - 1) // mult) * mult
        if m == n:
            return np.ascontiguousarray(x, dtype=np.float32), n
        out = np.zeros((m,) + x.shape[1:], np.float32)
        out[:n] = x
        return out, n

    def forward(self, x):
        x, n = self._pad(np.atleast_2d(x))
        out = np.empty((x.shape[0], self.dims[-1]), np.float32)
        for s in range(0, x.shape[0], self.batch_max):
            xs = np.ascontiguousarray(x[s:s + self.batch_max])
            ys = np.empty((xs.shape[0], self.dims[-1]), np.float32)
            _chk(N.libgw().gwm_forward(self._n, _p(xs), xs.shape[0], _p(ys), 0), self._n)
            out[s:s + xs.shape[0]] = ys
        return out[:n]

    def train_step(self, x, t, lr):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = C.c_float()
        _chk(N.libgw().gwm_train_step(self._n, _p(x), _p(t), x.shape[0], C.c_float(lr), 0, C.byref(loss)), self._n)
        return loss.value

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        gw = [np.empty((self.dims[l + 1], self.dims[l]), np.float32) for l in range(self.n_layers)]
        gb = [np.empty(self.dims[l + 1], np.float32) for l in range(self.n_layers)]
        pw = (C.c_void_p * self.n_layers)(*[g.ctypes.data for g in gw])
        pb = (C.c_void_p * self.n_layers)(*[g.ctypes.data for g in gb])
        loss = C.c_float()
        _chk(N.libgw().gwm_gradients(self._n, _p(x), _p(t), x.shape[0], pw, pb, C.byref(loss)), self._n)
        return gw, gb, loss.value

    def close(self):
        if getattr(self, "_n", None):
            N.libgw().gwm_destroy(self._n)
            self._n = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cosine_lr(step, total, lr0, lr_min=0.0):
    return lr_min + 0.5 * (lr0 - lr_min) * (1.0 + math.cos(math.pi * min(step, total) / max(total, 1)))


def training_data(engine, wl, n, seed=0, inflate=1.5, k=64):
    """n parameter draws from the prior inflated by `inflate`, reweighted by
    the exact engine: returns (theta [n x P], log sum of weights [n x B],
    per-bin mean of sum(w^2)/sum(w))."""
    thetas = wl.draw_points(n, seed, inflate=inflate)
    logs = np.empty((n, wl.n_bins))
    ratio = np.zeros(wl.n_bins)
    for s in range(0, n, k):
        sums, sums2, _, _ = engine.eval(thetas[s:s + k])
        logs[s:s + k] = np.log(np.maximum(sums, 1e-300))
        ratio += (sums2 / np.maximum(sums, 1e-300)).sum(axis=0)
    return thetas, logs, ratio / n


class Surrogate:
    """Affine base + MLP residual, for standardised parameters."""

    def __init__(self, n_params, n_bins, hidden=(512, 512, 512), batch_max=4096, device=0, seed=0):
        self.n_params, self.n_bins = n_params, n_bins
        self.mlp = MLP([n_params, *hidden, n_bins], batch_max=batch_max, device=device)
        self.mlp.init(seed)
        self.seed = seed

    def _z(self, theta):
        return (np.atleast_2d(theta) - self.mu) / self.sd

    def fit(self, thetas, logs, epochs=20, lr=1e-3, batch=2048, log=None):
        """Least-squares affine base, then Adam (cosine-decayed lr) on the residual."""
        self.mu = thetas.mean(axis=0)
        self.sd = thetas.std(axis=0) + 1e-12
        z = self._z(thetas)
        X = np.hstack([np.ones((z.shape[0], 1)), z])
        self.A = np.linalg.lstsq(X, logs, rcond=None)[0]  # [(1 + P) x B]
        resid = logs - X @ self.A
        self.r_mu = resid.mean(axis=0)
        self.r_sd = resid.std(axis=0) + 1e-12
        target = ((resid - self.r_mu) / self.r_sd).astype(np.float32)
        zf = z.astype(np.float32)
        n = zf.shape[0]
        steps_per_epoch = max(1, n // batch)
        total = epochs * steps_per_epoch
        rng = np.random.default_rng(self.seed + 1)
        history = []
        step = 0
        for ep in range(epochs):
            perm = rng.permutation(n)
            acc = 0.0
            for s in range(steps_per_epoch):
                idx = perm[s * batch:(s + 1) * batch]
                acc += self.mlp.train_step(zf[idx], target[idx], cosine_lr(step, total, lr))
                step += 1
            history.append(acc / steps_per_epoch)
            if log:
                log(f"epoch {ep}: residual mse {history[-1]:.4g}")
        self.history = history
        return history

    def log_rates(self, theta):
        z = self._z(theta)
        base = np.hstack([np.ones((z.shape[0], 1)), z]) @ self.A
        return base + self.r_mu + self.r_sd * self.mlp.forward(z.astype(np.float32)).astype(np.float64)

    def attach(self, data, ratio, llh_type):
        """Moves the head (standardisation, affine base, output scaling, the
        sum(w^2)/sum(w) ratio and the data) onto the GPU for ``stat_llh``."""
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        self.llh_type = int(llh_type)
        _chk(N.libgw().gwm_set_head(self.mlp._n, _p(f32(self.mu)), _p(f32(self.sd)), _p(f32(self.A[1:].T)),
                                    _p(f32(self.A[0])), _p(f32(self.r_mu)), _p(f32(self.r_sd)), _p(f32(ratio)),
                                    _p(np.ascontiguousarray(data, dtype=np.float64))), self.mlp._n)

    def stat_llh(self, theta):
        """Surrogate statistical likelihood (-2 log L) of each parameter point, on the GPU."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        out = np.empty(th.shape[0])
        bm = self.mlp.batch_max
        for s in range(0, th.shape[0], bm):
            part = np.ascontiguousarray(th[s:s + bm])
            o = np.empty(part.shape[0])
            _chk(N.libgw().gwm_predict(self.mlp._n, _p(part), part.shape[0], self.llh_type, _p(o), None),
                 self.mlp._n)
            out[s:s + part.shape[0]] = o
        return out

    def log_rates_linear(self, theta):
        z = self._z(theta)
        return np.hstack([np.ones((z.shape[0], 1)), z]) @ self.A + self.r_mu

    def close(self):
        self.mlp.close()
