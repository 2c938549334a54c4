"""Learned surrogate of the binned expected rates.

log rate_b(theta) ~= base_b(theta) + sigma_b * MLP(z(theta))_b

* base: a least-squares fit of the log rates (FP64 on the host), affine in
  the standardised parameters or additive (one piecewise-linear function per
  parameter and bin), which carries the bulk of the response;
* MLP: dims[0] = n_params -> 512 -> 512 -> 512 -> n_bins, SiLU, BF16 weights
  with FP32 accumulation, trained and evaluated by the tcgen05 kernels of
  libgw (gwm_* in include/gw.h) on the standardised residual.

Training data are parameter draws (the prior, or the region of the
posterior, with its covariance inflated) reweighted exactly by the engine.
Small sets go through the host (``training_data`` + ``Surrogate.fit``); the
full-size path keeps the set on the device: ``fit_affine`` on a pilot subset,
``attach``, then ``reserve`` / ``append_eval`` (the engine reweights on the
device and the targets are formed there) and ``train`` (the whole Adam loop in
libgw, no host round trip per step).
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
        self.kind, self.nodes, self.lim = "affine", 0, 0.0
        self.rb = self.rw = None
        self.mlp = MLP([n_params, *hidden, n_bins], batch_max=batch_max, device=device)
        self.mlp.init(seed)
        self.seed = seed

    def _z(self, theta):
        return (np.atleast_2d(theta) - self.mu) / self.sd

    def _features(self, z):
        """Design matrix of the base: [1, z] (affine) or [1, hat_k,j(z_k)]
        (additive: piecewise-linear interpolation weights of z_k between
        ``nodes`` equally spaced values over [-lim, lim], the same weights the
        device head uses)."""
        n = z.shape[0]
        if self.kind == "affine":
            return np.hstack([np.ones((n, 1)), z])
        G, lim = self.nodes, self.lim
        zc = np.clip(z, -lim, lim)
        u = (zc + lim) * ((G - 1) / (2.0 * lim))
        i = np.minimum(np.floor(u).astype(np.int64), G - 2)
        t = u - i
        F = np.zeros((n, 1 + z.shape[1] * G))
        F[:, 0] = 1.0
        rows = np.arange(n)[:, None]
        col = 1 + np.arange(z.shape[1])[None, :] * G + i
        F[rows, col] = 1.0 - t
        F[rows, col + 1] = t
        return F

    def _fit_base(self, thetas, logs, ridge):
        self.mu = thetas.mean(axis=0)
        self.sd = thetas.std(axis=0) + 1e-12
        z = self._z(thetas)
        X = self._features(z)
        G = X.T @ X
        G[np.diag_indices_from(G)] += ridge * np.mean(np.diag(G))
        self.A = np.linalg.solve(G, X.T @ logs)  # [(1 + features) x B]
        resid = logs - X @ self.A
        self.r_mu = resid.mean(axis=0)
        sd = resid.std(axis=0)
        # bins the base reproduces exactly (e.g. always empty) keep unit scale:
        # their FP32 rounding on the device must not become a large target
        self.r_sd = np.where(sd > 1e-6, sd, 1.0)
        return resid, z

    def fit_affine(self, thetas, logs):
        """Input standardisation, the least-squares affine base (FP64) and the
        per-bin mean / spread of its residual; returns the residual."""
        self.kind, self.nodes, self.lim = "affine", 0, 0.0
        self.rb = self.rw = None
        return self._fit_base(thetas, logs, 1e-12)[0]

    def fit_additive(self, thetas, logs, log_ratio=None, nodes=8, lim=3.0, ridge=1e-6):
        """Input standardisation and an additive base: per bin, a sum over
        parameters of piecewise-linear functions of each standardised
        parameter (``nodes`` values over [-lim, lim]), fitted by ridge least
        squares in FP64.  The network then learns what one parameter at a
        time cannot express.  log_ratio [n x B] = log(sum w^2 / sum w) of the
        same points, when given, is fitted as an affine function of the
        parameters (the head's model of sum w^2).  Returns the residual."""
        self.kind, self.nodes, self.lim = "additive", int(nodes), float(lim)
        resid, z = self._fit_base(thetas, logs, ridge)
        self.rb = self.rw = None
        if log_ratio is not None:
            X = np.hstack([np.ones((z.shape[0], 1)), z])
            R = np.linalg.lstsq(X, log_ratio, rcond=None)[0]
            self.rb, self.rw = R[0], R[1:].T  # [B], [B x P]
        return resid

    def fit(self, thetas, logs, epochs=20, lr=1e-3, batch=2048, log=None):
        """Least-squares affine base, then Adam (cosine-decayed lr) on the residual (host data)."""
        resid = self.fit_affine(thetas, logs)
        z = self._z(thetas)
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

    # ---- device-resident training set ----
    def reserve(self, n):
        _chk(N.libgw().gwm_train_reserve(self.mlp._n, int(n)), self.mlp._n)

    def size(self):
        c = C.c_int64()
        _chk(N.libgw().gwm_train_size(self.mlp._n, C.byref(c)), self.mlp._n)
        return c.value

    def append(self, thetas, sums):
        """Adds points with bin sums already computed (host arrays)."""
        th = np.ascontiguousarray(np.atleast_2d(thetas), dtype=np.float64)
        sm = np.ascontiguousarray(np.atleast_2d(sums), dtype=np.float64)
        bm = self.mlp.batch_max
        for s in range(0, th.shape[0], bm):
            a, b = th[s:s + bm], sm[s:s + bm]
            _chk(N.libgw().gwm_train_append(self.mlp._n, _p(np.ascontiguousarray(a)), _p(np.ascontiguousarray(b)),
                                            a.shape[0], 0), self.mlp._n)

    def append_eval(self, engine, thetas, k=64):
        """Adds points reweighted by ``engine`` on the device, k per launch."""
        th = np.ascontiguousarray(np.atleast_2d(thetas), dtype=np.float64)
        for s in range(0, th.shape[0], k):
            part = np.ascontiguousarray(th[s:s + k])
            _chk(N.libgw().gwm_train_append_eval(self.mlp._n, engine._e, _p(part), part.shape[0]), self.mlp._n)

    def read(self, first, count):
        """Rows of the device-resident set: (standardised inputs, targets)."""
        x = np.empty((count, self.n_params), np.float32)
        t = np.empty((count, self.n_bins), np.float32)
        _chk(N.libgw().gwm_train_read(self.mlp._n, int(first), int(count), _p(x), _p(t)), self.mlp._n)
        return x, t

    def train(self, epochs=20, lr=1e-3, batch=2048, lr_min=0.0, seed=None):
        """The Adam loop over the device-resident set; returns the loss per epoch."""
        losses = np.zeros(epochs, np.float32)
        seed = self.seed + 1 if seed is None else seed
        _chk(N.libgw().gwm_train_epochs(self.mlp._n, epochs, batch, C.c_float(lr), C.c_float(lr_min),
                                        C.c_uint64(seed), _p(losses)), self.mlp._n)
        self.history = [float(x) for x in losses]
        return self.history

    def base(self, theta):
        return self._features(self._z(theta)) @ self.A

    def log_rates(self, theta):
        z = self._z(theta)
        return self._features(z) @ self.A + self.r_mu + \
            self.r_sd * self.mlp.forward(z.astype(np.float32)).astype(np.float64)

    def attach(self, data, ratio, llh_type):
        """Moves the head (standardisation, base, output scaling, the model of
        sum(w^2) and the data) onto the GPU for ``stat_llh`` and the training
        set.  ratio [B]: sum(w^2)/sum(w) per bin as a constant; None: the
        affine model fitted by ``fit_additive``."""
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        self.llh_type = int(llh_type)
        d = _p(np.ascontiguousarray(data, dtype=np.float64))
        if self.kind == "affine":
            if ratio is None:
                raise ValueError("the affine head needs a constant sum(w^2)/sum(w) ratio")
            rc = N.libgw().gwm_set_head(self.mlp._n, _p(f32(self.mu)), _p(f32(self.sd)), _p(f32(self.A[1:].T)),
                                        _p(f32(self.A[0])), _p(f32(self.r_mu)), _p(f32(self.r_sd)), _p(f32(ratio)), d)
        else:
            if ratio is not None:
                rb, rw = np.log(np.maximum(np.asarray(ratio, dtype=np.float64), 1e-300)), None
            elif self.rb is not None:
                rb, rw = self.rb, self.rw
            else:
                raise ValueError("no sum(w^2) model: pass ratio or fit_additive(..., log_ratio=...)")
            rc = N.libgw().gwm_set_head_additive(self.mlp._n, _p(f32(self.mu)), _p(f32(self.sd)), self.nodes,
                                                 C.c_float(self.lim), _p(f32(self.A[1:])), _p(f32(self.A[0])),
                                                 _p(f32(self.r_mu)), _p(f32(self.r_sd)),
                                                 None if rw is None else _p(f32(rw)), _p(f32(rb)), d)
        _chk(rc, self.mlp._n)
        self._attached = (np.asarray(data, dtype=np.float64).copy(), None if ratio is None else np.array(ratio))

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

    def device_log_rates(self, theta):
        """(statistical LLH, log rates) of each point through the device head."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        llh = np.empty(th.shape[0])
        lr = np.empty((th.shape[0], self.n_bins))
        bm = self.mlp.batch_max
        for s in range(0, th.shape[0], bm):
            part = np.ascontiguousarray(th[s:s + bm])
            o = np.empty(part.shape[0])
            r = np.empty((part.shape[0], self.n_bins))
            _chk(N.libgw().gwm_predict(self.mlp._n, _p(part), part.shape[0], self.llh_type, _p(o), _p(r)),
                 self.mlp._n)
            llh[s:s + part.shape[0]], lr[s:s + part.shape[0]] = o, r
        return llh, lr

    # ---- stage 1 of delayed acceptance on the device ----
    def set_chain(self, prop_chol, prior_mean=None, prior_icov=None):
        a = np.ascontiguousarray(prop_chol, dtype=np.float64)
        m = None if prior_mean is None else np.ascontiguousarray(prior_mean, dtype=np.float64)
        c = None if prior_icov is None else np.ascontiguousarray(prior_icov, dtype=np.float64)
        _chk(N.libgw().gwm_set_chain(self.mlp._n, _p(a), _p(m), _p(c)), self.mlp._n)

    def substeps(self, theta, fs, n_sub, seed):
        """n_sub surrogate Metropolis steps of every chain on the device;
        fs None: the values at theta are evaluated first.  Returns
        (end points, their f_s, accepted sub-steps per chain)."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        Cn = th.shape[0]
        phi = np.empty_like(th)
        fphi = np.empty(Cn)
        nacc = np.empty(Cn, np.int32)
        f0 = None if fs is None else np.ascontiguousarray(fs, dtype=np.float64)
        _chk(N.libgw().gwm_substeps(self.mlp._n, _p(th), _p(f0), Cn, int(n_sub), self.llh_type,
                                    C.c_uint64(int(seed) & 0xFFFFFFFFFFFFFFFF), _p(phi), _p(fphi), _p(nacc)),
             self.mlp._n)
        return phi, fphi, nacc

    def value_grad(self, theta):
        """(f_s, d f_s / d theta) at each point, on the device: the surrogate
        -2 log L plus the prior penalty given to set_chain."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        f = np.empty(th.shape[0])
        g = np.empty_like(th)
        bm = self.mlp.batch_max
        for s in range(0, th.shape[0], bm):
            part = np.ascontiguousarray(th[s:s + bm])
            fo = np.empty(part.shape[0])
            go = np.empty_like(part)
            _chk(N.libgw().gwm_value_grad(self.mlp._n, _p(part), part.shape[0], self.llh_type, _p(fo), _p(go)),
                 self.mlp._n)
            f[s:s + part.shape[0]], g[s:s + part.shape[0]] = fo, go
        return f, g

    def linear_twin(self):
        """A surrogate with the same head (standardisation, base, output
        scaling, sum(w^2) model) and a network whose output is zero: the
        method without the trained network, for comparison."""
        t = Surrogate(self.n_params, self.n_bins, hidden=tuple(self.mlp.dims[1:-1]), batch_max=self.mlp.batch_max,
                      seed=self.seed)
        L = t.mlp.n_layers
        t.mlp.set_layer(L - 1, np.zeros((self.mlp.dims[-1], self.mlp.dims[-2]), np.float32),
                        np.zeros(self.mlp.dims[-1], np.float32))
        for a in ("kind", "nodes", "lim", "mu", "sd", "A", "r_mu", "r_sd", "rb", "rw"):
            setattr(t, a, getattr(self, a))
        return t

    def log_rates_linear(self, theta):
        """The base alone (no network)."""
        return self.base(theta) + self.r_mu

    def close(self):
        self.mlp.close()
