"""The tensor-core (tcgen05) MLP kernels of the surrogate.

* the GEMM against an FP64 product of the same BF16 inputs;
* the backward pass against an FP64 numpy forward/backward on the same
  BF16-rounded weights and inputs (the CPU oracle of the network);
* training lowers the loss, and the trained surrogate beats its affine base.
"""
import numpy as np
import pytest

from gundam_gb300 import _native as N
from gundam_gb300.surrogate import MLP, Surrogate

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_round(x):
    return (bf16_bits(x).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("M,N_,K", [(128, 64, 64), (256, 256, 512), (200, 3000, 512), (512, 512, 200),
                                    (96, 136, 24), (1024, 200, 4096)])
def test_tcgen05_gemm_matches_fp64(M, N_, K):
    import ctypes as C
    rng = np.random.default_rng(M + N_ + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N_, K)).astype(np.float32)
    a16, b16 = bf16_bits(A), bf16_bits(B)
    out = np.empty((M, N_), np.float32)
    rc = N.libgw().gwm_gemm_test(a16.ctypes.data_as(C.c_void_p), b16.ctypes.data_as(C.c_void_p), M, N_, K,
                                 out.ctypes.data_as(C.c_void_p))
    assert rc == 0
    ref = bf16_round(A) @ bf16_round(B).T
    err = np.abs(out - ref) / (np.sqrt(K) + np.abs(ref))
    assert err.max() < 3e-5  # FP32 accumulation over up to 4096 terms


def _np_forward_backward(ws, bs, x, t):
    """FP64 reference of the network on BF16-rounded weights and inputs,
    rounding activations to BF16 where the kernels store them."""
    hs, zs = [bf16_round(x)], []
    L = len(ws)
    for l in range(L):
        z = hs[-1] @ bf16_round(ws[l]).T + bs[l]
        zs.append(z)
        if l + 1 < L:
            s = 1 / (1 + np.exp(-z))
            hs.append(bf16_round(z * s))
    y = zs[-1]
    n = y.size
    loss = np.mean((y - t) ** 2)
    dz = bf16_round(2 * (y - t) / n)
    gws, gbs = [None] * L, [None] * L
    for l in range(L - 1, -1, -1):
        gws[l] = dz.T @ hs[l]
        gbs[l] = dz.sum(axis=0)
        if l > 0:
            dh = dz @ bf16_round(ws[l])
            z = zs[l - 1]
            s = 1 / (1 + np.exp(-z))
            dz = bf16_round(dh * s * (1 + z * (1 - s)))
    return loss, gws, gbs


def test_gradients_match_fp64_reference():
    dims = [200, 64, 64, 136]
    net = MLP(dims, batch_max=256)
    net.init(3)
    rng = np.random.default_rng(4)
    B = 128
    x = rng.standard_normal((B, dims[0])).astype(np.float32)
    t = rng.standard_normal((B, dims[-1])).astype(np.float32)
    ws, bs = [], []
    for l in range(len(dims) - 1):
        w, b = net.get_layer(l)
        b = rng.normal(0, 0.1, b.shape).astype(np.float32)
        net.set_layer(l, w, b)
        ws.append(w.astype(np.float64))
        bs.append(b.astype(np.float64))
    gw, gb, loss = net.gradients(x, t)
    rl, rgw, rgb = _np_forward_backward(ws, bs, x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - rl) <= 1e-3 * rl
    for l in range(len(dims) - 1):
        scale = np.abs(rgw[l]).max()
        assert np.abs(gw[l] - rgw[l]).max() <= 2e-2 * scale, l
        cos = np.sum(gw[l] * rgw[l]) / np.sqrt(np.sum(gw[l] ** 2) * np.sum(rgw[l] ** 2))
        assert cos > 0.999, l
        assert np.abs(gb[l] - rgb[l]).max() <= 2e-2 * np.abs(rgb[l]).max() + 1e-7, l
    net.close()


def test_forward_matches_fp64_reference():
    dims = [200, 512, 512, 512, 3000]
    net = MLP(dims, batch_max=256)
    net.init(7)
    x = np.random.default_rng(8).standard_normal((64, 200)).astype(np.float32)
    y = net.forward(x)
    ws = [net.get_layer(l)[0].astype(np.float64) for l in range(4)]
    bs = [net.get_layer(l)[1].astype(np.float64) for l in range(4)]
    h = bf16_round(x)
    for l in range(4):
        z = h @ bf16_round(ws[l]).T + bs[l]
        h = bf16_round(z / (1 + np.exp(-z))) if l < 3 else z
    assert np.abs(y - h).max() <= 1e-2 * np.abs(h).max()
    net.close()


def test_training_lowers_loss_and_beats_affine_base():
    rng = np.random.default_rng(11)
    P, B = 16, 64
    W = rng.normal(0, 0.3, (B, P))
    def truth(th):
        return th @ W.T + 0.3 * np.sin(th[:, :1] * 2.0) + 0.2 * th[:, 1:2] ** 2
    th = rng.standard_normal((8192, P))
    y = truth(th)
    s = Surrogate(P, B, hidden=(128, 128), batch_max=1024, seed=1)
    hist = s.fit(th, y, epochs=40, lr=2e-3, batch=512)
    assert hist[-1] < 0.25 * hist[0]
    te = rng.standard_normal((1024, P))
    full = np.mean((s.log_rates(te) - truth(te)) ** 2)
    lin = np.mean((s.log_rates_linear(te) - truth(te)) ** 2)
    assert full < 0.5 * lin
    s.close()


def test_device_training_set_and_loop():
    """Targets formed on the device (engine -> log sums -> affine residual)
    equal the FP64 host formula, the host-sums and engine paths agree, the
    native Adam loop lowers the loss, and on held-out points the trained
    network's log rates are closer to the exact ones than the base alone."""
    from gundam_gb300.engine import Engine
    from gundam_gb300.workload import Workload
    import gundam_gb300._native as Nn
    wl = Workload("c2", n_events=200000, seed=4)
    eng = Engine.from_workload(wl, precision="fp32", k_max=64, llh_type=Nn.GW_LLH_BARLOW_BEESTON_OA2021)
    rng = np.random.default_rng(5)
    chol = np.linalg.cholesky(wl.prior_cov)
    # wide enough that the response is visibly non-linear
    th = rng.standard_normal((8192, wl.n_params)) @ chol.T * 0.4
    sums = np.empty((1024, wl.n_bins))
    sums2 = np.empty_like(sums)
    for s0 in range(0, 1024, 64):
        a, b, _, _ = eng.eval(th[s0:s0 + 64])
        sums[s0:s0 + 64], sums2[s0:s0 + 64] = a, b
    logs = np.log(np.maximum(sums, 1e-300))
    sur = Surrogate(wl.n_params, wl.n_bins, hidden=(256, 256), batch_max=512, seed=3)
    sur.fit_affine(th[:1024], logs)
    ratio = np.where(sums > 0, sums2 / np.maximum(sums, 1e-300), 1.0).mean(axis=0)
    sur.attach(np.round(sums.mean(axis=0)), ratio, Nn.GW_LLH_BARLOW_BEESTON_OA2021)
    sur.reserve(8192 + 64)
    sur.append(th[:512], sums[:512])
    sur.append_eval(eng, th[512:], k=64)
    sur.append_eval(eng, th[:64], k=64)
    assert sur.size() == 8192 + 64
    x, t = sur.read(0, 1024)
    z = (th[:1024] - sur.mu) / sur.sd
    ref = (logs - (np.hstack([np.ones((z.shape[0], 1)), z]) @ sur.A) - sur.r_mu) / sur.r_sd
    assert np.abs(x - z).max() < 1e-5 * max(1.0, np.abs(z).max())
    scale = np.abs(logs).max() / sur.r_sd.min()
    assert np.abs(t - ref).max() < 2e-6 * scale
    assert np.array_equal(sur.read(8192, 64)[1], t[:64])  # engine path == host-sums path, bit for bit
    hist = sur.train(epochs=80, lr=1e-3, batch=512)
    assert hist[-1] < 0.8 * hist[0], hist
    te = rng.standard_normal((256, wl.n_params)) @ chol.T * 0.4
    ex = np.concatenate([np.log(np.maximum(eng.eval(te[i:i + 64])[0], 1e-300)) for i in range(0, 256, 64)])
    live = (sums > 0).all(axis=0)
    e_full = np.mean((sur.log_rates(te) - ex)[:, live] ** 2)
    e_base = np.mean((sur.log_rates_linear(te) - ex)[:, live] ** 2)
    assert e_full < 0.95 * e_base, (e_full, e_base)
    sur.close()
    eng.close()


M64 = (1 << 64) - 1


def _mix64(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def _hash4(seed, step, chain, k):
    h = _mix64((seed + 0x9E3779B97F4A7C15) & M64)
    h = _mix64(h ^ ((step * 0xD1B54A32D192ED03) & M64))
    h = _mix64(h ^ ((chain * 0xABC98388FB8FAC03) & M64))
    return _mix64(h ^ ((k * 0x8CB92BA72F3D8DD7) & M64))


def _u01(h):
    return ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0)


def _normals(seed, step, chain, P):
    # the device computes these in FP32 from the same uniforms
    n = np.empty(P)
    for k2 in range((P + 1) // 2):
        r = np.sqrt(-2.0 * np.log(np.float32(_u01(_hash4(seed, step, chain, 2 * k2)))))
        a = 2.0 * np.pi * np.float32(_u01(_hash4(seed, step, chain, 2 * k2 + 1)))
        n[2 * k2] = r * np.cos(a)
        if 2 * k2 + 1 < P:
            n[2 * k2 + 1] = r * np.sin(a)
    return n


@pytest.fixture(scope="module")
def c2_small():
    from gundam_gb300.engine import Engine
    from gundam_gb300.workload import Workload
    import gundam_gb300._native as Nn
    wl = Workload("c2", n_events=200000, seed=4)
    eng = Engine.from_workload(wl, precision="fp32", k_max=64, llh_type=Nn.GW_LLH_BARLOW_BEESTON_OA2021)
    rng = np.random.default_rng(6)
    chol = np.linalg.cholesky(wl.prior_cov)
    th = rng.standard_normal((1024, wl.n_params)) @ chol.T * 0.1
    sums = np.empty((th.shape[0], wl.n_bins))
    sums2 = np.empty_like(sums)
    for s0 in range(0, th.shape[0], 64):
        a, b, _, _ = eng.eval(th[s0:s0 + 64])
        sums[s0:s0 + 64], sums2[s0:s0 + 64] = a, b
    sur = Surrogate(wl.n_params, wl.n_bins, hidden=(128, 128), batch_max=512, seed=3)
    ok = sums > 0  # this small workload has empty bins
    logs = np.log(np.where(ok, sums, 1e-300))
    lratio = np.where(ok, np.log(np.where(ok, sums2, 1.0)) - np.log(np.where(ok, sums, 1.0)), 0.0)
    sur.fit_additive(th, logs, log_ratio=lratio, nodes=6)
    # data consistent with this small sample (no counts in bins it leaves empty)
    data = np.round(sums.mean(axis=0))
    sur.attach(data, None, Nn.GW_LLH_BARLOW_BEESTON_OA2021)
    sur.test_data = data
    yield wl, eng, sur, th, sums
    sur.close()
    eng.close()


def test_additive_head_matches_host(c2_small):
    """Device head (FP32 additive base + network) against the FP64 host
    formula; device LLH against the oracle's per-bin likelihood of the same
    rates and modelled sum of w^2; device targets against the host residual."""
    from oracle.oracle import llh_bin
    import gundam_gb300._native as Nn
    wl, eng, sur, th, sums = c2_small
    pts = th[:16]
    llh, lr = sur.device_log_rates(pts)
    host = sur.log_rates(pts)
    live = (sums > 0).all(axis=0)
    assert np.abs(lr - host)[:, live].max() < 2e-5 * max(1.0, np.abs(host[:, live]).max())
    z = (pts - sur.mu) / sur.sd
    lratio = sur.rb[None, :] + z @ sur.rw.T
    for m in range(4):
        mu = np.exp(lr[m])
        s2 = np.exp(lr[m] + lratio[m])
        ref = sum(llh_bin(Nn.GW_LLH_BARLOW_BEESTON_OA2021, sur.test_data[b], mu[b], np.sqrt(s2[b]))
                  for b in range(wl.n_bins))
        # stage-1 terms are FP32 per bin (summed in FP64): ~1e-5 per bin
        assert abs(llh[m] - ref) < 1e-6 * max(1.0, abs(ref)) + 2e-2
    sur.reserve(64)
    sur.append(th[:64], sums[:64])
    _, t = sur.read(0, 64)
    ls = np.log(np.maximum(sums, 1e-300))
    ref_t = (ls[:64] - sur.base(th[:64]) - sur.r_mu) / sur.r_sd
    live = (sums > 0).all(axis=0)
    scale = np.abs(ls[:, live]).max() / sur.r_sd[live].min()
    t, ref_t = t[:, live], ref_t[:, live]
    assert np.abs(t - ref_t).max() < 2e-6 * scale


def test_device_subchain_matches_host_replica(c2_small):
    """The device sub-chain takes the same steps as a host replica fed with
    the same counter-based random numbers and the device surrogate values."""
    wl, eng, sur, th, sums = c2_small
    P = wl.n_params
    icov = wl.prior_icov
    L = np.linalg.cholesky(0.02 * 2.38 ** 2 / P * wl.prior_cov)
    sur.set_chain(L, wl.prior_mean, icov)
    C, n_sub, seed = 8, 4, 12345
    th0 = th[100:100 + C].copy()

    def f(x):
        d = np.atleast_2d(x) - wl.prior_mean
        return sur.stat_llh(x) + np.sum((d @ icov) * d, axis=1)
    _, f_init, _ = sur.substeps(th0, None, 0, seed)
    # the device penalty is FP32 (the host one FP64)
    assert np.allclose(f_init, f(th0), rtol=1e-6, atol=1e-4)
    phi, fphi, nacc = sur.substeps(th0, f_init, n_sub, seed)
    phi2, fphi2, nacc2 = sur.substeps(th0, f_init, n_sub, seed)
    assert np.array_equal(phi, phi2) and np.array_equal(fphi, fphi2) and np.array_equal(nacc, nacc2)
    cur, fc, acc = th0.copy(), f_init.copy(), np.zeros(C, np.int64)
    for st in range(1, n_sub + 1):
        prop = np.stack([cur[c] + L @ _normals(seed, st, c, P) for c in range(C)])
        fp = f(prop)
        for c in range(C):
            if np.log(_u01(_hash4(seed, st, c, 0xFFFFFFFF))) < -(fp[c] - fc[c]) / 2:
                cur[c], fc[c], acc[c] = prop[c], fp[c], acc[c] + 1
    assert np.array_equal(nacc, acc)
    # increments are FP32 on the device
    assert np.allclose(phi, cur, rtol=0, atol=1e-6)
    assert np.allclose(fphi, fc, rtol=1e-6, atol=1e-4)
    assert acc.sum() > 0


def test_value_grad_matches_finite_differences(c2_small):
    """The device gradient of the surrogate -2 log L + prior penalty agrees
    with central differences of the device value along random directions,
    and the value equals the one the sub-chains use up to the penalty's
    summation order."""
    wl, eng, sur, th, sums = c2_small
    P = wl.n_params
    sur.set_chain(np.linalg.cholesky(1e-3 * wl.prior_cov), wl.prior_mean, wl.prior_icov)
    pts = th[:4]
    f, g = sur.value_grad(pts)
    _, f_sub, _ = sur.substeps(pts, None, 0, 1)
    np.testing.assert_allclose(f, f_sub, rtol=1e-6, atol=1e-3)
    rng = np.random.default_rng(3)
    h = 1e-3
    rel = []
    for _ in range(6):
        v = rng.standard_normal((4, P))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        fp, _ = sur.value_grad(pts + h * v)
        fm, _ = sur.value_grad(pts - h * v)
        fd = (fp - fm) / (2 * h)
        an = np.sum(g * v, axis=1)
        rel.extend((np.abs(fd - an) / np.maximum(np.abs(an), 1.0)).tolist())
    assert np.median(rel) < 0.03, rel
    assert np.max(rel) < 0.2, rel
    f2, g2 = sur.value_grad(pts)
    assert np.array_equal(f, f2) and np.array_equal(g, g2)
