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
