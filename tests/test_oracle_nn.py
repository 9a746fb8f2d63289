"""The convolution-network oracle (oracle/nn_oracle.c) checked on the CPU:
BF16 rounding, the forward convolution against a direct numpy evaluation, the
weight gradient against numpy, and the whole network's backpropagation against
central finite differences (FP64, no rounding)."""
import numpy as np
import pytest


def np_conv(x, w, b):
    """y[b,y,x,co] = b[co] + sum_{tap,ci} x[(y+dy)%H, (x+dx)%W, ci] w[tap, co, ci] (FP64)."""
    out = np.zeros(x.shape[:3] + (w.shape[1],))
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        xs = np.roll(np.roll(x, -dy, axis=1), -dx, axis=2)
        out += xs @ w[t].T
    return out + b


def test_bf16_rounding(port):
    rng = np.random.default_rng(0)
    f = np.concatenate([rng.normal(size=1000).astype(np.float32),
                        np.array([1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 65504.0], np.float32)])
    want = port.bf16(f)
    got = np.array([port.lib.orc_bf16_from_float(float(v)) for v in f], np.uint16)
    assert np.array_equal(got, want)
    # ties go to even
    assert port.from_bf16(port.bf16(np.float32(1.0 + 2 ** -8)))[()] == 1.0
    assert port.from_bf16(port.bf16(np.float32(1.0 + 3 * 2 ** -8)))[()] == np.float32(1.0 + 2 ** -6)


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16)])
def test_conv_forward_matches_numpy(port, cin, cout):
    rng = np.random.default_rng(1)
    x = port.bf16(rng.normal(size=(2, 3, 8, cin)))
    w = rng.normal(size=(9, cout, cin)).astype(np.float32) / np.sqrt(9 * cin)
    b = rng.normal(size=cout).astype(np.float32) * 0.1
    wq = port.from_bf16(port.bf16(w)).astype(np.float64)
    ref = np_conv(port.from_bf16(x).astype(np.float64), wq, b.astype(np.float64))
    got = port.from_bf16(port.conv_fwd(x, w, b, relu=True))
    want = port.from_bf16(port.bf16(np.maximum(ref.astype(np.float32), 0)))
    assert np.max(np.abs(got - want)) <= 2 ** -7 * np.max(np.abs(want))
    out = port.conv_fwd(x, w, b, relu=False)
    assert np.allclose(out, ref[..., 0], rtol=1e-6, atol=1e-6)


def test_conv_wgrad_matches_numpy(port):
    rng = np.random.default_rng(2)
    x = port.bf16(rng.normal(size=(1, 4, 8, 16)))
    g = port.bf16(rng.normal(size=(1, 4, 8, 32)))
    dw, db = port.conv_wgrad(x, g)
    xf, gf = port.from_bf16(x).astype(np.float64), port.from_bf16(g).astype(np.float64)
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        xs = np.roll(np.roll(xf, -dy, axis=1), -dx, axis=2)
        assert np.allclose(dw[t], np.einsum("bhwc,bhwo->oc", xs, gf), rtol=1e-12, atol=1e-12)
    assert np.allclose(db, gf.sum(axis=(0, 1, 2)))


def test_net_gradient_finite_differences(port):
    rng = np.random.default_rng(3)
    n = port.net_param_count()
    params = (rng.normal(size=n) * 0.2).astype(np.float32)
    inp = rng.normal(size=(1, 3, 4)).astype(np.float32)
    tgt = rng.normal(size=(1, 3, 4)).astype(np.float32)
    loss, grad = port.net_loss_grad(params, inp, tgt, quantize=False)
    assert np.isfinite(loss) and np.any(grad != 0)
    idx = rng.choice(np.flatnonzero(grad), 25, replace=False)
    for i in idx:
        h = 1e-3 * max(1.0, abs(float(params[i])))
        pp, pm = params.copy(), params.copy()
        pp[i] += np.float32(h)
        pm[i] -= np.float32(h)
        hp = float(pp[i]) - float(params[i])
        hm = float(params[i]) - float(pm[i])
        lp, _ = port.net_loss_grad(pp, inp, tgt, quantize=False)
        lm, _ = port.net_loss_grad(pm, inp, tgt, quantize=False)
        fd = (lp - lm) / (hp + hm)
        assert abs(fd - grad[i]) <= 1e-3 * abs(grad[i]) + 1e-7, (i, fd, grad[i])
