"""The tensor-core convolution kernels (tcgen05, BF16 x BF16 -> FP32) against the
oracle (oracle/nn_oracle.c, FP64 sums), layer by layer.

Tolerance per element: one BF16 unit in the last place at the larger of the
two values (both sides round a sum to BF16, from FP32 on the GPU and from FP64
here) plus 2^-16 times the sum of the magnitudes of the products, which bounds
the tensor cores' FP32 accumulation error where the sum cancels. FP32 outputs
and weight gradients: 2^-16 times the sum of magnitudes as well.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHANNELS = [(16, 32), (32, 32), (32, 16), (16, 16)]


def rand_case(port, rng, B, H, W, cin, cout):
    x = port.bf16(rng.normal(size=(B, H, W, cin)))
    w = (rng.normal(size=(9, cout, cin)) / np.sqrt(9 * cin)).astype(np.float32)
    b = (rng.normal(size=cout) * 0.1).astype(np.float32)
    return x, w, b


def roll_taps(x, sign):
    """[(tap, x shifted by sign*(dy, dx))] for the 9 taps, periodic."""
    out = []
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        out.append((t, np.roll(np.roll(x, -sign * dy, axis=1), -sign * dx, axis=2)))
    return out


def abs_sum_fwd(port, x, w):
    xa, wa = np.abs(port.from_bf16(x).astype(np.float64)), np.abs(port.from_bf16(port.bf16(w)).astype(np.float64))
    return sum(xs @ wa[t].T for t, xs in roll_taps(xa, 1))


def abs_sum_dgrad(port, g, w):
    ga, wa = np.abs(port.from_bf16(g).astype(np.float64)), np.abs(port.from_bf16(port.bf16(w)).astype(np.float64))
    return sum(gs @ wa[t] for t, gs in roll_taps(ga, -1))


def bf16_close(port, got, want, mag):
    g, w = port.from_bf16(got).astype(np.float64), port.from_bf16(want).astype(np.float64)
    tol = np.maximum(np.abs(w), np.abs(g)) * 2.0 ** -7 + mag * 2.0 ** -16
    bad = np.abs(g - w) > tol
    info = list(zip(g[bad][:4], w[bad][:4], mag[bad][:4]))
    return not bad.any(), int(bad.sum()), info


@pytest.mark.parametrize("cin,cout", CHANNELS)
@pytest.mark.parametrize("shape", [(1, 1, 128), (2, 5, 256), (1, 9, 384)])
def test_forward_relu(port, pg, cin, cout, shape):
    rng = np.random.default_rng(10 + cin + cout)
    x, w, b = rand_case(port, rng, *shape, cin, cout)
    got = pg.nn_conv3x3(pg.NN_FWD_RELU, x, w, b, cin=cin, cout=cout)
    want = port.conv_fwd(x, w, b, relu=True)
    ok, nbad, info = bf16_close(port, got, want, abs_sum_fwd(port, x, w))
    assert ok, (nbad, info)


@pytest.mark.parametrize("cin,cout", CHANNELS)
def test_forward_linear_out(port, pg, cin, cout):
    rng = np.random.default_rng(20 + cin + cout)
    x, w, b = rand_case(port, rng, 2, 6, 256, cin, cout)
    got = pg.nn_conv3x3(pg.NN_FWD_OUT, x, w, b, cin=cin, cout=cout)
    want = port.conv_fwd(x, w, b, relu=False)
    assert np.all(np.abs(got - want) <= abs_sum_fwd(port, x, w)[..., 0] * 2.0 ** -16 + 1e-30)


@pytest.mark.parametrize("cin,cout", CHANNELS)
def test_input_gradient(port, pg, cin, cout):
    rng = np.random.default_rng(30 + cin + cout)
    g = port.bf16(rng.normal(size=(2, 6, 256, cout)))
    mask = port.bf16(rng.normal(size=(2, 6, 256, cin)))
    w = (rng.normal(size=(9, cout, cin)) / np.sqrt(9 * cout)).astype(np.float32)
    got = pg.nn_conv3x3(pg.NN_DGRAD, g, w, aux=mask, cin=cin, cout=cout)
    want = port.conv_dgrad(g, w, mask)
    ok, nbad, info = bf16_close(port, got, want, abs_sum_dgrad(port, g, w))
    assert ok, (nbad, info)
    assert np.all(got[port.from_bf16(mask) <= 0] == 0)


@pytest.mark.parametrize("cin,cout", CHANNELS)
@pytest.mark.parametrize("shape", [(1, 1, 64), (2, 7, 256)])
def test_weight_gradient(port, pg, cin, cout, shape):
    rng = np.random.default_rng(40 + cin + cout)
    x = port.bf16(rng.normal(size=shape + (cin,)))
    g = port.bf16(rng.normal(size=shape + (cout,)))
    dw, db = pg.nn_conv3x3(pg.NN_WGRAD, x, aux=g, cin=cin, cout=cout)
    want_w, want_b = port.conv_wgrad(x, g)
    mag_w, mag_b = port.conv_wgrad(port.bf16(np.abs(port.from_bf16(x))), port.bf16(np.abs(port.from_bf16(g))))
    assert np.all(np.abs(dw - want_w) <= mag_w * 2.0 ** -16 + 1e-30)
    assert np.all(np.abs(db - want_b) <= mag_b * 2.0 ** -16 + 1e-30)


@pytest.mark.parametrize("cin,cout", [(32, 32), (32, 16), (16, 32)])
def test_weight_gradient_many_blocks_per_cta(port, pg, cin, cout):
    """4 x 96 x 512 pixels: 768 blocks of 8 rows x 32 pixels on at most 304
    CTAs, so CTAs run several blocks through their ring of two staging buffers
    (TMA copies for the interior of a row, cp.async for its two ends)."""
    rng = np.random.default_rng(7 + cin + cout)
    shape = (4, 96, 512)
    x = port.bf16(rng.normal(size=shape + (cin,)))
    g = port.bf16(rng.normal(size=shape + (cout,)))
    dw, db = pg.nn_conv3x3(pg.NN_WGRAD, x, aux=g, cin=cin, cout=cout)
    want_w, want_b = port.conv_wgrad(x, g)
    mag_w, mag_b = port.conv_wgrad(port.bf16(np.abs(port.from_bf16(x))), port.bf16(np.abs(port.from_bf16(g))))
    assert np.all(np.abs(dw - want_w) <= mag_w * 2.0 ** -16 + 1e-30)
    assert np.all(np.abs(db - want_b) <= mag_b * 2.0 ** -16 + 1e-30)
