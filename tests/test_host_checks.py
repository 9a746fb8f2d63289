"""Host-side argument checks of the Python binding (no GPU: each call must fail
before it reaches the C ABI).

The C ABI takes plain pointers and reads as many values as the grid or the
particle count says; the binding is where a host array of the wrong size is
caught, so that the library never reads past the end of a caller's buffer."""
import numpy as np
import pytest

import pic_gb300 as pg


def fake_context(nx=16, ny=8):
    # a Context object without a device context: the checks run before any C call
    c = object.__new__(pg.Context)
    c.nx, c.ny, c.lx, c.ly = nx, ny, float(nx), float(ny)
    c.G = nx * ny
    c.capacity = 100
    c.h = None
    return c


def test_upload_rejects_arrays_of_different_lengths():
    c = fake_context()
    x = np.zeros(10)
    with pytest.raises(ValueError, match="^y:"):
        c.upload(x, np.zeros(9), np.zeros(10))
    with pytest.raises(ValueError, match="^q:"):
        c.upload(x, np.zeros(10), np.zeros(11))
    with pytest.raises(ValueError, match="^vx:"):
        c.upload(x, np.zeros(10), np.zeros(10), vx=np.zeros(3))
    with pytest.raises(ValueError, match="^m:"):
        c.upload(x, np.zeros(10), np.zeros(10), m=np.zeros(12))


def test_grid_arrays_must_hold_one_value_per_cell():
    c = fake_context()
    with pytest.raises(ValueError, match="^rho:"):
        c.set_rho(np.zeros(c.G - 1))
    with pytest.raises(ValueError, match="^ex:"):
        c.set_fields(phi=np.zeros(c.G), ex=np.zeros(c.G + 1))
    with pytest.raises(ValueError, match="^field:"):
        c.ws_predict(np.zeros((c.ny, c.nx + 1), np.float32))
    with pytest.raises(ValueError, match="^targets:"):
        c.ws_loss_grad(np.zeros((2, c.ny, c.nx), np.float32), np.zeros((1, c.ny, c.nx), np.float32))


@pytest.mark.parametrize("op,kw,bad", [
    (pg.NN_FWD_RELU, dict(weight=np.zeros((9, 32, 16)), bias=np.zeros(32)), "x"),  # x has 32 channels, cin 16
    (pg.NN_FWD_RELU, dict(weight=np.zeros((9, 16, 32)), bias=np.zeros(16)), "weight"),
    (pg.NN_FWD_OUT, dict(weight=np.zeros((9, 32, 32)), bias=np.zeros(16)), "bias"),
    (pg.NN_DGRAD, dict(weight=np.zeros((9, 32, 32)), aux=np.zeros((1, 2, 128, 16), np.uint16)), "aux"),
    (pg.NN_WGRAD, dict(aux=np.zeros((1, 2, 64, 16), np.uint16)), "aux"),
])
def test_conv_layer_shapes(op, kw, bad):
    x = np.zeros((1, 2, 128 if op != pg.NN_WGRAD else 64, 32), np.uint16)
    cin = 16 if bad == "x" else 32
    with pytest.raises(ValueError, match=f"^{bad}:"):
        pg.nn_conv3x3(op, x, cin=cin, cout=32, **kw)
