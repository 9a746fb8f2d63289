"""The learned warm start (pic_gpu_ws_*): the network's loss and gradient against
the oracle's backpropagation (oracle/nn_oracle.c, same BF16 rounding points,
FP64 sums), training on the run's own solutions, and the solve reaching the
same answer from every starting guess.

Gradient tolerance: 2e-2 relative L2 per layer. Both sides round every stored
activation and gradient to BF16 at the same points, from FP32 sums on the GPU
and FP64 sums in the oracle; the few values that land on the other side of a
rounding boundary move the gradient by well under 1%."""
import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu

LAYERS = [(16, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 16)]


def layer_slices():
    off, out = 0, []
    for cin, cout in LAYERS:
        nw = 9 * cin * cout
        out.append((slice(off, off + nw), slice(off + nw, off + nw + cout)))
        off += nw + cout
    return out


def landau(nx, ny, ppc, amp=0.05, vth=1.0, seed=5):
    p = workloads.density_cos(nx, ny, ppc, amp, vth, seed=seed)
    n = len(p["x"])
    p["q"] = np.full(n, -1.0 / n)  # the reference's convention: total charge -1, m = 1
    return p


def test_loss_and_gradient_match_oracle(port, pg):
    nx, ny, B = 128, 8, 2
    with pg.Context(nx, ny, float(nx), float(ny), 16) as c:
        c.ws_init(seed=3)
        rng = np.random.default_rng(4)
        params = c.ws_params()
        # perturb the zero-initialised padding-free entries a little so every layer is active
        params = params + (params != 0) * rng.normal(0, 0.02, params.size).astype(np.float32)
        c.ws_set_params(params)
        inp = port.from_bf16(port.bf16(rng.normal(size=(B, ny, nx))))
        tgt = port.from_bf16(port.bf16(rng.normal(size=(B, ny, nx))))
        loss, grad = c.ws_loss_grad(inp, tgt)
    want_loss, want_grad = port.net_loss_grad(params, inp, tgt, quantize=True)
    assert abs(loss - want_loss) <= 1e-3 * want_loss
    for l, (sw, sb) in enumerate(layer_slices()):
        for sl in (sw, sb):
            g, w = grad[sl].astype(np.float64), want_grad[sl]
            if np.linalg.norm(w) == 0:
                assert np.linalg.norm(g) == 0
                continue
            assert np.linalg.norm(g - w) <= 2e-2 * np.linalg.norm(w), (l, np.linalg.norm(g - w) / np.linalg.norm(w))


def test_training_lowers_loss_and_solves_agree(pg):
    nx, ny, ppc, dt = 256, 64, 16, 0.1
    p = landau(nx, ny, ppc)
    n = len(p["x"])
    with pg.Context(nx, ny, float(nx), float(ny), n) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"])
        c.ws_init(seed=1, dataset_capacity=128)
        bg = 1.0 / (nx * ny)
        npairs = c.ws_generate(96, dt, bg, sort_interval=10)
        assert npairs == 93
        loss = c.ws_train(epochs=6, batch=4, lr=2e-3)
        assert np.all(np.isfinite(loss)) and loss[-1] < 0.8 * loss[0], loss
        st = c.ws_study(3, dt, bg, sort_interval=10, tol=1e-8, check_every=16)
        phi, _, _ = c.fields()
    assert np.all(st["resid"] <= 1e-8)
    assert np.all(st["guess_resid"][:, 1] < st["guess_resid"][:, 0])
    assert np.all(st["phi_diff"] <= 1e-4 * np.sqrt(np.mean(phi ** 2)))


@pytest.mark.parametrize("mode", [1, 2])
def test_time_step_warm_start_keeps_the_answer(pg, mode):
    """pic_gpu_run with a red-black Gauss-Seidel solve warm-started from the
    extrapolation (1) or extrapolation + network (2) follows the same trajectory
    as the previous-phi start (0): every solve reaches the same tolerance."""
    nx, ny, ppc, dt = 128, 32, 16, 0.1
    p = landau(nx, ny, ppc, seed=11)
    n = len(p["x"])
    bg = 1.0 / (nx * ny)
    out = []
    for m in (0, mode):
        with pg.Context(nx, ny, float(nx), float(ny), n) as c:
            c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"])
            c.ws_init(seed=2)
            c.ws_generate(4, dt, bg, sort_interval=0)  # three solutions in the history
            h = c.run(6, scheme=1, dt=dt, background=bg, poisson=1, rbgs_tol=1e-10, rbgs_max_iters=400000,
                      rbgs_check_every=16, rbgs_warm=m)
            out.append((h, c.fields()[0]))
    (h0, phi0), (h1, phi1) = out
    assert np.allclose(h0[:, 3:], h1[:, 3:], rtol=1e-7, atol=0)
    assert np.max(np.abs(phi0 - phi1)) <= 1e-6 * np.max(np.abs(phi0))


def test_network_needs_fewer_sweeps_than_extrapolation(pg):
    """What the trained network gains over the same method without it: on a
    256x64 slice of the 512x512 warm-start set-up (64 per cell, density
    1 + 0.05 cos(2 pi x / 256), vth = 1, dt = 0.1), extrapolation + network
    reaches the 1e-8 relative residual in fewer red-black sweeps (FP64) than
    the extrapolation alone, summed over the same 8 steps, and both need fewer
    than the previous-phi start."""
    nx, ny, ppc, dt = 256, 64, 64, 0.1
    p = landau(nx, ny, ppc, seed=21)
    n = len(p["x"])
    bg = 1.0 / (nx * ny)
    with pg.Context(nx, ny, float(nx), float(ny), n) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"])
        c.set_rbgs_precision(False)
        c.ws_init(seed=1, dataset_capacity=2000)
        assert c.ws_generate(2003, dt, bg, sort_interval=20) == 2000
        loss = c.ws_train(epochs=8, batch=16, lr=1e-3)
        assert loss[-1] < loss[0]
        st = c.ws_study(8, dt, bg, sort_interval=20, tol=1e-8, check_every=16)
    it = st["iters"].sum(axis=0)
    assert np.all(st["resid"] <= 1e-8)
    assert it[2] < it[1] < it[0], it
