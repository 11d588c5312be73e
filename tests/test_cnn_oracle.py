"""Pins the CPU network used to check the GPU kernels: convolution convention, adjointness of
the input gradient, finite-difference parameter gradients, BF16 rounding."""
import numpy as np
import pytest

from oracle import cnn_ref as C


def test_bf16_rounding_ties_to_even():
    one = 1.0
    ulp = 2.0**-7  # bf16 spacing at 1
    assert C.bf16(np.array([one + ulp / 2]))[0] == one  # tie -> even (1.0)
    assert C.bf16(np.array([one + 3 * ulp / 2]))[0] == one + 2 * ulp  # tie -> even
    assert C.bf16(np.array([one + 0.51 * ulp]))[0] == one + ulp
    assert C.bf16(np.array([-2.5]))[0] == -2.5


def test_conv_tap_convention():
    x = np.zeros((1, 4, 5, 2))
    x[0, 1, 2, 1] = 1.0
    w = np.zeros((9, 1, 2))
    w[0, 0, 1] = 1.0  # tap 0 = (dy, dx) = (-1, -1): out(y, x) = in(y-1, x-1)
    out = C.conv(x, w)
    assert out[0, 2, 3, 0] == 1.0 and out.sum() == 1.0
    x[0, 0, 0, 1] = 2.0  # periodic wrap: out(1, 1) reads in(0, 0); out(0, 0) reads in(3, 4)
    assert C.conv(x, w)[0, 1, 1, 0] == 2.0


def test_input_gradient_is_the_adjoint():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 4, 6, 3))
    w = rng.standard_normal((9, 5, 3))
    y = rng.standard_normal((2, 4, 6, 5))
    lhs = np.sum(C.conv(x, w) * y)
    rhs = np.sum(x * C.conv_input_grad(y, w))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("layer", [0, 2, 5])
def test_parameter_gradients_by_finite_differences(layer):
    rng = np.random.default_rng(2)
    params = C.init_params(seed=5)
    x = np.zeros((1, 4, 5, 16))
    x[..., :9] = rng.standard_normal((1, 4, 5, 9))
    target = rng.standard_normal((1, 4, 5, 3))
    pred, cache = C.forward(x, params, bf=False)
    _, g = C.loss_and_grad(pred, target)
    grads = C.backward(cache, g, params, bf=False)
    w, b = params[layer]
    rout = 3 if layer == 5 else w.shape[1]
    rin = 9 if layer == 0 else w.shape[2]
    h = 1e-6
    for _ in range(4):
        idx = (rng.integers(9), rng.integers(rout), rng.integers(rin))
        old = w[idx]
        w[idx] = old + h
        lp, _ = C.loss_and_grad(C.forward(x, params, bf=False)[0], target)
        w[idx] = old - h
        lm, _ = C.loss_and_grad(C.forward(x, params, bf=False)[0], target)
        w[idx] = old
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grads[layer][0][idx]) <= 1e-6 * max(1e-3, abs(fd))
    k = rng.integers(rout)
    old = b[k]
    b[k] = old + h
    lp, _ = C.loss_and_grad(C.forward(x, params, bf=False)[0], target)
    b[k] = old - h
    lm, _ = C.loss_and_grad(C.forward(x, params, bf=False)[0], target)
    b[k] = old
    assert abs((lp - lm) / (2 * h) - grads[layer][1][k]) <= 1e-6 * max(1e-3, abs((lp - lm) / (2 * h)))


def test_flatten_roundtrip_and_size():
    params = C.init_params(seed=3)
    flat = C.flatten(params)
    assert flat.size == C.nparams() == 93560
    back = C.unflatten(flat)
    for (w, b), (w2, b2) in zip(params, back):
        assert np.array_equal(w, w2) and np.array_equal(b, b2)
    # padding stays zero: layer 0 inputs 9..15 and layer 5 outputs 3..7
    assert not params[0][0][:, :, 9:].any() and not params[5][0][:, 3:, :].any()


def test_network_mask_is_block_diagonal_and_scales_are_per_group():
    from wumingpic2d_gb300 import cnn

    mask = cnn.param_mask()
    assert mask.size == cnn.NPARAMS
    P = C.unflatten(cnn.init_params(1))
    M = C.unflatten(mask)
    for (w, b), (mw, mb) in zip(P, M):
        assert not (w * (1 - mw)).any()  # weights outside the blocks start (and stay) at zero
    # layer 0: input group -> hidden block; layer 5: hidden block k -> output k only
    w0 = M[0][0]
    assert w0[0, 0:16, 0:3].all() and not w0[0, 0:16, 3:].any()
    assert w0[4, 32:48, 6:11].all() and not w0[4, 32:48, :6].any() and not w0[4, :, 11:].any()
    w5 = M[5][0]
    assert w5[8, 2, 32:48].all() and not w5[8, 2, :32].any() and not w5[:, 3:, :].any()
    # the normalisation divides each group by its own scale: scaling one group's raw inputs
    # leaves every packed channel unchanged
    rng = np.random.default_rng(0)
    xs = rng.standard_normal((2, 8, 16, 9))
    ys = rng.standard_normal((2, 8, 16, 3))
    x1, y1 = cnn.normalise(xs, ys)
    xs2 = xs.copy()
    xs2[..., [5, 0, 1, 6, 7]] *= 1e3  # the dBz group
    ys2 = ys.copy()
    ys2[..., 2] *= 1e3
    x2, y2 = cnn.normalise(xs2, ys2)
    assert np.allclose(x1, x2) and np.allclose(y1, y2)


@pytest.mark.parametrize("name", ["guess_weibel.npz", "guess_harris.npz"])
def test_shipped_guess_weights_are_block_diagonal(name):
    import json
    from pathlib import Path

    from wumingpic2d_gb300 import cnn

    z = np.load(Path(cnn.__file__).with_name(name))
    params = z["params"]
    assert params.shape == (cnn.NPARAMS,) and params.dtype == np.float32 and np.all(np.isfinite(params))
    assert not (params * (1 - cnn.param_mask())).any()
    meta = json.loads(str(z["meta"]))
    held = meta["cg_iterations_held_out"]
    assert held["1e-06"]["learned"] < held["1e-06"]["previous_step"]
