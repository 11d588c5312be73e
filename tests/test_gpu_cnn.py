"""The learned CG guess on the GPU: the BF16 tensor-core forward and backward kernels against the
CPU network (oracle/cnn_ref.py, which emulates the same BF16 roundings), training on pairs the
FP64 solver produced, and the iteration count it saves inside the resident step.

Stated bounds (normwise relative): the FP32 prediction 5e-3; quantities stored in BF16 (activations,
pre-activations, the BF16 outputs of the tcgen05 kernels against mma.sync and exact sums) 8e-3, just
above one BF16 unit in the last place (2^-7 = 7.8e-3 of an element at most); parameter gradients
3e-3 per layer; loss 1e-3.  The differences come from FP32 accumulation order against exact sums,
which moves a few BF16 roundings by one unit; a wrong descriptor, tap or epilogue gives errors of
order one.
"""
import numpy as np
import pytest
import torch

from oracle import cnn_ref as C
from tests.helpers import rel_err
from wumingpic2d_gb300 import cnn
from wumingpic2d_gb300.sim import Simulation
from wumingpic2d_gb300.weibel import WeibelConfig, weibel_particles

pytestmark = pytest.mark.gpu
BF16_ULP = 8e-3  # one unit in the last place of a BF16 value is at most 2^-7 = 7.8e-3 of it


def _case(seed, n=2, H=16, W=32, grouped=True):
    """grouped: the block-diagonal parameters of the learned guess; else dense weights."""
    rng = np.random.default_rng(seed)
    params = cnn.init_params(seed) if grouped else C.flatten(C.init_params(seed))
    P = C.unflatten(params)
    for l, (w, b) in enumerate(P):  # non-zero biases on the real channels
        rout = 3 if l == 5 else w.shape[1]
        b[:rout] = (0.1 * rng.standard_normal(rout)).astype(np.float32)
    params = C.flatten(P)
    x = np.zeros((n, H, W, 16))
    x[..., :9] = C.bf16(rng.standard_normal((n, H, W, 9)))
    target = rng.standard_normal((n, H, W, 3)).astype(np.float32)
    return params, C.unflatten(params), x, target


def _dev_x(x):
    return torch.tensor(x, dtype=torch.float32).to("cuda", torch.bfloat16)


@pytest.mark.parametrize("grouped", [True, False])
def test_forward_matches_oracle(gpu, grouped):
    params, P, x, _ = _case(1, grouped=grouped)
    net = cnn.GuessNet(params, grouped=grouped)
    pred_i, _ = net.forward(_dev_x(x), train=False)
    pred_t, (acts, zs) = net.forward(_dev_x(x), train=True)
    torch.cuda.synchronize()
    ref, (racts, rzs) = C.forward(x, P, bf=True)
    e_inf = rel_err(pred_i.cpu().numpy()[..., :3], ref[..., :3])
    e_tr = rel_err(pred_t.cpu().numpy()[..., :3], ref[..., :3])
    e_act = max(rel_err(a.float().cpu().numpy(), r) for a, r in zip(acts[1:], racts[1:]))
    e_z = max(rel_err(z.float().cpu().numpy(), r) for z, r in zip(zs, rzs))
    print(f"\nforward vs oracle: infer {e_inf:.2e} train {e_tr:.2e} activations {e_act:.2e} pre-activations {e_z:.2e}")
    assert e_inf <= 5e-3 and e_tr <= 5e-3 and e_act <= BF16_ULP and e_z <= BF16_ULP
    assert np.array_equal(pred_i.cpu().numpy(), pred_t.cpu().numpy())  # same arithmetic in both modes
    assert not pred_i.cpu().numpy()[..., 3:].any()  # padded outputs stay zero


@pytest.mark.parametrize("grouped", [True, False])
def test_gradients_match_oracle(gpu, grouped):
    params, P, x, target = _case(2, grouped=grouped)
    net = cnn.GuessNet(params, grouped=grouped)
    tr = cnn.Trainer(net, masked=grouped)
    loss = tr.loss_and_grad(_dev_x(x), torch.tensor(target, device="cuda"))
    torch.cuda.synchronize()
    pred, cache = C.forward(x, P, bf=True)
    rloss, g = C.loss_and_grad(pred, target)
    grads = C.backward(cache, g, P, bf=True)
    gflat = C.unflatten(tr.grad.cpu().numpy())
    if grouped:  # the grouped (48, 48) kernels return the gradient on the diagonal blocks only
        M = C.unflatten(cnn.param_mask())
        assert all(not (gflat[l][0] * (1 - M[l][0])).any() for l in range(1, 5))
        grads = [(dw * m, db * mb) for (dw, db), (m, mb) in zip(grads, M)]
        gflat = [(dw * m, db * mb) for (dw, db), (m, mb) in zip(gflat, M)]
    errs = []
    for l, ((dw, db), (rdw, rdb)) in enumerate(zip(gflat, grads)):
        errs.append((rel_err(dw, rdw), rel_err(db[:rdb.size], rdb)))
    print("\ngradients vs oracle (dW, db) per layer: " + ", ".join(f"({a:.1e}, {b:.1e})" for a, b in errs)
          + f"; loss {float(loss.item()):.6e} vs {rloss:.6e}")
    assert abs(float(loss.item()) - rloss) <= 1e-3 * rloss
    for a, b in errs:
        assert a <= 3e-3 and b <= 3e-3


def _weibel_sim(seed, nx=128, ny=128, ppc=16, cg_err=1e-6):
    cfg = WeibelConfig(nx=nx, ny=ny, ppc=ppc, seed=seed)
    d = cfg.dims()
    up, np2 = weibel_particles(cfg)
    sim = Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="fp64", cg_err=cg_err)
    sim.load(up, d.alloc_uf(), np2)
    return sim


@pytest.fixture(scope="module")
def trained():
    xs, ys = [], []
    for seed in (11, 13):  # two seeded runs of 160 steps: (E, B, new J) -> converged dB
        with _weibel_sim(seed) as sim:
            a, b = cnn.capture_pairs(sim, 160, every=1)
        xs.append(a)
        ys.append(b)
    xn, yn = cnn.normalise(np.concatenate(xs), np.concatenate(ys))
    x, y = cnn.to_device(xn, yn)
    net = cnn.GuessNet(seed=3)
    hist = cnn.train(net, x, y, steps=6000, batch=16, lr=3e-3, seed=4, log_every=1000)
    return net, hist


def test_training_reduces_the_loss(gpu, trained):
    _, hist = trained
    print("\ntraining loss: " + ", ".join(f"{it}:{l:.3e}" for it, l in hist))
    assert hist[-1][1] < 0.05 * hist[0][1]


@pytest.mark.parametrize("cg_err", [1e-6, 1e-10])
def test_learned_guess_saves_cg_iterations(gpu, trained, cg_err):
    net, _ = trained
    params = net.host_params()
    runs = {}
    for mode in ("prev", "net"):
        with _weibel_sim(12, cg_err=cg_err) as sim:
            sim.step(20)  # leave the first steps, where both guesses are trivial
            if mode == "net":
                sim.set_guess(params)
            its, taken, rel = [], 0, []
            for _ in range(40):
                sim.step(1)
                its.append(sim.cg_iters().sum())
                if mode == "net":
                    st = sim.guess_stats()
                    taken += int(st[6:9].sum())
                    rel.append(np.sqrt(st[0:6] / np.concatenate([st[9:12], st[9:12]])))
            runs[mode] = (np.array(its), taken, sim.energy(), np.array(rel))
    it_prev, it_net = runs["prev"][0], runs["net"][0]
    rel = runs["net"][3]
    print(f"\nCG to {cg_err:g}: iterations per step (3 components): previous-step guess {it_prev.mean():.2f}, "
          f"learned guess {it_net.mean():.2f}; network guess taken {runs['net'][1]} of {3 * len(it_net)} solves; "
          f"median initial relative residual per component: network {np.median(rel[:, :3], axis=0)}, "
          f"previous step {np.median(rel[:, 3:], axis=0)}")
    # the network's start is closer to the solution for the two in-plane components, and the
    # solve never takes more iterations from the better of the two starts
    assert np.all(np.median(rel[:, :2], axis=0) < 0.5 * np.median(rel[:, 3:5], axis=0))
    assert it_net.mean() <= it_prev.mean()
    if cg_err < 1e-8:
        assert it_net.mean() < it_prev.mean()
    # the answer does not depend on the guess beyond the solver tolerance
    e_prev, e_net = runs["prev"][2], runs["net"][2]
    assert abs(e_net.sum() - e_prev.sum()) <= 1e-6 * e_prev.sum()


@pytest.mark.parametrize("cin,grouped", [(16, False), (48, True), (48, False)])
@pytest.mark.parametrize("train", [False, True])
@pytest.mark.parametrize("shape", [(2, 32, 48), (1, 64, 80)])
def test_tensor_core_conv_matches_mma_sync_and_exact_sums(gpu, cin, grouped, train, shape):
    """The forward convolutions with 48 outputs run on tcgen05 (accumulators in tensor memory).
    Against the warp-level mma.sync kernel on the same BF16 operands, and against exact float64
    sums of those operands: the BF16 outputs agree to one BF16 unit (8e-3) normwise (only the FP32 accumulation
    order differs, which moves a few roundings by one unit), and the kernel reports no timeout.
    On 32 x 48 every tile's halo wraps around the periodic edges (plain loads); on 64 x 80 the
    inner tiles' halos come by TMA."""
    import ctypes

    from wumingpic2d_gb300._native import check, lib

    rng = np.random.default_rng(cin + 7 * grouped + 3 * train)
    n, H, W = shape
    xb = C.bf16(rng.standard_normal((n, H, W, cin)))
    w = C.bf16(0.2 * rng.standard_normal((9, 48, cin)))
    if grouped:
        for go in range(3):
            for gi in range(3):
                if go != gi:
                    w[:, 16 * go:16 * go + 16, 16 * gi:16 * gi + 16] = 0.0
    b = (0.1 * rng.standard_normal(48)).astype(np.float32)
    x_d = torch.tensor(xb, dtype=torch.float32).to("cuda", torch.bfloat16)
    w_d = torch.tensor(w, dtype=torch.float32).to("cuda", torch.bfloat16)
    b_d = torch.tensor(b, device="cuda")
    outs = {}
    for legacy in (False, True):
        out = torch.empty((n, H, W, 48), dtype=torch.bfloat16, device="cuda")
        z = torch.empty_like(out)
        mode = (cnn.FWD_TRAIN if train else cnn.FWD_INFER) | (cnn.GROUPED if grouped else 0) | (32 if legacy else 0)
        check(lib().wm_cnn_conv3x3(ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(w_d.data_ptr()), ctypes.c_void_p(b_d.data_ptr()),
                                   cin, 48, mode, n, H, W, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(z.data_ptr()), None, None),
              "wm_cnn_conv3x3")
        torch.cuda.synchronize()
        outs[legacy] = (out.float().cpu().numpy(), z.float().cpu().numpy())
    check(lib().wm_cnn_status(1), "wm_cnn_status")
    # exact pre-activation from the same BF16 operands
    zx = np.zeros((n, H, W, 48))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        zx += np.einsum("nhwc,oc->nhwo", np.roll(xb, (-dy, -dx), axis=(1, 2)).astype(np.float64), w[tap].astype(np.float64))
    zx += b
    gx = 0.5 * zx * (1 + np.vectorize(__import__("math").erf)(zx / np.sqrt(2)))
    (a_tc, z_tc), (a_mma, z_mma) = outs[False], outs[True]
    print(f"\ntcgen05 vs mma.sync {rel_err(a_tc, a_mma):.2e}, vs exact {rel_err(a_tc, gx):.2e} (mma.sync vs exact {rel_err(a_mma, gx):.2e})")
    assert rel_err(a_tc, a_mma) <= BF16_ULP and rel_err(a_tc, gx) <= BF16_ULP
    if train:
        assert rel_err(z_tc, zx) <= BF16_ULP and rel_err(z_tc, z_mma) <= BF16_ULP


@pytest.mark.parametrize("shape", [(2, 32, 48), (1, 64, 80)])
def test_tensor_core_linear_layer_matches_mma_sync(gpu, shape):
    """The last layer (48 -> 8 channels, FP32 output) on tcgen05 with N padded to 16 zero-weight
    channels, against the mma.sync kernel (FP32 sums in another order: 1e-5) and exact sums."""
    import ctypes

    from wumingpic2d_gb300._native import check, lib

    rng = np.random.default_rng(11)
    n, H, W = shape
    xb = C.bf16(rng.standard_normal((n, H, W, 48)))
    w = C.bf16(0.2 * rng.standard_normal((9, 8, 48)))
    b = (0.1 * rng.standard_normal(8)).astype(np.float32)
    x_d = torch.tensor(xb, dtype=torch.float32).to("cuda", torch.bfloat16)
    w_d = torch.tensor(w, dtype=torch.float32).to("cuda", torch.bfloat16)
    b_d = torch.tensor(b, device="cuda")
    outs = {}
    for legacy in (False, True):
        out = torch.empty((n, H, W, 8), dtype=torch.float32, device="cuda")
        check(lib().wm_cnn_conv3x3(ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(w_d.data_ptr()), ctypes.c_void_p(b_d.data_ptr()),
                                   48, 8, cnn.FWD_LINEAR | (32 if legacy else 0), n, H, W, ctypes.c_void_p(out.data_ptr()), None, None,
                                   None), "wm_cnn_conv3x3")
        torch.cuda.synchronize()
        outs[legacy] = out.cpu().numpy()
    check(lib().wm_cnn_status(1), "wm_cnn_status")
    zx = np.zeros((n, H, W, 8))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        zx += np.einsum("nhwc,oc->nhwo", np.roll(xb, (-dy, -dx), axis=(1, 2)).astype(np.float64), w[tap].astype(np.float64))
    zx += b
    e_mma, e_exact = rel_err(outs[False], outs[True]), rel_err(outs[False], zx)
    print(f"\nlinear layer tcgen05 vs mma.sync {e_mma:.2e}, vs exact {e_exact:.2e}")
    assert e_mma <= 1e-5 and e_exact <= 1e-5


@pytest.mark.parametrize("cin", [16, 48])
@pytest.mark.parametrize("shape", [(2, 32, 48), (1, 64, 80)])
def test_tensor_core_input_gradient_matches_mma_sync(gpu, cin, shape):
    """The input-gradient convolution of training (out = conv * GELU'(zprev), no bias) on tcgen05
    against the mma.sync kernel and against exact sums of the same BF16 operands."""
    import ctypes
    import math

    from wumingpic2d_gb300._native import check, lib

    rng = np.random.default_rng(cin + 1)
    n, H, W = shape
    xb = C.bf16(rng.standard_normal((n, H, W, cin)))
    w = C.bf16(0.2 * rng.standard_normal((9, 48, cin)))
    zp = C.bf16(rng.standard_normal((n, H, W, 48)))
    x_d = torch.tensor(xb, dtype=torch.float32).to("cuda", torch.bfloat16)
    w_d = torch.tensor(w, dtype=torch.float32).to("cuda", torch.bfloat16)
    z_d = torch.tensor(zp, dtype=torch.float32).to("cuda", torch.bfloat16)
    outs = {}
    for legacy in (False, True):
        out = torch.empty((n, H, W, 48), dtype=torch.bfloat16, device="cuda")
        check(lib().wm_cnn_conv3x3(ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(w_d.data_ptr()), None, cin, 48,
                                   cnn.BWD | (32 if legacy else 0), n, H, W, ctypes.c_void_p(out.data_ptr()), None,
                                   ctypes.c_void_p(z_d.data_ptr()), None), "wm_cnn_conv3x3")
        torch.cuda.synchronize()
        outs[legacy] = out.float().cpu().numpy()
    check(lib().wm_cnn_status(1), "wm_cnn_status")
    acc = np.zeros((n, H, W, 48))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        acc += np.einsum("nhwc,oc->nhwo", np.roll(xb, (-dy, -dx), axis=(1, 2)).astype(np.float64), w[tap].astype(np.float64))
    erf = np.vectorize(math.erf)
    gp = 0.5 * (1 + erf(zp / np.sqrt(2))) + zp * np.exp(-0.5 * zp**2) / np.sqrt(2 * np.pi)
    ref = acc * gp
    e_mma, e_exact = rel_err(outs[False], outs[True]), rel_err(outs[False], ref)
    print(f"\ninput gradient tcgen05 vs mma.sync {e_mma:.2e}, vs exact {e_exact:.2e}")
    assert e_mma <= BF16_ULP and e_exact <= BF16_ULP


@pytest.mark.parametrize("cin,coutp,cout,grouped", [(16, 48, 48, False), (48, 48, 48, True), (48, 48, 48, False), (48, 16, 3, False)])
@pytest.mark.parametrize("shape", [(2, 32, 48), (1, 64, 80)])
def test_tensor_core_weight_gradient_matches_mma_sync(gpu, cin, coutp, cout, grouped, shape):
    """The weight and bias gradients of training on tcgen05 (dz and the shifted input as MN-major
    operands, one FP32 accumulator per tap column in tensor memory) against the mma.sync kernel and
    against exact float64 sums of the same BF16 operands.  Both kernels sum exact BF16 products in
    FP32, in different orders: 1e-5 normwise.  Grouped: the off-block gradients are returned as
    zero.  The last layer's shape (cin 48, coutp 16, cout 3) reads 16 gradient channels and
    returns 3."""
    import ctypes

    from wumingpic2d_gb300._native import check, lib

    rng = np.random.default_rng(cin + coutp + 5 * grouped + shape[1])
    n, H, W = shape
    xb = C.bf16(rng.standard_normal((n, H, W, cin)))
    dzb = C.bf16(rng.standard_normal((n, H, W, coutp)))
    x_d = torch.tensor(xb, dtype=torch.float32).to("cuda", torch.bfloat16)
    dz_d = torch.tensor(dzb, dtype=torch.float32).to("cuda", torch.bfloat16)
    scratch = torch.empty(cnn.WGRAD_SCRATCH, dtype=torch.float32, device="cuda")
    outs = {}
    for legacy in (False, True):
        dw = torch.full((9 * cout * cin,), float("nan"), device="cuda")
        db = torch.full((cout,), float("nan"), device="cuda")
        flags = (cnn.GROUPED if grouped else 0) | (32 if legacy else 0)
        check(lib().wm_cnn_conv3x3_wgrad(ctypes.c_void_p(x_d.data_ptr()), ctypes.c_void_p(dz_d.data_ptr()), cin, coutp, cout, n, H, W, flags,
                                         ctypes.c_void_p(dw.data_ptr()), ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(scratch.data_ptr()),
                                         scratch.numel(), None), "wm_cnn_conv3x3_wgrad")
        torch.cuda.synchronize()
        outs[legacy] = (dw.cpu().numpy().reshape(9, cout, cin), db.cpu().numpy())
    check(lib().wm_cnn_status(1), "wm_cnn_status")
    ref = np.zeros((9, cout, cin))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        xs = np.roll(xb, (-dy, -dx), axis=(1, 2)).astype(np.float64)
        ref[tap] = np.einsum("nhwo,nhwc->oc", dzb[..., :cout].astype(np.float64), xs)
    off = np.zeros((9, cout, cin), dtype=bool)  # the off-block entries of a grouped layer
    if grouped:
        for go in range(3):
            for gi in range(3):
                if go != gi:
                    off[:, 16 * go:16 * go + 16, 16 * gi:16 * gi + 16] = True
        ref[off] = 0.0
    rdb = dzb[..., :cout].astype(np.float64).sum(axis=(0, 1, 2))
    (dw_tc, db_tc), (dw_mma, db_mma) = outs[False], outs[True]
    e_mma, e_exact, e_db = rel_err(dw_tc, dw_mma), rel_err(dw_tc, ref), rel_err(db_tc, rdb)
    print(f"\nweight gradient tcgen05 vs mma.sync {e_mma:.2e}, vs exact {e_exact:.2e}; bias gradient vs exact {e_db:.2e}")
    assert np.isfinite(dw_tc).all() and np.isfinite(db_tc).all()
    assert e_mma <= 1e-5 and e_exact <= 1e-5 and e_db <= 1e-5
    assert not dw_tc[off].any()


def test_interior_loss_leaves_the_crop_border_out(gpu):
    """wm_cnn_mse_interior: the loss over the interior of each image and a zero gradient within
    `border` pixels of its edges (training on crops of a larger field)."""
    import ctypes

    from wumingpic2d_gb300._native import check, lib

    rng = np.random.default_rng(5)
    n, H, W, b = 3, 32, 48, 8
    pred = rng.standard_normal((n, H, W, 8)).astype(np.float32)
    tgt = rng.standard_normal((n, H, W, 3)).astype(np.float32)
    p_d, t_d = torch.tensor(pred, device="cuda"), torch.tensor(tgt, device="cuda")
    dz = torch.full((n, H, W, 16), 1.0, dtype=torch.bfloat16, device="cuda")
    part = torch.empty(64, dtype=torch.float64, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    check(lib().wm_cnn_mse_interior(ctypes.c_void_p(p_d.data_ptr()), ctypes.c_void_p(t_d.data_ptr()), n, H, W, b,
                                    ctypes.c_void_p(dz.data_ptr()), ctypes.c_void_p(part.data_ptr()), 64, ctypes.c_void_p(loss.data_ptr()),
                                    None), "wm_cnn_mse_interior")
    torch.cuda.synchronize()
    e = (pred[..., :3].astype(np.float64) - tgt)[:, b:H - b, b:W - b]
    count = e.size
    assert abs(loss.item() - 0.5 * np.sum(e * e) / count) <= 1e-6 * loss.item()
    g = dz.float().cpu().numpy()
    inner = np.zeros((n, H, W), dtype=bool)
    inner[:, b:H - b, b:W - b] = True
    assert not g[~inner].any() and not g[..., 3:].any()
    assert rel_err(g[inner][:, :3], (e / count).reshape(-1, 3)) <= BF16_ULP


def test_standalone_guess_workload_runs(gpu):
    """The standalone learned-guess workload end to end on small boxes: crops from a Weibel and a
    Harris run, training with the interior loss on the tensor-core kernels, and CG iterations at
    1e-10 both ways on a periodic Weibel system; the guess changes only the iteration count."""
    from wumingpic2d_gb300 import guess_standalone as G

    r = G.run(pairs=96, size=48, steps=20, every=10, train_steps=40, batch=8, n=128, ppc=8, warm=5, measure_steps=3,
              weibel=(128, 8), harris=(256, 128))
    print("\n" + str({k: v for k, v in r.items() if k != "params"}))
    assert r["pairs"]["count"] == 96
    assert all(np.isfinite(l) for _, l in r["training"]["loss_history"])
    for mode in ("previous_step", "learned"):
        assert r["cg"][mode]["cg_iters_per_step"] > 0
    assert np.isfinite(r["params"]).all()
