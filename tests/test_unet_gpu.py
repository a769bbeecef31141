"""The surrogate U-Net through the C ABI against the float64 oracle
(oracle/unet.py) on small frames.

The GPU computes with BF16 weights and activations and FP32 accumulation.
The oracle runs in float64 on the same BF16-rounded weights and input
channels, twice: exactly, and with every stored activation and activation
gradient rounded to BF16 where the kernels store them (oracle/unet.py rnd).
BF16 storage perturbs each pre-activation by ~2^-9 relative, which flips
the ReLU decisions of values near zero; those flips make the gradients of
deep layers differ by a few percent between any two roundings (the rounded
oracle against the exact one shows the same spread).  Bounds per weight and
bias tensor: relative L2 to the exact oracle below 0.15 and below three
times the rounded oracle's own distance to it plus 0.01; direction cosine
above 0.99.  Forward output: 2e-2 relative L2.  The convolution kernels
themselves are checked to BF16 output rounding in test_unet_conv_gpu.py.
"""
import numpy as np
import pytest
import torch

from openholo_gb300 import surrogate
from oracle import unet as U

pytestmark = pytest.mark.gpu


def bf16_round(a):
    return torch.from_numpy(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


def oracle_inputs(rgbd, lut):
    x = np.concatenate([rgbd[..., :3].astype(np.float64) / 255.0, lut[rgbd[..., 3]][..., None]], axis=3)
    return bf16_round(x)


def oracle_params(flat):
    p = surrogate.unflatten(flat.astype(np.float64))
    return {k: ((bf16_round(W) if k != "head" else W), b) for k, (W, b) in p.items()}


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def net(ctx):
    n = surrogate.UNet(ctx, max_batch=2, max_height=64, max_width=64, seed=5, out_scale=2.0)
    yield n
    n.close()


def make_batch(seed, n, h, w):
    rng = np.random.default_rng(seed)
    rgbd = rng.integers(0, 256, (n, h, w, 4), dtype=np.uint8)
    target = (rng.standard_normal((n, h, w, 2)) * 0.5).astype(np.float32)
    return rgbd, target


@pytest.mark.parametrize("shape", [(2, 32, 32), (1, 64, 16)])
def test_unet_forward_and_gradients_vs_oracle(ctx, net, shape):
    n, h, w = shape
    rgbd, target = make_batch(n * 100 + h, n, h, w)
    lut = np.arange(256) / 255.0
    flat = net.get_params()
    d_rgbd = torch.from_numpy(rgbd).cuda()
    d_tgt = torch.from_numpy(target).cuda()
    out = net.forward(d_rgbd)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    net.compute_grads(d_rgbd, d_tgt, loss)
    torch.cuda.synchronize()
    g = net.get_grads()
    P = oracle_params(flat)
    x = oracle_inputs(rgbd, lut)
    ref_loss, ref_g, pred = U.loss_and_grads(P, x, target.astype(np.float64) / 2.0)
    _, emu_g, _ = U.loss_and_grads(P, x, target.astype(np.float64) / 2.0, rnd=bf16_round)
    got = out.cpu().numpy()
    assert rel(np.stack([got.real, got.imag], -1), 2.0 * pred) < 2e-2
    assert abs(float(loss.item()) - ref_loss) < 2e-2 * ref_loss
    gg = surrogate.unflatten(g.astype(np.float64))
    report = []
    for name, *_ in surrogate.layer_shapes():
        for part in (0, 1):
            got_t, ref_t, emu_t = gg[name][part], ref_g[name][part], emu_g[name][part]
            cos = float(np.sum(got_t * ref_t) / (np.linalg.norm(got_t) * np.linalg.norm(ref_t) + 1e-300))
            report.append((name + ("/W" if part == 0 else "/b"), rel(got_t, ref_t), rel(emu_t, ref_t), cos))
    for r in report:
        print("%-10s gpu vs exact %.2e  rounded oracle vs exact %.2e  cos %.5f" % r)
    for name, r_gpu, r_emu, cos in report:
        assert r_gpu < 0.15 and r_gpu < 3 * r_emu + 0.01, name
        assert cos > 0.99, name


def test_unet_params_round_trip_and_training_reduces_loss(ctx):
    net = surrogate.UNet(ctx, max_batch=1, max_height=32, max_width=32, seed=9, out_scale=1.0)
    try:
        flat = net.get_params()
        net.set_params(flat * 0.5)
        assert np.array_equal(net.get_params(), (flat * 0.5).astype(np.float32))
        net.set_params(flat)
        rgbd, _ = make_batch(7, 1, 32, 32)
        # a target the network can represent: a pointwise function of the inputs
        target = np.stack([rgbd[..., 0] / 255.0 - 0.5, rgbd[..., 3] / 255.0 - 0.5], -1).astype(np.float32)
        d_rgbd = torch.from_numpy(rgbd).cuda()
        d_tgt = torch.from_numpy(target).cuda()
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        losses = []
        for _ in range(100):
            net.train_step(d_rgbd, d_tgt, 2e-3, loss)
            losses.append(float(loss.item()))
        print("training losses", losses[::10], losses[-1])
        assert losses[-1] < 0.1 * losses[0], losses[::10]
    finally:
        net.close()
