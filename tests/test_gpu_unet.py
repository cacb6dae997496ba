"""GPU checks of the U-Net (forward and backward on the tensor cores, weight
gradients on the CUDA cores, Adam) against the FP64 oracle with the same
BF16 storage points."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import unet_ref as U

pytestmark = pytest.mark.gpu


def fields(seed, n, h, w):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn(n, h, w, generator=g)
    # a smooth target the network can learn: a blurred, scaled copy of x
    k = torch.tensor([[1., 2., 1.], [2., 4., 2.], [1., 2., 1.]]) / 16
    t = torch.nn.functional.conv2d(x[:, None], k[None, None], padding=1)[:, 0] * 3.0
    return x.cuda().contiguous(), t.cuda().contiguous()


def layer_bounds():
    off = U.offsets()
    return [0] + off + [U.num_params()]


def test_forward_matches_oracle(gpu_lib):
    from carpio_gb300.unet import UNet
    net = UNet(seed=1)
    p = net.params().astype(np.float64)
    for (n, h, w) in ((2, 64, 64), (1, 128, 64)):
        x, _ = fields(n + h, n, h, w)
        z = net.forward(x).cpu().numpy()
        zr, _ = U.forward(p, x.cpu().numpy(), emulate_bf16=True)
        assert rel_l2(z, zr) < 2e-2, rel_l2(z, zr)


@pytest.mark.parametrize("loss_kind", ["mse", "energy"])
def test_gradient_matches_oracle(gpu_lib, loss_kind):
    from carpio_gb300.unet import UNet
    net = UNet(seed=2)
    p = net.params().astype(np.float64)
    x, t = fields(7, 2, 64, 64)
    loss, g = net.grad(x, t, loss=loss_kind)
    lr_, gr = U.loss_and_grad(p, x.cpu().numpy(), t.cpu().numpy(), emulate_bf16=True,
                              loss=loss_kind)
    assert abs(loss - lr_) <= 1e-2 * lr_
    g = g.astype(np.float64)
    cos = g @ gr / (np.linalg.norm(g) * np.linalg.norm(gr))
    assert cos > 0.999, cos
    b = layer_bounds()
    for k, (a, c) in enumerate(zip(b[:-1], b[1:])):
        if np.linalg.norm(gr[a:c]) > 1e-6 * np.linalg.norm(gr):
            assert rel_l2(g[a:c], gr[a:c]) < 6e-2, (k, rel_l2(g[a:c], gr[a:c]))


def test_training_reduces_the_loss(gpu_lib):
    from carpio_gb300.unet import UNet
    net = UNet(seed=3)
    x, t = fields(11, 4, 64, 64)
    losses = [net.train_step(x, t, 1e-3) for _ in range(40)]
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])
    # the loss the step reports is the loss of the weights it started from
    l2, _ = net.grad(x, t)
    assert l2 < losses[-1]


def test_set_and_get_parameters_round_trip(gpu_lib):
    from carpio_gb300.unet import UNet
    a, b = UNet(seed=4), UNet(seed=5)
    assert not np.array_equal(a.params(), b.params())
    b.set_params(a.params())
    assert np.array_equal(a.params(), b.params())
    x, _ = fields(3, 2, 64, 64)
    za, zb = a.forward(x), b.forward(x)
    assert np.array_equal(za.cpu().numpy(), zb.cpu().numpy())
