"""GPU checks of the tensor-core 3x3 convolution (tcgen05 implicit GEMM,
carpio_gpu_nn_conv3x3) against an FP64 numpy convolution of the same BF16
inputs: tile shapes across image rows and across images, two concatenated
inputs, split outputs, ReLU and ReLU masks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def conv_ref(x, wt):
    """x [n, h, w, ci] float64, wt [9, co, ci]: zero-padded 3x3 convolution"""
    n, h, w, ci = x.shape
    xp = np.zeros((n, h + 2, w + 2, ci))
    xp[:, 1:-1, 1:-1] = x
    out = np.zeros((n, h, w, wt.shape[1]))
    for dy in range(3):
        for dx in range(3):
            out += np.einsum("nhwc,oc->nhwo", xp[:, dy:dy + h, dx:dx + w], wt[dy * 3 + dx])
    return out


def bf16(rng, shape, scale=1.0):
    import torch
    a = torch.from_numpy(rng.uniform(-scale, scale, shape).astype(np.float32))
    t = a.to(torch.bfloat16).cuda().contiguous()
    return t, t.float().cpu().numpy().astype(np.float64)


def run(gpu_lib, n, h, w, cin0, cin1, cout, split=0, relu=0, masks=False, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    x0, x0h = bf16(rng, (n, h, w, cin0))
    x1, x1h = (bf16(rng, (n, h, w, cin1)) if cin1 else (None, None))
    ci = cin0 + cin1
    wt, wth = bf16(rng, (9, cout, ci), 1.0 / np.sqrt(9 * ci))
    s = split or cout
    out0 = torch.zeros((n, h, w, s), dtype=torch.bfloat16, device="cuda")
    out1 = torch.zeros((n, h, w, cout - s), dtype=torch.bfloat16, device="cuda") if s < cout else None
    m0 = m1 = None
    if masks:
        m0 = torch.from_numpy(rng.uniform(-1, 1, (n, h, w, s)).astype(np.float32)).to(torch.bfloat16).cuda()
        if out1 is not None:
            m1 = torch.from_numpy(rng.uniform(-1, 1, (n, h, w, cout - s)).astype(np.float32)).to(torch.bfloat16).cuda()
    p = lambda t: None if t is None else t.data_ptr()
    rc = gpu_lib.carpio_gpu_nn_conv3x3(p(x0), cin0, p(x1), cin1, n, h, w, p(wt), cout,
                                       p(out0), split, p(out1), p(m0), p(m1), relu, None)
    assert rc == 0, rc
    xin = x0h if x1h is None else np.concatenate([x0h, x1h], axis=3)
    ref = conv_ref(xin, wth)
    if relu:
        ref = np.maximum(ref, 0)
    got = out0.float().cpu().numpy()
    if out1 is not None:
        got = np.concatenate([got, out1.float().cpu().numpy()], axis=3)
    if masks:
        mk = m0.float().cpu().numpy()
        if m1 is not None:
            mk = np.concatenate([mk, m1.float().cpu().numpy()], axis=3)
        ref = np.where(mk > 0, ref, 0.0)
    # FP32 accumulation of exact BF16 products, one BF16 rounding of the result
    err = np.abs(got - ref)
    tol = 2.0 ** -8 * np.abs(ref) + 1e-3 * np.abs(ref).max() + 1e-6
    assert np.all(err <= tol), (err.max(), np.abs(ref).max())
    return got


def test_conv_tile_within_rows(gpu_lib):
    run(gpu_lib, 2, 8, 128, 32, 0, 32)


def test_conv_tile_across_rows_and_images(gpu_lib):
    run(gpu_lib, 2, 16, 64, 64, 0, 64, seed=1)       # 64 x 2 pixel tiles
    run(gpu_lib, 8, 4, 4, 32, 0, 32, seed=2)         # 8 whole 4x4 images per tile


def test_conv_wide_output_and_relu(gpu_lib):
    run(gpu_lib, 1, 16, 32, 128, 0, 256, relu=1, seed=3)


def test_conv_concatenated_inputs(gpu_lib):
    run(gpu_lib, 2, 8, 32, 64, 32, 64, relu=1, seed=4)


def test_conv_split_outputs_with_masks(gpu_lib):
    # the backward pass of a concatenating layer: 384 = 256 + 128 channels
    run(gpu_lib, 1, 8, 16, 128, 0, 384, split=256, masks=True, seed=5)
    run(gpu_lib, 1, 8, 16, 64, 0, 96, split=64, masks=True, seed=6)
