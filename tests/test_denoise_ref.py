"""The denoiser's FP64 CPU restatement is pinned before it checks the GPU:
its hand-written backward equals torch autograd on the unrounded graph, and
its layer table / parameter packing equal the library's.  No GPU needed."""
import numpy as np
import pytest
import torch

import unet_ref as R
from voidray_gb300 import denoise as D


def random_params(seed=0, scale=1.0):
    offs, total = R.offsets()
    rng = np.random.default_rng(seed)
    p = np.zeros(total, np.float32)
    for l, L in enumerate(R.LAYERS):
        c = R.cin(L)
        n = L[4] * 9 * c
        p[offs[l][0]:offs[l][0] + n] = rng.standard_normal(n) * scale * np.sqrt(2.0 / (9 * c))
        p[offs[l][1]:offs[l][1] + L[4]] = rng.standard_normal(L[4]) * 0.05
    return p


def random_batch(n, h, w, seed=1):
    rng = np.random.default_rng(seed)
    rad = rng.gamma(1.0, 0.5, (n, h, w, 4)).astype(np.float32)
    alb = rng.uniform(0.05, 0.95, (n, h, w, 4)).astype(np.float32)
    nrm = rng.standard_normal((n, h, w, 4)).astype(np.float32)
    nrm[..., :3] /= np.linalg.norm(nrm[..., :3], axis=-1, keepdims=True)
    tgt = (rad * rng.uniform(0.7, 1.3, rad.shape)).astype(np.float32)
    return rad, alb, nrm, tgt


def test_reference_backward_equals_autograd():
    p = random_params()
    rad, alb, nrm, tgt = random_batch(2, 16, 16)
    loss, g, _ = R.loss_and_grads(p, rad, alb, nrm, tgt, round_bf16=False)
    loss_a, g_a = R.autograd_grads(p, rad, alb, nrm, tgt)
    assert abs(loss - loss_a) <= 1e-12 * abs(loss_a)
    offs, _ = R.offsets()
    for l in range(len(R.LAYERS)):
        for a, b in [(offs[l][0], offs[l][1]), (offs[l][1], offs[l][1] + R.LAYERS[l][4])]:
            ref = g_a[a:b]
            assert np.max(np.abs(g[a:b] - ref)) <= 1e-10 * max(np.max(np.abs(ref)), 1e-30), l


def test_rounded_reference_stays_close_to_exact():
    """bf16 rounding of activations and activation gradients perturbs the
    gradient by a few tenths of a percent, not more."""
    p = random_params(3)
    rad, alb, nrm, tgt = random_batch(1, 16, 16, seed=4)
    _, g, _ = R.loss_and_grads(p, rad, alb, nrm, tgt, round_bf16=False)
    _, gr, _ = R.loss_and_grads(p, rad, alb, nrm, tgt, round_bf16=True)
    assert np.linalg.norm(gr - g) <= 0.1 * np.linalg.norm(g)


def test_layer_table_matches_library(native):
    offs, total = R.offsets()
    table = D.layers()
    assert len(table) == len(R.LAYERS)
    for l, (L, T) in enumerate(zip(R.LAYERS, table)):
        c1 = R.ACTS[L[0]][0]
        c2 = R.ACTS[L[1]][0] if L[1] else 0
        assert (T.c1, T.c2, T.up1, T.cout, T.relu) == (c1, c2, L[2], L[4], L[5]), l
        assert (T.w_offset, T.b_offset) == offs[l], l
    info = native._native.vr_denoiser_info()
    import ctypes as C

    native._native.check(native.lib().vr_denoiser_info_get(None, C.byref(info)))
    assert info.param_count == total == 1955216
    assert info.flops_per_pixel == pytest.approx(R.flops_per_pixel())
    assert info.input_channels == 9


def test_bf16_bit_helpers_round_to_nearest_even():
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.standard_normal(10000).astype(np.float32) * 100,
                        np.array([1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -0.0, 65504.0, 1e-38], np.float32)])
    bits = D.f32_to_bf16_bits(x)
    ref = torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(bits, ref)
    assert np.array_equal(D.bf16_bits_to_f32(bits), torch.from_numpy(x).to(torch.bfloat16).float().numpy())
