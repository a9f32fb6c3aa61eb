"""The tcgen05 (TMEM accumulator, TMA-staged operands) convolution against the
FP64 CPU restatement, with the same bound as the mma.sync kernel: half a bf16
ulp of the exact result plus the fp32 accumulation error; and the whole
network's forward pass on tcgen05 against its mma.sync forward pass."""
import os
import subprocess
import sys

import numpy as np
import pytest

import unet_ref as R
from voidray_gb300 import denoise as D

from test_gpu_denoise import batch_arrays, conv_ref, rand_bf16, ulp_bf16

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TC_CASES = [  # c1, c2, cout, n, h, w, relu, bias, f32 (mask when relu == 2)
    (16, 0, 32, 1, 8, 16, 1, 1, 0),      # one tile, first-layer shape (16-channel chunks)
    (16, 0, 32, 2, 16, 16, 1, 1, 0),
    (32, 0, 64, 1, 24, 40, 1, 1, 0),     # partial tiles at the right edge
    (64, 0, 128, 2, 8, 8, 1, 1, 0),      # image smaller than a tile
    (128, 0, 256, 1, 8, 16, 1, 1, 0),
    (256, 128, 128, 1, 16, 16, 1, 1, 0),  # concatenated sources (128-byte swizzle)
    (64, 32, 32, 2, 16, 8, 1, 1, 0),     # 64 + 32: 32-channel chunks
    (32, 0, 16, 1, 16, 16, 0, 1, 1),     # output layer, fp32
    (64, 0, 192, 1, 8, 24, 0, 0, 0),
    (16, 0, 32, 1, 16, 16, 2, 0, 0),     # backward-data shapes: ReLU mask epilogue
    (128, 0, 384, 1, 8, 8, 2, 0, 0),     # 384 output channels: two 192-channel tiles
    (32, 0, 96, 2, 8, 16, 2, 0, 0),
]


@pytest.mark.parametrize("case", TC_CASES)
def test_conv3x3_tc_matches_fp64(gpu, case):
    c1, c2, cout, n, h, w, relu, bias, f32 = case
    rng = np.random.default_rng(100 + sum(case))
    x1 = rand_bf16((n, h, w, c1), rng)
    x2 = rand_bf16((n, h, w, c2), rng) if c2 else None
    wgt = rand_bf16((cout, 9, c1 + c2), rng, scale=np.sqrt(2.0 / (9 * (c1 + c2))))
    b = torch.from_numpy(rng.standard_normal(cout).astype(np.float32) * 0.1) if bias else None
    y, s = conv_ref(x1, x2, 0, wgt, b)
    m = rand_bf16((n, h, w, cout), rng) if relu == 2 else None
    if relu == 1:
        y = np.maximum(y, 0.0)
    if m is not None:
        y = np.where(m.float().numpy() > 0, y, 0.0)
    dev = lambda t: None if t is None else t.cuda()
    out = torch.full((n, h, w, cout), 7.0, dtype=torch.float32 if f32 else torch.bfloat16, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    D.conv3x3_tc(dev(x1), c1, dev(wgt), cout, n, h, w, src2=dev(x2), c2=c2, bias=dev(b), mask=dev(m),
                 out_bf16=None if f32 else out, out_f32=out if f32 else None, relu=relu == 1, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    g = out.double().cpu().numpy()
    tol = (0.0 if f32 else 0.5 * ulp_bf16(y)) + 2.0 ** -20 * s + 1e-30
    bad = np.abs(g - y) > tol
    assert not bad.any(), (np.argwhere(bad)[:5], g[bad][:5], y[bad][:5])


@pytest.mark.parametrize("variant", ["tile", "halo"])
def test_conv3x3_tc_each_variant_on_every_case(gpu, variant):
    """The library picks the tile or the halo kernel by output-channel count;
    forcing one variant (VR_DN_TC_VARIANT, read once per process) runs every
    case above through it, in a child process."""
    env = dict(os.environ, VR_DN_TC_VARIANT=variant)
    r = subprocess.run([sys.executable, "-m", "pytest", os.path.abspath(__file__), "-q", "-p", "no:cacheprovider",
                        "-k", "test_conv3x3_tc_matches_fp64"], env=env, capture_output=True, text=True,
                       timeout=900, cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]


def test_tc_rejects_what_it_does_not_cover(gpu):
    x = torch.zeros(64 * 128, dtype=torch.bfloat16, device="cuda")
    with pytest.raises(D.N.VoidrayError) as e:   # Cout 24: not a multiple of 16
        D.conv3x3_tc(x, 16, x, 24, 1, 8, 8, out_bf16=x)
    assert e.value.status == 2


def test_network_forward_tc_equals_mma_sync(gpu):
    """Inference through the tcgen05 forward (with materialised upsampling)
    against the mma.sync forward and the FP64 restatement."""
    net = D.Denoiser(seed=8)
    try:
        p = net.params()
        h, w = 64, 48
        rad, alb, nrm, _ = batch_arrays(1, h, w, 12)
        t = [torch.from_numpy(a[0]).cuda() for a in (rad, alb, nrm)]
        outs = []
        for backend in (D.Denoiser.MMA_SYNC, D.Denoiser.TCGEN05):
            net.set_backend(backend)
            o = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
            net.denoise(*t, 1.0, o, w, h)
            assert net.status() == 0
            outs.append(o.cpu().numpy())
        ref = R.denoise(p, rad[0], alb[0], nrm[0], 1.0)
        for o in outs:
            rel = np.mean((o[..., :3] - ref[..., :3]) ** 2 / (ref[..., :3] ** 2 + 1e-2))
            assert rel < 1e-4, rel
        rel = np.mean((outs[0][..., :3] - outs[1][..., :3]) ** 2 / (outs[0][..., :3] ** 2 + 1e-2))
        assert rel < 1e-4, rel
    finally:
        net.destroy()


def test_network_gradients_tc_backend_match_fp64(gpu):
    """Training on the tcgen05 backend (forward and backward-data on tcgen05,
    weight gradients on mma.sync).  Every single convolution is within half a
    bf16 ulp plus the fp32 accumulation bound (above); through the network
    the tensor-core accumulation order flips a few bf16 roundings of the
    activations by one ulp and the flips compound down the backward pass, so
    the per-layer bound is the one the mma.sync network test uses where
    flips occur (5% L2 per layer, cosine > 0.999 overall), far from what a
    wrong index or a missing term produces."""
    net = D.Denoiser(seed=11)
    try:
        net.set_backend(D.Denoiser.TCGEN05)
        p = net.params()
        offs, _ = R.offsets()
        n, h, w = 1, 16, 16
        rad, alb, nrm, _ = batch_arrays(n, h, w, 3)
        tgt = (1e4 * (rad + 0.5)).astype(np.float32)
        t = [torch.from_numpy(a).cuda() for a in (rad, alb, nrm, tgt)]
        loss, g = net.gradients(*t, n, w, h)
        assert net.status() == 0
        loss_r, g_r, _ = R.loss_and_grads(p, rad, alb, nrm, tgt)
        assert loss == pytest.approx(loss_r, rel=2e-3)
        errs = []
        for l, L in enumerate(R.LAYERS):
            for a, b in [(offs[l][0], offs[l][1]), (offs[l][1], offs[l][1] + L[4])]:
                ref = g_r[a:b]
                nr = np.linalg.norm(ref)
                if nr == 0:
                    assert np.all(g[a:b] == 0)
                    continue
                errs.append((l, float(np.linalg.norm(g[a:b] - ref) / nr)))
        assert max(e for _, e in errs) <= 5e-2, errs
        cos = float(np.dot(g, g_r) / (np.linalg.norm(g) * np.linalg.norm(g_r)))
        assert cos > 0.999, (cos, errs)
    finally:
        net.destroy()
