"""FP64 CPU restatement of the denoiser network — TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and bench.py's CPU legs may import this module;
the product never does.  voidray has no denoiser (it only accumulates
samples, voidray_renderer/src/render/iterative.rs:11-55), so this file
restates the library's own network definition (include/voidray_denoise.h)
independently, in float64 with torch on the CPU:

  * forward: the same 15 3x3 convolutions, 2x2 average pools, nearest 2x
    upsampling and skip concatenation, with activations rounded to bf16 at
    the points where the GPU kernels store bf16 (so the comparison isolates
    accumulation-order effects);
  * backward: written out by hand in the order the GPU runs it, rounding the
    activation gradients to bf16 at the same points (the L1 loss gradient,
    each backward-data output, the concatenation gradient, the upsample and
    skip backward results); weight and bias gradients stay float64.

With rounding switched off the hand-written backward must equal torch
autograd on the same float64 graph (tests/test_denoise_ref.py pins this).
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

DEMOD_EPS = 0.01
OUT_C = 16
# activation name -> (channels, level)
ACTS = {"X0": (16, 0), "A0A": (32, 0), "S0": (32, 0), "P0": (32, 1), "A1A": (64, 1), "S1": (64, 1), "P1": (64, 2),
        "A2A": (128, 2), "S2": (128, 2), "P2": (128, 3), "BA": (256, 3), "BT": (256, 3), "D2A": (128, 2),
        "U2": (128, 2), "D1A": (64, 1), "U1": (64, 1), "D0A": (32, 0), "U0": (32, 0)}
# (in1, in2, up1, out, cout, relu)
LAYERS = [("X0", None, 0, "A0A", 32, 1), ("A0A", None, 0, "S0", 32, 1), ("P0", None, 0, "A1A", 64, 1),
          ("A1A", None, 0, "S1", 64, 1), ("P1", None, 0, "A2A", 128, 1), ("A2A", None, 0, "S2", 128, 1),
          ("P2", None, 0, "BA", 256, 1), ("BA", None, 0, "BT", 256, 1), ("BT", "S2", 1, "D2A", 128, 1),
          ("D2A", None, 0, "U2", 128, 1), ("U2", "S1", 1, "D1A", 64, 1), ("D1A", None, 0, "U1", 64, 1),
          ("U1", "S0", 1, "D0A", 32, 1), ("D0A", None, 0, "U0", 32, 1), ("U0", None, 0, "OUT", OUT_C, 0)]
POOLS = {1: ("S0", "P0"), 3: ("S1", "P1"), 5: ("S2", "P2")}
SKIP_CONSUMER = {"S0": 12, "S1": 10, "S2": 8}


def cin(layer) -> int:
    in1, in2 = layer[0], layer[1]
    return ACTS[in1][0] + (ACTS[in2][0] if in2 else 0)


def offsets():
    """(w_offset, b_offset) per layer and the parameter count, packed like the library."""
    out, at = [], 0
    for L in LAYERS:
        w = at
        at += L[4] * 9 * cin(L)
        out.append((w, at))
        at += L[4]
    return out, at


def flops_per_pixel() -> float:
    f = 0.0
    for L in LAYERS:
        lvl = ACTS[L[1]][1] if L[1] else ACTS[L[0]][1]
        f += 2.0 * 9 * cin(L) * L[4] / 4 ** lvl
    return f


def bf16(t: torch.Tensor, on: bool = True) -> torch.Tensor:
    return t.to(torch.bfloat16).to(torch.float64) if on else t


def weights(params: np.ndarray, l: int, round_bf16: bool = True):
    """Layer l's (weight (cout, cin, 3, 3), bias) as float64; weight bf16-rounded like the kernels."""
    offs, _ = offsets()
    wo, bo = offs[l]
    L = LAYERS[l]
    c = cin(L)
    w = torch.from_numpy(np.asarray(params[wo:wo + L[4] * 9 * c], np.float32))
    w = w.to(torch.float64).reshape(L[4], 3, 3, c).permute(0, 3, 1, 2).contiguous()
    b = torch.from_numpy(np.asarray(params[bo:bo + L[4]], np.float32)).to(torch.float64)
    return bf16(w, round_bf16), b


def preprocess(rad, alb, nrm, scale: float, round_bf16: bool = True) -> torch.Tensor:
    """(N, H, W, 4) f32 arrays -> X0 (N, 16, H, W) float64."""
    r = torch.from_numpy(np.asarray(rad, np.float32)).to(torch.float64) * scale
    a = torch.from_numpy(np.asarray(alb, np.float32)).to(torch.float64) * scale
    q = torch.from_numpy(np.asarray(nrm, np.float32)).to(torch.float64) * scale
    lg = torch.log1p(torch.clamp(r[..., :3], min=0.0) / (a[..., :3] + DEMOD_EPS))
    x = torch.cat([lg, a[..., :3], q[..., :3], torch.zeros(*r.shape[:3], 7, dtype=torch.float64)], -1)
    return bf16(x.permute(0, 3, 1, 2).contiguous(), round_bf16)


def log_target(target, alb, scale_target: float, scale_in: float) -> torch.Tensor:
    t = torch.from_numpy(np.asarray(target, np.float32)).to(torch.float64)[..., :3] * scale_target
    a = torch.from_numpy(np.asarray(alb, np.float32)).to(torch.float64)[..., :3] * scale_in
    return torch.log1p(torch.clamp(t, min=0.0) / (a + DEMOD_EPS)).permute(0, 3, 1, 2)


def _input(acts, L):
    a = acts[L[0]]
    if L[2]:
        a = a.repeat_interleave(2, -2).repeat_interleave(2, -1)
    if L[1]:
        a = torch.cat([a, acts[L[1]]], 1)
    return a


def forward(params: np.ndarray, x0: torch.Tensor, round_bf16: bool = True) -> dict:
    acts = {"X0": x0}
    for l, L in enumerate(LAYERS):
        w, b = weights(params, l, round_bf16)
        z = F.conv2d(_input(acts, L), w, b, padding=1)
        if L[5]:
            z = torch.relu(z)
        acts[L[3]] = z if L[3] == "OUT" else bf16(z, round_bf16)
        if l in POOLS:
            s, p = POOLS[l]
            acts[p] = bf16(F.avg_pool2d(acts[s], 2), round_bf16)
    return acts


def l1_loss_grad(out: torch.Tensor, tlog: torch.Tensor, round_bf16: bool = True):
    """Mean |o - t| over the 3 colour channels and its gradient (N, OUT_C, H, W)."""
    d = out[:, :3] - tlog
    count = d.numel()
    g = torch.zeros_like(out)
    g[:, :3] = torch.sign(d) / count
    return float(d.abs().sum() / count), bf16(g, round_bf16)


def backward(params: np.ndarray, acts: dict, gout: torch.Tensor, round_bf16: bool = True) -> np.ndarray:
    """Parameter gradient (float64, packed like the parameter vector)."""
    offs, total = offsets()
    grads = np.zeros(total, np.float64)
    cur = gout
    dcat = {}
    for l in range(len(LAYERS) - 1, -1, -1):
        L = LAYERS[l]
        w, _ = weights(params, l, round_bf16)
        x = _input(acts, L)
        dw = torch.nn.grad.conv2d_weight(x, w.shape, cur, padding=1)      # (cout, cin, 3, 3)
        grads[offs[l][0]:offs[l][0] + dw.numel()] = dw.permute(0, 2, 3, 1).reshape(-1).numpy()
        grads[offs[l][1]:offs[l][1] + L[4]] = cur.sum((0, 2, 3)).numpy()
        if l == 0:
            break
        dx = torch.nn.grad.conv2d_input(x.shape, w, cur, padding=1)
        if L[1]:
            dcat[l] = bf16(dx, round_bf16)
            c1 = ACTS[L[0]][0]
            up = dcat[l][:, :c1]
            du = up[:, :, 0::2, 0::2] + up[:, :, 0::2, 1::2] + up[:, :, 1::2, 0::2] + up[:, :, 1::2, 1::2]
            nxt = bf16(du * (acts[L[0]] > 0), round_bf16)
        elif L[0] in ("P0", "P1", "P2"):
            dpool = bf16(dx, round_bf16)
            s = {"P0": "S0", "P1": "S1", "P2": "S2"}[L[0]]
            k = SKIP_CONSUMER[s]
            c1k = ACTS[LAYERS[k][0]][0]
            up = dpool.repeat_interleave(2, -2).repeat_interleave(2, -1)
            nxt = bf16((dcat[k][:, c1k:] + 0.25 * up) * (acts[s] > 0), round_bf16)
        else:
            nxt = bf16(dx * (acts[L[0]] > 0), round_bf16)
        cur = nxt
    return grads


def loss_and_grads(params, rad, alb, nrm, target, scale_in=1.0, scale_target=1.0, round_bf16=True):
    x0 = preprocess(rad, alb, nrm, scale_in, round_bf16)
    acts = forward(params, x0, round_bf16)
    loss, g = l1_loss_grad(acts["OUT"], log_target(target, alb, scale_target, scale_in), round_bf16)
    return loss, backward(params, acts, g, round_bf16), acts


def denoise(params, rad, alb, nrm, scale=1.0) -> np.ndarray:
    """Inference on (H, W, 4) buffers with H, W multiples of 8 -> (H, W, 4) float64 radiance, alpha 1."""
    x0 = preprocess(rad[None], alb[None], nrm[None], scale)
    o = forward(params, x0)["OUT"][0, :3].permute(1, 2, 0)
    a = torch.from_numpy(np.asarray(alb, np.float32)).to(torch.float64)[..., :3] * scale
    rgb = torch.expm1(torch.clamp(o, 0.0, 80.0)) * (a + DEMOD_EPS)
    return torch.cat([rgb, torch.ones_like(rgb[..., :1])], -1).numpy()


def autograd_grads(params, rad, alb, nrm, target, scale_in=1.0, scale_target=1.0):
    """Loss gradient by torch autograd on the unrounded float64 graph (pins backward())."""
    offs, total = offsets()
    x0 = preprocess(rad, alb, nrm, scale_in, False)
    ws, bs = [], []
    for l in range(len(LAYERS)):
        w, b = weights(params, l, False)
        ws.append(w.clone().requires_grad_(True))
        bs.append(b.clone().requires_grad_(True))
    acts = {"X0": x0}
    for l, L in enumerate(LAYERS):
        z = F.conv2d(_input(acts, L), ws[l], bs[l], padding=1)
        acts[L[3]] = torch.relu(z) if L[5] else z
        if l in POOLS:
            s, p = POOLS[l]
            acts[p] = F.avg_pool2d(acts[s], 2)
    tlog = log_target(target, alb, scale_target, scale_in)
    loss = (acts["OUT"][:, :3] - tlog).abs().mean()
    loss.backward()
    grads = np.zeros(total, np.float64)
    for l in range(len(LAYERS)):
        dw = ws[l].grad
        grads[offs[l][0]:offs[l][0] + dw.numel()] = dw.permute(0, 2, 3, 1).reshape(-1).numpy()
        grads[offs[l][1]:offs[l][1] + LAYERS[l][4]] = bs[l].grad.numpy()
    return float(loss.detach()), grads
