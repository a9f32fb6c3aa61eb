"""Learned denoiser: Python side of include/voidray_denoise.h.

The network (U-Net, 4 levels of 32/64/128/256 channels, BF16 tensor-core
kernels with fp32 accumulation) lives in the native library; this module
holds the handle, parameter I/O and the calls the renderer and the serving
loop make.  Trained weights ship as ``weights/unet_bf16.npy`` (the parameter
vector rounded to bf16, stored as uint16 bit patterns).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _native as N
from ._native import check, lib

WEIGHTS = Path(__file__).resolve().parent / "weights" / "unet_bf16.npy"


def _p(x) -> C.c_void_p:
    """Device pointer of a torch tensor or a raw int address."""
    if x is None:
        return C.c_void_p(None)
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    return C.c_void_p(int(x) or None)


def bf16_bits_to_f32(bits: np.ndarray) -> np.ndarray:
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def f32_to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even float32 -> bf16 bit patterns."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    nan = np.isnan(np.asarray(x, np.float32))
    out = r.astype(np.uint16)
    out[nan] = 0x7FC0
    return out


def layers() -> list[N.vr_denoiser_layer]:
    out = []
    info = N.vr_denoiser_info()
    check(lib().vr_denoiser_info_get(None, C.byref(info)))
    for i in range(info.num_layers):
        L = N.vr_denoiser_layer()
        check(lib().vr_denoiser_layer_get(i, C.byref(L)))
        out.append(L)
    return out


class Denoiser:
    """vr_denoiser handle (device parameters, Adam state, workspace)."""

    def __init__(self, seed: int = 0, params: np.ndarray | None = None):
        h = C.c_void_p()
        check(lib().vr_denoiser_create(int(seed), C.byref(h)))
        self._h = h
        self.backend = 0
        if params is not None:
            self.set_params(params)

    def clone(self) -> "Denoiser":
        """A second handle with the same weights and backend (its own
        workspace, for use on another stream)."""
        d = Denoiser(params=self.params())
        d.set_backend(self.backend)
        return d

    @classmethod
    def pretrained(cls, path: Path | str = WEIGHTS) -> "Denoiser":
        bits = np.load(path)
        return cls(params=bf16_bits_to_f32(bits))

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise N.VoidrayError(1, "denoiser destroyed")
        return self._h

    def info(self) -> N.vr_denoiser_info:
        info = N.vr_denoiser_info()
        check(lib().vr_denoiser_info_get(self.handle, C.byref(info)))
        return info

    LOSS_L1_LOG = 0
    LOSS_RELMSE = 1

    MMA_SYNC = 0
    TCGEN05 = 1

    def set_backend(self, backend: int) -> None:
        """Forward convolutions on mma.sync (0) or tcgen05 + TMEM + TMA (1)."""
        check(lib().vr_denoiser_set_backend(self.handle, int(backend)))
        self.backend = int(backend)

    def status(self) -> int:
        """Synchronises; raises VoidrayError if a tcgen05 kernel gave up a bounded wait."""
        f = C.c_uint32()
        check(lib().vr_denoiser_status(self.handle, C.byref(f)))
        return f.value

    def set_loss(self, kind: int) -> None:
        check(lib().vr_denoiser_set_loss(self.handle, int(kind)))

    def params(self) -> np.ndarray:
        n = self.info().param_count
        out = np.empty(n, np.float32)
        check(lib().vr_denoiser_get_params(self.handle, out.ctypes.data, n))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(lib().vr_denoiser_set_params(self.handle, p.ctypes.data, p.size))

    def save(self, path: Path | str) -> None:
        np.save(path, f32_to_bf16_bits(self.params()))

    def denoise(self, rgba, albedo, normal, scale: float, out, width: int, height: int, stream: int = 0) -> None:
        """Device buffers (torch tensors or addresses), RGBA f32 width x height."""
        check(lib().vr_denoise_device(self.handle, _p(rgba), _p(albedo), _p(normal), float(scale), _p(out),
                                      int(width), int(height), C.c_void_p(stream or None)))

    def denoise_batch(self, rgba, albedo, normal, scales, out, width: int, height: int, stream: int = 0) -> None:
        """Images stacked as [batch][height][width][4] device buffers; scales: one float per image."""
        sc = np.ascontiguousarray(scales, np.float32)
        check(lib().vr_denoise_batch_device(self.handle, _p(rgba), _p(albedo), _p(normal), sc.ctypes.data, _p(out),
                                            int(sc.size), int(width), int(height), C.c_void_p(stream or None)))

    def gradients(self, rgba, albedo, normal, target, batch: int, width: int, height: int, scale_in: float = 1.0,
                  scale_target: float = 1.0, stream: int = 0):
        """(loss, gradient vector) of one batch, no update."""
        loss = C.c_float()
        g = np.empty(self.info().param_count, np.float32)
        check(lib().vr_denoiser_gradients_device(self.handle, _p(rgba), _p(albedo), _p(normal), _p(target),
                                                 float(scale_in), float(scale_target), int(batch), int(width),
                                                 int(height), C.byref(loss), g.ctypes.data,
                                                 C.c_void_p(stream or None)))
        return float(loss.value), g

    def train_step(self, rgba, albedo, normal, target, batch: int, width: int, height: int, lr: float,
                   scale_in: float = 1.0, scale_target: float = 1.0, want_loss: bool = False, stream: int = 0):
        loss = C.c_float()
        check(lib().vr_denoiser_train_step_device(self.handle, _p(rgba), _p(albedo), _p(normal), _p(target),
                                                  float(scale_in), float(scale_target), int(batch), int(width),
                                                  int(height), float(lr), C.byref(loss) if want_loss else None,
                                                  C.c_void_p(stream or None)))
        return float(loss.value) if want_loss else None

    def destroy(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().vr_denoiser_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def conv3x3(src1, c1: int, weight, cout: int, n: int, h: int, w: int, *, src2=None, c2: int = 0, up1: bool = False,
            bias=None, mask=None, out_bf16=None, out_f32=None, relu: bool = False, stream: int = 0) -> None:
    """Single forward / backward-data convolution kernel (device pointers)."""
    check(lib().vr_dn_conv3x3_device(_p(src1), int(c1), int(up1), _p(src2), int(c2), _p(weight), _p(bias), _p(mask),
                                     _p(out_bf16), _p(out_f32), int(cout), int(n), int(h), int(w), int(relu),
                                     C.c_void_p(stream or None)))


def conv3x3_tc(src1, c1: int, weight, cout: int, n: int, h: int, w: int, *, src2=None, c2: int = 0, bias=None,
               mask=None, out_bf16=None, out_f32=None, relu: bool = False, status=None, stream: int = 0) -> None:
    """Single convolution on tcgen05 (device pointers)."""
    check(lib().vr_dn_conv3x3_tc_device(_p(src1), int(c1), _p(src2), int(c2), _p(weight), _p(bias), _p(mask),
                                        _p(out_bf16), _p(out_f32), int(cout), int(n), int(h), int(w), int(relu),
                                        _p(status), C.c_void_p(stream or None)))


def conv3x3_wgrad(dz, src1, c1: int, dw, cout: int, n: int, h: int, w: int, *, src2=None, c2: int = 0,
                  up1: bool = False, stream: int = 0) -> None:
    """Single weight-gradient kernel: dw (f32, [cout][9][c1+c2]) += ..."""
    check(lib().vr_dn_conv3x3_wgrad_device(_p(dz), _p(src1), int(c1), int(up1), _p(src2), int(c2), _p(dw), int(cout),
                                           int(n), int(h), int(w), C.c_void_p(stream or None)))
