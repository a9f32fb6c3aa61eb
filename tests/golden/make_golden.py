"""Generates tests/golden/tonemap_f64.npz: an FP64 numpy evaluation of
post_process.glsl:23-49 and tonemapping.glsl:2-40 (reference files of
LevKruglyak/voidray, voidray_renderer/src/shaders/), independent of the C++
oracle.  GLSL mat3(a,...,i) is column major: columns (a,b,c), (d,e,f), (g,h,i).
Also tests/golden/tonemap_legacy_f64.npz: the legacy viewport's
post-processing (voidray/src/shaders/viewport_fragment.glsl:27-67 with
voidray/src/shaders/tonemapping.glsl:1-69): linear exposure, Filmic without
gamma, alpha scaled and kept when transparent.

Run: python tests/golden/make_golden.py
"""
from pathlib import Path

import numpy as np


def aces(c):
    a = np.array([0.59719, 0.076, 0.0284, 0.35458, 0.90834, 0.13383, 0.04823, 0.01566, 0.83777]).reshape(3, 3).T
    b = np.array([1.60475, -0.10208, -0.00327, -0.53108, 1.10813, -0.07276, -0.07367, -0.00605, 1.07602]).reshape(3, 3).T
    c = c @ a.T
    c = (c * (c + 0.0245786) - 0.000090537) / (c * (0.983729 * c + 0.432951) + 0.238081)
    return c @ b.T


def reinhard(c):
    white = 2.0
    luma = c @ np.array([0.2126, 0.7152, 0.0722])
    tml = luma * (1.0 + luma / (white * white)) / (1.0 + luma)
    return c * (tml / luma)[..., None]


def filmic(c):
    c = np.maximum(0.0, c - 0.004)
    return (c * (6.2 * c + 0.5)) / (c * (6.2 * c + 1.7) + 0.06)


def uncharted2(c):
    A, B, C, D, E, F, W = 0.15, 0.50, 0.10, 0.20, 0.02, 0.30, 11.2
    f = lambda x: ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F
    return f(c * 2.0) / f(W)


def main():
    rng = np.random.default_rng(2024)
    x = np.concatenate([rng.random((500, 4)) * 3.0, rng.random((100, 4)) * 50.0,
                        np.array([[0, 0, 0, 1], [1, 1, 1, 1], [0.004, 0.5, 2, 1]])]).astype(np.float32)
    gamma, exposure, scale = 2.2, 0.5, 0.8
    c = x[:, :3].astype(np.float64) * scale * 2.0 ** exposure
    out = {"input": x, "gamma": gamma, "exposure": exposure, "scale": scale}
    for k, fn in enumerate([lambda v: v, aces, reinhard, filmic, uncharted2]):
        with np.errstate(all="ignore"):
            y = np.power(fn(c), 1.0 / gamma)
        o = np.ones((len(x), 4))
        o[:, :3] = y
        out[f"out_{k}"] = o
    np.savez(Path(__file__).with_name("tonemap_f64.npz"), **out)

    # legacy viewport: numbering 0..7, exposure multiplies, transparent keeps alpha
    def simple_reinhard(c):
        e = 1.5
        return c * (e / (1.0 + c / e))

    def luma_reinhard(c):
        luma = c @ np.array([0.2126, 0.7152, 0.0722])
        return c * ((luma / (1.0 + luma)) / luma)[..., None]

    def rombindahouse(c):
        return np.exp(-1.0 / (2.72 * c + 0.15))

    legacy = [lambda v: v, aces, simple_reinhard, luma_reinhard, reinhard, rombindahouse, filmic, uncharted2]
    gamma, exposure, scale = 2.2, 1.3, 0.8
    c = x[:, :3].astype(np.float64) * scale * exposure
    lout = {"input": x, "gamma": gamma, "exposure": exposure, "scale": scale}
    for k, fn in enumerate(legacy):
        g = 1.0 if k == 6 else gamma
        with np.errstate(all="ignore"):
            y = np.power(fn(c), 1.0 / g)
        o = np.empty((len(x), 4))
        o[:, :3] = y
        o[:, 3] = x[:, 3].astype(np.float64) * scale  # transparent
        lout[f"out_{k}"] = o
    np.savez(Path(__file__).with_name("tonemap_legacy_f64.npz"), **lout)


if __name__ == "__main__":
    main()
