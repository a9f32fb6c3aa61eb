"""GPU parity for the legacy extras: MixMaterial scenes against the oracle
(same sample streams, so pixels match bit for bit where the arithmetic is
free of transcendentals), and the legacy viewport tonemaps against the
oracle's restatement."""
import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import workloads as W

from test_gpu_render import exact_fraction, gpu_render

pytestmark = pytest.mark.gpu


def test_mix_scene_bit_parity(gpu, oracle):
    s, st = W.mix_scene()
    g = gpu_render(s, st, 4, 48, 32)
    o, _ = oracle.OracleScene(s).render(st, 4, 48, 32)
    assert exact_fraction(g, o) >= 0.99


def test_mix_scene_nee_matches_reference_estimator(gpu):
    """With the NEE estimator under an importance-sampled HDRI, mixed
    Lambertian vertices take light samples; both estimators converge to the
    same image.  The reference estimator rarely finds the small sun, so its
    own noise dominates: on the oracle, two reference renders of this scene
    differ by relMSE 0.36 at 256 spp and 0.07 at 1024, NEE against reference
    by 0.10 and 0.030 (the 1/spp decay of noise, no bias); at 4096 spp the
    expected gap is about 0.008."""
    s, st = W.mix_scene(hdri=True)
    acc = s.build_acceleration()
    spp = 4096
    st.total_samples = spp
    ref = gpu_render(s, st, spp, 32, 24, acc=acc, seed=1)
    st.estimator = vr.Estimator.NEE
    nee = gpu_render(s, st, spp, 32, 24, acc=acc, seed=2)
    a, b = ref[..., :3].astype(np.float64), nee[..., :3].astype(np.float64)
    rel = np.mean((a - b) ** 2 / (b ** 2 + 1e-2))
    assert rel < 0.025, rel
    assert abs(a.mean() - b.mean()) < 0.01 * b.mean()


@pytest.mark.parametrize("tm", range(8))
@pytest.mark.parametrize("transparent", [False, True])
def test_legacy_tonemap(gpu, oracle, tm, transparent):
    rng = np.random.default_rng(tm)
    img = (rng.random((37, 53, 4)) * 4).astype(np.float32)
    g = vr.tonemap_legacy(img, vr.LegacyTonemap(tm), 2.2, 1.3, transparent, 0.7)
    o = oracle.tonemap_legacy(img, tm, 2.2, 1.3, transparent, 0.7)
    assert np.allclose(g, o, rtol=2e-6, atol=1e-7, equal_nan=True)
