"""The optional depth pre-filter (VH_FLAG_DEPTH_FILTER): the GPU filter
equals a numpy restatement, a filtered frame stream fuses exactly like the
same frames pre-filtered and passed as float depth, and the filter brings the
depth closer to the noise-free scene."""
import numpy as np
import pytest

from helpers import assert_same_blocks, small_scene, volume_for
from vhsdf import _native as N

pytestmark = pytest.mark.gpu


def bilateral_reference(d_mm, min_depth, max_depth, scale=0.001):
    d = d_mm.astype(np.float64) * np.float32(scale)
    h, w = d.shape
    valid = (d > min_depth) & (d <= max_depth)
    out = np.zeros_like(d)
    for v in range(h):
        for u in range(w):
            if not valid[v, u]:
                continue
            d0 = d[v, u]
            sr = 0.005 + 4.5e-3 * d0 * d0
            num = den = 0.0
            for dy in range(-2, 3):
                for dx in range(-2, 3):
                    x, y = u + dx, v + dy
                    if not (0 <= x < w and 0 <= y < h) or not valid[y, x]:
                        continue
                    if abs(d[y, x] - d0) >= 3 * sr:
                        continue
                    wt = np.exp(-(dx * dx + dy * dy) / 8.0 - (d[y, x] - d0) ** 2 / (2 * sr * sr))
                    num += wt * d[y, x]
                    den += wt
            out[v, u] = num / den
    return out


def test_filter_matches_reference(gpu):
    scene = small_scene(w=64, h=48)
    vol = volume_for(scene)
    d, _, _ = scene.render(2)
    got = vol.filter_depth(d)
    want = bilateral_reference(d, vol.params.min_depth, vol.params.max_depth)
    assert np.array_equal(got > 0, want > 0)
    assert np.max(np.abs(got - want)) < 2e-6


def test_filtered_stream_equals_prefiltered_frames(gpu):
    scene = small_scene()
    a = volume_for(scene, flags=N.VH_FLAG_SYNC | N.VH_FLAG_DEPTH_FILTER)
    b = volume_for(scene)
    for f in range(4):
        d, c, p = scene.render(f)
        a.integrate(d, c, p)
        b.integrate(b.filter_depth(d), c, p)
    assert_same_blocks(a.export_blocks(), b.export_blocks())


def test_filter_reduces_depth_noise(gpu):
    scene = small_scene()
    vol = volume_for(scene)
    noisy, _, _ = scene.render(5)
    clean, _, _ = scene.render(5, noise=False)
    f = vol.filter_depth(noisy)
    m = (noisy > 0) & (clean > 0) & (f > 0)
    # away from depth edges, where the filter cannot mix surfaces
    gy, gx = np.gradient(clean.astype(np.float64))
    m &= np.hypot(gx, gy) < 20
    truth = clean[m] * 1e-3
    raw_err = np.sqrt(np.mean((noisy[m] * 1e-3 - truth) ** 2))
    filt_err = np.sqrt(np.mean((f[m] - truth) ** 2))
    assert filt_err < 0.7 * raw_err
