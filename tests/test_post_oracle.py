"""Tonemapping and denoising oracles on the CPU: the tonemap restatement
against the reference's own include/cuda/color.cuh (golden vectors from
tests/golden/gen_golden.py), bit for bit; the denoiser restatement's basic
properties (a constant image is a fixed point; noise falls; edges between a
hit and a miss are kept)."""
import json
import os

import numpy as np

from oracle import post_ref, pyoracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")


def test_tonemap_matches_reference_color_cuh():
    kat = json.load(open(GOLDEN))["tonemap"]
    hdr = np.array([e["c"] + [1.0] for e in kat], np.float32).reshape(1, -1, 4)
    for mode, key in ((0, "aces"), (1, "srgb")):
        got = pyoracle.tonemap(hdr, mode)[0]
        ref = np.array([e[key] for e in kat], np.uint32)
        np.testing.assert_array_equal(got, ref)
        assert np.all(got >> 24 == 255)  # alpha in the top byte (cast.cuh to_ui32)


def test_tonemap_flips_rows():
    hdr = np.zeros((3, 2, 4), np.float32)
    hdr[0, :, :3] = 10.0  # top row white
    out = pyoracle.tonemap(hdr)
    assert np.all(out[2] == out[2][0]) and (out[2][0] & 0xFF) == 255  # written to the last row
    assert np.all(out[0] & 0xFF == 0)


def planar_scene(h=48, w=48, seed=0):
    rng = np.random.default_rng(seed)
    normal = np.zeros((h, w, 4), np.float32)
    normal[..., 2] = 1.0
    normal[:, : w // 4] = 0.0  # a band without hits
    albedo = np.full((h, w, 4), 0.5, np.float32)
    pos = np.zeros((h, w, 4), np.float32)
    pos[..., 0], pos[..., 1] = np.meshgrid(np.arange(w, dtype=np.float32), np.arange(h, dtype=np.float32))
    clean = np.zeros((h, w, 4), np.float32)
    clean[..., :3] = 0.4
    clean[:, : w // 4, :3] = 0.0
    noisy = clean.copy()
    noisy[:, w // 4:, :3] *= rng.exponential(1.0, (h, w - w // 4, 1)).astype(np.float32)
    return clean, noisy, normal, albedo, pos


def test_denoiser_oracle_properties():
    clean, noisy, normal, albedo, pos = planar_scene()
    g = post_ref.NORMAL | post_ref.ALBEDO | post_ref.POSITION
    const = post_ref.denoise(clean, normal, albedo, pos, g)
    np.testing.assert_allclose(const[..., :3], clean[..., :3], rtol=1e-5, atol=1e-7)
    out = post_ref.denoise(noisy, normal, albedo, pos, g)
    err = lambda x: np.mean((x[..., :3] - clean[..., :3]) ** 2)
    assert err(out) < 0.2 * err(noisy)
    assert np.all(out[:, : clean.shape[1] // 4, :3] == 0.0)  # misses stay black
