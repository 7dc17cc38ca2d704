"""Lightmap images (lighter_gb300.images): the test harness's TGA layout and
Radiance HDR, on small hand-made images (CPU only)."""
import numpy as np
import pytest

from lighter_gb300 import images


def test_tga_header_rows_and_channels():
    img = np.zeros((2, 3, 3), np.float32)
    img[0, 0] = (1.0, 0.5, 0.25)    # first lightmap row, first texel
    img[1, 2] = (0.0, 0.0, 2.0)     # last row, last texel: clamps to 255
    b = images.tga_bytes(img)
    assert len(b) == 18 + 2 * 3 * 3
    assert b[2] == 2 and b[16] == 24
    assert (b[12] | b[13] << 8, b[14] | b[15] << 8) == (3, 2)
    px = np.frombuffer(b, np.uint8, offset=18).reshape(2, 3, 3)
    # stored last row first, B G R, values truncated: 0.5 * 255 = 127.5 -> 127, 0.25 * 255 = 63.75 -> 63
    assert tuple(px[1, 0]) == (63, 127, 255)
    assert tuple(px[0, 2]) == (255, 0, 0)


def test_tga_top_scale_negative_and_alpha():
    img = np.array([[[-1.0, 2.0, 4.0, 0.5]]], np.float32)
    b = images.tga_bytes(img, top=4.0)
    assert b[16] == 32
    assert tuple(np.frombuffer(b, np.uint8, offset=18)) == (255, 127, 0, 31)   # B G R A, mult 63.75


def test_normals_for_display():
    n = np.array([[[-1.0, 0.0, 1.0, 0.7]]], np.float32)
    np.testing.assert_allclose(images.normals_for_display(n), [[[0.0, 0.5, 1.0, 0.7]]])


def test_hdr_round_trip_within_rgbe_precision(tmp_path):
    rng = np.random.default_rng(3)
    img = (rng.random((5, 7, 3)) * np.logspace(-3, 3, 7)[None, :, None]).astype(np.float32)
    img[0, 0] = 0.0
    p = tmp_path / "lm.hdr"
    images.write_hdr(str(p), img)
    back = images.read_hdr(p.read_bytes())
    assert back.shape == img.shape and float(back[0, 0].max()) == 0.0
    peak = img.max(axis=-1, keepdims=True)
    # the shared exponent keeps 8 bits of the largest channel: error < 1/128 of the texel's peak
    assert float((np.abs(back - img) / np.maximum(peak, 1e-30)).max()) < 1.0 / 128


def test_rejects_bad_shapes():
    with pytest.raises(ValueError):
        images.tga_bytes(np.zeros((2, 2), np.float32))
    with pytest.raises(ValueError):
        images.hdr_bytes(np.zeros((2, 2, 4), np.float32))
