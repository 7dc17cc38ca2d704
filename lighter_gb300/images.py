"""Lightmap images: the reference test harness's TGA dumps, and Radiance HDR.

`tga_bytes` / `write_tga` encode a work output the way the reference's test
harness dumps it (lighter_test.cpp:111-163, `dumpimg`): an uncompressed
true-colour TGA (image type 2, 24 bits, or 32 with alpha), 18-byte header,
rows stored from the last lightmap row to the first (the TGA origin is the
bottom left, so lightmap row 0 shows at the top), bytes in B, G, R(, A) order,
each value min(v * 255 / top, 255) truncated to a byte. Values below zero
give 0 here; the reference's cast of a negative float to a byte is undefined.
`normals_for_display` maps a normal/"focus" map to the harness's colours
(xyz * 0.5 + 0.5, lighter_test.cpp:456-463), written with alpha.

`write_hdr` keeps the float range: Radiance RGBE (shared exponent), flat
scanlines, "-Y h +X w" orientation (lightmap row 0 first).
"""
import struct

import numpy as np


def tga_bytes(img: np.ndarray, top: float = 1.0) -> bytes:
    """TGA file contents of an (h, w, 3) RGB or (h, w, 4) RGBA float image."""
    img = np.asarray(img, np.float32)
    if img.ndim != 3 or img.shape[2] not in (3, 4):
        raise ValueError("expected an (h, w, 3) or (h, w, 4) image")
    h, w, c = img.shape
    if not (0 < w < 65536 and 0 < h < 65536):
        raise ValueError("TGA sides are 1..65535")
    header = bytearray(18)
    header[2] = 2                       # uncompressed true-colour
    header[12:14] = struct.pack("<H", w)
    header[14:16] = struct.pack("<H", h)
    header[16] = 8 * c
    mult = np.float32(255.0 / top)
    v = np.minimum(img * mult, np.float32(255.0))
    v = np.where(v > 0, v, np.float32(0.0))          # NaN and negatives to 0
    px = v.astype(np.uint8)                           # truncation, as the reference's cast
    order = [2, 1, 0] + ([3] if c == 4 else [])
    body = px[::-1][:, :, order].tobytes()            # last row first, BGR(A)
    return bytes(header) + body


def write_tga(path: str, img: np.ndarray, top: float = 1.0) -> None:
    with open(path, "wb") as f:
        f.write(tga_bytes(img, top))


def normals_for_display(nrm: np.ndarray) -> np.ndarray:
    """(h, w, 4) normal/focus map -> colours: xyz * 0.5 + 0.5, the fourth channel kept."""
    out = np.array(nrm, np.float32, copy=True)
    out[:, :, :3] = out[:, :, :3] * np.float32(0.5) + np.float32(0.5)
    return out


def rgbe(rgb: np.ndarray) -> np.ndarray:
    """(..., 3) float -> (..., 4) uint8 shared-exponent RGBE (Ward's Radiance format)."""
    rgb = np.maximum(np.asarray(rgb, np.float64), 0.0)
    v = rgb.max(axis=-1)
    m, e = np.frexp(v)                                # v = m * 2^e, m in [0.5, 1)
    scale = np.where(v > 1e-32, m * 256.0 / np.where(v > 0, v, 1.0), 0.0)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.minimum(np.floor(rgb * scale[..., None]), 255).astype(np.uint8)
    out[..., 3] = np.where(v > 1e-32, e + 128, 0).astype(np.uint8)
    return out


def from_rgbe(px: np.ndarray) -> np.ndarray:
    """Inverse of `rgbe` (to the encoding's precision), centre of each mantissa step."""
    px = np.asarray(px)
    e = px[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(1.0, e - (128 + 8)), 0.0)
    return ((px[..., :3].astype(np.float64) + 0.5) * f[..., None]).astype(np.float32)


def hdr_bytes(rgb: np.ndarray) -> bytes:
    """Radiance .hdr file contents of an (h, w, 3) float image (flat scanlines)."""
    rgb = np.asarray(rgb, np.float32)
    if rgb.ndim != 3 or rgb.shape[2] != 3:
        raise ValueError("expected an (h, w, 3) image")
    h, w, _ = rgb.shape
    head = f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {h} +X {w}\n".encode("ascii")
    return head + rgbe(rgb).tobytes()


def write_hdr(path: str, rgb: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(hdr_bytes(rgb))


def read_hdr(data: bytes) -> np.ndarray:
    """Reads what `hdr_bytes` writes (flat scanlines, -Y h +X w)."""
    head_end = data.index(b"\n\n") + 2
    line_end = data.index(b"\n", head_end)
    parts = data[head_end:line_end].decode("ascii").split()
    if len(parts) != 4 or parts[0] != "-Y" or parts[2] != "+X":
        raise ValueError("unsupported HDR orientation")
    h, w = int(parts[1]), int(parts[3])
    px = np.frombuffer(data, np.uint8, count=4 * w * h, offset=line_end + 1).reshape(h, w, 4)
    return from_rgbe(px)


__all__ = ["tga_bytes", "write_tga", "normals_for_display", "rgbe", "from_rgbe", "hdr_bytes", "write_hdr",
           "read_hdr"]
