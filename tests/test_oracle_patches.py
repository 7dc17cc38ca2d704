"""The oracle's patch-mode radiosity (CPU restatement of the GPU library's
radiosity_patches mode) checked for self-consistency on the CPU: patch count
near the target, patch areas summing to the sample areas, and totals that
satisfy the bounce recurrence in FP64 over the exported link factors."""
import os

import numpy as np

from lighter_gb300 import load_library, scenes
from lighter_gb300.scene import bake

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_patch_radiosity_is_consistent(built):
    orc = load_library(os.path.join(ROOT, "oracle", "liblighter_oracle.so"))
    d = scenes.cornell(2, lm=32, bounces=2, ao=False)
    r = bake(orc, d, threads=os.cpu_count() or 1, gpu_options={"radiosity_patches": 256, "radiosity_links": 1},
             radiosity=True)
    rad = r.radiosity
    n = rad["n"]
    assert 128 <= n <= 512
    area = sum(float(x["radinfo"][:, 3].astype(np.float64).sum()) for x in r.debug[1:])
    assert abs(float(rad["diff_area"][:, 3].astype(np.float64).sum()) - area) <= 1e-5 * area
    np.testing.assert_allclose(np.linalg.norm(rad["nrm"][:, :3], axis=1), 1.0, rtol=1e-5)
    # totals = sum_{m<=2} K^m E, K_ij = F_ij area_j diffuse_j, per colour channel, in FP64
    F = rad["F"].astype(np.float64)
    assert (F == F.T).all() and (F != 0).sum() > 0
    K = F * (rad["diff_area"][:, 3].astype(np.float64))[None, :]
    E = rad["emit"][:, :3].astype(np.float64)
    B, X = E.copy(), E.copy()
    for _ in range(2):
        X = (K[None, :, :] * rad["diff_area"][:, :3].T.astype(np.float64)[:, None, :] @ X.T[:, :, None])[..., 0].T
        B += X
    err = float(np.abs(B - rad["total"][:, :3]).max()) / float(np.abs(B).max())
    assert err <= 1e-5, err


def test_oracle_patch_mode_off_is_reference(built):
    """radiosity_patches = 0 leaves the oracle's reference-mode bake untouched."""
    orc = load_library(os.path.join(ROOT, "oracle", "liblighter_oracle.so"))
    d = scenes.cornell(3, lm=16, bounces=1, ao=False)
    a = bake(orc, d)
    b = bake(orc, d, gpu_options={"radiosity_patches": 0, "radiosity_links": 0})
    for x, y in zip(a.lightmaps, b.lightmaps):
        np.testing.assert_array_equal(x[3], y[3])
