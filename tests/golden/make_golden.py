#!/usr/bin/env python3
"""Generate the golden fixtures from the UNMODIFIED reference (oracle/_ref).

Each fixture is the reference's own output for one seeded procedural scene,
baked single-threaded through its C API (the byte-deterministic mode:
max_num_threads = 1, srand(seed) before ltr_LightAdd). The scenes are the
ones in CASES below; their inputs are regenerated from the seeds by
lighter_gb300.scenes, so only outputs are stored:

  lm_<uid>        lightmap (h, w, 3) float32
  nrm_<uid>       normal/focus map (h, w, 4) float32, when requested
  probes          probe-sample colours (S, 3)
  counts          per-instance sample counts
  s<inst>_<arr>   per-sample arrays (pos, nrm, loc, radinfo, color) when
                  `samples` is set for the case

Run here (needs the reference sources for oracle/_ref):
    make -C oracle ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lighter_gb300 import load_library, scenes  # noqa: E402
from lighter_gb300.scene import bake  # noqa: E402


def _probes(d):
    d.probes = [(7, (5.0, 5.0, 1.0), (0.0, 0.0, 1.0)), (9, (2.0, 8.0, 3.0), (1.0, 0.0, 0.0))]
    return d


def _cfg(d, **kw):
    d.config.update(kw)
    return d


# name -> (scene factory, store per-sample arrays)
CASES = {
    "basic": (scenes.basic, True),
    "hugeoverlap": (scenes.hugeoverlap, False),
    "cornell32_rad_ao_probes": (lambda: _probes(scenes.cornell(3, lm=32, bounces=1, ao=True)), True),
    "cornell32_normals_blur": (lambda: _cfg(scenes.cornell(5, lm=32, bounces=0, ao=True), generate_normalmap_data=1,
                                            blur_size=1.5), False),
    "cornell32_ds2x": (lambda: _cfg(scenes.cornell(6, lm=32, bounces=0, ao=False), ds2x=1), False),
    "mid128": (lambda: scenes.mid(3, lm=128, n_boxes=16, n_spheres=2, bounces=0, ao_rays=8), False),
}


def result_arrays(res, samples: bool):
    out = {}
    for uid, _, _, rgb, nrm in res.lightmaps:
        out[f"lm_{uid}"] = rgb
        if nrm is not None:
            out[f"nrm_{uid}"] = nrm
    out["probes"] = res.sample_colors
    out["counts"] = np.array([len(d["loc"]) for d in res.debug], np.int64)
    if samples:   # the per-sample arrays the reference harness exports (not the per-ray records)
        for i, d in enumerate(res.debug):
            for k in ("pos", "nrm", "loc", "radinfo", "color"):
                out[f"s{i}_{k}"] = d[k]
    return out


def main():
    ref = load_library(os.path.join(ROOT, "oracle", "_ref", "liblighter_ref.so"))
    for name, (factory, samples) in CASES.items():
        res = bake(ref, factory(), threads=1)
        arrs = result_arrays(res, samples)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrs)
        print(f"{name}: {len(res.lightmaps)} lightmaps -> {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
