#!/usr/bin/env python3
"""Benchmark of the GB300 lightmap bake on the mid-size seeded scene.

One step = one complete bake (ltr_Start .. finished) of the mid scene:
200x200 m ground, 400 boxes (0.5-8 m, random yaw) and 50 icospheres of 320
triangles (~21k triangles), four 1024^2 lightmaps, 8 point + 2 spot lights,
32 AO rays of radius 2 m and 2 radiosity bounces over 16k patches, FP32.

  value  rays/s with the scene resident on the device: rays counted by the
         library (shadow evaluations + AO rays + radiosity visibility rays)
         over the device time of the bake (CUDA events from the first kernel
         after the upload to the end of finalize), summed over ranks.
  e2e    the same rays over the host wall time of ltr_Start .. outputs on the
         host, i.e. through the C API with the upload and readback inside.
  roofline  the direct-light kernel (sphere-traced shadows), the dominant one:
         algorithmic bytes = BVH node visits x 64 B + triangle tests x 48 B.
  cpu_baseline  the CPU oracle port (all host threads) on a bounded sample.

--impl reference times the reference's CPU bake on the host cores instead
(the oracle port: the reference's own sources are not present where the
bench runs).
Multi-GPU runs are replicas (each rank bakes its own copy); the bake has no
exchange step, so there is no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s & s/radiosity bounce: batched FP16-F vs plain FP32 GPU @1e-3 rel err"
WORKLOAD = ("mid: 200x200 m ground + 400 boxes + 50 icospheres (320 tris), ~21k tris, 4 x 1024^2 lightmaps, "
            "8 point + 2 spot lights, AO 32 rays r=2 m, radiosity 2 bounces over 16k patches, FP32")
WORKLOAD_LARGE = ("large: fBm terrain 1024x512 quads (1.05M tris) in 16 tiles + 2000 80-tri rocks, ~1.2M tris, "
                  "16 x 2048^2 lightmaps, 1 directional + 32 point lights, AO 64 rays r=2 m, radiosity 3 bounces "
                  "over ~64k patches, FP32")
CPU_SAMPLE = ("same mid scene (geometry, lights, AO) at 256^2 lightmaps = 1/16 of the texels, "
              "radiosity off (texel-level radiosity of the reference is not runnable at this size)")
NODE_BYTES = 64
TRI_BYTES = 48


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _peaks_tensor():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


def _traffic_from_profile(name="k_direct_mid.md"):
    """dram bytes per launch of a kernel from its committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch_full:"):
                    return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    from lighter_gb300 import replicas
    return replicas.init()


def _barrier(dist):
    from lighter_gb300 import replicas
    replicas.barrier(dist)


def _oracle_bake(desc, threads, keep=False):
    """One bake of `desc` on the CPU oracle port; returns (rays, seconds, counters),
    plus the bake's result when `keep`."""
    import ctypes as C
    from lighter_gb300 import load_library
    from lighter_gb300.scene import bake
    orc = load_library(os.path.join(ROOT, "oracle", "liblighter_oracle.so"),
                       extra={"orc_GetCounters": (None, [C.c_void_p])})
    t0 = time.perf_counter()
    res = bake(orc, desc, threads=threads, debug=False)
    dt = time.perf_counter() - t0
    cnt = (C.c_ulonglong * 4)()
    orc.orc_GetCounters(C.cast(cnt, C.c_void_p))
    rays = cnt[0] + cnt[2] + cnt[3]
    if keep:
        return rays, dt, list(cnt), res
    return rays, dt, list(cnt)


def _parity(gpu_res, orc_res):
    """Per-texel agreement of two bakes of the same scene: the largest and the
    mean |gpu - oracle| over every lightmap relative to that lightmap's peak, and
    the fraction of texels off by more than 1e-3 of it (the parity tests' bars)."""
    import numpy as np
    mx = mean = 0.0
    over = tot = 0
    for a, b in zip(gpu_res.lightmaps, orc_res.lightmaps):
        la, lb = a[3], b[3]
        peak = max(float(np.abs(lb).max()), 1e-6)
        d = np.abs(la - lb)
        mx = max(mx, float(d.max()) / peak)
        mean = max(mean, float(d.mean()) / peak)
        over += int((d.max(-1) > 1e-3 * peak).sum())
        tot += d.shape[0] * d.shape[1]
    return {"max_abs_rel": mx, "mean_abs_rel": mean, "frac_over_1e-3": over / max(tot, 1),
            "lightmaps": len(gpu_res.lightmaps), "bars": {"max_abs_rel": 1e-5, "mean_abs_rel": 1e-6, "frac_over_1e-3": 0.0}}


def _profile_fields(name):
    """`measured:` key=value pairs of a committed ncu summary under profiles/ (floats)."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if line.startswith("measured:"):
                    for kv in line.split(":", 1)[1].split():
                        k, v = kv.split("=", 1)
                        out[k] = float(v)
    except OSError:
        pass
    return out


def _trace_roofline(kernel, profile, items, ms, sm_mhz, n_sm, unit_name):
    """Roofline block of a BVH trace kernel against the resource it is bound by:
    instruction issue (one warp instruction per scheduler and clock, 4 schedulers
    per SM). achieved = warp instructions per item (ncu, same scene at a quarter
    of the texels) x items / the kernel's CUDA-event time; the ncu fractions of
    the captured launch (issue slots, lanes per instruction, L1) come with it."""
    m = _profile_fields(profile)
    ipi = m.get("warp_inst_per_item")
    block = {"kernel": kernel, "bound": "issue", "unit": "warp-instructions/s", "items": items,
             "item": unit_name, "kernel_ms": ms, "source": "profiles/" + profile, "ncu": m or None}
    if ipi and ms > 0 and sm_mhz:
        ach = ipi * items / (ms / 1000.0)
        peak = 4.0 * n_sm * sm_mhz * 1e6
        block.update({"achieved": ach, "peak": peak, "frac": ach / peak,
                      "peak_source": "4 schedulers x %d SMs x the median SM clock sampled during the run" % n_sm})
    return block


def run_reference(args, world, rank, dist):
    from lighter_gb300 import scenes
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    desc = scenes.mid(seed=1, lm=args.cpu_lm, bounces=0)
    for _ in range(args.warmup):
        _oracle_bake(desc, threads)
    rays_tot, t_tot = 0, 0.0
    for _ in range(args.steps):
        r, dt, _ = _oracle_bake(desc, threads)
        rays_tot += r
        t_tot += dt
    v = rays_tot / t_tot
    line = {
        "metric": METRIC, "value": v, "unit": "rays/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * t_tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "sample": CPU_SAMPLE, "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "rays/s", "cores": threads, "kind": "port", "sample": CPU_SAMPLE},
        "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, world, rank, local, dist):
    from lighter_gb300 import library, scenes
    from lighter_gb300.ext import get_stats

    lib = library()
    if args.scene == "large":
        desc = scenes.large(seed=1, lm=args.lm)
    else:
        desc = scenes.mid(seed=1, lm=args.lm)
    gpu_opts = {"device": local, "radiosity_patches": args.patches, "radiosity_links": 1}
    # ingest once through the C API; every step is ltr_Start .. finished
    from lighter_gb300.scene import ingest
    scene, keep = ingest(lib, desc, gpu_options=gpu_opts)
    tuning = None
    try:
        if not args.no_autotune:   # launch shapes of the trace kernels, tuned on this scene
            from lighter_gb300.ext import autotune
            tuning = autotune(lib, scene)
        for _ in range(args.warmup):
            _bake_once(lib, scene)
        _barrier(dist)
        sampler = ClockSampler(local)
        sampler.start()
        stats = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            _bake_once(lib, scene)
            stats.append(get_stats(lib, scene))
        wall = time.perf_counter() - t0
        clocks = sampler.stop()
        _barrier(dist)
    finally:
        lib.ltr_DestroyScene(scene)
        del keep
    rays = sum(s["shadow_evals"] + s["ao_rays"] + s["rad_vis_rays"] for s in stats)
    dev_ms = sum(s["ms_device"] for s in stats)
    launches = sum(s["kernel_launches"] for s in stats)
    return rays, dev_ms, wall, stats, clocks, stats[-1]["bytes_h2d"], stats[-1]["bytes_d2h"], launches, tuning


# algorithmic bytes per lightmap texel of the finalize stage: scatter 13, three dilations x 26, two blur passes x 24
TEXEL_STAGE_BYTES = 13 + 3 * 26 + 2 * 24

# bake radiosity precisions: (name, LTRG_F_*, refine_steps)
RAD_MODES = (("fp32", 0, 0), ("fp16", 1, 0), ("fp16_refine1", 1, 1), ("bf16", 2, 0), ("bf16_refine1", 2, 1))


def run_rad_precisions(args, lib, desc, gpu_opts, bounces):
    """One bake of the scene per form-factor precision (after one warm-up bake):
    seconds per radiosity bounce and the largest lightmap difference from the FP32
    bake, relative to each lightmap's peak."""
    import numpy as np
    from lighter_gb300.ext import get_stats
    from lighter_gb300.scene import _collect, ingest
    out, base = {}, None
    for name, prec, refine in RAD_MODES:
        scene, keep = ingest(lib, desc, gpu_options=dict(gpu_opts, radiosity_precision=prec, refine_steps=refine))
        try:
            _bake_once(lib, scene)
            _bake_once(lib, scene)
            st = get_stats(lib, scene)
            lms = [x[3] for x in _collect(lib, scene, False, [], 0.0, "finished").lightmaps]
        finally:
            lib.ltr_DestroyScene(scene)
            del keep
        if base is None:
            base = lms
        err = max(float(np.abs(a - b).max()) / max(float(np.abs(b).max()), 1e-12) for a, b in zip(lms, base))
        n = st["rad_elements"]
        f_bytes = n * ((n + 7) // 8 * 8) * (4 if prec == 0 else 2)   # F rows padded to 8 entries
        spb = st["ms_rad_bounce"] / bounces / 1000.0
        out[name] = {"s_per_bounce": spb, "ms_rad_links": st["ms_rad_links"], "max_rel_err_vs_fp32": err,
                     "elements": n, "f_bytes": f_bytes, "f_gbs": f_bytes / spb / 1e9 if spb > 0 else 0.0}
    return out


GATHER_WORKLOAD = ("multi-RHS radiosity: seeded room with furniture, {n} patches, {t} triangles, "
                   "{c} light configurations (R = {r} RGB right-hand sides), {b} bounces")
# (name, precision, refine, TMEM accumulation length in k blocks)
GATHER_MODES = [("fp32", 0, 0, 0), ("fp16", 1, 0, 0), ("fp16_rhs", 1, 1, 0), ("bf16_rhs", 2, 1, 0),
                ("fp16_full", 1, 2, 0), ("bf16_full", 2, 2, 0), ("fp16_full_chunk64", 1, 2, 64)]


def run_gather(args, local):
    """Form factors once, then timed solves of every precision mode on device-resident
    inputs; errors against an FP64 Jacobi (torch float64 on the device over the FP32
    form factors) for the first 8 configurations."""
    import numpy as np
    import torch

    from lighter_gb300 import library, patches
    from lighter_gb300.gather import Gather

    lib = library()
    sc = patches.room(seed=1, n_patches=args.gather_patches, n_configs=args.gather_configs)
    n, R, bounces = len(sc["pos"]), sc["emission"].shape[1], args.gather_bounces
    dev = torch.device("cuda", local)
    out = {"workload": GATHER_WORKLOAD.format(n=n, t=len(sc["tri"]), c=args.gather_configs, r=R, b=bounces)}
    with Gather(lib, sc["tri"], sc["pos"], sc["nrm"], sc["area"], device=local) as g:
        alb = torch.from_numpy(sc["albedo"]).to(dev)
        E = torch.from_numpy(sc["emission"]).to(dev)
        B = torch.empty((n, R), dtype=torch.float32, device=dev)
        # FP64 reference for the first 8 configurations
        ncheck = min(R, 24)
        Gd = torch.from_numpy(g.G()).to(dev)
        albc = alb[:, torch.arange(ncheck, device=dev) % 3].double()
        E64 = E[:, :ncheck].double()
        B64 = E64.clone()
        for _ in range(bounces):
            X = albc * B64
            Y = torch.empty_like(B64)
            for r0 in range(0, n, 4096):
                Y[r0:r0 + 4096] = Gd[r0:r0 + 4096].double() @ X
            B64 = E64 + Y
        # library reference point for plain FP32 on the GPU: cuBLAS SGEMM (TF32 off) of one bounce
        tf32 = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        X32 = alb[:, torch.arange(R, device=dev) % 3] * E
        for _ in range(2):
            Yc = torch.mm(Gd, X32)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(3):
            Yc = E + torch.mm(Gd, X32)
        ev[1].record()
        torch.cuda.synchronize()
        cublas_s = ev[0].elapsed_time(ev[1]) / 3 / 1000.0
        torch.backends.cuda.matmul.allow_tf32 = tf32
        del Gd, X32, Yc
        torch.cuda.empty_cache()
        modes = {}
        for name, prec, refine, chunk in GATHER_MODES:
            g.set_chunk(chunk)
            st = g.solve_device(alb.data_ptr(), E.data_ptr(), R, bounces, B.data_ptr(), prec, refine)   # warm-up
            conv = st["ms_convert"]
            per = []
            for _ in range(args.gather_steps):
                st = g.solve_device(alb.data_ptr(), E.data_ptr(), R, bounces, B.data_ptr(), prec, refine)
                per.append(st)
            d = B[:, :ncheck].double() - B64
            fro = float(torch.linalg.norm(d) / torch.linalg.norm(B64))
            mx = float((d.abs() / B64.abs().amax(dim=0, keepdim=True).clamp_min(1e-30)).max())
            spb = statistics.median(p["ms_per_bounce"] for p in per) / 1000.0
            gemm = statistics.median(p["ms_gemm"] for p in per) / 1000.0 / max(1, bounces)
            modes[name] = {
                "s_per_bounce": spb, "gemm_s_per_bounce": gemm,
                "tflops": st["flops_per_bounce"] / gemm / 1e12 if gemm > 0 else 0.0,
                "f_gbs": st["bytes_per_bounce"] / gemm / 1e9 if gemm > 0 else 0.0,
                "bytes_per_bounce": st["bytes_per_bounce"], "products": st["products"],
                "tensor_cores": bool(st["tensor_cores"]), "stages": st["stages"], "ctas": st["ctas"],
                "convert_ms": conv, "rel_err_fro_vs_fp64": fro, "rel_err_max_vs_fp64": mx, "k_chunk": chunk,
            }
        g.set_chunk(0)
        # end to end through the host-buffer entry point (inputs and result cross the
        # CPU-GPU link), into one host output buffer the caller keeps, as an application would
        hout = np.empty((n, R), np.float32)

        def e2e_time():
            g.solve(sc["albedo"], sc["emission"], bounces, 1, 1, out=hout)
            t0 = time.perf_counter()
            for _ in range(args.gather_steps):
                g.solve(sc["albedo"], sc["emission"], bounces, 1, 1, out=hout)
            return (time.perf_counter() - t0) / args.gather_steps

        host_path = {1: "staged", 2: "direct"}
        g.host_path(1)
        e2e_staged = e2e_time()
        g.host_path(0)
        e2e = e2e_time()
        path = host_path[g.host_path()]
        dev_fp16_rhs = modes["fp16_rhs"]["s_per_bounce"] * bounces
        st0 = g.solve_device(alb.data_ptr(), E.data_ptr(), R, 0, B.data_ptr(), 1, 1)
        out.update({
            "build_ms": st0["ms_build"], "visibility_rays": st0["vis_rays"], "links": st0["links"],
            "visibility_rays_per_s": st0["vis_rays"] / (st0["ms_build"] / 1000.0),
            "modes": modes,
            "e2e_s_per_solve_fp16_rhs": e2e, "e2e_bytes": {"h2d": int(n * (R + 3) * 4), "d2h": int(n * R * 4)},
            "device_s_per_solve_fp16_rhs": dev_fp16_rhs, "e2e_over_device_fp16_rhs": e2e / dev_fp16_rhs,
            "e2e_host_path": path, "e2e_s_per_solve_fp16_rhs_staged": e2e_staged,
            "speedup_fp16_rhs_vs_fp32": modes["fp32"]["s_per_bounce"] / modes["fp16_rhs"]["s_per_bounce"],
            "speedup_fp16_vs_fp32": modes["fp32"]["s_per_bounce"] / modes["fp16"]["s_per_bounce"],
            "fp32_cublas_sgemm_s_per_bounce": cublas_s,
            "speedup_fp16_vs_cublas_fp32": cublas_s / modes["fp16"]["s_per_bounce"],
            "error_reference": "FP64 Jacobi (torch float64 on the device) over the FP32 form factors, "
                               "first %d right-hand sides" % ncheck,
        })
    return out


BATCH_WORKLOAD = ("batch: {n} seeded scenes, triangles lognormal (median 2k, 200-20k), lightmap side log-uniform "
                  "64-512, 1-8 point lights with 16-64 samples, AO 16 rays r=2 m, no radiosity")


def run_batch(args, local):
    """The batch workload baked one scene after another (ltr_Start, ltrg_Wait) and
    as one batch (ltrg_StartBatch): wall time of all scenes through the C API."""
    import ctypes as C

    from lighter_gb300 import library, scenes
    from lighter_gb300.ext import get_stats
    from lighter_gb300.scene import ingest

    lib = library()
    descs = [scenes.batch_scene(s) for s in range(1, args.batch_scenes + 1)]
    handles = [ingest(lib, d, gpu_options={"device": local}) for d in descs]
    arr = (C.c_void_p * len(handles))(*[h for h, _ in handles])
    try:
        def sequential():
            t0 = time.perf_counter()
            for h, _ in handles:
                lib.ltr_Start(h)
                if not lib.ltrg_Wait(h):
                    raise RuntimeError("bake failed: " + (lib.ltrg_LastError(h) or b"").decode())
            return time.perf_counter() - t0

        def batched():
            t0 = time.perf_counter()
            if not lib.ltrg_StartBatch(arr, len(handles)):
                raise RuntimeError("ltrg_StartBatch rejected the batch")
            for h, _ in handles:
                if not lib.ltrg_Wait(h):
                    raise RuntimeError("batch bake failed: " + (lib.ltrg_LastError(h) or b"").decode())
            return time.perf_counter() - t0

        sequential()
        t_seq = min(sequential() for _ in range(max(1, args.batch_steps)))
        batched()
        t_bat = min(batched() for _ in range(max(1, args.batch_steps)))
        st = [get_stats(lib, h) for h, _ in handles]
    finally:
        for h, _ in handles:
            lib.ltr_DestroyScene(h)
    rays = sum(x["shadow_evals"] + x["ao_rays"] for x in st)
    texels = sum(x["samples"] for x in st)
    return {
        "workload": BATCH_WORKLOAD.format(n=len(descs)),
        "sequential_s": t_seq, "batch_s": t_bat, "speedup": t_seq / t_bat,
        "rays": rays, "rays_per_s_sequential": rays / t_seq, "rays_per_s_batch": rays / t_bat,
        "texels": texels, "texels_per_s_batch": texels / t_bat,
        "triangles": sum(x["triangles"] for x in st),
        "timing": "host wall clock of all scenes through the C API, best of %d after one warm-up" % max(1, args.batch_steps),
    }


HEADLINE_WORKLOAD = ("{n} mid scenes (seeds 1..{n}, as the single-scene workload) in one ltrg_StartBatch, FP16 form "
                     "factors with per-row scales, the last of 2 bounces refined in FP32")


def run_headline(args, local, single):
    """The batched mixed-precision bake against the plain FP32 single-scene bake:
    `--headline-scenes` mid scenes baked as one batch with FP16 F (one refinement
    bounce), host wall clock through the C API, against the single FP32 bake's
    end-to-end and device figures of the same line."""
    import ctypes as C

    from lighter_gb300 import library, scenes
    from lighter_gb300.ext import get_stats
    from lighter_gb300.scene import ingest

    lib = library()
    n = args.headline_scenes
    opts = {"device": local, "radiosity_patches": args.patches, "radiosity_links": 1, "radiosity_precision": 1,
            "refine_steps": 1}
    handles = [ingest(lib, scenes.mid(seed=s, lm=args.lm), gpu_options=opts) for s in range(1, n + 1)]
    arr = (C.c_void_p * n)(*[h for h, _ in handles])
    try:
        def batched():
            t0 = time.perf_counter()
            if not lib.ltrg_StartBatch(arr, n):
                raise RuntimeError("ltrg_StartBatch rejected the batch")
            for h, _ in handles:
                if not lib.ltrg_Wait(h):
                    raise RuntimeError("batch bake failed: " + (lib.ltrg_LastError(h) or b"").decode())
            return time.perf_counter() - t0

        batched()
        times = [batched() for _ in range(max(1, args.batch_steps))]
        st = [get_stats(lib, h) for h, _ in handles]
    finally:
        for h, _ in handles:
            lib.ltr_DestroyScene(h)
    t = statistics.median(times)
    rays = sum(x["shadow_evals"] + x["ao_rays"] + x["rad_vis_rays"] for x in st)
    in_batch = statistics.median(x["ms_rad_bounce"] / 2 / 1000.0 for x in st)
    solo = (single.get("bake_radiosity_precisions") or {}).get("fp16_refine1", {}).get("s_per_bounce")
    return {
        "workload": HEADLINE_WORKLOAD.format(n=n), "wall_s": t, "rays": rays, "rays_per_s": rays / t,
        "s_per_bounce": solo,
        "s_per_bounce_note": "FP16 F with one refinement bounce, one scene baked alone (the same settings as the batch)",
        "s_per_bounce_in_batch": in_batch,
        "s_per_bounce_in_batch_note": "per-scene CUDA-event time of the bounces while the batch's other scenes' "
                                      "trace kernels hold the GPU (waiting included)",
        "plain_fp32_single_scene": {"rays_per_s_e2e": single["e2e"]["value"], "rays_per_s_device": single["value"],
                                    "s_per_bounce": single["s_per_bounce"]},
        "rays_per_s_vs_plain_e2e": rays / t / single["e2e"]["value"],
        "timing": "host wall clock, median of %d batches after one warm-up" % len(times),
    }


SAMPLED_WORKLOAD = ("mid scene as the headline workload (seed 1) with sampled soft shadows: shadow_sample_count = 64 "
                    "visibility rays per (sample, light) pair on a disk of radius 0.2 m around each point and spot light; "
                    "one shadow ray counted per (texel, light, sample)")


def run_sampled(args, local):
    """The headline scene with LTRG_SHADOW_SAMPLED: the configured 64 shadow rays per
    (sample, light) pair. One warm-up bake, then the median of three timed bakes:
    shadow rays/s over the shadow-trace kernel's CUDA-event time."""
    from lighter_gb300 import library, scenes
    from lighter_gb300.ext import get_stats
    from lighter_gb300.scene import ingest
    lib = library()
    desc = scenes.large(seed=1, lm=args.lm) if args.scene == "large" else scenes.mid(seed=1, lm=args.lm)
    scene, keep = ingest(lib, desc, gpu_options={"device": local, "radiosity_patches": args.patches,
                                                 "radiosity_links": 1, "shadow_mode": 1})
    try:
        _bake_once(lib, scene)
        st = []
        for _ in range(3):
            _bake_once(lib, scene)
            st.append(get_stats(lib, scene))
    finally:
        lib.ltr_DestroyScene(scene)
        del keep
    st.sort(key=lambda x: x["ms_direct_trace"])
    m = st[1]
    rays = m["shadow_evals"]
    return {"workload": SAMPLED_WORKLOAD, "shadow_rays": rays, "shadow_pairs": m["shadow_pairs"],
            "kernel_ms": m["ms_direct_trace"], "stage_ms": m["ms_direct"],
            "shadow_rays_per_s": rays / (m["ms_direct_trace"] / 1000.0) if m["ms_direct_trace"] > 0 else None,
            "bake_device_ms": m["ms_device"],
            "rays_per_s_device": (rays + m["ao_rays"] + m["rad_vis_rays"]) / (m["ms_device"] / 1000.0)}


LARGE_WORKLOAD = ("large (C3): fBm terrain 1024x512 quads (1.05M tris) in 16 tiles + 2000 80-tri rocks, ~1.2M tris, "
                  "16 x 2048^2 lightmaps, 1 directional + 32 point lights, AO 64 rays r=2 m, radiosity 3 bounces over "
                  "~64k patches; FP32 F, then FP16 F with the last bounce refined")


def run_large(args, local):
    """The large terrain scene: one warm-up bake and one timed bake with FP32 form
    factors, then the same with FP16 F (last of 3 bounces refined in FP32): device and
    wall times, rays/s, s per bounce and the FP16 bake's largest lightmap
    difference from the FP32 one (relative to each lightmap's peak)."""
    import numpy as np
    from lighter_gb300 import library, scenes
    from lighter_gb300.ext import get_stats
    from lighter_gb300.scene import _collect, ingest
    lib = library()
    desc = scenes.large(seed=1, lm=2048)
    out = {"workload": LARGE_WORKLOAD}
    base = None
    for name, prec, refine in (("fp32", 0, 0), ("fp16_refine1", 1, 1)):
        scene, keep = ingest(lib, desc, gpu_options={"device": local, "radiosity_patches": 65536, "radiosity_links": 1,
                                                     "radiosity_precision": prec, "refine_steps": refine})
        try:
            # a warm-up bake for both, so both timed bakes are the second after ingest and
            # draw the same AO offsets from the caller's rand() sequence
            _bake_once(lib, scene)
            t0 = time.perf_counter()
            _bake_once(lib, scene)
            wall = time.perf_counter() - t0
            st = get_stats(lib, scene)
            lms = [x[3] for x in _collect(lib, scene, False, [], 0.0, "finished").lightmaps]
        finally:
            lib.ltr_DestroyScene(scene)
            del keep
        rays = st["shadow_evals"] + st["ao_rays"] + st["rad_vis_rays"]
        rec = {"device_ms": st["ms_device"], "wall_ms": wall * 1000.0, "rays": rays,
               "rays_per_s_device": rays / (st["ms_device"] / 1000.0), "rays_per_s_e2e": rays / wall,
               "s_per_bounce": st["ms_rad_bounce"] / 3 / 1000.0, "patches": st["rad_elements"],
               "ms_direct_trace": st["ms_direct_trace"], "ms_ao_trace": st["ms_ao_trace"],
               "shadow_pairs": st["shadow_pairs"], "ao_rays": st["ao_rays"], "triangles": st["triangles"]}
        if base is None:
            base = lms
        else:
            rec["max_rel_err_vs_fp32"] = max(float(np.abs(a - b).max()) / max(float(np.abs(b).max()), 1e-12)
                                             for a, b in zip(lms, base))
        out[name] = rec
    return out


def _bake_once(lib, scene):
    lib.ltr_Start(scene)
    if not lib.ltrg_Wait(scene):
        msg = lib.ltrg_LastError(scene)
        raise RuntimeError("bake failed: " + (msg.decode() if msg else "unknown"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scene", choices=["mid", "large"], default="mid",
                    help="mid: the headline workload; large: 1.2M-triangle terrain, 16 x 2048^2 lightmaps")
    ap.add_argument("--lm", type=int, default=None, help="lightmap side (default 1024 mid, 2048 large)")
    ap.add_argument("--patches", type=int, default=16384)
    ap.add_argument("--cpu-lm", type=int, default=256, help="lightmap side of the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--gather-patches", type=int, default=32768)
    ap.add_argument("--gather-configs", type=int, default=64)
    ap.add_argument("--gather-bounces", type=int, default=4)
    ap.add_argument("--gather-steps", type=int, default=3)
    ap.add_argument("--no-gather", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-sampled", action="store_true", help="skip the sampled soft-shadow bake")
    ap.add_argument("--no-large", action="store_true", help="skip the large terrain scene's bakes")
    ap.add_argument("--headline-scenes", type=int, default=4)
    ap.add_argument("--no-headline", action="store_true",
                    help="skip the batched FP16 mid-scene bake compared with the plain FP32 one")
    ap.add_argument("--no-rad-precisions", action="store_true",
                    help="skip the per-precision bakes (FP32 / FP16 / BF16 form factors, with and without refinement)")
    ap.add_argument("--no-bake", action="store_true",
                    help="gather only (profiling of the gather kernels on a smaller patch set)")
    args = ap.parse_args()
    if args.lm is None:
        args.lm = 2048 if args.scene == "large" else 1024
    if args.scene == "large" and args.patches == 16384:
        args.patches = 65536
    world, rank, local, dist = _dist()
    if args.impl == "reference":
        return run_reference(args, world, rank, dist)
    if args.no_bake:
        if rank == 0:
            print(json.dumps({"gather": run_gather(args, local)}), flush=True)
        return 0

    rays, dev_ms, wall, stats, clocks, h2d, d2h, launches, tuning = run_ours(args, world, rank, local, dist)
    from lighter_gb300 import replicas
    rays_all, dev_ms_max, wall_max = replicas.aggregate(dist, rays, dev_ms, wall)
    if rank != 0:
        return 0

    s0 = stats[-1]
    peak, peak_kind = _peaks()
    # node and leaf fetches of the shadow kernel's walks (a walk a warp shares counts once)
    direct_bytes = s0["node_visits"] * NODE_BYTES + s0["tri_tests"] * TRI_BYTES
    kms = s0["ms_direct_trace"] if s0["ms_direct_trace"] > 0 else s0["ms_direct"]
    achieved = direct_bytes / (kms / 1000.0) / 1e9 if kms > 0 else 0.0
    bounces = 3 if args.scene == "large" else 2
    line = {
        "metric": METRIC,
        "value": rays_all / (dev_ms_max / 1000.0),
        "unit": "rays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded procedural scene, seed 1)",
        "config": {
            "workload": WORKLOAD if args.scene == "mid" else WORKLOAD_LARGE,
            "lightmap": args.lm,
            "radiosity_patches": args.patches,
            "radiosity_links": "visible pairs (patch mode)",
            "l2": "inputs larger than L2: per-bake sample buffers of %.0f MB, scene re-uploaded every step"
                  % (s0["samples"] * 84 / 1e6),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "trace_launch_shapes": tuning or "defaults (autotuner off)",
        },
        "e2e": {"value": rays_all / wall_max, "unit": "rays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_direct_trace (sphere-traced shadows)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": _traffic_from_profile("k_direct_trace_mid512.md"),
                     "algorithmic_bytes_per_launch": direct_bytes,
                     "note": "bytes of the BVH nodes (64 B) and leaf records (48 B) the walks fetch, per warp for "
                             "shared walks; the kernel is bound by instruction issue, not by these bytes "
                             "(trace_rooflines.shadow)"},
        "clocks": clocks,
        "s_per_bounce": s0["ms_rad_bounce"] / bounces / 1000.0,
        "texels_per_s": s0["samples"] / (s0["ms_device"] / 1000.0),
        # the texel stage (scatter, three dilations, two blur passes) over every lightmap texel:
        # scatter 13 B (colour + mask written), a dilation 26 B (colour + mask read and written),
        # a blur pass 24 B (colour read and written) per texel
        "texel_roofline": {
            "bound": "hbm", "kernels": "k_scatter, 3 x k_dilate, 2 x k_conv_t (finalize stage)",
            "bytes_per_texel": TEXEL_STAGE_BYTES, "texels": s0["texels"],
            "achieved": s0["texels"] * TEXEL_STAGE_BYTES / (s0["ms_finalize"] / 1000.0) / 1e9 if s0["ms_finalize"] > 0 else 0.0,
            "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
            "frac": (s0["texels"] * TEXEL_STAGE_BYTES / (s0["ms_finalize"] / 1000.0) / 1e9 / peak) if s0["ms_finalize"] > 0 else 0.0,
        },
        "rays_per_step": {"shadow": s0["shadow_evals"], "ao": s0["ao_rays"], "radiosity_visibility": s0["rad_vis_rays"]},
        # the two trace kernels apart: 97% of the rays above are short AO rays, while the
        # sphere-traced shadow pairs take the larger share of the device time
        "shadow_pairs_per_s": s0["shadow_pairs"] / (s0["ms_direct_trace"] / 1000.0) if s0["ms_direct_trace"] > 0 else None,
        "ao_rays_per_s": s0["ao_rays"] / (s0["ms_ao_trace"] / 1000.0) if s0["ms_ao_trace"] > 0 else None,
        "trace_kernels_ms": {"k_direct_trace": s0["ms_direct_trace"], "k_ao_rays": s0["ms_ao_trace"]},
        "distance_queries_per_s": s0["distance_queries"] / (s0["ms_device"] / 1000.0),
        "stages_ms": {k: round(s0[k], 3) for k in ("ms_upload", "ms_bvh", "ms_samples", "ms_direct", "ms_rad_links",
                                                    "ms_rad_bounce", "ms_ao", "ms_finalize", "ms_download",
                                                    "ms_device", "ms_total")},
    }
    try:
        import torch
        n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    except Exception:
        n_sm = 152
    line["trace_rooflines"] = {
        "shadow": _trace_roofline("k_direct_trace", "k_direct_trace_mid512.md", s0["shadow_pairs"],
                                  s0["ms_direct_trace"], clocks.get("sm_mhz"), n_sm, "(sample, light) pair"),
        "ao": _trace_roofline("k_ao_rays", "k_ao_rays_mid512.md", s0["ao_rays"], s0["ms_ao_trace"],
                              clocks.get("sm_mhz"), n_sm, "AO ray"),
    }
    # the resource that binds the dominant kernel, beside its HBM figure
    sh = line["trace_rooflines"]["shadow"]
    if sh and sh.get("frac") is not None:
        line["roofline"]["binding_resource"] = "instruction issue (trace_rooflines.shadow)"
        line["roofline"]["binding_frac"] = sh["frac"]
    if not args.no_sampled:
        line["sampled_shadows"] = run_sampled(args, local)
        ss = line["sampled_shadows"]
        ss["roofline"] = _trace_roofline("k_direct_trace (sampled shadows)", "k_direct_trace_sampled_mid512.md",
                                         ss["shadow_rays"], ss["kernel_ms"], clocks.get("sm_mhz"), n_sm, "shadow ray")
    if not args.no_large and args.scene == "mid":
        line["large_scene"] = run_large(args, local)
    if not args.no_rad_precisions:
        from lighter_gb300 import library, scenes
        desc = scenes.large(seed=1, lm=args.lm) if args.scene == "large" else scenes.mid(seed=1, lm=args.lm)
        line["bake_radiosity_precisions"] = run_rad_precisions(
            args, library(), desc, {"device": local, "radiosity_patches": args.patches, "radiosity_links": 1}, bounces)
    if not args.no_headline and args.scene == "mid":
        line["batched_fp16_vs_plain_fp32"] = run_headline(args, local, line)
    if not args.no_batch:
        line["batch"] = run_batch(args, 0)
    if not args.no_gather:
        gat = run_gather(args, 0)
        line["gather"] = gat
        peak_tf = _peaks_tensor()
        gm = gat["modes"]
        m, mf = gm["fp16"], gm["fp16_full"]
        line["s_per_bounce"] = {"gather_fp16": m["s_per_bounce"], "gather_fp16_full": mf["s_per_bounce"],
                                "gather_fp32": gm["fp32"]["s_per_bounce"],
                                "gather_fp32_cublas_sgemm": gat["fp32_cublas_sgemm_s_per_bounce"],
                                "bake_mid_fp32": line["s_per_bounce"]}
        line["gather_roofline"] = {
            "kernel": "k_umma_gather (tcgen05, FP16 G, one product)", "bound": "hbm",
            "achieved": m["f_gbs"], "peak": peak, "unit": "GB/s", "frac": m["f_gbs"] / peak, "peak_source": peak_kind,
            "traffic": _traffic_from_profile("k_umma_gather_c5.md"),
            "algorithmic_bytes_per_launch": m["bytes_per_bounce"]}
        line["gather_roofline_tensor"] = {
            "kernel": "k_umma_gather (tcgen05, FP16 G + residual, split right-hand side: 3 products)",
            "bound": "tensor", "achieved": mf["tflops"], "peak": peak_tf, "unit": "TFLOP/s",
            "frac": mf["tflops"] / peak_tf, "peak_source": "measured bf16 dense burst (MEASURED_PEAKS.json)"}
    if args.scene == "large" and not args.no_cpu_baseline:
        line["cpu_baseline"] = None
        line["cpu_baseline_note"] = ("not run for the 1.2M-triangle scene: the reference's per-instance BSP "
                                     "(PickSplitPlane, O(points^2) per node) makes its sample stage impractical")
    elif not args.no_cpu_baseline:
        from lighter_gb300 import library, scenes
        from lighter_gb300.scene import bake
        threads = os.cpu_count() or 1
        desc = scenes.mid(seed=1, lm=args.cpu_lm, bounces=0)
        r, dt, cnt, ores = _oracle_bake(desc, threads, keep=True)
        line["cpu_baseline"] = {"value": r / dt, "unit": "rays/s", "cores": threads, "kind": "port",
                                "sample": CPU_SAMPLE, "seconds": dt}
        # the GPU's bake of the same sample against the oracle's output just made
        gres = bake(library(), desc, debug=False, gpu_options={"device": local})
        line["parity"] = dict(_parity(gres, ores), sample=CPU_SAMPLE, against="the oracle port's bake of the "
                              "cpu_baseline leg (the reference's algorithm restated, pinned to the reference's outputs)")
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
