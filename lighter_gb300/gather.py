"""Host side of the multi-right-hand-side radiosity gather (ltrg_Gather*).

The gather is the reference's bounce (Int_RDBounce, lighter.cpp:767-797)
run for many light configurations at once over dense form factors:
B_0 = E, B_k = E + K B_{k-1}, K_ij = f_ij area_j albedo_j(r mod 3).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ext

FP32, FP16, BF16 = ext.LTRG_F_FP32, ext.LTRG_F_FP16, ext.LTRG_F_BF16
REFINE_NONE, REFINE_RHS, REFINE_FULL = ext.LTRG_REFINE_NONE, ext.LTRG_REFINE_RHS, ext.LTRG_REFINE_FULL


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Gather:
    """Form factors of a patch set (built on the GPU at construction) and
    solves for many right-hand sides. Raises RuntimeError on GPU errors."""

    def __init__(self, lib, tri_xyz, pos, nrm, area, links=ext.LTRG_LINKS_VISIBLE, device=0):
        self.lib = lib
        tri = _f32(tri_xyz).reshape(-1, 9)
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        nrm = _f32(nrm, (n, 3))
        area = _f32(area, (n,))
        self.n = n
        self.h = lib.ltrg_GatherCreate(_ptr(tri), tri.shape[0], _ptr(pos), _ptr(nrm), _ptr(area), n, links, device)
        if not self.h:
            raise RuntimeError("ltrg_GatherCreate failed (see stderr)")

    def close(self):
        if self.h:
            self.lib.ltrg_GatherDestroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, what):
        msg = self.lib.ltrg_GatherLastError(self.h)
        raise RuntimeError(f"{what}: {msg.decode() if msg else 'unknown error'}")

    def set_chunk(self, k_blocks: int):
        """TMEM accumulation length in 64-wide k blocks (0: unlimited)."""
        if not self.lib.ltrg_GatherSetChunk(self.h, int(k_blocks)):
            raise RuntimeError("ltrg_GatherSetChunk failed")

    def host_path(self, mode: int | None = None) -> int:
        """ltrdbg_GatherHostPath: how solve() moves its host arrays (0 by device, 1 staged,
        2 read/written by the GPU in place); returns the path the next solve takes."""
        if mode is not None and not self.lib.ltrdbg_GatherHostPath(self.h, int(mode)):
            raise RuntimeError(f"host path {mode} is not available on this device")
        return int(self.lib.ltrdbg_GatherHostPathUsed(self.h))

    def stall_next_solve(self, wait_us: int):
        """ltrdbg_GatherStallNextSolve: the next 16-bit solve's waits expire after wait_us."""
        if not self.lib.ltrdbg_GatherStallNextSolve(self.h, int(wait_us)):
            raise RuntimeError("ltrdbg_GatherStallNextSolve rejected its argument")

    def G(self) -> np.ndarray:
        """G_ij = F_ij * area_j (FP32, n x n) as built on the device."""
        out = np.empty((self.n, self.n), np.float32)
        if not self.lib.ltrg_GatherGetG(self.h, _ptr(out)):
            raise RuntimeError("ltrg_GatherGetG failed")
        return out

    def solve(self, albedo, emission, bounces, precision=FP16, refine=REFINE_RHS, out=None):
        """B (n x R) from host arrays; returns (B, stats dict). `out` (n x R float32,
        C order) receives B when given, so a caller can reuse one host buffer."""
        albedo = _f32(albedo, (self.n, 3))
        emission = _f32(emission)
        if emission.ndim != 2 or emission.shape[0] != self.n:
            raise ValueError("emission must be n x R")
        R = emission.shape[1]
        if out is None:
            out = np.empty((self.n, R), np.float32)
        elif out.shape != (self.n, R) or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-ordered n x R float32 array")
        st = ext.GatherStats()
        if not self.lib.ltrg_GatherSolve(self.h, _ptr(albedo), _ptr(emission), R, bounces, precision, refine,
                                         _ptr(out), C.byref(st)):
            self._err("ltrg_GatherSolve")
        return out, st.as_dict()

    def solve_device(self, albedo_ptr, emission_ptr, R, bounces, out_ptr, precision=FP16, refine=REFINE_RHS,
                     stream=None):
        """Same on device pointers (ints) of the gather's device; returns stats."""
        st = ext.GatherStats()
        if not self.lib.ltrg_GatherSolveDevice(self.h, C.c_void_p(albedo_ptr), C.c_void_p(emission_ptr), R, bounces,
                                               precision, refine, C.c_void_p(out_ptr), C.byref(st),
                                               C.c_void_p(stream) if stream else None):
            self._err("ltrg_GatherSolveDevice")
        return st.as_dict()
