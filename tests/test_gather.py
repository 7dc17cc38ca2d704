"""Multi-right-hand-side radiosity gather (ltrg_Gather*) against the oracle.

The oracle is the FP64 Jacobi iteration of the reference's bounce
(oracle/radiosity_fp64.cpp) with the visibility bits of the FP32 pass, and
the reference-semantics form factors (orc_gather_form_factors: pair test and
VisibilityTest through the reference-shaped triangle tree).

Error measure: rel = ||B - B64||_F / ||B64||_F over all n x R entries, and
the largest per-entry error relative to the entry's column peak. Bars
(written next to each case): FP32 and LTRG_REFINE_FULL at FP32 level;
FP16 with the split right-hand side <= 1e-4; plain 16-bit products <= 1e-3.
"""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

from lighter_gb300 import ext, patches
from lighter_gb300.gather import BF16, FP16, FP32, REFINE_FULL, REFINE_NONE, REFINE_RHS, Gather

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
THREADS = max(1, min(16, os.cpu_count() or 1))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def oracle_G(oracle, sc, links=ext.LTRG_LINKS_VISIBLE):
    n = len(sc["pos"])
    G = np.empty((n, n), np.float32)
    oracle.orc_gather_form_factors.restype = None
    oracle.orc_gather_form_factors(_p(sc["tri"]), C.c_uint32(len(sc["tri"])), _p(sc["pos"]), _p(sc["nrm"]),
                                   _p(sc["area"]), C.c_uint32(n), C.c_int(links), _p(G), C.c_int(THREADS))
    return G


def oracle_B(oracle, sc, G_mask, E, bounces):
    n, R = E.shape
    out = np.empty((n, R), np.float64)
    oracle.orc_gather_jacobi_f64.restype = None
    E = np.ascontiguousarray(E, np.float32)
    oracle.orc_gather_jacobi_f64(C.c_uint32(n), C.c_uint32(R), _p(sc["pos"]), _p(sc["nrm"]), _p(sc["area"]),
                                 _p(np.ascontiguousarray(G_mask, np.float32)), _p(sc["albedo"]), _p(E),
                                 C.c_int(bounces), _p(out), C.c_int(THREADS))
    return out


def rel_err(B, B64):
    d = B.astype(np.float64) - B64
    fro = float(np.linalg.norm(d) / max(np.linalg.norm(B64), 1e-300))
    peak = np.maximum(np.abs(B64).max(axis=0, keepdims=True), 1e-30)
    return fro, float((np.abs(d) / peak).max())


# ----------------------------------------------------------------------------- CPU: the oracle itself

def _jacobi_numpy(pos, nrm, area, mask, albedo, E, bounces):
    P = pos.astype(np.float64)
    N = nrm.astype(np.float64)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    d = P[None, :, :] - P[:, None, :]            # d[i, j] = P_j - P_i
    dA = np.einsum("ik,ijk->ij", N, d)
    dB = -np.einsum("jk,ijk->ij", N, d)
    l2 = (d ** 2).sum(-1)
    np.fill_diagonal(l2, 1.0)
    G = np.where(mask != 0, dA * dB / (l2 * l2 * np.pi) * area[None, :].astype(np.float64), 0.0)
    R = E.shape[1]
    alb = albedo.astype(np.float64)[:, np.arange(R) % 3]
    B = E.astype(np.float64)
    for _ in range(bounces):
        B = E + G @ (alb * B)
    return B


def test_jacobi_oracle_matches_numpy(oracle):
    sc = patches.room(seed=3, n_patches=300, n_configs=4)
    G = oracle_G(oracle, sc)
    assert (G != 0).mean() > 0.05
    E = sc["emission"]
    got = oracle_B(oracle, sc, G, E, 3)
    want = _jacobi_numpy(sc["pos"], sc["nrm"], sc["area"], G, sc["albedo"], E, 3)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def _seg_tri_np(L1, L2, T):
    """Vectorised lighter_math.cpp:315-354 in float32 (reference operation order)."""
    f = np.float32
    P1, P2, P3 = T[:, 0:3], T[:, 3:6], T[:, 6:9]
    u, v = P2 - P1, P3 - P1

    def dot(a, b):
        return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]

    n = np.stack([u[:, 1] * v[:, 2] - u[:, 2] * v[:, 1], u[:, 2] * v[:, 0] - u[:, 0] * v[:, 2],
                  u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0]], 1)
    ok = ~np.all(np.abs(n) < f(0.001), axis=1)
    dirv = (L2 - L1)[None, :]
    w0 = L1[None, :] - P1
    a = -dot(n, w0)
    b = dot(n, np.broadcast_to(dirv, n.shape))
    with np.errstate(divide="ignore", invalid="ignore"):
        ok &= np.abs(b) >= f(0.001)
        r = a / b
        ok &= (r >= 0) & (r <= 1)
        I = L1[None, :] + r[:, None] * dirv
        uu, uv, vv = dot(u, u), dot(u, v), dot(v, v)
        w = I - P1
        wu, wv = dot(w, u), dot(w, v)
        D = uv * uv - uu * vv
        s = (uv * wv - vv * wu) / D
        ok &= (s >= 0) & (s <= 1)
        t = (uv * wu - uu * wv) / D
        ok &= (t >= 0) & ((s + t) <= 1)
    return bool(np.any(ok & (r < 1)))


def test_form_factor_oracle_matches_brute_force(oracle):
    sc = patches.room(seed=5, n_patches=120, n_configs=1)
    G = oracle_G(oracle, sc)
    pos, area = sc["pos"], sc["area"]
    nrm = sc["nrm"] / np.linalg.norm(sc["nrm"], axis=1, keepdims=True)
    tri = sc["tri"]
    f32 = np.float32
    agree, total = 0, 0
    for i in range(len(pos)):
        for j in range(i + 1, len(pos)):
            pd = pos[j] - pos[i]
            dA = nrm[i][0] * pd[0] + nrm[i][1] * pd[1] + nrm[i][2] * pd[2]
            dB = nrm[j][0] * -pd[0] + nrm[j][1] * -pd[1] + nrm[j][2] * -pd[2]
            if dA <= f32(0.001) or dB <= f32(0.001):
                assert G[i, j] == 0 and G[j, i] == 0
                continue
            l2 = pd[0] * pd[0] + pd[1] * pd[1] + pd[2] * pd[2]
            fval = f32(dA * dB) / (l2 * l2 * f32(np.pi))
            if fval < f32(0.001):
                assert G[i, j] == 0
                continue
            dn = pd / np.sqrt(l2)
            occ = _seg_tri_np(pos[i] + dn * f32(0.001), pos[j] - dn * f32(0.001), tri)
            total += 1
            want = 0.0 if occ else fval * area[j]
            if (G[i, j] != 0) == (want != 0):
                agree += 1
                if want:
                    assert abs(G[i, j] - want) <= 2e-5 * want   # normalisation rounding differs by ulps
    assert total > 100
    assert agree >= 0.99 * total


def test_gather_stats_layout_matches_header():
    probe = r"""
#include <stddef.h>
#include <stdio.h>
#include "lighter_gb300.h"
int main() {
  printf("%zu %zu %zu %zu %zu\n", sizeof(ltrg_GatherStats), offsetof(ltrg_GatherStats, bytes_per_bounce),
         offsetof(ltrg_GatherStats, links), offsetof(ltrg_GatherStats, tensor_cores),
         offsetof(ltrg_GatherStats, reserved));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "p.cpp"), os.path.join(d, "p")
        open(src, "w").write(probe)
        subprocess.run(["g++", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True, capture_output=True)
        vals = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    S = ext.GatherStats
    assert vals == [C.sizeof(S), S.bytes_per_bounce.offset, S.links.offset, S.tensor_cores.offset, S.reserved.offset]


# ----------------------------------------------------------------------------- GPU

@pytest.fixture(scope="module")
def small(gpu):
    sc = patches.room(seed=7, n_patches=1500, n_configs=8)
    g = Gather(gpu, sc["tri"], sc["pos"], sc["nrm"], sc["area"])
    yield sc, g
    g.close()


@pytest.mark.gpu
def test_form_factors_match_oracle(small, oracle):
    sc, g = small
    G = g.G()
    Go = oracle_G(oracle, sc)
    mg, mo = G != 0, Go != 0
    n = len(G)
    flips = int((mg != mo).sum())
    # visibility flips only at grazing configurations (box-boundary rounding of the reference tree)
    assert flips <= 1e-3 * max(1, int(mo.sum())), f"{flips} of {int(mo.sum())} links differ"
    both = mg & mo
    np.testing.assert_array_equal(G[both], Go[both])
    assert np.isfinite(G).all()
    assert n == g.n


@pytest.mark.gpu
@pytest.mark.parametrize("precision,refine,fro_tol,max_tol", [
    (FP32, REFINE_NONE, 2e-6, 2e-5),
    (FP16, REFINE_NONE, 1e-3, 4e-3),
    (FP16, REFINE_RHS, 1e-4, 1e-3),
    (FP16, REFINE_FULL, 2e-6, 2e-5),
    (BF16, REFINE_NONE, 4e-3, 2e-2),
    (BF16, REFINE_RHS, 1e-3, 1e-2),
    (BF16, REFINE_FULL, 2e-6, 2e-5),
])
def test_solve_vs_fp64_oracle(small, oracle, precision, refine, fro_tol, max_tol):
    sc, g = small
    G = g.G()
    E = sc["emission"]
    B64 = oracle_B(oracle, sc, G, E, 4)
    B, st = g.solve(sc["albedo"], E, 4, precision, refine)
    fro, mx = rel_err(B, B64)
    assert fro <= fro_tol and mx <= max_tol, (precision, refine, fro, mx)
    assert st["tensor_cores"] == (precision != FP32)
    assert st["ms_per_bounce"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("n,R,bounces", [(1000, 3, 1), (777, 48, 2), (2049, 192, 3), (300, 256, 2)])
def test_ragged_sizes(gpu, oracle, n, R, bounces):
    sc = patches.room(seed=11, n_patches=n, n_configs=(R + 2) // 3)
    E = np.ascontiguousarray(sc["emission"][:, :R])
    with Gather(gpu, sc["tri"], sc["pos"], sc["nrm"], sc["area"]) as g:
        G = g.G()
        B64 = oracle_B(oracle, sc, G, E, bounces)
        for prec, ref, tol in [(FP32, REFINE_NONE, 2e-6), (FP16, REFINE_RHS, 1e-4), (BF16, REFINE_FULL, 2e-6)]:
            B, _ = g.solve(sc["albedo"], E, bounces, prec, ref)
            fro, _ = rel_err(B, B64)
            assert fro <= tol, (n, R, prec, ref, fro)


@pytest.mark.gpu
def test_zero_bounces_and_determinism(small):
    sc, g = small
    E = sc["emission"]
    B0, _ = g.solve(sc["albedo"], E, 0, FP16, REFINE_RHS)
    np.testing.assert_array_equal(B0, E)
    a, _ = g.solve(sc["albedo"], E, 3, FP16, REFINE_RHS)
    b, _ = g.solve(sc["albedo"], E, 3, FP16, REFINE_RHS)
    np.testing.assert_array_equal(a, b)
    c, _ = g.solve(sc["albedo"], E, 3, FP32, REFINE_NONE)
    d, _ = g.solve(sc["albedo"], E, 3, FP32, REFINE_NONE)
    np.testing.assert_array_equal(c, d)


@pytest.mark.gpu
def test_device_entry_point_matches_host(small):
    torch = pytest.importorskip("torch")
    sc, g = small
    E = sc["emission"]
    n, R = E.shape
    dev = torch.device("cuda:0")
    alb = torch.from_numpy(sc["albedo"]).to(dev)
    Ed = torch.from_numpy(E).to(dev)
    out = torch.empty((n, R), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    st = g.solve_device(alb.data_ptr(), Ed.data_ptr(), R, 2, out.data_ptr(), FP16, REFINE_RHS)
    h, _ = g.solve(sc["albedo"], E, 2, FP16, REFINE_RHS)
    np.testing.assert_array_equal(out.cpu().numpy(), h)
    assert st["ctas"] > 0 and st["stages"] >= 2


@pytest.mark.gpu
def test_host_paths_agree(small):
    """The host-buffer solve through page-locked staging and through copy
    kernels that address the caller's pageable arrays directly (where the
    device can) return the same bits, for 16-byte aligned and misaligned
    arrays; the default path is the direct one on such devices."""
    sc, g = small
    E = sc["emission"]
    n, R = E.shape
    ref, _ = g.solve(sc["albedo"], E, 2, FP16, REFINE_RHS)
    # misaligned copies: views 4 bytes into larger arrays
    alb_buf = np.zeros(n * 3 + 1, np.float32)
    alb_buf[1:] = sc["albedo"].ravel()
    E_buf = np.zeros(n * R + 1, np.float32)
    E_buf[1:] = E.ravel()
    out_buf = np.full(n * R + 1, np.nan, np.float32)
    alb_m, E_m, out_m = alb_buf[1:].reshape(n, 3), E_buf[1:].reshape(n, R), out_buf[1:].reshape(n, R)
    assert alb_m.ctypes.data % 16 and out_m.ctypes.data % 16
    direct_ok = bool(g.lib.ltrdbg_GatherHostPath(g.h, 2))
    paths = [1, 2] if direct_ok else [1]
    try:
        for mode in paths:
            assert g.host_path(mode) == mode
            a, _ = g.solve(sc["albedo"], E, 2, FP16, REFINE_RHS)
            np.testing.assert_array_equal(a, ref)
            out_m[...] = np.nan
            g.solve(alb_m, E_m, 2, FP16, REFINE_RHS, out=out_m)
            np.testing.assert_array_equal(out_m, ref)
            assert np.isnan(out_buf[0])
    finally:
        g.host_path(0)
    assert g.host_path() == (2 if direct_ok else 1)


@pytest.mark.gpu
def test_rejects_too_many_rhs(small):
    sc, g = small
    E = np.zeros((g.n, 300), np.float32)
    with pytest.raises(RuntimeError, match="at most 256"):
        g.solve(sc["albedo"], E, 1, FP16, REFINE_RHS)
    with pytest.raises(RuntimeError, match="at most 256"):
        g.solve(sc["albedo"], E, 1, BF16, REFINE_FULL)


@pytest.mark.gpu
def test_bounded_wait_expires_and_the_next_solve_succeeds(gpu):
    """A solve whose copy producer issues nothing: the tensor-core kernel's
    mbarrier waits give up after 20 ms (test limit), the error word reaches
    ltrg_GatherLastError, the kernel frees its tensor memory and returns, and
    the next solve on the same gather matches an untouched one bit for bit."""
    sc = patches.room(seed=4, n_patches=600, n_configs=2)
    with Gather(gpu, sc["tri"], sc["pos"], sc["nrm"], sc["area"]) as g:
        ref, _ = g.solve(sc["albedo"], sc["emission"], 2, FP16, REFINE_RHS)
        g.stall_next_solve(20000)
        with pytest.raises(RuntimeError, match="wait expired"):
            g.solve(sc["albedo"], sc["emission"], 1, FP16, REFINE_RHS)
        assert b"error word" in gpu.ltrg_GatherLastError(g.h)
        again, st = g.solve(sc["albedo"], sc["emission"], 2, FP16, REFINE_RHS)
        assert st["tensor_cores"] == 1 and gpu.ltrg_GatherLastError(g.h) is None
        np.testing.assert_array_equal(again, ref)
