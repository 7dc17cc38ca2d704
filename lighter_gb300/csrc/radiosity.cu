// Dense radiosity of the bake (see radiosity.cuh).
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../../include/lighter_gb300.h"
#include "async.cuh"
#include "radiosity.cuh"

namespace lg {
namespace {

void rck(cudaError_t e, const char* what, int line)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) + " at radiosity.cu:" +
                                 std::to_string(line) + " (" + what + ")");
}
#define RCK(x) rck((x), #x, __LINE__)

template <class T> __device__ __forceinline__ T to_store(float f);
template <> __device__ __forceinline__ float to_store<float>(float f) { return f; }
template <> __device__ __forceinline__ __half to_store<__half>(float f) { return __float2half_rn(f); }
template <> __device__ __forceinline__ __nv_bfloat16 to_store<__nv_bfloat16>(float f) { return __float2bfloat16_rn(f); }

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

// Form factors in two passes, with the reference's pair test and factor
// (lighter.cpp:733-757) and its link predicate:
//  1. k_ff_pretest: every pair (i, j), i < j, of a 32 x 32 tile gets the
//     facing tests on the unnormalised offset and f = dA dB / (|d|^4 pi) >= SMALL_FLOAT;
//     F receives f (both (i, j) and (j, i), through a shared-memory transpose) or
//     0, and the pairs that passed are appended to a list.
//  2. k_ff_visibility: persistent warps take 32 listed pairs at a time and trace
//     ltr_Scene::VisibilityTest (lighter.cpp:138-147: segment shrunk by
//     SMALL_FLOAT at both ends, any occluder hit); a pair the predicate rejects
//     gets F = 0 back in both entries.
// The dense pair loop so runs at tile speed and the divergent rays run apart
// from it; F and the link count are those of one combined pass.
struct PairRef {
    u32 i, j;
};

__device__ __forceinline__ float pair_pretest(V3 AP, V3 AN, V3 BP, V3 BN)
{
    V3 pd = BP - AP;
    float dA = dot(AN, pd), dB = dot(BN, -pd);
    if (dA <= kSmall || dB <= kSmall) return 0.0f;
    float l2 = lensq(pd);
    float f = dA * dB / (l2 * l2 * 3.14159265358979323846f);
    return f < kSmall ? 0.0f : f;
}

// FP16 range. A factor grows as 1 / (pi |d|^2) for close elements, past FP16's
// largest value (65504) for elements a few millimetres apart, so an FP16 F is
// stored per row scaled by a power of two: row i holds f * 2^-e_i with e_i in
// [0, 14] chosen from the row's largest factor so that it stays below 2^15,
// and values past 65504 (rows that would need e_i > 14) saturate. With
// e_i <= 14 the smallest linked factor, SMALL_FLOAT, stays above FP16's
// smallest subnormal (0.001 * 2^-14 > 2^-24), so a factor is zero in FP16
// exactly where it is zero in FP32. The bounce multiplies each row's sum by
// 2^e_i, which is exact: rounding happens only where F is stored.
// Rows that need a scale are rare (close pairs), so k_ff_pretest stores FP16
// unscaled (saturating) and records the largest factor only of rows that hold
// one above 2^15 (k_row_scale then gives every other row e_i = 0);
// k_ff_rescale rewrites just the rows with e_i > 0, before the visibility pass.
constexpr int kF16MaxExp = 14;
constexpr float kF16Max = 65504.0f;
constexpr float kF16Big = 32768.0f;

// up[i] = 2^e_i, e_i = clamp(k - 15, 0, 14) where rowmax < 2^k (0 for rows without a big factor)
__global__ void k_row_scale(u32 n, const unsigned* __restrict__ rowmax, float* __restrict__ up)
{
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = 0;
    frexpf(__uint_as_float(rowmax[i]), &k);
    int e = min(max(k - 15, 0), kF16MaxExp);
    up[i] = __uint_as_float((u32) (127 + e) << 23);
}

template <class T> __device__ __forceinline__ T store_f(float f, const float* up, u32 row)
{
    if constexpr (std::is_same<T, __half>::value) {
        if (up) f = f / up[row];   // division by a power of two: exact
        f = fminf(f, kF16Max);
    }
    return to_store<T>(f);
}

// rowmax[i] = float bits of the largest factor of row i when it exceeds 2^15
// (f >= 0, so unsigned order is float order)
__device__ __forceinline__ void note_big(unsigned* rowmax, u32 row, float f)
{
    if (rowmax && f > kF16Big) atomicMax(&rowmax[row], __float_as_uint(f));
}

// counts[0]: pairs that passed (appended; entries past `cap` are dropped and
// the host runs the pass again with room for all of them)
template <class T>
__global__ void k_ff_pretest(u32 n, size_t ld, const float4* __restrict__ pos, const float4* __restrict__ nrm,
                             unsigned* __restrict__ rowmax, T* __restrict__ F, PairRef* __restrict__ cand,
                             unsigned long long cap, unsigned long long* counts)
{
    __shared__ float tile[32][33];
    const u32 bi = blockIdx.y, bj = blockIdx.x;
    if (bj < bi) return;
    const int tx = threadIdx.x, ty = threadIdx.y;   // a warp is one tile row ty (lanes tx)
    for (int k = 0; k < 4; ++k) {
        int r = ty + 8 * k;
        u32 i = bi * 32 + r, j = bj * 32 + tx;
        float f = 0.0f;
        if (i < j && j < n) f = pair_pretest(ld3(pos[i]), ld3(nrm[i]), ld3(pos[j]), ld3(nrm[j]));
        tile[r][tx] = f;
        const unsigned m = __ballot_sync(0xffffffffu, f != 0.0f);
        if (m) {
            unsigned long long base = 0;
            if (tx == 0) base = atomicAdd(&counts[0], (unsigned long long) __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (f != 0.0f) {
                unsigned long long at = base + __popc(m & ((1u << tx) - 1u));
                if (at < cap) cand[at] = PairRef{i, j};
            }
        }
    }
    __syncthreads();
    // columns n .. ld-1 (row padding, ld <= 32 * tiles) receive zeros
    for (int k = 0; k < 4; ++k) {
        int r = ty + 8 * k;
        if (bi == bj) {
            u32 i = bi * 32 + r, j = bj * 32 + tx;
            if (i < n && j < ld) {
                const float f = tile[r][tx] + tile[tx][r];
                note_big(rowmax, i, f);
                F[(size_t) i * ld + j] = store_f<T>(f, nullptr, i);
            }
        } else {
            u32 i = bi * 32 + r, j = bj * 32 + tx;
            if (i < n && j < ld) {
                note_big(rowmax, i, tile[r][tx]);
                F[(size_t) i * ld + j] = store_f<T>(tile[r][tx], nullptr, i);
            }
            u32 i2 = bj * 32 + r, j2 = bi * 32 + tx;
            if (i2 < n && j2 < ld) {
                note_big(rowmax, i2, tile[tx][r]);
                F[(size_t) i2 * ld + j2] = store_f<T>(tile[tx][r], nullptr, i2);
            }
        }
    }
}

// Rows with a scale (e_i > 0) written again, one warp per row: the factors of
// k_ff_pretest (lower index first) divided by 2^e_i. Runs before the visibility
// pass, which then zeroes the rejected pairs in the rescaled rows as well.
__global__ void k_ff_rescale(u32 n, size_t ld, const float4* __restrict__ pos, const float4* __restrict__ nrm,
                             const float* __restrict__ up, __half* __restrict__ F)
{
    const u32 i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n || up[i] == 1.0f) return;
    const V3 ap = ld3(pos[i]), an = ld3(nrm[i]);
    for (u32 j = lane; j < n; j += 32) {
        float f = 0.0f;
        if (j != i) {
            const V3 bp = ld3(pos[j]), bn = ld3(nrm[j]);
            f = i < j ? pair_pretest(ap, an, bp, bn) : pair_pretest(bp, bn, ap, an);
        }
        F[(size_t) i * ld + j] = store_f<__half>(f, up, i);
    }
}

// counts[1]: links kept
template <class T, bool kWide>
__global__ void k_ff_visibility(size_t ld, const float4* __restrict__ pos, BvhView bvh, ErrFlag err, int links,
                                T* __restrict__ F, const PairRef* __restrict__ cand, unsigned long long n_cand,
                                unsigned long long* next, unsigned long long* counts)
{
    const int lane = threadIdx.x & 31;
    unsigned long long kept = 0;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(next, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_cand) break;
        const unsigned long long k = base + lane;
        if (k < n_cand) {
            const PairRef pr = cand[k];
            V3 AP = ld3(pos[pr.i]), BP = ld3(pos[pr.j]);
            V3 dn = normalized(BP - AP);
            bool occluded = bvh_any_hit<kWide>(bvh, AP + dn * kSmall, BP - dn * kSmall, err);
            bool keep = links == 0 ? occluded : !occluded;
            if (keep) {
                ++kept;
            } else {
                F[(size_t) pr.i * ld + pr.j] = to_store<T>(0.0f);
                F[(size_t) pr.j * ld + pr.i] = to_store<T>(0.0f);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) kept += __shfl_down_sync(0xffffffffu, kept, o);
    if (lane == 0 && kept) atomicAdd(&counts[1], kept);
}

// X_j = (out_j * diffuse_j) * area_j (lighter.cpp:781-782 without the factor).
__global__ void k_rad_x(u32 n, const float4* __restrict__ out, const float4* __restrict__ da, float4* __restrict__ X)
{
    u32 j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float4 o = out[j], d = da[j];
    V3 x = (mk(o.x, o.y, o.z) * mk(d.x, d.y, d.z)) * d.w;
    X[j] = st4(x, 0.0f);
}

// Four entries of a 16-bit F (one 8-byte load, streamed once) and their values.
struct Raw4x16 {
    uint2 u;
    __device__ __forceinline__ void load(const void* p) { u = __ldcs(reinterpret_cast<const uint2*>(p)); }
    __device__ __forceinline__ unsigned bits() const { return u.x | u.y; }
};
template <class T> __device__ __forceinline__ void unpack4(const uint2& raw, float* v)
{
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        float2 f;
        if constexpr (std::is_same<T, __half>::value) f = __half22float2(reinterpret_cast<const __half2*>(&raw)[k]);
        else f = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(&raw)[k]);
        v[2 * k] = f.x; v[2 * k + 1] = f.y;
    }
}
// Bits of entry k of a 16-byte vector of F (entries of type T) held in words w.
template <class T> __device__ __forceinline__ unsigned entry_bits(const unsigned* w, int k)
{
    if constexpr (sizeof(T) == 4) return w[k];
    else return (w[k >> 1] >> (16 * (k & 1))) & 0xffffu;
}
template <class T> __device__ __forceinline__ float entry_f(const unsigned* w, int k)
{
    if constexpr (sizeof(T) == 4) return __uint_as_float(w[k]);
    else if constexpr (std::is_same<T, __half>::value)
        return __half2float(__ushort_as_half((unsigned short) entry_bits<T>(w, k)));
    else return __uint_as_float(entry_bits<T>(w, k) << 16);   // bf16 is the high half of a float
}

constexpr int kRadRows = 4;   // rows of F per warp in the bounce products
constexpr int kRadDepth = 4;  // steps of F a lane has in flight in the refined bounce

// One 16-byte vector (entries c V .. c V + V - 1) of each of a warp's rows,
// raw words w, added to the row sums of an F that is not refined. An entry's X
// is loaded when the entry is non-zero in any of the rows; the rows then add
// x * f without testing f: a zero entry adds +0 to a sum of non-negative terms,
// which leaves it unchanged bit for bit. A 16-bit F uses fused multiply-adds (its
// rounding is not the FP32 F's); FP32 keeps the separate multiply and add of the
// refined product, so both sum the same values in the same order.
template <class T>
__device__ __forceinline__ void plain_vector(const unsigned (&w)[kRadRows][4], u32 c, const float4* __restrict__ X,
                                             float (&acc)[kRadRows][3])
{
    constexpr int V = 16 / (int) sizeof(T);
    unsigned m[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        m[q] = w[0][q];
#pragma unroll
        for (int r = 1; r < kRadRows; ++r) m[q] |= w[r][q];
    }
    // F is sparse (pairs more than a few metres apart have factors below
    // SMALL_FLOAT, and occluded pairs are 0): a vector that is zero in all the
    // rows is skipped with one test (F holds no negative values and its zeros
    // are +0, so "no bit set" is "all entries zero")
    if (!(m[0] | m[1] | m[2] | m[3])) return;
#pragma unroll
    for (int k = 0; k < V; ++k) {
        if (!entry_bits<T>(m, k)) continue;
        const float4 x = __ldg(&X[c * V + k]);
#pragma unroll
        for (int r = 0; r < kRadRows; ++r) {
            const float fv = entry_f<T>(w[r], k);
            if constexpr (sizeof(T) == 4) {
                acc[r][0] += x.x * fv; acc[r][1] += x.y * fv; acc[r][2] += x.z * fv;
            } else {
                acc[r][0] = fmaf(x.x, fv, acc[r][0]);
                acc[r][1] = fmaf(x.y, fv, acc[r][1]);
                acc[r][2] = fmaf(x.z, fv, acc[r][2]);
            }
        }
    }
}

// Warp sums of the row sums and the bounce's updates (lane 0 writes).
__device__ __forceinline__ void bounce_epilogue(u32 n, u32 r0, float (&acc)[kRadRows][3], const float* __restrict__ up,
                                                const float4* __restrict__ da, float4* __restrict__ total,
                                                float4* __restrict__ out, float4* __restrict__ Xn)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < kRadRows; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            for (int o = 16; o > 0; o >>= 1) acc[r][q] += __shfl_down_sync(0xffffffffu, acc[r][q], o);
    if (lane == 0) {
#pragma unroll
        for (int r = 0; r < kRadRows; ++r) {
            const u32 j = r0 + r;
            if (j >= n) continue;
            const float s = up ? up[j] : 1.0f;   // row scale of an FP16 F (exact)
            const float4 y = make_float4(acc[r][0] * s, acc[r][1] * s, acc[r][2] * s, 0.0f);
            const float4 t = total[j], d = da[j];
            total[j] = make_float4(t.x + y.x, t.y + y.y, t.z + y.z, 0.0f);
            out[j] = y;
            Xn[j] = st4((mk(y.x, y.y, y.z) * mk(d.x, d.y, d.z)) * d.w, 0.0f);
        }
    }
}

// A refined bounce of a 16-bit F (lighter.cpp:767-797): Y = F X with F serving
// only as the link mask; the factor of every linked pair is recomputed in FP32
// with pair_pretest, lower index first as k_ff_pretest computes it, i.e. bit for
// bit the value an FP32 F holds (a linked factor is >= SMALL_FLOAT, which
// neither FP16 nor BF16 rounds to 0, so a 16-bit mask is the FP32 one). Then
// total += Y, out = Y and the next bounce's X in the epilogue. A warp takes
// kRadRows rows and reads them 4 entries per lane per row (8-byte loads, the
// loads of the next kDepth - 1 steps issued before a step's arithmetic); lane l
// takes the 4-entry vectors l, l + 32, ... in order, as k_rad_stream does for
// an FP32 F, so the refined product of a 16-bit F is the FP32 product. The
// recomputed factors make this kernel arithmetic-bound, not HBM-bound.
template <class T, int kDepth>
__global__ void __launch_bounds__(256) k_rad_refined(u32 n, size_t ld, const T* __restrict__ F,
                                                     const float4* __restrict__ pos, const float4* __restrict__ nrm,
                                                     const float4* __restrict__ X, const float4* __restrict__ da,
                                                     float4* __restrict__ total, float4* __restrict__ out,
                                                     float4* __restrict__ Xn)
{
    static_assert(sizeof(T) == 2, "the refined bounce reads a 16-bit F");
    constexpr int V = 4;
    using Raw = Raw4x16;
    const int lane = threadIdx.x & 31;
    const u32 r0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kRadRows;
    if (r0 >= n) return;
    const T* rows[kRadRows];
    V3 ap[kRadRows], an[kRadRows];
    u32 ri[kRadRows];
#pragma unroll
    for (int r = 0; r < kRadRows; ++r) {
        ri[r] = min(r0 + r, n - 1);   // rows past n repeat the last row and are not written
        rows[r] = F + (size_t) ri[r] * ld;
        ap[r] = ld3(pos[ri[r]]);
        an[r] = ld3(nrm[ri[r]]);
    }
    float acc[kRadRows][3];
#pragma unroll
    for (int r = 0; r < kRadRows; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0.0f;
    const u32 nv = (u32) (ld / V);
    Raw buf[kDepth][kRadRows];
#pragma unroll
    for (int d = 0; d < kDepth - 1; ++d) {
        const u32 cc = lane + 32u * d;
        if (cc < nv) {
#pragma unroll
            for (int r = 0; r < kRadRows; ++r) buf[d][r].load(rows[r] + (size_t) cc * V);
        }
    }
    for (u32 base = lane; base < nv; base += 32u * kDepth) {
#pragma unroll
        for (int d = 0; d < kDepth; ++d) {
            const u32 c = base + 32u * d;
            const u32 cl = c + 32u * (kDepth - 1);
            if (cl < nv) {
#pragma unroll
                for (int r = 0; r < kRadRows; ++r) buf[(d + kDepth - 1) % kDepth][r].load(rows[r] + (size_t) cl * V);
            }
            if (c >= nv) break;
            const Raw* cur = buf[d];
            unsigned nz = 0;   // all four rows unlinked over these 4 columns: nothing to add
#pragma unroll
            for (int r = 0; r < kRadRows; ++r) nz |= cur[r].bits();
            if (!nz) continue;
            float f[kRadRows][V];
#pragma unroll
            for (int r = 0; r < kRadRows; ++r) unpack4<T>(cur[r].u, f[r]);
#pragma unroll
            for (int k = 0; k < V; ++k) {
                bool any = false;
#pragma unroll
                for (int r = 0; r < kRadRows; ++r) any |= f[r][k] != 0.0f;
                if (any) {
                    const u32 j = c * V + k;
                    const float4 x = __ldg(&X[j]);
                    const V3 bp = ld3(pos[j]), bn = ld3(nrm[j]);
#pragma unroll
                    for (int r = 0; r < kRadRows; ++r) {
                        if (f[r][k] != 0.0f) {
                            const float fv = ri[r] < j ? pair_pretest(ap[r], an[r], bp, bn)
                                                       : pair_pretest(bp, bn, ap[r], an[r]);
                            acc[r][0] += x.x * fv; acc[r][1] += x.y * fv; acc[r][2] += x.z * fv;
                        }
                    }
                }
            }
        }
    }
    bounce_epilogue(n, r0, acc, nullptr, da, total, out, Xn);
}

constexpr u32 kErrWait = 2u;   // radiosity error word: a bounded wait for staged F expired

// ltrdbg_RadiosityStallNextBounce: wait limit (us) of the next unrefined bounce
// whose copy producer issues nothing; 0 = none pending.
std::atomic<uint32_t> g_stall_next_bounce{0};
constexpr unsigned long long kStreamWaitCycles = 4000000000ull;   // about 2 s at 2 GHz

// Launch shape of k_rad_stream: warps per CTA, ring stages per warp, and
// 16-byte vectors per lane, row and stage.
constexpr int kStreamWarps = 4, kStreamStages = 3, kStreamVec = 4;

constexpr size_t stream_smem_bytes(int warps, int stages, int vec)
{
    return (size_t) warps * stages * kRadRows * vec * 512 + (size_t) warps * stages * 8;
}

// The bounce of an F that is not refined, with F staged through shared memory
// by bulk asynchronous copies (cp.async.bulk, completing on an mbarrier per
// stage) instead of through registers: a warp keeps kStages stages of its
// kRadRows rows in flight (kStages x kRadRows x kVec x 512 bytes), far more
// than registers hold, which is what an HBM stream of this many independent
// rows needs to reach the memory's bandwidth. Each warp owns its rows and its
// ring; lane 0 issues the copies and refills a stage once the warp has read it.
// Lane l reads vectors l, l + 32, l + 64, ... of each row in increasing order,
// the register kernel's order, so both give the same bits.
template <class T, int kWarps, int kStages, int kVec>
__global__ void __launch_bounds__(kWarps * 32) k_rad_stream(u32 n, size_t ld, const T* __restrict__ F,
                                                            const float* __restrict__ up,
                                                            const float4* __restrict__ X,
                                                            const float4* __restrict__ da,
                                                            float4* __restrict__ total, float4* __restrict__ out,
                                                            float4* __restrict__ Xn, u32* err,
                                                            unsigned long long wait_cycles, u32 issue)
{
    constexpr int V = 16 / (int) sizeof(T);       // entries per 16-byte vector
    constexpr u32 kPart = kVec * 512u;            // bytes of one row in one stage
    constexpr u32 kPer = 32u * kVec;              // vectors of one row in one stage
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const u32 r0 = (blockIdx.x * kWarps + w) * kRadRows;
    if (r0 >= n) return;   // the whole warp
    unsigned char* ring = smem + (size_t) w * kStages * kRadRows * kPart;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + (size_t) kWarps * kStages * kRadRows * kPart) + w * kStages;
    const T* rows[kRadRows];
#pragma unroll
    for (int r = 0; r < kRadRows; ++r) rows[r] = F + (size_t) min(r0 + r, n - 1) * ld;   // rows past n: not written
    const u32 nv = (u32) (ld / V);               // vectors per row (ld V-aligned: rows on 16-byte boundaries)
    const u32 nch = (nv + kPer - 1) / kPer;      // stages per row sweep
    uint64_t policy = 0;
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < kStages; ++q) mbar_init(&bar[q], 1);
        mbar_init_fence();
        policy = l2_evict_first_policy();
    }
    __syncwarp();
    // lane 0: chunk k of every row into stage k % kStages (`issue` 0: never, the
    // test of the bounded waits)
    auto fill = [&](u32 k) {
        const u32 q = k % kStages;
        const u32 v0 = k * kPer;
        const u32 bytes = min(kPer, nv - v0) * 16u;
        mbar_expect_tx(&bar[q], bytes * kRadRows);
#pragma unroll
        for (int r = 0; r < kRadRows; ++r)
            bulk_g2s(ring + (size_t) (q * kRadRows + r) * kPart, rows[r] + (size_t) v0 * V, bytes, &bar[q], policy);
    };
    if (lane == 0 && issue)
        for (u32 k = 0; k < nch && k < (u32) kStages; ++k) fill(k);
    float acc[kRadRows][3];
#pragma unroll
    for (int r = 0; r < kRadRows; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0.0f;
    u32 k = 0;
    bool ok = true;
    for (; k < nch; ++k) {
        const u32 q = k % kStages;
        ok = __all_sync(full, mbar_wait(&bar[q], (k / kStages) & 1u, err, kErrWait, wait_cycles));
        if (!ok) break;
#pragma unroll
        for (int e = 0; e < kVec; ++e) {
            const u32 c = k * kPer + 32u * e + lane;
            if (c < nv) {
                unsigned wv[kRadRows][4];
#pragma unroll
                for (int r = 0; r < kRadRows; ++r) {
                    const uint4 u = *reinterpret_cast<const uint4*>(ring + (size_t) (q * kRadRows + r) * kPart +
                                                                    512u * e + 16u * lane);
                    wv[r][0] = u.x; wv[r][1] = u.y; wv[r][2] = u.z; wv[r][3] = u.w;
                }
                plain_vector<T>(wv, c, X, acc);
            }
        }
        __syncwarp();   // every lane has read stage q before it is refilled
        if (lane == 0 && issue && k + kStages < nch) fill(k + kStages);
    }
    if (!ok) {
        // a wait expired (error bit set): wait, bounded again, for the copies still
        // issued into this warp's ring before the CTA's shared memory is released
        if (lane == 0 && issue)
            for (u32 j = k; j < nch && j < k + kStages; ++j)
                if (!mbar_wait(&bar[j % kStages], (j / kStages) & 1u, err, kErrWait, wait_cycles)) break;
        return;
    }
    bounce_epilogue(n, r0, acc, up, da, total, out, Xn);
}

// F (n x ld, stored type) widened to n x n floats (debug copy).
template <class T>
__global__ void k_f_widen(u32 n, size_t ld, const T* __restrict__ F, const float* __restrict__ up,
                          float* __restrict__ out)
{
    size_t k = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t) n * n) return;
    out[k] = to_f(F[(k / n) * ld + k % n]) * (up ? up[k / n] : 1.0f);
}

// Both passes on `st`; returns the visibility-ray count and, when `counts_keep`
// is null, the link count (synchronises the stream after the first pass, to size
// the pair list, and then after the second for the link count). With
// `counts_keep` (3 device words the caller owns) the link count stays in
// counts_keep[1] and the function returns with the second pass still queued, so
// the caller's next kernels are enqueued behind it.
template <class T>
RadFormFactors build_ff(u32 n, size_t ld, const float4* pos, const float4* nrm, const BvhView& bvh, ErrFlag err,
                        int links, T* F, unsigned* rowmax, float* up, cudaStream_t st,
                        unsigned long long* counts_keep = nullptr)
{
    RadFormFactors out;
    if (n == 0) return out;
    const u32 nb = (n + 31) / 32;
    if (nb > 65535) throw std::runtime_error("radiosity: too many elements for the tile grid");
    if (ld < n || ld > (size_t) nb * 32) throw std::runtime_error("radiosity: bad leading dimension");
    const unsigned long long pairs = (unsigned long long) n * (n - 1) / 2;
    unsigned long long cap = std::min<unsigned long long>(pairs, std::max<unsigned long long>(1ull << 24, pairs / 16));
    unsigned long long* counts = nullptr;   // [0] pairs that passed, [1] links kept, [2] work counter
    PairRef* cand = nullptr;
    unsigned long long* own_counts = nullptr;
    if (counts_keep) counts = counts_keep;
    else RCK(cudaMallocAsync(&own_counts, 3 * sizeof(unsigned long long), st)), counts = own_counts;
    struct Free {
        cudaStream_t st; void** p[2];
        ~Free() { for (void** q : p) if (*q) cudaFreeAsync(*q, st); }
    } guard{st, {(void**) &own_counts, (void**) &cand}};
    unsigned long long n_cand = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
        RCK(cudaMallocAsync(&cand, std::max<unsigned long long>(cap, 1) * sizeof(PairRef), st));
        RCK(cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), st));
        if (rowmax) RCK(cudaMemsetAsync(rowmax, 0, n * sizeof(unsigned), st));
        k_ff_pretest<T><<<dim3(nb, nb), dim3(32, 8), 0, st>>>(n, ld, pos, nrm, rowmax, F, cand, cap, counts); note_launch();
        RCK(cudaGetLastError());
        RCK(cudaMemcpyAsync(&n_cand, counts, sizeof(n_cand), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(n_cand));
        RCK(cudaStreamSynchronize(st));
        if (n_cand <= cap) break;
        RCK(cudaFreeAsync(cand, st));   // again, with room for every pair that passed
        cand = nullptr;
        cap = n_cand;
    }
    if (n_cand > cap) throw std::runtime_error("radiosity: pair list overflow");
    if constexpr (std::is_same<T, __half>::value) {
        if (rowmax && up) {
            k_row_scale<<<(n + 255) / 256, 256, 0, st>>>(n, rowmax, up); note_launch();
            k_ff_rescale<<<(unsigned) (((size_t) n * 32 + 255) / 256), 256, 0, st>>>(n, ld, pos, nrm, up, F); note_launch();
            RCK(cudaGetLastError());
        }
    }
    if (n_cand) {
        int dev = 0, sms = 0;
        RCK(cudaGetDevice(&dev));
        RCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        unsigned grid = (unsigned) std::min<unsigned long long>((unsigned long long) sms * 8, (n_cand + 127) / 128);
        // the 4-wide walk for trees of 256k references and more (see walk_segment4)
        if (bvh.n_tris >= (1 << 18))
            k_ff_visibility<T, true><<<grid, 128, 0, st>>>(ld, pos, bvh, err, links, F, cand, n_cand, counts + 2, counts);
        else
            k_ff_visibility<T, false><<<grid, 128, 0, st>>>(ld, pos, bvh, err, links, F, cand, n_cand, counts + 2, counts);
        note_launch();
        RCK(cudaGetLastError());
    }
    out.vis_rays = n_cand;
    if (!counts_keep) {
        unsigned long long hc[2] = {0, 0};
        RCK(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(hc));
        RCK(cudaStreamSynchronize(st));
        out.links = hc[1];
    }
    return out;
}

template <class T>
RadResult solve_t(const RadDevInputs& in, const RadSettings& rs, const BvhView& bvh, ErrFlag err, cudaStream_t st,
                  float4* total_out, std::atomic<bool>* abort_flag)
{
    RadResult rr;
    const u32 n = in.n;
    size_t free_b = 0, total_b = 0;
    RCK(cudaMemGetInfo(&free_b, &total_b));
    const size_t ld = ((size_t) n + 7) / 8 * 8;   // rows on 16-byte boundaries
    size_t fbytes = (size_t) n * ld * sizeof(T);
    if (fbytes > free_b / 10 * 9)
        throw std::runtime_error("radiosity: dense form factors for " + std::to_string(n) + " elements need " +
                                 std::to_string(fbytes >> 20) + " MiB, more than the free device memory");
    T* F = nullptr;
    float4 *out, *X, *Y;
    unsigned long long* counts;   // the form-factor build's counters, read after the bounces
    RCK(cudaMallocAsync(&F, fbytes ? fbytes : 1, st));
    RCK(cudaMallocAsync(&out, n * sizeof(float4), st));
    RCK(cudaMallocAsync(&X, n * sizeof(float4), st));
    RCK(cudaMallocAsync(&Y, n * sizeof(float4), st));
    RCK(cudaMallocAsync(&counts, 3 * sizeof(unsigned long long), st));
    struct Free {
        cudaStream_t st; void* p[5];
        ~Free() { for (void* q : p) if (q) cudaFreeAsync(q, st); }
    } guard{st, {F, out, X, Y, counts}};
    float4* total = total_out;
    RCK(cudaMemcpyAsync(out, in.emit, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    if (total != in.emit) RCK(cudaMemcpyAsync(total, in.emit, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));

    cudaEvent_t e0, e1, e2;
    RCK(cudaEventCreate(&e0)); RCK(cudaEventCreate(&e1)); RCK(cudaEventCreate(&e2));
    RCK(cudaEventRecord(e0, st));
    float* up = nullptr;   // row scales of an FP16 F
    unsigned* rowmax = nullptr;
    struct FreeScale {
        cudaStream_t st; void** p[2];
        ~FreeScale() { for (void** q : p) if (*q) cudaFreeAsync(*q, st); }
    } guard_scale{st, {(void**) &up, (void**) &rowmax}};
    if (std::is_same<T, __half>::value) {
        RCK(cudaMallocAsync(&up, n * sizeof(float), st));
        RCK(cudaMallocAsync(&rowmax, n * sizeof(unsigned), st));
    }
    // the bounces are enqueued behind the visibility pass (no host wait between them)
    RadFormFactors ff = build_ff<T>(n, ld, in.pos, in.nrm, bvh, err, rs.links, F, rowmax, up, st, counts);
    RCK(cudaEventRecord(e1, st));
    if (rs.f_host) {
        const size_t nn = (size_t) n * n;
        float* wide = nullptr;
        RCK(cudaMallocAsync(&wide, nn * sizeof(float), st));
        k_f_widen<T><<<(unsigned) ((nn + 255) / 256), 256, 0, st>>>(n, ld, F, up, wide); note_launch();
        RCK(cudaGetLastError());
        RCK(cudaMemcpyAsync(rs.f_host, wide, nn * sizeof(float), cudaMemcpyDeviceToHost, st)); note_d2h(nn * sizeof(float));
        RCK(cudaFreeAsync(wide, st));
    }
    if (rs.bounces > 0) {
        k_rad_x<<<(n + 255) / 256, 256, 0, st>>>(n, out, in.diff_area, X); note_launch();
    }
    for (int b = 0; b < rs.bounces; ++b) {
        if (abort_flag && abort_flag->load()) break;
        const float4* Xb = (b & 1) ? Y : X;   // X of this bounce; the kernel writes the next one's
        float4* Xnext = (b & 1) ? X : Y;
        // the last refine_steps bounces of a 16-bit F recompute the factors in FP32
        const bool exact = sizeof(T) < 4 && b >= rs.bounces - rs.refine_steps;
        const unsigned grid = (unsigned) ((((size_t) n + kRadRows - 1) / kRadRows * 32 + 255) / 256);
        if constexpr (sizeof(T) == 2) {
            if (exact) {
                k_rad_refined<T, kRadDepth><<<grid, 256, 0, st>>>(n, ld, F, in.pos, in.nrm, Xb, in.diff_area, total,
                                                                   out, Xnext);
            }
        }
        if (!exact) {
            auto kern = k_rad_stream<T, kStreamWarps, kStreamStages, kStreamVec>;
            const size_t sm = stream_smem_bytes(kStreamWarps, kStreamStages, kStreamVec);
            RCK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm));
            const unsigned sgrid = (unsigned) (((size_t) n + kRadRows * kStreamWarps - 1) / (kRadRows * kStreamWarps));
            const uint32_t stall_us = g_stall_next_bounce.exchange(0);
            const unsigned long long wait = stall_us ? (unsigned long long) stall_us * 2000ull : kStreamWaitCycles;
            kern<<<sgrid, kStreamWarps * 32, sm, st>>>(n, ld, F, up, Xb, in.diff_area, total, out, Xnext, err.word,
                                                       wait, stall_us ? 0u : 1u);
        }
        note_launch();
        RCK(cudaGetLastError());
    }
    RCK(cudaEventRecord(e2, st));
    unsigned long long hc[3] = {0, 0, 0};
    RCK(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(hc));
    RCK(cudaStreamSynchronize(st));
    ff.links = n ? hc[1] : 0;
    float m1 = 0, m2 = 0;
    cudaEventElapsedTime(&m1, e0, e1);
    cudaEventElapsedTime(&m2, e1, e2);
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
    rr.links = ff.links;
    rr.vis_rays = ff.vis_rays;
    rr.pairs = (uint64_t) n * (n - 1) / 2;
    rr.ms_links = m1;
    rr.ms_bounce = m2;
    return rr;
}

}  // namespace

RadResult radiosity_solve_dev(const RadDevInputs& in, const RadSettings& rs, const BvhView& bvh, ErrFlag err,
                              cudaStream_t st, float4* total_out, std::atomic<bool>* abort_flag)
{
    if (in.n == 0) return RadResult();
    if (rs.precision == 1) return solve_t<__half>(in, rs, bvh, err, st, total_out, abort_flag);
    if (rs.precision == 2) return solve_t<__nv_bfloat16>(in, rs, bvh, err, st, total_out, abort_flag);
    return solve_t<float>(in, rs, bvh, err, st, total_out, abort_flag);
}

RadFormFactors radiosity_form_factors_f32(uint32_t n, const float4* pos, const float4* nrm, const BvhView& bvh,
                                          ErrFlag err, int links, float* F, cudaStream_t st)
{
    return build_ff<float>(n, n, pos, nrm, bvh, err, links, F, nullptr, nullptr, st);
}

RadResult radiosity_solve(const RadInputs& in, const RadSettings& rs, const BvhView& bvh, ErrFlag err, cudaStream_t st,
                          float4* lm_out, std::atomic<bool>* abort_flag)
{
    if (in.n == 0) return RadResult();
    const u32 n = in.n;
    float4* buf = nullptr;
    RCK(cudaMallocAsync(&buf, 4 * (size_t) n * sizeof(float4), st));
    struct Free { cudaStream_t st; void* p; ~Free() { cudaFreeAsync(p, st); } } guard{st, buf};
    const std::vector<float4>* src[4] = {&in.pos, &in.nrm, &in.diff_area, &in.emit};
    for (int k = 0; k < 4; ++k) {
        RCK(cudaMemcpyAsync(buf + (size_t) k * n, src[k]->data(), n * sizeof(float4), cudaMemcpyHostToDevice, st));
        note_h2d(n * sizeof(float4));
    }
    RadDevInputs d{n, buf, buf + n, buf + 2 * (size_t) n, buf + 3 * (size_t) n};
    return radiosity_solve_dev(d, rs, bvh, err, st, lm_out, abort_flag);
}

}  // namespace lg

extern "C" LTRAPI LTRBOOL ltrdbg_RadiosityStallNextBounce(u32 wait_us)
{
    if (wait_us == 0 || wait_us > 2000000u) return 0;
    lg::g_stall_next_bounce.store(wait_us);
    return 1;
}
