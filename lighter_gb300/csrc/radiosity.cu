// Dense radiosity of the bake (see radiosity.cuh).
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <type_traits>

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

// One vector load of V entries of F (16 or 8 bytes), and its entries as floats.
template <int B> struct RawF;
template <> struct RawF<16> {
    uint4 u;
    __device__ __forceinline__ void load(const void* p) { u = __ldcs(reinterpret_cast<const uint4*>(p)); }
    __device__ __forceinline__ unsigned bits() const { return u.x | u.y | u.z | u.w; }
};
template <> struct RawF<8> {
    uint2 u;
    __device__ __forceinline__ void load(const void* p) { u = __ldcs(reinterpret_cast<const uint2*>(p)); }
    __device__ __forceinline__ unsigned bits() const { return u.x | u.y; }
};
template <class T, int V> __device__ __forceinline__ void unpack(const void* raw, float* v)
{
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int k = 0; k < V; ++k) v[k] = reinterpret_cast<const float*>(raw)[k];
    } else {
#pragma unroll
        for (int k = 0; k < V / 2; ++k) {
            float2 f;
            if constexpr (std::is_same<T, __half>::value) f = __half22float2(reinterpret_cast<const __half2*>(raw)[k]);
            else f = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(raw)[k]);
            v[2 * k] = f.x; v[2 * k + 1] = f.y;
        }
    }
}

constexpr int kRadRows = 4;   // rows of F per warp in the bounce product
constexpr int kRadDepth = 4;  // steps of F a lane has in flight in the bounce product

// Y = F X (one bounce's gather). F is streamed once per bounce, so the kernel is
// HBM-bound: a warp takes kRadRows rows and reads them V entries per lane per
// row (16 bytes; the next step's loads issued before this step's arithmetic),
// and each X_j it loads serves all its rows. A zero entry (no link) skips its X
// load. Rows are ld entries apart, ld a multiple of 8 with zeros past n, so
// every row starts on a 16-byte boundary.
// kExact: F serves only as the link mask and the factor of every linked pair is
// recomputed in FP32 with pair_pretest, lower index first as k_ff_pretest
// computes it, i.e. bit-for-bit the value an FP32 F holds. A linked factor is
// >= SMALL_FLOAT, which neither FP16 nor BF16 rounds to 0, so a 16-bit mask is
// the FP32 one. kExact reads 4 entries per lane (8-byte loads of a 16-bit F),
// the FP32 kernel's split of columns over lanes, so both sum in the same order:
// the kExact product of a 16-bit F is the FP32 product.
template <class T, bool kExact, int kDepth = 2>
__global__ void __launch_bounds__(256) k_rad_gemv(u32 n, size_t ld, const T* __restrict__ F,
                                                  const float4* __restrict__ pos, const float4* __restrict__ nrm,
                                                  const float* __restrict__ up, const float4* __restrict__ X,
                                                  float4* __restrict__ Y)
{
    constexpr int V = kExact ? 4 : 16 / (int) sizeof(T);
    using Raw = RawF<V * sizeof(T)>;
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
        if (kExact) { ap[r] = ld3(pos[ri[r]]); an[r] = ld3(nrm[ri[r]]); }
    }
    float acc[kRadRows][3];
#pragma unroll
    for (int r = 0; r < kRadRows; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0.0f;
    const u32 nv = (u32) (ld / V);
    // software pipeline kDepth steps deep: the loads of step c + 32 (kDepth - 1)
    // are issued before step c's arithmetic (each lane still walks its columns
    // in increasing order, so the sums keep their order)
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
            // F is sparse (pairs more than a few metres apart have factors below
            // SMALL_FLOAT, and occluded pairs are 0): a vector that is zero in all the
            // warp's rows is skipped with one test (F holds no negative values and its
            // zeros are +0, so "no bit set" is "all entries zero")
            unsigned nz = 0;
#pragma unroll
            for (int r = 0; r < kRadRows; ++r) nz |= cur[r].bits();
            if (!nz) continue;
            float f[kRadRows][V];
#pragma unroll
            for (int r = 0; r < kRadRows; ++r) unpack<T, V>(&cur[r].u, f[r]);
#pragma unroll
            for (int k = 0; k < V; ++k) {
                bool any = false;
#pragma unroll
                for (int r = 0; r < kRadRows; ++r) any |= f[r][k] != 0.0f;
                if (any) {
                    const u32 j = c * V + k;
                    const float4 x = __ldg(&X[j]);
                    V3 bp, bn;
                    if (kExact) { bp = ld3(pos[j]); bn = ld3(nrm[j]); }
#pragma unroll
                    for (int r = 0; r < kRadRows; ++r) {
                        if (f[r][k] != 0.0f) {
                            float fv = f[r][k];
                            if (kExact) fv = ri[r] < j ? pair_pretest(ap[r], an[r], bp, bn) : pair_pretest(bp, bn, ap[r], an[r]);
                            acc[r][0] += x.x * fv; acc[r][1] += x.y * fv; acc[r][2] += x.z * fv;
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kRadRows; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            for (int o = 16; o > 0; o >>= 1) acc[r][q] += __shfl_down_sync(0xffffffffu, acc[r][q], o);
    if (lane == 0) {
#pragma unroll
        for (int r = 0; r < kRadRows; ++r) {
            if (r0 + r >= n) continue;
            const float s = (!kExact && up) ? up[r0 + r] : 1.0f;   // row scale of an FP16 F (exact)
            Y[r0 + r] = make_float4(acc[r][0] * s, acc[r][1] * s, acc[r][2] * s, 0.0f);
        }
    }
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

// total += Y, out = Y (lighter.cpp:784-796).
__global__ void k_rad_update(u32 n, const float4* __restrict__ Y, float4* __restrict__ total, float4* __restrict__ out)
{
    u32 j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float4 y = Y[j], t = total[j];
    total[j] = make_float4(t.x + y.x, t.y + y.y, t.z + y.z, 0.0f);
    out[j] = y;
}

// Both passes on `st`; returns the link and visibility-ray counts (synchronises
// the stream once after the first pass, to size the pair list).
template <class T>
RadFormFactors build_ff(u32 n, size_t ld, const float4* pos, const float4* nrm, const BvhView& bvh, ErrFlag err,
                        int links, T* F, unsigned* rowmax, float* up, cudaStream_t st)
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
    RCK(cudaMallocAsync(&counts, 3 * sizeof(unsigned long long), st));
    struct Free {
        cudaStream_t st; void** p[2];
        ~Free() { for (void** q : p) if (*q) cudaFreeAsync(*q, st); }
    } guard{st, {(void**) &counts, (void**) &cand}};
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
    unsigned long long hc[2] = {0, 0};
    RCK(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(hc));
    RCK(cudaStreamSynchronize(st));
    out.vis_rays = n_cand;
    out.links = hc[1];
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
    RCK(cudaMallocAsync(&F, fbytes ? fbytes : 1, st));
    RCK(cudaMallocAsync(&out, n * sizeof(float4), st));
    RCK(cudaMallocAsync(&X, n * sizeof(float4), st));
    RCK(cudaMallocAsync(&Y, n * sizeof(float4), st));
    struct Free {
        cudaStream_t st; void* p[4];
        ~Free() { for (void* q : p) if (q) cudaFreeAsync(q, st); }
    } guard{st, {F, out, X, Y}};
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
    RadFormFactors ff = build_ff<T>(n, ld, in.pos, in.nrm, bvh, err, rs.links, F, rowmax, up, st);
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
    for (int b = 0; b < rs.bounces; ++b) {
        if (abort_flag && abort_flag->load()) break;
        k_rad_x<<<(n + 255) / 256, 256, 0, st>>>(n, out, in.diff_area, X); note_launch();
        // the last refine_steps bounces of a 16-bit F recompute the factors in FP32
        const bool exact = sizeof(T) < 4 && b >= rs.bounces - rs.refine_steps;
        const unsigned grid = (unsigned) ((((size_t) n + kRadRows - 1) / kRadRows * 32 + 255) / 256);
        if (exact)
            k_rad_gemv<T, true, kRadDepth><<<grid, 256, 0, st>>>(n, ld, F, in.pos, in.nrm, up, X, Y);
        else
            k_rad_gemv<T, false, kRadDepth><<<grid, 256, 0, st>>>(n, ld, F, in.pos, in.nrm, up, X, Y);
        note_launch();
        k_rad_update<<<(n + 255) / 256, 256, 0, st>>>(n, Y, total, out); note_launch();
        RCK(cudaGetLastError());
    }
    RCK(cudaEventRecord(e2, st));
    RCK(cudaStreamSynchronize(st));
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
