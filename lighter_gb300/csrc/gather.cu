// Multi-right-hand-side radiosity gather on dense form factors.
//
// The reference's bounce (Int_RDBounce, lighter.cpp:767-797) is one sweep of
// B <- E + K B over sparse links, K_ij = f_ij area_j diffuse_j, for one light
// configuration. For R right-hand sides (RGB x light configurations) the sweep
// is the contraction
//     B_k = E + G X_{k-1},   G_ij = f_ij area_j,   X_j(r) = albedo_j(r mod 3) B_j(r)
// whose left operand G (N x N) streams from HBM once per bounce while X
// (N x R) stays in L2.
//
//   FP32        G in FP32, register-blocked SIMT GEMM              k_sgemm_bounce
//   FP16/BF16   G in 16 bits on the tcgen05 tensor cores            k_umma_gather
//               (FP32 accumulation in TMEM), with optional head/tail
//               splits of X and of G (LTRG_REFINE_*) whose extra products
//               accumulate into the same FP32 accumulator
//
// k_umma_gather is a persistent stream-K kernel: the (256-row block, 64-wide
// k block) units of the whole product are cut into one contiguous range per
// CTA, so every SM gets the same number of units whatever N is. Per CTA:
//   warp 0      TMA producer: 256 x 64 tile of G (+ residual), BN x 64 tiles of
//               X^T (head, tail), 128-byte swizzle, into an S-stage ring
//   warp 1      allocates 512 TMEM columns; one thread issues
//               tcgen05.mma.cta_group::1.kind::f16 (M=128, N=BN, K=16) for both
//               128-row halves into two FP32 accumulators (columns 0 and 256)
//   warps 2-5   epilogue: tcgen05.ld of the accumulators, partial sums of each
//               row block written to a workspace slot
// k_combine then adds E and the slots of every row block in a fixed order
// (deterministic) and writes B and the next bounce's X^T. Every mbarrier wait
// is bounded: on expiry the kernel sets a bit of the error word, stops its
// loops, waits (bounded) for its own copies and products and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lighter_gb300.h"
#include "bvh.cuh"
#include "async.cuh"
#include "radiosity.cuh"

namespace lg {
namespace {

void gck(cudaError_t e, const char* what, int line)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) + " at gather.cu:" +
                                 std::to_string(line) + " (" + what + ")");
}
#define GCK(x) gck((x), #x, __LINE__)

constexpr int BM = 128;                  // rows per tcgen05.mma (M)
constexpr int ROWS = 2 * BM;             // rows of G per work unit
constexpr int BK = 64;                   // k per work unit (and the padding of a row of G)
constexpr int UK = 16;                   // k per tcgen05.mma (kind::f16)
constexpr int MAX_BN = 256;
constexpr int TMEM_COLS = 512;           // two accumulators of up to 256 columns
constexpr int kThreads = 192;
constexpr int kMaxStages = 8;
constexpr int kSmemLimit = 232448;       // opt-in dynamic shared memory per block
constexpr int kSmemExtra = 1024 + 256;   // alignment slack + barriers
constexpr unsigned long long kWaitCycles = 4000000000ull;   // about 2 s at 2 GHz

// error word bits
constexpr u32 kErrProducer = 1u, kErrMma = 2u, kErrEpilogue = 4u, kErrDrain = 8u;

// ----------------------------------------------------------------------------- PTX helpers

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            saddr(dst)),
        "l"(map), "r"(saddr(bar)), "r"(x), "r"(y)
        : "memory");
}

// Matrix descriptor of a K-major operand tile written by TMA with the swizzle
// of its row length KB x 2 bytes: 128-byte rows (KB = 64, 128-byte swizzle) or
// 64-byte rows (KB = 32, 64-byte swizzle), groups of 8 rows 8 x row bytes
// apart. Advancing K by 16 elements inside a row adds 32 bytes to the start.
template <int KB>
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
    static_assert(KB == 64 || KB == 32, "stage k must be 64 or 32");
    uint64_t d = 0;
    d |= (uint64_t) ((addr >> 4) & 0x3FFFu);          // start address >> 4
    d |= (uint64_t) 1u << 16;                          // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t) ((8u * KB * 2) >> 4) << 32;        // stride byte offset: 8 rows
    d |= (uint64_t) 1u << 46;                          // descriptor version
    d |= (uint64_t) (KB == 64 ? 2u : 4u) << 61;        // 128-byte or 64-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B of format `fmt` (0 FP16, 1 BF16; bits 7-9 and 10-12), both K-major
// (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
uint32_t idesc_f16(uint32_t fmt, uint32_t bn)
{
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((bn >> 3) << 17) | ((uint32_t) (BM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// Arrives on `bar` once every tcgen05.mma issued so far by this thread completes.
__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* v)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ----------------------------------------------------------------------------- tcgen05 gather

struct UmmaArgs {
    u32 nkb;              // k blocks (ld / 64)
    u32 n_rp;             // 256-row blocks
    u32 R, BN;            // right-hand sides, MMA N (multiple of 32, >= R)
    u32 stages, stage_bytes;
    u32 mode;             // LTRG_REFINE_*
    u32 idesc;
    u32 max_slots;
    u32 kchunk;           // k blocks accumulated in TMEM before moving to the FP32 workspace (0: no limit)
    const u32* rp_first;  // first CTA whose range touches each row block
    float* partial;       // [rp][slot][R][256]
    u32* err;
    unsigned long long wait_cycles;   // limit of every mbarrier wait (kWaitCycles)
    u32 issue;            // 0: the producer issues no copies (ltrdbg_GatherStallNextSolve), else 1
};

// KB: k per pipeline stage (a 64-wide work unit takes 64 / KB stages).
template <int KB>
__global__ void __launch_bounds__(kThreads, 1)
    k_umma_gather(const __grid_constant__ CUtensorMap tmG, const __grid_constant__ CUtensorMap tmGl,
                  const __grid_constant__ CUtensorMap tmXh, const __grid_constant__ CUtensorMap tmXl, UmmaArgs a)
{
    constexpr int SPU = BK / KB;                 // stages per work unit
    constexpr u32 A_BYTES = ROWS * KB * 2;       // one 256-row tile of G per stage
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = (unsigned char*) ((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t) 1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + (size_t) a.stages * a.stage_bytes);
    uint64_t* full = bars;
    uint64_t* empty = bars + kMaxStages;
    uint64_t* accf = bars + 2 * kMaxStages;       // accumulators ready for the epilogue
    uint64_t* acce = accf + 1;                    // accumulators drained
    uint64_t* done = accf + 2;                    // all products of this CTA complete
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accf + 3);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t total = (uint64_t) a.n_rp * a.nkb;
    const uint64_t lo = (uint64_t) blockIdx.x * total / gridDim.x;
    const uint64_t hi = (uint64_t) (blockIdx.x + 1) * total / gridDim.x;
    const u32 b_bytes = a.BN * KB * 2;
    const u32 off_gl = A_BYTES;
    const u32 off_xh = a.mode == LTRG_REFINE_FULL ? 2 * A_BYTES : A_BYTES;
    const u32 off_xl = off_xh + b_bytes;
    const u32 tx_bytes = (a.mode == LTRG_REFINE_FULL ? 2 : 1) * A_BYTES + (a.mode >= LTRG_REFINE_RHS ? 2 : 1) * b_bytes;

    if (threadIdx.x == 0) {
        for (u32 s = 0; s < a.stages; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(accf, 1);
        mbar_init(acce, 4);
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // producer: stage counter i runs over the units' stages
            uint64_t i = 0;
            bool ok = true;
            for (uint64_t u = a.issue ? lo : hi; u < hi && ok; ++u) {
                for (int q = 0; q < SPU; ++q, ++i) {
                    const u32 s = (u32) (i % a.stages);
                    if (i >= a.stages &&
                        !mbar_wait(&empty[s], (u32) ((i / a.stages) - 1) & 1u, a.err, kErrProducer, a.wait_cycles)) {
                        ok = false;
                        break;
                    }
                    const int kx = (int) ((u % a.nkb) * BK + q * KB), ry = (int) ((u / a.nkb) * ROWS);
                    unsigned char* st = base + (size_t) s * a.stage_bytes;
                    mbar_expect_tx(&full[s], tx_bytes);
                    tma_load_2d(st, &tmG, &full[s], kx, ry);
                    if (a.mode == LTRG_REFINE_FULL) tma_load_2d(st + off_gl, &tmGl, &full[s], kx, ry);
                    tma_load_2d(st + off_xh, &tmXh, &full[s], kx, 0);
                    if (a.mode >= LTRG_REFINE_RHS) tma_load_2d(st + off_xl, &tmXl, &full[s], kx, 0);
                }
            }
            // wait for the copies still in flight (complete already unless a wait above expired)
            const uint64_t issued = i;
            for (uint64_t j = issued > a.stages ? issued - a.stages : 0; j < issued; ++j)
                if (!mbar_wait(&full[j % a.stages], (u32) (j / a.stages) & 1u, a.err, kErrDrain, a.wait_cycles)) break;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            uint64_t i = 0;
            u32 seg = 0;
            bool ok = true;
            for (uint64_t u = lo; u < hi && ok; ++u) {
                const u32 kb = (u32) (u % a.nkb);
                const bool first = u == lo || kb == 0 || (a.kchunk && kb % a.kchunk == 0);
                const bool last = u + 1 == hi || kb + 1 == a.nkb || (a.kchunk && (kb + 1) % a.kchunk == 0);
                if (first && seg > 0 && !mbar_wait(acce, (seg - 1) & 1u, a.err, kErrMma, a.wait_cycles)) break;
                for (int q = 0; q < SPU; ++q, ++i) {
                    const u32 s = (u32) (i % a.stages);
                    if (!mbar_wait(&full[s], (u32) (i / a.stages) & 1u, a.err, kErrMma, a.wait_cycles)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t st = saddr(base + (size_t) s * a.stage_bytes);
                    for (int k = 0; k < KB / UK; ++k) {
                        const uint64_t bh = sdesc<KB>(st + off_xh + k * UK * 2);
                        const uint64_t bl = sdesc<KB>(st + off_xl + k * UK * 2);
                        for (int h = 0; h < 2; ++h) {
                            const uint32_t d = tmem + h * 256;
                            const uint32_t ao = h * (BM * KB * 2) + k * UK * 2;
                            const uint64_t ad = sdesc<KB>(st + ao);
                            umma(d, ad, bh, a.idesc, (first && q == 0 && k == 0) ? 0u : 1u);
                            if (a.mode >= LTRG_REFINE_RHS) umma(d, ad, bl, a.idesc, 1u);
                            if (a.mode == LTRG_REFINE_FULL) umma(d, sdesc<KB>(st + off_gl + ao), bh, a.idesc, 1u);
                        }
                    }
                    umma_commit(&empty[s]);
                }
                if (ok && last) { umma_commit(accf); ++seg; }
            }
            umma_commit(done);
            mbar_wait(done, 0, a.err, kErrDrain, a.wait_cycles);
        }
    } else {
        // epilogue: TMEM lanes of quadrant q = rows 32q .. 32q+31 of each 128-row half
        const int q = warp & 3;
        // Segments (the MMA issuer's accumulations) in the same order: maximal runs of
        // units within one row block and, when kchunk > 0, within one k chunk. The
        // first segment of a row block writes its workspace slot, later ones add to it.
        uint64_t u = lo;
        for (u32 seg = 0; u < hi; ++seg) {
            const u32 rp = (u32) (u / a.nkb), kb = (u32) (u % a.nkb);
            const u32 kend = a.kchunk ? min(a.nkb, (kb / a.kchunk + 1) * a.kchunk) : a.nkb;
            const bool fresh = u == lo || kb == 0;
            u = min(hi, (uint64_t) rp * a.nkb + kend);
            // every lane waits; the warp goes on only if all of them saw the phase, so the
            // .sync.aligned loads below always run converged
            const bool ok = mbar_wait(accf, seg & 1u, a.err, kErrEpilogue, a.wait_cycles);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
            const u32 slot = blockIdx.x - __ldg(&a.rp_first[rp]);
            float* P = a.partial + ((size_t) rp * a.max_slots + slot) * a.R * ROWS;
            for (int h = 0; h < 2; ++h) {
                const u32 row = h * BM + q * 32 + lane;
                for (u32 c0 = 0; c0 < a.BN; c0 += 32) {
                    uint32_t v[32];
                    tmem_ld32(tmem + ((uint32_t) (q * 32) << 16) + h * 256 + c0, v);
                    float* d = P + (size_t) c0 * ROWS + row;
                    if (!fresh) {   // all loads first, then all stores: one round trip per 32 columns
                        float prev[32];
#pragma unroll
                        for (int c = 0; c < 32; ++c) prev[c] = c0 + c < a.R ? d[(size_t) c * ROWS] : 0.0f;
#pragma unroll
                        for (int c = 0; c < 32; ++c) v[c] = __float_as_uint(__uint_as_float(v[c]) + prev[c]);
                    }
#pragma unroll
                    for (int c = 0; c < 32; ++c)
                        if (c0 + c < a.R) d[(size_t) c * ROWS] = __uint_as_float(v[c]);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ----------------------------------------------------------------------------- combine

template <class T> __device__ __forceinline__ T to16(float f);
template <> __device__ __forceinline__ __half to16<__half>(float f) { return __float2half_rn(f); }
template <> __device__ __forceinline__ __nv_bfloat16 to16<__nv_bfloat16>(float f) { return __float2bfloat16_rn(f); }
__device__ __forceinline__ float from16(__half h) { return __half2float(h); }
__device__ __forceinline__ float from16(__nv_bfloat16 h) { return __bfloat162float(h); }

// Exponent of the power-of-two scale of X: the largest emission maps below
// 2^9, which leaves room for the bounced light to grow 100x and keeps small
// values out of the FP16 subnormal range.
__device__ __forceinline__ int x_scale_exp(const u32* emax_bits)
{
    const float emax = __uint_as_float(*emax_bits);
    if (!(emax > 0.0f) || !(emax < 3.0e38f)) return 0;
    int p;
    frexpf(emax, &p);
    return 9 - p;
}

// One 32 (patches) x 32 (right-hand sides) tile:
//   B[j][r] = E[j][r] + 2^-(g_exp + x_exp) * sum over the row block's slots of
//             the partials (slot order)
//   X^T[r][j] = head (+ tail) of 2^x_exp * albedo_j(r mod 3) * B[j][r], zero for
//             j >= n or r >= R
// The G operand holds 2^g_exp G, the X operand 2^x_exp X (exact scalings).
// B_out and xh may be null (not wanted); partial null means B = E.
template <class T>
__global__ void __launch_bounds__(256) k_combine(u32 n, u32 ld, u32 R, u32 Rpad, const float* __restrict__ partial,
                                                 u32 max_slots, const u32* __restrict__ rp_cnt,
                                                 const float* __restrict__ E, const float* __restrict__ albedo,
                                                 float* __restrict__ B_out, T* __restrict__ xh, T* __restrict__ xl,
                                                 int g_exp, const u32* __restrict__ emax_bits)
{
    __shared__ float tile[32][33];
    const u32 j0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x_exp = x_scale_exp(emax_bits);
    const float unscale = ldexpf(1.0f, -(g_exp + x_exp)), xscale = ldexpf(1.0f, x_exp);
    // the loads of the second phase (E, albedo) go out together with those of the first,
    // so a block waits for about one memory round trip instead of three
    float e[4], al[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {   // tx along r
        const u32 j = j0 + ty + 8 * i, r = r0 + tx;
        const bool in = j < n && r < R;
        e[i] = in ? __ldg(&E[(size_t) j * R + r]) : 0.0f;
        al[i] = in ? __ldg(&albedo[3 * j + r % 3]) : 0.0f;
    }
    // the 32 patches of a tile lie in one 256-row block (j0 is a multiple of 32)
    const u32 rp = j0 / ROWS, cnt = (partial && j0 < n) ? __ldg(&rp_cnt[rp]) : 0u;
    float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (u32 s = 0; s < cnt; ++s) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {   // tx along j
            const u32 r = r0 + ty + 8 * i, j = j0 + tx;
            if (j < n && r < R) v[i] += __ldg(&partial[(((size_t) rp * max_slots + s) * R + r) * ROWS + (j % ROWS)]);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) tile[ty + 8 * i][tx] = v[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {   // tx along r
        const int k = ty + 8 * i;
        const u32 j = j0 + k, r = r0 + tx;
        float x = 0.0f;
        if (j < n && r < R) {
            const float b = e[i] + tile[tx][k] * unscale;
            if (B_out) B_out[(size_t) j * R + r] = b;
            x = al[i] * b * xscale;
        }
        tile[tx][k] = x;
    }
    __syncthreads();
    if (!xh) return;
    for (int k = ty; k < 32; k += 8) {   // tx along j
        const u32 r = r0 + k, j = j0 + tx;
        if (r < Rpad && j < ld) {
            const float v = tile[k][tx];
            const T h = to16<T>(v);
            xh[(size_t) r * ld + j] = h;
            if (xl) xl[(size_t) r * ld + j] = to16<T>(v - from16(h));
        }
    }
}

// ----------------------------------------------------------------------------- FP32 SIMT gather

// B_new = E + G X, G (n x n FP32), X (n x R FP32, row-major): 128 x 192 tile
// per block, 16 x 16 threads with 8 x 12 outputs each, k tiles of 16 in two
// shared-memory buffers (one barrier per tile); the next tile's global loads
// are in flight in registers while the current tile is consumed.
constexpr int SBM = 128, SBN = 192, SBK = 16;
__global__ void __launch_bounds__(256) k_sgemm_bounce(u32 n, u32 R, const float* __restrict__ G,
                                                      const float* __restrict__ X, const float* __restrict__ E,
                                                      float* __restrict__ Bnew)
{
    __shared__ __align__(16) float As[2][SBK][SBM + 4];
    __shared__ __align__(16) float Bs[2][SBK][SBN];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const u32 m0 = blockIdx.x * SBM, n0 = blockIdx.y * SBN;
    // loader coordinates: A 128 rows x 16 k (row ar, k ak..ak+7); B 16 k x 192 (k bk, cols bc..bc+11)
    const int ar = tid >> 1, ak = (tid & 1) * 8, bk = tid >> 4, bc = (tid & 15) * 12;
    float pa[8], pb[12];
    auto fetch = [&](u32 k0) {
        const u32 gi = m0 + ar;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const u32 gk = k0 + ak + t;
            pa[t] = (gi < n && gk < n) ? __ldg(&G[(size_t) gi * n + gk]) : 0.0f;
        }
        const u32 gk = k0 + bk;
#pragma unroll
        for (int t = 0; t < 12; ++t) {
            const u32 gc = n0 + bc + t;
            pb[t] = (gk < n && gc < R) ? __ldg(&X[(size_t) gk * R + gc]) : 0.0f;
        }
    };
    auto stash = [&](int buf) {
#pragma unroll
        for (int t = 0; t < 8; ++t) As[buf][ak + t][ar] = pa[t];
#pragma unroll
        for (int t = 0; t < 12; ++t) Bs[buf][bk][bc + t] = pb[t];
    };
    float acc[8][12];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 12; ++j) acc[i][j] = 0.0f;
    fetch(0);
    stash(0);
    __syncthreads();
    int cur = 0;
    for (u32 k0 = 0; k0 < n; k0 += SBK) {
        const bool more = k0 + SBK < n;
        if (more) fetch(k0 + SBK);
#pragma unroll
        for (int k = 0; k < SBK; ++k) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 8]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 8 + 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 12]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 12 + 4]);
            const float4 b2 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 12 + 8]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[12] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w, b2.x, b2.y, b2.z, b2.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 12; ++j) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
        }
        if (more) stash(cur ^ 1);
        __syncthreads();
        cur ^= 1;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const u32 gi = m0 + ty * 8 + i;
        if (gi >= n) continue;
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            const u32 gc = n0 + tx * 12 + j;
            if (gc < R) {
                const size_t o = (size_t) gi * R + gc;
                Bnew[o] = E[o] + acc[i][j];
            }
        }
    }
}

// X_j(r) = albedo_j(r mod 3) B_j(r), FP32 row-major.
__global__ void k_make_x32(u32 n, u32 R, const float* __restrict__ albedo, const float* __restrict__ B,
                           float* __restrict__ X)
{
    const size_t t = blockIdx.x * (size_t) blockDim.x + threadIdx.x;
    if (t >= (size_t) n * R) return;
    const u32 j = (u32) (t / R), r = (u32) (t % R);
    X[t] = albedo[3 * j + r % 3] * B[t];
}

// ----------------------------------------------------------------------------- G preparation

// G_ij = F_ij * area_j, in place.
__global__ void k_scale_cols(u32 n, float* __restrict__ G, const float* __restrict__ area)
{
    const size_t t = blockIdx.x * (size_t) blockDim.x + threadIdx.x;
    if (t >= (size_t) n * n) return;
    G[t] *= area[t % n];
}

// *out = max |x| as float bits (non-negative floats order like their bits); *out starts at 0.
__global__ void k_absmax(const float* __restrict__ x, size_t count, u32* out)
{
    float m = 0.0f;
    for (size_t t = blockIdx.x * (size_t) blockDim.x + threadIdx.x; t < count; t += (size_t) gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[t]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// hi = 16-bit 2^g_exp G (row stride ld, zero columns j >= n); lo = 16-bit residual when requested.
template <class T>
__global__ void k_g_to_16(u32 n, u32 ld, const float* __restrict__ G, T* __restrict__ hi, T* __restrict__ lo,
                          float gscale)
{
    const size_t t = blockIdx.x * (size_t) blockDim.x + threadIdx.x;
    if (t >= (size_t) n * ld) return;
    const u32 i = (u32) (t / ld), j = (u32) (t % ld);
    const float g = j < n ? G[(size_t) i * n + j] * gscale : 0.0f;
    const T h = to16<T>(g);
    hi[t] = h;
    if (lo) lo[t] = to16<T>(g - from16(h));
}

// ----------------------------------------------------------------------------- host helpers

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000) p;
    });
    if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

// 2-D map over `rows` rows of `ld` 16-bit elements (row stride ld * 2 bytes,
// a multiple of 128), box of 64 elements (128 bytes) x box_rows, 128-byte
// swizzle; rows past the end read as zero.
CUtensorMap make_map(const void* ptr, CUtensorMapDataType dt, u32 ld, u32 rows, u32 box_rows, u32 box_k)
{
    if ((reinterpret_cast<uintptr_t>(ptr) & 127) || (ld % BK) || box_rows == 0 || box_rows > 256 ||
        (box_k != 64 && box_k != 32))
        throw std::runtime_error("tensor map: misaligned base, row length or box");
    CUtensorMap m;
    cuuint64_t dims[2] = {ld, rows};
    cuuint64_t strides[1] = {(cuuint64_t) ld * 2};
    cuuint32_t box[2] = {(cuuint32_t) box_k, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(&m, dt, 2, const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             box_k == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed with " + std::to_string((int) r));
    return m;
}

// k per pipeline stage of the tensor-core gather for a refine level. Measured
// on GB300 (32,768 patches, R = 192): 64 for one and two products (0.388 and
// 0.606 ms per contraction against 0.463 and 0.652 with 32); 32 for three
// products, whose stages hold two G tiles and two X tiles (0.719 against
// 0.738 ms; it also lets that mode take R = 256).
u32 stage_k(int refine) { return refine == LTRG_REFINE_FULL ? 32u : 64u; }

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t b)
    {
        if (b <= bytes) return;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        GCK(cudaMalloc(&p, b));
        bytes = b;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Page-locked host buffer kept by a gather (grown, never shrunk).
struct PinBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t b)
    {
        if (b <= bytes) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        GCK(cudaHostAlloc(&p, b, cudaHostAllocPortable));
        bytes = b;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

// Copy of `n` floats by the GPU where the host's pageable memory is directly
// addressable by kernels (cudaDevAttrPageableMemoryAccess, e.g. Grace systems:
// the GPU walks the host page tables over the CPU-GPU link): one of src and
// dst is the caller's pageable host buffer. 16-byte vectors when both are
// aligned, single floats otherwise.
__global__ void k_copy_floats(float* __restrict__ dst, const float* __restrict__ src, size_t n)
{
    const size_t stride = (size_t) gridDim.x * blockDim.x;
    const size_t t0 = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0) {
        const size_t n4 = n / 4;
        float4* d4 = reinterpret_cast<float4*>(dst);
        const float4* s4 = reinterpret_cast<const float4*>(src);
        for (size_t i = t0; i < n4; i += stride) d4[i] = s4[i];
        for (size_t i = 4 * n4 + t0; i < n; i += stride) dst[i] = src[i];
    } else {
        for (size_t i = t0; i < n; i += stride) dst[i] = src[i];
    }
}

// Whether kernels on `device` may address pageable host memory (queried once).
bool pageable_access(int device)
{
    static std::mutex mu;
    static int known[64] = {};   // 0 unknown, 1 no, 2 yes
    if (device < 0 || device >= 64) return false;
    std::lock_guard<std::mutex> lk(mu);
    if (!known[device]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) v = 0;
        known[device] = v ? 2 : 1;
    }
    return known[device] == 2;
}

// Host threads kept by a gather for its host-buffer copies: run(k, f) calls
// f(0 .. k-1) on the workers (and the caller) and returns when all are done.
struct StagePool {
    std::vector<std::thread> th;
    std::mutex mu;
    std::condition_variable cv_go, cv_done;
    std::function<void(int)> job;
    int n_job = 0, next = 0, done = 0;
    unsigned long long gen = 0;
    bool quit = false;

    void start(int workers)
    {
        for (int w = 0; w < workers; ++w)
            th.emplace_back([this]() {
                unsigned long long seen = 0;
                std::unique_lock<std::mutex> lk(mu);
                for (;;) {
                    cv_go.wait(lk, [&] { return quit || gen != seen; });
                    if (quit) return;
                    seen = gen;
                    drain(lk);
                }
            });
    }
    // takes items until none are left; called with the lock held
    void drain(std::unique_lock<std::mutex>& lk)
    {
        while (next < n_job) {
            const int t = next++;
            lk.unlock();
            job(t);
            lk.lock();
            if (++done == n_job) cv_done.notify_all();
        }
    }
    void run(int k, std::function<void(int)> f)
    {
        std::unique_lock<std::mutex> lk(mu);
        job = std::move(f);
        n_job = k;
        next = done = 0;
        ++gen;
        cv_go.notify_all();
        drain(lk);
        cv_done.wait(lk, [&] { return done == n_job; });
    }
    ~StagePool()
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            quit = true;
        }
        cv_go.notify_all();
        for (auto& t : th) t.join();
    }
};

// Host <-> device copies of the host-buffer entry point through kept
// page-locked buffers. A copy straight from the caller's pageable memory runs
// at about 10 GB/s; here the bytes are cut into slices, the pool's threads
// copy the slices into the page-locked buffer and each queues its slice's
// DMA at once, so the DMA of early slices overlaps the host copies of later
// ones (and the reverse for the result: each slice's DMA is followed by an
// event its thread waits on before copying the slice out).
constexpr size_t kStageMinSlice = 1 << 20;

int stage_slices(size_t bytes, int threads)
{
    return (int) std::max<size_t>(1, std::min<size_t>((size_t) threads, bytes / kStageMinSlice));
}

void stage_h2d(void* dev, const void* host, size_t bytes, PinBuf& pin, cudaStream_t s, StagePool& pool, int threads)
{
    if (!bytes) return;
    pin.ensure(bytes);
    const int k = stage_slices(bytes, threads);
    const size_t step = (bytes / k + 255) / 256 * 256;
    std::vector<cudaError_t> rc(k, cudaSuccess);
    pool.run(k, [&](int t) {
        const size_t a = std::min(bytes, t * step), b = std::min(bytes, a + step);
        if (a >= b) return;
        memcpy((char*) pin.p + a, (const char*) host + a, b - a);
        rc[t] = cudaMemcpyAsync((char*) dev + a, (char*) pin.p + a, b - a, cudaMemcpyHostToDevice, s);
    });
    for (cudaError_t e : rc) GCK(e);
}

void stage_d2h(void* host, const void* dev, size_t bytes, PinBuf& pin, cudaStream_t s, StagePool& pool, int threads)
{
    if (!bytes) return;
    pin.ensure(bytes);
    const int k = stage_slices(bytes, threads);
    const size_t step = (bytes / k + 255) / 256 * 256;
    std::vector<cudaEvent_t> ev(k, nullptr);
    for (int t = 0; t < k; ++t) {
        const size_t a = std::min(bytes, t * step), b = std::min(bytes, a + step);
        GCK(cudaEventCreateWithFlags(&ev[t], cudaEventDisableTiming));
        if (a < b) GCK(cudaMemcpyAsync((char*) pin.p + a, (const char*) dev + a, b - a, cudaMemcpyDeviceToHost, s));
        GCK(cudaEventRecord(ev[t], s));
    }
    std::vector<cudaError_t> rc(k, cudaSuccess);
    pool.run(k, [&](int t) {
        const size_t a = std::min(bytes, t * step), b = std::min(bytes, a + step);
        rc[t] = cudaEventSynchronize(ev[t]);
        if (rc[t] == cudaSuccess && a < b) memcpy((char*) host + a, (const char*) pin.p + a, b - a);
    });
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    for (cudaError_t e : rc) GCK(e);
}

}  // namespace
}  // namespace lg

using namespace lg;

struct ltrg_Gather {
    int device = 0;
    int sm_count = 0;
    cudaStream_t st = nullptr;
    u32 n = 0, ld = 0;
    DevBuf G32;                   // n x n FP32
    DevBuf G16, G16lo;            // n x ld 16-bit head and residual
    int g16_kind = -1;            // precision held in G16 (-1: none)
    int g_exp = 0;                // G16 holds 2^g_exp G: max |G| maps below 2^14
    bool g16_has_lo = false;
    // stream-K schedule of the tcgen05 kernel (fixed by n and the SM count)
    u32 n_rp = 0, nkb = 0, n_cta = 0, max_slots = 0;
    u32 kchunk = 0;               // k blocks per TMEM accumulation (0: whole range of a CTA)
    DevBuf rp_tab;                // rp_first[n_rp], rp_cnt[n_rp]
    // solve scratch
    DevBuf partial, xh, xl, x32, btmp, err, emax;
    DevBuf h_alb, h_E, h_out;     // device copies for the host-buffer entry point
    PinBuf pin_in, pin_out;       // its page-locked staging
    std::unique_ptr<StagePool> pool;   // its host copy threads (started by the first host-buffer solve)
    int pool_threads = 0;
    uint64_t links = 0, vis_rays = 0, pairs = 0;
    double ms_build = 0;
    u32 stall_us = 0;             // ltrdbg_GatherStallNextSolve
    int host_path = 0;            // ltrdbg_GatherHostPath: 0 by device, 1 staged, 2 direct
    std::string error;
    std::mutex mu;

    ~ltrg_Gather()
    {
        if (!st) return;
        cudaSetDevice(device);
        cudaStreamSynchronize(st);
        DevBuf* all[] = {&G32,  &G16, &G16lo, &rp_tab, &partial, &xh,    &xl,
                         &x32,  &btmp, &err,  &emax,   &h_alb,   &h_E,   &h_out};
        for (DevBuf* b : all) b->release();
        pin_in.release();
        pin_out.release();
        cudaStreamDestroy(st);
    }

    void schedule()
    {
        n_rp = (n + ROWS - 1) / ROWS;
        nkb = ld / BK;
        const uint64_t total = (uint64_t) n_rp * nkb;
        n_cta = (u32) std::min<uint64_t>((uint64_t) sm_count, total);
        std::vector<u32> first(n_rp, UINT32_MAX), cnt(n_rp, 0);
        for (u32 c = 0; c < n_cta; ++c) {
            const uint64_t lo = (uint64_t) c * total / n_cta, hi = (uint64_t) (c + 1) * total / n_cta;
            if (hi <= lo) continue;
            for (uint64_t rp = lo / nkb; rp <= (hi - 1) / nkb; ++rp) {
                if (first[rp] == UINT32_MAX) first[rp] = c;
                cnt[rp] = c - first[rp] + 1;
            }
        }
        max_slots = 0;
        for (u32 rp = 0; rp < n_rp; ++rp) max_slots = std::max(max_slots, cnt[rp]);
        std::vector<u32> tab(first);
        tab.insert(tab.end(), cnt.begin(), cnt.end());
        rp_tab.ensure(tab.size() * 4);
        GCK(cudaMemcpy(rp_tab.p, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
    }

    // B for R right-hand sides; all pointers on this device, enqueued on `s`.
    void solve(const float* alb, const float* E, u32 R, int bounces, int precision, int refine, float* out,
               ltrg_GatherStats* stats, cudaStream_t s);
};

void ltrg_Gather::solve(const float* alb, const float* E, u32 R, int bounces, int precision, int refine, float* out,
                        ltrg_GatherStats* stats, cudaStream_t s)
{
    const bool tc = precision != LTRG_F_FP32;
    if (tc && R > (u32) MAX_BN) throw std::runtime_error("tensor-core gather takes at most 256 right-hand sides");
    if (refine < LTRG_REFINE_NONE || refine > LTRG_REFINE_FULL) throw std::runtime_error("invalid refine level");
    err.ensure(4);
    GCK(cudaMemsetAsync(err.p, 0, 4, s));
    std::vector<cudaEvent_t> ev;
    auto event = [&]() {
        cudaEvent_t e;
        GCK(cudaEventCreate(&e));
        ev.push_back(e);
        GCK(cudaEventRecord(e, s));
        return e;
    };
    struct EvGuard {
        std::vector<cudaEvent_t>& v;
        ~EvGuard() { for (cudaEvent_t e : v) cudaEventDestroy(e); }
    } evg{ev};
    double ms_convert = 0, ms_gemm = 0, ms_bounces = 0;
    int stages = 0, products = 1;
    uint64_t bytes_bounce = 0;

    if (!tc) {
        // FP32: ping-pong between btmp and out so the last bounce lands in out
        btmp.ensure((size_t) n * R * 4);
        x32.ensure((size_t) n * R * 4);
        float* cur = (bounces % 2 == 0) ? out : btmp.as<float>();
        float* nxt = (bounces % 2 == 0) ? btmp.as<float>() : out;
        GCK(cudaMemcpyAsync(cur, E, (size_t) n * R * 4, cudaMemcpyDeviceToDevice, s));
        cudaEvent_t e0 = event();
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ge;
        for (int b = 0; b < bounces; ++b) {
            const size_t tot = (size_t) n * R;
            k_make_x32<<<(unsigned) ((tot + 255) / 256), 256, 0, s>>>(n, R, alb, cur, x32.as<float>()); note_launch();
            cudaEvent_t g0 = event();
            dim3 grid((n + SBM - 1) / SBM, (R + SBN - 1) / SBN);
            k_sgemm_bounce<<<grid, 256, 0, s>>>(n, R, G32.as<float>(), x32.as<float>(), E, nxt); note_launch();
            cudaEvent_t g1 = event();
            ge.push_back({g0, g1});
            GCK(cudaGetLastError());
            std::swap(cur, nxt);
        }
        cudaEvent_t e1 = event();
        GCK(cudaStreamSynchronize(s));
        float m = 0;
        cudaEventElapsedTime(&m, e0, e1);
        ms_bounces = m;
        for (auto& p : ge) { cudaEventElapsedTime(&m, p.first, p.second); ms_gemm += m; }
        bytes_bounce = (uint64_t) n * n * 4;
    } else {
        const bool need_lo = refine == LTRG_REFINE_FULL;
        if (g16_kind != precision || (need_lo && !g16_has_lo)) {
            cudaEvent_t c0 = event();
            G16.ensure((size_t) n * ld * 2);
            if (need_lo) G16lo.ensure((size_t) n * ld * 2);
            const size_t tot = (size_t) n * ld;
            const unsigned grid = (unsigned) ((tot + 255) / 256);
            const float gscale = ldexpf(1.0f, g_exp);
            if (precision == LTRG_F_FP16)
                k_g_to_16<__half><<<grid, 256, 0, s>>>(n, ld, G32.as<float>(), G16.as<__half>(),
                                                       need_lo ? G16lo.as<__half>() : nullptr, gscale);
            else
                k_g_to_16<__nv_bfloat16><<<grid, 256, 0, s>>>(n, ld, G32.as<float>(), G16.as<__nv_bfloat16>(),
                                                              need_lo ? G16lo.as<__nv_bfloat16>() : nullptr, gscale);
            note_launch();
            GCK(cudaGetLastError());
            cudaEvent_t c1 = event();
            GCK(cudaEventSynchronize(c1));
            float m = 0;
            cudaEventElapsedTime(&m, c0, c1);
            ms_convert = m;
            g16_kind = precision;
            g16_has_lo = need_lo;
        }
        const u32 BN = std::max<u32>(32, (R + 31) / 32 * 32);
        const u32 KB = stage_k(refine);
        const u32 b_bytes = BN * KB * 2, a_bytes = ROWS * KB * 2;
        const u32 stage_bytes = (need_lo ? 2 : 1) * a_bytes + (refine >= LTRG_REFINE_RHS ? 2 : 1) * b_bytes;
        stages = std::min<int>(kMaxStages, (kSmemLimit - kSmemExtra) / (int) stage_bytes);
        if (stages < 2) throw std::runtime_error("tensor-core gather: stage does not fit in shared memory");
        const size_t smem = (size_t) stages * stage_bytes + kSmemExtra;
        products = 1 + (refine >= LTRG_REFINE_RHS) + (refine == LTRG_REFINE_FULL);
        // every element of X^T (padding included) is written by the first k_combine
        xh.ensure((size_t) BN * ld * 2);
        xl.ensure((size_t) BN * ld * 2);
        partial.ensure((size_t) n_rp * max_slots * R * ROWS * 4);
        const CUtensorMapDataType dt =
            precision == LTRG_F_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
        const CUtensorMap mG = make_map(G16.p, dt, ld, n, ROWS, KB);
        const CUtensorMap mGl = make_map(need_lo ? G16lo.p : G16.p, dt, ld, n, ROWS, KB);
        const CUtensorMap mXh = make_map(xh.p, dt, ld, BN, BN, KB);
        const CUtensorMap mXl = make_map(xl.p, dt, ld, BN, BN, KB);
        auto kern = KB == 64 ? k_umma_gather<64> : k_umma_gather<32>;
        GCK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
        UmmaArgs ua;
        ua.nkb = nkb; ua.n_rp = n_rp; ua.R = R; ua.BN = BN;
        ua.stages = (u32) stages; ua.stage_bytes = stage_bytes; ua.mode = (u32) refine;
        ua.idesc = idesc_f16(precision == LTRG_F_BF16 ? 1u : 0u, BN);
        ua.max_slots = max_slots;
        ua.kchunk = kchunk;
        ua.rp_first = rp_tab.as<u32>();
        ua.partial = partial.as<float>();
        ua.err = err.as<u32>();
        ua.wait_cycles = kWaitCycles;
        ua.issue = 1;
        if (stall_us) {   // test hook: copies never issued, waits cut short
            ua.issue = 0;
            ua.wait_cycles = (unsigned long long) stall_us * 2000ull;
            stall_us = 0;
        }
        const u32* rp_cnt = rp_tab.as<u32>() + n_rp;
        emax.ensure(4);
        GCK(cudaMemsetAsync(emax.p, 0, 4, s));
        k_absmax<<<std::max<u32>(1, std::min<u32>(1024, (u32) (((size_t) n * R + 255) / 256))), 256, 0, s>>>(
            E, (size_t) n * R, emax.as<u32>()); note_launch();
        dim3 cb(32, 8), cg((ld + 31) / 32, (BN + 31) / 32);
        auto combine = [&](bool with_partial, bool last) {
            float* bo = last ? out : nullptr;
            const float* P = with_partial ? partial.as<float>() : nullptr;
            if (precision == LTRG_F_FP16)
                k_combine<__half><<<cg, cb, 0, s>>>(n, ld, R, BN, P, max_slots, rp_cnt, E, alb, bo,
                                                    last ? nullptr : xh.as<__half>(),
                                                    (last || refine == LTRG_REFINE_NONE) ? nullptr : xl.as<__half>(),
                                                    g_exp, emax.as<u32>());
            else
                k_combine<__nv_bfloat16><<<cg, cb, 0, s>>>(
                    n, ld, R, BN, P, max_slots, rp_cnt, E, alb, bo, last ? nullptr : xh.as<__nv_bfloat16>(),
                    (last || refine == LTRG_REFINE_NONE) ? nullptr : xl.as<__nv_bfloat16>(), g_exp, emax.as<u32>());
            note_launch();
        };
        cudaEvent_t e0 = event();
        combine(false, bounces == 0);
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ge;
        for (int b = 0; b < bounces; ++b) {
            cudaEvent_t g0 = event();
            kern<<<n_cta, kThreads, smem, s>>>(mG, mGl, mXh, mXl, ua); note_launch();
            cudaEvent_t g1 = event();
            ge.push_back({g0, g1});
            GCK(cudaGetLastError());
            combine(true, b + 1 == bounces);
        }
        cudaEvent_t e1 = event();
        GCK(cudaStreamSynchronize(s));
        u32 herr = 0;
        GCK(cudaMemcpy(&herr, err.p, 4, cudaMemcpyDeviceToHost));
        if (herr)
            throw std::runtime_error("tensor-core gather: a pipeline wait expired (error word " + std::to_string(herr) +
                                     ")");
        float m = 0;
        cudaEventElapsedTime(&m, e0, e1);
        ms_bounces = m;
        for (auto& p : ge) { cudaEventElapsedTime(&m, p.first, p.second); ms_gemm += m; }
        bytes_bounce = (uint64_t) n * ld * 2 * (need_lo ? 2 : 1);
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->ms_build = ms_build;
        stats->ms_convert = ms_convert;
        stats->ms_bounces = ms_bounces;
        stats->ms_per_bounce = bounces ? ms_bounces / bounces : 0;
        stats->ms_gemm = ms_gemm;
        stats->flops_per_bounce = 2.0 * n * (double) n * R * products;
        stats->bytes_per_bounce = bytes_bounce;
        stats->links = links;
        stats->vis_rays = vis_rays;
        stats->pairs = pairs;
        stats->tensor_cores = tc ? 1 : 0;
        stats->stages = stages;
        stats->ctas = tc ? (int32_t) n_cta : (int32_t) (((n + SBM - 1) / SBM) * ((R + SBN - 1) / SBN));
        stats->products = tc ? products : 1;
    }
}

extern "C" {

LTRAPI ltrg_Gather* ltrg_GatherCreate(const float* tri_xyz, u32 n_tris, const float* pos3, const float* nrm3,
                                      const float* area, u32 n, int links, int device)
{
    ltrg_Gather* g = new ltrg_Gather;
    try {
        if (!pos3 || !nrm3 || !area || n == 0 || (n_tris && !tri_xyz)) throw std::runtime_error("invalid arguments");
        if (links != LTRG_LINKS_REFERENCE && links != LTRG_LINKS_VISIBLE) throw std::runtime_error("invalid link predicate");
        if (n > 65535u * 32u) throw std::runtime_error("too many patches");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw std::runtime_error("no CUDA device available");
        if (device < 0 || device >= ndev) throw std::runtime_error("device out of range");
        g->device = device;
        GCK(cudaSetDevice(device));
        GCK(cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, device));
        GCK(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
        g->n = n;
        g->ld = (n + BK - 1) / BK * BK;
        cudaStream_t st = g->st;

        // occluder BVH (one instance, every triangle casts shadows)
        std::vector<float> xyz(tri_xyz, tri_xyz + 9 * (size_t) n_tris);
        std::vector<u32> meta(n_tris, kOccluderBit), local(n_tris);
        for (u32 i = 0; i < n_tris; ++i) local[i] = i;
        std::vector<u32> ref_tri;
        std::vector<float> ref_box;
        float cmin[3], cmax[3];
        build_refs_host(xyz, ref_tri, ref_box, cmin, cmax);
        std::vector<void*> tmp;
        struct TmpGuard {
            std::vector<void*>& v; cudaStream_t s;
            ~TmpGuard() { for (void* p : v) cudaFreeAsync(p, s); cudaStreamSynchronize(s); }
        } tg{tmp, st};
        auto up = [&](const void* h, size_t b) {
            void* d = nullptr;
            GCK(cudaMallocAsync(&d, b ? b : 16, st));
            tmp.push_back(d);
            if (b) GCK(cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, st));
            return d;
        };
        BvhBuildInput bin;
        bin.tri_xyz = (const float*) up(xyz.data(), xyz.size() * 4);
        bin.tri_meta = (const u32*) up(meta.data(), meta.size() * 4);
        bin.tri_local = (const u32*) up(local.data(), local.size() * 4);
        bin.ref_tri = (const u32*) up(ref_tri.data(), ref_tri.size() * 4);
        bin.ref_box = (const float*) up(ref_box.data(), ref_box.size() * 4);
        bin.n = (int) ref_tri.size();
        for (int c = 0; c < 3; ++c) {
            bin.scene_min[c] = bin.n ? cmin[c] : 0;
            bin.scene_max[c] = bin.n ? cmax[c] : 0;
        }
        BvhStorage bvh;
        if (bin.n) bvh_build(bin, bvh, st);
        struct BvhGuard {
            BvhStorage& b; cudaStream_t s; bool on;
            ~BvhGuard() { if (on) bvh_free(b, s); }
        } bg{bvh, st, bin.n > 0};

        // patches: position, unit normal (normalised as the reference's samples are)
        std::vector<float4> hp(n), hn(n);
        for (u32 i = 0; i < n; ++i) {
            hp[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], 0.0f);
            V3 nn = normalized(mk(nrm3[3 * i], nrm3[3 * i + 1], nrm3[3 * i + 2]));
            hn[i] = make_float4(nn.x, nn.y, nn.z, 0.0f);
        }
        const float4* dp = (const float4*) up(hp.data(), n * sizeof(float4));
        const float4* dn = (const float4*) up(hn.data(), n * sizeof(float4));
        const float* da = (const float*) up(area, n * sizeof(float));
        u32* derr = (u32*) up(nullptr, 0);
        GCK(cudaMemsetAsync(derr, 0, 4, st));
        g->G32.ensure((size_t) n * n * 4);

        cudaEvent_t e0, e1;
        GCK(cudaEventCreate(&e0));
        GCK(cudaEventCreate(&e1));
        GCK(cudaEventRecord(e0, st));
        BvhView view = bin.n ? bvh.view() : BvhView{nullptr, nullptr, nullptr, nullptr, 0, 0};
        RadFormFactors ff = radiosity_form_factors_f32(n, dp, dn, view, ErrFlag{derr}, links, g->G32.as<float>(), st);
        const size_t nn2 = (size_t) n * n;
        k_scale_cols<<<(unsigned) ((nn2 + 255) / 256), 256, 0, st>>>(n, g->G32.as<float>(), da); note_launch();
        GCK(cudaGetLastError());
        GCK(cudaEventRecord(e1, st));
        u32* dgmax = (u32*) up(nullptr, 0);
        GCK(cudaMemsetAsync(dgmax, 0, 4, st));
        k_absmax<<<1024, 256, 0, st>>>(g->G32.as<float>(), nn2, dgmax); note_launch();
        u32 herr = 0, hgmax = 0;
        GCK(cudaMemcpyAsync(&hgmax, dgmax, 4, cudaMemcpyDeviceToHost, st));
        GCK(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st));
        GCK(cudaStreamSynchronize(st));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (herr) throw std::runtime_error("form-factor traversal error word " + std::to_string(herr));
        float gmax;
        memcpy(&gmax, &hgmax, 4);
        if (gmax > 0.0f && gmax < 3.0e38f) {
            int p;
            frexpf(gmax, &p);
            g->g_exp = 14 - p;
        }
        g->ms_build = ms;
        g->links = ff.links;
        g->vis_rays = ff.vis_rays;
        g->pairs = (uint64_t) n * (n - 1) / 2;
        g->schedule();
    } catch (const std::exception& e) {
        fprintf(stderr, "ltrg_GatherCreate: %s\n", e.what());
        delete g;
        return nullptr;
    }
    return g;
}

LTRAPI void ltrg_GatherDestroy(ltrg_Gather* g) { delete g; }

LTRAPI LTRBOOL ltrg_GatherSetChunk(ltrg_Gather* g, u32 k_blocks)
{
    if (!g) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    g->kchunk = k_blocks;
    return 1;
}

LTRAPI u32 ltrg_GatherSize(ltrg_Gather* g) { return g ? g->n : 0; }

LTRAPI LTRBOOL ltrg_GatherGetG(ltrg_Gather* g, float* out)
{
    if (!g || !out) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    if (cudaSetDevice(g->device) != cudaSuccess) return 0;
    if (cudaStreamSynchronize(g->st) != cudaSuccess) return 0;
    if (cudaMemcpy(out, g->G32.p, (size_t) g->n * g->n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    return 1;
}

LTRAPI const char* ltrg_GatherLastError(ltrg_Gather* g) { return g && !g->error.empty() ? g->error.c_str() : nullptr; }

LTRAPI LTRBOOL ltrdbg_GatherStallNextSolve(ltrg_Gather* g, u32 wait_us)
{
    if (!g || wait_us == 0 || wait_us > 2000000u) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    g->stall_us = wait_us;
    return 1;
}

LTRAPI LTRBOOL ltrdbg_GatherHostPath(ltrg_Gather* g, int mode)
{
    if (!g || mode < 0 || mode > 2) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    if (mode == 2 && !pageable_access(g->device)) return 0;
    g->host_path = mode;
    return 1;
}

LTRAPI int ltrdbg_GatherHostPathUsed(ltrg_Gather* g)
{
    if (!g) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    return g->host_path ? g->host_path : (pageable_access(g->device) ? 2 : 1);
}

LTRAPI LTRBOOL ltrg_GatherSolveDevice(ltrg_Gather* g, const float* albedo_rgb, const float* emission, u32 R,
                                      int bounces, int precision, int refine, float* out, ltrg_GatherStats* stats,
                                      void* stream)
{
    if (!g) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    g->error.clear();
    try {
        if (!albedo_rgb || !emission || !out || R == 0 || bounces < 0 || precision < LTRG_F_FP32 ||
            precision > LTRG_F_BF16)
            throw std::runtime_error("invalid arguments");
        GCK(cudaSetDevice(g->device));
        g->solve(albedo_rgb, emission, R, bounces, precision, refine, out, stats,
                 stream ? (cudaStream_t) stream : g->st);
    } catch (const std::exception& e) {
        g->error = e.what();
        cudaGetLastError();   // the error is reported here; none is left for the caller's next CUDA call
        return 0;
    }
    return 1;
}

LTRAPI LTRBOOL ltrg_GatherSolve(ltrg_Gather* g, const float* albedo_rgb, const float* emission, u32 R, int bounces,
                                int precision, int refine, float* out, ltrg_GatherStats* stats)
{
    if (!g) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    g->error.clear();
    try {
        if (!albedo_rgb || !emission || !out || R == 0 || bounces < 0 || precision < LTRG_F_FP32 ||
            precision > LTRG_F_BF16)
            throw std::runtime_error("invalid arguments");
        GCK(cudaSetDevice(g->device));
        const u32 n = g->n;
        cudaStream_t s = g->st;
        g->h_alb.ensure((size_t) n * 3 * 4);
        g->h_E.ensure((size_t) n * R * 4);
        g->h_out.ensure((size_t) n * R * 4);
        const bool direct = g->host_path ? g->host_path == 2 : pageable_access(g->device);
        const unsigned cgrid = (unsigned) g->sm_count * 8;
        if (direct) {
            // the GPU reads the caller's arrays over the CPU-GPU link: no host copies
            k_copy_floats<<<cgrid, 256, 0, s>>>(g->h_alb.as<float>(), albedo_rgb, (size_t) n * 3); note_launch();
            k_copy_floats<<<cgrid, 256, 0, s>>>(g->h_E.as<float>(), emission, (size_t) n * R); note_launch();
            GCK(cudaGetLastError());
        } else {
            GCK(cudaMemcpyAsync(g->h_alb.p, albedo_rgb, (size_t) n * 3 * 4, cudaMemcpyHostToDevice, s));
            if (!g->pool) {
                g->pool_threads = std::max(1, std::min(16, (int) std::thread::hardware_concurrency()));
                g->pool.reset(new StagePool);
                g->pool->start(g->pool_threads - 1);   // the calling thread works too
            }
            stage_h2d(g->h_E.p, emission, (size_t) n * R * 4, g->pin_in, s, *g->pool, g->pool_threads);
        }
        note_h2d((size_t) n * (3 + R) * 4);
        g->solve(g->h_alb.as<float>(), g->h_E.as<float>(), R, bounces, precision, refine, g->h_out.as<float>(), stats,
                 s);
        if (direct) {
            k_copy_floats<<<cgrid, 256, 0, s>>>(out, g->h_out.as<float>(), (size_t) n * R); note_launch();
            GCK(cudaGetLastError());
        } else {
            stage_d2h(out, g->h_out.p, (size_t) n * R * 4, g->pin_out, s, *g->pool, g->pool_threads);
        }
        note_d2h((size_t) n * R * 4);
        GCK(cudaStreamSynchronize(s));
    } catch (const std::exception& e) {
        g->error = e.what();
        cudaGetLastError();   // the error is reported here; none is left for the caller's next CUDA call
        return 0;
    }
    return 1;
}

}  // extern "C"
