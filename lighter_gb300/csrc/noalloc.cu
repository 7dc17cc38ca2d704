// Finishing one lightmap without allocating device memory.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// finish a lightmap: code that runs while its stream is being captured into a
// CUDA graph (allocation is not a capturable operation), engine or editor
// plugins whose host application owns all device memory through its own
// allocator, and per-frame callbacks that must not stall the device (cudaFree
// synchronises). ltrg_FinalizeLightmapNoAlloc gives them the finalize step of
// the bake -- three extrapolating dilation sweeps followed by the separable
// Gaussian blur (lighter.cpp:880-961) -- on device buffers they own. The
// working masks and the blur's intermediate image live in one fixed scratch
// array compiled into the library instead of in freshly allocated memory.
//
// The scratch array is a file-scope __device__ variable, so every GPU that
// loads this library holds it (LTRG_NOALLOC_SCRATCH_BYTES, 14 MiB) until the
// process exits. Host code cannot use the array's name as a device address: a
// call whose stream is not being captured looks the address up with
// cudaGetSymbolAddress, with the caller's device current, and remembers it for
// that device and CUDA context; a call on a stream under capture uses the
// remembered address (looking it up only if there is none yet). So the first
// call in each context -- on each device, and again after a cudaDeviceReset,
// which destroys the context that held the array -- should come before any
// stream capture.
//
// All calls share the one array and it keeps the last call's contents, so
// each call re-initialises both masks before use. Calls whose work overlaps
// on the GPU (two streams, or two host threads on one device) race on the
// scratch and must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

#include "../../include/lighter_gb300.h"
#include "common.cuh"

namespace lg {
namespace {

constexpr unsigned kNaMaxTexels = LTRG_NOALLOC_MAX_TEXELS;
constexpr int kNaMaxExt = 16;
constexpr size_t kMaskBytes = kNaMaxTexels;                        // one u8 mask
constexpr size_t kImageOffset = 2 * kMaskBytes;                    // after two masks (256-byte aligned)
constexpr size_t kScratchBytes = kImageOffset + (size_t) kNaMaxTexels * 3 * sizeof(float);
static_assert(kScratchBytes == LTRG_NOALLOC_SCRATCH_BYTES, "scratch size mismatch with the header");

__device__ __align__(256) unsigned char g_na_scratch[kScratchBytes];

struct Taps { float k[2 * kNaMaxExt + 1]; };

constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
void* g_na_addr[kMaxDevices] = {};
CUcontext g_na_ctx[kMaxDevices] = {};

// The calling thread's current CUDA context (driver entry point, so the
// library needs no link-time dependency on the driver library).
CUcontext current_context()
{
    static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuCtxGetCurrent_v4000) p;
    });
    CUcontext c = nullptr;
    if (fn) fn(&c);
    return c;
}

// Device address of the scratch array for the current device and context:
// looked up afresh unless `capturing`, in which case the address remembered
// for this device and context is used; nullptr on failure.
void* scratch_address(bool capturing, cudaError_t* err)
{
    int dev = -1;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= kMaxDevices) { *err = cudaErrorInvalidDevice; return nullptr; }
    const CUcontext ctx = current_context();
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!capturing || !g_na_addr[dev] || g_na_ctx[dev] != ctx) {
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_na_scratch);
        if (*err != cudaSuccess) return nullptr;
        g_na_addr[dev] = p;
        g_na_ctx[dev] = ctx;
    }
    return g_na_addr[dev];
}

// out = rgb, mask A = input mask (the scratch keeps the previous call's bytes).
__global__ void k_na_init(unsigned n, const float* __restrict__ rgb, const unsigned char* __restrict__ mask,
                          float* out, unsigned char* __restrict__ ma)
{
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        out[3 * g + 0] = rgb[3 * g + 0];
        out[3 * g + 1] = rgb[3 * g + 1];
        out[3 * g + 2] = rgb[3 * g + 2];
        ma[g] = mask[g] ? 1 : 0;
    }
}

__global__ void k_na_copy_mask(unsigned n, const unsigned char* __restrict__ a, unsigned char* __restrict__ b)
{
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) b[g] = a[g];
}

// One dilation sweep (lighter.cpp:884-943) over a single w x h image: texels
// unset in `old` take the mean of their set 4-neighbours, each extrapolated
// linearly (2 c1 - c2) when the next texel out is set too, clamped at 0.
__global__ void k_na_dilate(unsigned w, unsigned h, const unsigned char* __restrict__ old, unsigned char* __restrict__ next,
                            float* img)
{
    const unsigned n = w * h;
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        if (old[g]) continue;
        unsigned x = g % w, y = g / w;
        auto isset = [&](unsigned xx, unsigned yy) { return xx < w && yy < h && old[xx + yy * w]; };
        auto col = [&](unsigned xx, unsigned yy) { const float* p = img + 3 * (xx + yy * w); return mk(p[0], p[1], p[2]); };
        V3 c = mk(0, 0, 0);
        int cnt = 0;
        if (isset(x - 1, y)) { c += isset(x - 2, y) ? lerp3(col(x - 2, y), col(x - 1, y), 2.0f) : col(x - 1, y); cnt++; }
        if (isset(x + 1, y)) { c += isset(x + 2, y) ? lerp3(col(x + 2, y), col(x + 1, y), 2.0f) : col(x + 1, y); cnt++; }
        if (isset(x, y - 1)) { c += isset(x, y - 2) ? lerp3(col(x, y - 2), col(x, y - 1), 2.0f) : col(x, y - 1); cnt++; }
        if (isset(x, y + 1)) { c += isset(x, y + 2) ? lerp3(col(x, y + 2), col(x, y + 1), 2.0f) : col(x, y + 1); cnt++; }
        if (cnt) {
            c = c / (float) cnt;
            float* p = img + 3 * g;
            p[0] = fmax_(c.x, 0.0f);
            p[1] = fmax_(c.y, 0.0f);
            p[2] = fmax_(c.z, 0.0f);
            next[g] = 1;
        }
    }
}

// Clamp-to-edge row convolution written transposed (lighter_math.cpp:367-398):
// src is W x H, dst is H x W.
__global__ void k_na_conv_t(unsigned W, unsigned H, int ext, Taps taps, const float* __restrict__ src, float* __restrict__ dst)
{
    const unsigned n = W * H;
    for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        unsigned x = g % W, y = g / W;
        const float* row = src + 3 * (size_t) y * W;
        float s0 = 0, s1 = 0, s2 = 0;
        for (int i = -ext; i <= ext; ++i) {
            int xx = (int) x + i;
            xx = xx < 0 ? 0 : (xx >= (int) W ? (int) W - 1 : xx);
            float kq = taps.k[i + ext];
            s0 += row[3 * xx + 0] * kq;
            s1 += row[3 * xx + 1] * kq;
            s2 += row[3 * xx + 2] * kq;
        }
        float* o = dst + 3 * ((size_t) y + (size_t) H * x);
        o[0] = s0; o[1] = s1; o[2] = s2;
    }
}

}  // namespace
}  // namespace lg

using namespace lg;

extern "C" LTRAPI int ltrg_FinalizeLightmapNoAlloc(const float* rgb, const unsigned char* mask, float* out,
                                                    u32 width, u32 height, float blur_size, void* stream)
{
    if (!rgb || !mask || !out || width == 0 || height == 0) return LTRG_NOALLOC_EINVAL;
    if ((unsigned long long) width * height > kNaMaxTexels) return LTRG_NOALLOC_ETOOBIG;
    if (!(blur_size >= 0.0f) || std::ceil(blur_size) > (float) kNaMaxExt) return LTRG_NOALLOC_EINVAL;
    cudaStream_t st = (cudaStream_t) stream;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const bool capturing = cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
    cudaError_t e;
    unsigned char* base = (unsigned char*) scratch_address(capturing, &e);
    if (!base) return LTRG_NOALLOC_ECUDA;
    unsigned char* ma = base;
    unsigned char* mb = base + kMaskBytes;
    float* tmp = (float*) (base + kImageOffset);
    const unsigned n = width * height;
    const unsigned threads = 256;
    const unsigned blocks = (n + threads - 1) / threads < 152u * 32u ? (n + threads - 1) / threads : 152u * 32u;

    k_na_init<<<blocks, threads, 0, st>>>(n, rgb, mask, out, ma);
    // three sweeps; the masks swap roles instead of being copied back
    unsigned char* cur = ma;
    unsigned char* nxt = mb;
    for (int it = 0; it < 3; ++it) {
        k_na_copy_mask<<<blocks, threads, 0, st>>>(n, cur, nxt);
        k_na_dilate<<<blocks, threads, 0, st>>>(width, height, cur, nxt, out);
        unsigned char* t = cur;
        cur = nxt;
        nxt = t;
    }
    if (blur_size != 0.0f) {
        // Gaussian taps on the host with the reference's formula
        // (Generate_Gaussian_Kernel, lighter_math.cpp:357-365)
        int ext = (int) std::ceil(blur_size);
        Taps taps;
        float sum = 0.0f;
        float mc = 1.0f / sqrtf(2.0f * 3.14159265358979323846f * blur_size * blur_size);
        for (int i = -ext; i <= ext; ++i) sum += taps.k[i + ext] = expf(-0.5f * powf((float) i / blur_size, 2.0f)) * mc;
        for (int i = -ext; i <= ext; ++i) taps.k[i + ext] /= sum;
        k_na_conv_t<<<blocks, threads, 0, st>>>(width, height, ext, taps, out, tmp);
        k_na_conv_t<<<blocks, threads, 0, st>>>(height, width, ext, taps, tmp, out);
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? LTRG_NOALLOC_OK : LTRG_NOALLOC_ECUDA;
}
