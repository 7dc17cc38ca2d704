// ltrdbg_TraceSegments: closest hits of arbitrary segments against a triangle
// soup, through the bake's BVH builder, traversal and segment tests. A test
// hook for the two intersection modes (LTRG_ISECT_*) and the traversal; the
// bake itself never calls it.
#include <cuda_runtime.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/lighter_gb300.h"
#include "bvh.cuh"

namespace lg {
namespace {

void tck(cudaError_t e, const char* what, int line)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) + " at trace.cu:" +
                                 std::to_string(line) + " (" + what + ")");
}
#define TCK(x) tck((x), #x, __LINE__)

// One thread per segment (6 floats: start, end): the smallest hit fraction
// over every triangle, kNoHit when none.
__global__ void k_trace_segments(BvhView b, ErrFlag err, const float* __restrict__ seg, u32 n, float* __restrict__ out)
{
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* s = seg + 6 * (size_t) i;
    out[i] = bvh_closest(b, mk(s[0], s[1], s[2]), mk(s[3], s[4], s[5]), err, nullptr);
}

}  // namespace
}  // namespace lg

using namespace lg;

extern "C" {

LTRAPI LTRBOOL ltrdbg_TraceSegments(const float* tri_xyz, u32 n_tris, const float* seg6, u32 n_segs,
                                    int intersect_mode, float* out_r, int device)
{
    if ((n_tris && !tri_xyz) || (n_segs && (!seg6 || !out_r))) return 0;
    if (intersect_mode != LTRG_ISECT_REFERENCE && intersect_mode != LTRG_ISECT_WATERTIGHT) return 0;
    cudaStream_t st = nullptr;
    std::vector<void*> bufs;
    BvhStorage bvh;
    bool built = false;
    LTRBOOL ok = 1;
    try {
        TCK(cudaSetDevice(device));
        TCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        // device buffer of `bytes`, filled from `h` when given
        auto dbuf = [&](const void* h, size_t bytes) {
            void* d = nullptr;
            TCK(cudaMallocAsync(&d, bytes ? bytes : 16, st));
            bufs.push_back(d);
            if (h && bytes) TCK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
            return d;
        };
        std::vector<float> xyz(tri_xyz, tri_xyz + 9 * (size_t) n_tris);
        std::vector<u32> meta(n_tris, kOccluderBit), local(n_tris);
        for (u32 i = 0; i < n_tris; ++i) local[i] = i;
        std::vector<u32> ref_tri;
        std::vector<float> ref_box;
        float cmin[3] = {0, 0, 0}, cmax[3] = {0, 0, 0};
        build_refs_host(xyz, ref_tri, ref_box, cmin, cmax);
        BvhBuildInput in;
        in.tri_xyz = (const float*) dbuf(xyz.data(), xyz.size() * 4);
        in.tri_meta = (const u32*) dbuf(meta.data(), meta.size() * 4);
        in.tri_local = (const u32*) dbuf(local.data(), local.size() * 4);
        in.ref_tri = (const u32*) dbuf(ref_tri.data(), ref_tri.size() * 4);
        in.ref_box = (const float*) dbuf(ref_box.data(), ref_box.size() * 4);
        in.n = (int) ref_tri.size();
        for (int c = 0; c < 3; ++c) { in.scene_min[c] = cmin[c]; in.scene_max[c] = cmax[c]; }
        BvhView view = {};
        if (in.n) {
            bvh_build(in, bvh, st);
            built = true;
            view = bvh.view();
        }
        view.watertight = intersect_mode == LTRG_ISECT_WATERTIGHT ? 1 : 0;
        const float* dseg = (const float*) dbuf(seg6, (size_t) n_segs * 6 * 4);
        float* dout = (float*) dbuf(nullptr, (size_t) n_segs * 4);
        u32* derr = (u32*) dbuf(nullptr, 4);
        TCK(cudaMemsetAsync(derr, 0, 4, st));
        if (n_segs) {
            k_trace_segments<<<(n_segs + 127) / 128, 128, 0, st>>>(view, ErrFlag{derr}, dseg, n_segs, dout);
            TCK(cudaGetLastError());
            TCK(cudaMemcpyAsync(out_r, dout, (size_t) n_segs * 4, cudaMemcpyDeviceToHost, st));
        }
        u32 herr = 0;
        TCK(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st));
        TCK(cudaStreamSynchronize(st));
        if (herr) throw std::runtime_error("traversal error word set");
    } catch (const std::exception& e) {
        fprintf(stderr, "ltrdbg_TraceSegments: %s\n", e.what());
        cudaGetLastError();   // leave no error state behind for the caller's next CUDA call
        ok = 0;
    }
    if (st) {
        if (built) bvh_free(bvh, st);
        for (void* p : bufs) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    return ok;
}

}  // extern "C"
