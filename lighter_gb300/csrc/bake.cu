// The bake on the GPU: the stage order of ltr_Scene::Job_MainProc
// (lighter.cpp:1046-1145) with every per-texel, per-light, per-pair and
// per-ray loop of the reference turned into CUDA kernels.
//
//   host   transform instances, size lightmaps (size_fn), build triangle and
//          raster records, cull lights against instance boxes
//   GPU    BVH build (bvh.cu)
//   GPU    sample generation: two raster passes with last-writer-wins keys,
//          compaction, concave-edge offset and overlap correction
//   GPU    direct light (sphere-traced penumbra per (light, sample))
//   GPU    radiosity: dense form factors + visibility, bounces as F x colours
//   GPU    ambient occlusion (one warp per sample, one lane per ray)
//   GPU    finalize: scatter, 3 dilation sweeps, separable blur, ds2x, normals
//   host   readback into scene-owned output buffers
#include <cuda_runtime.h>
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <unordered_map>
#include <chrono>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh.cuh"
#include "radiosity.cuh"
#include "reftree.hpp"
#include "scene.hpp"

namespace lg {

HostCounters& host_counters()
{
    static thread_local HostCounters c;
    return c;
}

namespace {

void ck(cudaError_t e, const char* what, int line)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) + " at bake.cu:" +
                                 std::to_string(line) + " (" + what + ")");
}
#define CK(x) ck((x), #x, __LINE__)

constexpr int kThreads = 256;
constexpr u32 kNoLoc = 0xffffffffu;

// f(begin, end) over [0, n) in contiguous chunks on up to 16 host threads
// (one thread below 2 * grain items).
template <class F>
void parallel_for(size_t n, size_t grain, F&& f)
{
    size_t nt = std::min<size_t>({(size_t) 16, (size_t) std::max(1u, std::thread::hardware_concurrency()),
                                  (n + grain - 1) / std::max<size_t>(grain, 1)});
    if (nt <= 1) {
        if (n) f((size_t) 0, n);
        return;
    }
    const size_t chunk = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t) {
        const size_t b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back([&f, b, e]() { f(b, e); });
    }
    for (auto& x : th) x.join();
}

// f(i) for i in [0, n) on up to 16 host threads taking items one at a time;
// the first exception is rethrown after all threads end.
template <class F>
void parallel_items(int n, F&& f)
{
    int nt = std::min({16, (int) std::max(1u, std::thread::hardware_concurrency()), n});
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int> next(0);
    std::exception_ptr err;
    std::mutex mu;
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&]() {
            for (int i = next++; i < n; i = next++) {
                try {
                    f(i);
                } catch (...) {
                    std::lock_guard<std::mutex> lk(mu);
                    if (!err) err = std::current_exception();
                }
            }
        });
    for (auto& x : th) x.join();
    if (err) std::rethrow_exception(err);
}

inline unsigned blocks_for(size_t n, int threads = kThreads, size_t cap = 152 * 64)
{
    size_t b = (n + threads - 1) / threads;
    if (b > cap) b = cap;
    return (unsigned) (b ? b : 1);
}

// ----------------------------------------------------------------------------- device-side records

struct DLight {
    int type;
    float pos[3], dir[3], color[3];
    float range, power, radius, out_rad, diff, curve;
    int ns, soff;   // LTRG_SHADOW_SAMPLED: shadow samples of the light at lsmp[soff .. soff + ns)
};

// Raster record of one triangle (RasterizeInstance, lighter.cpp:32-66):
//   [0..5] lightmap-space p1,p2,p3  [6..14] world pos  [15..23] world normal
//   [24..29] uv1  [30] part  [31] sample area
constexpr int kRT = 32;

struct Counters {
    unsigned long long shadow_evals, distance_queries, ao_rays, rad_pairs, rad_vis_rays, node_visits, tri_tests, shadow_pairs;
};

// Warp total of a per-thread count, added once per warp; every lane of the
// warp must call it (used after grid-stride loops, where all lanes arrive).
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

// ----------------------------------------------------------------------------- raster

// Texel (x, y) is covered by the triangle when it lies within `margin` of all
// three edges for either winding (lighter_math.cpp:281-300).
__device__ __forceinline__ bool raster_inside(const float* r, int x, int y, float margin)
{
    V2 p1 = mk2(r[0], r[1]), p2 = mk2(r[2], r[3]), p3 = mk2(r[4], r[5]);
    V2 e12 = p2 - p1, e13 = p3 - p1, e23 = p3 - p2;
    V2 n1 = normalized2(mk2(e12.y, -e12.x));
    V2 n2 = normalized2(mk2(e23.y, -e23.x));
    V2 n3t = normalized2(mk2(e13.y, -e13.x));
    V2 n3 = mk2(-n3t.x, -n3t.y);
    float d1 = dot2(n1, p1), d2 = dot2(n2, p2), d3 = dot2(n3, p3);
    V2 p = mk2((float) x, (float) y);
    float pd1 = dot2(p, n1), pd2 = dot2(p, n2), pd3 = dot2(p, n3);
    return (pd1 <= d1 + margin && pd2 <= d2 + margin && pd3 <= d3 + margin) ||
           (pd1 + margin >= d1 && pd2 + margin >= d2 && pd3 + margin >= d3);
}

__global__ void k_raster_mark(int pass, float margin, const float* __restrict__ rt, const u32* __restrict__ rinst,
                              const int4* __restrict__ bbox, const unsigned long long* __restrict__ off, int ntri,
                              unsigned long long nwork, const unsigned long long* __restrict__ tex_off,
                              const u32* __restrict__ inst_w, u32* __restrict__ keys)
{
    for (unsigned long long w = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; w < nwork;
         w += (unsigned long long) gridDim.x * blockDim.x) {
        int lo = 0, hi = ntri - 1;   // largest k with off[k] <= w
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= w) lo = mid; else hi = mid - 1;
        }
        int k = lo;
        int4 b = bbox[k];
        unsigned long long local = w - off[k];
        int x = b.x + (int) (local % (unsigned) b.z);
        int y = b.y + (int) (local / (unsigned) b.z);
        if (!raster_inside(rt + (size_t) k * kRT, x, y, margin)) continue;
        u32 inst = rinst[k];
        unsigned long long g = tex_off[inst] + (unsigned long long) x + (unsigned long long) inst_w[inst] * y;
        atomicMax(&keys[g], 1u + ((u32) pass << 30) + (u32) k);
    }
}

// Attribute interpolation of the winning triangle (lighter_math.cpp:285-299).
__global__ void k_raster_resolve(unsigned long long ntex, const u32* __restrict__ keys, const float* __restrict__ rt,
                                 const u32* __restrict__ rinst, const unsigned long long* __restrict__ tex_off,
                                 const u32* __restrict__ inst_w, float4* __restrict__ R1, float4* __restrict__ R2,
                                 float4* __restrict__ R3, u32* __restrict__ flags)
{
    for (unsigned long long g = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; g < ntex;
         g += (unsigned long long) gridDim.x * blockDim.x) {
        u32 key = keys[g];
        if (key == 0) { flags[g] = 0; continue; }
        u32 k = (key - 1u) & ((1u << 30) - 1u);
        const float* r = rt + (size_t) k * kRT;
        u32 inst = rinst[k];
        unsigned long long local = g - tex_off[inst];
        u32 w = inst_w[inst];
        int x = (int) (local % w), y = (int) (local / w);
        V2 p1 = mk2(r[0], r[1]), p2 = mk2(r[2], r[3]), p3 = mk2(r[4], r[5]);
        V2 e12 = p2 - p1, e13 = p3 - p1;
        float vc = cross2(e12, e13);
        V2 q = mk2(x - p1.x, y - p1.y);
        float s = cross2(q, e13) / vc;
        float t = cross2(e12, q) / vc;
        s = fmax_(fmin_(s, 1.0f), 0.0f);
        t = fmax_(fmin_(t, 1.0f), 0.0f);
        V3 a1 = mk(r[6], r[7], r[8]), a2 = mk(r[9], r[10], r[11]), a3 = mk(r[12], r[13], r[14]);
        V3 b1 = mk(r[15], r[16], r[17]), b2 = mk(r[18], r[19], r[20]), b3 = mk(r[21], r[22], r[23]);
        V3 pa = a1 + (a2 - a1) * s + (a3 - a1) * t;
        V3 pb = b1 + (b2 - b1) * s + (b3 - b1) * t;
        float c1x = r[24], c1y = r[25], c2x = r[26], c2y = r[27], c3x = r[28], c3y = r[29];
        float part = r[30], area = r[31];
        float4 pc = make_float4(c1x + (c2x - c1x) * s + (c3x - c1x) * t, c1y + (c2y - c1y) * s + (c3y - c1y) * t,
                                part + (part - part) * s + (part - part) * t, area + (area - area) * s + (area - area) * t);
        R1[g] = st4(pa, 0.0f);
        R2[g] = st4(pb, 0.0f);
        R3[g] = pc;
        flags[g] = is_zero(pb) ? 0u : 1u;
    }
}

__global__ void k_compact(unsigned long long ntex, const u32* __restrict__ flags, const u32* __restrict__ scan,
                          const float4* __restrict__ R1, const float4* __restrict__ R2, const float4* __restrict__ R3,
                          const unsigned long long* __restrict__ tex_off, int n_inst, u32 n_probe,
                          float4* __restrict__ spos, float4* __restrict__ snrm, float4* __restrict__ srad,
                          u32* __restrict__ sloc, u32* __restrict__ sinst)
{
    for (unsigned long long g = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; g < ntex;
         g += (unsigned long long) gridDim.x * blockDim.x) {
        if (!flags[g]) continue;
        int lo = 1, hi = n_inst - 1;   // instance with tex_off[inst] <= g (instance 0 owns no texels)
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (tex_off[mid] <= g) lo = mid; else hi = mid - 1;
        }
        u32 s = n_probe + scan[g];
        spos[s] = R1[g];
        snrm[s] = st4(normalized(ld3(R2[g])), 0.0f);
        srad[s] = R3[g];
        sloc[s] = (u32) (g - tex_off[lo]);
        sinst[s] = (u32) lo;
    }
}

// ----------------------------------------------------------------------------- sample offset + correction

struct FixupArgs {
    BvhView bvh;
    ErrFlag err;
    const float4* ref_nodes;   // 2 per node: (mn.xyz, mx.x), (mx.yz, ch, ido)
    const int* ref_items;      // <count, ids...> lists
    const int4* ref_inst;      // per instance: node offset, item offset, triangle offset, node count
    const float4* inst_box;    // per instance: (root mn.xyz, 0), (root mx.xyz, 0); inverted when empty
    const float* tri_xyz;      // shadow-part triangles, instance by instance in local order
    const float4* tri_box;     // per triangle: (box mn.xyz, 0), (box mx.xyz, 0); unbounded for slivers
    int n_inst;
    u32 n_probe, n_samples;
    float max_correct_dist, corr_min_dot;
    float4* spos;
    const float4* snrm;
    const float4* srad;
};

// Concave-edge push of TriTree::OffsetSample (lighter_math.cpp:991-1044) for
// one triangle, up to its visibility query: whether the push is a candidate,
// and then the query segment [qo, qe] (qe = the pushed position). The push
// applies when the query's closest hit among the instance's triangles is at
// 0.9 or beyond, or is this triangle.
__device__ __forceinline__ bool offset_candidate(V3 P1, V3 P2, V3 P3, V3 P, V3 N, float dist, V3& qo, V3& qe)
{
    float nd = point_tri_dist(P, P1, P2, P3);
    if (!(nd < dist)) return false;
    V3 TPN = -tri_normal_rev(P1, P2, P3);
    float TPD = dot(TPN, P1);
    float sig = dot(TPN, P) - TPD;
    if (!(sig <= kSmall)) return false;
    V3 Pextr = P + normalized(TPN + N) * -sig * 1.41f;
    if (!point_proj_on_tri(Pextr, P1, P2, P3)) return false;
    float pdot = dot(TPN, N);
    if (!(fabsf(pdot) < 0.95f)) return false;
    V3 proj = normalized(TPN - N * pdot);
    float df = 1.0f - fabsf(pdot);
    qe = P + proj * (-sig / df + kSmall);
    qo = P + (N + proj) * kSmall;
    return true;
}

// Boxes of the concave-edge pass's triangles, for its exact rejection test: the
// box of a well-shaped triangle (height at least 1% of its longest edge); an
// unbounded box for a thinner one, which the test then never rejects.
__global__ void k_tri_boxes(const float* __restrict__ tri_xyz, u32 n, float4* __restrict__ box)
{
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = tri_xyz + 9 * (size_t) i;
    const V3 a = mk(p[0], p[1], p[2]), b = mk(p[3], p[4], p[5]), c = mk(p[6], p[7], p[8]);
    const V3 cr = cross(b - a, c - a);
    const float l2 = fmaxf(dot(b - a, b - a), fmaxf(dot(c - b, c - b), dot(a - c, a - c)));
    if (dot(cr, cr) >= 1e-4f * l2 * l2 && l2 > 0.0f) {
        box[2 * i] = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0.0f);
        box[2 * i + 1] = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0.0f);
    } else {
        box[2 * i] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        box[2 * i + 1] = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
    }
}

// Whether the concave-edge push of a triangle with box (bmn, bmx) surely does
// nothing at P: the box lies more than r beyond P along an axis, r being dist
// plus a margin (1 mm + 1e-5 of P's largest coordinate) far above the rounding
// of point_tri_dist on a well-shaped triangle. The exact distance is at least
// the box's separation, the computed one within rounding of it, so it is not
// below dist and offset_candidate would return at its first test.
__device__ __forceinline__ bool fixup_rejects(float4 bmn, float4 bmx, V3 P, float dist)
{
    const float scale = fmaxf(fabsf(P.x), fmaxf(fabsf(P.y), fabsf(P.z)));
    const float r = dist * 1.0001f + 1e-3f + 1e-5f * scale;
    return P.x + r < bmn.x || P.x - r > bmx.x || P.y + r < bmn.y || P.y - r > bmx.y || P.z + r < bmn.z ||
           P.z - r > bmx.z;
}

// One instance of the concave-edge pass for the 32 lanes of a warp (every lane
// calls it with the same instance; `active` marks the lanes with a sample). A
// lane's pass is a depth-first walk of the instance's reference-shaped tree
// (node items, then node + 1's subtree, then the other child's) with the query
// box P +- dist fixed at the start while P moves. The warp walks the tree once
// in that order, a node's lanes being those whose box meets the node and all
// its ancestors -- the lanes whose own walk reaches it -- so each lane handles
// exactly its own walk's triangles in its own walk's order. Node and triangle
// loads are broadcasts; the stack (node, lane mask) is warp-uniform, entry i in
// lane i % 32.
__device__ __forceinline__ void fixup_instance_warp(const FixupArgs& a, int k, bool active, V3& P, V3 N, float dist)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int4 ri = a.ref_inst[k];
    if (ri.w == 0) return;
    const V3 qmn = P - splat(dist), qmx = P + splat(dist);
    int s0 = 0, s1 = 0, sp = 0;          // pending subtrees
    unsigned m0 = 0, m1 = 0;             // the lanes that reached their parents
    int node = 0;
    unsigned in = __ballot_sync(full, active);
    for (;;) {
        bool ov = false;
        if (in) {
            const float4 n0 = __ldg(&a.ref_nodes[2 * (ri.x + node)]);
            const float4 n1 = __ldg(&a.ref_nodes[2 * (ri.x + node) + 1]);
            ov = ((in >> lane) & 1u) &&
                 !(qmn.x > n0.w || qmx.x < n0.x || qmn.y > n1.x || qmx.y < n0.y || qmn.z > n1.y || qmx.z < n0.z);
            const unsigned m = __ballot_sync(full, ov);
            if (m) {
                const int ch = __float_as_int(n1.z), ido = __float_as_int(n1.w);
                if (ido != -1) {
                    const int* it = a.ref_items + ri.y + ido;
                    const int cnt = __ldg(it);
                    for (int i = 0; i < cnt; ++i) {
                        const int id = __ldg(it + 1 + i);
                        bool want = false;
                        V3 qo = mk(0, 0, 0), qe = mk(0, 0, 0);
                        if (ov && !fixup_rejects(__ldg(&a.tri_box[2 * (size_t) (ri.z + id)]),
                                                 __ldg(&a.tri_box[2 * (size_t) (ri.z + id) + 1]), P, dist)) {
                            const float* p = a.tri_xyz + 9 * (size_t) (ri.z + id);
                            want = offset_candidate(mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8]),
                                                    P, N, dist, qo, qe);
                        }
                        // the candidates' visibility queries, one walk shared by the warp
                        if (__any_sync(full, want)) {
                            int hit_local = -1;
                            const float r = warp_closest_inst(a.bvh, qo, qe, (u32) k, want, a.err, &hit_local);
                            if (want && (r >= 0.9f || hit_local == id)) P = qe;
                        }
                    }
                }
                if (ch != -1) {
                    // the lane's own walk pushes ch, then node + 1, and pops node + 1 first
                    if (sp < 64) {
                        if (lane == (sp & 31)) {
                            if (sp < 32) { s0 = ch; m0 = m; } else { s1 = ch; m1 = m; }
                        }
                        ++sp;
                    } else if (lane == 0) {
                        raise_err(a.err, 1u);
                    }
                    node = node + 1;
                    in = m;
                    continue;
                }
            }
        }
        if (sp == 0) break;
        --sp;
        node = __shfl_sync(full, sp < 32 ? s0 : s1, sp & 31);
        in = __shfl_sync(full, sp < 32 ? m0 : m1, sp & 31);
    }
}

constexpr int kFixupThreads = 128;
constexpr int kFixupCand = 256;   // candidate instances listed per warp

// The concave-edge pass tests every instance's tree, in instance order
// (lighter.cpp:445-446); an instance whose root box misses the query box
// leaves P unchanged. A warp (32 consecutive samples) first lists, in order,
// the instances whose root box meets the union of its query boxes grown by
// G > M, and its lanes walk only those. A lane whose P has moved more than M
// (per axis) from its start could meet an unlisted instance, so once any lane
// has, the warp walks every remaining instance. Either way each lane visits
// every instance its query box meets, in order: the reference's result.
__global__ void __launch_bounds__(kFixupThreads) k_fixup(FixupArgs a)
{
    __shared__ int cand[kFixupThreads / 32][kFixupCand];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const u32 s = a.n_probe + blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < a.n_samples;
    if (!__any_sync(full, active)) return;
    V3 P = mk(0, 0, 0), N = mk(0, 0, 0);
    float dist = 0.0f;
    if (active) {
        P = ld3(a.spos[s]);
        N = ld3(a.snrm[s]);
        dist = sqrtf(a.srad[s].w);
    }
    const V3 P0 = P;
    float lo[3] = {active ? P.x - dist : 3.0e38f, active ? P.y - dist : 3.0e38f, active ? P.z - dist : 3.0e38f};
    float hi[3] = {active ? P.x + dist : -3.0e38f, active ? P.y + dist : -3.0e38f, active ? P.z + dist : -3.0e38f};
    float dmax = dist;
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(full, lo[c], o));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(full, hi[c], o));
        }
        dmax = fmaxf(dmax, __shfl_xor_sync(full, dmax, o));
    }
    const float M = 4.0f * dmax + 0.05f;
    const float G = 1.5f * M + 1e-3f;   // the extra covers rounding of the box arithmetic
#pragma unroll
    for (int c = 0; c < 3; ++c) { lo[c] -= G; hi[c] += G; }
    int ncand = 0;
    for (int base = 1; base < a.n_inst; base += 32) {
        const int k = base + lane;
        bool hit = false;
        if (k < a.n_inst) {
            const float4 b0 = __ldg(&a.inst_box[2 * k]), b1 = __ldg(&a.inst_box[2 * k + 1]);
            hit = !(lo[0] > b1.x || hi[0] < b0.x || lo[1] > b1.y || hi[1] < b0.y || lo[2] > b1.z || hi[2] < b0.z);
        }
        const unsigned m = __ballot_sync(full, hit);
        if (hit) {
            const int at = ncand + __popc(m & ((1u << lane) - 1u));
            if (at < kFixupCand) cand[w][at] = k;
        }
        ncand += __popc(m);
    }
    __syncwarp();
    bool slow = ncand > kFixupCand;   // list overflow: every instance
    int ci = 0, k = 1;
    for (;;) {
        if (!slow) {
            if (ci >= ncand) break;
            k = cand[w][ci++];
        } else if (k >= a.n_inst) {
            break;
        }
        fixup_instance_warp(a, k, active, P, N, dist);
        const bool far = fabsf(P.x - P0.x) > M || fabsf(P.y - P0.y) > M || fabsf(P.z - P0.z) > M;
        if (!slow && __any_sync(full, far)) slow = true;
        ++k;
    }
    if (!active) return;
    // push in front of overlapping faces (lighter.cpp:449-465); the
    // reference's BSP query is replaced by the closest hit over occluders
    if (a.max_correct_dist != 0.0f) {
        int left = 100;
        float md = a.max_correct_dist;
        V3 PEnd = P + N * md;
        while (md > kSmall && left-- > 0) {
            V3 dn = normalized(PEnd - P);
            V3 mA = P + dn * kSmall, mB = PEnd - dn * kSmall;
            int ht = -1;
            float q = bvh_closest(a.bvh, mA, mB, a.err, &ht);
            V3 hn = mk(0, 0, 0);
            if (ht >= 0) {
                V3 P1, P2, P3; u32 meta, local;
                load_tri(a.bvh, ht, P1, P2, P3, meta, local);
                hn = tri_normal_rev(P1, P2, P3);
            }
            if (-dot(hn, N) < a.corr_min_dot) break;
            if (q < kSmall) q = kSmall;
            P = P * (1.0f - q) + PEnd * q;
            md *= (1.0f - q);
        }
    }
    a.spos[s] = st4(P, 0.0f);
}

// ----------------------------------------------------------------------------- direct light

// Sphere-traced soft-shadow factor (ltr_Scene::CalcInvShadowFactor, lighter.cpp:190-207).
template <class Stack>
__device__ __forceinline__ float inv_shadow(const BvhView& bvh, V3 from, V3 to, float k, ErrFlag err, u32& nq, u32& nv,
                                            u32& nt, Stack& st)
{
    V3 rd = normalized(to - from);
    float maxt = len(to - from);
    float res = 1.0f;
    // Warm start: the nearest triangle of the previous point lies within
    // h_prev + step of the next one (triangle inequality), so the query starts
    // with that radius (plus slack for rounding) instead of MAX_PENUMBRA_SIZE.
    // If nothing lies inside it, the query is repeated with the full radius,
    // so the result is the reference's min(MAX_PENUMBRA_SIZE, nearest distance)
    // either way (Distance() starts at MAX_PENUMBRA_SIZE, lighter.cpp:150-188).
    float reach = kMaxPenumbraSize;
    for (float t = 0.001f; t < maxt;) {
        V3 p = from + rd * t;
        float r0 = fminf(kMaxPenumbraSize, reach * 1.0001f + 1e-5f);
        float h = bvh_distance_s(bvh, p, r0, err, st, &nv, &nt);
        ++nq;
        if (!(h < r0) && r0 < kMaxPenumbraSize) {
            h = bvh_distance_s(bvh, p, kMaxPenumbraSize, err, st, &nv, &nt);
            ++nq;
        }
        if (h < 0.001f) return 0.0f;
        res = fmin_(res, h / fmin_(t * k, kMaxPenumbraSize));
        float step = fmin_(h, kMaxPenumbraStep);
        reach = h + step;
        t += step;
    }
    return res;
}

// inv_shadow for the 32 lanes of a warp at once (every lane calls it; `has`
// marks the lanes with a pair): each step runs one warp_distance for all lanes
// still marching, so the lanes walk the BVH together instead of 32 divergent
// walks. Every lane makes the same queries (points and radii) as inv_shadow
// and gets the same distances, so the factor is inv_shadow's bit for bit.
__device__ __forceinline__ float inv_shadow_warp(const BvhView& bvh, bool has, V3 from, V3 to, float k, ErrFlag err,
                                                 u32& nq, u32& nv, u32& nt)
{
    V3 rd = mk(0, 0, 0);
    float maxt = 0.0f;
    if (has) {
        rd = normalized(to - from);
        maxt = len(to - from);
    }
    float res = 1.0f;
    float reach = kMaxPenumbraSize;
    float t = 0.001f;
    bool active = has && t < maxt;
    while (__any_sync(0xffffffffu, active)) {
        const V3 p = from + rd * t;
        const float r0 = fminf(kMaxPenumbraSize, reach * 1.0001f + 1e-5f);
        float h = warp_distance(bvh, p, r0, active, err, nv, nt);
        if (active) ++nq;
        const bool again = active && !(h < r0) && r0 < kMaxPenumbraSize;
        if (__any_sync(0xffffffffu, again)) {
            const float h2 = warp_distance(bvh, p, kMaxPenumbraSize, again, err, nv, nt);
            if (again) { h = h2; ++nq; }
        }
        if (active) {
            if (h < 0.001f) {
                res = 0.0f;
                active = false;
            } else {
                res = fmin_(res, h / fmin_(t * k, kMaxPenumbraSize));
                const float step = fmin_(h, kMaxPenumbraStep);
                reach = h + step;
                t += step;
                active = t < maxt;
            }
        }
    }
    return res;
}

struct DirectArgs {
    BvhView bvh;
    ErrFlag err;
    const DLight* lights;
    int n_lights, n_inst;
    const unsigned char* lit;   // [light][instance]
    u32 n_samples;
    const float4* spos;
    const float4* snrm;
    const u32* sinst;
    float* kval;                // [light][sample] colour multiplier, 0 when nothing is added
    float4* ndir;               // [light][sample] normal-map contribution, w = 1 when recorded (may be null)
    Counters* counters;
    float* vis;                 // [light][sample] shadow factor, -1 when not traced (debug record, may be null)
    const u32* order;           // samples in trace order (see k_order_keys)
    int shadow_mode;            // LTRG_SHADOW_*
    const float4* lsmp;         // LTRG_SHADOW_SAMPLED: per-light ray directions (directional) or disk offsets
    const volatile u32* abort_word;   // mapped host word set by ltr_Abort (may be null)
};

// Unshadowed terms of one (light, sample) pair of
// Job_LMRender_{Point,Spot,Direct}_Inner (lighter.cpp:485-600). Returns
// whether the pair needs a shadow trace; `from`/`to` are its segment.
struct LightTerms {
    float f_dist, f_ndotl, f_dir;
    V3 dir;   // sample-to-light (point/spot) or light direction (directional)
    V3 from, to;
};

__device__ __forceinline__ bool light_terms(const DirectArgs& a, const DLight& L, u32 s, LightTerms& o)
{
    V3 SP = ld3(a.spos[s]), SN = ld3(a.snrm[s]);
    V3 Lpos = mk(L.pos[0], L.pos[1], L.pos[2]);
    V3 Ldir = mk(L.dir[0], L.dir[1], L.dir[2]);
    o.f_dir = 1.0f;
    o.from = SP + SN * kShadowOffset;
    if (L.type == 1 || L.type == 2) {
        V3 s2l = Lpos - SP;
        float dist = len(s2l);
        if (dist) s2l = s2l / dist;
        o.f_dist = powf(1 - fmin_(1.0f, dist / L.range), L.power);
        o.f_ndotl = fmax_(0.0f, dot(s2l, SN));
        o.dir = s2l;
        o.to = Lpos;
        if (L.type == 2) {
            float ang = acosf(fmin_(1.0f, dot(s2l, -Ldir)));
            o.f_dir = fmax_(0.0f, fmin_(1.0f, (ang - L.out_rad) / L.diff));
            o.f_dir = powf(o.f_dir, L.curve);
            return !(o.f_dist * o.f_ndotl * o.f_dir <= 0);
        }
        return !(o.f_dist * o.f_ndotl <= 0);
    }
    if (L.type == 3) {
        o.f_dist = 1.0f;
        o.dir = Ldir;
        if (a.shadow_mode == 1) {
            // sampled block of Job_LMRender_Direct_Inner (lighter.cpp:566-584): N.L
            // averaged over the light's ray directions, rays from the sample itself
            float f = 0.0f;
            for (int k = 0; k < L.ns; ++k) f += fmax_(0.0f, dot(ld3(a.lsmp[L.soff + k]), SN));
            o.f_ndotl = f / L.ns;
            o.from = SP;
            o.to = SP;
            return o.f_ndotl > 0.0f;
        }
        o.f_ndotl = fmax_(0.0f, dot(Ldir, SN));
        o.to = SP + Ldir * L.range;
        // the reference traces even when N.L = 0; its term is then 0 * vis = 0,
        // so the trace is skipped without changing the result
        return o.f_ndotl > 0.0f;
    }
    return false;
}

// ltr_Scene::VisibilityTest (lighter.cpp:112-147): an occluder on the segment
// A -> B shortened by SMALL_FLOAT at both ends.
template <class Stack>
__device__ __forceinline__ bool occluded(const BvhView& bvh, V3 A, V3 B, ErrFlag err, Stack& st)
{
    V3 dn = normalized(B - A);
    return bvh_any_hit_s<false>(bvh, A + dn * kSmall, B - dn * kSmall, err, st);
}

// LTRG_SHADOW_SAMPLED: the fraction of the light's ns shadow rays that reach
// it. Directional lights: rays from the sample along each stored direction
// over `range` (lighter.cpp:566-584). Point and spot lights: rays from the
// offset sample position to the stored disk points, placed on the disk of
// radius light_radius around the light that faces the sample (basis built
// from the sample-to-light direction as in CreateSpiralDirVector,
// lighter_int.hpp:465-467).
template <class Stack>
__device__ __forceinline__ float sampled_vis(const DirectArgs& a, const DLight& L, const LightTerms& t, Stack& st)
{
    float f = 0.0f;
    if (L.type == 3) {
        for (int k = 0; k < L.ns; ++k) {
            V3 adj = ld3(a.lsmp[L.soff + k]);
            if (occluded(a.bvh, t.from, t.from + adj * L.range, a.err, st)) f += 1.0f;
        }
    } else {
        V3 dir = t.dir;
        V3 diffvec = mk(dir.y, -dir.z, dir.x);
        V3 up = normalized(cross(dir, diffvec));
        V3 rt = cross(dir, up);
        V3 Lpos = mk(L.pos[0], L.pos[1], L.pos[2]);
        for (int k = 0; k < L.ns; ++k) {
            float4 d = a.lsmp[L.soff + k];
            V3 T = Lpos + rt * d.x + up * d.y;
            if (occluded(a.bvh, t.from, T, a.err, st)) f += 1.0f;
        }
    }
    f /= L.ns;
    return 1.0f - f;
}

// sampled_vis for the 32 lanes of a warp at once (every lane calls it; `has`
// marks the lanes with a pair): shadow sample k of every lane's light is
// traced by one warp_any_hit for all lanes, so neighbouring samples' rays to
// the same light point share their walk. Same rays, same hit counts, same
// factor as sampled_vis.
__device__ __forceinline__ float sampled_vis_warp(const DirectArgs& a, bool has, const DLight& L, const LightTerms& t)
{
    const int ns = has ? L.ns : 0;
    int n_max = ns;
    for (int o = 16; o > 0; o >>= 1) n_max = max(n_max, __shfl_xor_sync(0xffffffffu, n_max, o));
    V3 rt = mk(0, 0, 0), up = mk(0, 0, 0);
    const V3 Lpos = mk(L.pos[0], L.pos[1], L.pos[2]);
    if (has && L.type != 3) {
        V3 dir = t.dir;
        V3 diffvec = mk(dir.y, -dir.z, dir.x);
        up = normalized(cross(dir, diffvec));
        rt = cross(dir, up);
    }
    float f = 0.0f;
    for (int k = 0; k < n_max; ++k) {
        const bool go = k < ns;
        V3 A = t.from, B = t.from;
        if (go) {
            const float4 q = a.lsmp[L.soff + k];
            B = L.type == 3 ? t.from + ld3(q) * L.range : Lpos + rt * q.x + up * q.y;
        }
        const V3 dn = normalized(B - A);
        if (warp_any_hit(a.bvh, A + dn * kSmall, B - dn * kSmall, go, a.err)) f += 1.0f;
    }
    if (!has) return 1.0f;
    f /= L.ns;
    return 1.0f - f;
}

// Pass 1 over every (light, sample) pair: zero the outputs and flag the
// pairs that need a shadow trace (lit instance, positive unshadowed term).
// flags[v] is indexed in trace order, v = light * n_samples + rank, the pair
// being w = light * n_samples + order[rank].
__global__ void k_direct_setup(DirectArgs a, u32* __restrict__ flags)
{
    unsigned long long total = (unsigned long long) a.n_lights * a.n_samples;
    for (unsigned long long v = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; v < total;
         v += (unsigned long long) gridDim.x * blockDim.x) {
        int l = (int) (v / a.n_samples);
        u32 s = a.order ? a.order[v % a.n_samples] : (u32) (v % a.n_samples);
        const unsigned long long w = (unsigned long long) l * a.n_samples + s;
        const DLight L = a.lights[l];
        u32 inst = a.sinst[s];
        bool go = false;
        if (a.lit[(size_t) l * a.n_inst + inst]) {
            LightTerms t;
            go = light_terms(a, L, s, t);
        }
        a.kval[w] = 0.0f;
        if (a.ndir) a.ndir[w] = make_float4(0, 0, 0, 0);
        if (a.vis) a.vis[w] = -1.0f;
        flags[v] = go ? 1u : 0u;
    }
}

// The traced pairs w in trace order.
__global__ void k_direct_compact(unsigned long long total, u32 n_samples, const u32* __restrict__ order,
                                 const u32* __restrict__ flags, const u32* __restrict__ scan, u32* __restrict__ items)
{
    for (unsigned long long v = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; v < total;
         v += (unsigned long long) gridDim.x * blockDim.x)
        if (flags[v]) items[scan[v]] = order ? (u32) ((v / n_samples) * n_samples + order[v % n_samples]) : (u32) v;
}

// Trace orders of the samples (tuning direct_order / ao_order): the warps of
// the trace kernels take their pairs and rays in this order, so 32
// consecutive entries should lie close together. 1: by instance, then by the
// Morton (Z-order) code of the texel in its lightmap (a compact block of
// texels instead of a row segment); 2: by the 3D Morton code of the sample
// position in the scene bounds (close in the world, across charts and
// instances). 0 keeps the sample order. Outputs stay indexed by sample.
__device__ __forceinline__ u32 spread16(u32 v)
{
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__device__ __forceinline__ u32 spread10(u32 v)
{
    v &= 0x3ffu;
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_order_keys(int mode, u32 n, const u32* __restrict__ sinst, const u32* __restrict__ sloc,
                             const u32* __restrict__ inst_w, const float4* __restrict__ spos, float3 mn, float3 inv_ext,
                             unsigned long long* __restrict__ keys, u32* __restrict__ vals)
{
    for (u32 s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        if (mode == 1) {
            const u32 inst = sinst[s], w = max(inst_w[inst], 1u), loc = sloc[s];
            const u32 x = loc % w, y = loc / w;
            keys[s] = ((unsigned long long) inst << 32) | (spread16(x) | (spread16(y) << 1));
        } else {
            const float4 p = spos[s];
            auto q = [](float v) { return (u32) fminf(fmaxf(v * 1024.0f, 0.0f), 1023.0f); };
            const u32 x = q((p.x - mn.x) * inv_ext.x), y = q((p.y - mn.y) * inv_ext.y), z = q((p.z - mn.z) * inv_ext.z);
            keys[s] = (spread10(x) << 2) | (spread10(y) << 1) | spread10(z);
        }
        vals[s] = s;
    }
}

// Pass 2: persistent warps over the compacted pairs: a warp takes the next 32
// pairs (one light, 32 samples neighbouring in the trace order), so its lanes
// walk the BVH along nearby paths. Coherence pays for the lanes that wait on
// the warp's longest sphere trace: per-thread fetching, and lanes refilled
// from larger per-warp chunks, both measured slower on the mid scene.
// One traced (light, sample) pair w = light * n_samples + sample.
__device__ __forceinline__ void direct_pair_finish(const DirectArgs& a, u32 w, const DLight& L, const LightTerms& t,
                                                   float vis);

template <class Stack>
__device__ __forceinline__ void direct_pair(const DirectArgs& a, u32 w, u32& nq, u32& nv, u32& nt, Stack& st)
{
    int l = (int) (w / a.n_samples);
    u32 s = w % a.n_samples;
    const DLight L = a.lights[l];
    LightTerms t;
    light_terms(a, L, s, t);
    float vis = a.shadow_mode == 1 ? sampled_vis(a, L, t, st) : inv_shadow(a.bvh, t.from, t.to, L.radius, a.err, nq, nv, nt, st);
    direct_pair_finish(a, w, L, t, vis);
}

// The traced pairs of a warp (lanes with has = false take part without a
// pair), traced together: inv_shadow_warp for sphere-traced shadows,
// sampled_vis_warp for sampled ones.
__device__ __forceinline__ void direct_pair_warp(const DirectArgs& a, bool has, u32 w, u32& nq, u32& nv, u32& nt)
{
    DLight L = {};
    LightTerms t;
    t.from = t.to = t.dir = mk(0, 0, 0);
    if (has) {
        L = a.lights[w / a.n_samples];
        light_terms(a, L, w % a.n_samples, t);
    }
    const float vis = a.shadow_mode == 1 ? sampled_vis_warp(a, has, L, t)
                                         : inv_shadow_warp(a.bvh, has, t.from, t.to, L.radius, a.err, nq, nv, nt);
    if (has) direct_pair_finish(a, w, L, t, vis);
}

// Outputs of one traced pair from its shadow factor.
__device__ __forceinline__ void direct_pair_finish(const DirectArgs& a, u32 w, const DLight& L, const LightTerms& t,
                                                   float vis)
{
    const u32 s = w % a.n_samples;
    if (a.vis) a.vis[w] = vis;
    V3 Lcol = mk(L.color[0], L.color[1], L.color[2]);
    float kv, fac;
    if (L.type == 2) {
        kv = t.f_dist * t.f_ndotl * t.f_dir * vis;
        fac = t.f_dist * t.f_dir * vis * t.f_ndotl * brightness(Lcol);
    } else if (L.type == 1) {
        kv = t.f_dist * t.f_ndotl * vis;
        fac = t.f_dist * vis * t.f_ndotl * brightness(Lcol);
    } else {
        kv = t.f_ndotl * vis;
        fac = vis * t.f_ndotl * brightness(Lcol);
    }
    a.kval[w] = kv;
    if (a.ndir && a.sinst[s] != 0 && fac > 0) a.ndir[w] = st4(t.dir * fac, 1.0f);
}

// kMinBlocks 2 caps the registers at 64 (two blocks of 512 threads per SM):
// more warps in flight for the latency-bound walks, at the price of a few
// spills; which is faster depends on the scene (tuning direct_regs).
// The shadow-trace kernel: k_direct_trace as compiled for blocks of up to 512
// threads, k_direct_trace_capped with at most kRegCap registers per thread (64,
// 72, 80: more warps per SM for the latency-bound walks, at the price of
// spills; tuning direct_regs / sampled_regs). kStackK:
// traversal-stack entries kept in shared memory by the per-lane walks (TStack;
// tuning direct_stack). kPacket: the shadow traces of a warp's 32 pairs run
// together (inv_shadow_warp, sampled_vis_warp; tuning direct_packet).
template <int kStackK, bool kPacket>
__device__ __forceinline__ void direct_trace_body(const DirectArgs& a, const u32* __restrict__ items,
                                                  const u32* __restrict__ n_items_dev, u32* __restrict__ next)
{
    extern __shared__ __align__(16) unsigned char smem[];
    TStack<kStackK> st = make_stack<kStackK>(smem);
    unsigned long long c_traced = 0, c_nq = 0, c_nv = 0, c_nt = 0, c_pairs = 0;
    const u32 n_items = *n_items_dev;
    const int lane = threadIdx.x & 31;
    for (;;) {
        u32 base = 0;
        if (lane == 0) {
            base = atomicAdd(next, 32u);
            if (a.abort_word && *a.abort_word) base = n_items;   // ltr_Abort: take no more work
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        const u32 i = base + lane;
        if (kPacket) {
            const bool has = i < n_items;
            u32 nq = 0, nv = 0, nt = 0;
            const u32 w = has ? items[i] : 0u;
            direct_pair_warp(a, has, w, nq, nv, nt);
            if (has) {
                c_traced += a.shadow_mode == 1 ? (unsigned) a.lights[w / a.n_samples].ns : 1u;
                c_pairs += 1;
                c_nq += nq;
                c_nv += nv;
                c_nt += nt;
            }
        } else if (i < n_items) {
            u32 nq = 0, nv = 0, nt = 0;
            const u32 w = items[i];
            direct_pair(a, w, nq, nv, nt, st);
            c_traced += a.shadow_mode == 1 ? (unsigned) a.lights[w / a.n_samples].ns : 1u;
            c_pairs += 1;
            c_nq += nq;
            c_nv += nv;
            c_nt += nt;
        }
    }
    if (a.counters) {
        warp_add(&a.counters->shadow_pairs, c_pairs);
        warp_add(&a.counters->shadow_evals, c_traced);
        warp_add(&a.counters->distance_queries, c_nq);
        warp_add(&a.counters->node_visits, c_nv);
        warp_add(&a.counters->tri_tests, c_nt);
    }
}

template <int kRegCap, int kStackK, bool kPacket>
__global__ void __launch_bounds__(512) __maxnreg__(kRegCap)
    k_direct_trace_capped(DirectArgs a, const u32* __restrict__ items, const u32* __restrict__ n_items_dev,
                          u32* __restrict__ next)
{
    direct_trace_body<kStackK, kPacket>(a, items, n_items_dev, next);
}

template <int kStackK, bool kPacket>
__global__ void __launch_bounds__(512, 1)
    k_direct_trace(DirectArgs a, const u32* __restrict__ items, const u32* __restrict__ n_items_dev, u32* __restrict__ next)
{
    direct_trace_body<kStackK, kPacket>(a, items, n_items_dev, next);
}

// Per sample, ambient plus every light's term in light order (lighter.cpp:504, 542, 589).
__global__ void k_accumulate(u32 n_samples, int n_lights, const DLight* __restrict__ lights, const float* __restrict__ kval,
                             float amb_r, float amb_g, float amb_b, float4* __restrict__ lm)
{
    u32 s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_samples) return;
    V3 c = mk(amb_r, amb_g, amb_b);
    for (int l = 0; l < n_lights; ++l) {
        float k = kval[(size_t) l * n_samples + s];
        if (k != 0.0f) c += mk(lights[l].color[0], lights[l].color[1], lights[l].color[2]) * k;
    }
    lm[s] = st4(c, 0.0f);
}

// ----------------------------------------------------------------------------- radiosity inputs

// One radiosity element per sample (lighter.cpp:676-718): unit normal,
// sample_fn albedo and the sample's area (0 and black for probes), emission =
// lit colour + sample_fn emission.
__global__ void k_rad_sample_inputs(u32 n, const float4* __restrict__ spos, const float4* __restrict__ snrm,
                                    const float4* __restrict__ srad, const u32* __restrict__ sinst,
                                    const float4* __restrict__ diff, const float4* __restrict__ emis,
                                    const float4* __restrict__ lm, float4* __restrict__ pos, float4* __restrict__ nrm,
                                    float4* __restrict__ da, float4* __restrict__ emit)
{
    u32 s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    pos[s] = spos[s];
    nrm[s] = st4(normalized(ld3(snrm[s])), 0.0f);
    float4 d = diff[s];
    da[s] = make_float4(d.x, d.y, d.z, sinst[s] == 0 ? 0.0f : srad[s].w);
    V3 e = ld3(lm[s]);
    e += ld3(emis[s]);
    emit[s] = st4(e, 0.0f);
}

// ltrg_TableSampleFn (api.cpp) evaluated on the device with the same
// contract: the entry is chosen by (u32) tex0u (radinfo.x); negative or
// out-of-range ids keep the defaults (albedo 1, no emission); probes are
// black (lighter.cpp:685-714). has_fn = 0 stands for a NULL sample_fn.
__global__ void k_table_samples(u32 n, const float4* __restrict__ srad, const u32* __restrict__ sinst, int has_fn,
                                u32 count, const float* __restrict__ tdiff, const float* __restrict__ temis,
                                float4* __restrict__ diff, float4* __restrict__ emis)
{
    u32 s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    V3 d = mk(1, 1, 1), e = mk(0, 0, 0);
    if (sinst[s] == 0) {
        d = mk(0, 0, 0);
    } else if (has_fn) {
        float fid = srad[s].x;
        if (fid >= 0.0f) {
            u32 id = (u32) fid;
            if (id < count) {
                if (tdiff) d = mk(tdiff[3 * id], tdiff[3 * id + 1], tdiff[3 * id + 2]);
                if (temis) e = mk(temis[3 * id], temis[3 * id + 1], temis[3 * id + 2]);
            }
        }
    }
    diff[s] = st4(d, 0.0f);
    emis[s] = st4(e, 0.0f);
}

// Patch slot of a sample: (instance, lightmap tile, dominant axis of its
// unit normal); marks the slot occupied. With n_occ set, counts the occupied
// slots instead (a trial of a tile size).
__global__ void k_patch_slots(u32 n, const float4* __restrict__ snrm, const u32* __restrict__ sloc,
                              const u32* __restrict__ sinst, const u32* __restrict__ inst_w,
                              const u32* __restrict__ slot_base, const u32* __restrict__ ntx, u32 tile,
                              u32* __restrict__ slot_of, u32* __restrict__ occ, u32* __restrict__ n_occ)
{
    u32 s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    u32 inst = sinst[s];
    if (inst == 0) { slot_of[s] = 0xffffffffu; return; }
    u32 w = inst_w[inst], L = sloc[s];
    u32 tx = (L % w) / tile, ty = (L / w) / tile;
    V3 nn = normalized(ld3(snrm[s]));
    float ax = fabsf(nn.x), ay = fabsf(nn.y), az = fabsf(nn.z);
    u32 axis = (ax >= ay && ax >= az) ? (nn.x >= 0 ? 0 : 1) : (ay >= az ? (nn.y >= 0 ? 2 : 3) : (nn.z >= 0 ? 4 : 5));
    u32 slot = slot_base[inst] + (ty * ntx[inst] + tx) * 6 + axis;
    if (n_occ) {
        if (occ[slot] == 0 && atomicExch(&occ[slot], 1u) == 0) atomicAdd(n_occ, 1u);
        return;
    }
    slot_of[s] = slot;
    occ[slot] = 1;
}

// Patch id = rank of the slot among occupied slots; (patch, sample) pairs
// of the covered samples for the stable sort that lists each patch's samples.
__global__ void k_patch_ids(u32 n, u32 n_probe, const u32* __restrict__ slot_of, const u32* __restrict__ slot_scan,
                            int* __restrict__ patch_of, u32* __restrict__ keys, u32* __restrict__ vals)
{
    u32 s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    u32 slot = slot_of[s];
    int p = slot == 0xffffffffu ? -1 : (int) slot_scan[slot];
    patch_of[s] = p;
    if (s >= n_probe) {
        keys[s - n_probe] = (u32) p;
        vals[s - n_probe] = s;
    }
}

// First position of each patch in the sorted list (every patch id occurs).
__global__ void k_patch_offsets(u32 n, u32 np, const u32* __restrict__ sorted_keys, u32* __restrict__ off)
{
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u32 k = sorted_keys[i];
    if (i == 0 || sorted_keys[i - 1] != k) off[k] = i;
    if (i == 0) off[np] = n;
}

// Patch element from its samples (in sample order): total area and
// area-weighted position, normal, albedo and emission, accumulated in FP64.
__global__ void k_patch_inputs(u32 np, const u32* __restrict__ off, const u32* __restrict__ idx,
                               const float4* __restrict__ spos, const float4* __restrict__ snrm,
                               const float4* __restrict__ srad, const float4* __restrict__ diff,
                               const float4* __restrict__ emis, const float4* __restrict__ lm, float4* __restrict__ ppos,
                               float4* __restrict__ pnrm, float4* __restrict__ pda, float4* __restrict__ pemit)
{
    // one warp per patch: lanes take every 32nd sample of the patch's list, then
    // a fixed shuffle tree sums the lanes (deterministic order)
    const int lane = threadIdx.x & 31;
    const u32 p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (p >= np) return;
    double q[13] = {0};
    for (u32 k = off[p] + lane; k < off[p + 1]; k += 32) {
        u32 s = idx[k];
        double a = srad[s].w;
        V3 n = normalized(ld3(snrm[s]));
        float4 P = spos[s], D = diff[s];
        V3 e = ld3(lm[s]);
        e += ld3(emis[s]);
        q[0] += a;
        q[1] += a * P.x; q[2] += a * P.y; q[3] += a * P.z;
        q[4] += a * n.x; q[5] += a * n.y; q[6] += a * n.z;
        q[7] += a * D.x; q[8] += a * D.y; q[9] += a * D.z;
        q[10] += a * e.x; q[11] += a * e.y; q[12] += a * e.z;
    }
#pragma unroll
    for (int c = 0; c < 13; ++c)
        for (int o = 16; o > 0; o >>= 1) q[c] += __shfl_down_sync(0xffffffffu, q[c], o);
    if (lane != 0) return;
    double a = q[0] > 0 ? q[0] : 1.0;
    V3 nn = normalized(mk((float) (q[4] / a), (float) (q[5] / a), (float) (q[6] / a)));
    ppos[p] = make_float4((float) (q[1] / a), (float) (q[2] / a), (float) (q[3] / a), 0);
    pnrm[p] = st4(nn, 0.0f);
    pda[p] = make_float4((float) (q[7] / a), (float) (q[8] / a), (float) (q[9] / a), (float) q[0]);
    pemit[p] = make_float4((float) (q[10] / a), (float) (q[11] / a), (float) (q[12] / a), 0);
}

// Texel colour = its own emission + its patch's gathered light.
__global__ void k_patch_apply(u32 n, const int* __restrict__ patch_of, const float4* __restrict__ emis,
                              const float4* __restrict__ ptot, const float4* __restrict__ pemit, float4* lm)
{
    u32 s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    V3 e = ld3(lm[s]);
    e += ld3(emis[s]);
    int p = patch_of[s];
    if (p >= 0) {
        e.x += ptot[p].x - pemit[p].x;
        e.y += ptot[p].y - pemit[p].y;
        e.z += ptot[p].z - pemit[p].z;
    }
    lm[s] = st4(e, 0.0f);
}

// ----------------------------------------------------------------------------- ambient occlusion

__device__ __forceinline__ V3 spiral_dir(V3 dir, float randoff, int i, int count)
{
    float q = (i + 0.5f) / count;
    float cos_side = sqrtf(q);
    float sin_side = sinf(acosf(cos_side));
    float angle = (i + randoff) * (137.508f / 180.0f * 3.14159265358979323846f);
    float ca = cosf(angle), sa = sinf(angle);
    V3 diffvec = mk(dir.y, -dir.z, dir.x);
    V3 up = normalized(cross(dir, diffvec));
    V3 rt = cross(dir, up);
    return ca * sin_side * rt + sa * sin_side * up + cos_side * dir;
}

struct AoArgs {
    BvhView bvh;
    ErrFlag err;
    u32 n_samples;
    const float4* spos;
    const float4* snrm;
    const float* randoff;
    float4* lm;
    float dist, falloff, mult, effect;
    int ns;
    float aoc[3];
    Counters* counters;
    const u32* order;   // samples in trace order (see k_order_keys)
    const volatile u32* abort_word;   // mapped host word set by ltr_Abort (may be null)
};

// Job_AORender_Inner (lighter.cpp:799-841), pass 1: every (sample, ray) is an
// independent closest-hit query; persistent warps take 32 x ao_chunk rays at a
// time (see ao_item for their order) and store the hit fractions. One ray per
// lane per fetch measured fastest (mid scene: 9.2 ms against 16.0 ms with four):
// a lane that ends its ray early waits for the warp's longest ray only once
// instead of running ahead into its next ray on a diverged path. The batch
// kernel takes kAoChunk rays per lane as well.
constexpr unsigned kAoChunk = 1;

// Ray r of sample s (i = s * ns + r): closest-hit fraction along the AO segment.
template <class Stack>
__device__ __forceinline__ void ao_ray(const AoArgs& a, float* __restrict__ hits, unsigned long long i, Stack& st)
{
    u32 s = (u32) (i / a.ns);
    int r = (int) (i % a.ns);
    V3 SP = ld3(a.spos[s]), SN = ld3(a.snrm[s]);
    V3 ro = SP + SN * (kSmall * 2);
    V3 rd = spiral_dir(SN, a.randoff[s], r, a.ns) * a.dist;
    V3 B = ro + rd;
    V3 dn = normalized(B - ro);
    hits[i] = bvh_closest_s(a.bvh, ro + dn * kSmall, B - dn * kSmall, a.err, nullptr, st);
}

// AO work items in sample-tile order: tiles of 32 consecutive samples, and in a
// tile, ray r of the 32 samples are items 32 r .. 32 r + 31. A warp takes 32 x
// kAoChunk items and lane l traces items base + l + 32 k, so at every step its
// lanes trace the same spiral direction from 32 neighbouring samples (coherent
// traversals). Only the assignment of rays to threads changes: each hit lands
// in its own slot s * ns + r, which the ordered reduction reads.
__host__ __device__ __forceinline__ unsigned long long ao_items(u32 n_samples, int ns)
{
    return ((unsigned long long) (n_samples + 31) / 32) * 32ull * (unsigned long long) ns;
}

__device__ __forceinline__ bool ao_item(unsigned long long g, u32 n_samples, int ns, const u32* order,
                                        unsigned long long& i)
{
    const unsigned long long per_tile = 32ull * (unsigned long long) ns;
    const unsigned long long tile = g / per_tile, w = g % per_tile;
    const unsigned long long rank = tile * 32 + w % 32;
    if (rank >= n_samples) return false;
    const unsigned long long s = order ? order[rank] : rank;
    i = s * (unsigned long long) ns + w / 32;
    return true;
}

// AO ray of item g for every lane of a warp at once (warp_closest); lanes
// whose item is past the end or past the samples take part without a ray.
__device__ __forceinline__ bool ao_ray_warp(const AoArgs& a, float* __restrict__ hits, unsigned long long g,
                                            unsigned long long n_items)
{
    unsigned long long i = 0;
    const bool has = g < n_items && ao_item(g, a.n_samples, a.ns, a.order, i);
    V3 A = mk(0, 0, 0), B = mk(0, 0, 0);
    if (has) {
        const u32 s = (u32) (i / a.ns);
        const int r = (int) (i % a.ns);
        const V3 SP = ld3(a.spos[s]), SN = ld3(a.snrm[s]);
        const V3 ro = SP + SN * (kSmall * 2);
        const V3 rd = spiral_dir(SN, a.randoff[s], r, a.ns) * a.dist;
        const V3 E = ro + rd;
        const V3 dn = normalized(E - ro);
        A = ro + dn * kSmall;
        B = E - dn * kSmall;
    }
    const float h = warp_closest(a.bvh, A, B, has, a.err);
    if (has) hits[i] = h;
    return has;
}

// kStackK: traversal-stack entries kept in shared memory (TStack; tuning
// ao_stack); `chunk`: rays per lane per work fetch (tuning ao_chunk);
// kPacket: the warp's 32 rays of a step share one walk (ao_ray_warp; tuning
// ao_packet).
template <int kStackK, bool kPacket = false>
__global__ void k_ao_rays(AoArgs a, float* __restrict__ hits, unsigned long long n_items, unsigned long long* next,
                          unsigned chunk)
{
    extern __shared__ __align__(16) unsigned char smem[];
    TStack<kStackK> st = make_stack<kStackK>(smem);
    const int lane = threadIdx.x & 31;
    unsigned long long c_rays = 0;
    for (u32 fetch = 0;; ++fetch) {
        unsigned long long base = 0;
        if (lane == 0) {
            base = atomicAdd(next, 32ull * chunk);
            // ltr_Abort: take no more work (polled every 16th fetch: an AO fetch is short)
            if (a.abort_word && (fetch & 15u) == 0 && *a.abort_word) base = n_items;
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        for (unsigned k = 0; k < chunk; ++k) {
            const unsigned long long g = base + 32ull * k + lane;
            if (kPacket) {
                if (ao_ray_warp(a, hits, g, n_items)) ++c_rays;
                continue;
            }
            unsigned long long i;
            if (g < n_items && ao_item(g, a.n_samples, a.ns, a.order, i)) {
                ao_ray(a, hits, i, st);
                ++c_rays;
            }
        }
    }
    if (a.counters) warp_add(&a.counters->ao_rays, c_rays);
}

// Launch of the two trace kernels with the tuning's register budget, stack
// split, walk sharing and wavefront size. Dynamic shared memory: the short
// stacks, K entries of 8 bytes per thread.
template <int kRegCap, int K, bool kPacket = false>
void launch_direct_k(unsigned grid, unsigned block, cudaStream_t st, const DirectArgs& da, const u32* items,
                     const u32* n_items, u32* next)
{
    const size_t smem = (size_t) K * block * 8;
    if constexpr (kRegCap == 128) {
        if (smem > 48 * 1024)
            CK(cudaFuncSetAttribute(k_direct_trace<K, kPacket>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
        k_direct_trace<K, kPacket><<<grid, block, smem, st>>>(da, items, n_items, next);
    } else {
        if (smem > 48 * 1024)
            CK(cudaFuncSetAttribute(k_direct_trace_capped<kRegCap, K, kPacket>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
        k_direct_trace_capped<kRegCap, K, kPacket><<<grid, block, smem, st>>>(da, items, n_items, next);
    }
}

// The shared-memory stack split is built for the per-lane walks with 128 and
// 64 registers; the other budgets run the per-lane walks with local stacks.
template <int kRegCap>
void launch_direct_r(unsigned stack, bool packet, unsigned grid, unsigned block, cudaStream_t st, const DirectArgs& da,
                     const u32* items, const u32* n_items, u32* next)
{
    if (packet) {   // the warp's walks share one stack in registers; the shared-memory split does not apply
        launch_direct_k<kRegCap, 0, true>(grid, block, st, da, items, n_items, next);
        return;
    }
    if constexpr (kRegCap == 128 || kRegCap == 64) {
        switch (stack) {
        case 4: launch_direct_k<kRegCap, 4>(grid, block, st, da, items, n_items, next); return;
        case 8: launch_direct_k<kRegCap, 8>(grid, block, st, da, items, n_items, next); return;
        case 16: launch_direct_k<kRegCap, 16>(grid, block, st, da, items, n_items, next); return;
        default: break;
        }
    }
    launch_direct_k<kRegCap, 0>(grid, block, st, da, items, n_items, next);
}

void launch_direct_trace(const ltrg_Tuning& tu, unsigned grid, cudaStream_t st, const DirectArgs& da, const u32* items,
                         const u32* n_items, u32* next)
{
    const bool packet = tu.direct_packet != 0;
    const u32 regs = da.shadow_mode == LTRG_SHADOW_SAMPLED ? tu.sampled_regs : tu.direct_regs;
    switch (regs) {
    case 1: launch_direct_r<64>(tu.direct_stack, packet, grid, tu.direct_block, st, da, items, n_items, next); break;
    case 2: launch_direct_r<72>(tu.direct_stack, packet, grid, tu.direct_block, st, da, items, n_items, next); break;
    case 3: launch_direct_r<80>(tu.direct_stack, packet, grid, tu.direct_block, st, da, items, n_items, next); break;
    default: launch_direct_r<128>(tu.direct_stack, packet, grid, tu.direct_block, st, da, items, n_items, next); break;
    }
}

template <int K, bool kPacket = false>
void launch_ao_k(unsigned grid, unsigned block, cudaStream_t st, const AoArgs& aa, float* hits,
                 unsigned long long n_items, unsigned long long* next, unsigned chunk)
{
    const size_t smem = (size_t) K * block * 8;
    if (smem > 48 * 1024)
        CK(cudaFuncSetAttribute(k_ao_rays<K, kPacket>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
    k_ao_rays<K, kPacket><<<grid, block, smem, st>>>(aa, hits, n_items, next, chunk);
}

void launch_ao_rays(const ltrg_Tuning& tu, unsigned grid, cudaStream_t st, const AoArgs& aa, float* hits,
                    unsigned long long n_items, unsigned long long* next)
{
    const unsigned chunk = tu.ao_chunk ? tu.ao_chunk : kAoChunk;
    if (tu.ao_packet) {   // one shared walk per step: the shared-memory stack split does not apply
        launch_ao_k<0, true>(grid, tu.ao_block, st, aa, hits, n_items, next, chunk);
        return;
    }
    switch (tu.ao_stack) {
    case 4: launch_ao_k<4>(grid, tu.ao_block, st, aa, hits, n_items, next, chunk); break;
    case 8: launch_ao_k<8>(grid, tu.ao_block, st, aa, hits, n_items, next, chunk); break;
    case 16: launch_ao_k<16>(grid, tu.ao_block, st, aa, hits, n_items, next, chunk); break;
    default: launch_ao_k<0>(grid, tu.ao_block, st, aa, hits, n_items, next, chunk); break;
    }
}

// ----------------------------------------------------------------------------- batches of scenes
// A batch of scenes (ltrg_StartBatch) traces the direct-light pairs and the AO
// rays of all its scenes in one persistent launch each: job k holds scene k's
// arguments and work list, off[] the exclusive prefix sums of the jobs' item
// counts; item g belongs to the job k with off[k] <= g < off[k + 1].

struct DirectJob {
    DirectArgs args;
    const u32* items;   // traced pairs (light * n_samples + sample)
    const u32* count;   // device: number of items (null: none)
};

struct AoJob {
    AoArgs args;
    float* hits;        // n_samples * ns hit fractions
};

__device__ __forceinline__ int find_job(const unsigned long long* __restrict__ off, int n, unsigned long long g)
{
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Job k's items take [off[k], off[k] + count_k) of the batch's item space, and
// off[k + 1] - off[k] is count_k rounded up to a multiple of 32: a warp's 32
// items (the kernel hands out 32 at a time) then always come from one job, so
// its lanes can share a BVH walk; the items of the padding are skipped.
__global__ void k_direct_batch_offsets(const DirectJob* __restrict__ jobs, int n, unsigned long long* __restrict__ off)
{
    if (blockIdx.x || threadIdx.x) return;
    unsigned long long acc = 0;
    for (int k = 0; k < n; ++k) {
        off[k] = acc;
        acc += ((jobs[k].count ? *jobs[k].count : 0u) + 31ull) / 32ull * 32ull;
    }
    off[n] = acc;
}

__device__ __forceinline__ void flush_direct(Counters* c, unsigned long long& tr, unsigned long long& nq,
                                             unsigned long long& nv, unsigned long long& nt, unsigned long long& np)
{
    if (c && tr) {
        atomicAdd(&c->shadow_pairs, np);
        atomicAdd(&c->shadow_evals, tr);
        atomicAdd(&c->distance_queries, nq);
        atomicAdd(&c->node_visits, nv);
        atomicAdd(&c->tri_tests, nt);
    }
    tr = nq = nv = nt = np = 0;
}

// kPacket: a warp's 32 pairs (all of one scene) share their walks
// (direct_pair_warp), as in k_direct_trace; otherwise each lane walks alone.
template <bool kPacket>
__global__ void k_direct_trace_batch(const DirectJob* __restrict__ jobs, int n, const unsigned long long* __restrict__ off,
                                     unsigned long long* __restrict__ next)
{
    const unsigned long long total = off[n];
    unsigned long long c_traced = 0, c_nq = 0, c_nv = 0, c_nt = 0, c_pairs = 0;
    int cur = -1;
    DirectArgs a;
    const u32* items = nullptr;
    unsigned long long base = 0;
    u32 count = 0;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(next, 32ull);
        wb = __shfl_sync(0xffffffffu, wb, 0);
        if (wb >= total) break;
        const int k = find_job(off, n, wb);   // the warp's job (job ranges are multiples of 32)
        if (k != cur) {
            if (cur >= 0) flush_direct(a.counters, c_traced, c_nq, c_nv, c_nt, c_pairs);
            cur = k;
            a = jobs[k].args;
            items = jobs[k].items;
            base = off[k];
            count = jobs[k].count ? *jobs[k].count : 0u;
        }
        const unsigned long long i = wb + lane - base;
        const bool has = i < count;
        u32 nq = 0, nv = 0, nt = 0;
        const u32 w = has ? items[i] : 0u;
        if (kPacket) {
            direct_pair_warp(a, has, w, nq, nv, nt);
        } else if (has) {
            TStack<0> st;
            direct_pair(a, w, nq, nv, nt, st);
        }
        if (has) {
            c_traced += a.shadow_mode == 1 ? (unsigned) a.lights[w / a.n_samples].ns : 1u;
            c_pairs += 1;
        }
        c_nq += nq;
        c_nv += nv;
        c_nt += nt;
    }
    if (cur >= 0) flush_direct(a.counters, c_traced, c_nq, c_nv, c_nt, c_pairs);
}

// Job ranges are ao_items long, a multiple of 32: a warp's 32 rays of a step
// are one scene's, so with kPacket they share one walk (ao_ray_warp).
template <bool kPacket>
__global__ void k_ao_rays_batch(const AoJob* __restrict__ jobs, int n, const unsigned long long* __restrict__ off,
                                unsigned long long* __restrict__ next)
{
    const unsigned long long total = off[n];
    const int lane = threadIdx.x & 31;
    unsigned long long c_rays = 0;
    int cur = -1;
    AoArgs a;
    float* hits = nullptr;
    unsigned long long job0 = 0;
    for (;;) {
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(next, 32ull * kAoChunk);
        wb = __shfl_sync(0xffffffffu, wb, 0);
        if (wb >= total) break;
        for (unsigned kk = 0; kk < kAoChunk; ++kk) {
            const unsigned long long gw = wb + 32ull * kk;   // the warp's first item of this step
            if (gw >= total) break;
            const unsigned long long g = gw + lane;
            const int k = find_job(off, n, gw);
            if (k != cur) {
                if (cur >= 0 && a.counters && c_rays) atomicAdd(&a.counters->ao_rays, c_rays);
                c_rays = 0;
                cur = k;
                a = jobs[k].args;
                hits = jobs[k].hits;
                job0 = off[k];
            }
            if (kPacket) {
                if (ao_ray_warp(a, hits, g - job0, off[k + 1] - job0)) ++c_rays;
                continue;
            }
            unsigned long long i;
            if (ao_item(g - job0, a.n_samples, a.ns, a.order, i)) {
                TStack<0> st;
                ao_ray(a, hits, i, st);
                ++c_rays;
            }
        }
    }
    if (cur >= 0 && a.counters && c_rays) atomicAdd(&a.counters->ao_rays, c_rays);
}

// Pass 2: per sample, the hit fractions summed in ray order like the
// reference loop, then the AO factor and colour blend.
__global__ void k_ao(AoArgs a, const float* __restrict__ hits)
{
    for (unsigned long long s = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; s < a.n_samples;
         s += (unsigned long long) gridDim.x * blockDim.x) {
        const float* h = hits + s * (unsigned long long) a.ns;
        float f = 0;
        if ((a.ns & 3) == 0) {   // 16-byte loads (each sample's run starts on a 16-byte boundary); same order
            const float4* h4 = reinterpret_cast<const float4*>(h);
            for (int r = 0; r < a.ns / 4; ++r) {
                const float4 v = __ldcs(&h4[r]);
                if (v.x < 1.0f) f += 1.0f - v.x;
                if (v.y < 1.0f) f += 1.0f - v.y;
                if (v.z < 1.0f) f += 1.0f - v.z;
                if (v.w < 1.0f) f += 1.0f - v.w;
            }
        } else {
            for (int r = 0; r < a.ns; ++r) {
                float v = h[r];
                if (v < 1.0f) f += 1.0f - v;
            }
        }
        {
            f /= a.ns;
            f = fmin_(f * a.mult, 1.0f);
            if (a.falloff) f = powf(f, a.falloff);
            V3 out = ld3(a.lm[s]);
            V3 aoc = mk(a.aoc[0], a.aoc[1], a.aoc[2]);
            if (a.effect >= 0) out = out * (1 - f * (1 - a.effect)) + aoc * f;
            else out = lerp3(out, lerp3(aoc, aoc * out, -a.effect), f);
            a.lm[s] = st4(out, 0.0f);
        }
    }
}

// ----------------------------------------------------------------------------- finalize

__device__ __forceinline__ int find_inst(const unsigned long long* off, int n_inst, unsigned long long g)
{
    int lo = 1, hi = n_inst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_scatter(u32 n_probe, u32 n_samples, const u32* __restrict__ sloc, const u32* __restrict__ sinst,
                          const float4* __restrict__ lm, const unsigned long long* __restrict__ tex_off,
                          float* __restrict__ img, unsigned char* __restrict__ mask)
{
    u32 s = n_probe + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_samples) return;
    unsigned long long g = tex_off[sinst[s]] + sloc[s];
    float4 c = lm[s];
    img[3 * g + 0] = c.x;
    img[3 * g + 1] = c.y;
    img[3 * g + 2] = c.z;
    mask[g] = 1;
}

// One extrapolating dilation sweep (lighter.cpp:884-943): `old` is the mask
// before the sweep, `next` receives newly set texels; colours of texels set
// in `old` are never written during the sweep, so reading them is race-free.
__global__ void k_dilate(unsigned long long ntex, int n_inst, const unsigned long long* __restrict__ tex_off,
                         const u32* __restrict__ inst_w, const u32* __restrict__ inst_h,
                         const unsigned char* __restrict__ old, unsigned char* __restrict__ next, float* img)
{
    for (unsigned long long g = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; g < ntex;
         g += (unsigned long long) gridDim.x * blockDim.x) {
        if (old[g]) continue;
        int inst = find_inst(tex_off, n_inst, g);
        unsigned long long base = tex_off[inst];
        u32 w = inst_w[inst], h = inst_h[inst];
        unsigned long long local = g - base;
        u32 x = (u32) (local % w), y = (u32) (local / w);
        auto isset = [&](u32 xx, u32 yy) { return xx < w && yy < h && old[base + xx + (unsigned long long) yy * w]; };
        auto col = [&](u32 xx, u32 yy) {
            const float* p = img + 3 * (base + xx + (unsigned long long) yy * w);
            return mk(p[0], p[1], p[2]);
        };
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

// Row convolution with clamp-to-edge taps, written transposed
// (Convolve_Transpose, lighter_math.cpp:367-398). `transposed` selects the
// second pass, whose input rows are the instance's columns.
__global__ void k_conv_t(unsigned long long ntex, int n_inst, const unsigned long long* __restrict__ tex_off,
                         const u32* __restrict__ inst_w, const u32* __restrict__ inst_h, int transposed, int ext,
                         const float* __restrict__ kern, const float* __restrict__ src, float* __restrict__ dst)
{
    for (unsigned long long g = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; g < ntex;
         g += (unsigned long long) gridDim.x * blockDim.x) {
        int inst = find_inst(tex_off, n_inst, g);
        unsigned long long base = tex_off[inst];
        u32 W = transposed ? inst_h[inst] : inst_w[inst];
        u32 H = transposed ? inst_w[inst] : inst_h[inst];
        unsigned long long local = g - base;
        u32 x = (u32) (local % W), y = (u32) (local / W);
        const float* row = src + 3 * (base + (unsigned long long) y * W);
        float s0 = 0, s1 = 0, s2 = 0;
        for (int i = -ext; i <= ext; ++i) {
            int xx = (int) x + i;
            xx = xx < 0 ? 0 : (xx >= (int) W ? (int) W - 1 : xx);
            float kq = kern[i + ext];
            s0 += row[3 * xx + 0] * kq;
            s1 += row[3 * xx + 1] * kq;
            s2 += row[3 * xx + 2] * kq;
        }
        float* o = dst + 3 * (base + y + (unsigned long long) H * x);
        o[0] = s0; o[1] = s1; o[2] = s2;
    }
}

// Downsample2X (lighter_math.cpp:400-424) into a separate per-instance layout.
// Radiance RGBE of float RGB texels (Ward's shared-exponent format, "Real Pixels",
// Graphics Gems II): v = the largest channel (negatives clamp to 0); for
// v > 1e-32, v = m 2^e with m in [0.5, 1), each channel becomes
// min(255, floor(c m 256 / v)) and the fourth byte e + 128; else all four are 0.
// Computed in double, as the host encoder does, so both give the same bytes.
__global__ void k_encode_rgbe(unsigned long long n, const float* __restrict__ rgb, uchar4* __restrict__ out)
{
    for (unsigned long long g = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; g < n;
         g += (unsigned long long) gridDim.x * blockDim.x) {
        const double r = fmax((double) rgb[3 * g], 0.0), gr = fmax((double) rgb[3 * g + 1], 0.0),
                     b = fmax((double) rgb[3 * g + 2], 0.0);
        const double v = fmax(r, fmax(gr, b));
        uchar4 o = make_uchar4(0, 0, 0, 0);
        if (v > 1e-32) {
            int e = 0;
            const double m = frexp(v, &e);
            const double sc = m * 256.0 / v;
            o.x = (unsigned char) fmin(floor(r * sc), 255.0);
            o.y = (unsigned char) fmin(floor(gr * sc), 255.0);
            o.z = (unsigned char) fmin(floor(b * sc), 255.0);
            o.w = (unsigned char) (e + 128);
        }
        out[g] = o;
    }
}

__global__ void k_ds2x(unsigned long long nout, int n_inst, const unsigned long long* __restrict__ out_off,
                       const unsigned long long* __restrict__ tex_off, const u32* __restrict__ inst_w,
                       const u32* __restrict__ inst_h, const float* __restrict__ src, float* __restrict__ dst)
{
    for (unsigned long long g = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; g < nout;
         g += (unsigned long long) gridDim.x * blockDim.x) {
        int inst = find_inst(out_off, n_inst, g);
        u32 w = inst_w[inst], h = inst_h[inst];
        u32 hw = max(w / 2, 1u);
        unsigned long long local = g - out_off[inst];
        u32 x = (u32) (local % hw), y = (u32) (local / hw);
        u32 sx0 = (x * 2) % w, sy0 = (y * 2) % h, sx1 = (x * 2 + 1) % w, sy1 = (y * 2 + 1) % h;
        const float* b = src + 3 * tex_off[inst];
        auto col = [&](u32 xx, u32 yy) { const float* p = b + 3 * (xx + (unsigned long long) yy * w); return mk(p[0], p[1], p[2]); };
        V3 avg = (col(sx0, sy0) + col(sx1, sy0) + col(sx0, sy1) + col(sx1, sy1)) * 0.25f;
        float* o = dst + 3 * g;
        o[0] = avg.x; o[1] = avg.y; o[2] = avg.z;
    }
}

// Normal/"focus" data per sample (lighter.cpp:977-1027): ambient-weighted
// normal plus the recorded light directions in light order, then the product
// of the per-light agreement terms.
__global__ void k_normals(u32 n_probe, u32 n_samples, int n_lights, const float4* __restrict__ ndir,
                          const float4* __restrict__ snrm, const u32* __restrict__ sloc, const u32* __restrict__ sinst,
                          const unsigned long long* __restrict__ nout_off, const u32* __restrict__ cap, float amb,
                          float* __restrict__ out)
{
    u32 s = n_probe + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_samples) return;
    V3 n = ld3(snrm[s]) * amb;
    int cnt = 1;
    for (int l = 0; l < n_lights; ++l) {
        float4 c = ndir[(size_t) l * n_samples + s];
        if (c.w != 0.0f) { n += ld3(c); cnt++; }
    }
    n = n / (float) cnt;
    float mindot = 1;
    for (int l = 0; l < n_lights; ++l) {
        float4 c = ndir[(size_t) l * n_samples + s];
        if (c.w == 0.0f) continue;
        V3 cn = ld3(c);
        float d = fmax_(dot(normalized(n), normalized(cn)), 0.0f);
        float t = fmin_(len(cn) / len(n), 1.0f);
        d = 1.0f * (1.0f - t) + d * t;
        mindot *= d;
    }
    u32 inst = sinst[s];
    if (sloc[s] >= cap[inst]) return;   // ds2x shrinks the image but keeps full-size texel ids
    V3 N = normalized(n);
    float* o = out + 4 * (nout_off[inst] + sloc[s]);
    o[0] = N.x; o[1] = N.y; o[2] = N.z; o[3] = mindot;
}

// ----------------------------------------------------------------------------- host helpers

// Device arena: every buffer of one bake, freed (stream-ordered) at the end.
struct Arena {
    cudaStream_t st = nullptr;
    std::vector<void*> ptrs;
    size_t bytes = 0;
    template <class T> T* alloc(size_t n)
    {
        void* p = nullptr;
        size_t b = (n ? n : 1) * sizeof(T);
        CK(cudaMallocAsync(&p, b, st));
        ptrs.push_back(p);
        bytes += b;
        return (T*) p;
    }
    template <class T> T* upload(const std::vector<T>& v)
    {
        T* d = alloc<T>(v.size());
        if (!v.empty()) CK(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        note_h2d(v.size() * sizeof(T));
        return d;
    }
    template <class T> T* zeros(size_t n)
    {
        T* d = alloc<T>(n);
        CK(cudaMemsetAsync(d, 0, (n ? n : 1) * sizeof(T), st));
        return d;
    }
    void release()
    {
        for (void* p : ptrs) cudaFreeAsync(p, st);
        ptrs.clear();
    }
    ~Arena()
    {
        release();
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    }
};

struct StageClock {
    cudaStream_t st;
    std::vector<cudaEvent_t> evs;
    cudaEvent_t mark()
    {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        CK(cudaEventRecord(e, st));
        evs.push_back(e);
        return e;
    }
    static double ms(cudaEvent_t a, cudaEvent_t b)
    {
        float m = 0;
        cudaEventElapsedTime(&m, a, b);
        return m;
    }
    ~StageClock()
    {
        for (auto e : evs) cudaEventDestroy(e);
    }
};


void check_abort(ltr_Scene* s)
{
    if (s->abort_flag.load()) throw std::runtime_error("aborted by ltr_Abort");
}

// Row-vector transform and normal matrix of Job_PreXForm_Inner (lighter.cpp:292-341,
// lighter_int.hpp:511-545). The 2x2 minors keep the operand order of the
// 4x4 cofactor expansion of Mat4::InvertTo applied to [R 0; 0 1].
void prexform(ltr_Scene* S, HostInst* mi)
{
    const float* m = mi->matrix;   // m[r*4+c]
    ltr_Mesh* me = mi->mesh;
    size_t nv = me->pos.size();
    mi->vpos.resize(nv); mi->vnrm.resize(nv); mi->vtex.resize(nv); mi->ltex.resize(nv);
    const float a0 = m[0], a1 = m[1], a2 = m[2], a4 = m[4], a5 = m[5], a6 = m[6], a8 = m[8], a9 = m[9], a10 = m[10];
    float c[16] = {0};
    c[0] = a5 * a10 - a9 * a6;
    c[4] = -(a4 * a10) + a8 * a6;
    c[8] = a4 * a9 - a8 * a5;
    c[1] = -(a1 * a10) + a9 * a2;
    c[5] = a0 * a10 - a8 * a2;
    c[9] = -(a0 * a9) + a8 * a1;
    c[2] = a1 * a6 - a5 * a2;
    c[6] = -(a0 * a6) + a4 * a2;
    c[10] = a0 * a5 - a4 * a1;
    float det = a0 * c[0] + a1 * c[4] + a2 * c[8];
    float inv[16];
    if (det == 0) {
        for (int i = 0; i < 16; ++i) inv[i] = 0;
        inv[0] = a0; inv[1] = a1; inv[2] = a2; inv[4] = a4; inv[5] = a5; inv[6] = a6; inv[8] = a8; inv[9] = a9;
        inv[10] = a10;
    } else {
        float d = 1.0f / det;
        for (int i = 0; i < 16; ++i) inv[i] = c[i] * d;
    }
    // normal matrix N[r][k] = inv[k*4+r]; transform of (n, 0) by rows
    for (size_t i = 0; i < nv; ++i) {
        V3 v = me->pos[i];
        mi->vpos[i] = mk(v.x * m[0] + v.y * m[4] + v.z * m[8] + m[12] * 1.0f,
                         v.x * m[1] + v.y * m[5] + v.z * m[9] + m[13] * 1.0f,
                         v.x * m[2] + v.y * m[6] + v.z * m[10] + m[14] * 1.0f);
        V3 n = me->nrm[i];
        mi->vnrm[i] = normalized(mk(n.x * inv[0] + n.y * inv[1] + n.z * inv[2] + inv[3] * 0.0f,
                                    n.x * inv[4] + n.y * inv[5] + n.z * inv[6] + inv[7] * 0.0f,
                                    n.x * inv[8] + n.y * inv[9] + n.z * inv[10] + inv[11] * 0.0f));
    }
    float area = 0.0f;
    for (const HostPart& p : me->parts) {
        const V3* vb = &mi->vpos[p.voff];
        const u32* ib = &me->idx[p.ioff];
        for (u32 t = 0; t < p.icount; t += 3) area += tri_area3(vb[ib[t]], vb[ib[t + 1]], vb[ib[t + 2]]);
    }
    u32 size[2] = {S->cfg.default_width, S->cfg.default_height};
    if (!S->cfg.size_fn || !S->cfg.size_fn(&S->cfg, me->ident.c_str(), me->ident.size(), mi->ident.c_str(),
                                           mi->ident.size(), area, mi->importance, size)) {
        size[0] = S->cfg.default_width;
        size[1] = S->cfg.default_height;
    }
    mi->w = size[0];
    mi->h = size[1];
    float fw = (float) mi->w, fh = (float) mi->h;
    for (size_t i = 0; i < nv; ++i) {
        mi->vtex[i] = me->tex1[i];
        mi->ltex[i] = mk2(me->tex2[i].x * fw - 0.5f, me->tex2[i].y * fh - 0.5f);
    }
}

// ---- leaf references for the BVH
//
// A triangle much larger than the scene's typical triangle (a 200 m ground
// quad) gives every BVH node above it a scene-sized box, so nearly every
// query descends there. Such triangles are split into several leaf
// references: the triangle is clipped (Sutherland-Hodgman) against recursive
// midpoint splits of its box until the pieces are no longer than `limit`, and
// each reference keeps the whole triangle with the clipped piece's box.

struct ClipPoly {
    V3 v[24];
    int n = 0;
};

inline float axis_of(V3 p, int a) { return a == 0 ? p.x : (a == 1 ? p.y : p.z); }

void clip_half(const ClipPoly& in, int axis, float c, bool below, ClipPoly& out)
{
    out.n = 0;
    for (int i = 0; i < in.n; ++i) {
        V3 a = in.v[i], b = in.v[(i + 1) % in.n];
        float da = axis_of(a, axis) - c, db = axis_of(b, axis) - c;
        bool ia = below ? da <= 0 : da >= 0, ib = below ? db <= 0 : db >= 0;
        if (ia && out.n < 24) out.v[out.n++] = a;
        if (ia != ib && out.n < 24) {
            float t = da / (da - db);
            V3 p = a + (b - a) * t;
            // pin the cut coordinate on the plane
            if (axis == 0) p.x = c; else if (axis == 1) p.y = c; else p.z = c;
            out.v[out.n++] = p;
        }
    }
}

void split_ref(const ClipPoly& p, float limit, int depth, u32 tri, std::vector<u32>& ref_tri, std::vector<float>& ref_box)
{
    V3 mn = splat(FLT_MAX), mx = splat(-FLT_MAX);
    for (int i = 0; i < p.n; ++i) { mn = vmin(mn, p.v[i]); mx = vmax(mx, p.v[i]); }
    V3 e = mx - mn;
    int axis = (e.x >= e.y && e.x >= e.z) ? 0 : (e.y >= e.z ? 1 : 2);
    float ext = axis_of(e, axis);
    if (ext <= limit || depth >= 12 || p.n < 3) {
        ref_tri.push_back(tri);
        ref_box.insert(ref_box.end(), {mn.x, mn.y, mn.z, mx.x, mx.y, mx.z});
        return;
    }
    float c = (axis_of(mn, axis) + axis_of(mx, axis)) * 0.5f;
    ClipPoly lo, hi;
    clip_half(p, axis, c, true, lo);
    clip_half(p, axis, c, false, hi);
    if (lo.n) split_ref(lo, limit, depth + 1, tri, ref_tri, ref_box);
    if (hi.n) split_ref(hi, limit, depth + 1, tri, ref_tri, ref_box);
}

// References for all triangles; the split limit is four times the median
// triangle extent (and at least 1/512 of the scene).
void build_refs(const std::vector<float>& xyz, std::vector<u32>& ref_tri, std::vector<float>& ref_box, float* cmin,
                float* cmax)
{
    const size_t n = xyz.size() / 9;
    std::vector<float> ext(n);
    V3 smn = splat(FLT_MAX), smx = splat(-FLT_MAX);
    for (size_t i = 0; i < n; ++i) {
        const float* q = &xyz[9 * i];
        V3 a = mk(q[0], q[1], q[2]), b = mk(q[3], q[4], q[5]), c = mk(q[6], q[7], q[8]);
        V3 mn = vmin(a, vmin(b, c)), mx = vmax(a, vmax(b, c)), e = mx - mn;
        ext[i] = fmax_(e.x, fmax_(e.y, e.z));
        smn = vmin(smn, mn);
        smx = vmax(smx, mx);
    }
    float limit = FLT_MAX;
    if (n) {
        std::vector<float> tmp(ext);
        std::nth_element(tmp.begin(), tmp.begin() + n / 2, tmp.end());
        V3 se = smx - smn;
        limit = fmax_(4.0f * tmp[n / 2], fmax_(se.x, fmax_(se.y, se.z)) / 512.0f);
    }
    ref_tri.clear();
    ref_box.clear();
    ref_tri.reserve(n);
    ref_box.reserve(6 * n);
    for (size_t i = 0; i < n; ++i) {
        const float* q = &xyz[9 * i];
        ClipPoly p;
        p.n = 3;
        p.v[0] = mk(q[0], q[1], q[2]);
        p.v[1] = mk(q[3], q[4], q[5]);
        p.v[2] = mk(q[6], q[7], q[8]);
        split_ref(p, limit, 0, (u32) i, ref_tri, ref_box);
    }
    for (int c = 0; c < 3; ++c) { cmin[c] = FLT_MAX; cmax[c] = -FLT_MAX; }
    for (size_t r = 0; r < ref_tri.size(); ++r)
        for (int c = 0; c < 3; ++c) {
            float m = (ref_box[6 * r + c] + ref_box[6 * r + 3 + c]) * 0.5f;
            cmin[c] = fminf(cmin[c], m);
            cmax[c] = fmaxf(cmax[c], m);
        }
}

// Gaussian taps (Generate_Gaussian_Kernel, lighter_math.cpp:357-365), on the
// host so the weights are the reference's glibc values.
std::vector<float> gauss_taps(int ext, float radius)
{
    std::vector<float> k(ext * 2 + 1);
    float sum = 0.0f;
    float mc = 1.0f / sqrtf(2.0f * 3.14159265358979323846f * radius * radius);
    for (int i = -ext; i <= ext; ++i) sum += k[i + ext] = expf(-0.5f * powf((float) i / radius, 2.0f)) * mc;
    for (int i = -ext; i <= ext; ++i) k[i + ext] /= sum;
    return k;
}

}  // namespace

void build_refs_host(const std::vector<float>& xyz, std::vector<u32>& ref_tri, std::vector<float>& ref_box, float* cmin,
                     float* cmax)
{
    build_refs(xyz, ref_tri, ref_box, cmin, cmax);
}

// ----------------------------------------------------------------------------- batches of scenes (host)
//
// The scenes of one ltrg_StartBatch run their bakes on their own host threads
// and streams as usual. At the direct-light and the AO stage every scene
// joins a rendezvous with its job; the last one to arrive (or to leave, when
// a scene ends early) launches one trace kernel for all jobs on the batch's
// stream, after events that mark each scene's inputs ready, and every scene's
// stream waits on the launch's completion event. The per-sample rand() draws
// of AO take turns in scene order, so a batch gives every scene the random
// offsets it would get from bakes run one after another in that order.
// A scene of a batch whose trace phase has at least this many work items
// (pairs or rays) launches that phase alone on its own stream instead of
// waiting for the others: such a launch fills the GPU by itself, and the
// scenes' other stages overlap.
constexpr unsigned long long kBatchSoloItems = 1ull << 22;

struct BatchCtx {
    BatchCtx(int n_, int device_)
        : n(n_), device(device_), rand_done(n_, 0), member(n_, 0), started(n_, 0), cv_turn(n_), cv_start(n_)
    {
        for (Phase& p : phase) p.expected = n_;
        // more scenes at a time measured slower (64 on 16 cores: 0.87 -> 1.21 s for
        // 256 scenes; each scene's small kernels and waits queue behind the others'),
        // and so did blocking instead of spinning waits (0.77 -> 0.79 s)
        slots = std::max(2, std::min(16, (int) std::thread::hardware_concurrency()));
        trace = getenv("LTRG_TRACE") != nullptr;
        t0 = std::chrono::steady_clock::now();
    }
    ~BatchCtx()
    {
        for (Phase& p : phase) {
            for (cudaEvent_t e : p.ready) cudaEventDestroy(e);
            if (p.done) cudaEventDestroy(p.done);
        }
        if (bst) {
            cudaStreamSynchronize(bst);
            cudaStreamDestroy(bst);
        }
    }

    struct Phase {
        int expected = 0, arrived = 0;
        bool launched = false;
        std::string error;
        std::vector<DirectJob> djobs;
        std::vector<AoJob> ajobs;
        std::vector<unsigned long long> rays;   // AO work items per job (ao_items)
        std::vector<cudaEvent_t> ready;
        cudaEvent_t done = nullptr;
    };

    const int n, device;
    std::mutex mu;
    std::vector<char> rand_done;   // per scene: its AO draws are over (or it draws none)
    int rand_turn = 0;
    std::vector<int> member;       // per scene: phases joined (bit p) or left
    std::vector<char> started;     // per scene: took its first slot (or left before)
    int next_start = 0;
    // Each kind of wait has its own condition variable, and the per-scene turns
    // one per scene, so a step of the ordered chains wakes one thread, not all.
    std::vector<std::condition_variable> cv_turn;    // scene's turn to draw
    std::vector<std::condition_variable> cv_start;   // scene's turn to start
    std::condition_variable cv_slot;                 // a slot for a scene back from a wait
    std::condition_variable cv_phase[2];             // the phase was launched
    int slots = 16;                                  // scenes allowed to work at a time
    int returners = 0;                               // scenes waiting in cv_slot
    Phase phase[2];                                  // 0: direct light, 1: AO
    cudaStream_t bst = nullptr;
    bool trace = false;
    std::chrono::steady_clock::time_point t0;
    static constexpr auto kWait = std::chrono::seconds(900);

    void note(const char* what, int p, int k)
    {
        if (trace)
            fprintf(stderr, "[ltrg batch] %9.3f ms  phase %d %s %d\n",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(), p, what, k);
    }

    // --- slots: at most `slots` scenes do host work (and issue CUDA calls) at a
    // time; a scene gives its slot back while it waits at a rendezvous or for its
    // turn to draw. Scenes take their first slot in batch order, so the chain of
    // ordered AO draws can begin with scene 0 at once. Called with `mu` held:
    void grant()
    {
        if (slots <= 0) return;
        if (returners > 0) cv_slot.notify_one();
        else if (next_start < n) cv_start[next_start].notify_one();
    }
    void advance_start()
    {
        while (next_start < n && started[next_start]) ++next_start;
        grant();
    }
    void take_slot(std::unique_lock<std::mutex>& lk)
    {
        ++returners;
        bool ok = cv_slot.wait_for(lk, kWait, [&] { return slots > 0; });
        --returners;
        if (!ok) throw std::runtime_error("batch: timed out waiting for a slot");
        --slots;
        grant();
    }

    void acquire_start(int idx)
    {
        std::unique_lock<std::mutex> lk(mu);
        if (!cv_start[idx].wait_for(lk, kWait, [&] { return slots > 0 && next_start == idx && returners == 0; }))
            throw std::runtime_error("batch: timed out waiting for a slot");
        --slots;
        started[idx] = 1;
        advance_start();
    }
    void acquire()
    {
        std::unique_lock<std::mutex> lk(mu);
        take_slot(lk);
    }
    void release()
    {
        std::lock_guard<std::mutex> lk(mu);
        ++slots;
        grant();
    }

    // --- AO draw turns, in scene order
    void advance_turn()
    {
        while (rand_turn < n && rand_done[rand_turn]) ++rand_turn;
        if (rand_turn < n) cv_turn[rand_turn].notify_one();
    }
    void rand_begin(int idx)
    {
        std::unique_lock<std::mutex> lk(mu);
        if (!cv_turn[idx].wait_for(lk, kWait, [&] { return rand_turn >= idx; }))
            throw std::runtime_error("batch: timed out waiting for the random draws of earlier scenes");
    }
    void rand_end(int idx)
    {
        std::lock_guard<std::mutex> lk(mu);
        if (idx % 32 == 0 || idx == n - 1) note("draws done, scene", 9, idx);
        rand_done[idx] = 1;
        advance_turn();
    }

    // --- rendezvous. Joins phase p with scene idx's job; returns the event its
    // stream waits on (the scene holds a slot again on return).
    cudaEvent_t join(int p, int idx, cudaStream_t st, const DirectJob* dj, const AoJob* aj, unsigned long long rays)
    {
        cudaEvent_t ready;
        CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
        CK(cudaEventRecord(ready, st));
        std::unique_lock<std::mutex> lk(mu);
        Phase& ph = phase[p];
        ph.ready.push_back(ready);
        if (dj) ph.djobs.push_back(*dj);
        if (aj) {
            ph.ajobs.push_back(*aj);
            ph.rays.push_back(rays);
        }
        ph.arrived++;
        member[idx] |= 1 << p;
        if (ph.arrived == 1 || ph.arrived == ph.expected) note("arrival", p, ph.arrived);
        if (ph.arrived == ph.expected) {
            launch(p);
            if (trace && ph.done) {   // timeline only: wait for the kernel without holding the lock
                lk.unlock();
                cudaEventSynchronize(ph.done);
                lk.lock();
                note("kernel done", p, ph.arrived);
            }
        }
        ++slots;   // the slot goes to scenes that still have to arrive
        grant();
        if (!cv_phase[p].wait_for(lk, kWait, [&] { return ph.launched; }))
            throw std::runtime_error("batch: timed out waiting for the other scenes of the batch");
        take_slot(lk);
        if (!ph.error.empty()) throw std::runtime_error("batch launch failed: " + ph.error);
        return ph.done;
    }

    // Scene idx has no work for phase p (it will not join it).
    void skip(int p, int idx)
    {
        std::lock_guard<std::mutex> lk(mu);
        if (member[idx] & (1 << p)) return;
        member[idx] |= 1 << p;
        Phase& ph = phase[p];
        ph.expected--;
        if (!ph.launched && ph.arrived > 0 && ph.arrived == ph.expected) launch(p);
    }

    // Scene idx will join no further phase (its bake ended or failed).
    void leave(int idx)
    {
        std::lock_guard<std::mutex> lk(mu);
        for (int p = 0; p < 2; ++p) {
            if (member[idx] & (1 << p)) continue;
            member[idx] |= 1 << p;
            Phase& ph = phase[p];
            ph.expected--;
            if (!ph.launched && ph.arrived > 0 && ph.arrived == ph.expected) launch(p);
        }
        if (!rand_done[idx]) {
            rand_done[idx] = 1;
            advance_turn();
        }
        if (!started[idx]) {
            started[idx] = 1;
            advance_start();
        }
    }

  private:
    // Called with `mu` held, once per phase, when every remaining scene has joined.
    void launch(int p)
    {
        Phase& ph = phase[p];
        try {
            CK(cudaSetDevice(device));
            if (!bst) CK(cudaStreamCreateWithFlags(&bst, cudaStreamNonBlocking));
            for (cudaEvent_t e : ph.ready) CK(cudaStreamWaitEvent(bst, e, 0));
            int sms = 0;
            CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
            const int nj = p == 0 ? (int) ph.djobs.size() : (int) ph.ajobs.size();
            if (nj > 0) {
                unsigned long long* d_off = nullptr;
                unsigned long long* d_next = nullptr;
                void* d_jobs = nullptr;
                const size_t jb = p == 0 ? nj * sizeof(DirectJob) : nj * sizeof(AoJob);
                CK(cudaMallocAsync(&d_jobs, jb, bst));
                CK(cudaMallocAsync((void**) &d_off, (nj + 1) * sizeof(unsigned long long), bst));
                CK(cudaMallocAsync((void**) &d_next, sizeof(unsigned long long), bst));
                CK(cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), bst));
                if (p == 0) {
                    CK(cudaMemcpyAsync(d_jobs, ph.djobs.data(), jb, cudaMemcpyHostToDevice, bst));
                    k_direct_batch_offsets<<<1, 32, 0, bst>>>((const DirectJob*) d_jobs, nj, d_off); note_launch();
                    const ltrg_Tuning tu = get_tuning(device);
                    const unsigned grid = (unsigned) sms * tu.direct_blocks_per_sm;
                    if (tu.direct_packet)
                        k_direct_trace_batch<true><<<grid, tu.direct_block, 0, bst>>>((const DirectJob*) d_jobs, nj, d_off,
                                                                                      d_next);
                    else
                        k_direct_trace_batch<false><<<grid, tu.direct_block, 0, bst>>>((const DirectJob*) d_jobs, nj, d_off,
                                                                                       d_next);
                    note_launch();
                } else {
                    std::vector<unsigned long long> off(nj + 1, 0);
                    for (int k = 0; k < nj; ++k) off[k + 1] = off[k] + ph.rays[k];
                    CK(cudaMemcpyAsync(d_jobs, ph.ajobs.data(), jb, cudaMemcpyHostToDevice, bst));
                    CK(cudaMemcpyAsync(d_off, off.data(), off.size() * sizeof(unsigned long long),
                                       cudaMemcpyHostToDevice, bst));
                    // the pageable copies above are staged before they return, so `off` may go
                    const ltrg_Tuning tu = get_tuning(device);
                    const unsigned grid = (unsigned) sms * tu.ao_blocks_per_sm;
                    if (tu.ao_packet)
                        k_ao_rays_batch<true><<<grid, tu.ao_block, 0, bst>>>((const AoJob*) d_jobs, nj, d_off, d_next);
                    else
                        k_ao_rays_batch<false><<<grid, tu.ao_block, 0, bst>>>((const AoJob*) d_jobs, nj, d_off, d_next);
                    note_launch();
                }
                CK(cudaGetLastError());
                cudaFreeAsync(d_jobs, bst);
                cudaFreeAsync(d_off, bst);
                cudaFreeAsync(d_next, bst);
            }
            CK(cudaEventCreateWithFlags(&ph.done, cudaEventDisableTiming));
            CK(cudaEventRecord(ph.done, bst));
            note("launched, jobs", p, nj);
        } catch (const std::exception& e) {
            ph.error = e.what();
        }
        ph.launched = true;
        cv_phase[p].notify_all();
    }
};

std::shared_ptr<BatchCtx> make_batch(int n, int device) { return std::make_shared<BatchCtx>(n, device); }
void batch_leave(BatchCtx* b, int idx) { b->leave(idx); }

// ----------------------------------------------------------------------------- the bake

// The default stream-ordered memory pool returns its memory to the driver at
// every synchronisation (release threshold 0), so each bake's few dozen
// cudaMallocAsync calls would map fresh memory. Keeping up to 8 GiB cached
// per device makes a repeated bake's allocations pool hits.
void keep_pool_memory(int device)
{
    static std::mutex mu;
    static std::vector<char> done;
    std::lock_guard<std::mutex> lk(mu);
    if ((int) done.size() <= device) done.resize(device + 1, 0);
    if (done[device]) return;
    // The pool keeps up to half the device's memory across synchronisations,
    // so a scene baked again reuses its buffers instead of mapping them anew.
    cudaMemPool_t pool;
    size_t free_b = 0, total_b = 0;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = 8ull << 30;
        int prev = -1;
        if (cudaGetDevice(&prev) == cudaSuccess && cudaSetDevice(device) == cudaSuccess) {
            if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) keep = std::max<uint64_t>(keep, total_b / 2);
            cudaSetDevice(prev);
        }
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done[device] = 1;
}

void run_bake(ltr_Scene* S)
{
    const ltr_Config& cfg = S->cfg;
    memset(&S->stats, 0, sizeof(S->stats));
    host_counters() = HostCounters();
    S->rad_links = 0;

    // member of a batch (ltrg_StartBatch): leaves it however the bake ends
    BatchCtx* batch = S->batch.get();
    const int bidx = S->batch_index;
    struct BatchLeave {
        BatchCtx* b; int i; bool slot = false;
        ~BatchLeave() { if (b) { b->leave(i); if (slot) b->release(); } }
    } batch_leave_end{batch, bidx};

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw std::runtime_error("no CUDA device available");
    if (S->opt.device >= ndev) throw std::runtime_error("ltrg_Options.device out of range");
    CK(cudaSetDevice(S->opt.device));
    keep_pool_memory(S->opt.device);
    // the abort word (see ltr_Scene::abort_word): 0, published, then the flag read again
    if (!S->abort_alloc) CK(cudaHostAlloc(&S->abort_alloc, 64, cudaHostAllocMapped | cudaHostAllocPortable));
    u32* abort_host = (u32*) S->abort_alloc;
    *(volatile u32*) abort_host = 0u;
    S->abort_word.store(abort_host);
    if (S->abort_flag.load()) *(volatile u32*) abort_host = 1u;
    u32* d_abort = nullptr;
    CK(cudaHostGetDevicePointer((void**) &d_abort, abort_host, 0));
    if (batch) {
        batch->acquire_start(bidx);
        batch_leave_end.slot = true;
    }

    Arena A;
    CK(cudaStreamCreateWithFlags(&A.st, cudaStreamNonBlocking));
    StageClock clock{A.st};
    cudaStream_t st = A.st;

    // ---- host: transform + lightmap sizing (Job_PreXForm)
    // LTRG_TRACE=1: host timeline of the bake on stderr
    const bool trace_on = getenv("LTRG_TRACE") != nullptr;
    const auto t_start = std::chrono::steady_clock::now();
    auto TRACE = [&](const char* what) {
        if (!trace_on) return;
        const auto now = std::chrono::steady_clock::now();
        if (batch)   // scene index and time since the batch started, for merging the scenes' lines
            fprintf(stderr, "[ltrg s%d] %9.3f ms (batch %9.3f ms)  %s\n", bidx,
                    std::chrono::duration<double, std::milli>(now - t_start).count(),
                    std::chrono::duration<double, std::milli>(now - batch->t0).count(), what);
        else
            fprintf(stderr, "[ltrg] %9.3f ms  %s\n", std::chrono::duration<double, std::milli>(now - t_start).count(),
                    what);
    };
    S->stage = "transforming spatial data";
    const int n_inst = (int) S->insts.size();
    // instances in parallel: the reference too calls size_fn from its pool threads
    parallel_items(n_inst - 1, [&](int k) { prexform(S, S->insts[k + 1]); });
    check_abort(S);

    // ---- host: triangle soup of shadow parts (Job_ColInfo) + instance boxes
    TRACE("prexform done");
    S->stage = "generating data structures";
    // per instance in parallel, then concatenated in instance order
    struct InstSoup {
        std::vector<float> xyz;
        float smin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, smax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    };
    std::vector<InstSoup> soup(n_inst);
    std::vector<float> inst_box(6 * n_inst);
    parallel_items(n_inst, [&](int i) {
        HostInst* mi = S->insts[i];
        InstSoup& o = soup[i];
        V3 bmn = splat(FLT_MAX), bmx = splat(-FLT_MAX);
        if (!mi->container) {
            ltr_Mesh* me = mi->mesh;
            for (const HostPart& p : me->parts) {
                if (!p.shadow) continue;
                const V3* vb = &mi->vpos[p.voff];
                const u32* ib = &me->idx[p.ioff];
                for (u32 t = 0; t < p.icount; t += 3) {
                    V3 P1 = vb[ib[t]], P2 = vb[ib[t + 1]], P3 = vb[ib[t + 2]];
                    if (near_zero(cross(P2 - P1, P3 - P1))) continue;   // Triangle::CheckIsUseful
                    const V3 ps[3] = {P1, P2, P3};
                    for (const V3& q : ps) {
                        o.xyz.push_back(q.x); o.xyz.push_back(q.y); o.xyz.push_back(q.z);
                        bmn = vmin(bmn, q); bmx = vmax(bmx, q);
                    }
                    float cx = (P1.x + P2.x + P3.x) * (1.0f / 3.0f), cy = (P1.y + P2.y + P3.y) * (1.0f / 3.0f),
                          cz = (P1.z + P2.z + P3.z) * (1.0f / 3.0f);
                    o.smin[0] = fminf(o.smin[0], cx); o.smin[1] = fminf(o.smin[1], cy); o.smin[2] = fminf(o.smin[2], cz);
                    o.smax[0] = fmaxf(o.smax[0], cx); o.smax[1] = fmaxf(o.smax[1], cy); o.smax[2] = fmaxf(o.smax[2], cz);
                }
            }
        }
        inst_box[6 * i + 0] = bmn.x; inst_box[6 * i + 1] = bmn.y; inst_box[6 * i + 2] = bmn.z;
        inst_box[6 * i + 3] = bmx.x; inst_box[6 * i + 4] = bmx.y; inst_box[6 * i + 5] = bmx.z;
    });
    std::vector<float> tri_xyz;
    std::vector<u32> tri_meta, tri_local;
    float smin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, smax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    {
        size_t total = 0;
        for (const InstSoup& o : soup) total += o.xyz.size() / 9;
        tri_xyz.reserve(9 * total);
        tri_meta.reserve(total);
        tri_local.reserve(total);
        for (int i = 0; i < n_inst; ++i) {
            const InstSoup& o = soup[i];
            const u32 nt_i = (u32) (o.xyz.size() / 9);
            tri_xyz.insert(tri_xyz.end(), o.xyz.begin(), o.xyz.end());
            const u32 meta = (u32) i | (S->insts[i]->shadow ? kOccluderBit : 0u);
            for (u32 t = 0; t < nt_i; ++t) {
                tri_meta.push_back(meta);
                tri_local.push_back(t);
            }
            for (int c = 0; c < 3; ++c) {
                smin[c] = fminf(smin[c], o.smin[c]);
                smax[c] = fmaxf(smax[c], o.smax[c]);
            }
        }
        soup.clear();
    }
    const int n_tris = (int) tri_meta.size();
    S->stats.triangles = (uint64_t) n_tris;
    TRACE("triangle soup done");
    float gmin[3] = {0, 0, 0}, gmax[3] = {0, 0, 0};   // bounds of all occluder geometry
    {
        bool any = false;
        for (int i = 0; i < n_inst; ++i) {
            const float* b = &inst_box[6 * i];
            if (!(b[0] <= b[3] && b[1] <= b[4] && b[2] <= b[5])) continue;
            for (int c = 0; c < 3; ++c) {
                gmin[c] = any ? fminf(gmin[c], b[c]) : b[c];
                gmax[c] = any ? fmaxf(gmax[c], b[3 + c]) : b[3 + c];
            }
            any = true;
        }
    }

    // reference-shaped per-instance trees for the sample-offset pass
    std::vector<int> inst_tri_off(n_inst + 1, 0);
    for (int t = 0; t < n_tris; ++t) inst_tri_off[(tri_meta[t] & kInstMask) + 1]++;
    for (int i = 0; i < n_inst; ++i) inst_tri_off[i + 1] += inst_tri_off[i];
    // The reference-shaped trees serve only the sample fixup: they are built on
    // a side thread while the upload, the BVH build and the raster run, and
    // joined before the fixup launch.
    std::vector<float4> ref_nodes;
    std::vector<int> ref_items;
    std::vector<int4> ref_inst(n_inst, make_int4(0, 0, 0, 0));
    std::vector<float4> fix_box(2 * (size_t) n_inst);   // root boxes for the fixup's instance culling
    std::exception_ptr reftree_error;
    std::thread reftree_thread([&]() {
        try {
            std::vector<RefTree> rtrees(n_inst);
            {
                std::vector<std::thread> pool;
                std::atomic<int> next(1);
                int nth = std::max(1, std::min({8, (int) std::thread::hardware_concurrency(), n_inst - 1}));
                for (int t = 0; t < nth; ++t)
                    pool.emplace_back([&]() {
                        for (int i = next++; i < n_inst; i = next++)
                            build_ref_tree(tri_xyz.data() + 9 * (size_t) inst_tri_off[i],
                                           (size_t) (inst_tri_off[i + 1] - inst_tri_off[i]), rtrees[i]);
                    });
                for (auto& th : pool) th.join();
            }
            for (int i = 0; i < n_inst; ++i) {
                fix_box[2 * i] = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.0f);
                fix_box[2 * i + 1] = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.0f);
            }
            for (int i = 1; i < n_inst; ++i) {
                const RefTree& rt_i = rtrees[i];
                if (inst_tri_off[i + 1] == inst_tri_off[i]) continue;
                if (!rt_i.nodes.empty()) {
                    const RefNode& root = rt_i.nodes[0];
                    fix_box[2 * i] = make_float4(root.mn[0], root.mn[1], root.mn[2], 0.0f);
                    fix_box[2 * i + 1] = make_float4(root.mx[0], root.mx[1], root.mx[2], 0.0f);
                }
                ref_inst[i] = make_int4((int) (ref_nodes.size() / 2), (int) ref_items.size(), inst_tri_off[i],
                                        (int) rt_i.nodes.size());
                for (const RefNode& nd : rt_i.nodes) {
                    float chf, idof;
                    memcpy(&chf, &nd.ch, 4);
                    memcpy(&idof, &nd.ido, 4);
                    ref_nodes.push_back(make_float4(nd.mn[0], nd.mn[1], nd.mn[2], nd.mx[0]));
                    ref_nodes.push_back(make_float4(nd.mx[1], nd.mx[2], chf, idof));
                }
                ref_items.insert(ref_items.end(), rt_i.items.begin(), rt_i.items.end());
            }
        } catch (...) {
            reftree_error = std::current_exception();
        }
    });
    struct JoinReftree {   // joined on every way out (the thread reads this frame's vectors)
        std::thread& th;
        ~JoinReftree() { if (th.joinable()) th.join(); }
    } join_reftree{reftree_thread};

    // ---- BVH: built on its own stream and host thread as soon as the triangle
    // soup exists, while this thread prepares the raster records (the build
    // reads its cluster count back now and then, which would hold this thread);
    // the sample stage waits for it.
    cudaEvent_t e_dev0 = clock.mark();   // the bake's first device work
    float* d_tri_xyz = A.upload(tri_xyz);
    u32* d_tri_meta = A.upload(tri_meta);
    u32* d_tri_local = A.upload(tri_local);
    cudaEvent_t e_tri = clock.mark();
    BvhStorage bvh;
    BvhBuildInput bin;
    bin.tri_xyz = d_tri_xyz;
    bin.tri_meta = d_tri_meta;
    bin.tri_local = d_tri_local;
    bin.builder = (int) S->opt.bvh_builder;
    struct BvhSide {   // its stream, start/end events, and the BVH's storage, released last
        cudaStream_t st_main = nullptr, st = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        BvhStorage* bvh = nullptr;
        ~BvhSide()
        {
            if (st) cudaStreamSynchronize(st);
            if (st_main) cudaStreamSynchronize(st_main);
            if (bvh) bvh_free(*bvh, st_main);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            if (st) cudaStreamDestroy(st);
        }
    } bside;
    bside.st_main = st;
    bside.bvh = &bvh;
    if (!batch) CK(cudaStreamCreateWithFlags(&bside.st, cudaStreamNonBlocking));
    CK(cudaEventCreate(&bside.e0));
    CK(cudaEventCreate(&bside.e1));
    std::exception_ptr bvh_error;
    HostCounters bvh_counts;
    auto bvh_job = [&]() {
        try {
            CK(cudaSetDevice(S->opt.device));
            cudaStream_t bs = bside.st ? bside.st : st;
            if (bs != st) CK(cudaStreamWaitEvent(bs, e_tri, 0));
            CK(cudaEventRecord(bside.e0, bs));
            std::vector<u32> ref_tri;
            std::vector<float> ref_box;
            float rmin[3], rmax[3];
            build_refs(tri_xyz, ref_tri, ref_box, rmin, rmax);
            u32* d_ref_tri = nullptr;
            float* d_ref_box = nullptr;
            CK(cudaMallocAsync(&d_ref_tri, std::max<size_t>(ref_tri.size(), 1) * sizeof(u32), bs));
            CK(cudaMallocAsync(&d_ref_box, std::max<size_t>(ref_box.size(), 1) * sizeof(float), bs));
            struct FreeRefs {
                cudaStream_t s; void* p[2];
                ~FreeRefs() { for (void* q : p) cudaFreeAsync(q, s); }
            } free_refs{bs, {d_ref_tri, d_ref_box}};
            if (!ref_tri.empty())
                CK(cudaMemcpyAsync(d_ref_tri, ref_tri.data(), ref_tri.size() * sizeof(u32), cudaMemcpyHostToDevice, bs));
            if (!ref_box.empty())
                CK(cudaMemcpyAsync(d_ref_box, ref_box.data(), ref_box.size() * sizeof(float), cudaMemcpyHostToDevice, bs));
            note_h2d(ref_tri.size() * sizeof(u32) + ref_box.size() * sizeof(float));
            bin.ref_tri = d_ref_tri;
            bin.ref_box = d_ref_box;
            bin.n = (int) ref_tri.size();
            for (int c = 0; c < 3; ++c) { bin.scene_min[c] = bin.n ? rmin[c] : 0; bin.scene_max[c] = bin.n ? rmax[c] : 0; }
            bvh_build(bin, bvh, bs);
            CK(cudaEventRecord(bside.e1, bs));
        } catch (...) {
            bvh_error = std::current_exception();
        }
    };
    // A scene of a batch builds on its own thread and stream: the other scenes'
    // work fills the GPU and the host meanwhile, an extra waiting thread per scene
    // (the build's read-backs) would take host cores from the scenes still
    // preparing, and with a second stream per scene the 256-scene batch measured
    // 5.0 s instead of 0.8 s.
    std::thread bvh_thread;
    if (batch) {
        bvh_job();
    } else {
        bvh_thread = std::thread([&]() {
            bvh_job();
            bvh_counts = host_counters();   // this thread's launches and copies
        });
    }
    struct JoinBvh {   // joined on every way out (the thread uses this frame's variables)
        std::thread& th;
        ~JoinBvh() { if (th.joinable()) th.join(); }
    } join_bvh{bvh_thread};

    const int n_lights = (int) S->lights.size();
    std::vector<unsigned char> lit((size_t) n_lights * n_inst, 0);
    std::vector<DLight> dl(n_lights);
    std::vector<float4> lsmp;   // shadow samples of every light (LTRG_SHADOW_SAMPLED)
    for (int l = 0; l < n_lights; ++l) {
        const HostLight& L = S->lights[l];
        DLight& d = dl[l];
        d.ns = L.nsamples;
        d.soff = (int) lsmp.size();
        if (S->opt.shadow_mode == LTRG_SHADOW_SAMPLED)
            for (const V3& v : light_shadow_samples(L)) lsmp.push_back(make_float4(v.x, v.y, v.z, 0.0f));
        d.type = (int) L.type;
        d.pos[0] = L.pos.x; d.pos[1] = L.pos.y; d.pos[2] = L.pos.z;
        d.dir[0] = L.dir.x; d.dir[1] = L.dir.y; d.dir[2] = L.dir.z;
        d.color[0] = L.color.x; d.color[1] = L.color.y; d.color[2] = L.color.z;
        d.range = L.range; d.power = L.power; d.radius = L.radius; d.curve = L.curve;
        d.out_rad = 0; d.diff = 0;
        if (L.type == 2) {   // lighter.cpp:641-644
            float out_rad = L.out / 180.0f * 3.14159265358979323846f, in_rad = L.in / 180.0f * 3.14159265358979323846f;
            if (in_rad == out_rad) in_rad -= kSmall;
            d.out_rad = out_rad;
            d.diff = in_rad - out_rad;
        }
        lit[(size_t) l * n_inst + 0] = 1;
        for (int i = 1; i < n_inst; ++i) {
            const float* b = &inst_box[6 * i];
            bool valid = b[0] <= b[3] && b[1] <= b[4] && b[2] <= b[5];
            if (!valid) continue;
            if (L.type == 1 || L.type == 2) {
                V3 r3 = splat(L.range);
                V3 qmn = L.pos - r3, qmx = L.pos + r3;
                bool ov = !(qmn.x > b[3] || qmx.x < b[0] || qmn.y > b[4] || qmx.y < b[1] || qmn.z > b[5] || qmx.z < b[2]);
                lit[(size_t) l * n_inst + i] = ov ? 1 : 0;
            } else if (L.type == 3) {
                lit[(size_t) l * n_inst + i] = 1;
            }
        }
    }

    // Raster records and per-pass bounding boxes (RasterizeInstance /
    // RasterizeTriangle2D_x2_ex set-up, lighter.cpp:32-66, lighter_math.cpp:251-267).
    TRACE("light culling done");
    // Raster records (kRT floats per triangle, in instance / part / triangle
    // order) and their bounding boxes, filled in parallel over the triangles.
    std::vector<unsigned long long> tex_off(n_inst + 1, 0);
    std::vector<u32> inst_w(n_inst, 0), inst_h(n_inst, 0);
    unsigned long long ntex = 0;
    struct Seg { int inst; u32 part; size_t first; };   // a part's triangles start at record `first`
    std::vector<Seg> segs;
    size_t n_rec = 0;
    for (int i = 0; i < n_inst; ++i) {
        HostInst* mi = S->insts[i];
        tex_off[i] = ntex;
        if (mi->container) continue;
        inst_w[i] = mi->w;
        inst_h[i] = mi->h;
        ntex += (unsigned long long) mi->w * mi->h;
        for (u32 part = 0; part < mi->mesh->parts.size(); ++part) {
            segs.push_back(Seg{i, part, n_rec});
            n_rec += mi->mesh->parts[part].icount / 3;
        }
    }
    std::vector<float> rt(n_rec * kRT);
    std::vector<u32> rinst(n_rec);
    parallel_for(n_rec, 4096, [&](size_t k0, size_t k1) {
        size_t si = std::upper_bound(segs.begin(), segs.end(), k0, [](size_t k, const Seg& g) { return k < g.first; }) -
                    segs.begin() - 1;
        for (size_t k = k0; k < k1; ++k) {
            while (si + 1 < segs.size() && segs[si + 1].first <= k) ++si;
            const Seg& g = segs[si];
            HostInst* mi = S->insts[g.inst];
            const HostPart& p = mi->mesh->parts[g.part];
            const u32* ib = &mi->mesh->idx[p.ioff];
            const u32 t = (u32) (k - g.first) * 3;
            u32 i1 = p.voff + ib[t], i2 = p.voff + ib[t + 1], i3 = p.voff + ib[t + 2];
            float lmarea = tri_area2(mi->ltex[i1], mi->ltex[i2], mi->ltex[i3]);
            float coarea = tri_area3(mi->vpos[i1], mi->vpos[i2], mi->vpos[i3]);
            float sa = lmarea > 0 ? coarea / lmarea : 0;
            const u32 ids[3] = {i1, i2, i3};
            float* o = &rt[k * kRT];
            for (u32 v : ids) { *o++ = mi->ltex[v].x; *o++ = mi->ltex[v].y; }
            for (u32 v : ids) { *o++ = mi->vpos[v].x; *o++ = mi->vpos[v].y; *o++ = mi->vpos[v].z; }
            for (u32 v : ids) { *o++ = mi->vnrm[v].x; *o++ = mi->vnrm[v].y; *o++ = mi->vnrm[v].z; }
            for (u32 v : ids) { *o++ = mi->vtex[v].x; *o++ = mi->vtex[v].y; }
            *o++ = (float) g.part;
            *o++ = sa;
            rinst[k] = (u32) g.inst;
        }
    });
    tex_off[n_inst] = ntex;
    TRACE("raster records done");
    const int n_rt = (int) rinst.size();
    if (n_rt >= (1 << 30) - 1) throw std::runtime_error("too many triangles for the raster keys");
    S->stats.texels = ntex;
    std::vector<int4> bbox[2];
    std::vector<unsigned long long> woff[2];
    const float margins[2] = {0.5f + kSmall, 0.0f};
    for (int pass = 0; pass < 2; ++pass) {
        bbox[pass].resize(n_rt);
        woff[pass].resize(n_rt + 1);
        const float mg = margins[pass];
        parallel_for((size_t) n_rt, 4096, [&](size_t k0, size_t k1) {
            for (size_t k = k0; k < k1; ++k) {
                const float* r = &rt[k * kRT];
                u32 inst = rinst[k];
                int w = (int) inst_w[inst], h = (int) inst_h[inst];
                int maxX = (int) (fmax_(r[0], fmax_(r[2], r[4])) + mg);
                int minX = (int) (fmin_(r[0], fmin_(r[2], r[4])) - mg);
                int maxY = (int) (fmax_(r[1], fmax_(r[3], r[5])) + mg);
                int minY = (int) (fmin_(r[1], fmin_(r[3], r[5])) - mg);
                bool empty = maxX < 0 || minX >= w || maxY < 0 || minY >= h;
                if (minX < 0) minX = 0;
                if (maxX >= w) maxX = w - 1;
                if (minY < 0) minY = 0;
                if (maxY >= h) maxY = h - 1;
                V2 p1 = mk2(r[0], r[1]), p2 = mk2(r[2], r[3]), p3 = mk2(r[4], r[5]);
                if (cross2(p2 - p1, p3 - p1) == 0) empty = true;
                if (maxX < minX || maxY < minY) empty = true;
                bbox[pass][k] = empty ? make_int4(0, 0, 1, 0) : make_int4(minX, minY, maxX - minX + 1, maxY - minY + 1);
            }
        });
        unsigned long long acc = 0;   // work offsets (texels covered by each box), in order
        for (int k = 0; k < n_rt; ++k) {
            woff[pass][k] = acc;
            const int4 b = bbox[pass][k];
            if (b.w > 0) acc += (unsigned long long) b.z * (unsigned long long) b.w;
        }
        woff[pass][n_rt] = acc;
    }

    TRACE("host records done");
    // ---- upload
    cudaEvent_t e_up0 = clock.mark();
    const u32 n_probe = (u32) S->samples.size();
    unsigned char* d_lit = A.upload(lit);
    DLight* d_lights = A.upload(dl);
    float* d_rt = A.upload(rt);
    u32* d_rinst = A.upload(rinst);
    unsigned long long* d_tex_off = A.upload(tex_off);
    u32* d_inst_w = A.upload(inst_w);
    u32* d_inst_h = A.upload(inst_h);
    int4* d_bbox[2];
    unsigned long long* d_woff[2];
    for (int p = 0; p < 2; ++p) { d_bbox[p] = A.upload(bbox[p]); d_woff[p] = A.upload(woff[p]); }
    // one error word per stage kernel: 0 fixup, 1 direct, 2 radiosity, 3 AO
    u32* d_err = A.zeros<u32>(8);
    Counters* d_cnt = A.zeros<Counters>(1);
    ErrFlag err_fix{d_err + 0}, err_direct{d_err + 1}, err_rad{d_err + 2}, err_ao{d_err + 3};
    cudaEvent_t e_up1 = clock.mark();
    check_abort(S);

    TRACE("upload issued");
    // ---- BVH (joined)
    if (bvh_thread.joinable()) bvh_thread.join();
    if (bvh_error) std::rethrow_exception(bvh_error);
    host_counters().launches += bvh_counts.launches;
    host_counters().h2d += bvh_counts.h2d;
    host_counters().d2h += bvh_counts.d2h;
    if (bside.st) CK(cudaStreamWaitEvent(st, bside.e1, 0));
    S->stats.reserved[0] = (uint64_t) bin.n;   // leaf references
    BvhView bv = bvh.view();
    bv.watertight = S->opt.intersect_mode == LTRG_ISECT_WATERTIGHT ? 1 : 0;
    {
        // rounding bound of the distance test against the plane distance: a few
        // single-precision dot products over coordinates up to the scene's largest
        float mx = 0.0f;
        for (float v : tri_xyz) mx = fmaxf(mx, fabsf(v));
        bv.dist_margin = std::isfinite(mx) ? 4e-6f * (1.0f + mx) : INFINITY;
    }
    cudaEvent_t e_bvh = clock.mark();
    // LTRG_VALIDATE=1: re-check the BVH topology after every stage
    const bool validate = getenv("LTRG_VALIDATE") && getenv("LTRG_VALIDATE")[0] == '1';
    auto checkpoint = [&](const char* where) {
        if (!validate) return;
        CK(cudaStreamSynchronize(st));
        std::string e = bvh_validate(bvh, st);
        if (!e.empty()) throw std::runtime_error(std::string("BVH corrupted after ") + where + ": " + e);
    };
    checkpoint("build");

    // ---- samples (Job_Samples)
    TRACE("bvh issued");
    S->stage = "generating samples";
    u32* d_keys = A.zeros<u32>(ntex);
    for (int pass = 0; pass < 2; ++pass) {
        unsigned long long nw = woff[pass][n_rt];
        if (nw == 0) continue;
        k_raster_mark<<<blocks_for(nw), kThreads, 0, st>>>(pass, margins[pass], d_rt, d_rinst, d_bbox[pass],
                                                           d_woff[pass], n_rt, nw, d_tex_off, d_inst_w, d_keys); note_launch();
        CK(cudaGetLastError());
        checkpoint("raster mark");
    }
    float4* d_R1 = A.alloc<float4>(ntex);
    float4* d_R2 = A.alloc<float4>(ntex);
    float4* d_R3 = A.alloc<float4>(ntex);
    u32* d_flags = A.alloc<u32>(ntex + 1);
    u32* d_scan = A.alloc<u32>(ntex + 1);
    CK(cudaMemsetAsync(d_flags + ntex, 0, sizeof(u32), st));
    if (ntex) {
        k_raster_resolve<<<blocks_for(ntex), kThreads, 0, st>>>(ntex, d_keys, d_rt, d_rinst, d_tex_off, d_inst_w,
                                                                d_R1, d_R2, d_R3, d_flags); note_launch();
        CK(cudaGetLastError());
        checkpoint("raster resolve");
    }
    {
        size_t tb = 0;
        CK(cub::DeviceScan::ExclusiveSum(nullptr, tb, d_flags, d_scan, (int64_t) (ntex + 1), st));
        void* tmp = A.alloc<char>(tb);
        CK(cub::DeviceScan::ExclusiveSum(tmp, tb, d_flags, d_scan, (int64_t) (ntex + 1), st));
    }
    // per-instance sample starts = scan at each instance's first texel
    std::vector<u32> inst_sbeg(n_inst + 1, 0);
    for (int i = 1; i <= n_inst; ++i)
        CK(cudaMemcpyAsync(&inst_sbeg[i], d_scan + tex_off[i == n_inst ? n_inst : i], sizeof(u32),
                           cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const u32 n_cov = inst_sbeg[n_inst];
    TRACE("sample counts read");
    const u32 n_samples = n_probe + n_cov;
    S->stats.samples = n_samples;
    // sample ranges: instance 0 = probes [0, n_probe); instance i = n_probe + [scan(tex_off[i]), scan(tex_off[i+1]))
    std::vector<u32> sbeg(n_inst + 1), scount(n_inst);
    sbeg[0] = 0;
    scount[0] = n_probe;
    for (int i = 1; i < n_inst; ++i) {
        u32 b = n_probe + inst_sbeg[i];
        u32 e = n_probe + (i + 1 < n_inst ? inst_sbeg[i + 1] : n_cov);
        sbeg[i] = b;
        scount[i] = e - b;
    }

    // sample_fn runs on the device when it is the library's table function
    // (or NULL); any other callback is called on this thread, in sample order.
    const bool gpu_sample_fn = !cfg.sample_fn || cfg.sample_fn == ltrg_TableSampleFn;
    // AO's per-sample rand() draws (lighter.cpp:819) come after every user
    // callback that could call rand() itself: here unless a host sample_fn
    // still has to run, in which case they follow its calls.
    // drawn into page-locked memory the scene keeps, so their upload does not wait
    // for the kernels queued before it
    float* ao_randoff = nullptr;
    if (n_samples && cfg.ao_distance && cfg.ao_num_samples > 0) {
        if (S->ao_pinned_n < n_samples) {
            if (S->ao_pinned) cudaFreeHost(S->ao_pinned);
            S->ao_pinned = nullptr;
            S->ao_pinned_n = 0;
            CK(cudaHostAlloc((void**) &S->ao_pinned, (size_t) n_samples * sizeof(float), cudaHostAllocDefault));
            S->ao_pinned_n = n_samples;
        }
        ao_randoff = S->ao_pinned;
    }
    std::thread ao_thread;
    const bool do_ao = cfg.ao_distance && n_samples && cfg.ao_num_samples > 0;
    if (batch && !do_ao) batch->rand_end(bidx);   // draws nothing: the next scene's turn
    if (do_ao && (gpu_sample_fn || !cfg.bounce_count))
        ao_thread = std::thread([ao_randoff, n_samples, batch, bidx]() {
            if (batch) batch->rand_begin(bidx);
            rand_floats(ao_randoff, n_samples);   // instance order, sample order
            if (batch) batch->rand_end(bidx);
        });
    struct JoinGuard { std::thread& t; ~JoinGuard() { if (t.joinable()) t.join(); } } ao_guard{ao_thread};
    // leaving the batch's rendezvous before the join above waits on a draw turn
    // keeps a failed scene from holding the others
    struct BatchLeaveEarly {
        BatchCtx* b; int i;
        ~BatchLeaveEarly() { if (b) b->leave(i); }
    } batch_leave_early{batch, bidx};

    float4* d_spos = A.alloc<float4>(n_samples);
    float4* d_snrm = A.alloc<float4>(n_samples);
    float4* d_srad = A.zeros<float4>(n_samples);
    u32* d_sloc = A.alloc<u32>(n_samples);
    u32* d_sinst = A.alloc<u32>(n_samples);
    if (n_probe) {
        std::vector<float4> pp(n_probe), pn(n_probe);
        std::vector<u32> pl(n_probe, kNoLoc), pi(n_probe, 0);
        for (u32 i = 0; i < n_probe; ++i) {
            const ltr_SampleInfo& si = S->samples[i];
            pp[i] = make_float4(si.position[0], si.position[1], si.position[2], 0);
            pn[i] = make_float4(si.normal[0], si.normal[1], si.normal[2], 0);
        }
        CK(cudaMemcpyAsync(d_spos, pp.data(), n_probe * sizeof(float4), cudaMemcpyHostToDevice, st)); note_h2d(n_probe * sizeof(float4));
        CK(cudaMemcpyAsync(d_snrm, pn.data(), n_probe * sizeof(float4), cudaMemcpyHostToDevice, st)); note_h2d(n_probe * sizeof(float4));
        CK(cudaMemcpyAsync(d_sloc, pl.data(), n_probe * sizeof(u32), cudaMemcpyHostToDevice, st)); note_h2d(n_probe * sizeof(u32));
        CK(cudaMemcpyAsync(d_sinst, pi.data(), n_probe * sizeof(u32), cudaMemcpyHostToDevice, st)); note_h2d(n_probe * sizeof(u32));
        CK(cudaStreamSynchronize(st));
    }
    if (ntex) {
        k_compact<<<blocks_for(ntex), kThreads, 0, st>>>(ntex, d_flags, d_scan, d_R1, d_R2, d_R3, d_tex_off, n_inst,
                                                         n_probe, d_spos, d_snrm, d_srad, d_sloc, d_sinst); note_launch();
        CK(cudaGetLastError());
        checkpoint("compaction");
    }
    // trace orders of the two trace stages (null: sample order)
    const u32* d_order_dir = nullptr;
    const u32* d_order_ao = nullptr;
    {
        const ltrg_Tuning tu = get_tuning(S->opt.device);
        u32* made[3] = {nullptr, nullptr, nullptr};
        auto order_for = [&](u32 mode) -> const u32* {
            if (mode == 0 || mode > 2 || !n_samples) return nullptr;
            if (made[mode]) return made[mode];
            u32* d_ord = A.alloc<u32>(n_samples);
            unsigned long long* d_okeys = A.alloc<unsigned long long>(n_samples);
            unsigned long long* d_okeys2 = A.alloc<unsigned long long>(n_samples);
            u32* d_ovals = A.alloc<u32>(n_samples);
            float3 mn = make_float3(gmin[0], gmin[1], gmin[2]);
            float3 ie = make_float3(gmax[0] > gmin[0] ? 1.0f / (gmax[0] - gmin[0]) : 0.0f,
                                    gmax[1] > gmin[1] ? 1.0f / (gmax[1] - gmin[1]) : 0.0f,
                                    gmax[2] > gmin[2] ? 1.0f / (gmax[2] - gmin[2]) : 0.0f);
            k_order_keys<<<blocks_for(n_samples), kThreads, 0, st>>>((int) mode, n_samples, d_sinst, d_sloc, d_inst_w, d_spos,
                                                                    mn, ie, d_okeys, d_ovals);
            note_launch();
            CK(cudaGetLastError());
            int end_bit = 32;
            if (mode == 1)
                while (end_bit < 64 && ((unsigned long long) n_inst >> (end_bit - 32)) != 0) ++end_bit;
            size_t tb = 0;
            CK(cub::DeviceRadixSort::SortPairs(nullptr, tb, d_okeys, d_okeys2, d_ovals, d_ord, (int) n_samples, 0, end_bit, st));
            void* tmp = A.alloc<char>(tb);
            CK(cub::DeviceRadixSort::SortPairs(tmp, tb, d_okeys, d_okeys2, d_ovals, d_ord, (int) n_samples, 0, end_bit, st));
            made[mode] = d_ord;
            return d_ord;
        };
        d_order_dir = order_for(tu.direct_order);
        d_order_ao = order_for(tu.ao_order);
    }
    reftree_thread.join();
    TRACE("reference trees joined");
    if (reftree_error) std::rethrow_exception(reftree_error);
    float4* d_ref_nodes = A.upload(ref_nodes);
    int* d_ref_items = A.upload(ref_items);
    int4* d_ref_inst = A.upload(ref_inst);
    float4* d_fix_box = A.upload(fix_box);
    if (n_cov) {
        FixupArgs fa;
        fa.bvh = bv;
        fa.err = err_fix;
        fa.ref_nodes = d_ref_nodes;
        fa.ref_items = d_ref_items;
        fa.ref_inst = d_ref_inst;
        fa.inst_box = d_fix_box;
        fa.tri_xyz = d_tri_xyz;
        const u32 n_fix_tris = (u32) (tri_xyz.size() / 9);
        float4* d_tri_box = A.alloc<float4>(2 * (size_t) std::max<u32>(n_fix_tris, 1));
        if (n_fix_tris) {
            k_tri_boxes<<<(n_fix_tris + 255) / 256, 256, 0, st>>>(d_tri_xyz, n_fix_tris, d_tri_box); note_launch();
        }
        fa.tri_box = d_tri_box;
        fa.n_inst = n_inst;
        fa.n_probe = n_probe;
        fa.n_samples = n_samples;
        fa.max_correct_dist = cfg.max_correct_dist;
        fa.corr_min_dot = cosf(cfg.max_correct_angle / 180.0f * 3.14159265358979323846f);
        fa.spos = d_spos;
        fa.snrm = d_snrm;
        fa.srad = d_srad;
        k_fixup<<<(n_cov + kFixupThreads - 1) / kFixupThreads, kFixupThreads, 0, st>>>(fa); note_launch();
        CK(cudaGetLastError());
        checkpoint("sample fixup");
    }
    TRACE("fixup issued");
    cudaEvent_t e_samples = clock.mark();
    cudaEvent_t e_dtr0 = nullptr, e_dtr1 = nullptr, e_aotr0 = nullptr, e_aotr1 = nullptr;   // the trace kernels alone
    check_abort(S);

    // ---- direct light (Int_LMRender per light)
    float4* d_lm = A.alloc<float4>(n_samples);
    float* d_kval = nullptr;
    float4* d_ndir = nullptr;
    S->stage = "rendering lightmaps";
    const bool want_normals = cfg.generate_normalmap_data != 0;
    float* d_vis = nullptr;       // debug records (keep_samples)
    float* d_ao_hits = nullptr;
    if (n_lights && n_samples) {
        d_kval = A.alloc<float>((size_t) n_lights * n_samples);
        if (S->opt.keep_samples) d_vis = A.alloc<float>((size_t) n_lights * n_samples);
        if (want_normals) d_ndir = A.alloc<float4>((size_t) n_lights * n_samples);
        DirectArgs da;
        da.bvh = bv;
        da.err = err_direct;
        da.lights = d_lights;
        da.n_lights = n_lights;
        da.n_inst = n_inst;
        da.lit = d_lit;
        da.n_samples = n_samples;
        da.spos = d_spos;
        da.snrm = d_snrm;
        da.sinst = d_sinst;
        da.kval = d_kval;
        da.ndir = d_ndir;
        da.counters = d_cnt;
        da.vis = d_vis;
        da.order = d_order_dir;
        da.shadow_mode = (int) S->opt.shadow_mode;
        da.lsmp = lsmp.empty() ? nullptr : A.upload(lsmp);
        da.abort_word = d_abort;
        unsigned long long items = (unsigned long long) n_lights * n_samples;
        if (items >= 0xffffffffull) throw std::runtime_error("too many (light, sample) pairs for one bake");
        u32* d_dflags = A.alloc<u32>(items + 1);
        u32* d_dscan = A.alloc<u32>(items + 1);
        CK(cudaMemsetAsync(d_dflags + items, 0, sizeof(u32), st));
        k_direct_setup<<<blocks_for(items), kThreads, 0, st>>>(da, d_dflags); note_launch();
        CK(cudaGetLastError());
        size_t tb = 0;
        CK(cub::DeviceScan::ExclusiveSum(nullptr, tb, d_dflags, d_dscan, (int64_t) (items + 1), st));
        void* tmp = A.alloc<char>(tb);
        CK(cub::DeviceScan::ExclusiveSum(tmp, tb, d_dflags, d_dscan, (int64_t) (items + 1), st));
        u32* d_items = A.alloc<u32>(items);
        k_direct_compact<<<blocks_for(items), kThreads, 0, st>>>(items, n_samples, d_order_dir, d_dflags, d_dscan, d_items);
        note_launch();
        CK(cudaGetLastError());
        // persistent grid of a few blocks per SM; the number of traced pairs
        // stays on the device (scan total), so the host does not wait here
        u32* d_next = A.zeros<u32>(1);
        int dev_sms = 0;
        CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, S->opt.device));
        if (batch && items < kBatchSoloItems) {   // one trace launch for the whole batch
            DirectJob job{da, d_items, d_dscan + items};
            CK(cudaStreamWaitEvent(st, batch->join(0, bidx, st, &job, nullptr, 0), 0));
        } else {
            if (batch) batch->skip(0, bidx);   // enough pairs to fill the GPU alone
            const ltrg_Tuning tu = get_tuning(S->opt.device);
            unsigned grid = (unsigned) std::min<unsigned long long>((unsigned long long) dev_sms * tu.direct_blocks_per_sm,
                                                                    (items + tu.direct_block - 1) / tu.direct_block);
            e_dtr0 = clock.mark();
            launch_direct_trace(tu, grid, st, da, d_items, d_dscan + items, d_next);
            note_launch();
            CK(cudaGetLastError());
            e_dtr1 = clock.mark();
        }
    } else if (batch) {
        batch->skip(0, bidx);
    }
    if (n_samples) {
        k_accumulate<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
            n_samples, n_lights, d_lights, d_kval, cfg.ambient_color[0], cfg.ambient_color[1], cfg.ambient_color[2], d_lm); note_launch();
        CK(cudaGetLastError());
    }
    TRACE("direct issued");
    cudaEvent_t e_direct = clock.mark();

    // Copies on a side stream overlap the direct-light kernels: the sample
    // arrays the host needs for sample_fn and patch grouping are final once
    // the sample stage has ended (event e_samples).
    cudaStream_t st2 = nullptr;
    CK(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    } st2_guard{st2};
    const bool do_rad = cfg.bounce_count && n_samples;
    std::vector<float4> hpos, hnrm, hrad;
    std::vector<u32> hloc;
    if (do_rad) {
        CK(cudaStreamWaitEvent(st2, e_samples, 0));
        if (!gpu_sample_fn) {   // the host calls sample_fn with position and texcoords
            hpos.resize(n_samples); hrad.resize(n_samples);
            CK(cudaMemcpyAsync(hpos.data(), d_spos, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st2)); note_d2h(n_samples * sizeof(float4));
            CK(cudaMemcpyAsync(hrad.data(), d_srad, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st2)); note_d2h(n_samples * sizeof(float4));
        }
        if (!gpu_sample_fn) {   // sample_fn requests
            hnrm.resize(n_samples); hloc.resize(n_samples);
            CK(cudaMemcpyAsync(hnrm.data(), d_snrm, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st2)); note_d2h(n_samples * sizeof(float4));
            CK(cudaMemcpyAsync(hloc.data(), d_sloc, n_samples * sizeof(u32), cudaMemcpyDeviceToHost, st2)); note_d2h(n_samples * sizeof(u32));
        }
    }
    check_abort(S);

    // ---- radiosity (Int_RDGenLinks + Int_RDBounce)
    // The host part (sample_fn per sample, patch grouping) runs while the
    // direct-light kernels are still tracing: the sample arrays it needs were
    // copied on the side stream as soon as the sample stage ended.
    cudaEvent_t e_rad_links = e_direct, e_rad_bounce = e_direct;
    if (do_rad) {
        S->stage = "calculating radiosity";
        CK(cudaStreamSynchronize(st2));
        TRACE("sample copies done");
        float4* d_diff = A.alloc<float4>(n_samples);
        float4* d_emis = A.alloc<float4>(n_samples);
        std::vector<float4> hdiff, hemis;
        if (gpu_sample_fn) {
            const ltrg_SampleTable* tab = cfg.sample_fn ? (const ltrg_SampleTable*) cfg.userdata : nullptr;
            u32 count = tab ? tab->count : 0;
            std::vector<float> td, te;
            if (tab && tab->diffuse_rgb) td.assign(tab->diffuse_rgb, tab->diffuse_rgb + 3 * (size_t) count);
            if (tab && tab->emissive_rgb) te.assign(tab->emissive_rgb, tab->emissive_rgb + 3 * (size_t) count);
            float* d_td = td.empty() ? nullptr : A.upload(td);
            float* d_te = te.empty() ? nullptr : A.upload(te);
            k_table_samples<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                n_samples, d_srad, d_sinst, cfg.sample_fn != nullptr && tab != nullptr, count, d_td, d_te, d_diff, d_emis); note_launch();
            CK(cudaGetLastError());
        } else {
        hdiff.resize(n_samples);
        hemis.resize(n_samples);
        for (int i = 0; i < n_inst; ++i) {
            HostInst* mi = S->insts[i];
            for (u32 k = 0; k < scount[i]; ++k) {
                u32 s = sbeg[i] + k;
                V3 diff = mk(1, 1, 1), emis = mk(0, 0, 0);
                if (mi->container) {
                    diff = mk(0, 0, 0);
                } else if (cfg.sample_fn) {   // lighter.cpp:692-714
                    V3 P = mk(hpos[s].x, hpos[s].y, hpos[s].z);
                    V3 N = normalized(mk(hnrm[s].x, hnrm[s].y, hnrm[s].z));
                    u32 L = hloc[s];
                    int lx = (int) (L % mi->w), ly = (int) (L / mi->w);
                    ltr_SampleRequest req;
                    req.position[0] = P.x; req.position[1] = P.y; req.position[2] = P.z;
                    req.normal[0] = N.x; req.normal[1] = N.y; req.normal[2] = N.z;
                    req.tex0u = hrad[s].x; req.tex0v = hrad[s].y;
                    req.tex1u = (lx + 0.5f) / mi->w; req.tex1v = (ly + 0.5f) / mi->h;
                    req.part_id = (uint32_t) hrad[s].z;
                    req.mesh_ident = mi->mesh->ident.c_str(); req.mesh_ident_size = mi->mesh->ident.size();
                    req.inst_ident = mi->ident.c_str(); req.inst_ident_size = mi->ident.size();
                    req.out_diffuse_color[0] = req.out_diffuse_color[1] = req.out_diffuse_color[2] = 1;
                    req.out_emissive_color[0] = req.out_emissive_color[1] = req.out_emissive_color[2] = 0;
                    if (cfg.sample_fn(const_cast<ltr_Config*>(&cfg), &req)) {
                        diff = mk(req.out_diffuse_color[0], req.out_diffuse_color[1], req.out_diffuse_color[2]);
                        emis = mk(req.out_emissive_color[0], req.out_emissive_color[1], req.out_emissive_color[2]);
                    }
                }
                hdiff[s] = make_float4(diff.x, diff.y, diff.z, 0);
                hemis[s] = make_float4(emis.x, emis.y, emis.z, 0);
            }
        }
        // AO draws its per-sample random offsets after the last sample_fn call,
        // as the reference's AO stage comes after radiosity
        if (do_ao && !ao_thread.joinable()) {
            // in a batch no slot is held while waiting for the turn (and drawing)
            if (batch) {
                batch->release();
                batch->rand_begin(bidx);
            }
            rand_floats(ao_randoff, n_samples);
            if (batch) {
                batch->rand_end(bidx);
                batch->acquire();
            }
        }
        CK(cudaMemcpyAsync(d_diff, hdiff.data(), n_samples * sizeof(float4), cudaMemcpyHostToDevice, st2)); note_h2d(n_samples * sizeof(float4));
        CK(cudaMemcpyAsync(d_emis, hemis.data(), n_samples * sizeof(float4), cudaMemcpyHostToDevice, st2)); note_h2d(n_samples * sizeof(float4));
        }
        // per-sample radiosity inputs once direct light is done
        float4* d_rpos = A.alloc<float4>(n_samples);
        float4* d_rnrm = A.alloc<float4>(n_samples);
        float4* d_rda = A.alloc<float4>(n_samples);
        float4* d_remit = A.alloc<float4>(n_samples);

        RadSettings rs;
        rs.links = S->opt.radiosity_links;
        rs.precision = S->opt.radiosity_precision;
        rs.refine_steps = S->opt.refine_steps;
        rs.bounces = cfg.bounce_count;
        RadResult rr;
        // debug records of the radiosity elements (keep_samples)
        auto rad_dump_begin = [&](u32 n) {
            if (!S->opt.keep_samples) return;
            S->rad_dump.n = n;
            if (n <= RadDump::kRadDumpMaxF) {
                S->rad_dump.F.resize((size_t) n * n);
                rs.f_host = S->rad_dump.F.data();
            }
        };
        auto rad_dump_end = [&](u32 n, const float4* pos, const float4* nrm, const float4* da, const float4* emit,
                                const float4* total) {
            if (!S->opt.keep_samples) return;
            RadDump& d = S->rad_dump;
            std::vector<float>* dst[5] = {&d.pos, &d.nrm, &d.diff_area, &d.emit, &d.total};
            const float4* src[5] = {pos, nrm, da, emit, total};
            for (int k = 0; k < 5; ++k) {
                dst[k]->resize(4 * (size_t) n);
                CK(cudaMemcpyAsync(dst[k]->data(), src[k], n * sizeof(float4), cudaMemcpyDeviceToHost, st)); note_d2h(n * sizeof(float4));
            }
            CK(cudaStreamSynchronize(st));
        };
        if (S->opt.radiosity_patches == 0) {
            cudaEvent_t up = nullptr;
            CK(cudaEventCreateWithFlags(&up, cudaEventDisableTiming));
            CK(cudaEventRecord(up, st2));
            CK(cudaStreamWaitEvent(st, up, 0));
            k_rad_sample_inputs<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                n_samples, d_spos, d_snrm, d_srad, d_sinst, d_diff, d_emis, d_lm, d_rpos, d_rnrm, d_rda, d_remit); note_launch();
            CK(cudaGetLastError());
            cudaEventDestroy(up);
            RadDevInputs ri{n_samples, d_rpos, d_rnrm, d_rda, d_remit};
            rad_dump_begin(n_samples);
            rr = radiosity_solve_dev(ri, rs, bv, err_rad, st, d_lm, &S->abort_flag);
            rad_dump_end(n_samples, d_rpos, d_rnrm, d_rda, d_remit, d_lm);
            S->stats.rad_elements = n_samples;
        } else {
            // Patch mode: group samples by (instance, lightmap tile, dominant
            // normal axis) on the device. Patches are numbered in slot order;
            // each patch's samples are listed in sample order (stable sort).
            // The tile side (texels) is chosen so the patch count comes closest to
            // the requested one: the first guess sqrt(covered texels / target)
            // ignores partly covered tiles and the split by normal axis, so a
            // few trials count the occupied slots of neighbouring sides.
            u32 target = S->opt.radiosity_patches;
            std::vector<u32> slot_base(n_inst + 1, 0), ntx(n_inst, 0);
            auto layout = [&](u32 t) {
                for (int i = 0; i < n_inst; ++i) {
                    HostInst* mi = S->insts[i];
                    ntx[i] = mi->container ? 0 : (mi->w + t - 1) / t;
                    u32 ns = mi->container ? 0 : ntx[i] * ((mi->h + t - 1) / t) * 6;
                    slot_base[i + 1] = slot_base[i] + ns;
                }
                return slot_base[n_inst];
            };
            u32* d_slot_of = A.alloc<u32>(n_samples);
            u32* d_count = A.alloc<u32>(1);
            auto trial = [&](u32 t) -> u32 {
                const u32 ns = layout(t);
                u32* d_sb = A.upload(slot_base);
                u32* d_nt = A.upload(ntx);
                u32* d_o = A.zeros<u32>(ns + 1);
                CK(cudaMemsetAsync(d_count, 0, sizeof(u32), st));
                k_patch_slots<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                    n_samples, d_snrm, d_sloc, d_sinst, d_inst_w, d_sb, d_nt, t, d_slot_of, d_o, d_count); note_launch();
                CK(cudaGetLastError());
                u32 c = 0;
                CK(cudaMemcpyAsync(&c, d_count, sizeof(u32), cudaMemcpyDeviceToHost, st)); note_d2h(4);
                CK(cudaStreamSynchronize(st));
                return c;
            };
            u32 tile = (u32) std::max(1.0, std::floor(std::sqrt(std::max(1.0, (double) n_cov / target)) + 0.5));
            {
                auto off = [&](u32 c) { return std::fabs(std::log(std::max(1.0, (double) c) / target)); };
                u32 c = trial(tile), best = tile;
                double best_off = off(c);
                const int dir = c > target ? 1 : -1;
                for (int k = 0; k < 8; ++k) {
                    if ((dir > 0 && c <= target) || (dir < 0 && (c >= target || tile == 1))) break;
                    // next side from the area scaling, at least one texel on
                    u32 t2 = (u32) std::floor(tile * std::sqrt((double) c / target) + 0.5);
                    t2 = dir > 0 ? std::max(t2, tile + 1) : std::max(1u, std::min(t2, tile - 1));
                    tile = t2;
                    c = trial(tile);
                    if (off(c) < best_off) { best_off = off(c); best = tile; }
                }
                tile = best;
            }
            const u32 nslots = layout(tile);
            u32* d_slot_base = A.upload(slot_base);
            u32* d_ntx = A.upload(ntx);
            u32* d_occ = A.zeros<u32>(nslots + 1);
            u32* d_slot_scan = A.alloc<u32>(nslots + 1);
            k_patch_slots<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                n_samples, d_snrm, d_sloc, d_sinst, d_inst_w, d_slot_base, d_ntx, tile, d_slot_of, d_occ, nullptr); note_launch();
            CK(cudaGetLastError());
            {
                size_t tb = 0;
                CK(cub::DeviceScan::ExclusiveSum(nullptr, tb, d_occ, d_slot_scan, (int64_t) (nslots + 1), st));
                void* tmp = A.alloc<char>(tb);
                CK(cub::DeviceScan::ExclusiveSum(tmp, tb, d_occ, d_slot_scan, (int64_t) (nslots + 1), st));
            }
            u32 np = 0;
            CK(cudaMemcpyAsync(&np, d_slot_scan + nslots, sizeof(u32), cudaMemcpyDeviceToHost, st)); note_d2h(4);
            int* d_patch_of = A.alloc<int>(n_samples);
            u32* d_keys_in = A.alloc<u32>(n_cov);
            u32* d_keys_out = A.alloc<u32>(n_cov);
            u32* d_vals_in = A.alloc<u32>(n_cov);
            u32* d_csr_idx = A.alloc<u32>(n_cov);
            k_patch_ids<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                n_samples, n_probe, d_slot_of, d_slot_scan, d_patch_of, d_keys_in, d_vals_in); note_launch();
            CK(cudaGetLastError());
            {
                size_t tb = 0;
                CK(cub::DeviceRadixSort::SortPairs(nullptr, tb, d_keys_in, d_keys_out, d_vals_in, d_csr_idx, (int) n_cov, 0, 32, st));
                void* tmp = A.alloc<char>(tb);
                CK(cub::DeviceRadixSort::SortPairs(tmp, tb, d_keys_in, d_keys_out, d_vals_in, d_csr_idx, (int) n_cov, 0, 32, st));
            }
            CK(cudaStreamSynchronize(st));
            u32* d_csr_off = A.alloc<u32>(np + 1);
            k_patch_offsets<<<(n_cov + kThreads - 1) / kThreads, kThreads, 0, st>>>(n_cov, np, d_keys_out, d_csr_off); note_launch();
            CK(cudaGetLastError());
            float4* d_ppos = A.alloc<float4>(np);
            float4* d_pnrm = A.alloc<float4>(np);
            float4* d_pda = A.alloc<float4>(np);
            float4* d_pemit = A.alloc<float4>(np);
            float4* d_ptot = A.alloc<float4>(np);
            if (np) {
                k_patch_inputs<<<(unsigned) (((size_t) np * 32 + 255) / 256), 256, 0, st>>>(np, d_csr_off, d_csr_idx, d_spos, d_snrm, d_srad, d_diff,
                                                                 d_emis, d_lm, d_ppos, d_pnrm, d_pda, d_pemit); note_launch();
                CK(cudaGetLastError());
                RadDevInputs pi{np, d_ppos, d_pnrm, d_pda, d_pemit};
                rad_dump_begin(np);
                rr = radiosity_solve_dev(pi, rs, bv, err_rad, st, d_ptot, &S->abort_flag);
                rad_dump_end(np, d_ppos, d_pnrm, d_pda, d_pemit, d_ptot);
                k_patch_apply<<<(n_samples + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                    n_samples, d_patch_of, d_emis, d_ptot, d_pemit, d_lm); note_launch();
                CK(cudaGetLastError());
            }
            S->stats.rad_elements = np;
        }
        TRACE("radiosity done");
        S->rad_links = (u32) rr.links;
        S->stats.rad_pairs = rr.pairs;
        S->stats.rad_vis_rays = rr.vis_rays;
        S->stats.ms_rad_links = rr.ms_links;
        S->stats.ms_rad_bounce = rr.ms_bounce;
        S->stage = "committing radiosity";
        e_rad_links = e_rad_bounce = clock.mark();
    }
    if (ao_thread.joinable()) {   // the draws may wait for earlier scenes of a batch: no slot held meanwhile
        if (batch) batch->release();
        ao_thread.join();
        if (batch) batch->acquire();
    }
    TRACE("ao draws joined");
    check_abort(S);

    // ---- ambient occlusion (Job_AORender)
    cudaEvent_t e_ao0 = clock.mark();
    if (do_ao) {
        S->stage = "rendering ambient occlusion";
        float* d_ro = A.alloc<float>(n_samples);
        CK(cudaMemcpyAsync(d_ro, ao_randoff, (size_t) n_samples * sizeof(float), cudaMemcpyHostToDevice, st));
        note_h2d((size_t) n_samples * sizeof(float));
        AoArgs aa;
        aa.bvh = bv;
        aa.err = err_ao;
        aa.n_samples = n_samples;
        aa.spos = d_spos;
        aa.snrm = d_snrm;
        aa.randoff = d_ro;
        aa.lm = d_lm;
        aa.dist = cfg.ao_distance;
        aa.falloff = cfg.ao_falloff;
        aa.mult = cfg.ao_multiplier;
        aa.effect = cfg.ao_effect;
        aa.ns = cfg.ao_num_samples;
        aa.order = d_order_ao;
        aa.abort_word = d_abort;
        for (int c = 0; c < 3; ++c) aa.aoc[c] = cfg.ao_color_rgb[c];
        aa.counters = d_cnt;
        if (aa.ns > 0) {
            unsigned long long n_rays = (unsigned long long) n_samples * aa.ns;
            float* d_hits = A.alloc<float>(n_rays);
            d_ao_hits = d_hits;
            unsigned long long* d_next = A.zeros<unsigned long long>(1);
            int dev_sms = 0;
            CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, S->opt.device));
            const unsigned long long n_items = ao_items(n_samples, aa.ns);
            if (batch && n_items < kBatchSoloItems) {   // one trace launch for the whole batch
                AoJob job{aa, d_hits};
                CK(cudaStreamWaitEvent(st, batch->join(1, bidx, st, nullptr, &job, n_items), 0));
            } else {
                if (batch) batch->skip(1, bidx);   // enough rays to fill the GPU alone
                const ltrg_Tuning tu = get_tuning(S->opt.device);
                unsigned grid = (unsigned) std::min<unsigned long long>((unsigned long long) dev_sms * tu.ao_blocks_per_sm,
                                                                        (n_items + tu.ao_block - 1) / tu.ao_block);
                e_aotr0 = clock.mark();
                launch_ao_rays(tu, grid, st, aa, d_hits, n_items, d_next); note_launch();
                CK(cudaGetLastError());
                e_aotr1 = clock.mark();
            }
            k_ao<<<blocks_for(n_samples), kThreads, 0, st>>>(aa, d_hits); note_launch();
            CK(cudaGetLastError());
        }
    } else if (batch) {
        batch->skip(1, bidx);
    }
    TRACE("ao issued");
    cudaEvent_t e_ao1 = clock.mark();
    check_abort(S);

    // ---- finalize (Int_Finalize)
    S->stage = "exporting lightmaps";
    float* d_img = A.zeros<float>(3 * ntex);
    unsigned char* d_maskA = A.zeros<unsigned char>(ntex);
    unsigned char* d_maskB = A.alloc<unsigned char>(ntex);
    if (n_cov) {
        k_scatter<<<(n_cov + kThreads - 1) / kThreads, kThreads, 0, st>>>(n_probe, n_samples, d_sloc, d_sinst, d_lm,
                                                                          d_tex_off, d_img, d_maskA); note_launch();
        CK(cudaGetLastError());
    }
    if (ntex) {
        for (int it = 0; it < 3; ++it) {
            CK(cudaMemcpyAsync(d_maskB, d_maskA, ntex, cudaMemcpyDeviceToDevice, st));
            k_dilate<<<blocks_for(ntex), kThreads, 0, st>>>(ntex, n_inst, d_tex_off, d_inst_w, d_inst_h, d_maskA,
                                                            d_maskB, d_img); note_launch();
            CK(cudaGetLastError());
            std::swap(d_maskA, d_maskB);
        }
    }
    if (cfg.blur_size && ntex) {
        int ext = (int) ceilf(cfg.blur_size);
        std::vector<float> taps = gauss_taps(ext, cfg.blur_size);
        float* d_taps = A.upload(taps);
        float* d_tmp = A.alloc<float>(3 * ntex);
        k_conv_t<<<blocks_for(ntex), kThreads, 0, st>>>(ntex, n_inst, d_tex_off, d_inst_w, d_inst_h, 0, ext, d_taps,
                                                        d_img, d_tmp); note_launch();
        CK(cudaGetLastError());
        k_conv_t<<<blocks_for(ntex), kThreads, 0, st>>>(ntex, n_inst, d_tex_off, d_inst_w, d_inst_h, 1, ext, d_taps,
                                                        d_tmp, d_img); note_launch();
        CK(cudaGetLastError());
    }
    // output layout (after optional ds2x)
    std::vector<unsigned long long> out_off(n_inst + 1, 0);
    std::vector<u32> out_w(n_inst, 0), out_h(n_inst, 0);
    unsigned long long nout = 0;
    for (int i = 0; i < n_inst; ++i) {
        out_off[i] = nout;
        if (S->insts[i]->container) continue;
        u32 w = inst_w[i], h = inst_h[i];
        if (cfg.ds2x) { w = std::max(w / 2, 1u); h = std::max(h / 2, 1u); }
        out_w[i] = w;
        out_h[i] = h;
        nout += (unsigned long long) w * h;
    }
    out_off[n_inst] = nout;
    float* d_out = d_img;
    if (cfg.ds2x && nout) {
        unsigned long long* d_out_off = A.upload(out_off);
        d_out = A.alloc<float>(3 * nout);
        k_ds2x<<<blocks_for(nout), kThreads, 0, st>>>(nout, n_inst, d_out_off, d_tex_off, d_inst_w, d_inst_h, d_img, d_out); note_launch();
        CK(cudaGetLastError());
    }
    float* d_nimg = nullptr;
    if (want_normals && nout) {
        std::vector<u32> cap(n_inst);
        for (int i = 0; i < n_inst; ++i) cap[i] = out_w[i] * out_h[i];
        unsigned long long* d_nout_off = A.upload(out_off);
        u32* d_cap = A.upload(cap);
        d_nimg = A.zeros<float>(4 * nout);
        float amb = brightness(mk(cfg.ambient_color[0], cfg.ambient_color[1], cfg.ambient_color[2]));
        if (n_cov && d_ndir) {
            k_normals<<<(n_cov + kThreads - 1) / kThreads, kThreads, 0, st>>>(n_probe, n_samples, n_lights, d_ndir, d_snrm,
                                                                              d_sloc, d_sinst, d_nout_off, d_cap, amb, d_nimg); note_launch();
            CK(cudaGetLastError());
        } else if (n_cov) {
            float4* d_zero = A.zeros<float4>(1);
            k_normals<<<(n_cov + kThreads - 1) / kThreads, kThreads, 0, st>>>(n_probe, n_samples, 0, d_zero, d_snrm,
                                                                              d_sloc, d_sinst, d_nout_off, d_cap, amb, d_nimg); note_launch();
            CK(cudaGetLastError());
        }
    }
    uchar4* d_rgbe = nullptr;
    if (S->opt.encode_rgbe && nout) {
        d_rgbe = A.alloc<uchar4>(nout);
        k_encode_rgbe<<<blocks_for(nout), kThreads, 0, st>>>(nout, d_out, d_rgbe); note_launch();
        CK(cudaGetLastError());
    }
    TRACE("finalize issued");
    cudaEvent_t e_fin = clock.mark();

    // ---- readback
    u32 err_words[8] = {0};
    Counters cnt;
    CK(cudaMemcpyAsync(err_words, d_err, sizeof(err_words), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(err_words));
    CK(cudaMemcpyAsync(&cnt, d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(Counters));
    // Outputs land directly in the scene's page-locked buffer (kept across
    // bakes, freed with the scene); the work outputs point into it.
    const size_t out_floats = 3 * (size_t) nout + (d_nimg ? 4 * (size_t) nout : 0) + (d_rgbe ? (size_t) nout : 0);
    if (S->pinned_bytes < out_floats * sizeof(float)) {
        if (S->pinned) cudaFreeHost(S->pinned);
        S->pinned = nullptr;
        S->pinned_bytes = 0;
        CK(cudaHostAlloc(&S->pinned, std::max<size_t>(out_floats * sizeof(float), 1), cudaHostAllocDefault));
        S->pinned_bytes = out_floats * sizeof(float);
    }
    float* himg = (float*) S->pinned;
    float* hnimg = himg + 3 * (size_t) nout;
    if (nout) CK(cudaMemcpyAsync(himg, d_out, 3 * (size_t) nout * sizeof(float), cudaMemcpyDeviceToHost, st)); note_d2h(3 * (size_t) nout * sizeof(float));
    if (d_nimg) CK(cudaMemcpyAsync(hnimg, d_nimg, 4 * (size_t) nout * sizeof(float), cudaMemcpyDeviceToHost, st)); note_d2h(4 * (size_t) nout * sizeof(float));
    unsigned char* hrgbe = (unsigned char*) (hnimg + (d_nimg ? 4 * (size_t) nout : 0));
    if (d_rgbe) { CK(cudaMemcpyAsync(hrgbe, d_rgbe, 4 * (size_t) nout, cudaMemcpyDeviceToHost, st)); note_d2h(4 * (size_t) nout); }
    std::vector<float4> probe_lm(n_probe);
    if (n_probe) CK(cudaMemcpyAsync(probe_lm.data(), d_lm, n_probe * sizeof(float4), cudaMemcpyDeviceToHost, st)); note_d2h(n_probe * sizeof(float4));
    std::vector<float4> dpos, dnrm, drad, dlm;
    std::vector<u32> dloc;
    std::vector<float> dvis, dao;
    const int ao_ns = d_ao_hits ? cfg.ao_num_samples : 0;
    if (S->opt.keep_samples && n_samples) {
        if (d_vis) {
            dvis.resize((size_t) n_lights * n_samples);
            CK(cudaMemcpyAsync(dvis.data(), d_vis, dvis.size() * sizeof(float), cudaMemcpyDeviceToHost, st)); note_d2h(dvis.size() * sizeof(float));
        }
        if (d_ao_hits) {
            dao.resize((size_t) n_samples * ao_ns);
            CK(cudaMemcpyAsync(dao.data(), d_ao_hits, dao.size() * sizeof(float), cudaMemcpyDeviceToHost, st)); note_d2h(dao.size() * sizeof(float));
        }
        dpos.resize(n_samples); dnrm.resize(n_samples); drad.resize(n_samples); dlm.resize(n_samples); dloc.resize(n_samples);
        CK(cudaMemcpyAsync(dpos.data(), d_spos, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st)); note_d2h(n_samples * sizeof(float4));
        CK(cudaMemcpyAsync(dnrm.data(), d_snrm, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st)); note_d2h(n_samples * sizeof(float4));
        CK(cudaMemcpyAsync(drad.data(), d_srad, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st)); note_d2h(n_samples * sizeof(float4));
        CK(cudaMemcpyAsync(dlm.data(), d_lm, n_samples * sizeof(float4), cudaMemcpyDeviceToHost, st)); note_d2h(n_samples * sizeof(float4));
        CK(cudaMemcpyAsync(dloc.data(), d_sloc, n_samples * sizeof(u32), cudaMemcpyDeviceToHost, st)); note_d2h(n_samples * sizeof(u32));
    }
    cudaEvent_t e_down = clock.mark();
    CK(cudaStreamSynchronize(st));
    TRACE("readback done");
    // the host queues the whole bake and waits here; an ltr_Abort during that
    // wait stopped the trace kernels early, so their outputs are incomplete
    check_abort(S);
    static const char* kStageName[4] = {"sample fixup", "direct light", "radiosity", "ambient occlusion"};
    for (int k = 0; k < 4; ++k) {
        if (!err_words[k]) continue;
        char msg[160];
        snprintf(msg, sizeof(msg), "%s kernel reported error word 0x%08x (bit 0: traversal stack overflow; bit 1 (radiosity): a bounded wait for staged form factors expired)", kStageName[k], err_words[k]);
        throw std::runtime_error(msg);
    }

    // ---- outputs (scene-owned, lighter.cpp:1029-1042)
    for (u32 i = 0; i < n_probe; ++i) {
        S->samples[i].out_color[0] = probe_lm[i].x;
        S->samples[i].out_color[1] = probe_lm[i].y;
        S->samples[i].out_color[2] = probe_lm[i].z;
    }
    for (int i = 0; i < n_inst; ++i) {
        HostInst* mi = S->insts[i];
        if (mi->container) continue;
        float* img = himg + 3 * out_off[i];
        float* nimg = d_nimg ? hnimg + 4 * out_off[i] : nullptr;
        if (cfg.ds2x) { mi->w = out_w[i]; mi->h = out_h[i]; }
        ltr_WorkOutput wo = {(u32) i, mi->mesh->ident.c_str(), mi->mesh->ident.size(), mi->ident.c_str(),
                             mi->ident.size(), img, nimg, out_w[i], out_h[i]};
        S->outputs.push_back(wo);
        if (d_rgbe) S->outputs_rgbe.push_back(hrgbe + 4 * out_off[i]);
    }
    if (S->opt.keep_samples) {
        S->dump.assign(n_inst, SampleDump());
        for (int i = 0; i < n_inst && n_samples; ++i) {
            SampleDump& d = S->dump[i];
            for (u32 k = 0; k < scount[i]; ++k) {
                u32 s = sbeg[i] + k;
                d.pos.insert(d.pos.end(), {dpos[s].x, dpos[s].y, dpos[s].z});
                d.nrm.insert(d.nrm.end(), {dnrm[s].x, dnrm[s].y, dnrm[s].z});
                d.radinfo.insert(d.radinfo.end(), {drad[s].x, drad[s].y, drad[s].z, drad[s].w});
                d.color.insert(d.color.end(), {dlm[s].x, dlm[s].y, dlm[s].z});
                d.loc.push_back(dloc[s]);
            }
            d.n_lights = (u32) n_lights;
            d.ao_ns = (u32) ao_ns;
            d.vis.assign((size_t) n_lights * scount[i], -1.0f);
            if (!dvis.empty())
                for (int l = 0; l < n_lights; ++l)
                    for (u32 k = 0; k < scount[i]; ++k)
                        d.vis[(size_t) l * scount[i] + k] = dvis[(size_t) l * n_samples + sbeg[i] + k];
            if (!dao.empty())
                d.ao.assign(dao.begin() + (size_t) sbeg[i] * ao_ns, dao.begin() + (size_t) (sbeg[i] + scount[i]) * ao_ns);
        }
    }

    TRACE("outputs assembled");
    S->stats.ms_upload = StageClock::ms(e_up0, e_up1);
    S->stats.ms_bvh = StageClock::ms(bside.e0, bside.e1);
    S->stats.ms_samples = StageClock::ms(e_bvh, e_samples);
    S->stats.ms_direct = StageClock::ms(e_samples, e_direct);
    S->stats.ms_ao = StageClock::ms(e_ao0, e_ao1);
    S->stats.ms_direct_trace = e_dtr0 ? StageClock::ms(e_dtr0, e_dtr1) : 0.0;
    S->stats.ms_ao_trace = e_aotr0 ? StageClock::ms(e_aotr0, e_aotr1) : 0.0;
    S->stats.shadow_pairs = cnt.shadow_pairs;
    S->stats.ms_finalize = StageClock::ms(e_ao1, e_fin);
    S->stats.ms_download = StageClock::ms(e_fin, e_down);
    S->stats.shadow_evals = cnt.shadow_evals;
    S->stats.distance_queries = cnt.distance_queries;
    S->stats.ao_rays = cnt.ao_rays;
    S->stats.node_visits = cnt.node_visits;
    S->stats.tri_tests = cnt.tri_tests;
    S->stats.kernel_launches = host_counters().launches;
    S->stats.bytes_h2d = host_counters().h2d;
    S->stats.bytes_d2h = host_counters().d2h;
    S->stats.ms_device = StageClock::ms(e_dev0, e_fin);
    (void) e_rad_links;
    (void) e_rad_bounce;
}

}  // namespace lg
