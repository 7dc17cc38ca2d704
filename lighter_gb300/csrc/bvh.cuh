// Flat world-space BVH over the shadow-casting triangles of one scene, and the
// traversal routines the bake kernels use in place of the reference's
// two-level AABBTree/TriTree walks (lighter_int.hpp:742-814,
// lighter_math.cpp:804-1044, lighter.cpp:112-289).
//
// Layout in HBM (built by bvh.cu, LBVH with single-triangle leaves):
//   nodes : 4 x float4 per internal node (64 B, one 128-byte line pair):
//           n0 = (L.min.xyz, L.max.x)  n1 = (L.max.yz, R.min.xy)
//           n2 = (R.min.z, R.max.xyz)  n3 = (int L, int R, -, -)
//           child >= 0: internal node; child < 0: leaf holding triangle ~child.
//   tris  : 3 x float4 per leaf (triangle reference) in leaf order:
//           (P1.xyz, meta) (P2.xyz, local index) (P3.xyz, build index)
//           meta = instance index (bits 0-29) | occluder flag (bit 31).
// Child boxes are inflated by a few ulps at build time, so the slab and
// sphere tests below are conservative: they never drop a triangle the exact
// reference tests would accept. Results of the queries are therefore
// independent of the tree shape (any-hit, closest fraction, minimum distance).
#pragma once

#include <string>

#include "common.cuh"

namespace lg {

constexpr int kStack = 64;
constexpr u32 kOccluderBit = 0x80000000u;
constexpr u32 kInstMask = 0x3fffffffu;

struct BvhView {
    const float4* nodes;
    const float4* tris;
    int n_tris;      // 0: empty scene
    int root;        // >= 0 internal node, < 0 leaf (single triangle)
};

// Error word shared by all kernels of one bake: bit 0 stack overflow, bit 1
// candidate-list overflow, bit 2 index out of range.
struct ErrFlag { u32* word; };

#ifdef __CUDACC__

__device__ __forceinline__ void raise_err(ErrFlag e, u32 bit)
{
    if (e.word) atomicOr(e.word, bit);
}

__device__ __forceinline__ void load_tri(const BvhView& b, int t, V3& P1, V3& P2, V3& P3, u32& meta, u32& local)
{
    float4 a = __ldg(&b.tris[3 * t + 0]);
    float4 c = __ldg(&b.tris[3 * t + 1]);
    float4 d = __ldg(&b.tris[3 * t + 2]);
    P1 = mk(a.x, a.y, a.z); P2 = mk(c.x, c.y, c.z); P3 = mk(d.x, d.y, d.z);
    meta = __float_as_uint(a.w);
    local = __float_as_uint(c.w);
}

struct NodeBoxes { V3 lmin, lmax, rmin, rmax; int l, r; };

__device__ __forceinline__ NodeBoxes load_node(const BvhView& b, int n)
{
    const float4* p = b.nodes + 4 * n;
    float4 n0 = __ldg(p), n1 = __ldg(p + 1), n2 = __ldg(p + 2), n3 = __ldg(p + 3);
    NodeBoxes o;
    o.lmin = mk(n0.x, n0.y, n0.z); o.lmax = mk(n0.w, n1.x, n1.y);
    o.rmin = mk(n1.z, n1.w, n2.x); o.rmax = mk(n2.y, n2.z, n2.w);
    o.l = __float_as_int(n3.x); o.r = __float_as_int(n3.y);
    return o;
}

// Segment o + t*d, t in [0, tlimit], against a box; returns the entry t.
__device__ __forceinline__ bool slab(V3 mn, V3 mx, V3 o, V3 inv, float tlimit, float& tin)
{
    float tx0 = (mn.x - o.x) * inv.x, tx1 = (mx.x - o.x) * inv.x;
    float ty0 = (mn.y - o.y) * inv.y, ty1 = (mx.y - o.y) * inv.y;
    float tz0 = (mn.z - o.z) * inv.z, tz1 = (mx.z - o.z) * inv.z;
    float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tlimit));
    tin = t0;
    return t0 <= t1;
}

__device__ __forceinline__ V3 inv_dir(V3 d)
{
    return mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
}

// Squared distance from p to a box (0 inside).
__device__ __forceinline__ float box_d2(V3 mn, V3 mx, V3 p)
{
    float dx = fmaxf(fmaxf(mn.x - p.x, p.x - mx.x), 0.0f);
    float dy = fmaxf(fmaxf(mn.y - p.y, p.y - mx.y), 0.0f);
    float dz = fmaxf(fmaxf(mn.z - p.z, p.z - mx.z), 0.0f);
    return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ bool box_overlap(V3 mn, V3 mx, V3 qmn, V3 qmx)
{
    return !(qmn.x > mx.x || qmx.x < mn.x || qmn.y > mx.y || qmx.y < mn.y || qmn.z > mx.z || qmx.z < mn.z);
}

// Generic segment walk: visits leaves whose boxes the segment [o, e] enters
// before `tlimit` (updated by the leaf functor), nearer child first.
// Leaf functor: bool f(int tri, float& tlimit) -> false stops the walk.
template <class Leaf>
__device__ __forceinline__ void walk_segment(const BvhView& b, V3 o, V3 e, ErrFlag err, Leaf&& leaf)
{
    if (b.n_tris <= 0) return;
    V3 d = e - o;
    V3 inv = inv_dir(d);
    float tlimit = 1.0f;
    int stack[kStack];
    float stack_t[kStack];
    int sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            NodeBoxes nb = load_node(b, cur);
            float tl, tr;
            bool hl = slab(nb.lmin, nb.lmax, o, inv, tlimit, tl);
            bool hr = slab(nb.rmin, nb.rmax, o, inv, tlimit, tr);
            if (hl && hr) {
                bool lfirst = tl <= tr;
                if (sp < kStack) { stack[sp] = lfirst ? nb.r : nb.l; stack_t[sp] = lfirst ? tr : tl; ++sp; }
                else raise_err(err, 1u);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (hl) { cur = nb.l; continue; }
            if (hr) { cur = nb.r; continue; }
        } else {
            if (!leaf(~cur, tlimit)) return;
        }
        // pop, dropping subtrees whose entry lies beyond the (shrunken) limit
        for (;;) {
            if (sp == 0) return;
            --sp;
            if (stack_t[sp] <= tlimit) break;
        }
        cur = stack[sp];
    }
}

// Any occluder triangle hit with r < 1 on [o, e] (TriTree::IntersectRay,
// lighter_math.cpp:804-832, over every shadowing instance).
__device__ __forceinline__ bool bvh_any_hit(const BvhView& b, V3 o, V3 e, ErrFlag err)
{
    bool hit = false;
    walk_segment(b, o, e, err, [&](int t, float&) {
        V3 P1, P2, P3; u32 meta, local;
        load_tri(b, t, P1, P2, P3, meta, local);
        if (!(meta & kOccluderBit)) return true;
        if (seg_tri(o, e, P1, P2, P3) < 1.0f) { hit = true; return false; }
        return true;
    });
    return hit;
}

// Smallest hit fraction over occluders (TriTree::IntersectRayDist,
// lighter_math.cpp:835-871); *tri_out = leaf-order index of the hit triangle.
__device__ __forceinline__ float bvh_closest(const BvhView& b, V3 o, V3 e, ErrFlag err, int* tri_out)
{
    float best = kNoHit;
    int bt = -1;
    walk_segment(b, o, e, err, [&](int t, float& tlimit) {
        V3 P1, P2, P3; u32 meta, local;
        load_tri(b, t, P1, P2, P3, meta, local);
        if (!(meta & kOccluderBit)) return true;
        float r = seg_tri(o, e, P1, P2, P3);
        if (r < best || (r == best && r < kNoHit && t < bt)) {
            best = r; bt = t;
            tlimit = fminf(1.0f, r);
        }
        return true;
    });
    if (tri_out) *tri_out = bt;
    return best;
}

// Closest hit restricted to one instance's triangles, occluder or not
// (the per-instance tree of TriTree::OffsetSample, lighter_math.cpp:1024);
// *local_out = the triangle's index within its instance.
__device__ __forceinline__ float bvh_closest_inst(const BvhView& b, V3 o, V3 e, u32 inst, ErrFlag err, int* local_out)
{
    float best = kNoHit;
    int bl = -1;
    walk_segment(b, o, e, err, [&](int t, float& tlimit) {
        V3 P1, P2, P3; u32 meta, local;
        load_tri(b, t, P1, P2, P3, meta, local);
        if ((meta & kInstMask) != inst) return true;
        float r = seg_tri(o, e, P1, P2, P3);
        if (r < best || (r == best && r < kNoHit && (int) local < bl)) {
            best = r; bl = (int) local;
            tlimit = fminf(1.0f, r);
        }
        return true;
    });
    if (local_out) *local_out = bl;
    return best;
}

// Distance from p to the nearest occluder triangle, capped at d0
// (ltr_Scene::Distance + TriTree::GetDistance, lighter.cpp:150-188,
// lighter_math.cpp:954-989). The reference shrinks a query cube; a sphere
// test against the child boxes prunes the same triangles.
__device__ __forceinline__ float bvh_distance(const BvhView& b, V3 p, float d0, ErrFlag err, u32* visits = nullptr,
                                              u32* tests = nullptr)
{
    u32 nt = 0;
    float dist = d0;
    if (b.n_tris <= 0) return dist;
    int stack[kStack];
    float stack_d[kStack];
    int sp = 0;
    int cur = b.root;
    u32 nv = 0;
    for (;;) {
        if (cur >= 0) {
            NodeBoxes nb = load_node(b, cur);
            ++nv;
            float dl = box_d2(nb.lmin, nb.lmax, p);
            float dr = box_d2(nb.rmin, nb.rmax, p);
            float lim = dist * dist;
            bool hl = dl <= lim, hr = dr <= lim;
            if (hl && hr) {
                bool lfirst = dl <= dr;
                if (sp < kStack) { stack[sp] = lfirst ? nb.r : nb.l; stack_d[sp] = lfirst ? dr : dl; ++sp; }
                else raise_err(err, 1u);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (hl) { cur = nb.l; continue; }
            if (hr) { cur = nb.r; continue; }
        } else {
            V3 P1, P2, P3; u32 meta, local;
            load_tri(b, ~cur, P1, P2, P3, meta, local);
            if (meta & kOccluderBit) {
                float nd = point_tri_dist(p, P1, P2, P3);
                ++nt;
                if (nd < dist) dist = nd;
            }
        }
        bool done = false;
        for (;;) {
            if (sp == 0) { done = true; break; }
            --sp;
            if (stack_d[sp] <= dist * dist) break;
        }
        if (done) break;
        cur = stack[sp];
    }
    if (visits) *visits += nv;
    if (tests) *tests += nt;
    return dist;
}

// Among the triangles of instance `inst` whose boxes overlap [qmn, qmx]
// (AABBTree::Query over one instance, lighter_int.hpp:786-806), the one with
// the smallest instance-local index greater than `after`. Repeated calls
// visit the overlapping triangles in the instance's own order without a
// candidate buffer. Returns the leaf-order index or -1.
__device__ __forceinline__ int bvh_next_inst(const BvhView& b, V3 qmn, V3 qmx, u32 inst, int after, int* local_out,
                                             ErrFlag err)
{
    if (b.n_tris <= 0) return -1;
    int best_t = -1;
    u32 best_l = 0xffffffffu;
    int stack[kStack];
    int sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            NodeBoxes nb = load_node(b, cur);
            bool hl = box_overlap(nb.lmin, nb.lmax, qmn, qmx);
            bool hr = box_overlap(nb.rmin, nb.rmax, qmn, qmx);
            if (hl && hr) {
                if (sp < kStack) stack[sp++] = nb.r; else raise_err(err, 1u);
                cur = nb.l;
                continue;
            }
            if (hl) { cur = nb.l; continue; }
            if (hr) { cur = nb.r; continue; }
        } else {
            int t = ~cur;
            u32 meta = __float_as_uint(__ldg(&b.tris[3 * t]).w);
            if ((meta & kInstMask) == inst) {
                u32 l = __float_as_uint(__ldg(&b.tris[3 * t + 1]).w);
                if ((int) l > after && l < best_l) { best_l = l; best_t = t; }
            }
        }
        if (sp == 0) break;
        cur = stack[--sp];
    }
    *local_out = (int) best_l;
    return best_t;
}

#endif  // __CUDACC__

// Host side of the build (bvh.cu).
struct BvhBuildInput {
    const float* tri_xyz;   // device: 9 floats per triangle (P1, P2, P3)
    const u32* tri_meta;    // device: instance | occluder bit
    const u32* tri_local;   // device: index within its instance
    const u32* ref_tri;     // device: triangle of each leaf reference
    const float* ref_box;   // device: exact box of each reference (min xyz, max xyz)
    int n;                  // number of references (leaves)
    float scene_min[3], scene_max[3];   // bounds of the reference box centres
};

struct BvhStorage {
    float4* nodes = nullptr;   // 4 per internal node
    float4* tris = nullptr;    // 3 per triangle
    int n_tris = 0;
    int root = 0;
    size_t bytes = 0;
    void* scratch = nullptr;   // build scratch, freed by bvh_free
    BvhView view() const { BvhView v = {nodes, tris, n_tris, root}; return v; }
};

// Builds into `out` on `stream` (allocations with cudaMallocAsync on that stream).
void bvh_build(const BvhBuildInput& in, BvhStorage& out, void* stream);
void bvh_free(BvhStorage& s, void* stream);
std::string bvh_validate(const BvhStorage& s, void* stream);

}  // namespace lg
