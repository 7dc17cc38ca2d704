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
#include <vector>

#include "common.cuh"

namespace lg {

constexpr int kStack = 64;
constexpr int kNoChild = (int) 0x80000000;   // empty slot of a 4-wide node
constexpr u32 kOccluderBit = 0x80000000u;
constexpr u32 kInstMask = 0x3fffffffu;

struct BvhView {
    const float4* nodes;
    const float4* tris;
    const float4* srec;   // 4 per leaf: segment-test record (see below)
    const float4* drec;   // 8 per leaf: distance-test record (see below)
    int n_tris;      // number of leaves; 0: empty scene
    int root;        // >= 0 internal node, < 0 leaf (single triangle)
    const float4* nodes4;   // 4-wide nodes (see below)
    int root4;              // >= 0 4-wide node, < 0 leaf
    int watertight;         // segment queries use seg_tri_wt instead of the reference's test
    float dist_margin = INFINITY;   // warp_distance: bound on how far the exact point/triangle test can
                            // fall below the triangle's plane distance by rounding (infinite: the
                            // plane test that skips hopeless leaves is off)
};

// 4-wide nodes, used by the any-hit walk: the binary nodes at even depth with
// their grandchildren as children (2-4 per node), 8 float4 = 128 B:
//   (min.x of children 0-3) (max.x) (min.y) (max.y) (min.z) (max.z)
//   (child 0-3 as int bits: >= 0 4-wide node, < 0 leaf ~t, kNoChild empty) (-)
// Child boxes are the binary tree's inflated boxes.

// Per-leaf records with the triangle-only terms of the two exact tests,
// computed once per bake with the reference's own expressions (so a test
// that reads them rounds exactly like one that recomputes them):
//   srec: (P1, meta) (u = P2-P1, uu) (v = P3-P1, uv) (n = u x v, vv)
//   drec: (nrm, nrm.t0) (tan0, tan0.t0) (tan1, tan1.t1) (tan2, tan2.t2)
//         (tan0.t1, tan1.t2, tan2.t0, meta) (en0, en0.t0) (en1, en1.t1) (en2, en2.t2)
// with nrm = |(t1-t0) x (t2-t0)|, tan0..2 the unit edges and en0..2 the unit
// edge normals of PointTriangleDistance (lighter_math.cpp:875-913).

// Error word shared by all kernels of one bake: bit 0 stack overflow, bit 1
// candidate-list overflow, bit 2 index out of range.
struct ErrFlag { u32* word; };

#ifdef __CUDACC__

__device__ __forceinline__ void raise_err(ErrFlag e, u32 bit)
{
    if (e.word) atomicOr(e.word, bit);
}

// Traversal stack of one thread: entries (node, entry key) with the first K
// in shared memory -- this thread's column of a K x blockDim array, so the 32
// lanes of a warp hit 32 different banks -- and deeper entries in local
// memory. K = 0 keeps the whole stack in local memory. The walks push only
// when both children qualify, so most walks stay within a few entries; which
// K is fastest is a per-device tuning choice (ltrg_Tuning.direct_stack /
// ao_stack). A push past kStack entries records error bit 0 and drops the entry.
template <int K>
struct TStack {
    int* sn;
    float* sk;
    int stride;
    int sp = 0;
    int ln[kStack - K];
    float lk[kStack - K];
    __device__ __forceinline__ TStack(int* s_n, float* s_k, int st) : sn(s_n), sk(s_k), stride(st) {}
    __device__ __forceinline__ void push(int n, float k, ErrFlag err)
    {
        if (sp < K) { sn[sp * stride] = n; sk[sp * stride] = k; }
        else if (sp < kStack) { ln[sp - K] = n; lk[sp - K] = k; }
        else { raise_err(err, 1u); return; }
        ++sp;
    }
    __device__ __forceinline__ void pop(int& n, float& k)
    {
        --sp;
        if (sp < K) { n = sn[sp * stride]; k = sk[sp * stride]; }
        else { n = ln[sp - K]; k = lk[sp - K]; }
    }
};

template <>
struct TStack<0> {
    int sp = 0;
    int ln[kStack];
    float lk[kStack];
    __device__ __forceinline__ TStack() {}
    __device__ __forceinline__ TStack(int*, float*, int) {}
    __device__ __forceinline__ void push(int n, float k, ErrFlag err)
    {
        if (sp < kStack) { ln[sp] = n; lk[sp] = k; ++sp; }
        else raise_err(err, 1u);
    }
    __device__ __forceinline__ void pop(int& n, float& k) { --sp; n = ln[sp]; k = lk[sp]; }
};

// This thread's short stack over the block's dynamic shared memory (K x
// blockDim node ids, then K x blockDim keys: K x blockDim x 8 bytes).
template <int K>
__device__ __forceinline__ TStack<K> make_stack(unsigned char* smem)
{
    int* sn = reinterpret_cast<int*>(smem) + threadIdx.x;
    float* sk = reinterpret_cast<float*>(smem + (size_t) K * blockDim.x * sizeof(int)) + threadIdx.x;
    return TStack<K>(sn, sk, (int) blockDim.x);
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
// `oinv` = o * inv, so each plane costs one FMA; the boxes are inflated, so
// the FMA's different rounding cannot drop a triangle the exact test keeps.
__device__ __forceinline__ bool slab(V3 mn, V3 mx, V3 oinv, V3 inv, float tlimit, float& tin)
{
    float tx0 = __fmaf_rn(mn.x, inv.x, -oinv.x), tx1 = __fmaf_rn(mx.x, inv.x, -oinv.x);
    float ty0 = __fmaf_rn(mn.y, inv.y, -oinv.y), ty1 = __fmaf_rn(mx.y, inv.y, -oinv.y);
    float tz0 = __fmaf_rn(mn.z, inv.z, -oinv.z), tz1 = __fmaf_rn(mx.z, inv.z, -oinv.z);
    float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tlimit));
    tin = t0;
    return t0 <= t1;
}

// 1/d with zero components replaced by +-1e-30 (finite, no NaN in the slab).
__device__ __forceinline__ V3 inv_dir(V3 d)
{
    const float tiny = 1e-30f;
    float x = fabsf(d.x) < tiny ? copysignf(tiny, d.x) : d.x;
    float y = fabsf(d.y) < tiny ? copysignf(tiny, d.y) : d.y;
    float z = fabsf(d.z) < tiny ? copysignf(tiny, d.z) : d.z;
    return mk(1.0f / x, 1.0f / y, 1.0f / z);
}

// Squared distance from p to a box (0 inside).
__device__ __forceinline__ float box_d2(V3 mn, V3 mx, V3 p)
{
    float dx = fmaxf(fmaxf(mn.x - p.x, p.x - mx.x), 0.0f);
    float dy = fmaxf(fmaxf(mn.y - p.y, p.y - mx.y), 0.0f);
    float dz = fmaxf(fmaxf(mn.z - p.z, p.z - mx.z), 0.0f);
    // a pruning bound only (never a result): fused multiply-adds are within an ulp
    // of the separate products, far inside the boxes' inflation
    return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
}

__device__ __forceinline__ bool box_overlap(V3 mn, V3 mx, V3 qmn, V3 qmx)
{
    return !(qmn.x > mx.x || qmx.x < mn.x || qmn.y > mx.y || qmx.y < mn.y || qmn.z > mx.z || qmx.z < mn.z);
}

struct Node4 {
    float4 x0, x1, y0, y1, z0, z1;
    int c[4];
};

__device__ __forceinline__ Node4 load_node4(const BvhView& b, int n)
{
    const float4* p = b.nodes4 + 8 * (size_t) n;
    Node4 o;
    o.x0 = __ldg(p); o.x1 = __ldg(p + 1); o.y0 = __ldg(p + 2); o.y1 = __ldg(p + 3); o.z0 = __ldg(p + 4); o.z1 = __ldg(p + 5);
    float4 cc = __ldg(p + 6);
    o.c[0] = __float_as_int(cc.x); o.c[1] = __float_as_int(cc.y); o.c[2] = __float_as_int(cc.z); o.c[3] = __float_as_int(cc.w);
    return o;
}

__device__ __forceinline__ float f4k(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }

// Four (key, child) pairs, absent ones with key +inf, put in ascending key order
// by a five-comparator network on registers.
struct Near4 {
    float k0 = INFINITY, k1 = INFINITY, k2 = INFINITY, k3 = INFINITY;
    int c0 = -1, c1 = -1, c2 = -1, c3 = -1;
    __device__ __forceinline__ void set(int slot, float k, int c)
    {
        if (slot == 0) { k0 = k; c0 = c; } else if (slot == 1) { k1 = k; c1 = c; }
        else if (slot == 2) { k2 = k; c2 = c; } else { k3 = k; c3 = c; }
    }
    __device__ __forceinline__ static void cs(float& ka, int& ca, float& kb, int& cb)
    {
        if (kb < ka) { float t = ka; ka = kb; kb = t; int u = ca; ca = cb; cb = u; }
    }
    __device__ __forceinline__ void sort()
    {
        cs(k0, c0, k1, c1); cs(k2, c2, k3, c3); cs(k0, c0, k2, c2); cs(k1, c1, k3, c3); cs(k1, c1, k2, c2);
    }
};

// walk_segment over the 4-wide nodes: at a node the leaf children are tested
// at once, then the internal ones are visited nearest entry first. Half the
// depth of the binary walk pays for long any-hit segments in big trees (the
// form factors' visibility rays on the 1.2M-triangle terrain: 115 -> 28 ms),
// not in small ones (the 67k-triangle room of the gather: 64 -> 76 ms); the
// short AO rays and the sphere-trace queries are faster on the binary nodes,
// whose two-box tests prune more tightly.
template <class Stack, class Leaf>
__device__ __forceinline__ void walk_segment4(const BvhView& b, V3 o, V3 e, ErrFlag err, Stack& st, Leaf&& leaf)
{
    st.sp = 0;
    if (b.n_tris <= 0) return;
    V3 d = e - o;
    V3 inv = inv_dir(d);
    V3 oinv = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    float tlimit = 1.0f;
    if (b.root4 < 0) { leaf(~b.root4, tlimit); return; }
    int cur = b.root4;
    for (;;) {
        const Node4 nd = load_node4(b, cur);
        Near4 near;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = nd.c[k];
            if (c == kNoChild) continue;
            float tin;
            if (!slab(mk(f4k(nd.x0, k), f4k(nd.y0, k), f4k(nd.z0, k)), mk(f4k(nd.x1, k), f4k(nd.y1, k), f4k(nd.z1, k)), oinv,
                      inv, tlimit, tin))
                continue;
            if (c < 0) {
                if (!leaf(~c, tlimit)) return;
            } else {
                near.set(k, tin, c);
            }
        }
        // visit the nearest internal child now, the others later (farthest pushed first);
        // the leaf tests may have shrunk the limit
        near.sort();
        if (near.k3 <= tlimit) st.push(near.c3, near.k3, err);
        if (near.k2 <= tlimit) st.push(near.c2, near.k2, err);
        if (near.k1 <= tlimit) st.push(near.c1, near.k1, err);
        if (near.k0 <= tlimit) { cur = near.c0; continue; }
        // pop, dropping subtrees whose entry lies beyond the (shrunken) limit
        for (;;) {
            if (st.sp == 0) return;
            float k;
            st.pop(cur, k);
            if (k <= tlimit) break;
        }
    }
}

// Generic segment walk: visits leaves whose boxes the segment [o, e] enters
// before `tlimit` (updated by the leaf functor), nearer child first.
// Leaf functor: bool f(int tri, float& tlimit) -> false stops the walk.
template <class Stack, class Leaf>
__device__ __forceinline__ void walk_segment(const BvhView& b, V3 o, V3 e, ErrFlag err, Stack& st, Leaf&& leaf)
{
    if (b.n_tris <= 0) return;
    V3 d = e - o;
    V3 inv = inv_dir(d);
    V3 oinv = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    float tlimit = 1.0f;
    st.sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            NodeBoxes nb = load_node(b, cur);
            float tl, tr;
            bool hl = slab(nb.lmin, nb.lmax, oinv, inv, tlimit, tl);
            bool hr = slab(nb.rmin, nb.rmax, oinv, inv, tlimit, tr);
            if (hl && hr) {
                bool lfirst = tl <= tr;
                st.push(lfirst ? nb.r : nb.l, lfirst ? tr : tl, err);
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
            if (st.sp == 0) return;
            float k;
            st.pop(cur, k);
            if (k <= tlimit) break;
        }
    }
}

// IntersectLineSegmentTriangle (lighter_math.cpp:315-354) with the
// triangle-only terms read from the leaf's record.
__device__ __forceinline__ float seg_tri_rec(V3 L1, V3 L2, const float4* r, u32& meta)
{
    float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
    meta = __float_as_uint(r0.w);
    V3 P1 = mk(r0.x, r0.y, r0.z), u = mk(r1.x, r1.y, r1.z), v = mk(r2.x, r2.y, r2.z), n = mk(r3.x, r3.y, r3.z);
    float uu = r1.w, uv = r2.w, vv = r3.w;
    if (near_zero(n)) return kNoHit;
    V3 dir = L2 - L1, w0 = L1 - P1;
    float a = -dot(n, w0);
    float b = dot(n, dir);
    if (fabsf(b) < kSmall) return kNoHit;
    float rr = a / b;
    if (rr < 0.0f || rr > 1.0f) return kNoHit;
    V3 I = L1 + rr * dir;
    V3 w = I - P1;
    float wu = dot(w, u), wv = dot(w, v);
    float D = uv * uv - uu * vv;
    float s = (uv * wv - vv * wu) / D;
    if (s < 0.0f || s > 1.0f) return kNoHit;
    float t = (uv * wu - uu * wv) / D;
    if (t < 0.0f || (s + t) > 1.0f) return kNoHit;
    return rr;
}

// PointTriangleDistance (lighter_math.cpp:875-913) with the triangle-only
// terms read from the leaf's record; the vertices are read only for the
// corner regions.
__device__ __forceinline__ float point_tri_dist_rec(const BvhView& b, int t, V3 pt)
{
    const float4* r = b.drec + 8 * (size_t) t;
    float4 f0 = __ldg(r), f1 = __ldg(r + 1), f2 = __ldg(r + 2), f3 = __ldg(r + 3), f4 = __ldg(r + 4);
    V3 nrm = mk(f0.x, f0.y, f0.z);
    float pd = fabsf(dot(nrm, pt) - f0.w);
    float t0p = dot(mk(f1.x, f1.y, f1.z), pt), t0min = f1.w, t0max = f4.x;
    float t1p = dot(mk(f2.x, f2.y, f2.z), pt), t1min = f2.w, t1max = f4.y;
    float t2p = dot(mk(f3.x, f3.y, f3.z), pt), t2min = f3.w, t2max = f4.z;
    if (t0min >= t0p && t2max <= t2p) { float4 v = __ldg(&b.tris[3 * (size_t) t]); return len(pt - mk(v.x, v.y, v.z)); }
    if (t1min >= t1p && t0max <= t0p) { float4 v = __ldg(&b.tris[3 * (size_t) t + 1]); return len(pt - mk(v.x, v.y, v.z)); }
    if (t2min >= t2p && t1max <= t1p) { float4 v = __ldg(&b.tris[3 * (size_t) t + 2]); return len(pt - mk(v.x, v.y, v.z)); }
    float4 f5 = __ldg(r + 5), f6 = __ldg(r + 6), f7 = __ldg(r + 7);
    float d0 = dot(mk(f5.x, f5.y, f5.z), pt) - f5.w;
    float d1 = dot(mk(f6.x, f6.y, f6.z), pt) - f6.w;
    float d2 = dot(mk(f7.x, f7.y, f7.z), pt) - f7.w;
    if (d0 >= 0 && t0p >= t0min && t0p <= t0max) return len2(mk2(pd, d0));
    if (d1 >= 0 && t1p >= t1min && t1p <= t1max) return len2(mk2(pd, d1));
    if (d2 >= 0 && t2p >= t2min && t2p <= t2max) return len2(mk2(pd, d2));
    return pd;
}

// Segment test of leaf t: the reference's (from the leaf's record) or the
// watertight one (from the leaf's vertices), per the view's mode.
__device__ __forceinline__ float seg_leaf(const BvhView& b, V3 o, V3 e, int t, u32& meta)
{
    if (b.watertight) {
        const float4 a = __ldg(&b.tris[3 * (size_t) t]), c = __ldg(&b.tris[3 * (size_t) t + 1]),
                     d = __ldg(&b.tris[3 * (size_t) t + 2]);
        meta = __float_as_uint(a.w);
        return seg_tri_wt(o, e, mk(a.x, a.y, a.z), mk(c.x, c.y, c.z), mk(d.x, d.y, d.z));
    }
    return seg_tri_rec(o, e, b.srec + 4 * (size_t) t, meta);
}

// Any occluder triangle hit with r < 1 on [o, e] (TriTree::IntersectRay,
// lighter_math.cpp:804-832, over every shadowing instance).
template <bool kWide, class Stack>
__device__ __forceinline__ bool bvh_any_hit_s(const BvhView& b, V3 o, V3 e, ErrFlag err, Stack& st)
{
    bool hit = false;
    auto leaf = [&](int t, float&) {
        u32 meta;
        float r = seg_leaf(b, o, e, t, meta);
        if (!(meta & kOccluderBit)) return true;
        if (r < 1.0f) { hit = true; return false; }
        return true;
    };
    if (kWide) walk_segment4(b, o, e, err, st, leaf);
    else walk_segment(b, o, e, err, st, leaf);
    return hit;
}

template <bool kWide = false>
__device__ __forceinline__ bool bvh_any_hit(const BvhView& b, V3 o, V3 e, ErrFlag err)
{
    TStack<0> st;
    return bvh_any_hit_s<kWide>(b, o, e, err, st);
}

// Smallest hit fraction over occluders (TriTree::IntersectRayDist,
// lighter_math.cpp:835-871); *tri_out = leaf-order index of the hit triangle.
template <class Stack>
__device__ __forceinline__ float bvh_closest_s(const BvhView& b, V3 o, V3 e, ErrFlag err, int* tri_out, Stack& st)
{
    float best = kNoHit;
    int bt = -1;
    walk_segment(b, o, e, err, st, [&](int t, float& tlimit) {
        u32 meta;
        float r = seg_leaf(b, o, e, t, meta);
        if (!(meta & kOccluderBit)) return true;
        if (r < best || (r == best && r < kNoHit && t < bt)) {
            best = r; bt = t;
            tlimit = fminf(1.0f, r);
        }
        return true;
    });
    if (tri_out) *tri_out = bt;
    return best;
}

__device__ __forceinline__ float bvh_closest(const BvhView& b, V3 o, V3 e, ErrFlag err, int* tri_out)
{
    TStack<0> st;
    return bvh_closest_s(b, o, e, err, tri_out, st);
}

// Distance from p to the nearest occluder triangle, capped at d0
// (ltr_Scene::Distance + TriTree::GetDistance, lighter.cpp:150-188,
// lighter_math.cpp:954-989). The reference shrinks a query cube; a sphere
// test against the child boxes prunes the same triangles.
template <class Stack>
__device__ __forceinline__ float bvh_distance_s(const BvhView& b, V3 p, float d0, ErrFlag err, Stack& st,
                                                u32* visits = nullptr, u32* tests = nullptr, int* best_leaf = nullptr)
{
    u32 nt = 0;
    float dist = d0;
    if (b.n_tris <= 0) return dist;
    st.sp = 0;
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
                st.push(lfirst ? nb.r : nb.l, lfirst ? dr : dl, err);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (hl) { cur = nb.l; continue; }
            if (hr) { cur = nb.r; continue; }
        } else {
            int t = ~cur;
            u32 meta = __float_as_uint(__ldg(&b.drec[8 * (size_t) t + 4]).w);
            if (meta & kOccluderBit) {
                float nd = point_tri_dist_rec(b, t, p);
                ++nt;
                if (nd < dist) {
                    dist = nd;
                    if (best_leaf) *best_leaf = t;
                }
            }
        }
        bool done = false;
        for (;;) {
            if (st.sp == 0) { done = true; break; }
            float k;
            st.pop(cur, k);
            if (k <= dist * dist) break;
        }
        if (done) break;
    }
    if (visits) *visits += nv;
    if (tests) *tests += nt;
    return dist;
}

__device__ __forceinline__ float bvh_distance(const BvhView& b, V3 p, float d0, ErrFlag err, u32* visits = nullptr,
                                              u32* tests = nullptr, int* best_leaf = nullptr)
{
    TStack<0> st;
    return bvh_distance_s(b, p, d0, err, st, visits, tests, best_leaf);
}

// ---- warp-cooperative queries. The 32 lanes of a warp walk the binary BVH
// together: a child is entered when the query of any lane still running
// reaches its box, node loads are broadcasts, and every lane runs each leaf
// test of the walk against its own query. The walk visits a superset of the
// nodes each lane's own walk would visit, and a subtree is dropped only when,
// for every lane, it lies beyond that lane's current limit, so every lane gets
// exactly the result of the per-lane query. The stack is warp-uniform and
// lives in registers spread over the lanes (entry i in lane i % 32, slot
// i / 32; 64 entries, more than the tree's depth). Every lane of the warp
// must call these (converged).

// Pushes `n` on the warp's stack (or records error bit 0 past 64 entries).
__device__ __forceinline__ void wstack_push(int& s0, int& s1, int& sp, int n, ErrFlag err)
{
    const int lane = threadIdx.x & 31;
    if (sp < 64) {
        if (lane == (sp & 31)) { if (sp < 32) s0 = n; else s1 = n; }
        ++sp;
    } else if (lane == 0) {
        raise_err(err, 1u);
    }
}

__device__ __forceinline__ int wstack_pop(int s0, int s1, int& sp)
{
    --sp;
    return __shfl_sync(0xffffffffu, sp < 32 ? s0 : s1, sp & 31);
}

// The child a warp enters first when the lanes reach both: the one more of
// those lanes find nearer.
__device__ __forceinline__ bool warp_left_first(bool hl, bool hr, bool lnear)
{
    const unsigned both = __ballot_sync(0xffffffffu, hl && hr);
    const unsigned ln = __ballot_sync(0xffffffffu, hl && hr && lnear);
    return 2 * __popc(ln) >= __popc(both);
}

// bvh_distance for the active lanes: min(d0, min over occluder triangles of
// the exact point-triangle distance), each lane with its own point and radius.
__device__ __forceinline__ float warp_distance(const BvhView& b, V3 p, float d0, bool active, ErrFlag err, u32& nv,
                                               u32& nt)
{
    float dist = d0;
    const unsigned am = __ballot_sync(0xffffffffu, active);
    if (b.n_tris <= 0 || !am) return dist;
    // the walk's node and leaf fetches are counted once for the warp, by its lowest active lane
    const bool counter = (int) (threadIdx.x & 31) == __ffs(am) - 1;
    int s0 = 0, s1 = 0, sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            const NodeBoxes nb = load_node(b, cur);
            if (counter) ++nv;
            const float lim = dist * dist;
            const float dl = box_d2(nb.lmin, nb.lmax, p), dr = box_d2(nb.rmin, nb.rmax, p);
            const bool hl = active && dl <= lim, hr = active && dr <= lim;
            const unsigned ml = __ballot_sync(0xffffffffu, hl), mr = __ballot_sync(0xffffffffu, hr);
            if (ml && mr) {
                const bool lfirst = warp_left_first(hl, hr, dl <= dr);
                wstack_push(s0, s1, sp, lfirst ? nb.r : nb.l, err);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (ml) { cur = nb.l; continue; }
            if (mr) { cur = nb.r; continue; }
        } else {
            const int t = ~cur;
            const float4* r = b.drec + 8 * (size_t) t;
            const u32 meta = __float_as_uint(__ldg(r + 4).w);
            if (meta & kOccluderBit) {
                // The exact test returns the plane distance pd or more (less rounding,
                // at most dist_margin), so a lane whose limit is below pd - margin
                // cannot take a smaller distance from this triangle; the warp runs the
                // test only if some lane can (then for every lane, as before).
                const float4 f0 = __ldg(r);
                // a skip test only: fused multiply-adds move pd by far less than the margin
                const float pd = fabsf(__fmaf_rn(f0.x, p.x, __fmaf_rn(f0.y, p.y, __fmaf_rn(f0.z, p.z, -f0.w))));
                const bool may = active && !(pd > dist + b.dist_margin);
                if (__any_sync(0xffffffffu, may)) {
                    if (counter) ++nt;
                    if (active) {
                        const float nd = point_tri_dist_rec(b, t, p);
                        if (nd < dist) dist = nd;
                    }
                }
            }
        }
        if (sp == 0) break;
        cur = wstack_pop(s0, s1, sp);
    }
    return dist;
}

// bvh_any_hit for the active lanes' segments: a lane stops searching at its
// first occluder hit (r < 1); the walk ends when no lane searches any more.
__device__ __forceinline__ bool warp_any_hit(const BvhView& b, V3 o, V3 e, bool active, ErrFlag err)
{
    bool hit = false;
    bool searching = active && b.n_tris > 0;
    if (!__any_sync(0xffffffffu, searching)) return false;
    const V3 d = e - o;
    const V3 inv = inv_dir(d);
    const V3 oinv = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    int s0 = 0, s1 = 0, sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            const NodeBoxes nb = load_node(b, cur);
            float tl, tr;
            const bool hl = searching && slab(nb.lmin, nb.lmax, oinv, inv, 1.0f, tl);
            const bool hr = searching && slab(nb.rmin, nb.rmax, oinv, inv, 1.0f, tr);
            const unsigned ml = __ballot_sync(0xffffffffu, hl), mr = __ballot_sync(0xffffffffu, hr);
            if (ml && mr) {
                const bool lfirst = warp_left_first(hl, hr, tl <= tr);
                wstack_push(s0, s1, sp, lfirst ? nb.r : nb.l, err);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (ml) { cur = nb.l; continue; }
            if (mr) { cur = nb.r; continue; }
        } else if (searching) {
            u32 meta;
            const float r = seg_leaf(b, o, e, ~cur, meta);
            if ((meta & kOccluderBit) && r < 1.0f) { hit = true; searching = false; }
        }
        if (sp == 0 || !__any_sync(0xffffffffu, searching)) break;
        cur = wstack_pop(s0, s1, sp);
    }
    return hit;
}

// bvh_closest for the active lanes' segments (the smallest occluder hit
// fraction, ties to the lower leaf -- a rule that does not depend on the
// visiting order), each lane shrinking its own limit.
__device__ __forceinline__ float warp_closest(const BvhView& b, V3 o, V3 e, bool active, ErrFlag err)
{
    float best = kNoHit;
    int bt = -1;
    if (b.n_tris <= 0 || !__any_sync(0xffffffffu, active)) return best;
    const V3 d = e - o;
    const V3 inv = inv_dir(d);
    const V3 oinv = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    float tlimit = 1.0f;
    int s0 = 0, s1 = 0, sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            const NodeBoxes nb = load_node(b, cur);
            float tl, tr;
            const bool hl = active && slab(nb.lmin, nb.lmax, oinv, inv, tlimit, tl);
            const bool hr = active && slab(nb.rmin, nb.rmax, oinv, inv, tlimit, tr);
            const unsigned ml = __ballot_sync(0xffffffffu, hl), mr = __ballot_sync(0xffffffffu, hr);
            if (ml && mr) {
                const bool lfirst = warp_left_first(hl, hr, tl <= tr);
                wstack_push(s0, s1, sp, lfirst ? nb.r : nb.l, err);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (ml) { cur = nb.l; continue; }
            if (mr) { cur = nb.r; continue; }
        } else if (active) {
            const int t = ~cur;
            u32 meta;
            const float r = seg_leaf(b, o, e, t, meta);
            if ((meta & kOccluderBit) && (r < best || (r == best && r < kNoHit && t < bt))) {
                best = r;
                bt = t;
                tlimit = fminf(1.0f, r);
            }
        }
        if (sp == 0) break;
        cur = wstack_pop(s0, s1, sp);
    }
    return best;
}

// Closest hit restricted to one instance's triangles, occluder or not (the
// per-instance tree query of TriTree::OffsetSample, lighter_math.cpp:1024),
// for the active lanes' segments: the smallest hit fraction, ties to the lower
// instance-local index (a rule that does not depend on the visiting order);
// *local_out gets the lane's triangle within its instance (or -1).
__device__ __forceinline__ float warp_closest_inst(const BvhView& b, V3 o, V3 e, u32 inst, bool active, ErrFlag err,
                                                   int* local_out)
{
    float best = kNoHit;
    int bl = -1;
    if (b.n_tris <= 0 || !__any_sync(0xffffffffu, active)) {
        *local_out = bl;
        return best;
    }
    const V3 d = e - o;
    const V3 inv = inv_dir(d);
    const V3 oinv = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    float tlimit = 1.0f;
    int s0 = 0, s1 = 0, sp = 0;
    int cur = b.root;
    for (;;) {
        if (cur >= 0) {
            const NodeBoxes nb = load_node(b, cur);
            float tl, tr;
            const bool hl = active && slab(nb.lmin, nb.lmax, oinv, inv, tlimit, tl);
            const bool hr = active && slab(nb.rmin, nb.rmax, oinv, inv, tlimit, tr);
            const unsigned ml = __ballot_sync(0xffffffffu, hl), mr = __ballot_sync(0xffffffffu, hr);
            if (ml && mr) {
                const bool lfirst = warp_left_first(hl, hr, tl <= tr);
                wstack_push(s0, s1, sp, lfirst ? nb.r : nb.l, err);
                cur = lfirst ? nb.l : nb.r;
                continue;
            }
            if (ml) { cur = nb.l; continue; }
            if (mr) { cur = nb.r; continue; }
        } else if (active) {
            const int t = ~cur;
            u32 meta;
            const float r = seg_leaf(b, o, e, t, meta);
            if ((meta & kInstMask) == inst) {
                const int local = (int) __float_as_uint(__ldg(&b.tris[3 * (size_t) t + 1]).w);
                if (r < best || (r == best && r < kNoHit && local < bl)) {
                    best = r;
                    bl = local;
                    tlimit = fminf(1.0f, r);
                }
            }
        }
        if (sp == 0) break;
        cur = wstack_pop(s0, s1, sp);
    }
    *local_out = bl;
    return best;
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
    int builder = 0;        // 0: locally-ordered clustering (PLOC), 1: Karras' radix hierarchy
};

struct BvhStorage {
    float4* nodes = nullptr;   // 4 per internal node
    float4* tris = nullptr;    // 3 per leaf
    float4* srec = nullptr;    // 4 per leaf
    float4* drec = nullptr;    // 8 per leaf
    float4* nodes4 = nullptr;  // 8 per 4-wide node
    int n_tris = 0;
    int root = 0;
    int root4 = 0;
    size_t bytes = 0;
    void* scratch = nullptr;   // build scratch, freed by bvh_free
    BvhView view() const { BvhView v = {nodes, tris, srec, drec, n_tris, root, nodes4, root4, 0, INFINITY}; return v; }
};

// Builds into `out` on `stream` (allocations with cudaMallocAsync on that stream).
void bvh_build(const BvhBuildInput& in, BvhStorage& out, void* stream);
void bvh_free(BvhStorage& s, void* stream);
std::string bvh_validate(const BvhStorage& s, void* stream);

// Leaf references of a triangle soup (9 floats per triangle): oversized
// triangles are split into several references with clipped boxes; cmin/cmax
// receive the bounds of the reference box centres (bake.cu).
void build_refs_host(const std::vector<float>& xyz, std::vector<u32>& ref_tri, std::vector<float>& ref_box, float* cmin,
                     float* cmax);

}  // namespace lg
