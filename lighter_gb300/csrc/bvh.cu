// GPU build of the flat scene BVH (layout in bvh.cuh).
//
// Replaces the reference's per-instance top-down AABBTree build
// (AABBTree::SetAABBs/_MakeNode, lighter_math.cpp:674-781) and its instance
// tree (lighter.cpp:1060-1069) with one linear BVH over all world-space
// shadow-casting triangles, built in five passes on the GPU:
//   1. 30-bit Morton code of each triangle centroid inside the scene bounds;
//   2. radix sort of (code, triangle) pairs;
//   3. Karras' (HPG 2012) top-down-by-prefix hierarchy, one thread per
//      internal node, ties between equal codes broken by index;
//   4. bottom-up box refit, one thread per leaf, second arrival at a node
//      computes its box (atomic arrival counters);
//   5. packing into 64-byte nodes that hold both child boxes, and
//      triangles reordered into leaf order.
// Leaves are triangle references: an oversized triangle may be split (on the
// host, bake.cu) into several references with clipped boxes, each holding the
// whole triangle, so every query still tests the original triangle.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <cfloat>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh.cuh"

namespace lg {
namespace {

#define BVH_CHECK(x)                                                                                  \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) throw std::runtime_error(std::string("bvh: ") + cudaGetErrorString(e_)); \
    } while (0)

__device__ __forceinline__ u32 spread10(u32 v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float* ref_box, int n, float3 mn, float3 inv_ext, u32* codes, u32* ids)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* b = ref_box + 6 * (size_t) i;
    float cx = (b[0] + b[3]) * 0.5f, cy = (b[1] + b[4]) * 0.5f, cz = (b[2] + b[5]) * 0.5f;
    float qx = fminf(fmaxf((cx - mn.x) * inv_ext.x * 1024.0f, 0.0f), 1023.0f);
    float qy = fminf(fmaxf((cy - mn.y) * inv_ext.y * 1024.0f, 0.0f), 1023.0f);
    float qz = fminf(fmaxf((cz - mn.z) * inv_ext.z * 1024.0f, 0.0f), 1023.0f);
    codes[i] = (spread10((u32) qx) << 2) | (spread10((u32) qy) << 1) | spread10((u32) qz);
    ids[i] = (u32) i;
}

__device__ __forceinline__ int prefix(const u32* codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    u32 a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((u32) i ^ (u32) j);
    return __clz(a ^ b);
}

__global__ void k_hierarchy(const u32* codes, int n, int* left, int* right, int* parent_int, int* parent_leaf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (prefix(codes, n, i, i + 1) - prefix(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = prefix(codes, n, i, i - d);
    int lmax = 2;
    while (prefix(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = prefix(codes, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        int t = (l + div - 1) / div;
        if (prefix(codes, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    int gamma = i + s * d + min(d, 0);
    int lc = (min(i, j) == gamma) ? ~gamma : gamma;
    int rc = (max(i, j) == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    if (lc < 0) parent_leaf[~lc] = i; else parent_int[lc] = i;
    if (rc < 0) parent_leaf[~rc] = i; else parent_int[rc] = i;
}

// Conservative leaf box: the reference's box widened by a few tens of ulps,
// which absorbs the rounding of the exact hit and distance tests.
__device__ __forceinline__ void leaf_box_of(const float* r, float* b)
{
    float mnx = r[0], mny = r[1], mnz = r[2], mxx = r[3], mxy = r[4], mxz = r[5];
    float m = fmaxf(fmaxf(fmaxf(fabsf(mnx), fabsf(mxx)), fmaxf(fabsf(mny), fabsf(mxy))), fmaxf(fabsf(mnz), fabsf(mxz)));
    float e = m * 2e-5f + 1e-6f;
    b[0] = mnx - e; b[1] = mny - e; b[2] = mnz - e;
    b[3] = mxx + e; b[4] = mxy + e; b[5] = mxz + e;
}

__device__ __forceinline__ void read_box(const float* boxes, int k, float* b)
{
    for (int c = 0; c < 6; ++c) b[c] = __ldcg(boxes + 6 * (size_t) k + c);
}

__global__ void k_refit(const float* ref_box, const u32* ids, int n, const int* parent_leaf, const int* parent_int,
                        const int* left, const int* right, float* leaf_box, float* int_box, u32* arrivals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float b[6];
    leaf_box_of(ref_box + 6 * (size_t) ids[i], b);
    for (int c = 0; c < 6; ++c) leaf_box[6 * (size_t) i + c] = b[c];
    __threadfence();
    int p = n > 1 ? parent_leaf[i] : -1;
    while (p >= 0) {
        if (atomicAdd(&arrivals[p], 1u) == 0u) return;
        __threadfence();
        float bl[6], br[6];
        int l = left[p], r = right[p];
        if (l < 0) read_box(leaf_box, ~l, bl); else read_box(int_box, l, bl);
        if (r < 0) read_box(leaf_box, ~r, br); else read_box(int_box, r, br);
        for (int c = 0; c < 3; ++c) {
            int_box[6 * (size_t) p + c] = fminf(bl[c], br[c]);
            int_box[6 * (size_t) p + 3 + c] = fmaxf(bl[3 + c], br[3 + c]);
        }
        __threadfence();
        p = parent_int[p];
    }
}

__global__ void k_pack_nodes(int n_int, const int* left, const int* right, const float* leaf_box, const float* int_box,
                             float4* nodes)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_int) return;
    int l = left[i], r = right[i];
    const float* L = l < 0 ? leaf_box + 6 * (size_t) (~l) : int_box + 6 * (size_t) l;
    const float* R = r < 0 ? leaf_box + 6 * (size_t) (~r) : int_box + 6 * (size_t) r;
    float4* o = nodes + 4 * (size_t) i;
    o[0] = make_float4(L[0], L[1], L[2], L[3]);
    o[1] = make_float4(L[4], L[5], R[0], R[1]);
    o[2] = make_float4(R[2], R[3], R[4], R[5]);
    o[3] = make_float4(__int_as_float(l), __int_as_float(r), 0.0f, 0.0f);
}

// ---- 4-wide nodes: the binary nodes at even depth, with their grandchildren as children

// flag[i] = 1 when internal node i lies at even depth (the root at depth 0).
__global__ void k_even_depth(int n_int, const int* __restrict__ parent_int, int* __restrict__ flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n_int) return;
    if (i == n_int) { flag[i] = 0; return; }
    int d = 0;
    for (int p = parent_int[i]; p >= 0 && d < 4096; p = parent_int[p]) ++d;
    flag[i] = (d & 1) == 0;
}

__device__ __forceinline__ void put_slot(float4* o, int k, const float* box, int child)
{
    reinterpret_cast<float*>(&o[0])[k] = box[0];
    reinterpret_cast<float*>(&o[1])[k] = box[3];
    reinterpret_cast<float*>(&o[2])[k] = box[1];
    reinterpret_cast<float*>(&o[3])[k] = box[4];
    reinterpret_cast<float*>(&o[4])[k] = box[2];
    reinterpret_cast<float*>(&o[5])[k] = box[5];
    reinterpret_cast<int*>(&o[6])[k] = child;
}

// Node layout in bvh.cuh (8 float4). Child boxes are the binary tree's, which
// are already inflated; a grandchild that is internal is referenced by its
// 4-wide index (it lies at even depth too), a leaf by ~leaf.
__global__ void k_pack4(int n_int, const int* __restrict__ flag, const int* __restrict__ idx4, const int* __restrict__ left,
                        const int* __restrict__ right, const float* __restrict__ leaf_box, const float* __restrict__ int_box,
                        float4* __restrict__ nodes4)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_int || !flag[i]) return;
    float4* o = nodes4 + 8 * (size_t) idx4[i];
    const float empty_box[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    int k = 0;
    const int kids[2] = {left[i], right[i]};
    for (int c : kids) {
        if (c < 0) {
            put_slot(o, k++, leaf_box + 6 * (size_t) (~c), c);
        } else {
            const int gk[2] = {left[c], right[c]};
            for (int g : gk) {
                const float* box = g < 0 ? leaf_box + 6 * (size_t) (~g) : int_box + 6 * (size_t) g;
                put_slot(o, k++, box, g < 0 ? g : idx4[g]);
            }
        }
    }
    for (; k < 4; ++k) put_slot(o, k, empty_box, kNoChild);
    o[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_pack_tris(int n, const u32* ids, const u32* ref_tri, const float* xyz, const u32* meta, const u32* local,
                            float4* tris)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u32 s = ref_tri[ids[i]];
    const float* p = xyz + 9 * (size_t) s;
    tris[3 * (size_t) i + 0] = make_float4(p[0], p[1], p[2], __uint_as_float(meta[s]));
    tris[3 * (size_t) i + 1] = make_float4(p[3], p[4], p[5], __uint_as_float(local[s]));
    tris[3 * (size_t) i + 2] = make_float4(p[6], p[7], p[8], __uint_as_float(s));
}

// Triangle-only terms of the two exact tests per leaf (layout in bvh.cuh),
// computed with the expressions of seg_tri / point_tri_dist in common.cuh.
__global__ void k_pack_records(int nleaf, const float4* __restrict__ tris, float4* __restrict__ srec,
                               float4* __restrict__ drec)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nleaf) return;
    float4 a = tris[3 * (size_t) i], b = tris[3 * (size_t) i + 1], c = tris[3 * (size_t) i + 2];
    V3 t0 = mk(a.x, a.y, a.z), t1 = mk(b.x, b.y, b.z), t2 = mk(c.x, c.y, c.z);
    float meta = a.w;
    V3 u = t1 - t0, v = t2 - t0;
    V3 n = cross(u, v);
    float4* s = srec + 4 * (size_t) i;
    s[0] = make_float4(t0.x, t0.y, t0.z, meta);
    s[1] = make_float4(u.x, u.y, u.z, dot(u, u));
    s[2] = make_float4(v.x, v.y, v.z, dot(u, v));
    s[3] = make_float4(n.x, n.y, n.z, dot(v, v));
    V3 nrm = normalized(cross(t1 - t0, t2 - t0));
    V3 tan0 = normalized(t1 - t0), tan1 = normalized(t2 - t1), tan2 = normalized(t0 - t2);
    V3 en0 = normalized(cross(t1 - t0, nrm)), en1 = normalized(cross(t2 - t1, nrm)), en2 = normalized(cross(t0 - t2, nrm));
    float4* d = drec + 8 * (size_t) i;
    d[0] = make_float4(nrm.x, nrm.y, nrm.z, dot(nrm, t0));
    d[1] = make_float4(tan0.x, tan0.y, tan0.z, dot(tan0, t0));
    d[2] = make_float4(tan1.x, tan1.y, tan1.z, dot(tan1, t1));
    d[3] = make_float4(tan2.x, tan2.y, tan2.z, dot(tan2, t2));
    d[4] = make_float4(dot(tan0, t1), dot(tan1, t2), dot(tan2, t0), meta);
    d[5] = make_float4(en0.x, en0.y, en0.z, dot(en0, t0));
    d[6] = make_float4(en1.x, en1.y, en1.z, dot(en1, t1));
    d[7] = make_float4(en2.x, en2.y, en2.z, dot(en2, t2));
}

// ---- locally-ordered clustering (PLOC; Meister and Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction",
// IEEE TVCG 2018). The leaves in Morton order are the first clusters; every
// iteration, each cluster finds within kPlocR positions on either side the one
// whose merged box has the least surface area, mutual nearest pairs merge into
// a new internal node at the lower position, and the list is compacted,
// keeping Morton order. Internal nodes are numbered down from n - 2 in merge
// order (ranks from a scan), so the last merge, the root, is node 0 as in
// Karras' layout. Ties between equal costs go by a key of the pair alone
// (distance in the list, then the lower position's parity, then the lower
// position), so the pairs are totally ordered: the least pair is always mutual
// (every iteration merges), and a run of equal boxes pairs up (0,1), (2,3), ...
// and halves each iteration instead of growing a chain.

constexpr int kPlocR = 16;
constexpr int kPlocB = 256;

__device__ __forceinline__ float merged_area(const float* a, const float* b)
{
    float ex = fmaxf(a[3], b[3]) - fminf(a[0], b[0]);
    float ey = fmaxf(a[4], b[4]) - fminf(a[1], b[1]);
    float ez = fmaxf(a[5], b[5]) - fminf(a[2], b[2]);
    return ex * ey + ey * ez + ez * ex;
}

__global__ void k_leaf_boxes(const float* ref_box, const u32* ids, int n, float* leaf_box, int* cl, float* cbox)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float b[6];
    leaf_box_of(ref_box + 6 * (size_t) ids[i], b);
    for (int c = 0; c < 6; ++c) {
        leaf_box[6 * (size_t) i + c] = b[c];
        cbox[6 * (size_t) i + c] = b[c];
    }
    cl[i] = ~i;
}

// The cluster count and the next node number live on the device (state[0],
// state[1]): the host launches every iteration's kernels for the count it last
// read (an upper bound), and threads past the current count do nothing.
__global__ void __launch_bounds__(kPlocB) k_ploc_nn(const int* __restrict__ state, const float* __restrict__ cbox,
                                                    int* __restrict__ nn)
{
    __shared__ float sb[(kPlocB + 2 * kPlocR) * 6];
    const int count = state[0];
    const int start = blockIdx.x * kPlocB;
    if (start >= count) return;
    for (int k = threadIdx.x; k < (kPlocB + 2 * kPlocR) * 6; k += blockDim.x) {
        const long g = (long) start * 6 - kPlocR * 6 + k;
        sb[k] = (g >= 0 && g < (long) count * 6) ? cbox[g] : 0.0f;
    }
    __syncthreads();
    const int i = start + threadIdx.x;
    if (i >= count) return;
    const float* me = sb + 6 * (threadIdx.x + kPlocR);
    float best = FLT_MAX;
    int bj = -1, bd = 1 << 30, bpar = 2, bmin = 1 << 30;
    for (int d = -kPlocR; d <= kPlocR; ++d) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= count) continue;
        const float c = merged_area(me, sb + 6 * (threadIdx.x + kPlocR + d));
        const int ad = d < 0 ? -d : d, mn = min(i, j), par = mn & 1;
        if (c < best || (c == best && (ad < bd || (ad == bd && (par < bpar || (par == bpar && mn < bmin)))))) {
            best = c; bj = j; bd = ad; bpar = par; bmin = mn;
        }
    }
    nn[i] = bj;
}

// flags[i]: merge (high word: i < nn[i] and mutual), keep (low word: not the
// upper half of a mutual pair); zero from the current count up to the bound
// `ub` the scan runs over. A single cluster keeps itself (an iteration after
// the root is done changes nothing).
__global__ void k_ploc_flags(const int* __restrict__ state, int ub, const int* __restrict__ nn,
                             unsigned long long* __restrict__ flags)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > ub) return;
    const int count = state[0];
    if (i >= count) { flags[i] = 0ull; return; }
    if (count == 1) { flags[i] = 1ull; return; }
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    const unsigned long long merge = (mutual && i < j) ? 1ull : 0ull;
    const unsigned long long keep = (mutual && i > j) ? 0ull : 1ull;
    flags[i] = (merge << 32) | keep;
}

__global__ void k_ploc_merge(const int* __restrict__ state, const int* __restrict__ nn, const unsigned long long* __restrict__ flags,
                             const unsigned long long* __restrict__ scan, const int* __restrict__ cl,
                             const float* __restrict__ cbox, int* __restrict__ ncl, float* __restrict__ ncbox,
                             int* __restrict__ left, int* __restrict__ right, int* __restrict__ parent_int,
                             float* __restrict__ int_box)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int count = state[0], base = state[1];
    if (i >= count) return;
    const unsigned long long f = flags[i];
    if (!(f & 0xffffffffull)) return;   // merged into its lower partner
    const int pos = (int) (scan[i] & 0xffffffffull);
    const float* a = cbox + 6 * (size_t) i;
    if (f >> 32) {
        const int j = nn[i];
        const int id = base - 1 - (int) (scan[i] >> 32);
        const float* b = cbox + 6 * (size_t) j;
        const int ca = cl[i], cb = cl[j];
        left[id] = ca;
        right[id] = cb;
        if (ca >= 0) parent_int[ca] = id;
        if (cb >= 0) parent_int[cb] = id;
        float u[6];
        for (int c = 0; c < 3; ++c) {
            u[c] = fminf(a[c], b[c]);
            u[3 + c] = fmaxf(a[3 + c], b[3 + c]);
        }
        for (int c = 0; c < 6; ++c) {
            int_box[6 * (size_t) id + c] = u[c];
            ncbox[6 * (size_t) pos + c] = u[c];
        }
        ncl[pos] = id;
    } else {
        for (int c = 0; c < 6; ++c) ncbox[6 * (size_t) pos + c] = a[c];
        ncl[pos] = cl[i];
    }
}

// state = (kept, base - merged) from the scan total at scan[ub]
__global__ void k_ploc_state(int* __restrict__ state, const unsigned long long* __restrict__ scan, int ub)
{
    const unsigned long long tot = scan[ub];
    state[1] -= (int) (tot >> 32);
    state[0] = (int) (tot & 0xffffffffull);
}

// depth (edges from the root) of the deepest internal node
__global__ void k_max_depth(int n_int, const int* __restrict__ parent_int, int* __restrict__ maxd)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_int) return;
    int d = 0;
    for (int p = parent_int[i]; p >= 0 && d < 4096; p = parent_int[p]) ++d;
    atomicMax(maxd, d);
}

template <class T>
T* alloc(size_t count, cudaStream_t st, size_t& bytes)
{
    void* p = nullptr;
    if (count == 0) count = 1;
    BVH_CHECK(cudaMallocAsync(&p, count * sizeof(T), st));
    bytes += count * sizeof(T);
    return (T*) p;
}

}  // namespace

void bvh_build(const BvhBuildInput& in, BvhStorage& out, void* stream)
{
    cudaStream_t st = (cudaStream_t) stream;
    const int n = in.n;
    out.n_tris = n;
    out.bytes = 0;
    if (n <= 0) { out.root = 0; return; }
    const int n_int = n > 1 ? n - 1 : 0;
    out.root = n > 1 ? 0 : ~0;

    size_t scratch_bytes = 0;
    u32* codes = alloc<u32>(n, st, scratch_bytes);
    u32* codes2 = alloc<u32>(n, st, scratch_bytes);
    u32* ids = alloc<u32>(n, st, scratch_bytes);
    u32* ids2 = alloc<u32>(n, st, scratch_bytes);
    int* left = alloc<int>(n_int, st, scratch_bytes);
    int* right = alloc<int>(n_int, st, scratch_bytes);
    int* parent_int = alloc<int>(n_int, st, scratch_bytes);
    int* parent_leaf = alloc<int>(n, st, scratch_bytes);
    float* leaf_box = alloc<float>(6 * (size_t) n, st, scratch_bytes);
    float* int_box = alloc<float>(6 * (size_t) n_int, st, scratch_bytes);
    u32* arrivals = alloc<u32>(n_int, st, scratch_bytes);

    const int B = 256;
    float3 mn = make_float3(in.scene_min[0], in.scene_min[1], in.scene_min[2]);
    float ex = in.scene_max[0] - in.scene_min[0], ey = in.scene_max[1] - in.scene_min[1], ez = in.scene_max[2] - in.scene_min[2];
    float3 inv_ext = make_float3(ex > 0 ? 1.0f / ex : 0.0f, ey > 0 ? 1.0f / ey : 0.0f, ez > 0 ? 1.0f / ez : 0.0f);
    k_morton<<<(n + B - 1) / B, B, 0, st>>>(in.ref_box, n, mn, inv_ext, codes, ids); note_launch();
    BVH_CHECK(cudaGetLastError());

    size_t temp_bytes = 0;
    BVH_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, codes, codes2, ids, ids2, n, 0, 30, st));
    void* temp = alloc<char>(temp_bytes, st, scratch_bytes);
    BVH_CHECK(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, codes, codes2, ids, ids2, n, 0, 30, st));

    // The walks keep a stack of kStack entries (the 4-wide walk up to 3 per
    // 4-wide level): a PLOC tree deeper than kPlocMaxDepth is replaced by the
    // radix hierarchy, whose depth is bounded by the code and index bits.
    constexpr int kPlocMaxDepth = 40;
    bool use_radix = in.builder == 1 || n_int == 0;
    if (!use_radix) {
        size_t pb = 0;
        int* cl = alloc<int>(n, st, pb);
        int* ncl = alloc<int>(n, st, pb);
        float* cbox = alloc<float>(6 * (size_t) n, st, pb);
        float* ncbox = alloc<float>(6 * (size_t) n, st, pb);
        int* nn = alloc<int>(n, st, pb);
        unsigned long long* flags = alloc<unsigned long long>(n + 1, st, pb);
        unsigned long long* scan = alloc<unsigned long long>(n + 1, st, pb);
        int* maxd = alloc<int>(1, st, pb);
        unsigned long long h_tot = 0;   // scan total: merges << 32 | kept
        size_t tb = 0;
        BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tb, flags, scan, n + 1, st));
        void* ptmp = alloc<char>(tb, st, pb);
        BVH_CHECK(cudaMemsetAsync(parent_int, 0xff, sizeof(int) * n_int, st));
        k_leaf_boxes<<<(n + B - 1) / B, B, 0, st>>>(in.ref_box, ids2, n, leaf_box, cl, cbox); note_launch();
        BVH_CHECK(cudaGetLastError());
        int* state = alloc<int>(2, st, pb);   // device: cluster count, next node number
        {
            const int init[2] = {n, n_int};
            BVH_CHECK(cudaMemcpyAsync(state, init, sizeof(init), cudaMemcpyHostToDevice, st));
        }
        int count = n, base = n_int;   // as last read back
        std::string fail;
        // Clustering steps run in blocks of kItersPerRead between reads of the
        // cluster count. A block is launched as one CUDA graph, captured once per
        // build with launch bounds for all n clusters: the kernels take the live
        // count from `state` (threads past it exit or write zero flags), so the
        // same graph serves every block; the even number of steps per block
        // returns the cluster buffers to their roles at its start. One graph
        // launch replaces 48 small launches (with the scan's two) and their gaps.
        constexpr int kItersPerRead = 8;
        static_assert(kItersPerRead % 2 == 0, "a block must end with the cluster buffers in their starting roles");
        cudaGraphExec_t block = nullptr;
        struct BlockGuard {
            cudaGraphExec_t& g;
            ~BlockGuard() { if (g) cudaGraphExecDestroy(g); }
        } block_guard{block};
        {
            const int ub = n;
            BVH_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            cudaError_t ce = cudaSuccess;
            for (int k = 0; k < kItersPerRead && ce == cudaSuccess; ++k) {
                k_ploc_nn<<<(ub + kPlocB - 1) / kPlocB, kPlocB, 0, st>>>(state, cbox, nn);
                k_ploc_flags<<<(ub + 1 + B - 1) / B, B, 0, st>>>(state, ub, nn, flags);
                size_t tb2 = tb;
                if (ce == cudaSuccess) ce = cudaGetLastError();
                if (ce == cudaSuccess) ce = cub::DeviceScan::ExclusiveSum(ptmp, tb2, flags, scan, ub + 1, st);
                k_ploc_merge<<<(ub + B - 1) / B, B, 0, st>>>(state, nn, flags, scan, cl, cbox, ncl, ncbox, left, right,
                                                             parent_int, int_box);
                k_ploc_state<<<1, 1, 0, st>>>(state, scan, ub);
                if (ce == cudaSuccess) ce = cudaGetLastError();
                std::swap(cl, ncl);
                std::swap(cbox, ncbox);
            }
            cudaGraph_t graph = nullptr;
            const cudaError_t ee = cudaStreamEndCapture(st, &graph);
            if (ce == cudaSuccess) ce = ee;
            if (ce == cudaSuccess) ce = cudaGraphInstantiate(&block, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            BVH_CHECK(ce);
        }
        for (int it = 0; count > 1;) {
            if (it >= 4 * n + 64) { fail = "bvh: clustering made no progress"; break; }
            BVH_CHECK(cudaGraphLaunch(block, st));
            for (int k = 0; k < 4 * kItersPerRead; ++k) note_launch();   // the graph's own kernels
            it += kItersPerRead;
            int hs[2] = {0, 0};
            BVH_CHECK(cudaMemcpyAsync(hs, state, sizeof(hs), cudaMemcpyDeviceToHost, st));
            note_d2h(sizeof(hs));
            BVH_CHECK(cudaStreamSynchronize(st));
            // every merge takes one cluster and one node number, so the next
            // number is count - 1; with more than one cluster every iteration merges
            if (hs[0] < 1 || hs[0] >= count || hs[1] != hs[0] - 1) { fail = "bvh: clustering step inconsistent"; break; }
            count = hs[0];
            base = hs[1];
        }
        if (fail.empty() && base != 0) fail = "bvh: clustering left " + std::to_string(base) + " nodes unnumbered";
        int depth = 0;
        if (fail.empty()) {
            BVH_CHECK(cudaMemsetAsync(maxd, 0, sizeof(int), st));
            k_max_depth<<<(n_int + B - 1) / B, B, 0, st>>>(n_int, parent_int, maxd); note_launch();
            BVH_CHECK(cudaGetLastError());
            BVH_CHECK(cudaMemcpyAsync(&depth, maxd, sizeof(int), cudaMemcpyDeviceToHost, st)); note_d2h(sizeof(int));
            BVH_CHECK(cudaStreamSynchronize(st));
        }
        void* pp[] = {cl, ncl, cbox, ncbox, nn, flags, scan, maxd, ptmp, state};
        for (void* p : pp) BVH_CHECK(cudaFreeAsync(p, st));
        if (!fail.empty()) {
            void* ptrs[] = {codes, codes2, ids, ids2, left, right, parent_int, parent_leaf, leaf_box, int_box, arrivals, temp};
            for (void* p : ptrs) cudaFreeAsync(p, st);
            throw std::runtime_error(fail);
        }
        use_radix = depth + 1 > kPlocMaxDepth;   // + 1: the leaves below the deepest internal node
    }
    if (use_radix) {
        if (n_int > 0) {
            BVH_CHECK(cudaMemsetAsync(parent_int, 0xff, sizeof(int) * n_int, st));
            BVH_CHECK(cudaMemsetAsync(arrivals, 0, sizeof(u32) * n_int, st));
            k_hierarchy<<<(n_int + B - 1) / B, B, 0, st>>>(codes2, n, left, right, parent_int, parent_leaf); note_launch();
            BVH_CHECK(cudaGetLastError());
        }
        k_refit<<<(n + B - 1) / B, B, 0, st>>>(in.ref_box, ids2, n, parent_leaf, parent_int, left, right, leaf_box, int_box,
                                                arrivals); note_launch();
        BVH_CHECK(cudaGetLastError());
    }

    out.nodes = alloc<float4>(4 * (size_t) (n_int > 0 ? n_int : 1), st, out.bytes);
    out.tris = alloc<float4>(3 * (size_t) n, st, out.bytes);
    if (n_int > 0) {
        k_pack_nodes<<<(n_int + B - 1) / B, B, 0, st>>>(n_int, left, right, leaf_box, int_box, out.nodes); note_launch();
        BVH_CHECK(cudaGetLastError());
    }
    // 4-wide nodes (at most one per binary node)
    out.nodes4 = alloc<float4>(8 * (size_t) (n_int > 0 ? n_int : 1), st, out.bytes);
    out.root4 = n_int > 0 ? 0 : ~0;   // the root is binary node 0 (both builders), at depth 0: 4-wide node 0
    if (n_int > 0) {
        int* flag = alloc<int>(n_int + 1, st, scratch_bytes);
        int* idx4 = alloc<int>(n_int + 1, st, scratch_bytes);
        k_even_depth<<<(n_int + 1 + B - 1) / B, B, 0, st>>>(n_int, parent_int, flag); note_launch();
        BVH_CHECK(cudaGetLastError());
        size_t tb4 = 0;
        BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tb4, flag, idx4, n_int + 1, st));
        void* t4 = alloc<char>(tb4, st, scratch_bytes);
        BVH_CHECK(cub::DeviceScan::ExclusiveSum(t4, tb4, flag, idx4, n_int + 1, st));
        k_pack4<<<(n_int + B - 1) / B, B, 0, st>>>(n_int, flag, idx4, left, right, leaf_box, int_box, out.nodes4);
        note_launch();
        BVH_CHECK(cudaGetLastError());
        BVH_CHECK(cudaFreeAsync(flag, st));
        BVH_CHECK(cudaFreeAsync(idx4, st));
        BVH_CHECK(cudaFreeAsync(t4, st));
    }
    k_pack_tris<<<(n + B - 1) / B, B, 0, st>>>(n, ids2, in.ref_tri, in.tri_xyz, in.tri_meta, in.tri_local,
                                                out.tris); note_launch();
    BVH_CHECK(cudaGetLastError());
    out.srec = alloc<float4>(4 * (size_t) n, st, out.bytes);
    out.drec = alloc<float4>(8 * (size_t) n, st, out.bytes);
    k_pack_records<<<(n + B - 1) / B, B, 0, st>>>(n, out.tris, out.srec, out.drec); note_launch();
    BVH_CHECK(cudaGetLastError());

    void* ptrs[] = {codes, codes2, ids, ids2, left, right, parent_int, parent_leaf, leaf_box, int_box, arrivals, temp};
    for (void* p : ptrs) BVH_CHECK(cudaFreeAsync(p, st));
}

// Copies the topology back and checks that a walk from the root reaches every
// internal node and every leaf exactly once; returns an empty string when the
// tree is sound. Used by the LTRG_VALIDATE=1 debug mode of the bake.
std::string bvh_validate(const BvhStorage& s, void* stream)
{
    if (s.n_tris <= 1) return "";
    const int n = s.n_tris, n_int = n - 1;
    std::vector<float4> nodes(4 * (size_t) n_int);
    BVH_CHECK(cudaMemcpyAsync(nodes.data(), s.nodes, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost,
                              (cudaStream_t) stream));
    BVH_CHECK(cudaStreamSynchronize((cudaStream_t) stream));
    std::vector<int> seen_int(n_int, 0), seen_leaf(n, 0);
    std::vector<int> stack(1, s.root);
    while (!stack.empty()) {
        int c = stack.back();
        stack.pop_back();
        if (c < 0) {
            if (~c >= n) return "leaf index out of range: " + std::to_string(~c);
            if (seen_leaf[~c]++) return "leaf reached twice: " + std::to_string(~c);
            continue;
        }
        if (c >= n_int) return "node index out of range: " + std::to_string(c);
        if (seen_int[c]++) return "node reached twice: " + std::to_string(c);
        float4 n3 = nodes[4 * (size_t) c + 3];
        int l, r;
        memcpy(&l, &n3.x, 4);
        memcpy(&r, &n3.y, 4);
        stack.push_back(l);
        stack.push_back(r);
    }
    for (int i = 0; i < n_int; ++i)
        if (!seen_int[i]) return "node unreachable: " + std::to_string(i);
    for (int i = 0; i < n; ++i)
        if (!seen_leaf[i]) return "leaf unreachable: " + std::to_string(i);
    return "";
}

void bvh_free(BvhStorage& s, void* stream)
{
    cudaStream_t st = (cudaStream_t) stream;
    if (s.nodes) cudaFreeAsync(s.nodes, st);
    if (s.nodes4) cudaFreeAsync(s.nodes4, st);
    s.nodes4 = nullptr;
    if (s.tris) cudaFreeAsync(s.tris, st);
    if (s.srec) cudaFreeAsync(s.srec, st);
    if (s.drec) cudaFreeAsync(s.drec, st);
    s.nodes = nullptr;
    s.tris = nullptr;
    s.srec = nullptr;
    s.drec = nullptr;
    s.n_tris = 0;
}

}  // namespace lg
