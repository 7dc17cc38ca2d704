// ORACLE -- test infrastructure, not product code.
//
// A plain C++ restatement of archo5/lighter's CPU bake (lighter.cpp,
// lighter_math.cpp, lighter_int.hpp), used only by tests/, smoke() and the
// cpu_baseline / --impl reference legs of bench.py as the checker. It exports
// the same ltr_* C API as the reference (plus the read-only ltrdbg_* accessors)
// so the same driver replays a scene through it, the reference build and the
// GPU library. Every function cites the reference file:line it follows; the
// float expressions keep the reference's operation order so that, built with
// -ffp-contract=off, its outputs match the reference bit for bit on one thread.
//
// Threads: max_num_threads > 1 runs the loops the reference runs on its worker
// pool (per instance: transform, trees, samples; per sample: direct light and
// AO) on std::threads. AO's per-texel random offsets are drawn up front in the
// single-threaded order, so results do not depend on the thread count.

#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <functional>
#include <string>
#include <thread>
#include <vector>

typedef uint32_t u32;
typedef int32_t i32;

namespace orc {

// Work counters of the last bake (shadow evaluations traced, sphere-trace
// steps, AO segment queries, radiosity visibility tests), for the CPU
// baseline's rays/s.
static std::atomic<unsigned long long> g_shadow_evals{0}, g_distance_queries{0}, g_ao_rays{0}, g_rad_vis{0};

// ---------------------------------------------------------------- math (lighter_int.hpp:261-557)
static const float kSmall = 0.001f;            // SMALL_FLOAT lighter_int.hpp:261
static const float kMaxPenumbraSize = 2.0f;    // lighter_int.hpp:964
static const float kMaxPenumbraStep = 1.0f;    // lighter_int.hpp:966
static const float kShadowOffset = 0.005f;     // lighter_int.hpp:967
static const float kPi = (float) M_PI;

struct V2 { float x, y; };
struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

static inline V3 mk(float x, float y, float z) { V3 v = {x, y, z}; return v; }
static inline V3 splat(float f) { return mk(f, f, f); }
static inline V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 operator*(V3 a, float f) { return mk(a.x * f, a.y * f, a.z * f); }
static inline V3 operator*(float f, V3 a) { return mk(f * a.x, f * a.y, f * a.z); }
static inline V3 operator/(V3 a, float f) { return mk(a.x / f, a.y / f, a.z / f); }
static inline V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
static inline V3& operator+=(V3& a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float lensq(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline float len(V3 a) { return sqrtf(lensq(a)); }
static inline V3 normalized(V3 a)
{
    float l = lensq(a);
    if (l == 0) return mk(0, 0, 0);
    float inv = 1.0f / sqrtf(l);
    return mk(a.x * inv, a.y * inv, a.z * inv);
}
static inline bool near_zero(V3 a) { return fabsf(a.x) < kSmall && fabsf(a.y) < kSmall && fabsf(a.z) < kSmall; }
static inline bool is_zero(V3 a) { return a.x == 0 && a.y == 0 && a.z == 0; }
static inline V3 vmin(V3 a, V3 b) { return mk(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z); }
static inline V3 vmax(V3 a, V3 b) { return mk(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z); }
static inline float fmin_(float a, float b) { return a < b ? a : b; }   // TMIN lighter_int.hpp:277
static inline float fmax_(float a, float b) { return a > b ? a : b; }   // TMAX lighter_int.hpp:278
static inline V3 lerp3(V3 a, V3 b, float s) { return a * (1.0f - s) + b * s; }  // TLERP lighter_int.hpp:285
static inline float brightness(V3 c) { return (c.x + c.y + c.z) * (1.0f / 3.0f); }  // lighter_int.hpp:926

static inline V2 mk2(float x, float y) { V2 v = {x, y}; return v; }
static inline V2 operator-(V2 a, V2 b) { return mk2(a.x - b.x, a.y - b.y); }
static inline float cross2(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }     // lighter_int.hpp:347-350
static inline float dot2(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
static inline float len2(V2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
static inline V2 normalized2(V2 a)                                           // lighter_int.hpp:325-336
{
    float l = a.x * a.x + a.y * a.y;
    if (l == 0) return mk2(0, 0);
    float inv = 1.0f / sqrtf(l);
    return mk2(a.x * inv, a.y * inv);
}

// Golden-angle spiral around `dir`, cos-weighted (lighter_int.hpp:457-471).
static V3 spiral_dir(V3 dir, float randoff, int i, int count)
{
    float q = (i + 0.5f) / count;
    float cos_side = std::sqrt(q);
    float sin_side = std::sin(std::acos(cos_side));
    float angle = (i + randoff) * (137.508f / 180.0f * (float) M_PI);
    float ca = std::cos(angle), sa = std::sin(angle);
    V3 diffvec = mk(dir.y, -dir.z, dir.x);
    V3 up = normalized(cross(dir, diffvec));
    V3 rt = cross(dir, up);
    return ca * sin_side * rt + sa * sin_side * up + cos_side * dir;
}

// Row-vector transform, translation in row 3 (lighter_int.hpp:511-520).
struct M4 { float m[4][4]; };
static inline V3 xform(const M4& M, V3 v, float w)
{
    return mk(v.x * M.m[0][0] + v.y * M.m[1][0] + v.z * M.m[2][0] + M.m[3][0] * w,
              v.x * M.m[0][1] + v.y * M.m[1][1] + v.z * M.m[2][1] + M.m[3][1] * w,
              v.x * M.m[0][2] + v.y * M.m[1][2] + v.z * M.m[2][2] + M.m[3][2] * w);
}

// Normal matrix = inverse-transpose of the upper 3x3 (Mat4::GenNormalMatrix,
// lighter_int.hpp:534-545, via Mat4::InvertTo lighter_math.cpp:19-147). With
// the 4x4 cofactor expansion applied to [R 0; 0 1], every term that holds a
// zero entry drops out exactly, leaving these 2x2 minors with the same factor
// order; det expands along row 0 and every cofactor is scaled by 1/det.
static M4 normal_matrix(const M4& M)
{
    const float a0 = M.m[0][0], a1 = M.m[0][1], a2 = M.m[0][2];
    const float a4 = M.m[1][0], a5 = M.m[1][1], a6 = M.m[1][2];
    const float a8 = M.m[2][0], a9 = M.m[2][1], a10 = M.m[2][2];
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
    c[15] = a0 * a5 * a10 - a0 * a6 * a9 - a4 * a1 * a10 + a4 * a2 * a9 + a8 * a1 * a6 - a8 * a2 * a5;
    float det = a0 * c[0] + a1 * c[4] + a2 * c[8];
    float inv[16];
    if (det == 0) {
        // InvertTo fails and leaves the padded matrix in place (lighter_math.cpp:138-139)
        for (int i = 0; i < 16; ++i) inv[i] = 0;
        inv[0] = a0; inv[1] = a1; inv[2] = a2; inv[4] = a4; inv[5] = a5; inv[6] = a6;
        inv[8] = a8; inv[9] = a9; inv[10] = a10; inv[15] = 1;
    } else {
        float d = 1.0f / det;
        for (int i = 0; i < 16; ++i) inv[i] = c[i] * d;
    }
    M4 out;
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) out.m[r][k] = inv[k * 4 + r];  // transpose
    return out;
}

// Heron's formula (lighter_math.cpp:150-173).
static inline float heron(float a, float b, float c)
{
    float p = (a + b + c) * 0.5f;
    float pre = p * (p - a) * (p - b) * (p - c);
    if (pre < 0) return 0;
    return sqrtf(pre);
}
static inline float tri_area3(V3 p1, V3 p2, V3 p3) { return heron(len(p2 - p1), len(p3 - p2), len(p1 - p3)); }
static inline float tri_area2(V2 p1, V2 p2, V2 p3) { return heron(len2(p2 - p1), len2(p3 - p2), len2(p1 - p3)); }
// lighter_math.cpp:175-181
static inline float sample_area(V2 t1, V2 t2, V2 t3, V3 p1, V3 p2, V3 p3)
{
    float lm = tri_area2(t1, t2, t3);
    float co = tri_area3(p1, p2, p3);
    return lm > 0 ? co / lm : 0;
}

// ---------------------------------------------------------------- geometry queries
struct Tri { V3 P1, P2, P3; };
struct Box { V3 mn, mx; };
static inline bool tri_useful(const Tri& t) { return !near_zero(cross(t.P2 - t.P1, t.P3 - t.P1)); }  // lighter_int.hpp:604-608
static inline Box tri_box(const Tri& t)                                                          // lighter_int.hpp:609-613
{
    Box b;
    b.mn = mk(fmin_(t.P1.x, fmin_(t.P2.x, t.P3.x)), fmin_(t.P1.y, fmin_(t.P2.y, t.P3.y)), fmin_(t.P1.z, fmin_(t.P2.z, t.P3.z)));
    b.mx = mk(fmax_(t.P1.x, fmax_(t.P2.x, t.P3.x)), fmax_(t.P1.y, fmax_(t.P2.y, t.P3.y)), fmax_(t.P1.z, fmax_(t.P2.z, t.P3.z)));
    return b;
}
static inline bool box_valid(const Box& b) { return b.mn.x <= b.mx.x && b.mn.y <= b.mx.y && b.mn.z <= b.mx.z; }
static inline float box_volume(const Box& b) { return (b.mx.x - b.mn.x) * (b.mx.y - b.mn.y) * (b.mx.z - b.mn.z); }
static inline V3 box_center(const Box& b) { return (b.mn + b.mx) * 0.5f; }
static inline V3 tri_normal_rev(const Tri& t) { return normalized(cross(t.P3 - t.P1, t.P2 - t.P1)); }  // lighter_int.hpp:614-617

// Segment/triangle: fraction r in [0,1] along L1->L2 or 2 (lighter_math.cpp:315-354).
static float seg_tri(V3 L1, V3 L2, V3 P1, V3 P2, V3 P3)
{
    V3 u = P2 - P1, v = P3 - P1;
    V3 n = cross(u, v);
    if (near_zero(n)) return 2.0f;
    V3 dir = L2 - L1, w0 = L1 - P1;
    float a = -dot(n, w0);
    float b = dot(n, dir);
    if (fabsf(b) < kSmall) return 2.0f;
    float r = a / b;
    if (r < 0.0f || r > 1.0f) return 2.0f;
    V3 I = L1 + r * dir;
    float uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
    V3 w = I - P1;
    float wu = dot(w, u), wv = dot(w, v);
    float D = uv * uv - uu * vv;
    float s = (uv * wv - vv * wu) / D;
    if (s < 0.0f || s > 1.0f) return 2.0f;
    float t = (uv * wu - uu * wv) / D;
    if (t < 0.0f || (s + t) > 1.0f) return 2.0f;
    return r;
}

// Watertight segment/triangle test (Woop, Benthin and Wald, JCGT 2013), the
// GPU library's LTRG_ISECT_WATERTIGHT mode: shear the triangle into the
// segment's frame (segment along +z over [0, 1]); the signs of the 2D edge
// functions decide inclusion, with an FP64 recomputation of any edge function
// that is exactly 0 in FP32. Fraction r in [0, 1] or 2.
static float comp3(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static float seg_tri_watertight(V3 L1, V3 L2, V3 P1, V3 P2, V3 P3)
{
    V3 D = L2 - L1;
    float ax = fabsf(D.x), ay = fabsf(D.y), az = fabsf(D.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    float dz = comp3(D, kz);
    if (dz == 0.0f) return 2.0f;
    if (dz < 0.0f) std::swap(kx, ky);
    float Sx = comp3(D, kx) / dz, Sy = comp3(D, ky) / dz, Sz = 1.0f / dz;
    V3 A = P1 - L1, B = P2 - L1, C = P3 - L1;
    float Ax = comp3(A, kx) - Sx * comp3(A, kz), Ay = comp3(A, ky) - Sy * comp3(A, kz);
    float Bx = comp3(B, kx) - Sx * comp3(B, kz), By = comp3(B, ky) - Sy * comp3(B, kz);
    float Cx = comp3(C, kx) - Sx * comp3(C, kz), Cy = comp3(C, ky) - Sy * comp3(C, kz);
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float) ((double) Cx * (double) By - (double) Cy * (double) Bx);
        V = (float) ((double) Ax * (double) Cy - (double) Ay * (double) Cx);
        W = (float) ((double) Bx * (double) Ay - (double) By * (double) Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 2.0f;
    float det = U + V + W;
    if (det == 0.0f) return 2.0f;
    float Az = Sz * comp3(A, kz), Bz = Sz * comp3(B, kz), Cz = Sz * comp3(C, kz);
    float T = U * Az + V * Bz + W * Cz;
    if (det > 0.0f ? (T < 0.0f || T > det) : (T > 0.0f || T < det)) return 2.0f;
    return T / det;
}

// The segment test of the bake in progress: the reference's, or the watertight
// one when the scene's intersect mode asks for it (set by ltr_Scene::run; the
// oracle bakes one scene at a time).
static bool g_watertight = false;
static float seg_test(V3 L1, V3 L2, V3 P1, V3 P2, V3 P3)
{
    return g_watertight ? seg_tri_watertight(L1, L2, P1, P2, P3) : seg_tri(L1, L2, P1, P2, P3);
}

// Unsigned point/triangle distance via corner/edge/face regions (lighter_math.cpp:875-913).
static float point_tri_dist(V3 pt, V3 t0, V3 t1, V3 t2)
{
    V3 nrm = normalized(cross(t1 - t0, t2 - t0));
    float pd = fabsf(dot(nrm, pt) - dot(nrm, t0));
    V3 tan0 = normalized(t1 - t0), tan1 = normalized(t2 - t1), tan2 = normalized(t0 - t2);
    float t0p = dot(tan0, pt), t0min = dot(tan0, t0), t0max = dot(tan0, t1);
    float t1p = dot(tan1, pt), t1min = dot(tan1, t1), t1max = dot(tan1, t2);
    float t2p = dot(tan2, pt), t2min = dot(tan2, t2), t2max = dot(tan2, t0);
    if (t0min >= t0p && t2max <= t2p) return len(pt - t0);
    if (t1min >= t1p && t0max <= t0p) return len(pt - t1);
    if (t2min >= t2p && t1max <= t1p) return len(pt - t2);
    V3 en0 = normalized(cross(t1 - t0, nrm)), en1 = normalized(cross(t2 - t1, nrm)), en2 = normalized(cross(t0 - t2, nrm));
    float d0 = dot(en0, pt) - dot(en0, t0), d1 = dot(en1, pt) - dot(en1, t1), d2 = dot(en2, pt) - dot(en2, t2);
    if (d0 >= 0 && t0p >= t0min && t0p <= t0max) return len2(mk2(pd, d0));
    if (d1 >= 0 && t1p >= t1min && t1p <= t1max) return len2(mk2(pd, d1));
    if (d2 >= 0 && t2p >= t2min && t2p <= t2max) return len2(mk2(pd, d2));
    return pd;
}

// Point projects into the triangle, with SMALL_FLOAT slack (lighter_math.cpp:915-952).
static bool point_proj_on_tri(V3 pt, V3 t0, V3 t1, V3 t2)
{
    V3 nrm = normalized(cross(t1 - t0, t2 - t0));
    V3 tan0 = normalized(t1 - t0), tan1 = normalized(t2 - t1), tan2 = normalized(t0 - t2);
    float t0p = dot(tan0, pt), t0min = dot(tan0, t0), t0max = dot(tan0, t1);
    float t1p = dot(tan1, pt), t1min = dot(tan1, t1), t1max = dot(tan1, t2);
    float t2p = dot(tan2, pt), t2min = dot(tan2, t2), t2max = dot(tan2, t0);
    if (t0min - kSmall > t0p && t2max + kSmall < t2p) return false;
    if (t1min - kSmall > t1p && t0max + kSmall < t0p) return false;
    if (t2min - kSmall > t2p && t1max + kSmall < t1p) return false;
    V3 en0 = normalized(cross(t1 - t0, nrm)), en1 = normalized(cross(t2 - t1, nrm)), en2 = normalized(cross(t0 - t2, nrm));
    float d0 = dot(en0, pt) - dot(en0, t0), d1 = dot(en1, pt) - dot(en1, t1), d2 = dot(en2, pt) - dot(en2, t2);
    if (d0 > kSmall && t0p - kSmall > t0min && t0p + kSmall < t0max) return false;
    if (d1 > kSmall && t1p - kSmall > t1min && t1p + kSmall < t1max) return false;
    if (d2 > kSmall && t2p - kSmall > t2min && t2p + kSmall < t2max) return false;
    return true;
}

// Slab test without a tmax>=0 check (lighter_math.cpp:618-650).
static bool ray_box(V3 ro, V3 inv, float length, V3 mn, V3 mx)
{
    float tmin = -FLT_MAX, tmax = FLT_MAX;
    if (inv.x != 0.0f) {
        float a = (mn.x - ro.x) * inv.x, b = (mx.x - ro.x) * inv.x;
        tmin = fmax_(tmin, fmin_(a, b)); tmax = fmin_(tmax, fmax_(a, b));
    }
    if (inv.y != 0.0f) {
        float a = (mn.y - ro.y) * inv.y, b = (mx.y - ro.y) * inv.y;
        tmin = fmax_(tmin, fmin_(a, b)); tmax = fmin_(tmax, fmax_(a, b));
    }
    if (inv.z != 0.0f) {
        float a = (mn.z - ro.z) * inv.z, b = (mx.z - ro.z) * inv.z;
        tmin = fmax_(tmin, fmin_(a, b)); tmax = fmin_(tmax, fmax_(a, b));
    }
    return tmax >= tmin && length >= tmin;
}

// Ray set-up of BaseRayQuery (lighter_int.hpp:680-702).
struct Ray {
    V3 o, end, inv;
    float length;
    void set(V3 r0, V3 r1)
    {
        o = r0; end = r1;
        length = len(r1 - r0);
        V3 d = normalized(r1 - r0);
        inv = mk(d.x ? 1 / d.x : 0, d.y ? 1 / d.y : 0, d.z ? 1 / d.z : 0);
    }
};

// ---------------------------------------------------------------- AABB tree (lighter_int.hpp:706-821, lighter_math.cpp:653-781)
struct BVH {
    struct Node { V3 mn, mx; i32 ch, ido; };
    std::vector<Node> nodes;
    std::vector<i32> items;   // per node: <count> then ids

    void build(const Box* boxes, size_t count)
    {
        nodes.clear(); items.clear();
        Node root; root.mn = splat(FLT_MAX); root.mx = splat(-FLT_MAX); root.ch = -1; root.ido = -1;
        nodes.push_back(root);
        if (!count) return;
        std::vector<i32> ids;
        for (size_t i = 0; i < count; ++i)
            if (box_valid(boxes[i])) ids.push_back((i32) i);
        make(0, boxes, ids.data(), ids.size(), 0);
    }
    void emit_items(i32 node, const i32* ids, size_t n)
    {
        nodes[node].ido = (i32) items.size();
        items.push_back((i32) n);
        for (size_t i = 0; i < n; ++i) items.push_back(ids[i]);
    }
    // Top-down split (lighter_math.cpp:696-781): leaf at <=4 items or depth 16;
    // items whose volume*3 >= node volume stay in the node; the rest are
    // sorted along the longest axis of their union and halved.
    void make(i32 node, const Box* boxes, const i32* ids, size_t n, int depth)
    {
        V3 mn = splat(FLT_MAX), mx = splat(-FLT_MAX);
        for (size_t i = 0; i < n; ++i) { mn = vmin(mn, boxes[ids[i]].mn); mx = vmax(mx, boxes[ids[i]].mx); }
        nodes[node].mn = mn; nodes[node].mx = mx;
        Box nb = {mn, mx};
        float nvol = box_volume(nb);
        if (n > 4 && depth < 16) {
            nodes[node].ido = -1; nodes[node].ch = -1;
            int nsplit = 0;
            V3 smn = splat(FLT_MAX), smx = splat(-FLT_MAX);
            for (size_t i = 0; i < n; ++i) {
                const Box& b = boxes[ids[i]];
                if (box_volume(b) * 3 < nvol) { nsplit++; smn = vmin(smn, b.mn); smx = vmax(smx, b.mx); }
            }
            V3 ss = smx - smn;
            V3 axis = mk(0, 0, 1);
            if (ss.x > ss.y && ss.x > ss.z) axis = mk(1, 0, 0);
            else if (ss.y > ss.x && ss.y > ss.z) axis = mk(0, 1, 0);
            if (nsplit >= 4) {
                std::vector<i32> self, split;
                for (size_t i = 0; i < n; ++i) {
                    if (box_volume(boxes[ids[i]]) * 3 < nvol) split.push_back(ids[i]);
                    else self.push_back(ids[i]);
                }
                if (!self.empty()) emit_items(node, self.data(), self.size());
                std::sort(split.begin(), split.end(), [&](i32 a, i32 b) {
                    return dot(axis, box_center(boxes[a])) < dot(axis, box_center(boxes[b]));
                });
                size_t mid = split.size() / 2;
                nodes.push_back(Node());
                make((i32) nodes.size() - 1, boxes, split.data(), mid, depth + 1);
                nodes[node].ch = (i32) nodes.size();
                nodes.push_back(Node());
                make((i32) nodes.size() - 1, boxes, split.data() + mid, split.size() - mid, depth + 1);
                return;
            }
        }
        emit_items(node, ids, n);
        nodes[node].ch = -1;
    }
    // DFS, node items before children, left child = node+1 (lighter_int.hpp:742-762);
    // cb returns false to stop.
    bool ray_query(const Ray& r, const std::function<bool(const i32*, i32)>& cb, i32 node = 0) const
    {
        const Node& N = nodes[node];
        if (!ray_box(r.o, r.inv, r.length, N.mn, N.mx)) return true;
        if (N.ido != -1 && !cb(&items[N.ido + 1], items[N.ido])) return false;
        if (N.ch != -1) {
            if (!ray_query(r, cb, node + 1)) return false;
            if (!ray_query(r, cb, N.ch)) return false;
        }
        return true;
    }
    // Box query whose box may shrink during the walk (lighter_int.hpp:764-784).
    template <class Q> void dyn_query(Q& q, i32 node = 0) const
    {
        const Node& N = nodes[node];
        if (q.mn.x > N.mx.x || q.mx.x < N.mn.x || q.mn.y > N.mx.y || q.mx.y < N.mn.y || q.mn.z > N.mx.z || q.mx.z < N.mn.z)
            return;
        if (N.ido != -1) q(&items[N.ido + 1], items[N.ido]);
        if (N.ch != -1) { dyn_query(q, node + 1); dyn_query(q, N.ch); }
    }
    // Fixed-box query (lighter_int.hpp:786-806).
    template <class F> void box_query(V3 qmn, V3 qmx, F& f, i32 node = 0) const
    {
        const Node& N = nodes[node];
        if (qmn.x > N.mx.x || qmx.x < N.mn.x || qmn.y > N.mx.y || qmx.y < N.mn.y || qmn.z > N.mx.z || qmx.z < N.mn.z)
            return;
        if (N.ido != -1) f(&items[N.ido + 1], items[N.ido]);
        if (N.ch != -1) { box_query(qmn, qmx, f, node + 1); box_query(qmn, qmx, f, N.ch); }
    }
    // All item lists in storage order (lighter_int.hpp:808-814).
    template <class F> void all(F& f) const
    {
        for (size_t i = 0; i < items.size(); i += 1 + items[i]) f(&items[i + 1], items[i]);
    }
};

// Triangle tree of one instance (lighter_math.cpp:785-1044).
struct TriTree {
    BVH bvh;
    std::vector<Tri> tris;
    void set(const Tri* t, size_t n)
    {
        tris.clear();
        std::vector<Box> boxes;
        for (size_t i = 0; i < n; ++i)
            if (tri_useful(t[i])) { boxes.push_back(tri_box(t[i])); tris.push_back(t[i]); }
        bvh.build(boxes.data(), boxes.size());
    }
    bool any_hit(V3 from, V3 to) const   // lighter_math.cpp:804-832
    {
        Ray r; r.set(from, to);
        bool hit = false;
        bvh.ray_query(r, [&](const i32* ids, i32 n) {
            for (i32 i = 0; i < n; ++i) {
                const Tri& T = tris[ids[i]];
                hit = seg_test(r.o, r.end, T.P1, T.P2, T.P3) < 1.0f;
                if (hit) return false;
            }
            return true;
        });
        return hit;
    }
    float closest(V3 from, V3 to, i32* tid) const   // lighter_math.cpp:835-871
    {
        Ray r; r.set(from, to);
        float best = 2; i32 hid = -1;
        bvh.ray_query(r, [&](const i32* ids, i32 n) {
            for (i32 i = 0; i < n; ++i) {
                const Tri& T = tris[ids[i]];
                float d = seg_test(r.o, r.end, T.P1, T.P2, T.P3);
                if (d < best) { best = d; hid = ids[i]; }
            }
            return true;
        });
        if (hid != -1 && tid) *tid = hid;
        return best;
    }
    float distance(V3 p, float d0) const   // lighter_math.cpp:954-989
    {
        struct Q {
            const TriTree* t; V3 pos, mn, mx; float dist;
            void recalc() { mn = pos - splat(dist); mx = pos + splat(dist); }
            void operator()(const i32* ids, i32 n)
            {
                for (i32 i = 0; i < n; ++i) {
                    const Tri& T = t->tris[ids[i]];
                    float nd = point_tri_dist(pos, T.P1, T.P2, T.P3);
                    if (nd < dist) { dist = nd; recalc(); }
                }
            }
        } q;
        q.t = this; q.pos = p; q.dist = d0; q.recalc();
        bvh.dyn_query(q);
        return q.dist;
    }
    // Push a sample out of concave edges (lighter_math.cpp:991-1044). The query
    // box is fixed at the start; P moves as triangles are processed.
    void offset_sample(V3& P, V3 N, float dist) const
    {
        auto f = [&](const i32* ids, i32 n) {
            for (i32 i = 0; i < n; ++i) {
                const Tri& T = tris[ids[i]];
                float nd = point_tri_dist(P, T.P1, T.P2, T.P3);
                if (nd < dist) {
                    V3 TPN = -tri_normal_rev(T);
                    float TPD = dot(TPN, T.P1);
                    float sig = dot(TPN, P) - TPD;
                    if (sig <= kSmall) {
                        V3 Pextr = P + normalized(TPN + N) * -sig * 1.41f;
                        if (point_proj_on_tri(Pextr, T.P1, T.P2, T.P3)) {
                            float pdot = dot(TPN, N);
                            if (fabsf(pdot) < 0.95f) {
                                V3 proj = normalized(TPN - N * pdot);
                                float df = 1.0f - fabsf(pdot);
                                V3 Pnew = P + proj * (-sig / df + kSmall);
                                i32 tid = -1;
                                if (closest(P + (N + proj) * kSmall, Pnew, &tid) >= 0.9f || tid == ids[i]) P = Pnew;
                            }
                        }
                    }
                }
            }
        };
        bvh.box_query(P - splat(dist), P + splat(dist), f);
    }
};

// ---------------------------------------------------------------- BSP (lighter_int.hpp:623-677, lighter_math.cpp:428-614)
struct BSP {
    V3 N = {0, 0, 0};
    float D = 0;
    BSP* front = nullptr;
    BSP* back = nullptr;
    std::vector<Tri> tris;
    ~BSP() { delete front; delete back; }

    // Unique vertices, longest pairwise direction through their centroid; accept
    // when both sides are populated, duplication stays under 1.7x and the
    // imbalance under 3:1 (lighter_math.cpp:547-614).
    bool pick_plane()
    {
        std::vector<V3> pts;
        auto add = [&](V3 p) {
            for (size_t k = 0; k < pts.size(); ++k)
                if (pts[k].x == p.x && pts[k].y == p.y && pts[k].z == p.z) return;
            pts.push_back(p);
        };
        for (const Tri& T : tris) { add(T.P1); add(T.P2); add(T.P3); }
        V3 center = mk(0, 0, 0), dir = mk(0, 0, 0);
        float best = 0;
        for (size_t i = 0; i < pts.size(); ++i) {
            center += pts[i];
            for (size_t j = i + 1; j < pts.size(); ++j) {
                V3 d = pts[j] - pts[i];
                float l = lensq(d);
                if (l > best) { dir = d; best = l; }
            }
        }
        if (pts.size()) center = center / (float) pts.size();
        N = normalized(dir);
        D = dot(N, center);
        int na = 0, nb = 0;
        for (const Tri& T : tris) {
            float d1 = dot(T.P1, N) - D, d2 = dot(T.P2, N) - D, d3 = dot(T.P3, N) - D;
            if (d1 * d2 > -kSmall && d2 * d3 > -kSmall) {
                if (d1 > 0) na++; else nb++;
            } else {
                na += (d1 > 0) + (d2 > 0) + (d3 > 0);
                nb += (d1 <= 0) + (d2 <= 0) + (d3 <= 0);
            }
        }
        if (na != 0 && nb != 0 && na + nb < tris.size() * 1.7f) {
            float q = (float) na / (float) nb;
            if (q < 1) q = 1 / q;
            return q < 3.0f;
        }
        return false;
    }
    // Straddling triangles go to both sides unsplit (lighter_math.cpp:459-488).
    void add_split(const Tri& T)
    {
        float p1 = dot(N, T.P1) - D, p2 = dot(N, T.P2) - D, p3 = dot(N, T.P3) - D;
        if (p1 * p2 >= -kSmall && p1 * p3 >= -kSmall) {
            (p1 + p2 + p3 > 0 ? front : back)->tris.push_back(T);
            return;
        }
        front->tris.push_back(T);
        back->tris.push_back(T);
    }
    void split(int depth)   // lighter_math.cpp:432-457
    {
        if (tris.size() > 16 && depth < 32 && pick_plane()) {
            front = new BSP; back = new BSP;
            for (const Tri& T : tris) add_split(T);
            if (front->tris.size() + back->tris.size() > tris.size() * 3 / 2) {
                delete front; delete back; front = back = nullptr;
                return;
            }
            std::vector<Tri>().swap(tris);
            front->split(depth + 1);
            back->split(depth + 1);
        }
    }
    // Near side first; the first side with a hit < 1 wins (lighter_math.cpp:490-533).
    float intersect(V3 from, V3 to, V3* outn) const
    {
        if (front) {
            float df = dot(from, N) - D, dt = dot(to, N) - D;
            if (df < 0) {
                float h = back->intersect(from, to, outn);
                if (h < 1.0f) return h;
                return dt > 0 ? front->intersect(from, to, outn) : 2.0f;
            }
            float h = front->intersect(from, to, outn);
            if (h < 1.0f) return h;
            return dt < 0 ? back->intersect(from, to, outn) : 2.0f;
        }
        float best = 2.0f;
        const Tri* bt = nullptr;
        for (const Tri& T : tris) {
            float h = seg_test(from, to, T.P1, T.P2, T.P3);
            if (h < best) { best = h; bt = &T; }
        }
        if (outn && bt) *outn = tri_normal_rev(*bt);
        return best;
    }
};

// ---------------------------------------------------------------- worker pool stand-in
static void parallel_for(int threads, size_t n, const std::function<void(size_t)>& fn)
{
    if (threads <= 1 || n < 2) { for (size_t i = 0; i < n; ++i) fn(i); return; }
    std::atomic<size_t> next(0);
    const size_t chunk = n > 4096 ? 64 : 1;
    std::vector<std::thread> pool;
    int nt = (int) std::min<size_t>((size_t) threads, n);
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                size_t b = next.fetch_add(chunk);
                if (b >= n) break;
                size_t e = std::min(n, b + chunk);
                for (size_t i = b; i < e; ++i) fn(i);
            }
        });
    for (auto& th : pool) th.join();
}

}  // namespace orc

// ---------------------------------------------------------------- public ABI types (layouts of lighter.h:64-233)
extern "C" {
typedef float ltr_VEC3[3];
typedef float ltr_VEC4[4];
typedef ltr_VEC4 ltr_MAT4[4];
struct ltr_MeshPartInfo {
    const void* positions_f3; const void* normals_f3; const void* texcoords1_f2; const void* texcoords2_f2;
    u32 stride_positions, stride_normals, stride_texcoords1, stride_texcoords2;
    const u32* indices; u32 vertex_count; u32 index_count; int shadow;
};
struct ltr_MeshInstanceInfo { ltr_MAT4 matrix; float importance; int shadow; const char* ident; size_t ident_size; };
struct ltr_LightInfo {
    u32 type; ltr_VEC3 position, direction, up_direction, color_rgb;
    float range, power, light_radius; int shadow_sample_count; float spot_angle_out, spot_angle_in, spot_curve;
};
struct ltr_SampleInfo { u32 id; ltr_VEC3 position, normal, out_color; };
struct ltr_SampleRequest {
    ltr_VEC3 position, normal; float tex0u, tex0v, tex1u, tex1v; uint32_t part_id;
    const char* mesh_ident; size_t mesh_ident_size; const char* inst_ident; size_t inst_ident_size;
    ltr_VEC3 out_diffuse_color, out_emissive_color;
};
struct ltr_Config {
    void* userdata;
    int (*size_fn)(ltr_Config*, const char*, size_t, const char*, size_t, float, float, u32*);
    int max_num_threads; size_t max_tree_memory; u32 max_lightmap_size, default_width, default_height;
    float global_size_factor, max_correct_dist, max_correct_angle;
    ltr_VEC3 clear_color, ambient_color;
    int bounce_count;
    int (*sample_fn)(ltr_Config*, ltr_SampleRequest*);
    float ao_distance, ao_multiplier, ao_falloff, ao_effect, ao_divergence;
    ltr_VEC3 ao_color_rgb; int ao_num_samples; float blur_size; int ds2x; int generate_normalmap_data;
};
struct ltr_WorkOutputInfo { u32 lightmap_count, sample_count; ltr_SampleInfo* samples; };
struct ltr_WorkOutput {
    u32 uid; const char* mesh_ident; size_t mesh_ident_size; const char* inst_ident; size_t inst_ident_size;
    float* lightmap_rgb; float* normals_xyzf; u32 width, height;
};
struct ltr_WorkStatus { float completion; const char* stage; };
#define API __attribute__((visibility("default")))
API u32 ltr_NextPowerOfTwo(u32 x);
API int ltr_DefaultSizeFunc(ltr_Config*, const char*, size_t, const char*, size_t, float, float, u32*);
struct ltr_Scene;
API void ltr_GetConfig(ltr_Config* cfg, ltr_Scene* opt);
}

using namespace orc;

struct OPart { u32 vcount, voff, icount, ioff; int shadow; };
struct ltr_Scene;
struct ltr_Mesh {
    ltr_Scene* scene;
    std::string ident;
    std::vector<V3> pos, nrm;
    std::vector<V2> tex1, tex2;
    std::vector<u32> idx;
    std::vector<OPart> parts;
};
struct Contrib { V3 n; i32 sid; };
struct OInst {
    ltr_Mesh* mesh = nullptr;
    std::string ident;
    float importance = 0;
    M4 matrix;
    u32 w = 128, h = 128;
    bool shadow = false, container = false;
    std::vector<V3> vpos, vnrm;
    std::vector<V2> vtex, ltex;
    BSP bsp;
    TriTree tree;
    std::vector<V3> spos, snrm;
    std::vector<u32> sloc;
    std::vector<V4> srad;
    std::vector<V3> lm;
    std::vector<Contrib> contrib;
    // per-ray records of the last bake, for the hit/miss comparison with the GPU:
    // dbg_vis[light * n + i] = CalcInvShadowFactor of (light, sample i), -1 when not traced;
    // dbg_ao[i * ao_num_samples + r] = closest-hit fraction of AO ray r of sample i
    std::vector<float> dbg_vis, dbg_ao;
};
struct OLight {
    u32 type; V3 pos, dir, up, color; float range, power, radius; int nsamples; float out, in, curve;
    float randoff;           // the light's randf() of ltr_LightAdd (lighter.cpp:1300)
    std::vector<V3> smp;     // shadow samples: ray directions (directional) or disk offsets (point, spot)
};
struct RadColors { V3 diff, total, out, in; float area; };
struct RadLink { u32 other; float f; };

struct ltr_Scene {
    ltr_Config cfg;
    std::vector<ltr_Mesh*> meshes;
    std::vector<OInst*> insts;
    std::vector<OLight> lights;
    std::vector<ltr_SampleInfo> samples;
    std::vector<ltr_WorkOutput> outputs;
    std::vector<V3> rad_pos, rad_nrm;
    std::vector<RadColors> rad_col;
    std::vector<V3> rad_emit;   // the emission each element's bounces start from
    std::vector<RadLink> links;
    std::vector<u32> linkmap;
    BVH inst_tree;
    // modes beyond the reference (orc_SetOptions); 0 everywhere is the reference bake
    u32 opt_shadow_mode = 0;      // 1: sampled soft shadows
    u32 opt_isect = 0;            // 1: watertight segment/triangle test
    u32 opt_patches = 0;          // > 0: patch radiosity over about this many patches
    u32 opt_links = 0;            // 1: link mutually visible pairs (0: occluded ones, lighter.cpp:751)
    std::atomic<const char*> stage{"not started"};
    std::atomic<float> completion{0};
    std::thread worker;
    ltr_Scene();
    ~ltr_Scene();

    // scene-level queries (lighter.cpp:112-289)
    bool occluded(V3 A, V3 B) const
    {
        V3 dn = normalized(B - A);
        V3 mA = A + dn * kSmall, mB = B - dn * kSmall;
        Ray r; r.set(mA, mB);
        bool hit = false;
        inst_tree.ray_query(r, [&](const i32* ids, i32 n) {
            for (i32 i = 0; i < n; ++i) {
                const OInst* mi = insts[ids[i]];
                if (mi->shadow) { hit = mi->tree.any_hit(r.o, mB); if (hit) return false; }
            }
            return true;
        });
        return hit;
    }
    float distance(V3 p) const
    {
        struct Q {
            const ltr_Scene* S; V3 pos, mn, mx; float dist;
            void recalc() { mn = pos - splat(dist); mx = pos + splat(dist); }
            void operator()(const i32* ids, i32 n)
            {
                for (i32 i = 0; i < n; ++i) {
                    const OInst* mi = S->insts[ids[i]];
                    if (mi->shadow) {
                        float nd = mi->tree.distance(pos, dist);
                        if (nd < dist) { dist = nd; recalc(); }
                    }
                }
            }
        } q;
        q.S = this; q.pos = p; q.dist = kMaxPenumbraSize; q.recalc();
        inst_tree.dyn_query(q);
        return q.dist;
    }
    float inv_shadow(V3 from, V3 to, float k) const   // lighter.cpp:190-207
    {
        g_shadow_evals.fetch_add(1, std::memory_order_relaxed);
        V3 rd = normalized(to - from);
        float maxt = len(to - from);
        float res = 1.0f;
        for (float t = 0.001f; t < maxt;) {
            float h = distance(from + rd * t);
            g_distance_queries.fetch_add(1, std::memory_order_relaxed);
            if (h < 0.001f) return 0.0f;
            res = fmin_(res, h / fmin_(t * k, kMaxPenumbraSize));
            h = fmin_(h, kMaxPenumbraStep);
            t += h;
        }
        return res;
    }
    // Sampled soft shadows: 1 - (occluded rays) / n over the light's shadow
    // samples. Directional: rays from `from` along each direction over range
    // (lighter.cpp:566-584). Point/spot: rays to the disk points around the
    // light in the plane facing the sample, with the basis of
    // CreateSpiralDirVector (lighter_int.hpp:465-467) built on `dir` (the
    // sample-to-light direction).
    float sampled_vis(const OLight& L, V3 from, V3 dir) const
    {
        g_shadow_evals.fetch_add((unsigned long long) L.nsamples, std::memory_order_relaxed);
        float f = 0.0f;
        if (L.type == 3) {
            for (int k = 0; k < L.nsamples; ++k)
                if (occluded(from, from + L.smp[k] * L.range)) f += 1.0f;
        } else {
            V3 diffvec = mk(dir.y, -dir.z, dir.x);
            V3 up = normalized(cross(dir, diffvec));
            V3 rt = cross(dir, up);
            for (int k = 0; k < L.nsamples; ++k) {
                V3 T = L.pos + rt * L.smp[k].x + up * L.smp[k].y;
                if (occluded(from, T)) f += 1.0f;
            }
        }
        f /= L.nsamples;
        return 1.0f - f;
    }
    float closest_bsp(V3 A, V3 B, V3* outn) const   // lighter.cpp:210-251
    {
        V3 dn = normalized(B - A);
        V3 mA = A + dn * kSmall, mB = B - dn * kSmall;
        Ray r; r.set(mA, mB);
        float best = 2;
        inst_tree.ray_query(r, [&](const i32* ids, i32 n) {
            for (i32 i = 0; i < n; ++i) {
                const OInst* mi = insts[ids[i]];
                if (mi->shadow) {
                    V3 nrm = mk(0, 0, 0);
                    float d = mi->bsp.intersect(r.o, mB, &nrm);
                    if (d < best) { best = d; if (outn) *outn = nrm; }
                }
            }
            return true;
        });
        return best;
    }
    float closest_tree(V3 A, V3 B) const   // lighter.cpp:254-289
    {
        V3 dn = normalized(B - A);
        V3 mA = A + dn * kSmall, mB = B - dn * kSmall;
        Ray r; r.set(mA, mB);
        float best = 2;
        inst_tree.ray_query(r, [&](const i32* ids, i32 n) {
            for (i32 i = 0; i < n; ++i) {
                const OInst* mi = insts[ids[i]];
                if (mi->shadow) { float d = mi->tree.closest(r.o, mB, nullptr); if (d < best) best = d; }
            }
            return true;
        });
        return best;
    }

    // min(max_num_threads, cpus), at least 1 (lighter.cpp:1149)
    int threads() const
    {
        int hw = (int) std::thread::hardware_concurrency();
        int n = cfg.max_num_threads < hw ? cfg.max_num_threads : hw;
        return n > 1 ? n : 1;
    }
    void prexform(OInst* mi);
    void colinfo(OInst* mi);
    void make_samples(OInst* mi);
    void render_light(const OLight& L, OInst* mi, size_t li);
    void rad_links();
    void rad_bounce();
    void rad_patches();
    void ao(OInst* mi, const std::vector<float>& randoff);
    void finalize();
    void run();
};

static u32 next_pow2(u32 x)   // lighter.cpp:1348-1357
{
    x--; x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
    return x + 1;
}

static float randf() { return (float) rand() / (float) RAND_MAX; }   // lighter_int.hpp:271

// lighter.cpp:292-341
void ltr_Scene::prexform(OInst* mi)
{
    if (mi->container) return;
    ltr_Mesh* me = mi->mesh;
    size_t nv = me->pos.size();
    mi->vpos.resize(nv); mi->vnrm.resize(nv); mi->vtex.resize(nv); mi->ltex.resize(nv);
    M4 nm = normal_matrix(mi->matrix);
    for (size_t i = 0; i < nv; ++i) {
        mi->vpos[i] = xform(mi->matrix, me->pos[i], 1.0f);
        mi->vnrm[i] = normalized(xform(nm, me->nrm[i], 0.0f));
    }
    float area = 0.0f;
    for (const OPart& p : me->parts) {
        const V3* vb = &mi->vpos[p.voff];
        const u32* ib = &me->idx[p.ioff];
        for (u32 t = 0; t < p.icount; t += 3) area += tri_area3(vb[ib[t]], vb[ib[t + 1]], vb[ib[t + 2]]);
    }
    u32 size[2] = {cfg.default_width, cfg.default_height};
    if (!cfg.size_fn(&cfg, me->ident.c_str(), me->ident.size(), mi->ident.c_str(), mi->ident.size(), area,
                     mi->importance, size)) {
        size[0] = cfg.default_width; size[1] = cfg.default_height;
    }
    mi->w = size[0]; mi->h = size[1];
    float fw = (float) mi->w, fh = (float) mi->h;
    for (size_t i = 0; i < nv; ++i) {
        mi->vtex[i] = me->tex1[i];
        mi->ltex[i] = mk2(me->tex2[i].x * fw - 0.5f, me->tex2[i].y * fh - 0.5f);
    }
}

// lighter.cpp:349-384
void ltr_Scene::colinfo(OInst* mi)
{
    if (mi->container) { mi->tree.set(nullptr, 0); return; }
    std::vector<Tri> tris;
    ltr_Mesh* me = mi->mesh;
    for (const OPart& p : me->parts) {
        if (!p.shadow) continue;
        const V3* vb = &mi->vpos[p.voff];
        const u32* ib = &me->idx[p.ioff];
        for (u32 t = 0; t < p.icount; t += 3) {
            Tri T = {vb[ib[t]], vb[ib[t + 1]], vb[ib[t + 2]]};
            if (tri_useful(T)) tris.push_back(T);
        }
    }
    if (!tris.empty()) { mi->bsp.tris = tris; mi->bsp.split(0); }
    mi->tree.set(tris.data(), tris.size());
}

// Texels within `margin` of the triangle (either winding) get the barycentric
// interpolation of three attribute sets; s and t are clamped separately
// (lighter_math.cpp:245-302).
static void raster_tri(V3* img1, V3* img2, V4* img3, i32 w, i32 h, float margin, V2 p1, V2 p2, V2 p3,
                       V3 a1, V3 a2, V3 a3, V3 b1, V3 b2, V3 b3, V4 c1, V4 c2, V4 c3)
{
    i32 maxX = (i32) (fmax_(p1.x, fmax_(p2.x, p3.x)) + margin);
    i32 minX = (i32) (fmin_(p1.x, fmin_(p2.x, p3.x)) - margin);
    i32 maxY = (i32) (fmax_(p1.y, fmax_(p2.y, p3.y)) + margin);
    i32 minY = (i32) (fmin_(p1.y, fmin_(p2.y, p3.y)) - margin);
    if (maxX < 0 || minX >= w || maxY < 0 || minY >= h) return;
    if (minX < 0) minX = 0;
    if (maxX >= w) maxX = w - 1;
    if (minY < 0) minY = 0;
    if (maxY >= h) maxY = h - 1;
    V2 e12 = p2 - p1, e13 = p3 - p1;
    float vc = cross2(e12, e13);
    if (vc == 0) return;
    V2 n1 = normalized2(mk2(e12.y, -e12.x));
    V2 e23 = p3 - p2;
    V2 n2 = normalized2(mk2(e23.y, -e23.x));
    V2 n3t = normalized2(mk2(e13.y, -e13.x));
    V2 n3 = mk2(-n3t.x, -n3t.y);
    float d1 = dot2(n1, p1), d2 = dot2(n2, p2), d3 = dot2(n3, p3);
    V3 da2 = a2 - a1, da3 = a3 - a1, db2 = b2 - b1, db3 = b3 - b1;
    V4 dc2 = {c2.x - c1.x, c2.y - c1.y, c2.z - c1.z, c2.w - c1.w};
    V4 dc3 = {c3.x - c1.x, c3.y - c1.y, c3.z - c1.z, c3.w - c1.w};
    for (i32 x = minX; x <= maxX; x++) {
        for (i32 y = minY; y <= maxY; y++) {
            V2 q = mk2(x - p1.x, y - p1.y);
            float s = cross2(q, e13) / vc;
            float t = cross2(e12, q) / vc;
            s = fmax_(fmin_(s, 1.0f), 0.0f);
            t = fmax_(fmin_(t, 1.0f), 0.0f);
            V2 p = mk2((float) x, (float) y);
            float pd1 = dot2(p, n1), pd2 = dot2(p, n2), pd3 = dot2(p, n3);
            if ((pd1 <= d1 + margin && pd2 <= d2 + margin && pd3 <= d3 + margin) ||
                (pd1 + margin >= d1 && pd2 + margin >= d2 && pd3 + margin >= d3)) {
                size_t o = (size_t) x + (size_t) w * y;
                img1[o] = a1 + da2 * s + da3 * t;
                img2[o] = b1 + db2 * s + db3 * t;
                V4 c = {c1.x + dc2.x * s + dc3.x * t, c1.y + dc2.y * s + dc3.y * t, c1.z + dc2.z * s + dc3.z * t,
                        c1.w + dc2.w * s + dc3.w * t};
                img3[o] = c;
            }
        }
    }
}

// lighter.cpp:32-66
static void raster_instance(OInst* mi, float margin, V3* R1, V3* R2, V4* R3)
{
    ltr_Mesh* me = mi->mesh;
    for (u32 part = 0; part < me->parts.size(); ++part) {
        const OPart& p = me->parts[part];
        const u32* ib = &me->idx[p.ioff];
        for (u32 t = 0; t < p.icount; t += 3) {
            u32 i1 = p.voff + ib[t], i2 = p.voff + ib[t + 1], i3 = p.voff + ib[t + 2];
            float sa = sample_area(mi->ltex[i1], mi->ltex[i2], mi->ltex[i3], mi->vpos[i1], mi->vpos[i2], mi->vpos[i3]);
            V4 c1 = {mi->vtex[i1].x, mi->vtex[i1].y, (float) part, sa};
            V4 c2 = {mi->vtex[i2].x, mi->vtex[i2].y, (float) part, sa};
            V4 c3 = {mi->vtex[i3].x, mi->vtex[i3].y, (float) part, sa};
            raster_tri(R1, R2, R3, (i32) mi->w, (i32) mi->h, margin, mi->ltex[i1], mi->ltex[i2], mi->ltex[i3],
                       mi->vpos[i1], mi->vpos[i2], mi->vpos[i3], mi->vnrm[i1], mi->vnrm[i2], mi->vnrm[i3], c1, c2, c3);
        }
    }
}

// lighter.cpp:392-476
void ltr_Scene::make_samples(OInst* mi)
{
    float corr_min_dot = cosf(cfg.max_correct_angle / 180.0f * (float) M_PI);
    V3 amb = mk(cfg.ambient_color[0], cfg.ambient_color[1], cfg.ambient_color[2]);
    if (mi->container) {
        for (auto& c : mi->lm) c = amb;
        return;
    }
    size_t n = (size_t) mi->w * mi->h;
    std::vector<V3> R1(n, mk(0, 0, 0)), R2(n, mk(0, 0, 0));
    V4 z4 = {0, 0, 0, 0};
    std::vector<V4> R3(n, z4);
    raster_instance(mi, 0.5f + kSmall, R1.data(), R2.data(), R3.data());
    raster_instance(mi, 0.0f, R1.data(), R2.data(), R3.data());
    for (size_t i = 0; i < n; ++i) {
        if (is_zero(R2[i])) continue;
        V3 N = normalized(R2[i]);
        V3 P = R1[i];
        V4 XD = R3[i];
        for (OInst* other : insts) other->tree.offset_sample(P, N, sqrtf(XD.w));
        if (cfg.max_correct_dist) {
            int left = 100;
            float md = cfg.max_correct_dist;
            V3 PEnd = P + N * md;
            while (md > kSmall && left-- > 0) {
                V3 hn = mk(0, 0, 0);
                float q = closest_bsp(P, PEnd, &hn);
                if (-dot(hn, N) < corr_min_dot) break;
                if (q < kSmall) q = kSmall;
                P = P * (1.0f - q) + PEnd * q;
                md *= (1.0f - q);
            }
        }
        mi->spos.push_back(P);
        mi->snrm.push_back(N);
        mi->sloc.push_back((u32) i);
        mi->srad.push_back(XD);
    }
    mi->lm.assign(mi->spos.size(), amb);
}

// Point / spot / directional direct light per sample (lighter.cpp:485-600, 623-665).
void ltr_Scene::render_light(const OLight& L, OInst* mi, size_t li)
{
    size_t n = mi->lm.size();
    float* dvis = &mi->dbg_vis[li * n];
    bool want_n = cfg.generate_normalmap_data && !mi->container;
    std::vector<Contrib> contribs;
    if (cfg.generate_normalmap_data) { Contrib z = {mk(0, 0, 0), -1}; contribs.assign(n, z); }
    float out_rad = 0, diff = 0;
    if (L.type == 2) {
        out_rad = L.out / 180.0f * (float) M_PI;
        float in_rad = L.in / 180.0f * (float) M_PI;
        if (in_rad == out_rad) in_rad -= kSmall;
        diff = in_rad - out_rad;
    }
    parallel_for(threads(), (L.type >= 1 && L.type <= 3) ? n : 0, [&](size_t i) {
        V3 SP = mi->spos[i], SN = mi->snrm[i];
        if (L.type == 1 || L.type == 2) {
            V3 s2l = L.pos - SP;
            float dist = len(s2l);
            if (dist) s2l = s2l / dist;
            float f_dist = std::pow(1 - fmin_(1.0f, dist / L.range), L.power);
            float f_ndotl = fmax_(0.0f, dot(s2l, SN));
            float f_dir = 1.0f;
            if (L.type == 2) {
                float ang = std::acos(fmin_(1.0f, dot(s2l, -L.dir)));
                f_dir = fmax_(0.0f, fmin_(1.0f, (ang - out_rad) / diff));
                f_dir = std::pow(f_dir, L.curve);
                if (f_dist * f_ndotl * f_dir <= 0) return;
            } else if (f_dist * f_ndotl <= 0) {
                return;
            }
            float vis = opt_shadow_mode == 1 ? sampled_vis(L, SP + SN * kShadowOffset, s2l)
                                             : inv_shadow(SP + SN * kShadowOffset, L.pos, L.radius);
            dvis[i] = vis;
            float k = L.type == 2 ? f_dist * f_ndotl * f_dir * vis : f_dist * f_ndotl * vis;
            mi->lm[i] += L.color * k;
            if (want_n) {
                float fac = L.type == 2 ? f_dist * f_dir * vis * f_ndotl * brightness(L.color)
                                        : f_dist * vis * f_ndotl * brightness(L.color);
                if (fac > 0) { Contrib c = {s2l * fac, (i32) i}; contribs[i] = c; }
            }
        } else if (opt_shadow_mode == 1) {
            // the sampled block of lighter.cpp:566-584 (ray origin SP, N.L averaged)
            float f_ndotl = 0.0f;
            for (int k = 0; k < L.nsamples; ++k) f_ndotl += fmax_(0.0f, dot(L.smp[k], SN));
            f_ndotl /= L.nsamples;
            float vis = sampled_vis(L, SP, L.dir);
            dvis[i] = vis;
            mi->lm[i] += L.color * (f_ndotl * vis);
            if (want_n) {
                float fac = vis * f_ndotl * brightness(L.color);
                if (fac > 0) { Contrib c = {L.dir * fac, (i32) i}; contribs[i] = c; }
            }
        } else {
            float f_ndotl = fmax_(0.0f, dot(L.dir, SN));
            float vis = inv_shadow(SP + SN * kShadowOffset, SP + L.dir * L.range, L.radius);
            dvis[i] = vis;
            mi->lm[i] += L.color * (f_ndotl * vis);
            if (want_n) {
                float fac = vis * f_ndotl * brightness(L.color);
                if (fac > 0) { Contrib c = {L.dir * fac, (i32) i}; contribs[i] = c; }
            }
        }
    });
    if (cfg.generate_normalmap_data)
        for (const Contrib& c : contribs)
            if (c.sid >= 0) mi->contrib.push_back(c);
}

// Sample gathering, then links for pairs that pass the facing/form-factor tests
// and for which VisibilityTest() reports an occluder (lighter.cpp:667-765).
void ltr_Scene::rad_links()
{
    rad_pos.clear(); rad_nrm.clear(); rad_col.clear(); rad_emit.clear(); links.clear(); linkmap.clear();
    for (OInst* mi : insts) {
        for (size_t i = 0; i < mi->lm.size(); ++i) {
            V3 P = mi->spos[i];
            V3 N = normalized(mi->snrm[i]);
            rad_pos.push_back(P);
            rad_nrm.push_back(N);
            V3 diffc = mk(1, 1, 1);
            V3 emit = mi->lm[i];
            float area = mi->container ? 0 : mi->srad[i].w;
            if (mi->container) {
                diffc = mk(0, 0, 0);
            } else if (cfg.sample_fn) {
                u32 L = mi->sloc[i];
                int lx = (int) (L % mi->w), ly = (int) (L / mi->w);
                ltr_SampleRequest req;
                req.position[0] = P.x; req.position[1] = P.y; req.position[2] = P.z;
                req.normal[0] = N.x; req.normal[1] = N.y; req.normal[2] = N.z;
                req.tex0u = mi->srad[i].x; req.tex0v = mi->srad[i].y;
                req.tex1u = (lx + 0.5f) / mi->w; req.tex1v = (ly + 0.5f) / mi->h;
                req.part_id = (uint32_t) mi->srad[i].z;
                req.mesh_ident = mi->mesh->ident.c_str(); req.mesh_ident_size = mi->mesh->ident.size();
                req.inst_ident = mi->ident.c_str(); req.inst_ident_size = mi->ident.size();
                req.out_diffuse_color[0] = 1; req.out_diffuse_color[1] = 1; req.out_diffuse_color[2] = 1;
                req.out_emissive_color[0] = 0; req.out_emissive_color[1] = 0; req.out_emissive_color[2] = 0;
                if (cfg.sample_fn(&cfg, &req)) {
                    diffc = mk(req.out_diffuse_color[0], req.out_diffuse_color[1], req.out_diffuse_color[2]);
                    emit += mk(req.out_emissive_color[0], req.out_emissive_color[1], req.out_emissive_color[2]);
                }
            }
            RadColors rc = {diffc, emit, emit, mk(0, 0, 0), area};
            rad_col.push_back(rc);
            rad_emit.push_back(emit);
        }
    }
    const size_t N = rad_pos.size();
    for (size_t i = 0; i < N; ++i) {
        linkmap.push_back((u32) links.size());
        linkmap.push_back(0);
        V3 AP = rad_pos[i], AN = rad_nrm[i];
        for (size_t j = i + 1; j < N; ++j) {
            V3 BP = rad_pos[j], BN = rad_nrm[j];
            V3 pd = BP - AP;
            float dA = dot(AN, pd), dB = dot(BN, -pd);
            if (dA <= kSmall || dB <= kSmall) continue;
            float l2 = lensq(pd);
            float f = dA * dB / (l2 * l2 * (float) M_PI);
            if (f < kSmall) continue;
            g_rad_vis.fetch_add(1, std::memory_order_relaxed);
            if (occluded(AP, BP) == false) continue;
            RadLink rl = {(u32) j, f};
            links.push_back(rl);
            linkmap.back()++;
        }
    }
}

// Patch radiosity, the GPU library's radiosity_patches mode (no reference
// counterpart; the pair factor, link test and bounce are the reference's,
// lighter.cpp:673-797, over patches instead of samples).
//  1. Per-sample inputs as rad_links gathers them: position, unit normal,
//     sample_fn diffuse and emission, sample area (probes: black, area 0).
//  2. A patch slot per covered sample: (instance, lightmap tile of side t
//     texels, dominant axis and sign of the unit normal), slots numbered
//     instance by instance, tile row by row, six axes per tile. The side t
//     starts at round(sqrt(covered / target)) and moves (at most 8 trials)
//     towards the side whose occupied-slot count comes closest to the target
//     in |log(count / target)|, stopping once the count crosses the target.
//  3. Patches = occupied slots in slot order; a patch's area is the sum of its
//     samples' areas and its position, normal (renormalised), diffuse and
//     emission the area-weighted means, summed in sample order in double.
//  4. Links between patches with the pair factor of lighter.cpp:733-757 and
//     the predicate opt_links (1: the pair is not occluded, 0: it is, as
//     lighter.cpp:751), then bounce_count sweeps of lighter.cpp:767-797.
//  5. Every covered sample receives its own emission plus its patch's
//     bounced light (total - emission); probes keep their direct light.
void ltr_Scene::rad_patches()
{
    struct SIn { V3 diff, emis; u32 inst; size_t idx; };
    std::vector<SIn> sin;
    size_t n_cov = 0;
    for (u32 ii = 0; ii < insts.size(); ++ii) {
        OInst* mi = insts[ii];
        for (size_t i = 0; i < mi->lm.size(); ++i) {
            V3 P = mi->spos[i];
            V3 N = normalized(mi->snrm[i]);
            V3 diffc = mk(1, 1, 1), emis = mk(0, 0, 0);
            if (mi->container) {
                diffc = mk(0, 0, 0);
            } else if (cfg.sample_fn) {
                u32 L = mi->sloc[i];
                int lx = (int) (L % mi->w), ly = (int) (L / mi->w);
                ltr_SampleRequest req;
                req.position[0] = P.x; req.position[1] = P.y; req.position[2] = P.z;
                req.normal[0] = N.x; req.normal[1] = N.y; req.normal[2] = N.z;
                req.tex0u = mi->srad[i].x; req.tex0v = mi->srad[i].y;
                req.tex1u = (lx + 0.5f) / mi->w; req.tex1v = (ly + 0.5f) / mi->h;
                req.part_id = (uint32_t) mi->srad[i].z;
                req.mesh_ident = mi->mesh->ident.c_str(); req.mesh_ident_size = mi->mesh->ident.size();
                req.inst_ident = mi->ident.c_str(); req.inst_ident_size = mi->ident.size();
                req.out_diffuse_color[0] = 1; req.out_diffuse_color[1] = 1; req.out_diffuse_color[2] = 1;
                req.out_emissive_color[0] = 0; req.out_emissive_color[1] = 0; req.out_emissive_color[2] = 0;
                if (cfg.sample_fn(&cfg, &req)) {
                    diffc = mk(req.out_diffuse_color[0], req.out_diffuse_color[1], req.out_diffuse_color[2]);
                    emis = mk(req.out_emissive_color[0], req.out_emissive_color[1], req.out_emissive_color[2]);
                }
            }
            SIn e = {diffc, emis, ii, i};
            sin.push_back(e);
            if (!mi->container) ++n_cov;
        }
    }
    // 2. slots
    const u32 target = opt_patches;
    std::vector<unsigned long long> slot_base(insts.size() + 1, 0);
    std::vector<u32> ntx(insts.size(), 0);
    auto layout = [&](u32 t) {
        for (size_t i = 0; i < insts.size(); ++i) {
            const OInst* mi = insts[i];
            ntx[i] = mi->container ? 0 : (mi->w + t - 1) / t;
            unsigned long long ns = mi->container ? 0 : (unsigned long long) ntx[i] * ((mi->h + t - 1) / t) * 6;
            slot_base[i + 1] = slot_base[i] + ns;
        }
        return slot_base[insts.size()];
    };
    auto slot_of = [&](const SIn& e, u32 t) -> unsigned long long {
        const OInst* mi = insts[e.inst];
        u32 L = mi->sloc[e.idx], w = mi->w;
        u32 tx = (L % w) / t, ty = (L / w) / t;
        V3 nn = normalized(mi->snrm[e.idx]);
        float ax = std::fabs(nn.x), ay = std::fabs(nn.y), az = std::fabs(nn.z);
        u32 axis = (ax >= ay && ax >= az) ? (nn.x >= 0 ? 0 : 1) : (ay >= az ? (nn.y >= 0 ? 2 : 3) : (nn.z >= 0 ? 4 : 5));
        return slot_base[e.inst] + ((unsigned long long) ty * ntx[e.inst] + tx) * 6 + axis;
    };
    auto trial = [&](u32 t) -> u32 {
        layout(t);
        std::vector<unsigned long long> sl;
        for (const SIn& e : sin)
            if (!insts[e.inst]->container) sl.push_back(slot_of(e, t));
        std::sort(sl.begin(), sl.end());
        return (u32) (std::unique(sl.begin(), sl.end()) - sl.begin());
    };
    u32 tile = (u32) std::max(1.0, std::floor(std::sqrt(std::max(1.0, (double) n_cov / target)) + 0.5));
    {
        auto off = [&](u32 c) { return std::fabs(std::log(std::max(1.0, (double) c) / target)); };
        u32 c = trial(tile), best = tile;
        double best_off = off(c);
        const int dir = c > target ? 1 : -1;
        for (int k = 0; k < 8; ++k) {
            if ((dir > 0 && c <= target) || (dir < 0 && (c >= target || tile == 1))) break;
            u32 t2 = (u32) std::floor(tile * std::sqrt((double) c / target) + 0.5);
            t2 = dir > 0 ? std::max(t2, tile + 1) : std::max(1u, std::min(t2, tile - 1));
            tile = t2;
            c = trial(tile);
            if (off(c) < best_off) { best_off = off(c); best = tile; }
        }
        tile = best;
    }
    layout(tile);
    // 3. patches in slot order, samples in sample order
    std::vector<unsigned long long> sslot(sin.size(), ~0ull);
    std::vector<unsigned long long> occ;
    for (size_t k = 0; k < sin.size(); ++k)
        if (!insts[sin[k].inst]->container) { sslot[k] = slot_of(sin[k], tile); occ.push_back(sslot[k]); }
    std::sort(occ.begin(), occ.end());
    occ.erase(std::unique(occ.begin(), occ.end()), occ.end());
    const size_t np = occ.size();
    std::vector<long long> pid(sin.size(), -1);
    std::vector<std::array<double, 13>> q(np);
    for (auto& a : q) a.fill(0.0);
    for (size_t k = 0; k < sin.size(); ++k) {
        if (sslot[k] == ~0ull) continue;
        size_t p = (size_t) (std::lower_bound(occ.begin(), occ.end(), sslot[k]) - occ.begin());
        pid[k] = (long long) p;
        const OInst* mi = insts[sin[k].inst];
        size_t i = sin[k].idx;
        double a = mi->srad[i].w;
        V3 n = normalized(mi->snrm[i]), P = mi->spos[i], D = sin[k].diff;
        V3 e = mi->lm[i];
        e += sin[k].emis;
        double v[13] = {a, a * P.x, a * P.y, a * P.z, a * n.x, a * n.y, a * n.z, a * D.x, a * D.y, a * D.z,
                        a * e.x, a * e.y, a * e.z};
        for (int c = 0; c < 13; ++c) q[p][c] += v[c];
    }
    rad_pos.assign(np, mk(0, 0, 0));
    rad_nrm.assign(np, mk(0, 0, 0));
    rad_col.assign(np, RadColors());
    rad_emit.assign(np, mk(0, 0, 0));
    for (size_t p = 0; p < np; ++p) {
        double a = q[p][0] > 0 ? q[p][0] : 1.0;
        rad_pos[p] = mk((float) (q[p][1] / a), (float) (q[p][2] / a), (float) (q[p][3] / a));
        rad_nrm[p] = normalized(mk((float) (q[p][4] / a), (float) (q[p][5] / a), (float) (q[p][6] / a)));
        V3 E = mk((float) (q[p][10] / a), (float) (q[p][11] / a), (float) (q[p][12] / a));
        RadColors rc = {mk((float) (q[p][7] / a), (float) (q[p][8] / a), (float) (q[p][9] / a)), E, E, mk(0, 0, 0),
                        (float) q[p][0]};
        rad_col[p] = rc;
        rad_emit[p] = E;
    }
    // 4. links (rows on parallel threads, concatenated in row order), then the sweeps
    std::vector<std::vector<RadLink>> rows(np);
    parallel_for(threads(), np, [&](size_t i) {
        V3 AP = rad_pos[i], AN = rad_nrm[i];
        for (size_t j = i + 1; j < np; ++j) {
            V3 BP = rad_pos[j], BN = rad_nrm[j];
            V3 pd = BP - AP;
            float dA = dot(AN, pd), dB = dot(BN, -pd);
            if (dA <= kSmall || dB <= kSmall) continue;
            float l2 = lensq(pd);
            float f = dA * dB / (l2 * l2 * (float) M_PI);
            if (f < kSmall) continue;
            g_rad_vis.fetch_add(1, std::memory_order_relaxed);
            bool occ_ij = occluded(AP, BP);
            if (opt_links == 1 ? occ_ij : !occ_ij) continue;
            RadLink rl = {(u32) j, f};
            rows[i].push_back(rl);
        }
    });
    links.clear();
    linkmap.clear();
    for (size_t i = 0; i < np; ++i) {
        linkmap.push_back((u32) links.size());
        linkmap.push_back((u32) rows[i].size());
        links.insert(links.end(), rows[i].begin(), rows[i].end());
    }
    stage = "bouncing light";
    for (int b = 0; b < cfg.bounce_count; ++b) rad_bounce();
    stage = "committing radiosity";
    // 5. own emission plus the patch's bounced light
    for (size_t k = 0; k < sin.size(); ++k) {
        OInst* mi = insts[sin[k].inst];
        V3& c = mi->lm[sin[k].idx];
        c += sin[k].emis;
        if (pid[k] >= 0) {
            const V3 T = rad_col[(size_t) pid[k]].total, E = rad_emit[(size_t) pid[k]];
            c.x += T.x - E.x;
            c.y += T.y - E.y;
            c.z += T.z - E.z;
        }
    }
}

// One symmetric sweep over the links (lighter.cpp:767-797).
void ltr_Scene::rad_bounce()
{
    for (size_t i = 0; i < linkmap.size() / 2; ++i) {
        size_t b = linkmap[i * 2], e = b + linkmap[i * 2 + 1];
        for (size_t s = b; s < e; ++s) {
            size_t j = links[s].other;
            float f = links[s].f;
            RadColors& A = rad_col[i];
            RadColors& B = rad_col[j];
            V3 Ao = (A.out * A.diff) * A.area * f;
            V3 Bo = (B.out * B.diff) * B.area * f;
            A.total += Bo; B.total += Ao;
            A.in += Bo; B.in += Ao;
        }
    }
    for (RadColors& c : rad_col) { c.out = c.in; c.in = mk(0, 0, 0); }
}

// lighter.cpp:799-841
void ltr_Scene::ao(OInst* mi, const std::vector<float>& randoff)
{
    float dist = cfg.ao_distance, falloff = cfg.ao_falloff, mult = cfg.ao_multiplier, effect = cfg.ao_effect;
    int ns = cfg.ao_num_samples;
    V3 aoc = mk(cfg.ao_color_rgb[0], cfg.ao_color_rgb[1], cfg.ao_color_rgb[2]);
    mi->dbg_ao.assign(mi->lm.size() * (size_t) (ns > 0 ? ns : 0), 2.0f);
    parallel_for(threads(), mi->lm.size(), [&](size_t i) {
        V3 SP = mi->spos[i], SN = mi->snrm[i];
        V3& out = mi->lm[i];
        V3 ro = SP + SN * (kSmall * 2);
        float f = 0;
        for (int s = 0; s < ns; ++s) {
            V3 rd = spiral_dir(SN, randoff[i], s, ns) * dist;
            float hit = closest_tree(ro, ro + rd);
            mi->dbg_ao[i * ns + s] = hit;
            g_ao_rays.fetch_add(1, std::memory_order_relaxed);
            if (hit < 1.0f) f += 1.0f - hit;
        }
        f /= ns;
        f = fmin_(f * mult, 1.0f);
        if (falloff) f = std::pow(f, falloff);
        if (effect >= 0) out = out * (1 - f * (1 - effect)) + aoc * f;
        else out = lerp3(out, lerp3(aoc, aoc * out, -effect), f);
    });
}

// Gaussian taps (lighter_math.cpp:357-365) and transposing row convolution
// with clamp-to-edge (lighter_math.cpp:367-398).
static void gauss_kernel(float* out, int ext, float radius)
{
    float sum = 0.0f;
    float mc = 1.0f / sqrtf(2.0f * (float) M_PI * radius * radius);
    for (int i = -ext; i <= ext; ++i) sum += out[i + ext] = std::exp(-0.5f * std::pow((float) i / radius, 2.0f)) * mc;
    for (int i = -ext; i <= ext; ++i) out[i + ext] /= sum;
}
static void convolve_transpose(const float* src, float* dst, u32 w, u32 h, int ext, const float* k, float* tmp)
{
    for (u32 y = 0; y < h; ++y) {
        memcpy(tmp + ext * 3, src + (size_t) y * w * 3, sizeof(float) * w * 3);
        for (int i = 0; i < ext; ++i)
            for (int c = 0; c < 3; ++c) {
                tmp[i * 3 + c] = tmp[ext * 3 + c];
                tmp[(ext + w + i) * 3 + c] = tmp[(ext + w - 1) * 3 + c];
            }
        for (u32 x = 0; x < w; ++x) {
            const float* sp = tmp + (x + ext) * 3;
            float* dp = dst + ((size_t) y + (size_t) h * x) * 3;
            float s0 = 0, s1 = 0, s2 = 0;
            for (int i = -ext; i <= ext; ++i) {
                float kq = k[i + ext];
                s0 += sp[i * 3 + 0] * kq; s1 += sp[i * 3 + 1] * kq; s2 += sp[i * 3 + 2] * kq;
            }
            dp[0] = s0; dp[1] = s1; dp[2] = s2;
        }
    }
}

// lighter.cpp:849-1044
void ltr_Scene::finalize()
{
    for (size_t mid = 0; mid < insts.size(); ++mid) {
        OInst* mi = insts[mid];
        if (mi->container) {
            for (size_t i = 0; i < mi->lm.size(); ++i) {
                samples[i].out_color[0] = mi->lm[i].x; samples[i].out_color[1] = mi->lm[i].y;
                samples[i].out_color[2] = mi->lm[i].z;
            }
            continue;
        }
        u32 w = mi->w, h = mi->h;
        float* img = new float[(size_t) w * h * 3];
        std::vector<char> set((size_t) w * h * 2, 0);
        std::fill(img, img + (size_t) w * h * 3, 0.0f);
        for (size_t i = 0; i < mi->sloc.size(); ++i) {
            size_t o = (size_t) mi->sloc[i] * 3;
            img[o] = mi->lm[i].x; img[o + 1] = mi->lm[i].y; img[o + 2] = mi->lm[i].z;
            set[mi->sloc[i]] = 1;
        }
        auto isset = [&](u32 x, u32 y) { return x < w && y < h && set[x + (size_t) y * w]; };
        auto col = [&](u32 x, u32 y) { size_t o = (x + (size_t) y * w) * 3; return mk(img[o], img[o + 1], img[o + 2]); };
        for (int it = 1; it <= 3; ++it) {
            memcpy(&set[(size_t) w * h], &set[0], (size_t) w * h);
            for (u32 y = 0; y < h; ++y)
                for (u32 x = 0; x < w; ++x) {
                    if (set[x + (size_t) y * w]) continue;
                    V3 c = mk(0, 0, 0);
                    int cnt = 0;
                    if (isset(x - 1, y)) { c += isset(x - 2, y) ? lerp3(col(x - 2, y), col(x - 1, y), 2.0f) : col(x - 1, y); cnt++; }
                    if (isset(x + 1, y)) { c += isset(x + 2, y) ? lerp3(col(x + 2, y), col(x + 1, y), 2.0f) : col(x + 1, y); cnt++; }
                    if (isset(x, y - 1)) { c += isset(x, y - 2) ? lerp3(col(x, y - 2), col(x, y - 1), 2.0f) : col(x, y - 1); cnt++; }
                    if (isset(x, y + 1)) { c += isset(x, y + 2) ? lerp3(col(x, y + 2), col(x, y + 1), 2.0f) : col(x, y + 1); cnt++; }
                    if (cnt) {
                        c = c / (float) cnt;
                        size_t o = (x + (size_t) y * w) * 3;
                        img[o] = fmax_(c.x, 0.0f); img[o + 1] = fmax_(c.y, 0.0f); img[o + 2] = fmax_(c.z, 0.0f);
                        set[x + (size_t) y * w + (size_t) w * h] = 1;
                    }
                }
            memcpy(&set[0], &set[(size_t) w * h], (size_t) w * h);
        }
        if (cfg.blur_size) {
            int ext = (int) std::ceil(cfg.blur_size);
            std::vector<float> tmpimg((size_t) w * h * 3), row(((size_t) std::max(w, h) + ext * 2) * 3), k(ext * 2 + 1);
            gauss_kernel(k.data(), ext, cfg.blur_size);
            convolve_transpose(img, tmpimg.data(), w, h, ext, k.data(), row.data());
            convolve_transpose(tmpimg.data(), img, h, w, ext, k.data(), row.data());
        }
        u32 ow = w, oh = h;
        if (cfg.ds2x) {   // lighter.cpp:963-975, lighter_math.cpp:400-424
            u32 hw = std::max(w / 2, 1u), hh = std::max(h / 2, 1u);
            float* ds = new float[(size_t) hw * hh * 3];
            for (u32 y = 0; y < hh; ++y)
                for (u32 x = 0; x < hw; ++x) {
                    u32 sx0 = (x * 2) % w, sy0 = (y * 2) % h, sx1 = (x * 2 + 1) % w, sy1 = (y * 2 + 1) % h;
                    V3 a = col(sx0, sy0), b = col(sx1, sy0), c = col(sx0, sy1), d = col(sx1, sy1);
                    V3 avg = (a + b + c + d) * 0.25f;
                    size_t o = ((size_t) x + (size_t) y * hw) * 3;
                    ds[o] = avg.x; ds[o + 1] = avg.y; ds[o + 2] = avg.z;
                }
            delete[] img;
            img = ds;
            mi->w = ow = hw; mi->h = oh = hh;
        }
        float* nimg = nullptr;
        if (cfg.generate_normalmap_data) {   // lighter.cpp:977-1027
            struct Sum { V3 n; float mindot; i32 count; };
            Sum tmpl = {mk(0, 0, 0), 1, 1};
            std::vector<Sum> cs(mi->sloc.size(), tmpl);
            float amb = brightness(mk(cfg.ambient_color[0], cfg.ambient_color[1], cfg.ambient_color[2]));
            for (size_t i = 0; i < mi->snrm.size(); ++i) cs[i].n = mi->snrm[i] * amb;
            for (const Contrib& c : mi->contrib) { cs[c.sid].n += c.n; cs[c.sid].count++; }
            for (Sum& s : cs) s.n = s.n / (float) s.count;
            for (const Contrib& c : mi->contrib) {
                Sum& s = cs[c.sid];
                float d = fmax_(dot(normalized(s.n), normalized(c.n)), 0.0f);
                float t = fmin_(len(c.n) / len(s.n), 1.0f);
                d = 1.0f * (1.0f - t) + d * t;
                s.mindot *= d;
            }
            size_t cap = (size_t) ow * oh;
            nimg = new float[cap * 4];
            std::fill(nimg, nimg + cap * 4, 0.0f);
            for (size_t i = 0; i < mi->sloc.size(); ++i) {
                // With ds2x the reference indexes the half-size buffer with
                // full-size texel ids; writes past its end are dropped here.
                if (mi->sloc[i] >= cap) continue;
                V3 N = normalized(cs[i].n);
                size_t o = (size_t) mi->sloc[i] * 4;
                nimg[o] = N.x; nimg[o + 1] = N.y; nimg[o + 2] = N.z; nimg[o + 3] = cs[i].mindot;
            }
        }
        ltr_WorkOutput wo = {(u32) mid, mi->mesh->ident.c_str(), mi->mesh->ident.size(), mi->ident.c_str(),
                             mi->ident.size(), img, nimg, ow, oh};
        outputs.push_back(wo);
    }
}

// Stage order of Job_MainProc (lighter.cpp:1046-1145).
void ltr_Scene::run()
{
    g_watertight = opt_isect == 1;
    int nt = threads();
    stage = "transforming spatial data"; completion = 0;
    parallel_for(nt, insts.size(), [&](size_t i) { prexform(insts[i]); });
    stage = "generating data structures"; completion = 0;
    parallel_for(nt, insts.size(), [&](size_t i) { colinfo(insts[i]); });
    std::vector<Box> boxes;
    for (OInst* mi : insts) { const BVH::Node& N = mi->tree.bvh.nodes[0]; Box b = {N.mn, N.mx}; boxes.push_back(b); }
    inst_tree.build(boxes.data(), boxes.size());
    stage = "generating samples"; completion = 0;
    parallel_for(nt, insts.size(), [&](size_t i) { make_samples(insts[i]); });
    if (!lights.empty()) {
        stage = "rendering lightmaps"; completion = 0;
        for (OInst* mi : insts) mi->dbg_vis.assign(lights.size() * mi->lm.size(), -1.0f);
        for (size_t li = 0; li < lights.size(); ++li) {
            const OLight& L = lights[li];
            std::vector<i32> ids(1, 0);
            auto add = [&](const i32* p, i32 n) { for (i32 k = 0; k < n; ++k) ids.push_back(p[k]); };
            if (L.type == 1 || L.type == 2) {   // lighter.cpp:80-98
                V3 r3 = splat(L.range);
                inst_tree.box_query(L.pos - r3, L.pos + r3, add);
            } else if (L.type == 3) {
                inst_tree.all(add);
            }
            std::sort(ids.begin(), ids.end());
            i32 prev = -1;
            for (size_t k = 0; k < ids.size(); ++k) {
                if (k > 0 && ids[k] == prev) continue;
                prev = ids[k];
                render_light(L, insts[prev], li);
            }
            completion = (li + 1) / float(lights.size());
        }
    }
    if (cfg.bounce_count && opt_patches) {
        stage = "calculating radiosity"; completion = 0;
        rad_patches();
    } else if (cfg.bounce_count) {
        stage = "calculating radiosity"; completion = 0;
        rad_links();
        stage = "bouncing light"; completion = 0;
        for (int b = 0; b < cfg.bounce_count; ++b) { rad_bounce(); completion = (b + 1) / float(cfg.bounce_count); }
        stage = "committing radiosity";
        size_t sp = 0;
        for (OInst* mi : insts)
            for (auto& c : mi->lm) c = rad_col[sp++].total;
    }
    if (cfg.ao_distance) {
        stage = "rendering ambient occlusion"; completion = 0;
        for (size_t m = 0; m < insts.size(); ++m) {
            std::vector<float> ro(insts[m]->lm.size());
            for (auto& r : ro) r = randf();
            ao(insts[m], ro);
            completion = (m + 1) / float(insts.size());
        }
    }
    stage = "exporting lightmaps"; completion = 0;
    finalize();
    completion = 1;
    stage = nullptr;
}

ltr_Scene::ltr_Scene()
{
    ltr_GetConfig(&cfg, nullptr);
    OInst* c = new OInst;
    c->container = true;
    c->w = c->h = 0;
    insts.push_back(c);
}

ltr_Scene::~ltr_Scene()
{
    if (worker.joinable()) worker.join();
    for (OInst* mi : insts) delete mi;
    for (ltr_Mesh* m : meshes) delete m;
    for (auto& o : outputs) { delete[] o.lightmap_rgb; delete[] o.normals_xyzf; }
}

// ---------------------------------------------------------------- C API (lighter.cpp:7-28, 101-109, 1147-1357)
extern "C" {

API u32 ltr_NextPowerOfTwo(u32 x) { return next_pow2(x); }

API int ltr_DefaultSizeFunc(ltr_Config* config, const char*, size_t, const char*, size_t, float area, float imp,
                            u32* out)
{
    float size = config->global_size_factor * sqrtf(area) * imp;
    if (size < 1) size = 1;
    u32 s = next_pow2((u32) size);
    if (s > config->max_lightmap_size) return 0;
    out[0] = s; out[1] = s;
    return 1;
}

API void ltr_GetConfig(ltr_Config* cfg, ltr_Scene* opt)
{
    if (opt) { memcpy(cfg, &opt->cfg, sizeof(*cfg)); return; }
    memset(cfg, 0, sizeof(*cfg));
    cfg->size_fn = ltr_DefaultSizeFunc;
    cfg->max_num_threads = 0x7fff;
    cfg->max_tree_memory = 128 * 1024 * 1024;
    cfg->max_lightmap_size = 1024;
    cfg->default_width = 64;
    cfg->default_height = 64;
    cfg->global_size_factor = 4;
    cfg->max_correct_dist = 0.1f;
    cfg->max_correct_angle = 60;
    cfg->ao_multiplier = 1.2f;
    cfg->ao_falloff = 1;
    cfg->ao_num_samples = 17;
    cfg->blur_size = 0.5f;
}

API int ltr_SetConfig(ltr_Scene* s, ltr_Config* cfg) { memcpy(&s->cfg, cfg, sizeof(*cfg)); return 1; }
API ltr_Scene* ltr_CreateScene() { return new ltr_Scene; }
API void ltr_DestroyScene(ltr_Scene* s) { delete s; }

API void ltr_Start(ltr_Scene* s)
{
    g_shadow_evals = 0; g_distance_queries = 0; g_ao_rays = 0; g_rad_vis = 0;
    s->stage = "starting";
    s->worker = std::thread([s]() { s->run(); });
}
API void ltr_Abort(ltr_Scene*) {}
API int ltr_GetStatus(ltr_Scene* s, ltr_WorkStatus* ws)
{
    const char* st = s->stage.load();
    ws->completion = s->completion.load();
    ws->stage = st ? st : "finished";
    if (!st && s->worker.joinable()) s->worker.join();
    return st != nullptr;
}
API void ltr_Sleep(int ms) { std::this_thread::sleep_for(std::chrono::milliseconds(ms)); }

API ltr_Mesh* ltr_CreateMesh(ltr_Scene* s, const char* ident, size_t n)
{
    ltr_Mesh* m = new ltr_Mesh;
    m->scene = s;
    if (ident) m->ident.assign(ident, n);
    s->meshes.push_back(m);
    return m;
}

API int ltr_MeshAddPart(ltr_Mesh* m, ltr_MeshPartInfo* p)   // lighter.cpp:1226-1264
{
    OPart op = {p->vertex_count, (u32) m->pos.size(), p->index_count, (u32) m->idx.size(), p->shadow};
    if (p->index_count < 3 && p->index_count % 3 != 0) return 0;
    for (u32 i = 0; i < p->vertex_count; ++i) {
        V3 a, b; V2 t1, t2;
        memcpy(&a, (const char*) p->positions_f3 + (size_t) p->stride_positions * i, 12);
        memcpy(&b, (const char*) p->normals_f3 + (size_t) p->stride_normals * i, 12);
        memcpy(&t1, (const char*) p->texcoords1_f2 + (size_t) p->stride_texcoords1 * i, 8);
        memcpy(&t2, (const char*) p->texcoords2_f2 + (size_t) p->stride_texcoords2 * i, 8);
        m->pos.push_back(a); m->nrm.push_back(b); m->tex1.push_back(t1); m->tex2.push_back(t2);
    }
    m->idx.insert(m->idx.end(), p->indices, p->indices + p->index_count);
    m->parts.push_back(op);
    return 1;
}

API int ltr_MeshAddInstance(ltr_Mesh* m, ltr_MeshInstanceInfo* ii)
{
    OInst* mi = new OInst;
    mi->mesh = m;
    mi->importance = ii->importance;
    mi->shadow = !!ii->shadow;
    if (ii->ident) mi->ident.assign(ii->ident, ii->ident_size);
    memcpy(mi->matrix.m, ii->matrix, sizeof(float) * 16);
    m->scene->insts.push_back(mi);
    return 1;
}

API void ltr_LightAdd(ltr_Scene* s, ltr_LightInfo* li)   // lighter.cpp:1282-1317
{
    OLight L;
    L.type = li->type;
    L.pos = mk(li->position[0], li->position[1], li->position[2]);
    L.dir = normalized(mk(li->direction[0], li->direction[1], li->direction[2]));
    L.up = normalized(mk(li->up_direction[0], li->up_direction[1], li->up_direction[2]));
    L.color = mk(li->color_rgb[0], li->color_rgb[1], li->color_rgb[2]);
    L.range = li->range; L.power = li->power; L.radius = li->light_radius;
    L.nsamples = li->shadow_sample_count > 1 ? li->shadow_sample_count : 1;
    L.out = li->spot_angle_out; L.in = li->spot_angle_in; L.curve = li->spot_curve;
    L.randoff = randf();
    // Shadow samples, read only in the sampled shadow mode (orc_SetOptions).
    // Directional: lighter.cpp:1300-1310 (the spiral around -direction pulled
    // towards +direction). Point and spot: golden-angle disk points of radius
    // light_radius, the project's definition (the reference leaves a TODO).
    for (int k = 0; k < L.nsamples; ++k) {
        if (L.type == 3) {
            V3 adj = spiral_dir(-L.dir, L.randoff, k, L.nsamples);
            adj = normalized(adj + (-L.dir) * std::tan((L.radius - 0.5f) * (float) M_PI * 0.999f));
            L.smp.push_back(adj);
        } else {
            float rho = L.radius * std::sqrt((k + 0.5f) / L.nsamples);
            float phi = (k + L.randoff) * (137.508f / 180.0f * (float) M_PI);
            L.smp.push_back(mk(rho * std::cos(phi), rho * std::sin(phi), 0.0f));
        }
    }
    s->lights.push_back(L);
}

API void ltr_SampleAdd(ltr_Scene* s, ltr_SampleInfo* si)   // lighter.cpp:1319-1329
{
    ltr_SampleInfo c = *si;
    c.out_color[0] = c.out_color[1] = c.out_color[2] = 0;
    OInst* cont = s->insts[0];
    cont->spos.push_back(mk(c.position[0], c.position[1], c.position[2]));
    cont->snrm.push_back(mk(c.normal[0], c.normal[1], c.normal[2]));
    cont->lm.push_back(mk(0, 0, 0));
    s->samples.push_back(c);
}

API void ltr_GetWorkOutputInfo(ltr_Scene* s, ltr_WorkOutputInfo* o)
{
    o->lightmap_count = (u32) s->outputs.size();
    o->sample_count = (u32) s->samples.size();
    o->samples = s->samples.empty() ? nullptr : s->samples.data();
}

API int ltr_GetWorkOutput(ltr_Scene* s, u32 which, ltr_WorkOutput* o)
{
    if (which >= s->outputs.size()) return 0;
    *o = s->outputs[which];
    return 1;
}

// ---- introspection (same contract as the GPU library's)
API u32 ltrdbg_InstanceCount(ltr_Scene* s) { return (u32) s->insts.size(); }
API u32 ltrdbg_SampleCount(ltr_Scene* s, u32 i) { return i < s->insts.size() ? (u32) s->insts[i]->lm.size() : 0; }
API int ltrdbg_LightmapSize(ltr_Scene* s, u32 i, u32* wh)
{
    if (i >= s->insts.size()) return 0;
    wh[0] = s->insts[i]->w; wh[1] = s->insts[i]->h;
    return 1;
}
API int ltrdbg_GetSamples(ltr_Scene* s, u32 inst, float* pos3, float* nrm3, u32* loc, float* rad4, float* col3)
{
    if (inst >= s->insts.size()) return 0;
    OInst* mi = s->insts[inst];
    for (size_t i = 0; i < mi->lm.size(); ++i) {
        if (pos3 && i < mi->spos.size()) { pos3[i*3] = mi->spos[i].x; pos3[i*3+1] = mi->spos[i].y; pos3[i*3+2] = mi->spos[i].z; }
        if (nrm3 && i < mi->snrm.size()) { nrm3[i*3] = mi->snrm[i].x; nrm3[i*3+1] = mi->snrm[i].y; nrm3[i*3+2] = mi->snrm[i].z; }
        if (loc) loc[i] = i < mi->sloc.size() ? mi->sloc[i] : 0xffffffffu;
        if (rad4 && i < mi->srad.size()) { rad4[i*4] = mi->srad[i].x; rad4[i*4+1] = mi->srad[i].y; rad4[i*4+2] = mi->srad[i].z; rad4[i*4+3] = mi->srad[i].w; }
        if (col3) { col3[i*3] = mi->lm[i].x; col3[i*3+1] = mi->lm[i].y; col3[i*3+2] = mi->lm[i].z; }
    }
    return 1;
}
API u32 ltrdbg_RadLinkCount(ltr_Scene* s) { return (u32) s->links.size(); }

// Per-ray records of instance `inst`: vis (n_lights x n samples) and ao (n x ao_num_samples),
// either may be NULL; 0 when the bake recorded none.
API int ltrdbg_GetRayData(ltr_Scene* s, u32 inst, float* vis, float* ao)
{
    if (inst >= s->insts.size()) return 0;
    const OInst* mi = s->insts[inst];
    if (vis) {
        if (mi->dbg_vis.size() != s->lights.size() * mi->lm.size()) return 0;
        memcpy(vis, mi->dbg_vis.data(), mi->dbg_vis.size() * sizeof(float));
    }
    if (ao) {
        if (mi->dbg_ao.empty() && !mi->lm.empty()) return 0;
        memcpy(ao, mi->dbg_ao.data(), mi->dbg_ao.size() * sizeof(float));
    }
    return 1;
}

// The radiosity elements of the last bake (samples, or patches in patch mode)
// in the layout of the GPU library's ltrdbg_GetRadiosity: float4 position,
// unit normal, (diffuse rgb, area), emission and total; F (may be NULL) the
// n x n link factors (0 where two elements are not linked).
API int ltrdbg_GetRadiosity(ltr_Scene* s, u32* n, float* pos4, float* nrm4, float* diff_area4, float* emit4,
                            float* total4, float* F)
{
    const size_t N = s->rad_col.size();
    if (n) *n = (u32) N;
    if (!N) return 0;
    for (size_t i = 0; i < N; ++i) {
        const RadColors& c = s->rad_col[i];
        const float v[5][4] = {{s->rad_pos[i].x, s->rad_pos[i].y, s->rad_pos[i].z, 0},
                               {s->rad_nrm[i].x, s->rad_nrm[i].y, s->rad_nrm[i].z, 0},
                               {c.diff.x, c.diff.y, c.diff.z, c.area},
                               {s->rad_emit[i].x, s->rad_emit[i].y, s->rad_emit[i].z, 0},
                               {c.total.x, c.total.y, c.total.z, 0}};
        float* dst[5] = {pos4, nrm4, diff_area4, emit4, total4};
        for (int k = 0; k < 5; ++k)
            if (dst[k]) memcpy(dst[k] + 4 * i, v[k], sizeof(v[k]));
    }
    if (F) {
        memset(F, 0, N * N * sizeof(float));
        for (size_t i = 0; i < N && 2 * i + 1 < s->linkmap.size(); ++i) {
            size_t b = s->linkmap[2 * i], e = b + s->linkmap[2 * i + 1];
            for (size_t k = b; k < e; ++k) {
                size_t j = s->links[k].other;
                F[i * N + j] = F[j * N + i] = s->links[k].f;
            }
        }
    }
    return 1;
}

// Modes beyond the reference bake, matching the GPU library's ltrg_Options
// fields of the same names: v[0] shadow_mode, v[1] intersect_mode, v[2]
// radiosity_patches, v[3] radiosity_links (n of them given; the rest keep 0).
API void orc_SetOptions(ltr_Scene* s, const u32* v, u32 n)
{
    u32 o[4] = {0, 0, 0, 0};
    for (u32 k = 0; k < n && k < 4; ++k) o[k] = v[k];
    s->opt_shadow_mode = o[0];
    s->opt_isect = o[1];
    s->opt_patches = o[2];
    s->opt_links = o[3];
}

// out[0..3] = shadow evaluations, sphere-trace steps, AO rays, radiosity visibility tests
API void orc_GetCounters(unsigned long long* out)
{
    out[0] = g_shadow_evals; out[1] = g_distance_queries; out[2] = g_ao_rays; out[3] = g_rad_vis;
}

// Form factors of a patch set, for checking the multi-right-hand-side gather:
// the reference's pair test and factor (lighter.cpp:733-757) and its
// VisibilityTest (lighter.cpp:138-147: segment shrunk by SMALL_FLOAT at both
// ends, any hit in the triangle tree, lighter_math.cpp:804-832) over one tree
// of all triangles (9 floats each). G_ij = f_ij * area_j for pairs that pass
// the predicate (links 0: occluded, as the reference; 1: unoccluded), else 0.
API void orc_gather_form_factors(const float* tri9, u32 n_tris, const float* pos3, const float* nrm3,
                                 const float* area, u32 n, int links, float* G, int threads)
{
    std::vector<Tri> tris(n_tris);
    for (u32 t = 0; t < n_tris; ++t) {
        const float* q = tri9 + 9 * (size_t) t;
        tris[t].P1 = mk(q[0], q[1], q[2]);
        tris[t].P2 = mk(q[3], q[4], q[5]);
        tris[t].P3 = mk(q[6], q[7], q[8]);
    }
    TriTree tree;
    tree.set(tris.data(), tris.size());
    std::vector<V3> P(n), N(n);
    for (u32 i = 0; i < n; ++i) {
        P[i] = mk(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]);
        N[i] = normalized(mk(nrm3[3 * i], nrm3[3 * i + 1], nrm3[3 * i + 2]));
    }
    memset(G, 0, sizeof(float) * (size_t) n * n);
    parallel_for(threads, n, [&](size_t i) {
        V3 AP = P[i], AN = N[i];
        for (size_t j = i + 1; j < n; ++j) {
            V3 BP = P[j], BN = N[j];
            V3 pd = BP - AP;
            float dA = dot(AN, pd), dB = dot(BN, -pd);
            if (dA <= kSmall || dB <= kSmall) continue;
            float l2 = lensq(pd);
            float f = dA * dB / (l2 * l2 * (float) M_PI);
            if (f < kSmall) continue;
            V3 dn = normalized(BP - AP);
            bool occ = tree.any_hit(AP + dn * kSmall, BP - dn * kSmall);
            if ((links == 0) != occ) continue;
            G[i * n + j] = f * area[j];
            G[j * n + i] = f * area[i];
        }
    });
}

struct ltrg_SampleTable { u32 count; const float* diffuse_rgb; const float* emissive_rgb; };
API int ltrg_TableSampleFn(ltr_Config* cfg, ltr_SampleRequest* req)
{
    const ltrg_SampleTable* t = (const ltrg_SampleTable*) cfg->userdata;
    if (!t) return 0;
    float fid = req->tex0u;
    if (!(fid >= 0.0f)) return 0;
    u32 id = (u32) fid;
    if (id >= t->count) return 0;
    if (t->diffuse_rgb) for (int c = 0; c < 3; ++c) req->out_diffuse_color[c] = t->diffuse_rgb[id * 3 + c];
    if (t->emissive_rgb) for (int c = 0; c < 3; ++c) req->out_emissive_color[c] = t->emissive_rgb[id * 3 + c];
    return 1;
}

}  // extern "C"
