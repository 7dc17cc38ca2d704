// Shared host/device math of the GB300 baker.
//
// The float expressions keep the operation order of archo5/lighter's math
// (lighter_int.hpp:261-557, lighter_math.cpp:150-354, 875-952). The library is
// built with --fmad=false and IEEE division/sqrt, so every stage that uses
// only + - * / sqrt reproduces the CPU bake bit for bit; stages that call
// powf/acosf/sinf/cosf differ by CUDA's ulp-level error in those functions.
#pragma once

#include <cstdint>
#include <cmath>
#include <cfloat>

#ifdef __CUDACC__
#define HD __host__ __device__ __forceinline__
#else
#define HD inline
#endif

namespace lg {

typedef uint32_t u32;
typedef int32_t i32;

constexpr float kSmall = 0.001f;          // SMALL_FLOAT, lighter_int.hpp:261
constexpr float kMaxPenumbraSize = 2.0f;  // lighter_int.hpp:964
constexpr float kMaxPenumbraStep = 1.0f;  // lighter_int.hpp:966
constexpr float kShadowOffset = 0.005f;   // lighter_int.hpp:967
constexpr float kNoHit = 2.0f;            // "no hit" fraction of the segment queries

struct V2 { float x, y; };
struct V3 { float x, y, z; };

HD V3 mk(float x, float y, float z) { V3 v = {x, y, z}; return v; }
HD V3 splat(float f) { return mk(f, f, f); }
HD V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
HD V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
HD V3 operator*(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
HD V3 operator*(V3 a, float f) { return mk(a.x * f, a.y * f, a.z * f); }
HD V3 operator*(float f, V3 a) { return mk(f * a.x, f * a.y, f * a.z); }
HD V3 operator/(V3 a, float f) { return mk(a.x / f, a.y / f, a.z / f); }
HD V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
HD V3& operator+=(V3& a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HD V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
HD float lensq(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
HD float len(V3 a) { return sqrtf(lensq(a)); }
HD V3 normalized(V3 a)
{
    float l = lensq(a);
    if (l == 0) return mk(0, 0, 0);
    float inv = 1.0f / sqrtf(l);
    return mk(a.x * inv, a.y * inv, a.z * inv);
}
HD bool near_zero(V3 a) { return fabsf(a.x) < kSmall && fabsf(a.y) < kSmall && fabsf(a.z) < kSmall; }
HD bool is_zero(V3 a) { return a.x == 0 && a.y == 0 && a.z == 0; }
HD float fmin_(float a, float b) { return a < b ? a : b; }   // TMIN, lighter_int.hpp:277
HD float fmax_(float a, float b) { return a > b ? a : b; }   // TMAX, lighter_int.hpp:278
HD V3 vmin(V3 a, V3 b) { return mk(fmin_(a.x, b.x), fmin_(a.y, b.y), fmin_(a.z, b.z)); }
HD V3 vmax(V3 a, V3 b) { return mk(fmax_(a.x, b.x), fmax_(a.y, b.y), fmax_(a.z, b.z)); }
HD V3 lerp3(V3 a, V3 b, float s) { return a * (1.0f - s) + b * s; }   // TLERP, lighter_int.hpp:285
HD float brightness(V3 c) { return (c.x + c.y + c.z) * (1.0f / 3.0f); }  // lighter_int.hpp:926

HD V2 mk2(float x, float y) { V2 v = {x, y}; return v; }
HD V2 operator-(V2 a, V2 b) { return mk2(a.x - b.x, a.y - b.y); }
HD float cross2(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
HD float dot2(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
HD float len2(V2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
HD V2 normalized2(V2 a)
{
    float l = a.x * a.x + a.y * a.y;
    if (l == 0) return mk2(0, 0);
    float inv = 1.0f / sqrtf(l);
    return mk2(a.x * inv, a.y * inv);
}

#ifdef __CUDACC__
HD V3 ld3(const float4& f) { return mk(f.x, f.y, f.z); }
HD float4 st4(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
#endif

// Heron's formula (lighter_math.cpp:150-181).
HD float heron(float a, float b, float c)
{
    float p = (a + b + c) * 0.5f;
    float pre = p * (p - a) * (p - b) * (p - c);
    if (pre < 0) return 0;
    return sqrtf(pre);
}
HD float tri_area3(V3 p1, V3 p2, V3 p3) { return heron(len(p2 - p1), len(p3 - p2), len(p1 - p3)); }
HD float tri_area2(V2 p1, V2 p2, V2 p3) { return heron(len2(p2 - p1), len2(p3 - p2), len2(p1 - p3)); }

// Segment L1->L2 against a triangle: fraction r in [0,1] or kNoHit. The epsilon
// on n.dir is absolute, not scale-invariant (lighter_math.cpp:315-354).
HD float seg_tri(V3 L1, V3 L2, V3 P1, V3 P2, V3 P3)
{
    V3 u = P2 - P1, v = P3 - P1;
    V3 n = cross(u, v);
    if (near_zero(n)) return kNoHit;
    V3 dir = L2 - L1, w0 = L1 - P1;
    float a = -dot(n, w0);
    float b = dot(n, dir);
    if (fabsf(b) < kSmall) return kNoHit;
    float r = a / b;
    if (r < 0.0f || r > 1.0f) return kNoHit;
    V3 I = L1 + r * dir;
    float uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
    V3 w = I - P1;
    float wu = dot(w, u), wv = dot(w, v);
    float D = uv * uv - uu * vv;
    float s = (uv * wv - vv * wu) / D;
    if (s < 0.0f || s > 1.0f) return kNoHit;
    float t = (uv * wu - uu * wv) / D;
    if (t < 0.0f || (s + t) > 1.0f) return kNoHit;
    return r;
}

// Watertight segment/triangle test (Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013), the LTRG_ISECT_WATERTIGHT
// alternative to seg_tri. The triangle is moved to the segment's start,
// sheared and scaled so that the segment runs along +z over [0, 1], and the
// signs of the three 2D edge functions U, V, W decide inclusion. An edge
// function that comes out exactly 0 in FP32 is recomputed from the same FP32
// coordinates in FP64, where the two products are exact, so its sign is the
// exact one: a segment through an edge or vertex shared by two triangles hits
// at least one of them. Both windings count; a degenerate projection (U + V +
// W = 0) misses. Returns the fraction r in [0, 1] along L1 -> L2, or kNoHit.
HD float wt_comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

HD float seg_tri_wt(V3 L1, V3 L2, V3 P1, V3 P2, V3 P3)
{
    V3 D = L2 - L1;
    const float ax = fabsf(D.x), ay = fabsf(D.y), az = fabsf(D.z);
    const int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    const float dz = wt_comp(D, kz);
    if (dz == 0.0f) return kNoHit;   // zero-length segment
    if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }   // keep the winding of the projection
    const float Sx = wt_comp(D, kx) / dz, Sy = wt_comp(D, ky) / dz, Sz = 1.0f / dz;
    const V3 A = P1 - L1, B = P2 - L1, C = P3 - L1;
    const float Ax = wt_comp(A, kx) - Sx * wt_comp(A, kz), Ay = wt_comp(A, ky) - Sy * wt_comp(A, kz);
    const float Bx = wt_comp(B, kx) - Sx * wt_comp(B, kz), By = wt_comp(B, ky) - Sy * wt_comp(B, kz);
    const float Cx = wt_comp(C, kx) - Sx * wt_comp(C, kz), Cy = wt_comp(C, ky) - Sy * wt_comp(C, kz);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float) ((double) Cx * (double) By - (double) Cy * (double) Bx);
        V = (float) ((double) Ax * (double) Cy - (double) Ay * (double) Cx);
        W = (float) ((double) Bx * (double) Ay - (double) By * (double) Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return kNoHit;
    const float det = U + V + W;
    if (det == 0.0f) return kNoHit;
    const float Az = Sz * wt_comp(A, kz), Bz = Sz * wt_comp(B, kz), Cz = Sz * wt_comp(C, kz);
    const float T = U * Az + V * Bz + W * Cz;
    if (det > 0.0f ? (T < 0.0f || T > det) : (T > 0.0f || T < det)) return kNoHit;
    return T / det;   // |T| <= |det| with equal signs: the rounded quotient stays in [0, 1]
}

// Unsigned point/triangle distance by corner, edge and face regions
// (lighter_math.cpp:875-913).
HD float point_tri_dist(V3 pt, V3 t0, V3 t1, V3 t2)
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

// Projection of a point falls inside the triangle, with SMALL_FLOAT slack
// (lighter_math.cpp:915-952).
HD bool point_proj_on_tri(V3 pt, V3 t0, V3 t1, V3 t2)
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

// Reverse-winding unit normal, Triangle::GetNormal (lighter_int.hpp:614-617).
HD V3 tri_normal_rev(V3 P1, V3 P2, V3 P3) { return normalized(cross(P3 - P1, P2 - P1)); }

// Host-side bookkeeping of one bake (the calling thread's): kernels this
// library launched and bytes it copied between host and device.
struct HostCounters {
    uint64_t launches = 0, h2d = 0, d2h = 0;
};
HostCounters& host_counters();
inline void note_launch() { host_counters().launches++; }
inline void note_h2d(size_t b) { host_counters().h2d += b; }
inline void note_d2h(size_t b) { host_counters().d2h += b; }


}  // namespace lg
