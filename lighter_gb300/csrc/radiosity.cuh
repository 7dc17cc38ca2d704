// Radiosity over the bake's samples (Int_RDGenLinks / Int_RDBounce,
// lighter.cpp:667-797) as a dense form-factor matrix on the GPU.
//
// The reference stores sparse symmetric links (j, f) for i < j and sweeps
// them once per bounce; here F is an N x N matrix in HBM (FP32, FP16 or BF16)
// whose (i, j) entry is the link factor or 0, so one bounce is
//   X_j = out_j * diffuse_j * area_j,   Y = F X,   total += Y,   out = Y
// with X and Y holding RGB. After n bounces `total` = sum_{m=0..n} K^m E with
// K_ij = F_ij area_j diffuse_j, the reference's result up to summation order.
#pragma once

#include <atomic>
#include <cstdint>
#include <vector>

#include "bvh.cuh"

namespace lg {

struct RadInputs {
    uint32_t n = 0;
    std::vector<float4> pos, nrm;   // unit normals
    std::vector<float4> diff_area;  // diffuse rgb, patch area
    std::vector<float4> emit;       // emitted rgb (direct light + sample_fn emission)
};

struct RadSettings {
    int links = 0;        // LTRG_LINKS_*
    int precision = 0;    // LTRG_F_*
    int refine_steps = 1;  // 16-bit F: the last refine_steps bounces recompute the factors in FP32
    int bounces = 1;
    float* f_host = nullptr;   // debug: receives F as n x n floats (the stored values, widened)
};

struct RadResult {
    uint64_t links = 0, pairs = 0, vis_rays = 0;
    double ms_links = 0, ms_bounce = 0;
};

// Inputs already on the device (same meaning as RadInputs).
struct RadDevInputs {
    uint32_t n;
    const float4* pos;
    const float4* nrm;
    const float4* diff_area;
    const float4* emit;
};

// Builds F, runs the bounces and writes `total` (float4 per element) to
// total_out, which may alias in.emit.
RadResult radiosity_solve_dev(const RadDevInputs& in, const RadSettings& rs, const BvhView& bvh, ErrFlag err,
                              cudaStream_t st, float4* total_out, std::atomic<bool>* abort_flag);

// Only the form factors: F (n x n FP32, row-major) with the pair test and the
// `links` predicate, in two passes (pair tests, then the visibility rays of the
// pairs that passed); returns the link and visibility-ray counts (synchronises
// the stream).
struct RadFormFactors {
    uint64_t links = 0, vis_rays = 0;
};
RadFormFactors radiosity_form_factors_f32(uint32_t n, const float4* pos, const float4* nrm, const BvhView& bvh,
                                          ErrFlag err, int links, float* F, cudaStream_t st);

// Same from host vectors (uploads them first).
RadResult radiosity_solve(const RadInputs& in, const RadSettings& rs, const BvhView& bvh, ErrFlag err, cudaStream_t st,
                          float4* lm_out, std::atomic<bool>* abort_flag);

}  // namespace lg
