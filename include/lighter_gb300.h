/*
 * lighter_gb300.h -- GPU extensions of the lighter C ABI (liblighter_gb300.so).
 *
 * Everything here is additive: an application that only uses lighter.h gets
 * the reference behaviour. The extensions select the CUDA device, opt into
 * the physically-based radiosity link predicate and the mixed-precision
 * gather, expose per-stage timings and counters, batch many scenes into one
 * bake, and provide read-only introspection used by the parity tests.
 */
#pragma once

#include "lighter.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Radiosity link predicate. The reference keeps a pair only when
 * ltr_Scene::VisibilityTest reports an occluder between the two samples
 * (lighter.cpp:751, `VisibilityTest(...) == false` skips unoccluded pairs). */
#define LTRG_LINKS_REFERENCE 0   /* link occluded pairs, as lighter.cpp:751 */
#define LTRG_LINKS_VISIBLE   1   /* link mutually visible pairs */

/* Storage type of the dense form-factor matrix F used by the gather. */
#define LTRG_F_FP32 0
#define LTRG_F_FP16 1
#define LTRG_F_BF16 2

/* How the direct lights' shadows are evaluated (ltrg_Options.shadow_mode). */
#define LTRG_SHADOW_SPHERE  0   /* the reference's sphere-traced soft-shadow factor per (sample, light)
                                   (CalcInvShadowFactor, lighter.cpp:190-207); light_radius is its
                                   penumbra factor and shadow_sample_count is not read */
#define LTRG_SHADOW_SAMPLED 1   /* shadow_sample_count visibility rays per (sample, light); the shadow
                                   factor is the fraction of them that reach the light. Directional
                                   lights: the ray directions of the reference's disabled sampled
                                   block (lighter.cpp:566-584), i.e. the spiral drawn by ltr_LightAdd
                                   (lighter.cpp:1295-1312), traced from the sample position over
                                   `range`, with N.L averaged over the directions. Point and spot
                                   lights (no reference code): the rays end on a disk of radius
                                   light_radius around the light, facing the sample, at golden-angle
                                   spiral points rho = radius * sqrt((s + 0.5) / n), phi = (s +
                                   randoff) * 137.508 deg, randoff being the light's rand() draw */

/* Segment/triangle test of every ray query (ltrg_Options.intersect_mode). */
#define LTRG_ISECT_REFERENCE  0  /* IntersectLineSegmentTriangle (lighter_math.cpp:315-354) */
#define LTRG_ISECT_WATERTIGHT 1  /* watertight test (shear to the ray's dominant axis, edge functions
                                    with a double-precision retry on exact zeros): no ray passes
                                    between two triangles that share an edge */

/* Scene BVH builders. */
#define LTRG_BVH_PLOC  0   /* locally-ordered clustering over the Morton order (closer to a SAH tree) */
#define LTRG_BVH_RADIX 1   /* Karras' radix-tree hierarchy over the Morton order (faster build) */

typedef struct ltrg_Options {
    int device;               /* CUDA device ordinal, default 0 */
    int keep_samples;         /* keep per-sample arrays for ltrdbg_* after the bake, default 0 */
    int radiosity_links;      /* LTRG_LINKS_*, default LTRG_LINKS_REFERENCE */
    int radiosity_precision;  /* LTRG_F_*, default LTRG_F_FP32 */
    int refine_steps;         /* FP16/BF16 F: the last refine_steps bounces use F only as the link
                                 mask and recompute each factor in FP32 (the FP32 result of those
                                 bounces, bit for bit); default 1, 0..16 */
    uint32_t radiosity_patches; /* 0: one radiosity element per sample (reference, lighter.cpp:673-719);
                                   N > 0: group samples into about N patches by (instance, lightmap
                                   tile, dominant normal axis); each texel then receives its patch's
                                   gathered (bounced) light on top of its own direct light */
    uint32_t bvh_builder;     /* LTRG_BVH_*: how the scene BVH is built; results do not depend on it,
                                 only the trace times do. Default LTRG_BVH_PLOC */
    uint32_t shadow_mode;     /* LTRG_SHADOW_*, default LTRG_SHADOW_SPHERE */
    uint32_t intersect_mode;  /* LTRG_ISECT_*, default LTRG_ISECT_REFERENCE */
    uint32_t encode_rgbe;     /* 1: the bake also encodes every lightmap as Radiance RGBE (4 bytes
                                 per texel, Ward's shared exponent) on the GPU after the finalize
                                 stage; read with ltrg_GetWorkOutputRGBE. Default 0 */
    uint32_t reserved[6];
} ltrg_Options;

/* Per-stage device times (CUDA events on the bake stream) and work counters
 * of the last finished bake. */
typedef struct ltrg_Stats {
    double ms_total;          /* host wall time from ltr_Start to finished */
    double ms_upload;         /* host->device copies of the scene */
    double ms_bvh;            /* BVH build */
    double ms_samples;        /* raster, compaction, offset and correction */
    double ms_direct;         /* direct light */
    double ms_rad_links;      /* form factors and their visibility rays */
    double ms_rad_bounce;     /* all bounces */
    double ms_ao;             /* ambient occlusion */
    double ms_finalize;       /* scatter, dilate, blur, ds2x, normal data */
    double ms_download;       /* device->host copies of the outputs */
    uint64_t texels;          /* lightmap texels rasterised */
    uint64_t samples;         /* covered texels + probe samples */
    uint64_t triangles;       /* shadow-casting triangles in the BVH */
    uint64_t shadow_evals;    /* shadow evaluations traced: one per (sample, light) pair, or one per
                                 (sample, light, shadow sample) ray with LTRG_SHADOW_SAMPLED */
    uint64_t distance_queries;/* sphere-trace steps (nearest-triangle queries) */
    uint64_t ao_rays;         /* AO segment queries */
    uint64_t rad_pairs;       /* radiosity pairs i<j examined */
    uint64_t rad_vis_rays;    /* pairs that passed the facing/form-factor tests */
    uint64_t node_visits;     /* BVH internal nodes fetched by the direct-light distance queries (a
                                 walk shared by a warp, ltrg_Tuning.direct_packet, counts a node once) */
    uint64_t tri_tests;       /* leaf triangles fetched for their point/triangle distance (likewise) */
    uint64_t rad_elements;    /* radiosity elements: samples, or patches in patch mode */
    uint64_t kernel_launches; /* CUDA kernels this library launched for the bake */
    uint64_t bytes_h2d;       /* host->device bytes copied for the bake */
    uint64_t bytes_d2h;       /* device->host bytes copied for the bake */
    double ms_device;         /* device time from the first kernel to the last (CUDA events) */
    double ms_direct_trace;   /* the shadow-trace kernel alone (CUDA events around its launch; 0 when
                                 the scene's pairs were traced in a batch launch) */
    double ms_ao_trace;       /* the AO-ray kernel alone (0 when traced in a batch launch) */
    uint64_t shadow_pairs;    /* (sample, light) pairs traced */
    uint64_t reserved[1];
} ltrg_Stats;

/* Options are read at ltr_Start; returns 0 on an invalid value. */
LTRAPI void ltrg_GetOptions(ltr_Scene* scene, ltrg_Options* out);
LTRAPI LTRBOOL ltrg_SetOptions(ltr_Scene* scene, const ltrg_Options* opt);
/* The RGBE encoding of work output `which` (ltrg_Options::encode_rgbe): w x h
 * pixels of 4 bytes (R, G, B mantissas, exponent + 128), rows as the float
 * image's; scene-owned, valid until the next bake or ltr_DestroyScene. Returns
 * 0 when the last bake did not encode. */
LTRAPI LTRBOOL ltrg_GetWorkOutputRGBE(ltr_Scene* scene, u32 which, const unsigned char** rgbe);
LTRAPI LTRBOOL ltrg_GetStats(ltr_Scene* scene, ltrg_Stats* out);
/* Text of the error that ended the last bake, or NULL. */
LTRAPI const char* ltrg_LastError(ltr_Scene* scene);
/* Blocks until the bake started by ltr_Start has finished; returns 1 on success. */
LTRAPI LTRBOOL ltrg_Wait(ltr_Scene* scene);

/* Table-driven sample_fn: config->userdata points at an ltrg_SampleTable and
 * the entry is chosen by (u32) request->tex0u, i.e. the mesh's first UV channel
 * carries a face id. Entries out of range keep the defaults (returns 0). */
typedef struct ltrg_SampleTable {
    u32 count;
    const float* diffuse_rgb;    /* count x 3, may be NULL */
    const float* emissive_rgb;   /* count x 3, may be NULL */
} ltrg_SampleTable;
LTRAPI LTRBOOL ltrg_TableSampleFn(ltr_Config* config, ltr_SampleRequest* req);

/* Lightmap finishing that allocates no device memory. No counterpart in the
 * reference: it exposes the bake's finalize step (three extrapolating dilation
 * sweeps, then the separable Gaussian blur; lighter.cpp:880-961) for callers
 * that cannot call cudaMalloc where they finish a lightmap -- code running
 * inside a CUDA stream capture, plugins whose host owns all device memory,
 * per-frame callbacks that must not synchronise the device.
 *   rgb    device, width*height*3 floats: the scattered sample colours
 *   mask   device, width*height bytes: nonzero where a sample was written
 *   out    device, width*height*3 floats: the finished lightmap (may equal rgb)
 *   stream cudaStream_t to enqueue on (NULL = default stream); the call does
 *          not wait for the GPU
 * Limits: width*height <= LTRG_NOALLOC_MAX_TEXELS (1024 x 1024) and
 * ceil(blur_size) <= 16. The scratch is one static device array of
 * LTRG_NOALLOC_SCRATCH_BYTES held by every GPU that loads the library until
 * exit. A call on a stream that is not being captured looks up the array's
 * device address for the current device and CUDA context; a call under stream
 * capture reuses the address remembered for that device and context, so make
 * the first call in each context (per device, and again after a
 * cudaDeviceReset) before any stream capture. Calls share the scratch: calls
 * that overlap on the GPU race and must be serialised by the caller.
 * Returns LTRG_NOALLOC_OK or a negative LTRG_NOALLOC_E* code. */
#define LTRG_NOALLOC_MAX_TEXELS (1u << 20)
#define LTRG_NOALLOC_SCRATCH_BYTES (2u * LTRG_NOALLOC_MAX_TEXELS + 12u * LTRG_NOALLOC_MAX_TEXELS)
#define LTRG_NOALLOC_OK 0
#define LTRG_NOALLOC_EINVAL (-1)   /* null pointer, zero size or blur_size out of range */
#define LTRG_NOALLOC_ETOOBIG (-2)  /* width*height above LTRG_NOALLOC_MAX_TEXELS */
#define LTRG_NOALLOC_ECUDA (-3)    /* no current device, symbol lookup or launch failed */
LTRAPI int ltrg_FinalizeLightmapNoAlloc(const float* rgb, const unsigned char* mask, float* out, u32 width,
                                        u32 height, float blur_size, void* stream);

/* Multi-right-hand-side radiosity gather. The reference runs its bounces
 * (Int_RDBounce, lighter.cpp:767-797) for one light configuration at a time,
 * over sparse links; here the form factors of a patch set are built once as
 * a dense matrix and many light configurations are bounced together:
 *   B_0 = E,  B_k = E + K B_{k-1},  K_ij = F_ij * area_j * albedo_j(c)
 * for R right-hand sides (column r uses albedo channel c = r mod 3, so R =
 * 3 x configurations for RGB). F_ij is the reference's pair factor
 * (lighter.cpp:733-757) for pairs that pass the link predicate, 0 elsewhere.
 *
 * ltrg_GatherCreate traces the visibility rays and keeps G_ij = F_ij * area_j
 * in FP32 on the device.
 *   tri_xyz  n_tris x 9 floats: occluders (world space)
 *   pos3, nrm3, area  per patch (normals need not be unit length)
 *   links    LTRG_LINKS_*
 * Returns NULL on error (message on stderr). */
typedef struct ltrg_Gather ltrg_Gather;

/* Contraction of one bounce for FP16/BF16 storage (ignored for FP32). Both
 * operands are scaled by exact powers of two (G's peak near 2^14, the
 * emission peak at 2^9) so that FP16 keeps small values out of its subnormal
 * range; the scaling is undone in FP32.
 *   LTRG_REFINE_NONE   G16 x X16, one tensor-core product
 *   LTRG_REFINE_RHS    X split into a 16-bit head and tail (two products), so
 *                      only G's own rounding remains
 *   LTRG_REFINE_FULL   also G's rounding residual G - G16, kept as a second
 *                      16-bit matrix, contracted with the head and added in
 *                      FP32 (three products; about 2^-16 relative per entry
 *                      for BF16 and 2^-22 for FP16) */
#define LTRG_REFINE_NONE 0
#define LTRG_REFINE_RHS  1
#define LTRG_REFINE_FULL 2

typedef struct ltrg_GatherStats {
    double ms_build;        /* form factors (pair tests + visibility rays), CUDA events */
    double ms_convert;      /* FP32 -> 16-bit copies of G made by this solve (0 when cached) */
    double ms_bounces;      /* all bounces, CUDA events */
    double ms_per_bounce;   /* ms_bounces / bounces */
    double ms_gemm;         /* contraction kernels only, summed over the bounces */
    double flops_per_bounce;     /* 2 n^2 R per product issued */
    uint64_t bytes_per_bounce;   /* bytes of G (and residual) streamed per bounce */
    uint64_t links, vis_rays, pairs;
    int32_t tensor_cores;   /* 1 when the tcgen05 path ran */
    int32_t stages, ctas, products;
    uint32_t reserved[8];
} ltrg_GatherStats;

LTRAPI ltrg_Gather* ltrg_GatherCreate(const float* tri_xyz, u32 n_tris, const float* pos3, const float* nrm3,
                                      const float* area, u32 n, int links, int device);
LTRAPI void ltrg_GatherDestroy(ltrg_Gather* g);
/* Accumulation length of the tensor-core path: the FP32 accumulator in TMEM
 * takes k_blocks x 64 products per row before it is added (round to nearest)
 * into the FP32 workspace and restarted. The tensor cores' own accumulation
 * drifts by a small systematic amount per step (about 1e-5 relative after
 * 32k products), which this bounds at the cost of workspace traffic. 0: no
 * limit (default). */
LTRAPI LTRBOOL ltrg_GatherSetChunk(ltrg_Gather* g, u32 k_blocks);
LTRAPI u32 ltrg_GatherSize(ltrg_Gather* g);
/* Copies G (n x n FP32, row-major) to host memory. */
LTRAPI LTRBOOL ltrg_GatherGetG(ltrg_Gather* g, float* out);
LTRAPI const char* ltrg_GatherLastError(ltrg_Gather* g);
/* Test hook for the bounded waits of the tensor-core gather: in the next FP16
 * or BF16 solve of `g`, the kernel's copy producer issues no copies and every
 * mbarrier wait gives up after about wait_us microseconds (instead of about
 * 2 s). The waits expire, the kernel records the expiry in its error word,
 * waits for its own products, frees its tensor memory and returns; that solve
 * fails with the error word in ltrg_GatherLastError, and later solves run
 * normally. No GPU fault or hang is involved. wait_us in 1..2000000. */
LTRAPI LTRBOOL ltrdbg_GatherStallNextSolve(ltrg_Gather* g, u32 wait_us);
/* Test hook for the bounded waits of the bake's radiosity bounce: in the next
 * bounce over an unrefined F (any bake of this process), the copy producer
 * issues nothing and every mbarrier wait gives up after about wait_us
 * microseconds (instead of about 2 s). The waits expire, the kernel records
 * bit 1 in the radiosity stage's error word and returns; that bake fails with
 * the error word in ltrg_LastError, and later bakes run normally. No GPU
 * fault or hang is involved. wait_us in 1..2000000. */
LTRAPI LTRBOOL ltrdbg_RadiosityStallNextBounce(u32 wait_us);
/* How ltrg_GatherSolve moves its host buffers (test and measurement hook).
 * mode 0: by device (the default): where kernels may address pageable host
 * memory (cudaDevAttrPageableMemoryAccess, e.g. Grace systems), copy kernels
 * read the inputs and write the result over the CPU-GPU link; elsewhere the
 * buffers go through page-locked staging filled by host threads. mode 1: the
 * staging always; mode 2: the copy kernels (returns 0 where the device
 * cannot address pageable memory). The results are the same. */
LTRAPI LTRBOOL ltrdbg_GatherHostPath(ltrg_Gather* g, int mode);
/* The path the next ltrg_GatherSolve takes: 1 staged, 2 direct. */
LTRAPI int ltrdbg_GatherHostPathUsed(ltrg_Gather* g);
/* B after `bounces` sweeps for R right-hand sides; host buffers:
 *   albedo_rgb n x 3, emission n x R, out n x R (row-major).
 * precision LTRG_F_*, refine LTRG_REFINE_*; for FP16/BF16 R <= 256.
 * Returns 1, or 0 with ltrg_GatherLastError set. */
LTRAPI LTRBOOL ltrg_GatherSolve(ltrg_Gather* g, const float* albedo_rgb, const float* emission, u32 R, int bounces,
                                int precision, int refine, float* out, ltrg_GatherStats* stats);
/* Same on device buffers of the gather's device, enqueued on `stream` (NULL:
 * the gather's own stream) and completed before return. */
LTRAPI LTRBOOL ltrg_GatherSolveDevice(ltrg_Gather* g, const float* albedo_rgb, const float* emission, u32 R,
                                      int bounces, int precision, int refine, float* out, ltrg_GatherStats* stats,
                                      void* stream);

/* Bakes `count` scenes as one batch. Each scene bakes as if ltr_Start had
 * been called on it (same outputs, status and ltrg_Wait), but the direct-light
 * shadow traces and the AO rays of all scenes run in one persistent kernel
 * launch each, so many small scenes fill the GPU together. The scenes' AO
 * rand() draws are taken in array order, as bakes run one after another in
 * that order would take them. All scenes must use the same device and none
 * may be running; returns 0 (starting nothing) otherwise. No counterpart in
 * the reference, which bakes one scene per ltr_Start. */
LTRAPI LTRBOOL ltrg_StartBatch(ltr_Scene** scenes, u32 count);

/* Launch shapes of the persistent trace kernels, per CUDA device. Results do
 * not depend on them (every pair and ray is traced by the same function
 * whatever thread takes it); only the time does. */
typedef struct ltrg_Tuning {
    u32 direct_block;         /* threads per block of the shadow-trace kernel, default 128 */
    u32 direct_blocks_per_sm; /* persistent blocks per SM, default 8 */
    u32 ao_block;             /* threads per block of the AO-ray kernel, default 128 */
    u32 ao_blocks_per_sm;     /* default 16 */
    u32 direct_order;         /* order in which the warps take the shadow-trace pairs of a light:
                                 0 = sample order, 1 = by lightmap texel (Morton order per instance),
                                 2 = by position (3D Morton order in the scene bounds); default 2 */
    u32 ao_order;             /* the same for the AO rays; default 1 */
    u32 direct_regs;          /* register budget of the shadow-trace kernel for sphere-traced shadows:
                                 0 = as compiled (at most 128), 1 = 64, 2 = 72, 3 = 80 per thread (more
                                 warps per SM, some spills); default 0 */
    u32 direct_stack;         /* traversal-stack entries per thread kept in shared memory by the
                                 shadow-trace kernel's per-lane walks with register budget 0 or 1
                                 (0, 4, 8 or 16; deeper entries stay in local memory); default 0 */
    u32 ao_stack;             /* the same for the AO-ray kernel; default 0 */
    u32 ao_chunk;             /* AO wavefront: rays per lane per work fetch of a warp (1..8; a warp
                                 takes 32 x ao_chunk rays); default 1 */
    u32 direct_packet;        /* 1: the shadow traces of a warp's 32 pairs share each BVH walk (one
                                 walk for the union of the lanes' query spheres or shadow rays, every
                                 lane keeping its own radius or segment and result); 0: one walk per
                                 lane. Same results either way; default 1 */
    u32 sampled_regs;         /* direct_regs for sampled shadows (LTRG_SHADOW_SAMPLED); default 1 */
    u32 ao_packet;            /* 1: the 32 AO rays a warp traces at a step share one BVH walk (each
                                 lane keeping its own segment and closest hit); default 1 */
    u32 reserved[3];
} ltrg_Tuning;
LTRAPI LTRBOOL ltrg_GetTuning(int device, ltrg_Tuning* out);
/* Values outside 32..512 threads (multiples of 32), 1..64 blocks per SM, orders above 2,
 * direct_regs or sampled_regs above 3, direct_packet or ao_packet above 1, stacks other than 0, 4, 8
 * and 16 or ao_chunk outside 1..8 are rejected. */
LTRAPI LTRBOOL ltrg_SetTuning(int device, const ltrg_Tuning* t);
/* Autotuner: bakes `scene` (not running; its device) repeatedly, coordinate
 * descent over the candidate shapes of each kernel, each timed by that
 * kernel's stage time (the best of two bakes), and keeps the fastest as the
 * device's tuning. `out` receives it (may be NULL); the scene keeps the outputs
 * of its last bake. Returns 0 if a bake fails. */
LTRAPI LTRBOOL ltrg_Autotune(ltr_Scene* scene, ltrg_Tuning* out);

/* Read-only introspection of a finished bake (requires keep_samples = 1).
 * Instance 0 is the probe-sample container of ltr_SampleAdd, as in the
 * reference (lighter_int.hpp:975-980). */
LTRAPI u32 ltrdbg_InstanceCount(ltr_Scene* scene);
LTRAPI u32 ltrdbg_SampleCount(ltr_Scene* scene, u32 inst);
LTRAPI LTRBOOL ltrdbg_LightmapSize(ltr_Scene* scene, u32 inst, u32* wh);
LTRAPI LTRBOOL ltrdbg_GetSamples(ltr_Scene* scene, u32 inst, float* pos3, float* nrm3, u32* loc, float* radinfo4,
                                 float* color3);
LTRAPI u32 ltrdbg_RadLinkCount(ltr_Scene* scene);
/* Per-ray records of instance `inst` (keep_samples = 1): vis receives
 * n_lights x n samples shadow factors (CalcInvShadowFactor, -1 where the pair
 * was not traced), ao receives n x ao_num_samples AO closest-hit fractions (2
 * for a miss); either may be NULL. Returns 0 when the bake recorded none. */
LTRAPI LTRBOOL ltrdbg_GetRayData(ltr_Scene* scene, u32 inst, float* vis, float* ao);
/* The radiosity elements of the last bake (keep_samples = 1): *n receives
 * their count (samples, or patches in patch mode); each non-NULL array
 * receives n float4: position, unit normal, (diffuse rgb, area), emitted rgb
 * (the light the bounces start from) and the radiosity total (sum over
 * m <= bounces of K^m E); F, when not NULL, receives the form factors as
 * n x n floats (the stored FP32/FP16/BF16 values, widened; kept for
 * n <= 24576). Returns 0 when the bake ran no radiosity or F was asked for
 * and not kept. */
LTRAPI LTRBOOL ltrdbg_GetRadiosity(ltr_Scene* scene, u32* n, float* pos4, float* nrm4, float* diff_area4, float* emit4,
                                   float* total4, float* F);
/* Closest hits of n_segs segments (6 floats each: start, end) against a
 * triangle soup (n_tris x 9 floats, every triangle an occluder), through the
 * bake's BVH, traversal and segment test of `intersect_mode` (LTRG_ISECT_*):
 * out_r[i] = smallest hit fraction in [0, 1] along segment i, or 2 for none.
 * The segments are traced as given (not shortened). Returns 0 on an error
 * (message on stderr). */
LTRAPI LTRBOOL ltrdbg_TraceSegments(const float* tri_xyz, u32 n_tris, const float* seg6, u32 n_segs,
                                    int intersect_mode, float* out_r, int device);
/* n values of (float) rand() / RAND_MAX exactly as n rand() calls would give
 * them, leaving the C library's generator where those calls would (the AO
 * stage's bulk draw, exposed for testing). */
LTRAPI void ltrdbg_DrawRandFloats(float* out, u32 n);
/* The sample-offset pass's reference-shaped tree over a triangle soup (n_tris x
 * 9 floats), built with (threads != 0) or without its threaded top levels:
 * out3 = {node count, item-list length, FNV-1a hash of the node and item
 * arrays}. Host only; for tests. */
LTRAPI LTRBOOL ltrdbg_RefTreeDigest(const float* tri_xyz, u32 n_tris, int threads, uint64_t* out3);

#ifdef __cplusplus
}
#endif
