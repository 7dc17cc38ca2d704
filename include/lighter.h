/*
 * lighter.h -- public C ABI of the GB300 lightmap baker.
 *
 * This header declares the same `ltr_*` entry points, constants and struct
 * layouts as archo5/lighter's lighter.h (MIT licence), so that an application
 * written against that library links against liblighter_gb300.so unchanged.
 * The layouts are ABI: every field keeps its type, order and meaning.
 *
 * Reference interface each declaration replaces (file:line in archo5/lighter):
 *   structs ............................ lighter.h:64-233
 *   scene management ................... lighter.h:237-244, lighter.cpp:101-109,1147-1214
 *   data input ......................... lighter.h:247-251, lighter.cpp:1217-1329
 *   data output ........................ lighter.h:254-255, lighter.cpp:1332-1345
 *   misc ............................... lighter.h:191-201,258, lighter.cpp:7-28,1348-1357
 *
 * Behaviour differences from the CPU library are limited to:
 *   - ltr_Start uploads the scene to the GPU and runs the bake in CUDA kernels on
 *     a host thread of its own; ltr_GetStatus polls it exactly as before.
 *   - ltr_Abort is implemented (the reference leaves it empty): the bake stops
 *     between stages and ltr_GetStatus reports stage "aborted".
 *   - a failure (no CUDA device, out of device memory, invalid input) ends the
 *     bake with stage text starting with "error:" and no work outputs.
 * GPU-specific extensions live in lighter_gb300.h.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32) && !defined(LTR_STATIC)
#  ifdef LTRBUILD
#    define LTRAPI __declspec(dllexport)
#  else
#    define LTRAPI __declspec(dllimport)
#  endif
#else
#  define LTRAPI __attribute__((visibility("default")))
#endif

#define LTRBOOL int
#define LTRCODE int

#include <stdlib.h>
#include <inttypes.h>

typedef int32_t i32;
typedef uint32_t u32;

typedef float ltr_VEC3[3];
typedef float ltr_VEC4[4];
typedef ltr_VEC4 ltr_MAT4[4];

#define LTR_VEC3_SET(v, x, y, z) do { (v)[0] = (x); (v)[1] = (y); (v)[2] = (z); } while (0)

#define LTRC_SUCCESS 0
#define LTRC_ATEND   1

/* light types (lighter.h:59-61) */
#define LTR_LT_POINT  1
#define LTR_LT_SPOT   2
#define LTR_LT_DIRECT 3

/* One mesh part: strided vertex streams plus a u32 triangle list.
 * Copied at ltr_MeshAddPart time (lighter.h:64-79). */
typedef struct ltr_MeshPartInfo {
    const void* positions_f3;
    const void* normals_f3;
    const void* texcoords1_f2;   /* passed through to sample_fn (tex0u/tex0v) */
    const void* texcoords2_f2;   /* lightmap UVs in [0,1] */
    u32 stride_positions;
    u32 stride_normals;
    u32 stride_texcoords1;
    u32 stride_texcoords2;
    const u32* indices;
    u32 vertex_count;
    u32 index_count;
    int shadow;                  /* part casts shadows */
} ltr_MeshPartInfo;

/* Placement of a mesh; matrix is row-vector convention, translation in
 * matrix[3] (lighter.h:81-89). */
typedef struct ltr_MeshInstanceInfo {
    ltr_MAT4 matrix;
    float importance;
    int shadow;                  /* instance occludes light */
    const char* ident;
    size_t ident_size;
} ltr_MeshInstanceInfo;

/* lighter.h:91-106 */
typedef struct ltr_LightInfo {
    u32 type;
    ltr_VEC3 position;
    ltr_VEC3 direction;
    ltr_VEC3 up_direction;
    ltr_VEC3 color_rgb;
    float range;
    float power;
    float light_radius;
    int shadow_sample_count;
    float spot_angle_out;
    float spot_angle_in;
    float spot_curve;
} ltr_LightInfo;

/* A free-standing probe point lit like a lightmap texel (lighter.h:108-115). */
typedef struct ltr_SampleInfo {
    u32 id;
    ltr_VEC3 position;
    ltr_VEC3 normal;
    ltr_VEC3 out_color;
} ltr_SampleInfo;

/* Argument of config.sample_fn, one call per radiosity sample (lighter.h:117-133). */
typedef struct ltr_SampleRequest {
    ltr_VEC3 position;
    ltr_VEC3 normal;
    float tex0u, tex0v;
    float tex1u, tex1v;
    uint32_t part_id;
    const char* mesh_ident;
    size_t mesh_ident_size;
    const char* inst_ident;
    size_t inst_ident_size;
    ltr_VEC3 out_diffuse_color;
    ltr_VEC3 out_emissive_color;
} ltr_SampleRequest;

/* Bake configuration; defaults come from ltr_GetConfig (lighter.h:135-189,
 * lighter.cpp:1171-1208). */
typedef struct ltr_Config ltr_Config;
struct ltr_Config {
    void* userdata;
    LTRBOOL (*size_fn)(ltr_Config* config, const char* mesh_ident, size_t mesh_ident_size,
                       const char* inst_ident, size_t inst_ident_size,
                       float computed_surface_area, float inst_importance, u32 out_size[2]);
    int max_num_threads;
    size_t max_tree_memory;
    u32 max_lightmap_size;
    u32 default_width;
    u32 default_height;
    float global_size_factor;
    float max_correct_dist;
    float max_correct_angle;
    ltr_VEC3 clear_color;
    ltr_VEC3 ambient_color;
    int bounce_count;
    LTRBOOL (*sample_fn)(ltr_Config* config, ltr_SampleRequest* req);
    float ao_distance;
    float ao_multiplier;
    float ao_falloff;
    float ao_effect;
    float ao_divergence;
    ltr_VEC3 ao_color_rgb;
    int ao_num_samples;
    float blur_size;
    int ds2x;
    int generate_normalmap_data;
};

LTRAPI LTRBOOL ltr_DefaultSizeFunc(ltr_Config* config, const char* mesh_ident, size_t mesh_ident_size,
                                   const char* inst_ident, size_t inst_ident_size,
                                   float computed_surface_area, float inst_importance, u32 out_size[2]);

/* lighter.h:203-209 */
typedef struct ltr_WorkOutputInfo {
    u32 lightmap_count;
    u32 sample_count;
    ltr_SampleInfo* samples;
} ltr_WorkOutputInfo;

/* One baked lightmap; buffers are owned by the scene (lighter.h:211-223). */
typedef struct ltr_WorkOutput {
    u32 uid;
    const char* mesh_ident;
    size_t mesh_ident_size;
    const char* inst_ident;
    size_t inst_ident_size;
    float* lightmap_rgb;
    float* normals_xyzf;
    u32 width;
    u32 height;
} ltr_WorkOutput;

typedef struct ltr_Mesh ltr_Mesh;
typedef struct ltr_Scene ltr_Scene;

/* lighter.h:228-233 */
typedef struct ltr_WorkStatus {
    float completion;
    const char* stage;
} ltr_WorkStatus;

/* scene management (lighter.h:237-244) */
LTRAPI ltr_Scene* ltr_CreateScene(void);
LTRAPI void ltr_DestroyScene(ltr_Scene* scene);
LTRAPI void ltr_Start(ltr_Scene* scene);
LTRAPI void ltr_Abort(ltr_Scene* scene);
LTRAPI LTRBOOL ltr_GetStatus(ltr_Scene* scene, ltr_WorkStatus* wsout);
LTRAPI void ltr_Sleep(int ms);
LTRAPI void ltr_GetConfig(ltr_Config* cfg, ltr_Scene* opt_scene);
LTRAPI LTRCODE ltr_SetConfig(ltr_Scene* scene, ltr_Config* cfg);

/* data input (lighter.h:247-251) */
LTRAPI ltr_Mesh* ltr_CreateMesh(ltr_Scene* scene, const char* ident, size_t ident_size);
LTRAPI LTRBOOL ltr_MeshAddPart(ltr_Mesh* mesh, ltr_MeshPartInfo* mpinfo);
LTRAPI LTRBOOL ltr_MeshAddInstance(ltr_Mesh* mesh, ltr_MeshInstanceInfo* mii);
LTRAPI void ltr_LightAdd(ltr_Scene* scene, ltr_LightInfo* li);
LTRAPI void ltr_SampleAdd(ltr_Scene* scene, ltr_SampleInfo* si);

/* data output (lighter.h:254-255) */
LTRAPI void ltr_GetWorkOutputInfo(ltr_Scene* scene, ltr_WorkOutputInfo* woutinfo);
LTRAPI LTRBOOL ltr_GetWorkOutput(ltr_Scene* scene, u32 which, ltr_WorkOutput* wout);

/* misc (lighter.h:258) */
LTRAPI u32 ltr_NextPowerOfTwo(u32 x);

#ifdef __cplusplus
}
#endif
