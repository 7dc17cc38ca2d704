// The ltr_* C API of lighter.h (lighter.cpp:7-28, 101-109, 1147-1357) over
// the GPU bake. Ingest, configuration and output ownership keep the
// reference's contract: parts are copied at ltr_MeshAddPart time, outputs are
// owned by the scene until ltr_DestroyScene, ltr_Start returns at once and
// ltr_GetStatus polls a bake running on a host thread of its own.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "scene.hpp"

using namespace lg;

ltr_Scene::ltr_Scene()
{
    ltr_GetConfig(&cfg, nullptr);
    memset(&opt, 0, sizeof(opt));
    opt.refine_steps = 1;
    memset(&stats, 0, sizeof(stats));
    HostInst* c = new HostInst;   // probe-sample container, lighter_int.hpp:975-980
    c->container = true;
    c->w = c->h = 0;
    insts.push_back(c);
}

void ltr_Scene::clear_outputs()
{
    outputs.clear();   // the buffers live in `pinned`, which the next bake reuses
    outputs_rgbe.clear();
    dump.clear();
    rad_dump = lg::RadDump();
}

ltr_Scene::~ltr_Scene()
{
    join_worker();
    clear_outputs();
    if (pinned) cudaFreeHost(pinned);
    if (ao_pinned) cudaFreeHost(ao_pinned);
    if (abort_alloc) cudaFreeHost(abort_alloc);
    // the bake's buffers stay cached in the device's memory pool for the next
    // bake; a destroyed scene gives back what the pool holds beyond 8 GiB
    // (an error of these calls is cleared: it must not surface in the caller's next CUDA call)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, opt.device) != cudaSuccess || cudaMemPoolTrimTo(pool, 8ull << 30) != cudaSuccess)
        (void) cudaGetLastError();
    for (HostInst* mi : insts) delete mi;
    for (ltr_Mesh* m : meshes) delete m;
}

// ---- launch shapes of the trace kernels, per device
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_tuning_mu;
ltrg_Tuning g_tuning[kMaxDevices];
bool g_tuning_set[kMaxDevices] = {};

ltrg_Tuning default_tuning()
{
    ltrg_Tuning t;
    memset(&t, 0, sizeof(t));
    t.direct_block = 128;
    t.direct_blocks_per_sm = 8;
    t.ao_block = 128;
    t.ao_blocks_per_sm = 16;
    t.direct_order = 2;
    t.ao_order = 1;
    t.ao_chunk = 1;
    t.direct_packet = 1;
    t.sampled_regs = 1;
    t.ao_packet = 1;
    return t;
}

bool tuning_valid(const ltrg_Tuning& t)
{
    auto block_ok = [](u32 b) { return b >= 32 && b <= 512 && b % 32 == 0; };
    auto bps_ok = [](u32 k) { return k >= 1 && k <= 64; };
    auto stack_ok = [](u32 k) { return k == 0 || k == 4 || k == 8 || k == 16; };
    return block_ok(t.direct_block) && block_ok(t.ao_block) && bps_ok(t.direct_blocks_per_sm) && bps_ok(t.ao_blocks_per_sm) &&
           t.direct_order <= 2 && t.ao_order <= 2 && t.direct_regs <= 3 && stack_ok(t.direct_stack) &&
           stack_ok(t.ao_stack) && t.ao_chunk >= 1 && t.ao_chunk <= 8 && t.direct_packet <= 1 &&
           t.sampled_regs <= 3 && t.ao_packet <= 1;
}
}  // namespace

ltrg_Tuning lg::get_tuning(int device)
{
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    if (device < 0 || device >= kMaxDevices || !g_tuning_set[device]) return default_tuning();
    return g_tuning[device];
}

static u32 next_pow2(u32 x)
{
    x--;
    x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
    return x + 1;
}

namespace lg {
// Golden-angle spiral around `dir` (Vec3::CreateSpiralDirVector,
// lighter_int.hpp:457-471), in float with the C library's functions.
static V3 spiral_dir_host(V3 dir, float randoff, int i, int count)
{
    float q = (i + 0.5f) / count;
    float cos_side = std::sqrt(q);
    float sin_side = std::sin(std::acos(cos_side));
    float angle = (i + randoff) * (137.508f / 180.0f * (float) M_PI);
    float cos_around = std::cos(angle);
    float sin_around = std::sin(angle);
    V3 diffvec = mk(dir.y, -dir.z, dir.x);
    V3 up = normalized(cross(dir, diffvec));
    V3 rt = cross(dir, up);
    return cos_around * sin_side * rt + sin_around * sin_side * up + cos_side * dir;
}

std::vector<V3> light_shadow_samples(const HostLight& L)
{
    std::vector<V3> out((size_t) L.nsamples);
    for (int s = 0; s < L.nsamples; ++s) {
        if (L.type == LTR_LT_DIRECT) {
            // lighter.cpp:1303-1305: the spiral around -direction pulled towards
            // +direction by tan((light_radius - 0.5) * pi * 0.999)
            V3 nd = -L.dir;
            V3 adj = spiral_dir_host(nd, L.randoff, s, L.nsamples);
            adj = normalized(adj + nd * std::tan((L.radius - 0.5f) * (float) M_PI * 0.999f));
            out[s] = adj;
        } else {
            // disk point s of the golden-angle spiral of radius light_radius
            float rho = L.radius * std::sqrt((s + 0.5f) / L.nsamples);
            float phi = (s + L.randoff) * (137.508f / 180.0f * (float) M_PI);
            out[s] = mk(rho * std::cos(phi), rho * std::sin(phi), 0.0f);
        }
    }
    return out;
}
}  // namespace lg

extern "C" {

LTRAPI u32 ltr_NextPowerOfTwo(u32 x) { return next_pow2(x); }

// size = global_size_factor * sqrt(area) * importance, at least 1, rounded up
// to a power of two; rejected above max_lightmap_size (lighter.cpp:7-28).
LTRAPI LTRBOOL ltr_DefaultSizeFunc(ltr_Config* config, const char*, size_t, const char*, size_t,
                                   float computed_surface_area, float inst_importance, u32 out_size[2])
{
    float size = config->global_size_factor * sqrtf(computed_surface_area) * inst_importance;
    if (size < 1) size = 1;
    u32 s = next_pow2((u32) size);
    if (s > config->max_lightmap_size) return 0;
    out_size[0] = s;
    out_size[1] = s;
    return 1;
}

// Defaults of lighter.cpp:1171-1208.
LTRAPI void ltr_GetConfig(ltr_Config* cfg, ltr_Scene* opt_scene)
{
    if (opt_scene) { memcpy(cfg, &opt_scene->cfg, sizeof(*cfg)); return; }
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

LTRAPI LTRCODE ltr_SetConfig(ltr_Scene* scene, ltr_Config* cfg)
{
    memcpy(&scene->cfg, cfg, sizeof(*cfg));
    return 1;
}

LTRAPI ltr_Scene* ltr_CreateScene(void) { return new ltr_Scene; }

LTRAPI void ltr_DestroyScene(ltr_Scene* scene)
{
    if (!scene) return;
    scene->abort_flag = true;
    delete scene;
}

static void start_bake(ltr_Scene* scene);

LTRAPI void ltr_Start(ltr_Scene* scene)
{
    scene->join_worker();
    scene->batch.reset();
    scene->batch_index = -1;
    start_bake(scene);
}

// Starts the bakes of `count` scenes as one batch (include/lighter_gb300.h).
LTRAPI LTRBOOL ltrg_StartBatch(ltr_Scene** scenes, u32 count)
{
    if (!scenes || count == 0) return 0;
    for (u32 k = 0; k < count; ++k) {
        if (!scenes[k] || scenes[k]->running.load()) return 0;
        if (scenes[k]->opt.device != scenes[0]->opt.device) return 0;
        for (u32 j = 0; j < k; ++j)
            if (scenes[j] == scenes[k]) return 0;
    }
    for (u32 k = 0; k < count; ++k)
        scenes[k]->join_worker();
    std::shared_ptr<BatchCtx> ctx = make_batch((int) count, scenes[0]->opt.device);
    for (u32 k = 0; k < count; ++k) {
        scenes[k]->batch = ctx;
        scenes[k]->batch_index = (int) k;
    }
    for (u32 k = 0; k < count; ++k) start_bake(scenes[k]);
    return 1;
}

static void start_bake(ltr_Scene* scene)
{
    scene->clear_outputs();
    scene->error.clear();
    scene->abort_flag = false;
    scene->completion = 0;
    scene->stage = "starting";
    scene->running = true;
    scene->worker = std::thread([scene]() {
        auto t0 = std::chrono::steady_clock::now();
        try {
            run_bake(scene);
            scene->stats.ms_total =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            scene->completion = 1;
            scene->stage = nullptr;
        } catch (const std::exception& e) {
            scene->clear_outputs();
            scene->error = e.what();
            scene->completion = 1;
            scene->stage = scene->abort_flag ? "aborted" : "error: bake failed (see ltrg_LastError)";
        }
        scene->batch.reset();
        scene->running = false;
    });
}

// The reference leaves this empty (lighter.cpp:1154-1157); here the bake
// stops at the next stage boundary and reports stage "aborted".
LTRAPI void ltr_Abort(ltr_Scene* scene)
{
    scene->abort_flag = true;
    if (u32* w = scene->abort_word.load()) *(volatile u32*) w = 1u;
}

// Returns 1 while the bake runs (lighter.cpp:1159-1164). A finished bake
// reports "finished"; a failed or aborted one returns 0 with a stage text
// starting with "error:" or "aborted" and no work outputs.
LTRAPI LTRBOOL ltr_GetStatus(ltr_Scene* scene, ltr_WorkStatus* wsout)
{
    bool running = scene->running.load();
    const char* st = scene->stage.load();
    wsout->completion = scene->completion.load();
    wsout->stage = st ? st : "finished";
    if (!running) scene->join_worker(false);   // a concurrent poller may be joining it already
    return running ? 1 : 0;
}

LTRAPI void ltr_Sleep(int ms) { std::this_thread::sleep_for(std::chrono::milliseconds(ms)); }

LTRAPI ltr_Mesh* ltr_CreateMesh(ltr_Scene* scene, const char* ident, size_t ident_size)
{
    ltr_Mesh* m = new ltr_Mesh;
    m->scene = scene;
    if (ident) m->ident.assign(ident, ident_size);
    scene->meshes.push_back(m);
    return m;
}

// Copies strided streams (lighter.cpp:1226-1264). The reference's validity
// test `index_count < 3 && index_count % 3 != 0` is kept; a part whose
// indices point past its vertices is rejected as well, since the GPU raster
// would otherwise read outside the vertex arrays.
LTRAPI LTRBOOL ltr_MeshAddPart(ltr_Mesh* mesh, ltr_MeshPartInfo* p)
{
    if (!mesh || !p) return 0;
    if (p->index_count < 3 && p->index_count % 3 != 0) return 0;
    if (p->index_count && !p->indices) return 0;
    for (u32 i = 0; i < p->index_count; ++i)
        if (p->indices[i] >= p->vertex_count) return 0;
    if (p->vertex_count && (!p->positions_f3 || !p->normals_f3 || !p->texcoords1_f2 || !p->texcoords2_f2)) return 0;
    HostPart hp = {p->vertex_count, (u32) mesh->pos.size(), p->index_count, (u32) mesh->idx.size(), p->shadow};
    for (u32 i = 0; i < p->vertex_count; ++i) {
        V3 a, b;
        V2 t1, t2;
        memcpy(&a, (const char*) p->positions_f3 + (size_t) p->stride_positions * i, 12);
        memcpy(&b, (const char*) p->normals_f3 + (size_t) p->stride_normals * i, 12);
        memcpy(&t1, (const char*) p->texcoords1_f2 + (size_t) p->stride_texcoords1 * i, 8);
        memcpy(&t2, (const char*) p->texcoords2_f2 + (size_t) p->stride_texcoords2 * i, 8);
        mesh->pos.push_back(a);
        mesh->nrm.push_back(b);
        mesh->tex1.push_back(t1);
        mesh->tex2.push_back(t2);
    }
    mesh->idx.insert(mesh->idx.end(), p->indices, p->indices + p->index_count);
    mesh->parts.push_back(hp);
    return 1;
}

LTRAPI LTRBOOL ltr_MeshAddInstance(ltr_Mesh* mesh, ltr_MeshInstanceInfo* mii)
{
    HostInst* mi = new HostInst;
    mi->mesh = mesh;
    mi->importance = mii->importance;
    mi->shadow = !!mii->shadow;
    if (mii->ident) mi->ident.assign(mii->ident, mii->ident_size);
    memcpy(mi->matrix, mii->matrix, sizeof(float) * 16);
    mesh->scene->insts.push_back(mi);
    return 1;
}

// Direction vectors normalised, at least one shadow sample, and one rand()
// draw per light as the reference makes (lighter.cpp:1282-1317), so that a
// caller's srand() sequence reaches the AO stage in the same state.
LTRAPI void ltr_LightAdd(ltr_Scene* scene, ltr_LightInfo* li)
{
    HostLight L;
    L.type = li->type;
    L.pos = mk(li->position[0], li->position[1], li->position[2]);
    L.dir = normalized(mk(li->direction[0], li->direction[1], li->direction[2]));
    L.up = normalized(mk(li->up_direction[0], li->up_direction[1], li->up_direction[2]));
    L.color = mk(li->color_rgb[0], li->color_rgb[1], li->color_rgb[2]);
    L.range = li->range;
    L.power = li->power;
    L.radius = li->light_radius;
    L.nsamples = li->shadow_sample_count > 1 ? li->shadow_sample_count : 1;
    L.out = li->spot_angle_out;
    L.in = li->spot_angle_in;
    L.curve = li->spot_curve;
    L.randoff = (float) rand() / (float) RAND_MAX;   // randf(), lighter_int.hpp:271
    scene->lights.push_back(L);
}

LTRAPI void ltr_SampleAdd(ltr_Scene* scene, ltr_SampleInfo* si)
{
    ltr_SampleInfo c = *si;
    c.out_color[0] = c.out_color[1] = c.out_color[2] = 0;
    scene->samples.push_back(c);
}

LTRAPI void ltr_GetWorkOutputInfo(ltr_Scene* scene, ltr_WorkOutputInfo* o)
{
    o->lightmap_count = (u32) scene->outputs.size();
    o->sample_count = (u32) scene->samples.size();
    o->samples = scene->samples.empty() ? nullptr : scene->samples.data();
}

LTRAPI LTRBOOL ltr_GetWorkOutput(ltr_Scene* scene, u32 which, ltr_WorkOutput* wout)
{
    if (which >= scene->outputs.size()) return 0;
    *wout = scene->outputs[which];
    return 1;
}

// ---- extensions (lighter_gb300.h)

LTRAPI void ltrg_GetOptions(ltr_Scene* scene, ltrg_Options* out) { *out = scene->opt; }

LTRAPI LTRBOOL ltrg_SetOptions(ltr_Scene* scene, const ltrg_Options* o)
{
    if (o->device < 0 || o->radiosity_links < 0 || o->radiosity_links > 1 || o->radiosity_precision < 0 ||
        o->radiosity_precision > 2 || o->refine_steps < 0 || o->refine_steps > 16 || o->bvh_builder > 1 ||
        o->shadow_mode > 1 || o->intersect_mode > 1 || o->encode_rgbe > 1)
        return 0;
    scene->opt = *o;
    return 1;
}

LTRAPI LTRBOOL ltrg_GetWorkOutputRGBE(ltr_Scene* scene, u32 which, const unsigned char** rgbe)
{
    if (!scene || !rgbe || scene->running.load() || which >= scene->outputs_rgbe.size()) return 0;
    *rgbe = scene->outputs_rgbe[which];
    return 1;
}

LTRAPI LTRBOOL ltrg_GetStats(ltr_Scene* scene, ltrg_Stats* out)
{
    if (scene->running.load()) return 0;
    *out = scene->stats;
    return scene->stage.load() == nullptr ? 1 : 0;
}

LTRAPI const char* ltrg_LastError(ltr_Scene* scene)
{
    if (scene->running.load()) return nullptr;
    return scene->error.empty() ? nullptr : scene->error.c_str();
}

LTRAPI LTRBOOL ltrg_GetTuning(int device, ltrg_Tuning* out)
{
    if (!out || device < 0 || device >= kMaxDevices) return 0;
    *out = get_tuning(device);
    return 1;
}

LTRAPI LTRBOOL ltrg_SetTuning(int device, const ltrg_Tuning* t)
{
    if (!t || device < 0 || device >= kMaxDevices || !tuning_valid(*t)) return 0;
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    g_tuning[device] = *t;
    g_tuning_set[device] = true;
    return 1;
}

// Coordinate descent: each launch parameter in turn takes the candidate whose
// bakes (best of two) give its kernel's stage the shortest device time.
LTRAPI LTRBOOL ltrg_Autotune(ltr_Scene* scene, ltrg_Tuning* out)
{
    if (!scene || scene->running.load()) return 0;
    const int dev = scene->opt.device;
    if (dev < 0 || dev >= kMaxDevices) return 0;
    ltrg_Tuning best = get_tuning(dev);
    auto bake_once = [&](const ltrg_Tuning& t, double& ms_direct, double& ms_ao) {
        ltrg_SetTuning(dev, &t);
        ltr_Start(scene);
        if (!ltrg_Wait(scene)) return false;
        ms_direct = scene->stats.ms_direct;
        ms_ao = scene->stats.ms_ao;
        return true;
    };
    // a stage's time varies from bake to bake by a few per cent: the least of three bakes
    auto measure = [&](const ltrg_Tuning& t, double& ms_direct, double& ms_ao) {
        ms_direct = ms_ao = 1e300;
        for (int r = 0; r < 3; ++r) {
            double d, a;
            if (!bake_once(t, d, a)) return false;
            ms_direct = std::min(ms_direct, d);
            ms_ao = std::min(ms_ao, a);
        }
        return true;
    };
    const ltrg_Tuning start = best;
    double bd, ba;
    if (!bake_once(best, bd, ba) || !measure(best, bd, ba)) {   // warm-up, then the baseline
        ltrg_SetTuning(dev, &best);
        return 0;
    }
    struct Param { u32 ltrg_Tuning::*field; bool direct; std::vector<u32> cand; };
    const Param params[] = {
        {&ltrg_Tuning::direct_blocks_per_sm, true, {2, 4, 8, 16, 32}},
        {&ltrg_Tuning::direct_block, true, {64, 128, 256}},
        {&ltrg_Tuning::direct_order, true, {0, 1, 2}},
        {&ltrg_Tuning::direct_regs, true, {0, 1, 2, 3}},
        {&ltrg_Tuning::direct_stack, true, {0, 4, 8, 16}},
        {&ltrg_Tuning::direct_packet, true, {0, 1}},
        {&ltrg_Tuning::sampled_regs, true, {0, 1, 2, 3}},
        {&ltrg_Tuning::ao_blocks_per_sm, false, {4, 8, 16, 32}},
        {&ltrg_Tuning::ao_block, false, {64, 128, 256}},
        {&ltrg_Tuning::ao_order, false, {0, 1, 2}},
        {&ltrg_Tuning::ao_stack, false, {0, 4, 8, 16}},
        {&ltrg_Tuning::ao_chunk, false, {1, 2, 4, 8}},
        {&ltrg_Tuning::ao_packet, false, {0, 1}},
    };
    for (const Param& p : params) {
        for (u32 v : p.cand) {
            if (best.*p.field == v) continue;
            ltrg_Tuning t = best;
            t.*p.field = v;
            double d, a;
            if (!measure(t, d, a)) {
                ltrg_SetTuning(dev, &best);
                return 0;
            }
            double& cur = p.direct ? bd : ba;
            double got = p.direct ? d : a;
            if (got < cur * 0.98) {   // a clear win only
                best = t;
                bd = p.direct ? d : bd;
                ba = p.direct ? ba : a;
            }
        }
    }
    // confirm each kernel's choice against the starting shapes, timed alternately
    if (memcmp(&best, &start, sizeof(best)) != 0) {
        double sd = 1e300, sa = 1e300, nd = 1e300, na = 1e300;
        for (int r = 0; r < 2; ++r) {
            double d, a;
            if (!measure(start, d, a)) { ltrg_SetTuning(dev, &start); return 0; }
            sd = std::min(sd, d); sa = std::min(sa, a);
            if (!measure(best, d, a)) { ltrg_SetTuning(dev, &start); return 0; }
            nd = std::min(nd, d); na = std::min(na, a);
        }
        if (!(nd < sd * 0.98)) {
            best.direct_block = start.direct_block;
            best.direct_blocks_per_sm = start.direct_blocks_per_sm;
            best.direct_order = start.direct_order;
            best.direct_regs = start.direct_regs;
            best.direct_stack = start.direct_stack;
            best.direct_packet = start.direct_packet;
            best.sampled_regs = start.sampled_regs;
        }
        if (!(na < sa * 0.98)) {
            best.ao_block = start.ao_block;
            best.ao_blocks_per_sm = start.ao_blocks_per_sm;
            best.ao_order = start.ao_order;
            best.ao_stack = start.ao_stack;
            best.ao_chunk = start.ao_chunk;
            best.ao_packet = start.ao_packet;
        }
    }
    ltrg_SetTuning(dev, &best);
    if (out) *out = best;
    return 1;
}

LTRAPI LTRBOOL ltrg_Wait(ltr_Scene* scene)
{
    scene->join_worker();
    return scene->error.empty() && scene->stage.load() == nullptr ? 1 : 0;
}

LTRAPI LTRBOOL ltrg_TableSampleFn(ltr_Config* cfg, ltr_SampleRequest* req)
{
    const ltrg_SampleTable* t = (const ltrg_SampleTable*) cfg->userdata;
    if (!t) return 0;
    float fid = req->tex0u;
    if (!(fid >= 0.0f)) return 0;
    u32 id = (u32) fid;
    if (id >= t->count) return 0;
    if (t->diffuse_rgb)
        for (int c = 0; c < 3; ++c) req->out_diffuse_color[c] = t->diffuse_rgb[id * 3 + c];
    if (t->emissive_rgb)
        for (int c = 0; c < 3; ++c) req->out_emissive_color[c] = t->emissive_rgb[id * 3 + c];
    return 1;
}

LTRAPI u32 ltrdbg_InstanceCount(ltr_Scene* s) { return (u32) s->insts.size(); }

LTRAPI u32 ltrdbg_SampleCount(ltr_Scene* s, u32 inst)
{
    if (inst >= s->dump.size()) return 0;
    return (u32) s->dump[inst].loc.size();
}

LTRAPI LTRBOOL ltrdbg_LightmapSize(ltr_Scene* s, u32 inst, u32* wh)
{
    if (inst >= s->insts.size()) return 0;
    wh[0] = s->insts[inst]->w;
    wh[1] = s->insts[inst]->h;
    return 1;
}

LTRAPI LTRBOOL ltrdbg_GetSamples(ltr_Scene* s, u32 inst, float* pos3, float* nrm3, u32* loc, float* radinfo4,
                                 float* color3)
{
    if (inst >= s->dump.size()) return 0;
    const SampleDump& d = s->dump[inst];
    size_t n = d.loc.size();
    if (pos3) memcpy(pos3, d.pos.data(), n * 12);
    if (nrm3) memcpy(nrm3, d.nrm.data(), n * 12);
    if (loc) memcpy(loc, d.loc.data(), n * 4);
    if (radinfo4) memcpy(radinfo4, d.radinfo.data(), n * 16);
    if (color3) memcpy(color3, d.color.data(), n * 12);
    return 1;
}

LTRAPI u32 ltrdbg_RadLinkCount(ltr_Scene* s) { return s->rad_links; }

LTRAPI LTRBOOL ltrdbg_GetRadiosity(ltr_Scene* scene, u32* n, float* pos4, float* nrm4, float* diff_area4, float* emit4,
                                   float* total4, float* F)
{
    if (scene->running.load()) return 0;
    const lg::RadDump& d = scene->rad_dump;
    if (n) *n = d.n;
    if (!d.n || d.total.size() != 4 * (size_t) d.n || (F && d.F.empty())) return 0;
    const std::vector<float>* src[5] = {&d.pos, &d.nrm, &d.diff_area, &d.emit, &d.total};
    float* dst[5] = {pos4, nrm4, diff_area4, emit4, total4};
    for (int k = 0; k < 5; ++k)
        if (dst[k]) memcpy(dst[k], src[k]->data(), src[k]->size() * sizeof(float));
    if (F) memcpy(F, d.F.data(), d.F.size() * sizeof(float));
    return 1;
}

LTRAPI LTRBOOL ltrdbg_GetRayData(ltr_Scene* scene, u32 inst, float* vis, float* ao)
{
    if (scene->running.load() || inst >= scene->dump.size()) return 0;
    const SampleDump& d = scene->dump[inst];
    if (vis) {
        if (d.vis.size() != (size_t) scene->lights.size() * d.loc.size()) return 0;
        if (!d.vis.empty()) memcpy(vis, d.vis.data(), d.vis.size() * sizeof(float));
    }
    if (ao) {
        if (d.ao.empty() && !d.loc.empty()) return 0;
        if (!d.ao.empty()) memcpy(ao, d.ao.data(), d.ao.size() * sizeof(float));
    }
    return 1;
}

}  // extern "C"
