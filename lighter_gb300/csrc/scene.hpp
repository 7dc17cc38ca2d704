// Host-side scene model behind the ltr_* API (replaces ltr_Scene/ltr_Mesh/
// ltr_MeshInstance/ltr_Light of lighter_int.hpp:837-1051). Ingest copies the
// caller's data here; ltr_Start hands the scene to the bake thread
// (bake.cu), which uploads it as structure-of-arrays device buffers.
#pragma once

#include <atomic>
#include <memory>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/lighter_gb300.h"
#include "common.cuh"

namespace lg {

struct HostPart { u32 vcount, voff, icount, ioff; int shadow; };

struct HostInst {
    ltr_Mesh* mesh = nullptr;
    std::string ident;
    float importance = 0;
    float matrix[16];
    bool shadow = false;
    bool container = false;
    u32 w = 128, h = 128;      // lightmap size (lighter.cpp:1277-1278 default)
    // filled by the bake (world space, lightmap texel space)
    std::vector<V3> vpos, vnrm;
    std::vector<V2> vtex, ltex;
};

struct HostLight {
    u32 type;
    V3 pos, dir, up, color;
    float range, power, radius;
    int nsamples;
    float out, in, curve;
    float randoff;   // the light's rand() draw of ltr_LightAdd (lighter.cpp:1300)
};

// Per-light shadow samples of LTRG_SHADOW_SAMPLED, computed on the host like
// ltr_LightAdd computes its samples (lighter.cpp:1295-1312): directional
// lights get nsamples unit ray directions, point and spot lights nsamples
// disk offsets (x, y, 0) in the plane facing the sample (api.cpp).
std::vector<V3> light_shadow_samples(const HostLight& L);

// Per-instance copies of the sample arrays, kept when keep_samples is set.
struct SampleDump {
    std::vector<float> pos, nrm, radinfo, color;
    std::vector<u32> loc;
    std::vector<float> vis;   // [light][sample] shadow factor, -1 when not traced
    std::vector<float> ao;    // [sample][ray] AO closest-hit fraction
    u32 n_lights = 0, ao_ns = 0;
};

// The radiosity elements of the last bake (samples, or patches in patch mode),
// kept when keep_samples is set: float4 per element, and F as n x n floats
// when n <= kRadDumpMaxF.
struct RadDump {
    static constexpr u32 kRadDumpMaxF = 24576;
    u32 n = 0;
    std::vector<float> pos, nrm, diff_area, emit, total, F;
};

}  // namespace lg

struct ltr_Mesh {
    ltr_Scene* scene;
    std::string ident;
    std::vector<lg::V3> pos, nrm;
    std::vector<lg::V2> tex1, tex2;
    std::vector<lg::u32> idx;
    std::vector<lg::HostPart> parts;
};

namespace lg {
struct BatchCtx;   // bake.cu: the rendezvous of the scenes of one ltrg_StartBatch
std::shared_ptr<BatchCtx> make_batch(int n, int device);
// Launch shapes of the trace kernels of one device (api.cpp).
ltrg_Tuning get_tuning(int device);
// n values of (float) rand() / RAND_MAX, as n rand() calls would give and leave the state (rng.cpp).
void rand_floats(float* out, size_t n);
}  // namespace lg

struct ltr_Scene {
    ltr_Config cfg;
    ltrg_Options opt;
    std::vector<ltr_Mesh*> meshes;
    std::vector<lg::HostInst*> insts;   // [0] = probe-sample container
    std::vector<lg::HostLight> lights;
    std::vector<ltr_SampleInfo> samples;
    std::vector<ltr_WorkOutput> outputs;   // buffers point into `pinned`
    std::vector<const unsigned char*> outputs_rgbe;   // RGBE encodings (ltrg_Options::encode_rgbe), in `pinned`
    void* pinned = nullptr;                 // page-locked output storage, reused across bakes
    size_t pinned_bytes = 0;
    float* ao_pinned = nullptr;             // page-locked AO random offsets, reused across bakes
    lg::u32 ao_pinned_n = 0;
    std::vector<lg::SampleDump> dump;
    lg::RadDump rad_dump;
    lg::u32 rad_links = 0;
    ltrg_Stats stats;
    std::string error;
    std::atomic<const char*> stage{"not started"};
    std::atomic<float> completion{0};
    std::atomic<bool> abort_flag{false};
    // Page-locked word mapped into the device's address space: ltr_Abort sets it
    // to 1 and the persistent trace kernels poll it at their work fetches, so an
    // abort ends a long trace launch within about one fetch. run_bake writes 0
    // and publishes the pointer before it reads abort_flag once more, so an
    // abort racing with the start of a bake is never lost.
    std::atomic<lg::u32*> abort_word{nullptr};
    void* abort_alloc = nullptr;
    std::atomic<bool> running{false};
    std::thread worker;
    std::mutex join_mu;                     // serialises joins of `worker` (pollers may run on several threads)
    std::shared_ptr<lg::BatchCtx> batch;   // set for the bake started by ltrg_StartBatch
    int batch_index = -1;

    ltr_Scene();
    ~ltr_Scene();
    void clear_outputs();
    // Joins the bake thread if there is one to join. `wait` false: returns at
    // once when another thread is joining it.
    void join_worker(bool wait = true)
    {
        std::unique_lock<std::mutex> lk(join_mu, std::defer_lock);
        if (wait) lk.lock();
        else if (!lk.try_lock()) return;
        if (worker.joinable()) worker.join();
    }
};

namespace lg {
// Runs the whole bake on the calling thread; throws std::runtime_error.
void run_bake(ltr_Scene* s);
}
