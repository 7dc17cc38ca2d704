// Test-infrastructure harness around the UNMODIFIED reference (archo5/lighter).
//
// Compiled together with the reference's own lighter.cpp and lighter_math.cpp
// (see oracle/Makefile) into oracle/_ref/liblighter_ref.so. It adds only the
// read-only `ltrdbg_*` introspection entry points that the oracle port and the
// GPU library also export, so one Python test harness can drive all three and
// compare per-stage arrays:
//   samples (pos/nrm/loc/radinfo) ... ltr_MeshInstance::m_samples_*  lighter_int.hpp:897-900
//   per-sample colour ............... ltr_MeshInstance::m_lightmap    lighter_int.hpp:901
// It also provides ltrg_TableSampleFn, the table-driven sample_fn the tests
// use for per-face albedo (same contract as the GPU library's one).
// Nothing here is shipped or measured: it exists to pin the oracle.

#include "lighter_int.hpp"

extern "C" {

__attribute__((visibility("default"))) u32 ltrdbg_InstanceCount(ltr_Scene* s)
{
    return (u32) s->m_meshInstances.size();
}

__attribute__((visibility("default"))) u32 ltrdbg_SampleCount(ltr_Scene* s, u32 inst)
{
    if (inst >= s->m_meshInstances.size()) return 0;
    return (u32) s->m_meshInstances[inst]->m_lightmap.size();
}

__attribute__((visibility("default"))) int ltrdbg_LightmapSize(ltr_Scene* s, u32 inst, u32* wh)
{
    if (inst >= s->m_meshInstances.size()) return 0;
    wh[0] = s->m_meshInstances[inst]->lm_width;
    wh[1] = s->m_meshInstances[inst]->lm_height;
    return 1;
}

// Copies the per-sample arrays of instance `inst`; any pointer may be NULL.
__attribute__((visibility("default"))) int ltrdbg_GetSamples(ltr_Scene* s, u32 inst, float* pos3, float* nrm3,
                                                             u32* loc, float* radinfo4, float* color3)
{
    if (inst >= s->m_meshInstances.size()) return 0;
    ltr_MeshInstance* mi = s->m_meshInstances[inst];
    size_t n = mi->m_lightmap.size();
    for (size_t i = 0; i < n; ++i) {
        if (pos3 && i < mi->m_samples_pos.size()) {
            pos3[i*3+0] = mi->m_samples_pos[i].x; pos3[i*3+1] = mi->m_samples_pos[i].y; pos3[i*3+2] = mi->m_samples_pos[i].z;
        }
        if (nrm3 && i < mi->m_samples_nrm.size()) {
            nrm3[i*3+0] = mi->m_samples_nrm[i].x; nrm3[i*3+1] = mi->m_samples_nrm[i].y; nrm3[i*3+2] = mi->m_samples_nrm[i].z;
        }
        if (loc) loc[i] = i < mi->m_samples_loc.size() ? mi->m_samples_loc[i] : 0xffffffffu;
        if (radinfo4 && i < mi->m_samples_radinfo.size()) {
            radinfo4[i*4+0] = mi->m_samples_radinfo[i].x; radinfo4[i*4+1] = mi->m_samples_radinfo[i].y;
            radinfo4[i*4+2] = mi->m_samples_radinfo[i].z; radinfo4[i*4+3] = mi->m_samples_radinfo[i].w;
        }
        if (color3) {
            color3[i*3+0] = mi->m_lightmap[i].x; color3[i*3+1] = mi->m_lightmap[i].y; color3[i*3+2] = mi->m_lightmap[i].z;
        }
    }
    return 1;
}

// Number of radiosity links the reference generated (lighter.cpp:755-757).
__attribute__((visibility("default"))) u32 ltrdbg_RadLinkCount(ltr_Scene* s)
{
    return (u32) s->m_radLinks.size();
}

// Table-driven sample_fn: config->userdata points at
//   { u32 count; const float* diffuse_rgb; const float* emissive_rgb; }
// and the entry is selected by (u32) req->tex0u, i.e. the mesh's first UV
// channel carries a face id. Out-of-range ids keep the defaults.
struct ltrg_SampleTable { u32 count; const float* diffuse_rgb; const float* emissive_rgb; };

__attribute__((visibility("default"))) int ltrg_TableSampleFn(ltr_Config* cfg, ltr_SampleRequest* req)
{
    const ltrg_SampleTable* t = (const ltrg_SampleTable*) cfg->userdata;
    if (!t) return 0;
    float fid = req->tex0u;
    if (!(fid >= 0.0f)) return 0;
    u32 id = (u32) fid;
    if (id >= t->count) return 0;
    if (t->diffuse_rgb) {
        req->out_diffuse_color[0] = t->diffuse_rgb[id*3+0];
        req->out_diffuse_color[1] = t->diffuse_rgb[id*3+1];
        req->out_diffuse_color[2] = t->diffuse_rgb[id*3+2];
    }
    if (t->emissive_rgb) {
        req->out_emissive_color[0] = t->emissive_rgb[id*3+0];
        req->out_emissive_color[1] = t->emissive_rgb[id*3+1];
        req->out_emissive_color[2] = t->emissive_rgb[id*3+2];
    }
    return 1;
}

}  // extern "C"
