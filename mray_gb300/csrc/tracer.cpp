// tracer.cpp -- MRay's TracerI (Source/Core/TracerI.h:150-376) over the
// library's accelerator and path tracer: typed groups, reservations and
// attribute pushes are host bookkeeping; mrg_tracer_commit_surfaces turns
// them into meshes, instances, materials and lights of one mrg_ctx, and the
// renderer calls drive mrg_pt_render over a device film.
//
// What follows MRay (TracerBase.cpp):
//   - the implicit groups 0 ((P)Empty, (Mt)Passthrough, (T)Identity with
//     transform 0, (L)Null with light 0, (Md)Vacuum), returned when their
//     names are created (TracerBase.cpp:579-600, 905-925, 1010-1035);
//   - ids as MRay's keys (TracerTypes.h:168-174), counters per kind;
//   - reservations before the commit, pushes after it, inclusive id ranges
//     (SceneLoaderMRay.cpp:1195-1215);
//   - surfaces become instances in creation order, then light surfaces;
//     light surfaces are never back-face culled (AcceleratorGroup::
//     LinearizeSurfaceData, AcceleratorCommon.cu:255-365);
//   - the renderer's options and defaults (PathTracerRendererShaders.h:36-45,
//     PathTracerRenderer.cu:128-142, 1386-1400).
#include "mray_gb300_tracer.h"
#include "mrg_ctx.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace {

constexpr uint32_t kPrimBatchShift = 28, kMatShift = 21, kTransShift = 24, kCamShift = 24;

struct Attr
{
    const char* name;
    uint32_t    dt;
    uint32_t    optional;
    uint32_t    texturable;
    uint32_t    isColor;
};

uint32_t dt_bytes(uint32_t dt)
{
    static const uint32_t b[] = { 4, 8, 12, 16, 16, 64, 4, 8, 12, 1, 0 };
    return dt <= MRG_DT_STRING ? b[dt] : 0u;
}

enum : uint32_t { kLightPrim = 1, kLightSky = 2, kRendRGB = 0, kRendSpectral = 1, kRendGuided = 2 };

struct TypeDef
{
    const char*       name;
    std::vector<Attr> attrs;
    uint32_t          code;       // material MRG_MAT_*, light kind, renderer kind
    bool              implicit;   // creation returns group 0
};

const std::vector<TypeDef>& types(uint32_t kind)
{
    using A = Attr;
    static const std::vector<TypeDef> prim = {
        { "(P)Triangle", { A{ "position", MRG_DT_VECTOR_3, 0, 0, 0 }, A{ "normal", MRG_DT_QUATERNION, 0, 0, 0 },
                           A{ "uv0", MRG_DT_VECTOR_2, 0, 0, 0 }, A{ "index", MRG_DT_VECTOR_3UI, 0, 0, 0 } }, 0, false },
        { "(P)Empty", {}, 0, true } };
    static const A albedo{ "albedo", MRG_DT_VECTOR_3, 0, MRG_ATTR_TEXTURE_OR_CONSTANT, 1 };
    static const A normalMap{ "normalMap", MRG_DT_VECTOR_3, 1, MRG_ATTR_TEXTURE_ONLY, 0 };
    static const std::vector<TypeDef> mat = {
        { "(Mt)Lambert", { albedo, normalMap }, MRG_MAT_LAMBERT, false },
        { "(Mt)Reflect", {}, MRG_MAT_REFLECT, false },
        { "(Mt)Refract", { A{ "cauchyBack", MRG_DT_VECTOR_3, 0, 0, 0 }, A{ "cauchyFront", MRG_DT_VECTOR_3, 0, 0, 0 } },
          MRG_MAT_REFRACT, false },
        { "(Mt)Unreal", { albedo, normalMap, A{ "roughness", MRG_DT_FLOAT, 0, MRG_ATTR_TEXTURE_OR_CONSTANT, 0 },
                          A{ "specular", MRG_DT_FLOAT, 0, MRG_ATTR_TEXTURE_OR_CONSTANT, 0 },
                          A{ "metallic", MRG_DT_FLOAT, 0, MRG_ATTR_TEXTURE_OR_CONSTANT, 0 } }, MRG_MAT_UNREAL, false },
        { "(Mt)Passthrough", {}, 0, true } };
    static const std::vector<TypeDef> trans = {
        { "(T)Single", { A{ "Transform", MRG_DT_MATRIX_4x4, 0, 0, 0 } }, 1, false },
        { "(T)Identity", {}, 0, true } };
    static const std::vector<TypeDef> cam = {
        { "(C)Pinhole", { A{ "FovAndPlanes", MRG_DT_VECTOR_4, 0, 0, 0 }, A{ "gaze", MRG_DT_VECTOR_3, 0, 0, 0 },
                          A{ "position", MRG_DT_VECTOR_3, 0, 0, 0 }, A{ "up", MRG_DT_VECTOR_3, 0, 0, 0 } }, 0, false } };
    static const std::vector<TypeDef> medium = { { "(Md)Vacuum", {}, 0, true } };
    static const A radiance{ "radiance", MRG_DT_VECTOR_3, 0, MRG_ATTR_TEXTURE_OR_CONSTANT, 1 };
    static const std::vector<TypeDef> light = {
        { "(L)Prim(P)Triangle", { radiance, A{ "isTwoSided", MRG_DT_BOOL, 0, 0, 0 } }, kLightPrim, false },
        { "(L)Skysphere_Spherical", { radiance }, kLightSky, false },
        { "(L)Null", {}, 0, true } };
    static const std::vector<Attr> rattr = {
        A{ "totalSPP", MRG_DT_UINT32, 0, 0, 0 }, A{ "burstSize", MRG_DT_UINT32, 1, 0, 0 },
        A{ "renderMode", MRG_DT_STRING, 0, 0, 0 }, A{ "sampleMode", MRG_DT_STRING, 0, 0, 0 },
        A{ "rrRange", MRG_DT_VECTOR_2UI, 0, 0, 0 }, A{ "neeSamplerType", MRG_DT_STRING, 0, 0, 0 } };
    // GuidedPTRenderer::StaticAttributeInfo (GuidedPTRenderer.cu:1273-1292)
    static const std::vector<Attr> gattr = {
        A{ "cacheEntryLimit", MRG_DT_UINT32, 1, 0, 0 }, A{ "cachePosBits", MRG_DT_UINT32, 1, 0, 0 },
        A{ "cacheNormalBits", MRG_DT_UINT32, 1, 0, 0 }, A{ "cacheMaxLvlOffset", MRG_DT_UINT32, 1, 0, 0 },
        A{ "cacheConeAperture", MRG_DT_FLOAT, 1, 0, 0 }, A{ "rrRange", MRG_DT_VECTOR_2UI, 0, 0, 0 },
        A{ "totalSPP", MRG_DT_UINT32, 0, 0, 0 }, A{ "lightSampler", MRG_DT_STRING, 1, 0, 0 },
        A{ "renderMode", MRG_DT_STRING, 0, 0, 0 }, A{ "burstSize", MRG_DT_UINT32, 1, 0, 0 },
        A{ "lobeProbability", MRG_DT_FLOAT, 1, 0, 0 }, A{ "displayMode", MRG_DT_STRING, 0, 0, 0 } };
    static const std::vector<TypeDef> rend = { { "(R)PathTracerRGB", rattr, kRendRGB, false },
                                               { "(R)PathTracerSpectral", rattr, kRendSpectral, false },
                                               { "(R)GuidedPathTracerSpectral", gattr, kRendGuided, false } };
    static const std::vector<TypeDef> none;
    switch(kind)
    {
        case MRG_KIND_PRIM: return prim;
        case MRG_KIND_MATERIAL: return mat;
        case MRG_KIND_TRANSFORM: return trans;
        case MRG_KIND_CAMERA: return cam;
        case MRG_KIND_MEDIUM: return medium;
        case MRG_KIND_LIGHT: return light;
        case MRG_KIND_RENDERER: return rend;
        default: return none;
    }
}

int find_type(uint32_t kind, const char* name)
{
    if(!name) return -1;
    const auto& v = types(kind);
    for(size_t i = 0; i < v.size(); i++)
        if(std::strcmp(v[i].name, name) == 0) return (int)i;
    return -1;
}

const char* kind_name(uint32_t kind)
{
    static const char* n[] = { "PrimitiveGroup", "MaterialGroup", "TransformGroup", "CameraGroup", "MediumGroup",
                               "LightGroup", "Renderer" };
    return kind <= MRG_KIND_RENDERER ? n[kind] : "Group";
}

mrg_status err(const std::string& msg) { return mrg::set_error(MRG_ERR_INVALID_ARG, msg); }

// A group of materials, transforms, lights or cameras: per attribute, the
// items' values, texture ids and pushed flags.
struct Group
{
    int      type = -1;
    bool     committed = false;
    bool     implicit = false;
    uint32_t count = 0;
    std::vector<std::vector<uint8_t>>  data;
    std::vector<std::vector<uint32_t>> tex;
    std::vector<std::vector<uint8_t>>  pushed;
    uint32_t primGroup = 0;                    // primitive-backed lights
    std::vector<uint32_t> primBatch;           // per light
};

struct PrimBatch
{
    uint32_t primCount = 0, attribCount = 0;
    uint32_t primBase = 0;                     // first primitive key of the batch in its group
    std::vector<float>    pos, normal, uv;
    std::vector<uint32_t> idx;
    std::vector<uint8_t>  pushed[4];           // per item
    uint32_t meshId = 0xFFFFFFFFu;
};

struct PrimGroup
{
    int  type = -1;
    bool committed = false;
    bool implicit = false;
    std::vector<PrimBatch> batches;
    uint32_t primTotal = 0;
};

struct Texture
{
    uint32_t w = 0, h = 0, mips = 0, pixel = 0;
    bool committed = false;
    std::vector<uint8_t> mip0;
    bool mip0Set = false;
    std::vector<std::vector<uint8_t>> upper;   // pushed levels >= 1 (index = level), empty = not pushed
    uint32_t ptId = 0xFFFFFFFFu;               // the path tracer's texture, after the surface commit
};

struct LightSurf { uint32_t light, transform; };
struct CamSurf   { uint32_t cam, transform; };

struct Renderer
{
    int      type = -1;
    bool     alive = false;
    uint32_t totalSpp = 16384, burst = 1;
    uint32_t sampleMode = MRG_PT_PURE;
    uint32_t rrStart = 4, maxDepth = 20;
    mrg_guide_params guide{};      // the guided renderer's grid options
};

struct Spectral
{
    uint32_t lutRes = 0, cieCount = 0;
    std::vector<float> lut, cie, spd;
    float integrals[3] = { 0, 0, 0 }, norm = 0, xyzToRgb[9] = {};
};

bool fully(const std::vector<uint8_t>& v)
{
    return std::all_of(v.begin(), v.end(), [](uint8_t x) { return x != 0; });
}

} // namespace

struct mrg_tracer
{
    mutable std::mutex m;
    mrg_tracer_params  params{};
    mrg_ctx*           ctx = nullptr;
    bool               surfacesCommitted = false;
    bool               texturesCommitted = false;

    std::vector<PrimGroup> prims;              // index = group id
    std::vector<Group>     groups[7];          // per kind (materials, transforms, lights, cameras, media)
    std::vector<Texture>   textures;           // index = texture id - 1
    std::vector<mrg_tracer_surface> surfaces;
    std::vector<LightSurf> lightSurfaces;
    bool      hasBoundary = false;
    LightSurf boundary{ 0, 0 };
    uint32_t  boundaryId = 0;
    uint32_t  lightSurfaceCounter = 0;
    std::vector<CamSurf>   camSurfaces;
    std::vector<Renderer>  renderers;
    Spectral  spectral;

    // rendering
    bool          rendering = false;
    uint32_t      renderer = 0;
    mrg_pt_params P{};
    float*        dFilm = nullptr;
    uint32_t      done = 0, totalSpp = 0, burst = 1;
    cudaEvent_t   ev[2] = { nullptr, nullptr };

    void reset_scene()
    {
        prims.clear();
        for(auto& g : groups) g.clear();
        // implicit groups 0
        PrimGroup e; e.implicit = true; e.committed = true; e.type = find_type(MRG_KIND_PRIM, "(P)Empty");
        prims.push_back(e);
        const uint32_t implicitKinds[] = { MRG_KIND_MATERIAL, MRG_KIND_TRANSFORM, MRG_KIND_MEDIUM, MRG_KIND_LIGHT };
        const char* implicitNames[] = { "(Mt)Passthrough", "(T)Identity", "(Md)Vacuum", "(L)Null" };
        for(int k = 0; k < 4; k++)
        {
            Group g;
            g.implicit = true;
            g.committed = true;
            g.count = 1;
            g.type = find_type(implicitKinds[k], implicitNames[k]);
            g.primBatch.push_back(0);
            groups[implicitKinds[k]].push_back(g);
        }
        textures.clear();
        surfaces.clear();
        lightSurfaces.clear();
        camSurfaces.clear();
        hasBoundary = false;
        lightSurfaceCounter = 0;
        surfacesCommitted = false;
        texturesCommitted = false;
    }

    void stop()
    {
        cudaFree(dFilm);
        dFilm = nullptr;
        rendering = false;
        done = 0;
    }

    void release_device()
    {
        stop();
        for(auto& e : ev)
            if(e) { cudaEventDestroy(e); e = nullptr; }
        if(ctx) mrg_destroy(ctx);
        ctx = nullptr;
    }
};

namespace {

uint32_t shift_of(uint32_t kind)
{
    switch(kind)
    {
        case MRG_KIND_MATERIAL: case MRG_KIND_LIGHT: return kMatShift;
        case MRG_KIND_TRANSFORM: return kTransShift;
        case MRG_KIND_CAMERA: case MRG_KIND_MEDIUM: return kCamShift;
        default: return kPrimBatchShift;
    }
}

// The group `gid` of `kind`, or an error naming it.
mrg_status get_group(mrg_tracer* t, uint32_t kind, uint32_t gid, Group*& g)
{
    if(gid >= t->groups[kind].size())
        return err(std::string("Unable to find ") + kind_name(kind) + "(" + std::to_string(gid) + ")");
    g = &t->groups[kind][gid];
    return MRG_OK;
}

mrg_status create_group(mrg_tracer* t, uint32_t kind, const char* name, uint32_t* gid)
{
    if(!gid) return err("null output id");
    if(t->surfacesCommitted) return err("surfaces are committed; ClearAll first");
    const int ty = find_type(kind, name);
    if(ty < 0) return err(std::string("Unable to find generator for ") + (name ? name : "(null)"));
    const TypeDef& td = types(kind)[ty];
    if(td.implicit)
    {
        if(kind == MRG_KIND_CAMERA || kind == MRG_KIND_RENDERER) return err("no implicit group");
        *gid = 0;
        return MRG_OK;
    }
    auto& v = t->groups[kind];
    if(v.size() >= (1ull << (32 - shift_of(kind))))
        return mrg::set_error(MRG_ERR_LIMIT, std::string("Too many ") + kind_name(kind) + "s");
    Group g;
    g.type = ty;
    g.data.resize(td.attrs.size());
    g.tex.resize(td.attrs.size());
    g.pushed.resize(td.attrs.size());
    *gid = (uint32_t)v.size();
    v.push_back(std::move(g));
    return MRG_OK;
}

mrg_status reserve(mrg_tracer* t, uint32_t kind, uint32_t gid, uint32_t n, uint32_t* ids)
{
    Group* g;
    mrg_status s = get_group(t, kind, gid, g);
    if(s != MRG_OK) return s;
    if(n && !ids) return err("null output ids");
    if(g->implicit)
    {
        for(uint32_t i = 0; i < n; i++) ids[i] = gid << shift_of(kind);
        return MRG_OK;
    }
    if(g->committed)
        return err(std::string(kind_name(kind)) + "(" + std::to_string(gid) + ") is committed; no more reservations");
    const uint64_t limit = 1ull << shift_of(kind);
    if((uint64_t)g->count + n > limit) return mrg::set_error(MRG_ERR_LIMIT, "too many items in one group");
    for(uint32_t i = 0; i < n; i++) ids[i] = (gid << shift_of(kind)) | (g->count + i);
    g->count += n;
    return MRG_OK;
}

mrg_status commit_group(mrg_tracer* t, uint32_t kind, uint32_t gid)
{
    Group* g;
    mrg_status s = get_group(t, kind, gid, g);
    if(s != MRG_OK) return s;
    if(g->implicit) return MRG_OK;
    if(g->committed) return err(std::string(kind_name(kind)) + "(" + std::to_string(gid) + ") is already committed");
    const TypeDef& td = types(kind)[g->type];
    for(size_t a = 0; a < td.attrs.size(); a++)
    {
        const uint32_t eb = std::max<uint32_t>(dt_bytes(td.attrs[a].dt), 1u);
        g->data[a].assign((size_t)g->count * eb, 0);
        g->tex[a].assign(g->count, 0);
        g->pushed[a].assign(g->count, 0);
    }
    if(g->primBatch.size() < g->count) g->primBatch.resize(g->count, 0);
    g->committed = true;
    return MRG_OK;
}

mrg_status is_committed(const mrg_tracer* t, uint32_t kind, uint32_t gid, uint32_t* out)
{
    if(!out) return err("null output");
    if(gid >= t->groups[kind].size())
        return err(std::string("Unable to find ") + kind_name(kind) + "(" + std::to_string(gid) + ")");
    *out = t->groups[kind][gid].committed ? 1u : 0u;
    return MRG_OK;
}

mrg_status push_group(mrg_tracer* t, uint32_t kind, uint32_t gid, uint32_t idBegin, uint32_t idEnd, uint32_t ai,
                      const void* data, size_t bytes, const uint32_t* texs)
{
    Group* g;
    mrg_status s = get_group(t, kind, gid, g);
    if(s != MRG_OK) return s;
    if(g->implicit) return err(std::string(kind_name(kind)) + "(0) takes no attributes");
    if(!g->committed) return err(std::string(kind_name(kind)) + "(" + std::to_string(gid) + ") is not committed");
    const TypeDef& td = types(kind)[g->type];
    if(ai >= td.attrs.size()) return err(std::string(td.name) + ": unknown attribute index " + std::to_string(ai));
    const Attr& at = td.attrs[ai];
    const uint32_t sh = shift_of(kind);
    if((idBegin >> sh) != gid || (idEnd >> sh) != gid) return err(std::string(td.name) + ": id range outside the group");
    const uint32_t b = idBegin & ((1u << sh) - 1u), e = idEnd & ((1u << sh) - 1u);
    if(e < b || e >= g->count) return err(std::string(td.name) + ": id range outside the reservations");
    const uint32_t n = e - b + 1u;
    const uint32_t eb = dt_bytes(at.dt);
    if(texs && at.texturable == MRG_ATTR_CONSTANT_ONLY)
        return err(std::string(td.name) + ": attribute \"" + at.name + "\" is not texturable");
    if(!texs && at.texturable == MRG_ATTR_TEXTURE_ONLY)
        return err(std::string(td.name) + ": attribute \"" + at.name + "\" takes textures only");
    bool needData = at.texturable != MRG_ATTR_TEXTURE_ONLY;
    if(texs && needData && !data)
    {
        for(uint32_t i = 0; i < n; i++)
            if(texs[i] == 0) return err(std::string(td.name) + ": constant missing for an item without a texture");
        needData = false;
    }
    if(needData)
    {
        if(!data || bytes != (size_t)n * eb)
            return err(std::string(td.name) + ": attribute \"" + at.name + "\" wants " + std::to_string((size_t)n * eb) +
                       " bytes, got " + std::to_string(bytes));
    }
    for(uint32_t i = 0; i < n; i++)
    {
        const uint32_t tid = texs ? texs[i] : 0u;
        if(tid && (tid > t->textures.size())) return err(std::string(td.name) + ": unknown texture " + std::to_string(tid));
    }
    if(needData) std::memcpy(g->data[ai].data() + (size_t)b * eb, data, bytes);
    for(uint32_t i = 0; i < n; i++)
    {
        g->tex[ai][b + i] = texs ? texs[i] : 0u;
        g->pushed[ai][b + i] = 1;
    }
    return MRG_OK;
}

// Item `id` of a group of `kind`: group and index, checked.
mrg_status item(mrg_tracer* t, uint32_t kind, uint32_t id, Group*& g, uint32_t& index)
{
    const uint32_t sh = shift_of(kind);
    mrg_status s = get_group(t, kind, id >> sh, g);
    if(s != MRG_OK) return s;
    index = id & ((1u << sh) - 1u);
    if(index >= g->count) return err(std::string(kind_name(kind)) + ": id " + std::to_string(id) + " was not reserved");
    return MRG_OK;
}

// The same, for reading its attributes: the group must be committed.
mrg_status committed_item(mrg_tracer* t, uint32_t kind, uint32_t id, Group*& g, uint32_t& index)
{
    mrg_status s = item(t, kind, id, g, index);
    if(s != MRG_OK) return s;
    if(!g->committed)
        return err(std::string(kind_name(kind)) + "(" + std::to_string(id >> shift_of(kind)) + ") is not committed");
    return MRG_OK;
}

template<class T> T value(const Group& g, uint32_t attr, uint32_t index)
{
    T v;
    std::memcpy(&v, g.data[attr].data() + (size_t)index * sizeof(T), sizeof(T));
    return v;
}

// Row-major 3x4 of a transform id.
mrg_status transform_of(mrg_tracer* t, uint32_t id, float m34[12])
{
    Group* g;
    uint32_t k;
    mrg_status s = committed_item(t, MRG_KIND_TRANSFORM, id, g, k);
    if(s != MRG_OK) return s;
    for(int i = 0; i < 12; i++) m34[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    if(g->implicit) return MRG_OK;
    if(!g->pushed[0][k]) return err("Transform " + std::to_string(id) + " has no matrix");
    std::memcpy(m34, g->data[0].data() + (size_t)k * 64, 12 * sizeof(float));
    return MRG_OK;
}

// n texels of a pushed level in RGBA f32 (single-channel types as r, r, r, 1)
void level_rgba_f32(uint32_t pixel, const uint8_t* data, size_t n, std::vector<float>& out)
{
    out.resize(4 * n);
    const float* f = reinterpret_cast<const float*>(data);
    for(size_t i = 0; i < n; i++)
    {
        float* o = &out[4 * i];
        switch(pixel)
        {
            case MRG_PIX_RGBA_FLOAT: o[0] = f[4 * i]; o[1] = f[4 * i + 1]; o[2] = f[4 * i + 2]; o[3] = f[4 * i + 3]; break;
            case MRG_PIX_RGB_FLOAT:  o[0] = f[3 * i]; o[1] = f[3 * i + 1]; o[2] = f[3 * i + 2]; o[3] = 1.0f; break;
            case MRG_PIX_R_FLOAT:    o[0] = o[1] = o[2] = f[i]; o[3] = 1.0f; break;
            case MRG_PIX_R8_UNORM:   o[0] = o[1] = o[2] = (float)data[i] / 255.0f; o[3] = 1.0f; break;
            default: for(int k = 0; k < 4; k++) o[k] = (float)data[4 * i + k] / 255.0f; break;
        }
    }
}

// A pushed level in the path tracer's own texture form: RGBA8 stays as it
// is, R8 becomes RGBA8 (r, r, r, 255) so that it keeps the UNORM read, the
// float types become RGBA f32.
const void* level_for_pt(uint32_t pixel, const std::vector<uint8_t>& in, size_t n, std::vector<uint8_t>& b8,
                         std::vector<float>& f32)
{
    if(pixel == MRG_PIX_RGBA8_UNORM || pixel == MRG_PIX_RGBA_FLOAT) return in.data();
    if(pixel == MRG_PIX_R8_UNORM)
    {
        b8.resize(4 * n);
        for(size_t i = 0; i < n; i++) { b8[4 * i] = b8[4 * i + 1] = b8[4 * i + 2] = in[i]; b8[4 * i + 3] = 255; }
        return b8.data();
    }
    level_rgba_f32(pixel, in.data(), n, f32);
    return f32.data();
}

mrg_status texture_rgba_f32(mrg_tracer* t, uint32_t tid, std::vector<float>& out, uint32_t& w, uint32_t& h)
{
    if(tid == 0 || tid > t->textures.size()) return err("unknown texture " + std::to_string(tid));
    const Texture& x = t->textures[tid - 1];
    if(!x.mip0Set) return err("texture " + std::to_string(tid) + " has no data");
    w = x.w; h = x.h;
    level_rgba_f32(x.pixel, x.mip0.data(), (size_t)x.w * x.h, out);
    return MRG_OK;
}

// The path tracer's texture of texture id `tid`, uploaded once.
mrg_status pt_texture(mrg_tracer* t, uint32_t tid, uint32_t& ptId)
{
    if(tid == 0 || tid > t->textures.size()) return err("unknown texture " + std::to_string(tid));
    Texture& x = t->textures[tid - 1];
    if(x.ptId != 0xFFFFFFFFu) { ptId = x.ptId; return MRG_OK; }
    if(!x.mip0Set) return err("texture " + std::to_string(tid) + " has no data");
    mrg_status s;
    uint32_t id = 0;
    const bool unorm = x.pixel == MRG_PIX_RGBA8_UNORM || x.pixel == MRG_PIX_R8_UNORM;
    std::vector<uint8_t> b8;
    std::vector<float> f32;
    s = mrg_pt_add_texture(t->ctx, x.w, x.h, unorm ? MRG_TEX_RGBA8 : MRG_TEX_RGBA32F,
                           level_for_pt(x.pixel, x.mip0, (size_t)x.w * x.h, b8, f32), 0, &id);
    if(s != MRG_OK) return s;
    // mips: TracerParameters::genMips fills every level the texture does not
    // have with mipGenFilter (TextureMemory.cpp:588-591, 826-830); pushed
    // levels are kept either way
    if(t->params.genMips)
    {
        const float r = t->params.mipGenFilterRadius > 0.0f ? t->params.mipGenFilterRadius : 2.0f;
        if((s = mrg_pt_generate_mips(t->ctx, id, r)) != MRG_OK) return s;
    }
    for(uint32_t m = 1; m < x.upper.size(); m++)
    {
        if(x.upper[m].empty()) continue;
        const size_t n = (size_t)std::max(x.w >> m, 1u) * std::max(x.h >> m, 1u);
        s = mrg_pt_set_texture_mip(t->ctx, id, m, level_for_pt(x.pixel, x.upper[m], n, b8, f32));
        if(s != MRG_OK) return s;
    }
    x.ptId = ptId = id;
    return MRG_OK;
}

// A surface material as the path tracer's description.
mrg_status material_of(mrg_tracer* t, uint32_t mid, mrg_pt_material& m, uint32_t& albedoTex, uint32_t paramTex[3])
{
    Group* g;
    uint32_t k;
    mrg_status s = committed_item(t, MRG_KIND_MATERIAL, mid, g, k);
    if(s != MRG_OK) return s;
    if(g->implicit) return err("(Mt)Passthrough surfaces are not rendered by this tracer (no media)");
    const TypeDef& td = types(MRG_KIND_MATERIAL)[g->type];
    for(size_t a = 0; a < td.attrs.size(); a++)
        if(!td.attrs[a].optional && !g->pushed[a][k])
            return err(std::string(td.name) + ": material " + std::to_string(mid) + " lacks \"" + td.attrs[a].name + "\"");
    m = mrg_pt_material{};
    m.type = td.code;
    m.specular = 0.5f;
    m.iorFront = 1.0f; m.iorBack = 1.5f;
    albedoTex = 0;
    paramTex[0] = paramTex[1] = paramTex[2] = 0;
    auto vec3 = [&](uint32_t a, float* o) { std::memcpy(o, g->data[a].data() + (size_t)k * 12, 12); };
    if(td.code == MRG_MAT_LAMBERT || td.code == MRG_MAT_UNREAL)
    {
        if(g->pushed[1][k] && g->tex[1][k]) return err(std::string(td.name) + ": normal maps are not supported");
        albedoTex = g->tex[0][k];
        if(!albedoTex) vec3(0, m.albedo);
    }
    if(td.code == MRG_MAT_UNREAL)
    {
        // roughness, specular, metallic: a texture (its first channel) or the constant
        m.roughness = g->tex[2][k] ? 0.0f : value<float>(*g, 2, k);
        m.specular = g->tex[3][k] ? 0.0f : value<float>(*g, 3, k);
        m.metallic = g->tex[4][k] ? 0.0f : value<float>(*g, 4, k);
        paramTex[0] = g->tex[2][k];
        paramTex[1] = g->tex[4][k];
        paramTex[2] = g->tex[3][k];
    }
    if(td.code == MRG_MAT_REFRACT)
    {
        float back[3], front[3];
        vec3(0, back);
        vec3(1, front);
        if(back[1] != 0.0f || back[2] != 0.0f || front[1] != 0.0f || front[2] != 0.0f)
            return err("(Mt)Refract: dispersive Cauchy coefficients are not supported");
        m.iorFront = front[0];
        m.iorBack = back[0];
    }
    return MRG_OK;
}

// Camera of a camera surface: position, gaze point, up, FovAndPlanes, with
// the surface's transform applied (points for position and gaze, the
// rotation for up), in double as the host loaders compute it.
mrg_status camera_of(const mrg_tracer* t, uint32_t csid, float cam[9], float fnp[4])
{
    if(csid >= t->camSurfaces.size()) return err("unknown camera surface " + std::to_string(csid));
    auto* tt = const_cast<mrg_tracer*>(t);
    const CamSurf& cs = t->camSurfaces[csid];
    Group* g;
    uint32_t k;
    mrg_status s = committed_item(tt, MRG_KIND_CAMERA, cs.cam, g, k);
    if(s != MRG_OK) return s;
    for(uint32_t a = 0; a < 4; a++)
        if(!g->pushed[a][k]) return err("(C)Pinhole: camera " + std::to_string(cs.cam) + " lacks an attribute");
    float m[12];
    if((s = transform_of(tt, cs.transform, m)) != MRG_OK) return s;
    std::memcpy(fnp, g->data[0].data() + (size_t)k * 16, 16);
    float gaze[3], pos[3], up[3];
    std::memcpy(gaze, g->data[1].data() + (size_t)k * 12, 12);
    std::memcpy(pos, g->data[2].data() + (size_t)k * 12, 12);
    std::memcpy(up, g->data[3].data() + (size_t)k * 12, 12);
    for(int r = 0; r < 3; r++)
    {
        double p = 0, q = 0, u = 0;
        for(int c = 0; c < 3; c++)
        {
            p += (double)m[4 * r + c] * pos[c];
            q += (double)m[4 * r + c] * gaze[c];
            u += (double)m[4 * r + c] * up[c];
        }
        cam[r] = (float)(p + m[4 * r + 3]);
        cam[3 + r] = (float)(q + m[4 * r + 3]);
        cam[6 + r] = (float)u;
    }
    return MRG_OK;
}

mrg_status prim_batch(mrg_tracer* t, uint32_t batchId, PrimGroup*& g, PrimBatch*& b)
{
    const uint32_t gid = batchId >> kPrimBatchShift, bi = batchId & ((1u << kPrimBatchShift) - 1u);
    if(gid >= t->prims.size()) return err("Unable to find PrimitiveGroup(" + std::to_string(gid) + ")");
    g = &t->prims[gid];
    if(g->implicit || bi >= g->batches.size()) return err("unknown primitive batch " + std::to_string(batchId));
    b = &g->batches[bi];
    return MRG_OK;
}

// Uploads a batch's mesh once (vertices in the batch's local indexing,
// primitive keys from the batch's base in its group).
mrg_status batch_mesh(mrg_tracer* t, uint32_t batchId, uint32_t& meshId)
{
    PrimGroup* g;
    PrimBatch* b;
    mrg_status s = prim_batch(t, batchId, g, b);
    if(s != MRG_OK) return s;
    if(b->meshId != 0xFFFFFFFFu) { meshId = b->meshId; return MRG_OK; }
    if(!g->committed) return err("PrimitiveGroup(" + std::to_string(batchId >> kPrimBatchShift) + ") is not committed");
    if(!fully(b->pushed[0]) || !fully(b->pushed[3]))
        return err("primitive batch " + std::to_string(batchId) + " lacks positions or indices");
    for(uint32_t v : b->idx)
        if(v >= b->attribCount) return err("primitive batch " + std::to_string(batchId) + ": index out of range");
    uint32_t id = 0;
    if((s = mrg_upload_mesh(t->ctx, b->pos.data(), b->attribCount, b->idx.data(), b->primCount, b->primBase, &id)) !=
       MRG_OK)
        return s;
    b->meshId = id;
    if(b->attribCount && fully(b->pushed[2]) &&
       (s = mrg_upload_mesh_uv(t->ctx, b->meshId, b->uv.data(), b->attribCount)) != MRG_OK)
        return s;
    meshId = b->meshId;
    return MRG_OK;
}

mrg_status commit_surfaces(mrg_tracer* t, mrg_tracer_commit_result* out)
{
    if(t->surfacesCommitted) return err("surfaces are already committed; ClearAll first");
    for(size_t i = 1; i < t->prims.size(); i++)
        if(!t->prims[i].committed) return err("PrimitiveGroup(" + std::to_string(i) + ") is not committed");
    mrg_params mp{};
    mp.device = t->params.device;
    mp.triangle_test = t->params.triangleTest;
    mrg_status s = mrg_create(&mp, &t->ctx);
    if(s != MRG_OK) { t->ctx = nullptr; return s; }
    uint32_t inst = 0;
    for(const auto& sf : t->surfaces)
    {
        float m[12];
        if((s = transform_of(t, sf.transformId, m)) != MRG_OK) return s;
        for(uint32_t j = 0; j < sf.count; j++)
        {
            uint32_t mesh, tex, ptex[3];
            mrg_pt_material mat;
            if((s = batch_mesh(t, sf.primBatches[j], mesh)) != MRG_OK) return s;
            if((s = material_of(t, sf.materials[j], mat, tex, ptex)) != MRG_OK) return s;
            uint32_t id;
            if((s = mrg_add_instance(t->ctx, mesh, m, sf.cullFace[j] ? MRG_INSTANCE_CULL_BACKFACE : 0u,
                                     sf.materials[j], inst, inst, &id)) != MRG_OK)
                return s;
            if((s = mrg_pt_set_material(t->ctx, id, &mat)) != MRG_OK) return s;
            if(tex)
            {
                uint32_t pid;
                if((s = pt_texture(t, tex, pid)) != MRG_OK) return s;
                if((s = mrg_pt_set_albedo_texture(t->ctx, id, pid)) != MRG_OK) return s;
            }
            if(ptex[0] | ptex[1] | ptex[2])
            {
                uint32_t pid[3] = { 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu };
                for(int q = 0; q < 3; q++)
                    if(ptex[q] && (s = pt_texture(t, ptex[q], pid[q])) != MRG_OK) return s;
                if((s = mrg_pt_set_unreal_textures(t->ctx, id, pid[0], pid[1], pid[2])) != MRG_OK) return s;
            }
            inst++;
        }
    }
    for(const auto& ls : t->lightSurfaces)
    {
        Group* g;
        uint32_t k;
        if((s = committed_item(t, MRG_KIND_LIGHT, ls.light, g, k)) != MRG_OK) return s;
        if(g->implicit) continue;                              // (L)Null: nothing to hit
        const TypeDef& td = types(MRG_KIND_LIGHT)[g->type];
        if(td.code != kLightPrim) return err(std::string(td.name) + " lights are boundary lights, not light surfaces");
        if(!g->pushed[0][k] || !g->pushed[1][k])
            return err(std::string(td.name) + ": light " + std::to_string(ls.light) + " lacks an attribute");
        if(g->tex[0][k]) return err(std::string(td.name) + ": textured radiance is not supported");
        float m[12], rad[3];
        if((s = transform_of(t, ls.transform, m)) != MRG_OK) return s;
        uint32_t mesh, id;
        if((s = batch_mesh(t, g->primBatch[k], mesh)) != MRG_OK) return s;
        if((s = mrg_add_instance(t->ctx, mesh, m, 0u, ls.light, inst, inst, &id)) != MRG_OK) return s;
        std::memcpy(rad, g->data[0].data() + (size_t)k * 12, 12);
        const uint32_t twoSided = g->data[1][k] ? 1u : 0u;
        if((s = mrg_pt_set_area_light(t->ctx, id, rad, twoSided)) != MRG_OK) return s;
        inst++;
    }
    if(t->hasBoundary)
    {
        Group* g;
        uint32_t k;
        if((s = committed_item(t, MRG_KIND_LIGHT, t->boundary.light, g, k)) != MRG_OK) return s;
        if(!g->implicit)
        {
            const TypeDef& td = types(MRG_KIND_LIGHT)[g->type];
            if(td.code != kLightSky) return err(std::string(td.name) + " cannot be the boundary light");
            if(!g->pushed[0][k]) return err(std::string(td.name) + ": boundary light lacks \"radiance\"");
            float m[12];
            if((s = transform_of(t, t->boundary.transform, m)) != MRG_OK) return s;
            std::vector<float> texels;
            uint32_t w = 1, h = 1;
            if(g->tex[0][k])
            {
                if((s = texture_rgba_f32(t, g->tex[0][k], texels, w, h)) != MRG_OK) return s;
            }
            else
            {
                texels.assign(4, 1.0f);
                std::memcpy(texels.data(), g->data[0].data() + (size_t)k * 12, 12);
            }
            if((s = mrg_pt_set_env(t->ctx, w, h, texels.data(), m)) != MRG_OK) return s;
        }
    }
    if((s = mrg_build(t->ctx)) != MRG_OK) return s;
    t->surfacesCommitted = true;
    if(out)
    {
        if((s = mrg_scene_aabb(t->ctx, out->aabb)) != MRG_OK) return s;
        mrg_accel_stats st;
        if((s = mrg_get_stats(t->ctx, &st)) != MRG_OK) return s;
        out->instanceCount = st.instances;
        out->acceleratorCount = st.accelerators;
    }
    return MRG_OK;
}

mrg_status cuda_status(cudaError_t e, const char* what)
{
    if(e == cudaSuccess) return MRG_OK;
    cudaGetLastError();
    return mrg::set_error(e == cudaErrorMemoryAllocation ? MRG_ERR_OUT_OF_MEMORY : MRG_ERR_CUDA,
                          std::string(what) + ": " + cudaGetErrorString(e));
}

mrg_status push_renderer(mrg_tracer* t, uint32_t rid, uint32_t ai, const void* data, size_t bytes)
{
    if(rid >= t->renderers.size() || !t->renderers[rid].alive) return err("unknown renderer " + std::to_string(rid));
    Renderer& r = t->renderers[rid];
    const TypeDef& td = types(MRG_KIND_RENDERER)[r.type];
    if(ai >= td.attrs.size()) return err(std::string(td.name) + " Unknown attribute index " + std::to_string(ai));
    if(!data) return err("null attribute data");
    const uint32_t dt = td.attrs[ai].dt;
    if(dt != MRG_DT_STRING && bytes != dt_bytes(dt))
        return err(std::string(td.name) + ": attribute \"" + td.attrs[ai].name + "\" wants " +
                   std::to_string(dt_bytes(dt)) + " bytes");
    const std::string str = dt == MRG_DT_STRING ? std::string(static_cast<const char*>(data), bytes) : std::string();
    uint32_t u[2] = { 0, 0 };
    if(dt != MRG_DT_STRING) std::memcpy(u, data, bytes);
    float f = 0.0f;
    if(dt == MRG_DT_FLOAT) std::memcpy(&f, data, 4);
    if(td.code == kRendGuided)
    {
        // GuidedPTRenderer::PushAttribute (GuidedPTRenderer.cu:489-540)
        switch(ai)
        {
            case 0:
                if(u[0] == 0 || u[0] > (1u << 27)) return err("cacheEntryLimit must be in [1, 2^27]");
                r.guide.entryLimit = u[0];
                break;
            case 1:
                if(u[0] > 15u) return err("cachePosBits exceeds the maximum 15");
                r.guide.posBits = u[0];
                break;
            case 2:
                if(u[0] > 3u) return err("cacheNormalBits exceeds the maximum 3");
                r.guide.normalBits = u[0];
                break;
            case 3: r.guide.maxLevelOffset = u[0]; break;
            case 4:
                if(!(f >= 0.0f)) return err("cacheConeAperture must be >= 0");
                r.guide.coneAperture = f;
                break;
            case 5:
                if(u[1] == 0 || u[0] > u[1]) return err("rrRange must satisfy start <= end, end > 0");
                r.rrStart = u[0]; r.maxDepth = u[1];
                break;
            case 6:
                if(u[0] == 0) return err("totalSPP must be positive");
                r.totalSpp = u[0];
                break;
            case 7:
                if(str != "Uniform") return err("unknown lightSampler \"" + str + "\" (Uniform only)");
                break;
            case 8:
                if(str != "Throughput" && str != "Latency") return err("unknown renderMode \"" + str + "\"");
                break;
            case 9: r.burst = std::max(1u, u[0]); break;
            case 10:
                if(!(f >= 0.0f && f <= 1.0f)) return err("lobeProbability must be in [0, 1]");
                r.guide.lobeProbability = f;
                break;
            case 11:
                // the debug displays (Grid, LightCache, MCTarget, ...) are
                // host-side reads of mrg_guide_read
                if(str != "Render") return err("displayMode \"" + str + "\": only Render is drawn");
                break;
        }
        return MRG_OK;
    }
    switch(ai)
    {
        case 0:
            if(u[0] == 0) return err("totalSPP must be positive");
            r.totalSpp = u[0];
            break;
        case 1: r.burst = std::max(1u, u[0]); break;
        case 2:
            if(str != "Throughput" && str != "Latency") return err("unknown renderMode \"" + str + "\"");
            break;
        case 3:
            if(str == "Pure") r.sampleMode = MRG_PT_PURE;
            else if(str == "WithNextEventEstimation") r.sampleMode = MRG_PT_NEE;
            else if(str == "WithNEEAndMIS") r.sampleMode = MRG_PT_NEE_MIS;
            else return err("unknown sampleMode \"" + str + "\"");
            break;
        case 4:
            if(u[1] == 0 || u[0] > u[1]) return err("rrRange must satisfy start <= end, end > 0");
            r.rrStart = u[0]; r.maxDepth = u[1];
            break;
        case 5:
            if(str != "Uniform") return err("unknown neeSamplerType \"" + str + "\" (Uniform only)");
            break;
    }
    return MRG_OK;
}

mrg_status start_render(mrg_tracer* t, uint32_t rid, uint32_t csid, uint32_t w, uint32_t h, const uint32_t* rmin,
                        const uint32_t* rmax, mrg_tracer_render_info* out)
{
    if(!t->surfacesCommitted) return err("StartRender before CommitSurfaces");
    if(rid >= t->renderers.size() || !t->renderers[rid].alive) return err("unknown renderer " + std::to_string(rid));
    if(w == 0 || h == 0) return err("empty film");
    if(rmin && rmax && (rmin[0] != 0 || rmin[1] != 0 || rmax[0] != w || rmax[1] != h))
        return err("only whole-film regions are rendered");
    const Renderer& r = t->renderers[rid];
    float cam[9], fnp[4];
    mrg_status s = camera_of(t, csid, cam, fnp);
    if(s != MRG_OK) return s;
    const uint32_t code = types(MRG_KIND_RENDERER)[r.type].code;
    const bool spectral = code == kRendSpectral || code == kRendGuided;
    if(code == kRendGuided && t->params.samplerType == MRG_TRACER_SAMPLER_ZSOBOL)
        return err("(R)GuidedPathTracerSpectral: the ZSobol sampler is not supported");
    if(spectral)
    {
        const Spectral& S = t->spectral;
        if(!S.lutRes)
            return err(std::string(types(MRG_KIND_RENDERER)[r.type].name) +
                       " needs the spectral data (mrg_tracer_set_spectral_data)");
        s = mrg_pt_set_spectral(t->ctx, S.lutRes, S.lut.data(), S.cieCount, S.cie.data(), S.integrals, S.spd.data(),
                                S.norm, S.xyzToRgb);
    }
    else
        s = mrg_pt_set_spectral(t->ctx, 0, nullptr, 0, nullptr, nullptr, nullptr, 0.0f, nullptr);
    if(s != MRG_OK) return s;
    t->stop();
    mrg_pt_params& P = t->P;
    P = mrg_pt_params{};
    P.width = w; P.height = h;
    P.rrStart = r.rrStart; P.maxDepth = r.maxDepth;
    P.sampleMode = r.sampleMode;
    P.seed = (uint32_t)(t->params.seed >> 32) ^ (uint32_t)t->params.seed;
    P.filterRadius = t->params.filmFilterRadius > 0.0f ? t->params.filmFilterRadius : 1.0f;
    std::memcpy(P.camPos, cam, 12);
    std::memcpy(P.camGaze, cam + 3, 12);
    std::memcpy(P.camUp, cam + 6, 12);
    P.fov[0] = fnp[0]; P.fov[1] = fnp[1];
    P.nearFar[0] = fnp[2]; P.nearFar[1] = fnp[3];
    P.partitionByMaterial = 2;
    P.sampler = t->params.samplerType == MRG_TRACER_SAMPLER_ZSOBOL ? MRG_PT_SAMPLER_ZSOBOL : MRG_PT_SAMPLER_PCG32;
    P.samplerMaxSpp = r.totalSpp;
    if((s = cuda_status(cudaSetDevice(t->params.device), "StartRender")) != MRG_OK) return s;
    // the guided renderer's grid is reset at every StartRender (HashGrid::Reset
    // over the scene box, GuidedPTRenderer.cu:1146-1161)
    if(code == kRendGuided && (s = mrg_guide_create(t->ctx, &r.guide)) != MRG_OK) return s;
    const size_t bytes = sizeof(float) * 4 * (size_t)w * h;
    if((s = cuda_status(cudaMalloc(&t->dFilm, bytes), "film")) != MRG_OK) return s;
    if((s = cuda_status(cudaMemset(t->dFilm, 0, bytes), "film")) != MRG_OK) return s;
    for(auto& e : t->ev)
        if(!e && (s = cuda_status(cudaEventCreate(&e), "events")) != MRG_OK) return s;
    t->rendering = true;
    t->renderer = rid;
    t->done = 0;
    t->totalSpp = r.totalSpp;
    t->burst = r.burst;
    if(out)
    {
        out->width = w; out->height = h;
        out->totalSpp = r.totalSpp;
        out->channels = 4;
        out->d_film = t->dFilm;
    }
    return MRG_OK;
}

mrg_status render_work(mrg_tracer* t, mrg_tracer_render_output* out)
{
    if(!t->rendering) return err("DoRenderWork without StartRender");
    mrg_tracer_render_output o{};
    const uint32_t n = std::min(t->burst, t->totalSpp - t->done);
    if(n)
    {
        t->P.spp = n;
        t->P.sampleStart = t->done;
        mrg_status s;
        if((s = cuda_status(cudaEventRecord(t->ev[0], nullptr), "DoRenderWork")) != MRG_OK) return s;
        const bool guided = types(MRG_KIND_RENDERER)[t->renderers[t->renderer].type].code == kRendGuided;
        if((s = guided ? mrg_pt_render_guided(t->ctx, &t->P, t->dFilm, nullptr)
                       : mrg_pt_render(t->ctx, &t->P, t->dFilm, nullptr)) != MRG_OK) return s;
        if((s = cuda_status(cudaEventRecord(t->ev[1], nullptr), "DoRenderWork")) != MRG_OK) return s;
        if((s = cuda_status(cudaEventSynchronize(t->ev[1]), "DoRenderWork")) != MRG_OK) return s;
        float ms = 0;
        cudaEventElapsedTime(&ms, t->ev[0], t->ev[1]);
        t->done += n;
        o.workMs = ms;
        o.pathsPerSecond = ms > 0 ? (double)t->P.width * t->P.height * n / (ms * 1e-3) : 0.0;
    }
    o.samplesDone = t->done;
    o.totalSpp = t->totalSpp;
    o.finished = t->done >= t->totalSpp ? 1u : 0u;
    if(out) *out = o;
    return MRG_OK;
}

} // namespace

#define TR_LOCK(t) if(!(t)) return err("null tracer"); std::lock_guard<std::mutex> lock_((t)->m)

extern "C" {

mrg_status mrg_tracer_create(const mrg_tracer_params* params, mrg_tracer** out)
{
    if(!out) return err("null output");
    *out = nullptr;
    mrg_tracer_params p = params ? *params : mrg_tracer_params{};
    if(p.samplerType > MRG_TRACER_SAMPLER_ZSOBOL) return err("unknown samplerType");
    if(p.triangleTest > MRG_TRI_WATERTIGHT) return err("unknown triangle test");
    if(p.device < 0) return err("bad device ordinal");
    if(!(p.filmFilterRadius >= 0.0f)) return err("film filter radius must be >= 0");
    if(!(p.mipGenFilterRadius >= 0.0f) || p.mipGenFilterRadius > 64.0f)
        return err("mip generation filter radius in [0, 64]");
    auto* t = new mrg_tracer;
    t->params = p;
    t->reset_scene();
    *out = t;
    return MRG_OK;
}

mrg_status mrg_tracer_destroy(mrg_tracer* t)
{
    if(!t) return MRG_OK;
    {
        std::lock_guard<std::mutex> lk(t->m);
        t->release_device();
    }
    delete t;
    return MRG_OK;
}

mrg_status mrg_tracer_parameters(const mrg_tracer* t, mrg_tracer_params* out)
{
    TR_LOCK(t);
    if(!out) return err("null output");
    *out = t->params;
    return MRG_OK;
}

mrg_status mrg_tracer_type_names(const mrg_tracer* t, uint32_t kind, char* buf, size_t cap, size_t* need)
{
    TR_LOCK(t);
    if(kind > MRG_KIND_RENDERER) return err("unknown kind");
    std::string s;
    for(const auto& td : types(kind))
    {
        if(td.implicit) continue;
        if(!s.empty()) s += '\n';
        s += td.name;
    }
    if(need) *need = s.size() + 1;
    if(buf)
    {
        if(cap < s.size() + 1) return err("buffer too small");
        std::memcpy(buf, s.c_str(), s.size() + 1);
    }
    return MRG_OK;
}

mrg_status mrg_tracer_attribute_info(const mrg_tracer* t, uint32_t kind, const char* type_name, uint32_t index,
                                     mrg_tracer_attrib_info* out, uint32_t* count)
{
    TR_LOCK(t);
    const int ty = find_type(kind, type_name);
    if(ty < 0) return err(std::string("Unable to find type ") + (type_name ? type_name : "(null)"));
    const TypeDef& td = types(kind)[ty];
    if(count) *count = (uint32_t)td.attrs.size();
    if(!out) return MRG_OK;
    if(index >= td.attrs.size()) return err(std::string(td.name) + ": attribute index out of range");
    const Attr& a = td.attrs[index];
    *out = mrg_tracer_attrib_info{};
    std::strncpy(out->name, a.name, sizeof(out->name) - 1);
    out->dataType = a.dt;
    out->elementBytes = dt_bytes(a.dt);
    out->optional = a.optional;
    out->texturable = a.texturable;
    out->isColor = a.isColor;
    return MRG_OK;
}

mrg_status mrg_tracer_group_type_name(const mrg_tracer* t, uint32_t kind, uint32_t group_id, char* buf, size_t cap)
{
    TR_LOCK(t);
    int ty = -1;
    if(kind == MRG_KIND_PRIM && group_id < t->prims.size()) ty = t->prims[group_id].type;
    else if(kind == MRG_KIND_RENDERER && group_id < t->renderers.size() && t->renderers[group_id].alive)
        ty = t->renderers[group_id].type;
    else if(kind <= MRG_KIND_LIGHT && kind != MRG_KIND_PRIM && group_id < t->groups[kind].size())
        ty = t->groups[kind][group_id].type;
    if(ty < 0) return err(std::string("Unable to find ") + kind_name(kind) + "(" + std::to_string(group_id) + ")");
    const char* n = types(kind)[ty].name;
    if(!buf || cap < std::strlen(n) + 1) return err("buffer too small");
    std::memcpy(buf, n, std::strlen(n) + 1);
    return MRG_OK;
}

// ---- primitives ----
mrg_status mrg_tracer_create_prim_group(mrg_tracer* t, const char* type_name, uint32_t* group_id)
{
    TR_LOCK(t);
    if(!group_id) return err("null output id");
    if(t->surfacesCommitted) return err("surfaces are committed; ClearAll first");
    const int ty = find_type(MRG_KIND_PRIM, type_name);
    if(ty < 0) return err(std::string("Unable to find generator for ") + (type_name ? type_name : "(null)"));
    if(types(MRG_KIND_PRIM)[ty].implicit) { *group_id = 0; return MRG_OK; }
    if(t->prims.size() >= (1u << (32 - kPrimBatchShift)))
        return mrg::set_error(MRG_ERR_LIMIT, "Too many PrimitiveGroups");
    PrimGroup g;
    g.type = ty;
    *group_id = (uint32_t)t->prims.size();
    t->prims.push_back(std::move(g));
    return MRG_OK;
}

mrg_status mrg_tracer_reserve_prim_batches(mrg_tracer* t, uint32_t group_id, const uint32_t* counts, uint32_t n,
                                           uint32_t* batch_ids)
{
    TR_LOCK(t);
    if(group_id >= t->prims.size()) return err("Unable to find PrimitiveGroup(" + std::to_string(group_id) + ")");
    PrimGroup& g = t->prims[group_id];
    if(g.implicit)
    {
        for(uint32_t i = 0; i < n && batch_ids; i++) batch_ids[i] = 0;
        return MRG_OK;
    }
    if(n && (!counts || !batch_ids)) return err("null counts or ids");
    if(g.committed) return err("PrimitiveGroup(" + std::to_string(group_id) + ") is committed; no more reservations");
    if((uint64_t)g.batches.size() + n > (1ull << kPrimBatchShift)) return mrg::set_error(MRG_ERR_LIMIT, "too many batches");
    uint64_t total = g.primTotal;
    for(uint32_t i = 0; i < n; i++) total += counts[2 * i];
    if(total > (1ull << kPrimBatchShift)) return mrg::set_error(MRG_ERR_LIMIT, "primitive keys must stay below 2^28");
    for(uint32_t i = 0; i < n; i++)
    {
        PrimBatch b;
        b.primCount = counts[2 * i];
        b.attribCount = counts[2 * i + 1];
        b.primBase = g.primTotal;
        g.primTotal += b.primCount;
        batch_ids[i] = (group_id << kPrimBatchShift) | (uint32_t)g.batches.size();
        g.batches.push_back(std::move(b));
    }
    return MRG_OK;
}

mrg_status mrg_tracer_commit_prim_reservations(mrg_tracer* t, uint32_t group_id)
{
    TR_LOCK(t);
    if(group_id >= t->prims.size()) return err("Unable to find PrimitiveGroup(" + std::to_string(group_id) + ")");
    PrimGroup& g = t->prims[group_id];
    if(g.implicit) return MRG_OK;
    if(g.committed) return err("PrimitiveGroup(" + std::to_string(group_id) + ") is already committed");
    for(auto& b : g.batches)
    {
        b.pos.assign(3ull * b.attribCount, 0.0f);
        b.normal.assign(4ull * b.attribCount, 0.0f);
        b.uv.assign(2ull * b.attribCount, 0.0f);
        b.idx.assign(3ull * b.primCount, 0u);
        for(int a = 0; a < 4; a++) b.pushed[a].assign(a == 3 ? b.primCount : b.attribCount, 0);
    }
    g.committed = true;
    return MRG_OK;
}

mrg_status mrg_tracer_is_prim_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out)
{
    TR_LOCK(t);
    if(!out) return err("null output");
    if(group_id >= t->prims.size()) return err("Unable to find PrimitiveGroup(" + std::to_string(group_id) + ")");
    *out = t->prims[group_id].committed ? 1u : 0u;
    return MRG_OK;
}

mrg_status mrg_tracer_push_prim_attribute(mrg_tracer* t, uint32_t group_id, uint32_t batch_id,
                                          uint32_t attribute_index, uint32_t sub_begin, uint32_t sub_end,
                                          const void* data, size_t bytes)
{
    TR_LOCK(t);
    if(group_id >= t->prims.size()) return err("Unable to find PrimitiveGroup(" + std::to_string(group_id) + ")");
    if((batch_id >> kPrimBatchShift) != group_id) return err("primitive batch of another group");
    PrimGroup* g;
    PrimBatch* b;
    mrg_status s = prim_batch(t, batch_id, g, b);
    if(s != MRG_OK) return s;
    if(!g->committed) return err("PrimitiveGroup(" + std::to_string(group_id) + ") is not committed");
    if(attribute_index > 3) return err("(P)Triangle: unknown attribute index " + std::to_string(attribute_index));
    const uint32_t items = attribute_index == 3 ? b->primCount : b->attribCount;
    if(sub_begin == 0 && sub_end == 0) sub_end = items;
    if(sub_end < sub_begin || sub_end > items) return err("(P)Triangle: sub-batch range outside the batch");
    static const uint32_t eb[4] = { 12, 16, 8, 12 };
    const size_t n = sub_end - sub_begin;
    if(!data || bytes != n * eb[attribute_index])
        return err("(P)Triangle: attribute " + std::to_string(attribute_index) + " wants " +
                   std::to_string(n * eb[attribute_index]) + " bytes, got " + std::to_string(bytes));
    void* dst = nullptr;
    switch(attribute_index)
    {
        case 0: dst = b->pos.data() + 3ull * sub_begin; break;
        case 1: dst = b->normal.data() + 4ull * sub_begin; break;
        case 2: dst = b->uv.data() + 2ull * sub_begin; break;
        default: dst = b->idx.data() + 3ull * sub_begin; break;
    }
    std::memcpy(dst, data, bytes);
    std::fill(b->pushed[attribute_index].begin() + sub_begin, b->pushed[attribute_index].begin() + sub_end, 1);
    return MRG_OK;
}

mrg_status mrg_tracer_transform_primitives(mrg_tracer* t, uint32_t group_id, const uint32_t* batch_ids,
                                           const float* m3x4, uint32_t n)
{
    TR_LOCK(t);
    if(n && (!batch_ids || !m3x4)) return err("null batches or matrices");
    if(t->surfacesCommitted) return err("surfaces are committed");
    for(uint32_t i = 0; i < n; i++)
    {
        if((batch_ids[i] >> kPrimBatchShift) != group_id) return err("primitive batch of another group");
        PrimGroup* g;
        PrimBatch* b;
        mrg_status s = prim_batch(t, batch_ids[i], g, b);
        if(s != MRG_OK) return s;
        if(!g->committed || !fully(b->pushed[0])) return err("TransformPrimitives before the positions were pushed");
        const float* m = m3x4 + 12ull * i;
        for(uint32_t v = 0; v < b->attribCount; v++)
        {
            float* p = &b->pos[3ull * v];
            const float x = p[0], y = p[1], z = p[2];
            for(int r = 0; r < 3; r++) p[r] = m[4 * r] * x + m[4 * r + 1] * y + m[4 * r + 2] * z + m[4 * r + 3];
        }
    }
    return MRG_OK;
}

// ---- materials / transforms / lights / cameras ----
mrg_status mrg_tracer_create_mat_group(mrg_tracer* t, const char* type_name, uint32_t* group_id)
{ TR_LOCK(t); return create_group(t, MRG_KIND_MATERIAL, type_name, group_id); }
mrg_status mrg_tracer_reserve_materials(mrg_tracer* t, uint32_t group_id, uint32_t n, uint32_t* ids)
{ TR_LOCK(t); return reserve(t, MRG_KIND_MATERIAL, group_id, n, ids); }
mrg_status mrg_tracer_commit_mat_reservations(mrg_tracer* t, uint32_t group_id)
{ TR_LOCK(t); return commit_group(t, MRG_KIND_MATERIAL, group_id); }
mrg_status mrg_tracer_is_mat_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out)
{ TR_LOCK(t); return is_committed(t, MRG_KIND_MATERIAL, group_id, out); }
mrg_status mrg_tracer_push_mat_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                         uint32_t attribute_index, const void* data, size_t bytes,
                                         const uint32_t* textures)
{ TR_LOCK(t); return push_group(t, MRG_KIND_MATERIAL, group_id, id_begin, id_end, attribute_index, data, bytes, textures); }

mrg_status mrg_tracer_create_trans_group(mrg_tracer* t, const char* type_name, uint32_t* group_id)
{ TR_LOCK(t); return create_group(t, MRG_KIND_TRANSFORM, type_name, group_id); }
mrg_status mrg_tracer_reserve_transforms(mrg_tracer* t, uint32_t group_id, uint32_t n, uint32_t* ids)
{ TR_LOCK(t); return reserve(t, MRG_KIND_TRANSFORM, group_id, n, ids); }
mrg_status mrg_tracer_commit_trans_reservations(mrg_tracer* t, uint32_t group_id)
{ TR_LOCK(t); return commit_group(t, MRG_KIND_TRANSFORM, group_id); }
mrg_status mrg_tracer_is_trans_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out)
{ TR_LOCK(t); return is_committed(t, MRG_KIND_TRANSFORM, group_id, out); }
mrg_status mrg_tracer_push_trans_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                           uint32_t attribute_index, const void* data, size_t bytes)
{ TR_LOCK(t); return push_group(t, MRG_KIND_TRANSFORM, group_id, id_begin, id_end, attribute_index, data, bytes, nullptr); }

mrg_status mrg_tracer_create_light_group(mrg_tracer* t, const char* type_name, uint32_t prim_group_id,
                                         uint32_t* group_id)
{
    TR_LOCK(t);
    const int ty = find_type(MRG_KIND_LIGHT, type_name);
    if(ty >= 0 && types(MRG_KIND_LIGHT)[ty].code == kLightPrim)
    {
        if(prim_group_id == 0 || prim_group_id >= t->prims.size())
            return err("Unable to locate PrimitiveGroup(" + std::to_string(prim_group_id) + ")");
        const char* pn = types(MRG_KIND_PRIM)[t->prims[prim_group_id].type].name;
        if(std::string(type_name) != std::string("(L)Prim") + pn)
            return err(std::string(type_name) + " does not light " + pn + " primitives");
    }
    mrg_status s = create_group(t, MRG_KIND_LIGHT, type_name, group_id);
    if(s == MRG_OK && *group_id != 0) t->groups[MRG_KIND_LIGHT][*group_id].primGroup = prim_group_id;
    return s;
}

mrg_status mrg_tracer_reserve_lights(mrg_tracer* t, uint32_t group_id, uint32_t n, const uint32_t* prim_batches,
                                     uint32_t* ids)
{
    TR_LOCK(t);
    Group* g;
    mrg_status s = get_group(t, MRG_KIND_LIGHT, group_id, g);
    if(s != MRG_OK) return s;
    const bool primBacked = !g->implicit && types(MRG_KIND_LIGHT)[g->type].code == kLightPrim;
    if(primBacked)
    {
        if(n && !prim_batches) return err("primitive-backed lights need their primitive batches");
        for(uint32_t i = 0; i < n; i++)
        {
            PrimGroup* pg;
            PrimBatch* pb;
            if((prim_batches[i] >> kPrimBatchShift) != g->primGroup) return err("light batch of another primitive group");
            if((s = prim_batch(t, prim_batches[i], pg, pb)) != MRG_OK) return s;
        }
    }
    const uint32_t first = g->count;
    if((s = reserve(t, MRG_KIND_LIGHT, group_id, n, ids)) != MRG_OK) return s;
    if(primBacked)
    {
        g->primBatch.resize(g->count, 0);
        for(uint32_t i = 0; i < n; i++) g->primBatch[first + i] = prim_batches[i];
    }
    return MRG_OK;
}

mrg_status mrg_tracer_commit_light_reservations(mrg_tracer* t, uint32_t group_id)
{ TR_LOCK(t); return commit_group(t, MRG_KIND_LIGHT, group_id); }
mrg_status mrg_tracer_is_light_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out)
{ TR_LOCK(t); return is_committed(t, MRG_KIND_LIGHT, group_id, out); }
mrg_status mrg_tracer_push_light_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                           uint32_t attribute_index, const void* data, size_t bytes,
                                           const uint32_t* textures)
{ TR_LOCK(t); return push_group(t, MRG_KIND_LIGHT, group_id, id_begin, id_end, attribute_index, data, bytes, textures); }

mrg_status mrg_tracer_create_camera_group(mrg_tracer* t, const char* type_name, uint32_t* group_id)
{ TR_LOCK(t); return create_group(t, MRG_KIND_CAMERA, type_name, group_id); }
mrg_status mrg_tracer_reserve_cameras(mrg_tracer* t, uint32_t group_id, uint32_t n, uint32_t* ids)
{ TR_LOCK(t); return reserve(t, MRG_KIND_CAMERA, group_id, n, ids); }
mrg_status mrg_tracer_commit_cam_reservations(mrg_tracer* t, uint32_t group_id)
{ TR_LOCK(t); return commit_group(t, MRG_KIND_CAMERA, group_id); }
mrg_status mrg_tracer_is_cam_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out)
{ TR_LOCK(t); return is_committed(t, MRG_KIND_CAMERA, group_id, out); }
mrg_status mrg_tracer_push_cam_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                         uint32_t attribute_index, const void* data, size_t bytes)
{ TR_LOCK(t); return push_group(t, MRG_KIND_CAMERA, group_id, id_begin, id_end, attribute_index, data, bytes, nullptr); }

// ---- textures ----
mrg_status mrg_tracer_create_texture2d(mrg_tracer* t, uint32_t width, uint32_t height, uint32_t mip_count,
                                       uint32_t pixel_type, uint32_t* texture_id)
{
    TR_LOCK(t);
    if(!texture_id) return err("null output id");
    if(t->texturesCommitted) return err("textures are committed; no more textures");
    if(width == 0 || height == 0 || mip_count == 0) return err("empty texture");
    if(pixel_type > MRG_PIX_R_FLOAT) return err("unsupported pixel type " + std::to_string(pixel_type));
    Texture x;
    x.w = width; x.h = height; x.mips = mip_count; x.pixel = pixel_type;
    t->textures.push_back(std::move(x));
    *texture_id = (uint32_t)t->textures.size();
    return MRG_OK;
}

mrg_status mrg_tracer_commit_textures(mrg_tracer* t)
{
    TR_LOCK(t);
    if(t->texturesCommitted) return err("textures are already committed");
    t->texturesCommitted = true;
    for(auto& x : t->textures) x.committed = true;
    return MRG_OK;
}

mrg_status mrg_tracer_push_texture_data(mrg_tracer* t, uint32_t texture_id, uint32_t mip_level, const void* data,
                                        size_t bytes)
{
    TR_LOCK(t);
    if(texture_id == 0 || texture_id > t->textures.size()) return err("unknown texture " + std::to_string(texture_id));
    Texture& x = t->textures[texture_id - 1];
    if(!x.committed) return err("PushTextureData before CommitTextures");
    if(mip_level >= x.mips) return err("mip level out of range");
    static const uint32_t pb[5] = { 4, 12, 16, 1, 4 };
    const size_t w = std::max(1u, x.w >> mip_level), h = std::max(1u, x.h >> mip_level);
    if(!data || bytes != w * h * pb[x.pixel])
        return err("texture " + std::to_string(texture_id) + " mip " + std::to_string(mip_level) + " wants " +
                   std::to_string(w * h * pb[x.pixel]) + " bytes");
    if(mip_level == 0)
    {
        x.mip0.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + bytes);
        x.mip0Set = true;
    }
    else
    {
        if(x.upper.size() < x.mips) x.upper.resize(x.mips);
        x.upper[mip_level].assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + bytes);
    }
    return MRG_OK;
}

// ---- surfaces ----
mrg_status mrg_tracer_create_surface(mrg_tracer* t, const mrg_tracer_surface* s, uint32_t* surface_id)
{
    TR_LOCK(t);
    if(!s || !surface_id) return err("null surface");
    if(t->surfacesCommitted) return err("surfaces are committed");
    if(s->count == 0 || s->count > MRG_TRACER_MAX_BATCHES_PER_SURFACE)
        return err("a surface holds 1 to 8 primitive batches");
    for(uint32_t j = 0; j < s->count; j++)
    {
        if(s->alphaMaps[j]) return err("alpha maps are not supported");
        if((s->primBatches[j] >> kPrimBatchShift) != (s->primBatches[0] >> kPrimBatchShift))
            return err("PrimitiveIds of a surface must be the same type!");
        PrimGroup* g;
        PrimBatch* b;
        mrg_status st = prim_batch(t, s->primBatches[j], g, b);
        if(st != MRG_OK) return st;
        Group* mg;
        uint32_t k;
        if((st = item(t, MRG_KIND_MATERIAL, s->materials[j], mg, k)) != MRG_OK) return st;
    }
    Group* tg;
    uint32_t k;
    mrg_status st = item(t, MRG_KIND_TRANSFORM, s->transformId, tg, k);
    if(st != MRG_OK) return st;
    *surface_id = (uint32_t)t->surfaces.size();
    t->surfaces.push_back(*s);
    return MRG_OK;
}

mrg_status mrg_tracer_set_boundary_surface(mrg_tracer* t, uint32_t light_id, uint32_t transform_id,
                                           uint32_t* light_surface_id)
{
    TR_LOCK(t);
    if(t->surfacesCommitted) return err("surfaces are committed");
    Group* g;
    uint32_t k;
    mrg_status s = item(t, MRG_KIND_LIGHT, light_id, g, k);
    if(s != MRG_OK) return s;
    if((s = item(t, MRG_KIND_TRANSFORM, transform_id, g, k)) != MRG_OK) return s;
    if(!t->hasBoundary) t->boundaryId = t->lightSurfaceCounter++;
    t->hasBoundary = true;
    t->boundary = LightSurf{ light_id, transform_id };
    if(light_surface_id) *light_surface_id = t->boundaryId;
    return MRG_OK;
}

mrg_status mrg_tracer_create_light_surface(mrg_tracer* t, uint32_t light_id, uint32_t transform_id,
                                           uint32_t* light_surface_id)
{
    TR_LOCK(t);
    if(t->surfacesCommitted) return err("surfaces are committed");
    Group* g;
    uint32_t k;
    mrg_status s = item(t, MRG_KIND_LIGHT, light_id, g, k);
    if(s != MRG_OK) return s;
    if((s = item(t, MRG_KIND_TRANSFORM, transform_id, g, k)) != MRG_OK) return s;
    t->lightSurfaces.push_back(LightSurf{ light_id, transform_id });
    const uint32_t id = t->lightSurfaceCounter++;
    if(light_surface_id) *light_surface_id = id;
    return MRG_OK;
}

mrg_status mrg_tracer_create_camera_surface(mrg_tracer* t, uint32_t camera_id, uint32_t transform_id,
                                            uint32_t* cam_surface_id)
{
    TR_LOCK(t);
    Group* g;
    uint32_t k;
    mrg_status s = item(t, MRG_KIND_CAMERA, camera_id, g, k);
    if(s != MRG_OK) return s;
    if((s = item(t, MRG_KIND_TRANSFORM, transform_id, g, k)) != MRG_OK) return s;
    if(cam_surface_id) *cam_surface_id = (uint32_t)t->camSurfaces.size();
    t->camSurfaces.push_back(CamSurf{ camera_id, transform_id });
    return MRG_OK;
}

mrg_status mrg_tracer_commit_surfaces(mrg_tracer* t, mrg_tracer_commit_result* out)
{
    TR_LOCK(t);
    mrg_status s = commit_surfaces(t, out);
    if(s != MRG_OK && !t->surfacesCommitted)
    {
        // leave no half-built device state behind; the scene stays as pushed
        const std::string keep = mrg_last_error();
        t->release_device();
        for(auto& g : t->prims)
            for(auto& b : g.batches) b.meshId = 0xFFFFFFFFu;
        for(auto& x : t->textures) x.ptId = 0xFFFFFFFFu;
        mrg::set_error(s, keep);
    }
    return s;
}

mrg_status mrg_tracer_get_cam_transform(const mrg_tracer* t, uint32_t cam_surface_id, float out[9])
{
    TR_LOCK(t);
    if(!out) return err("null output");
    float fnp[4];
    return camera_of(t, cam_surface_id, out, fnp);
}

mrg_status mrg_tracer_set_spectral_data(mrg_tracer* t, uint32_t lut_res, const float* lut, uint32_t cie_count,
                                        const float* cie_xyz, const float cie_integrals[3],
                                        const float* illuminant_spd, float illuminant_norm,
                                        const float xyz_to_rgb[9])
{
    TR_LOCK(t);
    if(lut_res == 0) { t->spectral = Spectral{}; return MRG_OK; }
    if(!lut || !cie_xyz || !cie_integrals || !illuminant_spd || !xyz_to_rgb || cie_count == 0)
        return err("incomplete spectral data");
    Spectral S;
    S.lutRes = lut_res;
    S.cieCount = cie_count;
    S.lut.assign(lut, lut + 9ull * lut_res * lut_res * lut_res);
    S.cie.assign(cie_xyz, cie_xyz + 3ull * cie_count);
    S.spd.assign(illuminant_spd, illuminant_spd + cie_count);
    std::memcpy(S.integrals, cie_integrals, sizeof(S.integrals));
    S.norm = illuminant_norm;
    std::memcpy(S.xyzToRgb, xyz_to_rgb, sizeof(S.xyzToRgb));
    t->spectral = std::move(S);
    return MRG_OK;
}

// ---- renderers ----
mrg_status mrg_tracer_create_renderer(mrg_tracer* t, const char* type_name, uint32_t* renderer_id)
{
    TR_LOCK(t);
    if(!renderer_id) return err("null output id");
    const int ty = find_type(MRG_KIND_RENDERER, type_name);
    if(ty < 0) return err(std::string("Unable to find generator for ") + (type_name ? type_name : "(null)"));
    Renderer r;
    r.type = ty;
    r.alive = true;
    mrg_guide_defaults(&r.guide);
    if(types(MRG_KIND_RENDERER)[ty].code == kRendGuided)
    {
        // GuidedPTRDetail::Options defaults (GuidedPTRendererShaders.h:79-133)
        r.rrStart = 2;
        r.maxDepth = 20;
    }
    *renderer_id = (uint32_t)t->renderers.size();
    t->renderers.push_back(r);
    return MRG_OK;
}

mrg_status mrg_tracer_destroy_renderer(mrg_tracer* t, uint32_t renderer_id)
{
    TR_LOCK(t);
    if(renderer_id >= t->renderers.size() || !t->renderers[renderer_id].alive)
        return err("unknown renderer " + std::to_string(renderer_id));
    if(t->rendering && t->renderer == renderer_id) t->stop();
    t->renderers[renderer_id].alive = false;
    return MRG_OK;
}

mrg_status mrg_tracer_push_renderer_attribute(mrg_tracer* t, uint32_t renderer_id, uint32_t attribute_index,
                                              const void* data, size_t bytes)
{ TR_LOCK(t); return push_renderer(t, renderer_id, attribute_index, data, bytes); }

mrg_status mrg_tracer_start_render(mrg_tracer* t, uint32_t renderer_id, uint32_t cam_surface_id, uint32_t width,
                                   uint32_t height, const uint32_t region_min[2], const uint32_t region_max[2],
                                   mrg_tracer_render_info* out)
{
    TR_LOCK(t);
    mrg_status s = start_render(t, renderer_id, cam_surface_id, width, height, region_min, region_max, out);
    if(s != MRG_OK)
    {
        const std::string keep = mrg_last_error();
        t->stop();
        mrg::set_error(s, keep);
    }
    return s;
}

mrg_status mrg_tracer_set_camera_transform(mrg_tracer* t, uint32_t renderer_id, const float cam[9])
{
    TR_LOCK(t);
    if(!cam) return err("null camera");
    if(!t->rendering || t->renderer != renderer_id)
        return err("renderer " + std::to_string(renderer_id) + " is not rendering");
    std::memcpy(t->P.camPos, cam, 12);
    std::memcpy(t->P.camGaze, cam + 3, 12);
    std::memcpy(t->P.camUp, cam + 6, 12);
    // a moved camera starts the accumulation again, and the guided renderer's
    // grid with it (a new camera resets the hash grid, GuidedPTRenderer.cu:988-1006)
    t->done = 0;
    if(types(MRG_KIND_RENDERER)[t->renderers[renderer_id].type].code == kRendGuided)
    {
        const mrg_status s = mrg_guide_clear(t->ctx);
        if(s != MRG_OK) return s;
    }
    return cuda_status(cudaMemset(t->dFilm, 0, sizeof(float) * 4 * (size_t)t->P.width * t->P.height), "film");
}

mrg_status mrg_tracer_do_render_work(mrg_tracer* t, mrg_tracer_render_output* out)
{ TR_LOCK(t); return render_work(t, out); }

mrg_status mrg_tracer_read_film(mrg_tracer* t, float* h_rgbw, size_t bytes)
{
    TR_LOCK(t);
    if(!t->rendering) return err("no render in progress");
    const size_t need = sizeof(float) * 4 * (size_t)t->P.width * t->P.height;
    if(!h_rgbw || bytes != need) return err("the film is " + std::to_string(need) + " bytes");
    return cuda_status(cudaMemcpy(h_rgbw, t->dFilm, need, cudaMemcpyDeviceToHost), "read film");
}

mrg_status mrg_tracer_stop_render(mrg_tracer* t)
{
    TR_LOCK(t);
    t->stop();
    return MRG_OK;
}

mrg_status mrg_tracer_clear_all(mrg_tracer* t)
{
    TR_LOCK(t);
    t->release_device();
    t->renderers.clear();
    t->spectral = Spectral{};
    t->reset_scene();
    return MRG_OK;
}

mrg_status mrg_tracer_flush(const mrg_tracer* t)
{
    TR_LOCK(t);
    if(!t->ctx) return MRG_OK;
    return cuda_status(cudaDeviceSynchronize(), "Flush");
}

mrg_status mrg_tracer_device_memory(const mrg_tracer* t, uint64_t* total, uint64_t* used)
{
    TR_LOCK(t);
    if(!total || !used) return err("null output");
    *total = *used = 0;
    if(!t->ctx) return MRG_OK;
    size_t fr = 0, tot = 0;
    mrg_status s = cuda_status(cudaMemGetInfo(&fr, &tot), "device memory");
    if(s != MRG_OK) return s;
    *total = tot;
    *used = tot - fr;
    return MRG_OK;
}

mrg_ctx* mrg_tracer_context(mrg_tracer* t)
{
    if(!t) return nullptr;
    std::lock_guard<std::mutex> lk(t->m);
    return t->ctx;
}

} // extern "C"
