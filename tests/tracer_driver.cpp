// tracer_driver.cpp -- a C++ client of include/mray_gb300_tracer.h in the
// role MRay's scene loader plays against TracerI (the MockTracer pattern of
// Source/Tests/SceneLoaderMRay/T_SceneLoaderMRay.cpp, here against the real
// tracer): it reads a scene dump, pushes it through the tracer calls in
// TracerI order (groups, reservations, commits, attribute pushes, surfaces,
// commit), renders with (R)PathTracerRGB and writes the film.
//
// Scene dump (little-endian 32-bit words):
//   n_surfaces, then per surface:
//     kind (0 material surface, 1 light surface), material (MRG_MAT_*), cull,
//     nv, nt, pos[3 nv] f32, idx[3 nt] u32, m34[12] f32, albedo or radiance[3] f32,
//     roughness, metallic, specular, iorFront, iorBack (f32)
//   camera: pos[3] gaze[3] up[3] fov[2] near far (f32)
//   render: width height totalSpp burst sampleMode rrStart maxDepth (u32), seed (u64)
// Usage: tracer_driver scene.bin film.bin
#include "mray_gb300_tracer.h"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Surf
{
    uint32_t kind, material, cull, nv, nt;
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    float m34[12], color[3], rough, metal, spec, iorF, iorB;
};

bool rd(FILE* f, void* p, size_t n) { return std::fread(p, 1, n, f) == n; }

int fail(const char* what)
{
    std::fprintf(stderr, "tracer_driver: %s: %s\n", what, mrg_last_error());
    return 1;
}

#define CHECK(call) do { if((call) != MRG_OK) return fail(#call); } while(0)

const char* mat_type(uint32_t m)
{
    switch(m)
    {
        case MRG_MAT_REFLECT: return "(Mt)Reflect";
        case MRG_MAT_REFRACT: return "(Mt)Refract";
        case MRG_MAT_UNREAL: return "(Mt)Unreal";
        default: return "(Mt)Lambert";
    }
}

} // namespace

int main(int argc, char** argv)
{
    if(argc != 3) { std::fprintf(stderr, "usage: tracer_driver scene.bin film.bin\n"); return 2; }
    FILE* f = std::fopen(argv[1], "rb");
    if(!f) { std::perror(argv[1]); return 2; }
    uint32_t ns = 0;
    if(!rd(f, &ns, 4)) return 2;
    std::vector<Surf> S(ns);
    for(auto& s : S)
    {
        uint32_t h[5];
        if(!rd(f, h, sizeof(h))) return 2;
        s.kind = h[0]; s.material = h[1]; s.cull = h[2]; s.nv = h[3]; s.nt = h[4];
        s.pos.resize(3ull * s.nv);
        s.idx.resize(3ull * s.nt);
        float tail[8];
        if(!rd(f, s.pos.data(), 12ull * s.nv) || !rd(f, s.idx.data(), 12ull * s.nt) || !rd(f, s.m34, 48) ||
           !rd(f, tail, sizeof(tail)))
            return 2;
        std::memcpy(s.color, tail, 12);
        s.rough = tail[3]; s.metal = tail[4]; s.spec = tail[5]; s.iorF = tail[6]; s.iorB = tail[7];
    }
    float cam[13];
    uint32_t ren[7];
    uint64_t seed;
    if(!rd(f, cam, sizeof(cam)) || !rd(f, ren, sizeof(ren)) || !rd(f, &seed, 8)) return 2;
    std::fclose(f);

    mrg_tracer_params tp{};
    tp.seed = seed;
    mrg_tracer* t = nullptr;
    CHECK(mrg_tracer_create(&tp, &t));

    // primitives: one (P)Triangle group, a batch per surface
    uint32_t pg;
    CHECK(mrg_tracer_create_prim_group(t, "(P)Triangle", &pg));
    std::vector<uint32_t> counts, batch(ns);
    for(const auto& s : S) { counts.push_back(s.nt); counts.push_back(s.nv); }
    CHECK(mrg_tracer_reserve_prim_batches(t, pg, counts.data(), ns, batch.data()));
    CHECK(mrg_tracer_commit_prim_reservations(t, pg));
    for(uint32_t i = 0; i < ns; i++)
    {
        CHECK(mrg_tracer_push_prim_attribute(t, pg, batch[i], 0, 0, 0, S[i].pos.data(), S[i].pos.size() * 4));
        CHECK(mrg_tracer_push_prim_attribute(t, pg, batch[i], 3, 0, 0, S[i].idx.data(), S[i].idx.size() * 4));
    }

    // transforms: one (T)Single per surface (row-major 4x4)
    uint32_t tg;
    std::vector<uint32_t> trans(ns);
    CHECK(mrg_tracer_create_trans_group(t, "(T)Single", &tg));
    CHECK(mrg_tracer_reserve_transforms(t, tg, ns, trans.data()));
    CHECK(mrg_tracer_commit_trans_reservations(t, tg));
    for(uint32_t i = 0; i < ns; i++)
    {
        float m[16] = {};
        std::memcpy(m, S[i].m34, 48);
        m[15] = 1.0f;
        CHECK(mrg_tracer_push_trans_attribute(t, tg, trans[i], trans[i], 0, m, sizeof(m)));
    }

    // materials: a group per type; lights: one primitive-backed group
    std::vector<uint32_t> matId(ns, 0), lightId(ns, 0);
    for(uint32_t type = 0; type < 4; type++)
    {
        std::vector<uint32_t> members;
        for(uint32_t i = 0; i < ns; i++)
            if(S[i].kind == 0 && S[i].material == type) members.push_back(i);
        if(members.empty()) continue;
        uint32_t mg;
        std::vector<uint32_t> ids(members.size());
        CHECK(mrg_tracer_create_mat_group(t, mat_type(type), &mg));
        CHECK(mrg_tracer_reserve_materials(t, mg, (uint32_t)members.size(), ids.data()));
        CHECK(mrg_tracer_commit_mat_reservations(t, mg));
        for(size_t k = 0; k < members.size(); k++)
        {
            const Surf& s = S[members[k]];
            const uint32_t id = ids[k], none = 0;
            matId[members[k]] = id;
            if(type == MRG_MAT_LAMBERT || type == MRG_MAT_UNREAL)
                CHECK(mrg_tracer_push_mat_attribute(t, mg, id, id, 0, s.color, 12, &none));
            if(type == MRG_MAT_UNREAL)
            {
                CHECK(mrg_tracer_push_mat_attribute(t, mg, id, id, 2, &s.rough, 4, &none));
                CHECK(mrg_tracer_push_mat_attribute(t, mg, id, id, 3, &s.spec, 4, &none));
                CHECK(mrg_tracer_push_mat_attribute(t, mg, id, id, 4, &s.metal, 4, &none));
            }
            if(type == MRG_MAT_REFRACT)
            {
                const float back[3] = { s.iorB, 0, 0 }, front[3] = { s.iorF, 0, 0 };
                CHECK(mrg_tracer_push_mat_attribute(t, mg, id, id, 0, back, 12, nullptr));
                CHECK(mrg_tracer_push_mat_attribute(t, mg, id, id, 1, front, 12, nullptr));
            }
        }
    }
    std::vector<uint32_t> lights, lightBatches;
    for(uint32_t i = 0; i < ns; i++)
        if(S[i].kind == 1) { lights.push_back(i); lightBatches.push_back(batch[i]); }
    if(!lights.empty())
    {
        uint32_t lg;
        std::vector<uint32_t> ids(lights.size());
        CHECK(mrg_tracer_create_light_group(t, "(L)Prim(P)Triangle", pg, &lg));
        CHECK(mrg_tracer_reserve_lights(t, lg, (uint32_t)lights.size(), lightBatches.data(), ids.data()));
        CHECK(mrg_tracer_commit_light_reservations(t, lg));
        for(size_t k = 0; k < lights.size(); k++)
        {
            const uint32_t id = ids[k], none = 0;
            const uint8_t twoSided = 0;
            lightId[lights[k]] = id;
            CHECK(mrg_tracer_push_light_attribute(t, lg, id, id, 0, S[lights[k]].color, 12, &none));
            CHECK(mrg_tracer_push_light_attribute(t, lg, id, id, 1, &twoSided, 1, nullptr));
        }
    }

    // camera
    uint32_t cg, camId;
    CHECK(mrg_tracer_create_camera_group(t, "(C)Pinhole", &cg));
    CHECK(mrg_tracer_reserve_cameras(t, cg, 1, &camId));
    CHECK(mrg_tracer_commit_cam_reservations(t, cg));
    const float fnp[4] = { cam[9], cam[10], cam[11], cam[12] };
    CHECK(mrg_tracer_push_cam_attribute(t, cg, camId, camId, 0, fnp, 16));
    CHECK(mrg_tracer_push_cam_attribute(t, cg, camId, camId, 1, cam + 3, 12));
    CHECK(mrg_tracer_push_cam_attribute(t, cg, camId, camId, 2, cam, 12));
    CHECK(mrg_tracer_push_cam_attribute(t, cg, camId, camId, 3, cam + 6, 12));

    // surfaces, light surfaces, boundary, camera surface, commit
    for(uint32_t i = 0; i < ns; i++)
    {
        if(S[i].kind != 0) continue;
        mrg_tracer_surface sf{};
        sf.count = 1;
        sf.primBatches[0] = batch[i];
        sf.materials[0] = matId[i];
        sf.cullFace[0] = S[i].cull;
        sf.transformId = trans[i];
        uint32_t sid;
        CHECK(mrg_tracer_create_surface(t, &sf, &sid));
    }
    for(uint32_t i : lights)
    {
        uint32_t lsid;
        CHECK(mrg_tracer_create_light_surface(t, lightId[i], trans[i], &lsid));
    }
    uint32_t bsid, csid;
    CHECK(mrg_tracer_set_boundary_surface(t, 0, 0, &bsid));
    CHECK(mrg_tracer_create_camera_surface(t, camId, 0, &csid));
    mrg_tracer_commit_result cr;
    CHECK(mrg_tracer_commit_surfaces(t, &cr));

    // render
    uint32_t rid;
    CHECK(mrg_tracer_create_renderer(t, "(R)PathTracerRGB", &rid));
    static const char* modes[3] = { "Pure", "WithNextEventEstimation", "WithNEEAndMIS" };
    const uint32_t rr[2] = { ren[5], ren[6] };
    CHECK(mrg_tracer_push_renderer_attribute(t, rid, 0, &ren[2], 4));
    CHECK(mrg_tracer_push_renderer_attribute(t, rid, 1, &ren[3], 4));
    CHECK(mrg_tracer_push_renderer_attribute(t, rid, 2, "Throughput", 10));
    CHECK(mrg_tracer_push_renderer_attribute(t, rid, 3, modes[ren[4] % 3], std::strlen(modes[ren[4] % 3])));
    CHECK(mrg_tracer_push_renderer_attribute(t, rid, 4, rr, 8));
    CHECK(mrg_tracer_push_renderer_attribute(t, rid, 5, "Uniform", 7));
    const uint32_t rmin[2] = { 0, 0 }, rmax[2] = { ren[0], ren[1] };
    mrg_tracer_render_info info;
    CHECK(mrg_tracer_start_render(t, rid, csid, ren[0], ren[1], rmin, rmax, &info));
    mrg_tracer_render_output out{};
    int works = 0;
    do { CHECK(mrg_tracer_do_render_work(t, &out)); works++; } while(!out.finished && works < 100000);
    std::vector<float> film(4ull * ren[0] * ren[1]);
    CHECK(mrg_tracer_read_film(t, film.data(), film.size() * 4));
    CHECK(mrg_tracer_stop_render(t));
    CHECK(mrg_tracer_destroy(t));
    FILE* o = std::fopen(argv[2], "wb");
    if(!o || std::fwrite(film.data(), 4, film.size(), o) != film.size()) return 2;
    std::fclose(o);
    std::printf("instances %llu works %d samples %u\n", (unsigned long long)cr.instanceCount, works, out.samplesDone);
    return 0;
}
