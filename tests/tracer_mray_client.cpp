// tracer_mray_client.cpp -- MRay's own client side of TracerI run against
// TracerGB300 (mray_gb300/shim/TracerGB300.h): the tracer is made by the
// ConstructTracer entry point, scene data is built in MRay's TransientData
// (AllocateTransientData / Push / AccessAsString, as SceneLoaderMRay.cpp and
// MRay/TracerThread.cpp:195-230 build it) and every failure arrives as an
// MRayError.  Built with MRay's host-backend flags against the MRay tree; it
// exercises everything up to the surface commit, which needs the device and
// is expected to throw where there is none.  Prints one line per check and
// exits non-zero on the first failure.
#define MRAY_GB300_TRACER_ENTRYPOINTS
#include "TracerGB300.h"

#include <cstdio>
#include <string>

namespace {

int failures = 0;

void check(bool ok, const char* what)
{
    std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
    if(!ok) failures++;
}

template<class T>
TransientData make(std::initializer_list<T> v)
{
    TransientData d(std::in_place_type_t<T>{}, v.size());
    d.Push(Span<const T>(v.begin(), v.size()));
    return d;
}

TransientData make_string(std::string_view s)
{
    TransientData d = AllocateTransientData(MRayDataTypeRT(MRayDataEnum::MR_STRING), s.size());
    d.ReserveAll();
    Span<char> out = d.AccessAsString();
    std::copy(s.cbegin(), s.cend(), out.begin());
    return d;
}

template<class F>
std::string throws(F&& f)
{
    try { f(); }
    catch(const MRayError& e) { return std::string(e.GetError()); }
    return std::string();
}

} // namespace

int main()
{
    TracerParameters tp;
    tp.seed = 42;
    TracerI* tr = ConstructTracer(tp);

    // type lists and attribute information in MRay's types
    const auto mats = tr->MaterialGroups();
    check(mats.size() == 4 && mats[0] == "(Mt)Lambert" && mats[3] == "(Mt)Unreal", "MaterialGroups");
    check(tr->Renderers().size() == 3 && tr->Renderers()[0] == "(R)PathTracerRGB" &&
          tr->Renderers()[2] == "(R)GuidedPathTracerSpectral", "Renderers");
    const auto lam = tr->AttributeInfoMat("(Mt)Lambert");
    check(lam.size() == 2 && lam[0].name == "albedo" &&
          lam[0].isTexturable == AttributeTexturable::MR_TEXTURE_OR_CONSTANT &&
          lam[0].dataType.Name() == MRayDataEnum::MR_VECTOR_3 && lam[0].isColor == AttributeIsColor::IS_COLOR &&
          lam[1].isOptional == AttributeOptionality::MR_OPTIONAL, "AttributeInfoMat(Lambert)");
    const auto tri = tr->AttributeInfoPrim("(P)Triangle");
    check(tri.size() == 4 && tri[3].logic.e == PrimitiveAttributeLogic::INDEX &&
          tri[1].dataType.Name() == MRayDataEnum::MR_QUATERNION, "AttributeInfoPrim(Triangle)");

    // primitives: a floor quad and a light quad
    const PrimGroupId pg = tr->CreatePrimitiveGroup("(P)Triangle");
    const PrimBatchIdList batches = tr->ReservePrimitiveBatches(pg, { PrimCount{ 2, 4 }, PrimCount{ 2, 4 } });
    check(static_cast<CommonId>(batches[1]) == ((1u << 28) | 1u), "PrimBatchId layout");
    std::string e = throws([&] { tr->PushPrimAttribute(pg, batches[0], 0, make<Vector3>({ Vector3(0, 0, 0) })); });
    check(e.find("not committed") != std::string::npos, "push before commit throws MRayError");
    tr->CommitPrimReservations(pg);
    check(tr->IsPrimCommitted(pg), "IsPrimCommitted");
    for(int q = 0; q < 2; q++)
    {
        const Float y = q ? Float(1) : Float(0);
        tr->PushPrimAttribute(pg, batches[q], 0, make<Vector3>({ Vector3(0, y, 0), Vector3(1, y, 0),
                                                                  Vector3(1, y, 1), Vector3(0, y, 1) }));
        tr->PushPrimAttribute(pg, batches[q], 2, make<Vector2>({ Vector2(0, 0), Vector2(1, 0),
                                                                  Vector2(1, 1), Vector2(0, 1) }));
        tr->PushPrimAttribute(pg, batches[q], 3, make<Vector3ui>({ Vector3ui(0, 1, 2), Vector3ui(0, 2, 3) }));
    }
    e = throws([&] { tr->PushPrimAttribute(pg, batches[0], 3, make<Vector3ui>({ Vector3ui(0, 1, 2) })); });
    check(e.find("wants 24 bytes") != std::string::npos, "wrong attribute size throws");

    // a Lambert material, a transform, a primitive-backed light, a camera
    const MatGroupId mg = tr->CreateMaterialGroup("(Mt)Lambert");
    const MaterialIdList m = tr->ReserveMaterials(mg, { AttributeCountList{} });
    tr->CommitMatReservations(mg);
    const auto mid = static_cast<CommonId>(m[0]);
    tr->PushMatAttribute(mg, CommonIdRange(mid, mid), 0, make<Vector3>({ Vector3(0.5, 0.4, 0.3) }),
                         std::vector<Optional<TextureId>>{ std::nullopt });
    const TransGroupId tg = tr->CreateTransformGroup("(T)Single");
    const TransformIdList tids = tr->ReserveTransformations(tg, { AttributeCountList{} });
    tr->CommitTransReservations(tg);
    const auto tid = static_cast<CommonId>(tids[0]);
    tr->PushTransAttribute(tg, CommonIdRange(tid, tid), 0, make<Matrix4x4>({ Matrix4x4::Identity() }));
    const LightGroupId lg = tr->CreateLightGroup("(L)Prim(P)Triangle", pg);
    const LightIdList lights = tr->ReserveLights(lg, { AttributeCountList{} }, { batches[1] });
    tr->CommitLightReservations(lg);
    const auto lid = static_cast<CommonId>(lights[0]);
    tr->PushLightAttribute(lg, CommonIdRange(lid, lid), 0, make<Vector3>({ Vector3(10, 10, 10) }),
                           std::vector<Optional<TextureId>>{ std::nullopt });
    tr->PushLightAttribute(lg, CommonIdRange(lid, lid), 1, make<bool>({ false }));
    const CameraGroupId cg = tr->CreateCameraGroup("(C)Pinhole");
    const CameraIdList cams = tr->ReserveCameras(cg, { AttributeCountList{} });
    tr->CommitCamReservations(cg);
    const auto cid = static_cast<CommonId>(cams[0]);
    tr->PushCamAttribute(cg, CommonIdRange(cid, cid), 0, make<Vector4>({ Vector4(0.8, 0.8, 0.01, 100) }));
    tr->PushCamAttribute(cg, CommonIdRange(cid, cid), 1, make<Vector3>({ Vector3(0.5, 0.5, 0.5) }));
    tr->PushCamAttribute(cg, CommonIdRange(cid, cid), 2, make<Vector3>({ Vector3(0.5, 0.5, -1) }));
    tr->PushCamAttribute(cg, CommonIdRange(cid, cid), 3, make<Vector3>({ Vector3(0, 1, 0) }));

    // surfaces
    SurfaceParams sp;
    sp.primBatches.push_back(batches[0]);
    sp.materials.push_back(m[0]);
    sp.transformId = tids[0];
    sp.alphaMaps.push_back(std::nullopt);
    sp.cullFaceFlags.push_back(true);
    const SurfaceId sid = tr->CreateSurface(sp);
    check(static_cast<CommonId>(sid) == 0, "CreateSurface");
    tr->CreateLightSurface(LightSurfaceParams{ lights[0], TracerConstants::IdentityTransformId, {} });
    tr->SetBoundarySurface(TracerConstants::NullLightId, TracerConstants::IdentityTransformId);
    const CamSurfaceId cs = tr->CreateCameraSurface(CameraSurfaceParams{ cams[0], TracerConstants::IdentityTransformId, {} });
    const CameraTransform ct = tr->GetCamTransform(cs);
    check(ct.position[2] == Float(-1) && ct.gazePoint[0] == Float(0.5) && ct.up[1] == Float(1), "GetCamTransform");

    // renderer options as MRay's tracer thread pushes them
    const RendererId rid = tr->CreateRenderer("(R)PathTracerRGB");
    tr->PushRendererAttribute(rid, 0, make<uint32_t>({ 16u }));
    tr->PushRendererAttribute(rid, 2, make_string("Throughput"));
    tr->PushRendererAttribute(rid, 3, make_string("WithNEEAndMIS"));
    tr->PushRendererAttribute(rid, 4, make<Vector2ui>({ Vector2ui(3, 8) }));
    tr->PushRendererAttribute(rid, 5, make_string("Uniform"));
    e = throws([&] { tr->PushRendererAttribute(rid, 3, make_string("NEE")); });
    check(e.find("unknown sampleMode") != std::string::npos, "bad sampleMode throws");
    const auto rinfo = tr->AttributeInfo(rid);
    check(rinfo.size() == 6 && rinfo[1].isOptional == AttributeOptionality::MR_OPTIONAL, "AttributeInfo(RendererId)");
    // the guided renderer's options in MRay's types (GuidedPTRenderer.cu:1273-1292)
    const RendererId gid = tr->CreateRenderer("(R)GuidedPathTracerSpectral");
    const auto ginfo = tr->AttributeInfo(gid);
    check(ginfo.size() == 12 && ginfo[4].name == "cacheConeAperture" &&
          ginfo[4].dataType.Name() == MRayDataEnum::MR_FLOAT && ginfo[5].dataType.Name() == MRayDataEnum::MR_VECTOR_2UI &&
          ginfo[10].isOptional == AttributeOptionality::MR_OPTIONAL, "AttributeInfo(guided renderer)");
    tr->PushRendererAttribute(gid, 4, make<Float>({ Float(0.8) }));
    tr->PushRendererAttribute(gid, 10, make<Float>({ Float(0.5) }));
    tr->PushRendererAttribute(gid, 11, make_string("Render"));
    e = throws([&] { tr->PushRendererAttribute(gid, 11, make_string("MCTarget")); });
    check(e.find("only Render") != std::string::npos, "guided displayMode throws");

    // the commit needs a device
    e = throws([&] { tr->CommitSurfaces(); });
    std::printf("commit: %s\n", e.empty() ? "ok" : "error");
    tr->ClearAll();
    check(static_cast<CommonId>(tr->CreatePrimitiveGroup("(P)Triangle")) == 1, "ClearAll resets the groups");
    DestroyTracer(tr);
    std::printf("%d failures\n", failures);
    return failures ? 1 : 0;
}
