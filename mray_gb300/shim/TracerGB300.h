// TracerGB300.h -- MRay-side tracer: a TracerI (Source/Core/TracerI.h:150-376)
// that forwards every call to the TracerI C ABI of libmray_gb300.so
// (include/mray_gb300_tracer.h), and the ConstructTracer / DestroyTracer
// entry points a TracerDLL exports (Source/TracerDLL/EntryPoint.h:12-18).
//
// This header is compiled inside an MRay build (it includes MRay's own
// headers); define MRAY_GB300_TRACER_ENTRYPOINTS in exactly one translation
// unit to emit the two entry points.  Ids pass through unchanged: the library
// returns MRay's key layouts (TracerTypes.h:168-174).  Scene data moves from
// MRay's TransientData to the C ABI as bytes.  The render buffer follows MRay's
// RenderImage protocol (Tracer/RenderImage.cpp:150-290): planar R, G, B and
// weight floats in a host staging buffer aligned to importAlignment, the
// visor's TimelineSemaphore acquired before each copy and released after it,
// the wait counter advanced by two per image.
#pragma once

#include "Core/TracerI.h"
#include "Core/TimelineSemaphore.h"
#include "Core/Error.h"
#include "Common/RenderImageStructs.h"

#include "mray_gb300_tracer.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

class TracerGB300 final : public TracerI
{
    mrg_tracer*         t = nullptr;
    TracerParameters    params;
    // storage behind the string_views of the type lists
    std::vector<std::string>    typeNameStore[7];
    // render buffer
    TimelineSemaphore*  sem = nullptr;
    uint32_t            importAlignment = 16;
    uint64_t            acquireValue = 0;
    Byte*               staging = nullptr;
    size_t              stagingBytes = 0;
    std::vector<float>  filmRGBW;
    Vector2ui           resolution = Vector2ui::Zero();
    uint32_t            volumeCounter = 0;

    static void Check(mrg_status s)
    {
        if(s != MRG_OK) throw MRayError("mray_gb300: {}", mrg_last_error());
    }
    template<class Id> static uint32_t Raw(Id id) { return static_cast<uint32_t>(static_cast<CommonId>(id)); }
    template<class Id> static Id       Make(uint32_t v) { return static_cast<Id>(CommonId(v)); }

    static MRayDataTypeRT DataType(uint32_t dt)
    {
        using enum MRayDataEnum;
        switch(dt)
        {
            case MRG_DT_FLOAT:      return MRayDataTypeRT(MR_FLOAT);
            case MRG_DT_VECTOR_2:   return MRayDataTypeRT(MR_VECTOR_2);
            case MRG_DT_VECTOR_3:   return MRayDataTypeRT(MR_VECTOR_3);
            case MRG_DT_VECTOR_4:   return MRayDataTypeRT(MR_VECTOR_4);
            case MRG_DT_QUATERNION: return MRayDataTypeRT(MR_QUATERNION);
            case MRG_DT_MATRIX_4x4: return MRayDataTypeRT(MR_MATRIX_4x4);
            case MRG_DT_UINT32:     return MRayDataTypeRT(MR_UINT32);
            case MRG_DT_VECTOR_2UI: return MRayDataTypeRT(MR_VECTOR_2UI);
            case MRG_DT_VECTOR_3UI: return MRayDataTypeRT(MR_VECTOR_3UI);
            case MRG_DT_BOOL:       return MRayDataTypeRT(MR_BOOL);
            default:                return MRayDataTypeRT(MR_STRING);
        }
    }

    std::vector<mrg_tracer_attrib_info> Infos(uint32_t kind, std::string_view type) const
    {
        const std::string name(type);
        uint32_t n = 0;
        Check(mrg_tracer_attribute_info(t, kind, name.c_str(), 0, nullptr, &n));
        std::vector<mrg_tracer_attrib_info> out(n);
        for(uint32_t i = 0; i < n; i++) Check(mrg_tracer_attribute_info(t, kind, name.c_str(), i, &out[i], nullptr));
        return out;
    }

    template<class List>
    List Textured(uint32_t kind, std::string_view type) const
    {
        List l;
        for(const auto& a : Infos(kind, type))
            l.push_back(TexturedAttributeInfo{ a.name, DataType(a.dataType), AttributeIsArray::IS_SCALAR,
                                               a.optional ? AttributeOptionality::MR_OPTIONAL
                                                          : AttributeOptionality::MR_MANDATORY,
                                               AttributeTexturable(a.texturable),
                                               a.isColor ? AttributeIsColor::IS_COLOR : AttributeIsColor::IS_PURE_DATA });
        return l;
    }

    template<class List>
    List Generic(uint32_t kind, std::string_view type) const
    {
        List l;
        for(const auto& a : Infos(kind, type))
            l.push_back(GenericAttributeInfo{ a.name, DataType(a.dataType), AttributeIsArray::IS_SCALAR,
                                              a.optional ? AttributeOptionality::MR_OPTIONAL
                                                         : AttributeOptionality::MR_MANDATORY });
        return l;
    }

    std::string GroupName(uint32_t kind, uint32_t id) const
    {
        char buf[64];
        Check(mrg_tracer_group_type_name(t, kind, id, buf, sizeof(buf)));
        return buf;
    }

    TypeNameList Names(uint32_t kind) const
    {
        auto* self = const_cast<TracerGB300*>(this);
        size_t need = 0;
        Check(mrg_tracer_type_names(t, kind, nullptr, 0, &need));
        std::string buf(need, '\0');
        Check(mrg_tracer_type_names(t, kind, buf.data(), need, nullptr));
        auto& store = self->typeNameStore[kind];
        store.clear();
        size_t b = 0;
        for(size_t i = 0; i < buf.size(); i++)
            if(buf[i] == '\n' || buf[i] == '\0')
            {
                if(i > b) store.emplace_back(buf.substr(b, i - b));
                b = i + 1;
                if(buf[i] == '\0') break;
            }
        return TypeNameList(store.begin(), store.end());
    }

    static std::vector<uint32_t> Textures(const std::vector<Optional<TextureId>>& v)
    {
        std::vector<uint32_t> out(v.size(), 0u);
        for(size_t i = 0; i < v.size(); i++) out[i] = v[i].has_value() ? Raw(v[i].value()) : 0u;
        return out;
    }
    static std::vector<uint32_t> Textures(const std::vector<TextureId>& v)
    {
        std::vector<uint32_t> out(v.size());
        for(size_t i = 0; i < v.size(); i++) out[i] = Raw(v[i]);
        return out;
    }
    // The pushed bytes of any TransientData (the Byte access has no type check).
    static const void* Bytes(const TransientData& d) { return d.AccessAs<Byte>().data(); }

    void FreeStaging()
    {
        std::free(staging);
        staging = nullptr;
        stagingBytes = 0;
    }

    public:
    explicit TracerGB300(const TracerParameters& p) : params(p)
    {
        if(p.samplerType.e == SamplerType::E::SOBOL)
            throw MRayError("mray_gb300: the SOBOL sampler is not available (INDEPENDENT, Z_SOBOL)");
        if(p.filmFilter.type != FilterType::E::GAUSSIAN)
            throw MRayError("mray_gb300: only the Gaussian film filter is available");
        mrg_tracer_params tp{};
        tp.seed = p.seed;
        tp.device = 0;
        tp.samplerType = (p.samplerType.e == SamplerType::E::Z_SOBOL) ? MRG_TRACER_SAMPLER_ZSOBOL
                                                                     : MRG_TRACER_SAMPLER_INDEPENDENT;
        tp.filmFilterRadius = p.filmFilter.radius;
        if(p.genMips && p.mipGenFilter.type != FilterType::E::GAUSSIAN)
            throw MRayError("mray_gb300: only the Gaussian mip generation filter is available");
        tp.genMips = p.genMips ? 1u : 0u;
        tp.mipGenFilterRadius = p.mipGenFilter.radius;
        Check(mrg_tracer_create(&tp, &t));
    }
    ~TracerGB300() override
    {
        FreeStaging();
        mrg_tracer_destroy(t);
    }

    // ---- generic ----
    TypeNameList PrimitiveGroups() const override { return Names(MRG_KIND_PRIM); }
    TypeNameList MaterialGroups() const override { return Names(MRG_KIND_MATERIAL); }
    TypeNameList TransformGroups() const override { return Names(MRG_KIND_TRANSFORM); }
    TypeNameList CameraGroups() const override { return Names(MRG_KIND_CAMERA); }
    TypeNameList MediumGroups() const override { return Names(MRG_KIND_MEDIUM); }
    TypeNameList LightGroups() const override { return Names(MRG_KIND_LIGHT); }
    TypeNameList Renderers() const override { return Names(MRG_KIND_RENDERER); }

    PrimAttributeInfoList AttributeInfo(PrimGroupId id) const override { return AttributeInfoPrim(GroupName(MRG_KIND_PRIM, Raw(id))); }
    CamAttributeInfoList AttributeInfo(CameraGroupId id) const override { return AttributeInfoCam(GroupName(MRG_KIND_CAMERA, Raw(id))); }
    MediumAttributeInfoList AttributeInfo(MediumGroupId id) const override { return AttributeInfoMedium(GroupName(MRG_KIND_MEDIUM, Raw(id))); }
    MatAttributeInfoList AttributeInfo(MatGroupId id) const override { return AttributeInfoMat(GroupName(MRG_KIND_MATERIAL, Raw(id))); }
    TransAttributeInfoList AttributeInfo(TransGroupId id) const override { return AttributeInfoTrans(GroupName(MRG_KIND_TRANSFORM, Raw(id))); }
    LightAttributeInfoList AttributeInfo(LightGroupId id) const override { return AttributeInfoLight(GroupName(MRG_KIND_LIGHT, Raw(id))); }
    RendererAttributeInfoList AttributeInfo(RendererId id) const override { return AttributeInfoRenderer(GroupName(MRG_KIND_RENDERER, Raw(id))); }

    PrimAttributeInfoList AttributeInfoPrim(std::string_view type) const override
    {
        // (P)Triangle: POSITION, NORMAL, UV0, INDEX (PrimitiveDefaultTriangle.cu:169-184)
        static constexpr PrimitiveAttributeLogic::E logic[4] = {
            PrimitiveAttributeLogic::POSITION, PrimitiveAttributeLogic::NORMAL,
            PrimitiveAttributeLogic::UV0, PrimitiveAttributeLogic::INDEX };
        PrimAttributeInfoList l;
        const auto infos = Infos(MRG_KIND_PRIM, type);
        for(size_t i = 0; i < infos.size() && i < 4; i++)
            l.push_back(PrimAttributeInfo{ logic[i], DataType(infos[i].dataType), AttributeIsArray::IS_SCALAR,
                                           AttributeOptionality::MR_MANDATORY });
        return l;
    }
    CamAttributeInfoList AttributeInfoCam(std::string_view type) const override { return Generic<CamAttributeInfoList>(MRG_KIND_CAMERA, type); }
    MediumAttributeInfoList AttributeInfoMedium(std::string_view type) const override { return Textured<MediumAttributeInfoList>(MRG_KIND_MEDIUM, type); }
    MatAttributeInfoList AttributeInfoMat(std::string_view type) const override { return Textured<MatAttributeInfoList>(MRG_KIND_MATERIAL, type); }
    TransAttributeInfoList AttributeInfoTrans(std::string_view type) const override { return Generic<TransAttributeInfoList>(MRG_KIND_TRANSFORM, type); }
    LightAttributeInfoList AttributeInfoLight(std::string_view type) const override { return Textured<LightAttributeInfoList>(MRG_KIND_LIGHT, type); }
    RendererAttributeInfoList AttributeInfoRenderer(std::string_view type) const override { return Generic<RendererAttributeInfoList>(MRG_KIND_RENDERER, type); }

    std::string TypeName(PrimGroupId id) const override { return GroupName(MRG_KIND_PRIM, Raw(id)); }
    std::string TypeName(CameraGroupId id) const override { return GroupName(MRG_KIND_CAMERA, Raw(id)); }
    std::string TypeName(MediumGroupId id) const override { return GroupName(MRG_KIND_MEDIUM, Raw(id)); }
    std::string TypeName(MatGroupId id) const override { return GroupName(MRG_KIND_MATERIAL, Raw(id)); }
    std::string TypeName(TransGroupId id) const override { return GroupName(MRG_KIND_TRANSFORM, Raw(id)); }
    std::string TypeName(LightGroupId id) const override { return GroupName(MRG_KIND_LIGHT, Raw(id)); }
    std::string TypeName(RendererId id) const override { return GroupName(MRG_KIND_RENDERER, Raw(id)); }

    // ---- primitives ----
    PrimGroupId CreatePrimitiveGroup(std::string type) override
    {
        uint32_t id;
        Check(mrg_tracer_create_prim_group(t, type.c_str(), &id));
        return Make<PrimGroupId>(id);
    }
    PrimBatchId ReservePrimitiveBatch(PrimGroupId g, PrimCount c) override
    {
        return ReservePrimitiveBatches(g, std::vector<PrimCount>{ c }).front();
    }
    PrimBatchIdList ReservePrimitiveBatches(PrimGroupId g, std::vector<PrimCount> counts) override
    {
        std::vector<uint32_t> c, ids(counts.size());
        for(const auto& x : counts) { c.push_back(x.primCount); c.push_back(x.attributeCount); }
        Check(mrg_tracer_reserve_prim_batches(t, Raw(g), c.data(), uint32_t(counts.size()), ids.data()));
        PrimBatchIdList out;
        for(uint32_t v : ids) out.push_back(Make<PrimBatchId>(v));
        return out;
    }
    void CommitPrimReservations(PrimGroupId g) override { Check(mrg_tracer_commit_prim_reservations(t, Raw(g))); }
    bool IsPrimCommitted(PrimGroupId g) const override
    {
        uint32_t c;
        Check(mrg_tracer_is_prim_committed(t, Raw(g), &c));
        return c != 0;
    }
    void PushPrimAttribute(PrimGroupId g, PrimBatchId b, uint32_t attrib, TransientData d) override
    {
        Check(mrg_tracer_push_prim_attribute(t, Raw(g), Raw(b), attrib, 0, 0, Bytes(d), d.ByteSize()));
    }
    void PushPrimAttribute(PrimGroupId g, PrimBatchId b, uint32_t attrib, Vector2ui range, TransientData d) override
    {
        if(range[0] == range[1]) return;
        Check(mrg_tracer_push_prim_attribute(t, Raw(g), Raw(b), attrib, range[0], range[1], Bytes(d), d.ByteSize()));
    }
    void TransformPrimitives(PrimGroupId g, std::vector<PrimBatchId> batches, std::vector<Matrix3x4> ms) override
    {
        if(batches.size() != ms.size()) throw MRayError("mray_gb300: TransformPrimitives: size mismatch");
        std::vector<uint32_t> ids;
        std::vector<float> m;
        for(size_t i = 0; i < batches.size(); i++)
        {
            ids.push_back(Raw(batches[i]));
            for(uint32_t r = 0; r < 3; r++)
                for(uint32_t c = 0; c < 4; c++) m.push_back(float(ms[i][r * 4 + c]));
        }
        Check(mrg_tracer_transform_primitives(t, Raw(g), ids.data(), m.data(), uint32_t(ids.size())));
    }

    // ---- materials ----
    MatGroupId CreateMaterialGroup(std::string type) override
    {
        uint32_t id;
        Check(mrg_tracer_create_mat_group(t, type.c_str(), &id));
        return Make<MatGroupId>(id);
    }
    MaterialId ReserveMaterial(MatGroupId g, AttributeCountList) override
    {
        uint32_t id;
        Check(mrg_tracer_reserve_materials(t, Raw(g), 1, &id));
        return Make<MaterialId>(id);
    }
    MaterialIdList ReserveMaterials(MatGroupId g, std::vector<AttributeCountList> l) override
    {
        std::vector<uint32_t> ids(l.size());
        Check(mrg_tracer_reserve_materials(t, Raw(g), uint32_t(l.size()), ids.data()));
        MaterialIdList out;
        for(uint32_t v : ids) out.push_back(Make<MaterialId>(v));
        return out;
    }
    void CommitMatReservations(MatGroupId g) override { Check(mrg_tracer_commit_mat_reservations(t, Raw(g))); }
    bool IsMatCommitted(MatGroupId g) const override
    {
        uint32_t c;
        Check(mrg_tracer_is_mat_committed(t, Raw(g), &c));
        return c != 0;
    }
    void PushMatAttribute(MatGroupId g, CommonIdRange r, uint32_t a, TransientData d) override
    {
        Check(mrg_tracer_push_mat_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, Bytes(d), d.ByteSize(), nullptr));
    }
    void PushMatAttribute(MatGroupId g, CommonIdRange r, uint32_t a, TransientData d,
                          std::vector<Optional<TextureId>> tex) override
    {
        const auto ids = Textures(tex);
        Check(mrg_tracer_push_mat_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, Bytes(d), d.ByteSize(), ids.data()));
    }
    void PushMatAttribute(MatGroupId g, CommonIdRange r, uint32_t a, std::vector<TextureId> tex) override
    {
        const auto ids = Textures(tex);
        Check(mrg_tracer_push_mat_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, nullptr, 0, ids.data()));
    }

    // ---- textures ----
    TextureId CreateTexture2D(Vector2ui size, uint32_t mips, MRayTextureParameters p) override
    {
        uint32_t pix;
        switch(p.pixelType.Name())
        {
            case MRayPixelEnum::MR_RGBA8_UNORM: pix = MRG_PIX_RGBA8_UNORM; break;
            case MRayPixelEnum::MR_RGB_FLOAT:   pix = MRG_PIX_RGB_FLOAT; break;
            case MRayPixelEnum::MR_RGBA_FLOAT:  pix = MRG_PIX_RGBA_FLOAT; break;
            case MRayPixelEnum::MR_R8_UNORM:    pix = MRG_PIX_R8_UNORM; break;
            case MRayPixelEnum::MR_R_FLOAT:     pix = MRG_PIX_R_FLOAT; break;
            default: throw MRayError("mray_gb300: texture pixel type is not supported "
                                     "(RGBA8 / R8 UNORM, R / RGB / RGBA float)");
        }
        uint32_t id;
        Check(mrg_tracer_create_texture2d(t, size[0], size[1], mips, pix, &id));
        return Make<TextureId>(id);
    }
    TextureId CreateTexture3D(Vector3ui, uint32_t, MRayTextureParameters) override
    {
        throw MRayError("mray_gb300: 3D textures are not supported");
    }
    void CommitTextures() override { Check(mrg_tracer_commit_textures(t)); }
    void PushTextureData(TextureId id, uint32_t mip, TransientData d) override
    {
        Check(mrg_tracer_push_texture_data(t, Raw(id), mip, Bytes(d), d.ByteSize()));
    }

    // ---- transforms ----
    TransGroupId CreateTransformGroup(std::string type) override
    {
        uint32_t id;
        Check(mrg_tracer_create_trans_group(t, type.c_str(), &id));
        return Make<TransGroupId>(id);
    }
    TransformId ReserveTransformation(TransGroupId g, AttributeCountList) override
    {
        uint32_t id;
        Check(mrg_tracer_reserve_transforms(t, Raw(g), 1, &id));
        return Make<TransformId>(id);
    }
    TransformIdList ReserveTransformations(TransGroupId g, std::vector<AttributeCountList> l) override
    {
        std::vector<uint32_t> ids(l.size());
        Check(mrg_tracer_reserve_transforms(t, Raw(g), uint32_t(l.size()), ids.data()));
        TransformIdList out;
        for(uint32_t v : ids) out.push_back(Make<TransformId>(v));
        return out;
    }
    void CommitTransReservations(TransGroupId g) override { Check(mrg_tracer_commit_trans_reservations(t, Raw(g))); }
    bool IsTransCommitted(TransGroupId g) const override
    {
        uint32_t c;
        Check(mrg_tracer_is_trans_committed(t, Raw(g), &c));
        return c != 0;
    }
    void PushTransAttribute(TransGroupId g, CommonIdRange r, uint32_t a, TransientData d) override
    {
        Check(mrg_tracer_push_trans_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, Bytes(d), d.ByteSize()));
    }

    // ---- lights ----
    LightGroupId CreateLightGroup(std::string type, PrimGroupId pg) override
    {
        uint32_t id;
        Check(mrg_tracer_create_light_group(t, type.c_str(), Raw(pg), &id));
        return Make<LightGroupId>(id);
    }
    LightId ReserveLight(LightGroupId g, AttributeCountList c, PrimBatchId b) override
    {
        return ReserveLights(g, { c }, { b }).front();
    }
    LightIdList ReserveLights(LightGroupId g, std::vector<AttributeCountList> l, std::vector<PrimBatchId> b) override
    {
        std::vector<uint32_t> ids(l.size()), batches;
        for(const auto& x : b) batches.push_back(Raw(x));
        const bool primBacked = !batches.empty() && batches.front() != 0u;
        Check(mrg_tracer_reserve_lights(t, Raw(g), uint32_t(l.size()), primBacked ? batches.data() : nullptr, ids.data()));
        LightIdList out;
        for(uint32_t v : ids) out.push_back(Make<LightId>(v));
        return out;
    }
    void CommitLightReservations(LightGroupId g) override { Check(mrg_tracer_commit_light_reservations(t, Raw(g))); }
    bool IsLightCommitted(LightGroupId g) const override
    {
        uint32_t c;
        Check(mrg_tracer_is_light_committed(t, Raw(g), &c));
        return c != 0;
    }
    void PushLightAttribute(LightGroupId g, CommonIdRange r, uint32_t a, TransientData d) override
    {
        Check(mrg_tracer_push_light_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, Bytes(d), d.ByteSize(), nullptr));
    }
    void PushLightAttribute(LightGroupId g, CommonIdRange r, uint32_t a, TransientData d,
                            std::vector<Optional<TextureId>> tex) override
    {
        const auto ids = Textures(tex);
        Check(mrg_tracer_push_light_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, Bytes(d), d.ByteSize(), ids.data()));
    }
    void PushLightAttribute(LightGroupId g, CommonIdRange r, uint32_t a, std::vector<TextureId> tex) override
    {
        const auto ids = Textures(tex);
        Check(mrg_tracer_push_light_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, nullptr, 0, ids.data()));
    }

    // ---- cameras ----
    CameraGroupId CreateCameraGroup(std::string type) override
    {
        uint32_t id;
        Check(mrg_tracer_create_camera_group(t, type.c_str(), &id));
        return Make<CameraGroupId>(id);
    }
    CameraId ReserveCamera(CameraGroupId g, AttributeCountList) override
    {
        uint32_t id;
        Check(mrg_tracer_reserve_cameras(t, Raw(g), 1, &id));
        return Make<CameraId>(id);
    }
    CameraIdList ReserveCameras(CameraGroupId g, std::vector<AttributeCountList> l) override
    {
        std::vector<uint32_t> ids(l.size());
        Check(mrg_tracer_reserve_cameras(t, Raw(g), uint32_t(l.size()), ids.data()));
        CameraIdList out;
        for(uint32_t v : ids) out.push_back(Make<CameraId>(v));
        return out;
    }
    void CommitCamReservations(CameraGroupId g) override { Check(mrg_tracer_commit_cam_reservations(t, Raw(g))); }
    bool IsCamCommitted(CameraGroupId g) const override
    {
        uint32_t c;
        Check(mrg_tracer_is_cam_committed(t, Raw(g), &c));
        return c != 0;
    }
    void PushCamAttribute(CameraGroupId g, CommonIdRange r, uint32_t a, TransientData d) override
    {
        Check(mrg_tracer_push_cam_attribute(t, Raw(g), uint32_t(r[0]), uint32_t(r[1]), a, Bytes(d), d.ByteSize()));
    }

    // ---- media: only the implicit vacuum ----
    MediumGroupId CreateMediumGroup(std::string type) override
    {
        if(type == TracerConstants::VacuumMediumName) return TracerConstants::VacuumMediumGroupId;
        throw MRayError("mray_gb300: participating media are not supported ({})", type);
    }
    MediumId ReserveMedium(MediumGroupId g, AttributeCountList) override
    {
        if(g != TracerConstants::VacuumMediumGroupId) throw MRayError("mray_gb300: unknown medium group");
        return TracerConstants::VacuumMediumId;
    }
    MediumIdList ReserveMediums(MediumGroupId g, std::vector<AttributeCountList> l) override
    {
        MediumIdList out;
        for(size_t i = 0; i < l.size(); i++) out.push_back(ReserveMedium(g, {}));
        return out;
    }
    void CommitMediumReservations(MediumGroupId) override {}
    bool IsMediumCommitted(MediumGroupId) const override { return true; }
    void PushMediumAttribute(MediumGroupId, CommonIdRange, uint32_t, TransientData) override
    {
        throw MRayError("mray_gb300: (Md)Vacuum takes no attributes");
    }
    void PushMediumAttribute(MediumGroupId, CommonIdRange, uint32_t, TransientData, std::vector<Optional<TextureId>>) override
    {
        throw MRayError("mray_gb300: (Md)Vacuum takes no attributes");
    }
    void PushMediumAttribute(MediumGroupId, CommonIdRange, uint32_t, std::vector<TextureId>) override
    {
        throw MRayError("mray_gb300: (Md)Vacuum takes no attributes");
    }

    // ---- surfaces ----
    SurfaceId CreateSurface(SurfaceParams p) override
    {
        mrg_tracer_surface s{};
        s.count = uint32_t(p.primBatches.size());
        if(s.count > MRG_TRACER_MAX_BATCHES_PER_SURFACE || p.materials.size() != p.primBatches.size())
            throw MRayError("mray_gb300: malformed surface");
        for(uint32_t i = 0; i < s.count; i++)
        {
            s.primBatches[i] = Raw(p.primBatches[i]);
            s.materials[i] = Raw(p.materials[i]);
            s.alphaMaps[i] = (i < p.alphaMaps.size() && p.alphaMaps[i].has_value()) ? Raw(p.alphaMaps[i].value()) : 0u;
            s.cullFace[i] = (i < p.cullFaceFlags.size()) ? uint32_t(p.cullFaceFlags[i]) : 1u;
        }
        s.transformId = Raw(p.transformId);
        uint32_t id;
        Check(mrg_tracer_create_surface(t, &s, &id));
        return Make<SurfaceId>(id);
    }
    LightSurfaceId SetBoundarySurface(LightId l, TransformId tr) override
    {
        uint32_t id;
        Check(mrg_tracer_set_boundary_surface(t, Raw(l), Raw(tr), &id));
        return Make<LightSurfaceId>(id);
    }
    LightSurfaceId CreateLightSurface(LightSurfaceParams p) override
    {
        uint32_t id;
        Check(mrg_tracer_create_light_surface(t, Raw(p.lightId), Raw(p.transformId), &id));
        return Make<LightSurfaceId>(id);
    }
    CamSurfaceId CreateCameraSurface(CameraSurfaceParams p) override
    {
        uint32_t id;
        Check(mrg_tracer_create_camera_surface(t, Raw(p.cameraId), Raw(p.transformId), &id));
        return Make<CamSurfaceId>(id);
    }
    SurfaceCommitResult CommitSurfaces() override
    {
        mrg_tracer_commit_result r;
        Check(mrg_tracer_commit_surfaces(t, &r));
        return SurfaceCommitResult{ AABB3(Vector3(r.aabb[0], r.aabb[1], r.aabb[2]), Vector3(r.aabb[3], r.aabb[4], r.aabb[5])),
                                    size_t(r.instanceCount), size_t(r.acceleratorCount) };
    }
    CameraTransform GetCamTransform(CamSurfaceId c) const override
    {
        float v[9];
        Check(mrg_tracer_get_cam_transform(t, Raw(c), v));
        return CameraTransform{ Vector3(v[0], v[1], v[2]), Vector3(v[3], v[4], v[5]), Vector3(v[6], v[7], v[8]) };
    }
    VolumeId RegisterVolume(VolumeParams) override { return Make<VolumeId>(volumeCounter++); }
    VolumeIdList RegisterVolumes(std::vector<VolumeParams> v) override
    {
        VolumeIdList out;
        for(const auto& x : v) out.push_back(RegisterVolume(x));
        return out;
    }
    void SetBoundaryVolume(VolumeId) override {}

    // ---- renderers ----
    RendererId CreateRenderer(std::string type) override
    {
        uint32_t id;
        Check(mrg_tracer_create_renderer(t, type.c_str(), &id));
        return Make<RendererId>(id);
    }
    void DestroyRenderer(RendererId r) override { Check(mrg_tracer_destroy_renderer(t, Raw(r))); }
    void PushRendererAttribute(RendererId r, uint32_t a, TransientData d) override
    {
        // renderMode, sampleMode and neeSamplerType are strings
        if(a == 2 || a == 3 || a == 5)
        {
            const std::string_view s = std::as_const(d).AccessAsString();
            Check(mrg_tracer_push_renderer_attribute(t, Raw(r), a, s.data(), s.size()));
        }
        else
            Check(mrg_tracer_push_renderer_attribute(t, Raw(r), a, Bytes(d), d.ByteSize()));
    }

    // ---- rendering ----
    void SetupRenderEnv(TimelineSemaphore* s, uint32_t alignment, uint64_t initialAcquire) override
    {
        sem = s;
        importAlignment = std::max<uint32_t>(alignment, 16u);
        acquireValue = initialAcquire;
    }
    RenderBufferInfo StartRender(RendererId r, CamSurfaceId c, RenderImageParams rip,
                                 Optional<uint32_t> logic0, Optional<uint32_t> logic1) override
    {
        mrg_tracer_render_info info;
        const uint32_t rmin[2] = { rip.regionMin[0], rip.regionMin[1] }, rmax[2] = { rip.regionMax[0], rip.regionMax[1] };
        Check(mrg_tracer_start_render(t, Raw(r), Raw(c), rip.resolution[0], rip.resolution[1], rmin, rmax, &info));
        resolution = rip.resolution;
        const size_t plane = sizeof(float) * size_t(info.width) * info.height;
        const size_t planeAligned = (plane + importAlignment - 1) / importAlignment * importAlignment;
        // the visor may still read the old buffer: take the semaphore for the
        // swap (RenderImage::Resize, RenderImage.cpp:230-290)
        if(sem && !sem->Acquire(acquireValue)) throw MRayError("mray_gb300: the render buffer was invalidated");
        FreeStaging();
        stagingBytes = 4 * planeAligned;
        staging = static_cast<Byte*>(std::aligned_alloc(importAlignment, stagingBytes));
        if(!staging) throw MRayError("mray_gb300: staging buffer allocation failed");
        std::memset(staging, 0, stagingBytes);
        if(sem) { sem->Release(); acquireValue += 1; }
        filmRGBW.assign(4 * size_t(info.width) * info.height, 0.0f);
        return RenderBufferInfo{ staging, stagingBytes, MRayColorSpaceEnum::MR_REC_709, rip.resolution,
                                 logic0.value_or(0u), logic1.value_or(0u) };
    }
    void SetCameraTransform(RendererId r, CameraTransform c) override
    {
        const float v[9] = { c.position[0], c.position[1], c.position[2], c.gazePoint[0], c.gazePoint[1],
                             c.gazePoint[2], c.up[0], c.up[1], c.up[2] };
        Check(mrg_tracer_set_camera_transform(t, Raw(r), v));
    }
    void StopRender() override { Check(mrg_tracer_stop_render(t)); }
    RendererOutput DoRenderWork() override
    {
        mrg_tracer_render_output o;
        Check(mrg_tracer_do_render_work(t, &o));
        RendererOutput out;
        uint64_t used = 0, total = 0;
        Check(mrg_tracer_device_memory(t, &total, &used));
        out.analytics = RendererAnalyticData{ o.pathsPerSecond * 1e-6, "M paths/s", double(o.samplesDone),
                                              double(o.totalSpp), "spp", o.workMs, resolution,
                                              MRayColorSpaceEnum::MR_REC_709, size_t(used), 0u, 0u };
        out.triggerSave = o.finished != 0;
        if(!sem || !staging) return out;
        // planar R, G, B, weight (RenderImage::TransferToHost, RenderImage.cpp:163-211)
        Check(mrg_tracer_read_film(t, filmRGBW.data(), filmRGBW.size() * sizeof(float)));
        if(!sem->Acquire(acquireValue)) return out;        // the visor is closing
        const size_t n = size_t(resolution[0]) * resolution[1];
        const size_t planeAligned = stagingBytes / 4;
        for(int c = 0; c < 4; c++)
        {
            float* dst = reinterpret_cast<float*>(staging + c * planeAligned);
            for(size_t i = 0; i < n; i++) dst[i] = filmRGBW[4 * i + c];
        }
        sem->Release();
        acquireValue += 2;
        out.imageOut = RenderImageSection{ Vector2ui::Zero(), resolution, Float(0), acquireValue - 1,
                                           { 0, planeAligned, 2 * planeAligned }, 3 * planeAligned };
        return out;
    }

    // ---- misc ----
    void ClearAll() override { Check(mrg_tracer_clear_all(t)); }
    void Flush() const override { Check(mrg_tracer_flush(t)); }
    GPUThreadInitFunction GetThreadInitFunction() const override { return +[]() {}; }
    void SetThreadPool(ThreadPool&) override {}
    size_t TotalDeviceMemory() const override
    {
        uint64_t total = 0, used = 0;
        Check(mrg_tracer_device_memory(t, &total, &used));
        return size_t(total);
    }
    size_t UsedDeviceMemory() const override
    {
        uint64_t total = 0, used = 0;
        Check(mrg_tracer_device_memory(t, &total, &used));
        return size_t(used);
    }
    const TracerParameters& Parameters() const override { return params; }
};

#ifdef MRAY_GB300_TRACER_ENTRYPOINTS
extern "C" MRAY_DLL_EXPORT TracerI* ConstructTracer(const TracerParameters& p) { return new TracerGB300(p); }
extern "C" MRAY_DLL_EXPORT void DestroyTracer(TracerI* p) { delete p; }
#endif
