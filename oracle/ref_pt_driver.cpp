// ref_pt_driver.cpp -- test infrastructure only: a thin extern "C" driver over
// MRay's OWN path-tracer building blocks, compiled from the MRay source tree
// (host backend, MRAY_GPU_BACKEND_CPU) by oracle/build.py:build_ref_pt().
// Nothing here restates MRay: every function constructs MRay's types and calls
// MRay's code, so the fixtures written through it (tests/golden/make_pt_golden.py)
// are the reference's outputs on fixed inputs.  The project's restatement
// (oracle/pt_oracle.c) is checked against them in tests/test_oracle_pt_golden.py.
//
// Materials are evaluated on a surface whose shading rotation is the identity
// quaternion, so the tangent frame is the world frame and the BxDF arithmetic
// is compared without a frame convention in between.
//
// Random numbers enter as the uint32 values MRay's RNGDispenser converts
// (RNGFunctions::ToFloat01, Tracer/Random.h:102-125).
#include "Tracer/MaterialsDefault.h"
#include "Tracer/MaterialsDefault.hpp"
#include "Tracer/LightsDefault.h"
#include "Tracer/LightsDefault.hpp"
#include "Tracer/LightSampler.h"
#include "Tracer/LightSampler.hpp"
#include "Tracer/CamerasDefault.h"
#include "Tracer/CamerasDefault.hpp"
#include "Tracer/Filters.h"
#include "Tracer/SpectrumContext.h"
#include "Tracer/Random.h"
#include "Tracer/DistributionFunctions.h"
#include "Tracer/Distributions.h"
#include "Tracer/PrimitiveDefaultTriangle.h"
#include "Tracer/PrimitiveDefaultTriangle.hpp"
#include "Tracer/TransformsDefault.h"
#include "Tracer/TransformsDefault.hpp"
#include "Tracer/TextureView.hpp"
#include "Tracer/HashGrid.h"
#include "Device/CPU/GPUSystemCPU.hpp"
// the wavelength sampler and the spectrum -> RGB conversion are free device
// functions of this translation unit of MRay (host backend)
#include "Tracer/SpectrumContext.cu"
// the ZSobol generator (ZSobolDetail::ZSobol) is defined in this unit of MRay
#include "Tracer/Random.cu"

#include <cstdint>
#include <cstring>
#include <vector>

namespace
{

Vector3 V3(const float* p) { return Vector3(p[0], p[1], p[2]); }
void put3(float* o, const Vector3& v) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; }
void put4(float* o, const Spectrum& s) { o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; o[3] = s[3]; }

DefaultSurface tangent_surface(const float* pos, bool backSide)
{
    return DefaultSurface
    {
        .position = V3(pos),
        .geoNormal = Vector3(0, 0, 1),
        .shadingTBN = Quaternion::Identity(),
        .uv = Vector2(0, 0),
        .dpdx = Vector2(0, 0),
        .dpdy = Vector2(0, 0),
        .backSide = backSide
    };
}

// One record of a material query (all vectors in the tangent frame).
//   in:  albedo[3], rough, metal, spec, iorFront, iorBack, backSide, pos[3],
//        wo[3], wiEval[3], xi[3] (uint32)
//   out: wi[3], wiPos[3], pdf, refl[4], passed, evalRefl[4], evalPdf, specularity
struct MatIn
{
    float albedo[3];
    float rough, metal, spec, iorF, iorB;
    uint32_t backSide;
    float pos[3];
    float wo[3];
    float wiEval[3];
    uint32_t xi[3];
};
struct MatOut
{
    float wi[3];
    float wiPos[3];
    float pdf;
    float refl[4];
    uint32_t passed;
    float evalRefl[4];
    float evalPdf;
    float specularity;
};
static_assert(sizeof(MatIn) == 21 * 4, "MatIn layout");
static_assert(sizeof(MatOut) == 18 * 4, "MatOut layout");

template<class M>
void run_material(const M& m, const MatIn& in, MatOut& out)
{
    RNGDispenser rng(Span<const uint32_t>(in.xi, 3), 0, 1);
    BxDFSample s = m.SampleBxDF(V3(in.wo), rng);
    put3(out.wi, s.wI.dir);
    put3(out.wiPos, s.wI.pos);
    out.pdf = s.pdf;
    put4(out.refl, s.eval.reflectance);
    out.passed = s.eval.isPassedThrough ? 1u : 0u;
    Ray wiE(V3(in.wiEval), V3(in.pos));
    BxDFEval e = m.Evaluate(wiE, V3(in.wo));
    put4(out.evalRefl, e.reflectance);
    out.evalPdf = m.Pdf(wiE, V3(in.wo));
    out.specularity = m.Specularity();
}

} // namespace

extern "C" {

int ref_pt_abi_version() { return 1; }

// kind: 0 Lambert, 1 Reflect, 2 Refract, 3 Unreal (MaterialsDefault.hpp)
void ref_material(int kind, const MatIn* in, MatOut* out, uint32_t n)
{
    using SC = SpectrumContextIdentity;
    SC::Converter conv;
    for(uint32_t i = 0; i < n; i++)
    {
        const MatIn& q = in[i];
        MatOut& o = out[i];
        std::memset(&o, 0, sizeof(o));
        DefaultSurface surf = tangent_surface(q.pos, q.backSide != 0);
        MaterialKey mk = MaterialKey::CombinedKey(0, 0);
        if(kind == 0)
        {
            std::vector<ParamVaryingData<2, Vector3>> alb = { ParamVaryingData<2, Vector3>(V3(q.albedo)) };
            std::vector<Optional<TracerTexView<2, Vector3>>> nm = { std::nullopt };
            LambertMatDetail::LambertMatData soa{ Span<const ParamVaryingData<2, Vector3>>(alb.data(), 1),
                                                  Span<const Optional<TracerTexView<2, Vector3>>>(nm.data(), 1) };
            LambertMatDetail::LambertMaterial<SC> m(conv, surf, soa, mk);
            run_material(m, q, o);
        }
        else if(kind == 1)
        {
            ReflectMatDetail::ReflectMatData soa{};
            ReflectMatDetail::ReflectMaterial<SC> m(conv, surf, soa, mk);
            run_material(m, q, o);
        }
        else if(kind == 2)
        {
            std::vector<Vector3> f = { Vector3(q.iorF, 0, 0) }, b = { Vector3(q.iorB, 0, 0) };
            RefractMatDetail::RefractMatData soa{ Span<const Vector3>(f.data(), 1), Span<const Vector3>(b.data(), 1) };
            RefractMatDetail::RefractMaterial<SC> m(conv, surf, soa, mk);
            run_material(m, q, o);
        }
        else
        {
            std::vector<ParamVaryingData<2, Vector3>> alb = { ParamVaryingData<2, Vector3>(V3(q.albedo)) };
            std::vector<Optional<TracerTexView<2, Vector3>>> nm = { std::nullopt };
            std::vector<ParamVaryingData<2, Float>> r = { ParamVaryingData<2, Float>(q.rough) };
            std::vector<ParamVaryingData<2, Float>> sp = { ParamVaryingData<2, Float>(q.spec) };
            std::vector<ParamVaryingData<2, Float>> mt = { ParamVaryingData<2, Float>(q.metal) };
            UnrealMatDetail::UnrealMatData soa{ Span<const ParamVaryingData<2, Vector3>>(alb.data(), 1),
                                                Span<const Optional<TracerTexView<2, Vector3>>>(nm.data(), 1),
                                                Span<const ParamVaryingData<2, Float>>(r.data(), 1),
                                                Span<const ParamVaryingData<2, Float>>(sp.data(), 1),
                                                Span<const ParamVaryingData<2, Float>>(mt.data(), 1) };
            UnrealMatDetail::UnrealMaterial<SC> m(conv, surf, soa, mk);
            run_material(m, q, o);
        }
    }
}

// BxDF building blocks (DistributionFunctions.h), one call per record:
// io[0..8] in, outputs after.
//  fresnel: in cosF, etaF, etaB -> out f
void ref_fresnel_dielectric(const float* in3, float* out, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
        out[i] = Distribution::BxDF::FresnelDielectric(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2]);
}

// VNDF sample: in V[3], alpha, xi[2] -> out H[3], pdf
void ref_vndf_sample(const float* in6, float* out4, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        auto s = Distribution::BxDF::VNDFGGXSmithSample(V3(q), q[3], Vector2(q[4], q[5]));
        put3(out4 + 4 * i, s.value);
        out4[4 * i + 3] = s.pdf;
    }
}

// Cosine-weighted hemisphere sample: xi[2] -> dir[3], pdf
void ref_cos_sample(const float* in2, float* out4, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        auto s = Distribution::Common::SampleCosDirection(Vector2(in2[2 * i], in2[2 * i + 1]));
        put3(out4 + 4 * i, s.value);
        out4[4 * i + 3] = s.pdf;
    }
}

// Russian roulette (Common::RussianRoulette): in thr[4], prob, xi ->
// out alive, thr'[4]
void ref_russian_roulette(const float* in6, float* out5, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        Spectrum t(q[0], q[1], q[2], q[3]);
        auto r = Distribution::Common::RussianRoulette(t, q[4], q[5]);
        out5[5 * i] = r.has_value() ? 1.0f : 0.0f;
        if(r.has_value()) put4(out5 + 5 * i + 1, *r);
        else for(int k = 1; k < 5; k++) out5[5 * i + k] = 0.0f;
    }
}

// MIS::BalanceCancelled<2>: in pdf[2], weight[2] -> out
void ref_balance_cancelled(const float* in4, float* out, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        std::array<Float, 2> p = { in4[4 * i], in4[4 * i + 1] }, w = { in4[4 * i + 2], in4[4 * i + 3] };
        out[i] = Distribution::MIS::BalanceCancelled<2>(p, w);
    }
}

// Ray::Nudge (Core/Ray.hpp:258-300): in pos[3], dir[3] -> out pos[3]
void ref_nudge(const float* in6, float* out3, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        Ray r(Vector3(0, 0, 1), V3(in6 + 6 * i));
        put3(out3 + 3 * i, r.Nudge(V3(in6 + 6 * i + 3)).pos);
    }
}

// Gaussian film filter (Filters.h:195-233; default radius 1):
// in radius, xi[2] -> out offset[2], pdf, weight (Evaluate), weight / pdf
void ref_gaussian_filter(const float* in3, float* out5, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        GaussianFilter f(in3[3 * i]);
        auto s = f.Sample(Vector2(in3[3 * i + 1], in3[3 * i + 2]));
        float* o = out5 + 5 * i;
        o[0] = s.value[0]; o[1] = s.value[1]; o[2] = s.pdf;
        o[3] = f.Evaluate(s.value);
        o[4] = o[3] / s.pdf;
    }
}

// Primitive-backed area light on one triangle (LightPrim<Triangle<
// TransformContextSingle>>, LightsDefault.hpp:14-165; Triangle sampling,
// PrimitiveDefaultTriangle.hpp:48-80).  The triangle's local vertices are
// moved to world space by the instance's 3x4 transform, as MRay does.
struct TriLightIn
{
    float m[12];            // row-major 3x4 local -> world
    float v9[9];            // local vertices
    uint32_t twoSided;
    float radiance[3];
    float distant[3];       // the shaded point
    uint32_t xi[2];
    float hit[2];           // (a, b) barycentrics of a light hit
    float dir[3];           // direction of the ray that hit it
    float wo[3];            // emission direction for EmitViaHit
};
struct TriLightOut
{
    float point[3];
    float samplePdf;
    float pdfSolidAngle;
    float emitHit[4];
    float emitPoint[4];     // EmitViaSurfacePoint towards the shaded point
    float area;
};
static_assert(sizeof(TriLightIn) == 38 * 4, "TriLightIn layout");
static_assert(sizeof(TriLightOut) == 14 * 4, "TriLightOut layout");

void ref_tri_light(const TriLightIn* in, TriLightOut* out, uint32_t n)
{
    using namespace DefaultTriangleDetail;
    using TC = TransformContextSingle;
    SpectrumContextIdentity::Converter conv;
    for(uint32_t i = 0; i < n; i++)
    {
        const TriLightIn& q = in[i];
        TriLightOut& o = out[i];
        std::memset(&o, 0, sizeof(o));
        Matrix3x4 mt(q.m[0], q.m[1], q.m[2], q.m[3], q.m[4], q.m[5], q.m[6], q.m[7],
                     q.m[8], q.m[9], q.m[10], q.m[11]);
        Matrix3x4 inv = mt.Inverse();
        TransformDetail::SingleTransformSoA tsoa{ Span<const Matrix3x4>(&mt, 1), Span<const Matrix3x4>(&inv, 1) };
        TC tc(tsoa, TransformKey::CombinedKey(0, 0));
        Vector3 pos[3] = { V3(q.v9), V3(q.v9 + 3), V3(q.v9 + 6) };
        Quaternion tbn[3] = { Quaternion::Identity(), Quaternion::Identity(), Quaternion::Identity() };
        Vector2 uv[3] = { Vector2(0, 0), Vector2(1, 0), Vector2(0, 1) };
        Vector3ui idx(0, 1, 2);
        TriangleData td{ Span<const Vector3>(pos, 3), Span<const Quaternion>(tbn, 3),
                         Span<const Vector2>(uv, 3), Span<const Vector3ui>(&idx, 1) };
        Triangle<TC> prim(tc, td, PrimitiveKey::CombinedKey(0, 0));
        std::vector<ParamVaryingData<2, Vector3>> rad = { ParamVaryingData<2, Vector3>(V3(q.radiance)) };
        bool two[1] = { q.twoSided != 0 };
        LightDetail::LightData lsoa{ Span<const ParamVaryingData<2, Vector3>>(rad.data(), 1), Span<const bool>(two, 1) };
        LightDetail::LightPrim<Triangle<TC>, SpectrumContextIdentity> light(conv, prim, lsoa, LightKey::CombinedKey(0, 0));
        RNGDispenser rng(Span<const uint32_t>(q.xi, 2), 0, 1);
        SampleT<Vector3> s = light.SampleSolidAngle(rng, V3(q.distant));
        put3(o.point, s.value);
        o.samplePdf = s.pdf;
        o.pdfSolidAngle = light.PdfSolidAngle(Vector2(q.hit[0], q.hit[1]), V3(q.distant), V3(q.dir));
        put4(o.emitHit, light.EmitViaHit(V3(q.wo), Vector2(q.hit[0], q.hit[1]), RayCone{}));
        Vector3 wO = Math::Normalize(V3(q.distant) - s.value);
        put4(o.emitPoint, light.EmitViaSurfacePoint(wO, s.value, RayCone{}));
        o.area = prim.GetSurfaceArea();
    }
}

// Lat-long mapping of the skysphere (SphericalCoordConverter,
// LightsDefault.hpp:174-215): in dir[3], uv[2], pdf -> out uv[2] (DirToUV),
// dir[3] (UVToDir), ToSolidAnglePdf(pdf, dir), ToSolidAnglePdf(pdf, uv)
void ref_spherical_coords(const float* in6, float* out7, uint32_t n)
{
    using C = LightDetail::SphericalCoordConverter;
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        float* o = out7 + 7 * i;
        Vector2 uv = C::DirToUV(V3(q));
        o[0] = uv[0]; o[1] = uv[1];
        put3(o + 2, C::UVToDir(Vector2(q[3], q[4])));
        o[5] = C::ToSolidAnglePdf(q[5], V3(q));
        o[6] = C::ToSolidAnglePdf(q[5], Vector2(q[3], q[4]));
    }
}

// Piecewise-constant 2D distribution sampling (DistributionPwC<2>,
// Distributions.h:120-270) over given CDFs: cdfX is h rows of w entries
// (each row's running sum normalised to end at 1), cdfY the h marginal
// entries.  in xi[2] -> out uv[2], pdf; in uvq[2] -> out PdfUV.
void ref_pwc2d(const float* cdfX, const float* cdfY, uint32_t w, uint32_t h,
               const float* xi2, float* out3, const float* uvq2, float* outPdf, uint32_t n)
{
    using namespace Distribution;
    std::vector<DistributionPwC<1>> rows;
    rows.reserve(h);
    for(uint32_t r = 0; r < h; r++) rows.emplace_back(Span<const Float>(cdfX + (size_t)r * w, w));
    DistributionPwC<1> marg(Span<const Float>(cdfY, h));
    DistributionPwC<2> d2(Span<const DistributionPwC<1>>(rows.data(), h), marg);
    for(uint32_t i = 0; i < n; i++)
    {
        auto s = d2.SampleUV(Vector2(xi2[2 * i], xi2[2 * i + 1]));
        out3[3 * i] = s.value[0]; out3[3 * i + 1] = s.value[1]; out3[3 * i + 2] = s.pdf;
        outPdf[i] = d2.PdfUV(Vector2(uvq2[2 * i], uvq2[2 * i + 1]));
    }
}

// Pinhole camera (CameraPinhole, CamerasDefault.hpp:8-36 and EvaluateRay
// :94-135).  cam: pos[3], gaze[3], up[3], fov[2] (radians), near, far.
// per ray in: pixel[2] (uint32), offset[2], range[2] -> out dir[3], pos[3]
void ref_camera(const float* cam13, const uint32_t res[2],
                const uint32_t* pix, const float* off4, float* out6, uint32_t n)
{
    using namespace CameraDetail;
    Vector3 p = V3(cam13), g = V3(cam13 + 3), u = V3(cam13 + 6);
    Vector4 fp(cam13[9], cam13[10], cam13[11], cam13[12]);
    CamPinholeData soa{ Span<const Vector4>(&fp, 1), Span<const Vector3>(&p, 1),
                        Span<const Vector3>(&g, 1), Span<const Vector3>(&u, 1) };
    CameraPinhole c(soa, CameraKey::CombinedKey(0, 0));
    for(uint32_t i = 0; i < n; i++)
    {
        CameraRaySample r = c.EvaluateRay(Vector2ui(pix[2 * i], pix[2 * i + 1]), Vector2ui(res[0], res[1]),
                                          Vector2(off4[4 * i], off4[4 * i + 1]),
                                          Vector2(off4[4 * i + 2], off4[4 * i + 3]));
        put3(out6 + 6 * i, r.value.ray.dir);
        put3(out6 + 6 * i + 3, r.value.ray.pos);
    }
}

// ---- spectral (Jakob 2019 converter, SpectrumContext.hpp/.cu) ----------
// The converter's data built exactly as SpectrumContextJakob2019's
// constructor builds it (SpectrumContext.cu:355-531) for Rec.709, over
// MRay's CPU texture views of a resolution-64 MR_SPECTRA LUT (the
// converter's compile-time resolution).
struct SpecCtx
{
    std::vector<float>   lut;                   // 9 * 64^3, file order
    std::vector<Vector4> observer;              // padded, normalised CIE 1931
    std::vector<float>   illuminant;            // normalised SPD
    const Byte*          ptrs[11];
    TextureInitParams<3> tp3;
    TextureInitParams<1> tp1;
    Jakob2019Detail::Data* data = nullptr;
};

void* ref_spec_create(const float* lut, uint32_t res)
{
    constexpr uint32_t N = Jakob2019Detail::Data::N;
    if(res != N) return nullptr;
    SpecCtx* c = new SpecCtx();
    c->lut.assign(lut, lut + 9ull * N * N * N);
    c->observer.resize(Color::CIE_1931_N);
    c->illuminant.resize(Color::CIE_1931_N);
    const auto cs = MRayColorSpaceEnum::MR_REC_709;
    const auto& spd = Color::SelectIlluminantSPD(cs);
    Float norm = Color::CIE_1931_Y_INTEGRAL;
    norm /= Color::SelectIlluminantSPDNormFactor(cs);
    for(uint32_t i = 0; i < Color::CIE_1931_N; i++)
    {
        static constexpr Vector3 SUM = Vector3(Color::CIE_1931_X_INTEGRAL, Color::CIE_1931_Y_INTEGRAL,
                                               Color::CIE_1931_Z_INTEGRAL);
        static constexpr Vector3 W = Vector3(1) / SUM;
        c->observer[i] = Vector4(Color::CIE_1931_XYZ[i] * W, 0);
        c->illuminant[i] = spd[i] * norm;
    }
    c->tp3 = TextureInitParams<3>{ .size = Vector3ui(N), .normIntegers = false,
                                   .interp = MRayTextureInterpEnum::MR_LINEAR,
                                   .eResolve = MRayTextureEdgeResolveEnum::MR_CLAMP };
    c->tp1 = TextureInitParams<1>{ .size = Color::CIE_1931_N, .normIntegers = false, .normCoordinates = false,
                                   .interp = MRayTextureInterpEnum::MR_LINEAR,
                                   .eResolve = MRayTextureEdgeResolveEnum::MR_CLAMP };
    for(int t = 0; t < 9; t++)
        c->ptrs[t] = reinterpret_cast<const Byte*>(c->lut.data() + (size_t)t * N * N * N);
    c->ptrs[9] = reinterpret_cast<const Byte*>(c->observer.data());
    c->ptrs[10] = reinterpret_cast<const Byte*>(c->illuminant.data());
    using TV3 = TextureView<3, Float>;
    const auto fEnum = MRayPixelTypeRT(static_cast<MRayPixelEnum>(mray::host::PixelTypeToEnum::template Find<Float>));
    const auto v4Enum = MRayPixelTypeRT(static_cast<MRayPixelEnum>(mray::host::PixelTypeToEnum::template Find<Vector4>));
    Matrix3x3 r2x = Color::SelectRGBToXYZMatrix(cs);
    c->data = new Jakob2019Detail::Data
    {
        .RGBToXYZ = r2x,
        .XYZToRGB = r2x.Inverse(),
        .lut =
        {
            Jakob2019Detail::Data::Table3D{ TV3(&c->ptrs[0], &c->tp3, fEnum), TV3(&c->ptrs[1], &c->tp3, fEnum),
                                            TV3(&c->ptrs[2], &c->tp3, fEnum) },
            Jakob2019Detail::Data::Table3D{ TV3(&c->ptrs[3], &c->tp3, fEnum), TV3(&c->ptrs[4], &c->tp3, fEnum),
                                            TV3(&c->ptrs[5], &c->tp3, fEnum) },
            Jakob2019Detail::Data::Table3D{ TV3(&c->ptrs[6], &c->tp3, fEnum), TV3(&c->ptrs[7], &c->tp3, fEnum),
                                            TV3(&c->ptrs[8], &c->tp3, fEnum) },
        },
        .spdObserverXYZ = TextureView<1, Vector3>(&c->ptrs[9], &c->tp1, v4Enum),
        .spdIlluminant = TextureView<1, Float>(&c->ptrs[10], &c->tp1, fEnum)
    };
    return c;
}

void ref_spec_destroy(void* p)
{
    SpecCtx* c = static_cast<SpecCtx*>(p);
    if(!c) return;
    delete c->data;
    delete c;
}

// ConvertAlbedo (radiance = 0) / ConvertRadiance (radiance = 1) of rgb[3] at waves[4]
void ref_spec_convert(void* p, int radiance, const float* rgb3, const float* waves4, float* out4, uint32_t n)
{
    SpecCtx* c = static_cast<SpecCtx*>(p);
    for(uint32_t i = 0; i < n; i++)
    {
        SpectrumWaves w;
        for(int k = 0; k < 4; k++) w[k] = waves4[4 * i + k];
        Jakob2019Detail::Converter conv(w, *c->data);
        Spectrum s = radiance ? conv.ConvertRadiance(V3(rgb3 + 3 * i)) : conv.ConvertAlbedo(V3(rgb3 + 3 * i));
        put4(out4 + 4 * i, s);
    }
}

// SingleSampleSpectrumWavelength (SpectrumContext.cu:9-130):
// mode 0 uniform, 1 Gaussian MIS, 2 hyperbolic (the renderer default)
void ref_spec_sample_waves(int mode, const uint32_t* xi, float* waves4, float* pdf4, uint32_t n)
{
    WavelengthSampleMode m((mode == 0) ? WavelengthSampleMode::UNIFORM
                           : (mode == 1) ? WavelengthSampleMode::GAUSSIAN_MIS : WavelengthSampleMode::HYPERBOLIC_PBRT);
    for(uint32_t i = 0; i < n; i++)
    {
        SpectrumWaves w;
        Spectrum pdf;
        RNGDispenser rng(Span<const uint32_t>(xi + i, 1), 0, 1);
        SingleSampleSpectrumWavelength(w, pdf, rng, m);
        for(int k = 0; k < 4; k++) { waves4[4 * i + k] = w[k]; pdf4[4 * i + k] = pdf[k]; }
    }
}

// ConvertSpectraToRGBSingle (SpectrumContext.cu:134-160)
void ref_spec_to_rgb(void* p, const float* value4, const float* waves4, const float* pdf4, float* rgb3, uint32_t n)
{
    SpecCtx* c = static_cast<SpecCtx*>(p);
    for(uint32_t i = 0; i < n; i++)
    {
        Spectrum v, pdf;
        SpectrumWaves w;
        for(int k = 0; k < 4; k++) { v[k] = value4[4 * i + k]; pdf[k] = pdf4[4 * i + k]; w[k] = waves4[4 * i + k]; }
        Spectrum r = ConvertSpectraToRGBSingle(v, w, pdf, c->data->spdObserverXYZ, c->data->XYZToRGB);
        for(int k = 0; k < 3; k++) rgb3[3 * i + k] = r[k];
    }
}

// ZSobolDetail::ZSobol (Random.cu:265-425): in px, py, seed, sampleIndex,
// initialMaxSPP, resMaxBits, dim, size (1..3) -> Next / Next2D / Next3D
// (out[0..size-1]); the pixel's Morton code is Graphics::MortonCode::Compose2D
// as RNGGroupZSobol computes it (Random.cu:1180-1190).
void ref_zsobol(const uint32_t* in8, uint32_t* out3, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const uint32_t* q = in8 + 8 * i;
        using Graphics::MortonCode::Compose2D;
        ZSobolDetail::LocalState ls{ .pixelMortonCode = Compose2D<uint64_t>(Vector2ui(q[0], q[1])),
                                     .sampleIndex = q[3], .seed = q[2] };
        ZSobolDetail::GlobalState gs{ .initialMaxSPP = q[4], .resMaxBits = q[5] };
        ZSobolDetail::ZSobol z(ls, gs);
        uint32_t* o = out3 + 3 * i;
        o[0] = o[1] = o[2] = 0;
        if(q[7] == 1) o[0] = z.Next(q[6]);
        else if(q[7] == 2) { Vector2ui v = z.Next2D(q[6]); o[0] = v[0]; o[1] = v[1]; }
        else { Vector3ui v = z.Next3D(q[6]); o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; }
    }
}

// Per-pixel seeds of the ZSobol group (RNGGroupZSobol ctor, Random.cu:
// 1175-1200): seed32 = hi ^ lo of the 64-bit seed, then the outputs of
// std::mt19937(seed32) in pixel order.
void ref_zsobol_seeds(uint64_t seed, uint32_t count, uint32_t* out)
{
    uint32_t seed32 = static_cast<uint32_t>((seed >> 32) ^ (seed & 0xFFFFFFFF));
    std::mt19937 rng(seed32);
    for(uint32_t i = 0; i < count; i++) out[i] = uint32_t(rng());
}

// MRay's independent sampler: PermutedCG32 (Random.h:762-842) seeded by
// GenerateState.  ref_pcg32_jump: out[i] = the number after Advance(delta[i])
// of the stream seeded by seeds[i]; ref_pcg32_seq: the first n numbers of one
// stream by successive Next calls.
void ref_pcg32_jump(const uint32_t* seeds, const uint32_t* delta, uint32_t count, uint32_t* out)
{
    for(uint32_t i = 0; i < count; i++)
    {
        PermutedCG32::State st = PermutedCG32::GenerateState(seeds[i]);
        PermutedCG32 rng(st);
        rng.Advance(delta[i]);
        out[i] = rng.Next();
    }
}

void ref_pcg32_seq(uint32_t seed, uint32_t n, uint32_t* out)
{
    PermutedCG32::State st = PermutedCG32::GenerateState(seed);
    PermutedCG32 rng(st);
    for(uint32_t i = 0; i < n; i++) out[i] = rng.Next();
}

// MRay's guided path tracer's building blocks.
// Gaussian (vMF) lobe: in7 = dir[3], kappa, xi0, xi1, (unused); w3 = a direction
// to evaluate.  out8 = alpha, sample dir[3], Pdf(sample), Pdf(w), XOverExp1M(-2 kappa),
// XOverExp1MRecip(-2 kappa).
void ref_guide_lobe(const float* in7, const float* w3, float* out8, uint32_t n)
{
    using Distribution::GaussianLobe;
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in7 + 7 * i;
        GaussianLobe l(Vector3(q[0], q[1], q[2]), q[3]);
        auto s = l.Sample(Vector2(q[4], q[5]));
        const float* w = w3 + 3 * i;
        float* o = out8 + 8 * i;
        o[0] = l.alpha;
        o[1] = s.value[0]; o[2] = s.value[1]; o[3] = s.value[2];
        o[4] = s.pdf;
        o[5] = l.Pdf(Vector3(w[0], w[1], w[2]));
        o[6] = GaussianLobe::XOverExp1M(-2.0f * q[3]);
        o[7] = GaussianLobe::XOverExp1MRecip(-2.0f * q[3]);
    }
}

// Concentric octahedral mapping: dir3 -> st (DirectionToConcentricOctahedral),
// st2 -> dir (ConcentricOctahedralToDirection).
void ref_conc_octa(const float* dir3, float* st2, const float* stIn, float* dirOut, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        Vector2 st = Graphics::DirectionToConcentricOctahedral(Vector3(dir3[3 * i], dir3[3 * i + 1], dir3[3 * i + 2]));
        st2[2 * i] = st[0]; st2[2 * i + 1] = st[1];
        Vector3 d = Graphics::ConcentricOctahedralToDirection(Vector2(stIn[2 * i], stIn[2 * i + 1]));
        dirOut[3 * i] = d[0]; dirOut[3 * i + 1] = d[1]; dirOut[3 * i + 2] = d[2];
    }
}

// Hash-grid codes of HashGridView (HashGrid.h): view = the grid's fields as
// floats / words [cam3, rmin3, rmax3, baseDelta, baseDim, normalDelta,
// normalDim, maxLevelOffset, tanConeHalfTimes2]; in6 = pos, normal; rng =
// PermutedCG32 states (updated).  out: GenCode, GenCodeStochastic.
void ref_guide_codes(const float* view15, const float* in6, uint32_t* rng, uint64_t* out2, uint32_t n)
{
    uint32_t counter = 0;
    HashGridView v{ Span<SpatioDirCode>(), Span<uint32_t, 1>(&counter, 1),
                    Vector3(view15[0], view15[1], view15[2]),
                    AABB3(Vector3(view15[3], view15[4], view15[5]), Vector3(view15[6], view15[7], view15[8])),
                    view15[9], uint32_t(view15[10]), view15[11], uint32_t(view15[12]), uint32_t(view15[13]),
                    0u, view15[14] };
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        const Vector3 p(q[0], q[1], q[2]), nn(q[3], q[4], q[5]);
        out2[2 * i] = uint64_t(v.GenCode(p, nn));
        BackupRNG r(rng[i]);
        out2[2 * i + 1] = uint64_t(v.GenCodeStochastic(p, nn, r));
    }
}

// HashGridView::TryInsert then Search over a table of `size` (a power of two)
// codes: slots[i] = TryInsert(codes[i]), found[i] = Search(probe[i]).
void ref_guide_table(const uint64_t* codes, uint32_t n, const uint64_t* probe, uint32_t m, uint32_t size,
                     uint32_t* slots, uint32_t* found)
{
    std::vector<SpatioDirCode> table(size, HashGridView::EMPTY_VAL);
    uint32_t counter = 0;
    HashGridView v{ Span<SpatioDirCode>(table.data(), size), Span<uint32_t, 1>(&counter, 1), Vector3::Zero(),
                    AABB3(Vector3::Zero(), Vector3(1)), 1.0f, 1u, 1.0f, 1u, 0u, size, 1.0f };
    for(uint32_t i = 0; i < n; i++) slots[i] = v.TryInsert(SpatioDirCode(codes[i])).allocationIndex;
    for(uint32_t i = 0; i < m; i++) found[i] = v.Search(SpatioDirCode(probe[i])).value_or(0xFFFFFFFFu);
}

// Ray cones (RayCone::Advance / Project, RayConeSurface::ConeAfterScatter,
// Source/Tracer/TracerTypes.h:323-380) and RefractMaterial::RefractRayCone
// (MaterialsDefault.hpp:353-462) on the tangent surface (geometric normal +z).
//   in:  aperture, width, t, f[3], d[3], betaN, wo[3], iorFront, iorBack,
//        backSide, wi[3], 0
//   out: advanced cone (aperture, width), a1[3], a2[3] (Project of the
//        advanced cone), the refracted back cone, ConeAfterScatter(wi, +z)
void ref_cone(const float* in20, float* out12, uint32_t n)
{
    using SC = SpectrumContextIdentity;
    SC::Converter conv;
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in20 + 20 * i;
        float* o = out12 + 12 * i;
        RayCone c;
        c.aperture = q[0];
        c.width = q[1];
        const RayCone adv = c.Advance(q[2]);
        const auto ax = adv.Project(V3(q + 3), V3(q + 6));
        o[0] = adv.aperture; o[1] = adv.width;
        put3(o + 2, ax[0]);
        put3(o + 5, ax[1]);
        const float zero[3] = { 0, 0, 0 };
        DefaultSurface surf = tangent_surface(zero, q[15] != 0.0f);
        std::vector<Vector3> f = { Vector3(q[13], 0, 0) }, b = { Vector3(q[14], 0, 0) };
        RefractMatDetail::RefractMatData soa{ Span<const Vector3>(f.data(), 1), Span<const Vector3>(b.data(), 1) };
        RefractMatDetail::RefractMaterial<SC> m(conv, surf, soa, MaterialKey::CombinedKey(0, 0));
        RayConeSurface rs;
        rs.rayConeFront = adv;
        rs.rayConeBack = adv;
        rs.betaN = q[9];
        const RayConeSurface rr = m.RefractRayCone(rs, V3(q + 10));
        o[8] = rr.rayConeBack.aperture; o[9] = rr.rayConeBack.width;
        const RayCone after = rr.ConeAfterScatter(V3(q + 16), Vector3(0, 0, 1));
        o[10] = after.aperture; o[11] = after.width;
    }
}

// Graphics::ConvertPixelIndices (GraphicsFunctions.h:527-538), 2D:
// in: index[2], toResolution[2], fromResolution[2] -> out[2]
void ref_pixel_indices(const float* in6, float* out2, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        const Vector2 r = Graphics::ConvertPixelIndices(Vector2(q[0], q[1]), Vector2(q[2], q[3]), Vector2(q[4], q[5]));
        out2[2 * i] = r[0];
        out2[2 * i + 1] = r[1];
    }
}

}  // extern "C"
