// pt_device.cuh -- device building blocks of the wavefront path tracers
// (materials, lights, skysphere, spectral conversion, random numbers,
// textures, NEE), shared by the plain path tracer (pt.cu) and the guided
// one (guided.cu).  Arithmetic that the CPU oracle mirrors uses the _rn
// intrinsics (no fused multiply-add), so both render the same paths up to
// the library's sin / cos / log, which differ between CUDA and the host C
// library by a few ulps.
#pragma once
#include "mrg_pt.h"
#include "zsobol.cuh"
#include "mrg_device.cuh"

namespace mrg {

namespace {

constexpr int kPtTPB = 256;
constexpr uint32_t kMissMark = 0xFFFFFFFFu;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;

__device__ __forceinline__ uint32_t pcg_hash(uint32_t v)
{
    const uint32_t state = v * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ uint32_t path_key(uint32_t seed, uint32_t pixel, uint32_t sample)
{
    return pcg_hash(pcg_hash(seed ^ 0x9E3779B9u) ^ pcg_hash(pixel) ^ pcg_hash(sample + 0x632BE5ABu));
}
__device__ __forceinline__ float rnd(uint32_t key, uint32_t bounce, uint32_t dim)
{
    const uint32_t h = pcg_hash(key ^ pcg_hash((bounce << 4) | dim));
    return __fmul_rn((float)(h >> 8), 1.0f / 16777216.0f);
}

// Unfused a*b + c and friends (the oracle is compiled without contraction);
// fma only where MRay's own code calls it.
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
// Math::Dot (Source/Core/Math.h:1585-1596): r = 0; r = fma(a_i, b_i, r).
__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmaf_rn(a.x, b.x, 0.0f)));
}
// LengthSqr of a 2-vector with the same fma chain.
__device__ __forceinline__ float len2_2(float x, float y) { return __fmaf_rn(y, y, __fmaf_rn(x, x, 0.0f)); }
// Math::Cross (Math.h:1627-1633): one fma per component.
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(__fmaf_rn(a.y, b.z, -mul(a.z, b.y)),
                       __fmaf_rn(a.z, b.x, -mul(a.x, b.z)),
                       __fmaf_rn(a.x, b.y, -mul(a.y, b.x)));
}
__device__ __forceinline__ float3 normalize3(float3 v)
{
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(v, v)));
    return make_float3(mul(v.x, inv), mul(v.y, inv), mul(v.z, inv));
}
__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }

// Ray::Nudge (Source/Core/Ray.hpp:258-300).
__device__ __forceinline__ float nudge1(float p, float n)
{
    const int32_t ofi = (int32_t)(mul(256.0f, n));
    int32_t pi = __float_as_int(p);
    pi += (p < 0.0f) ? -ofi : ofi;
    return (fabsf(p) < (1.0f / 32.0f)) ? add(p, mul(1.0f / 65536.0f, n)) : __int_as_float(pi);
}
__device__ __forceinline__ float3 nudge(float3 p, float3 n)
{
    return make_float3(nudge1(p.x, n.x), nudge1(p.y, n.y), nudge1(p.z, n.z));
}

// Duff et al. orthonormal basis about n.
__device__ __forceinline__ void onb(float3 n, float3& t, float3& b)
{
    const float sign = copysignf(1.0f, n.z);
    const float a = __fdiv_rn(-1.0f, add(sign, n.z));
    const float bb = mul(mul(n.x, n.y), a);
    t = make_float3(add(1.0f, mul(mul(mul(sign, n.x), n.x), a)), mul(sign, bb), -mul(sign, n.x));
    b = make_float3(bb, add(sign, mul(mul(n.y, n.y), a)), -n.y);
}


// ---------------------------------------------------------------------------
// Materials (MaterialsDefault.hpp, DistributionFunctions.h), unfused float
// arithmetic mirroring the oracle.  Vectors are in the tangent frame (z = n).
// ---------------------------------------------------------------------------
constexpr float kSpecularThreshold = 0.95f;   // MaterialC.h:11

__device__ __forceinline__ float sqrt_max(float x) { return __fsqrt_rn(fmaxf(x, 0.0f)); }

__device__ __forceinline__ float d_ggx(float ndh, float alpha)
{
    const float a2 = mul(alpha, alpha);
    float den = add(mul(mul(ndh, ndh), sub(a2, 1.0f)), 1.0f);
    den = mul(den, den);
    den = mul(den, kPi);
    return __fdiv_rn(a2, den);
}
__device__ __forceinline__ float lambda_smith(float3 v, float alpha)
{
    const float a2 = mul(alpha, alpha);
    const float inner = __fdiv_rn(mul(a2, add(mul(v.x, v.x), mul(v.y, v.y))), mul(v.z, v.z));
    return mul(sub(__fsqrt_rn(add(1.0f, inner)), 1.0f), 0.5f);
}
__device__ __forceinline__ float g_single(float3 v, float alpha)
{
    return __fdiv_rn(1.0f, add(1.0f, lambda_smith(v, alpha)));
}
__device__ __forceinline__ float g_correlated(float3 o, float3 i, float alpha)
{
    return __fdiv_rn(1.0f, add(add(lambda_smith(o, alpha), lambda_smith(i, alpha)), 1.0f));
}
__device__ __forceinline__ float schlick1(float vdh, float f0)
{
    const float pw = sub(1.0f, vdh);
    const float pw2 = mul(pw, pw);
    const float pw5 = mul(mul(pw2, pw2), pw);
    return add(mul(sub(1.0f, f0), pw5), f0);
}
__device__ __forceinline__ float vndf_pdf(float3 V, float3 H, float alpha)
{
    const float vdh = fmaxf(0.0f, dot3(H, V));
    const float ndh = fmaxf(0.0f, H.z);
    const float ndv = fmaxf(0.0f, V.z);
    const float D = d_ggx(ndh, alpha);
    const float G = g_single(V, alpha);
    if(ndv == 0.0f) return 0.0f;
    return __fdiv_rn(mul(mul(vdh, D), G), ndv);
}
// Heitz 2018, "Sampling the GGX Distribution of Visible Normals".
__device__ __forceinline__ float3 vndf_sample(float3 V, float a, float xi0, float xi1)
{
    float3 vh = normalize3(make_float3(mul(a, V.x), mul(a, V.y), V.z));
    const float len2 = len2_2(vh.x, vh.y);        // LengthSqr(Vector2(VHemi))
    float3 T1;
    if(len2 > 0.0f)
    {
        const float rs = __fdiv_rn(1.0f, __fsqrt_rn(len2));
        T1 = make_float3(mul(-vh.y, rs), mul(vh.x, rs), 0.0f);
    }
    else T1 = make_float3(1.0f, 0.0f, 0.0f);
    const float3 T2 = cross3(vh, T1);
    const float r = __fsqrt_rn(xi0);
    const float phi = mul(mul(2.0f, kPi), xi1);
    const float t1 = mul(r, cosf(phi));
    float t2 = mul(r, sinf(phi));
    const float sS = mul(0.5f, add(1.0f, vh.z));
    t2 = add(mul(sub(1.0f, sS), __fsqrt_rn(sub(1.0f, mul(t1, t1)))), mul(sS, t2));
    const float val = sub(sub(1.0f, mul(t1, t1)), mul(t2, t2));
    const float sq = sqrt_max(val);
    const float3 nh = make_float3(add(add(mul(t1, T1.x), mul(t2, T2.x)), mul(sq, vh.x)),
                                  add(add(mul(t1, T1.y), mul(t2, T2.y)), mul(sq, vh.y)),
                                  add(add(mul(t1, T1.z), mul(t2, T2.z)), mul(sq, vh.z)));
    const float3 nm = make_float3(mul(a, nh.x), mul(a, nh.y), sqrt_max(nh.z));
    const float n2 = dot3(nm, nm);
    if(n2 < 1.0e-5f) return make_float3(0.0f, 0.0f, 1.0f);
    const float rs = __fdiv_rn(1.0f, __fsqrt_rn(n2));
    return make_float3(mul(nm.x, rs), mul(nm.y, rs), mul(nm.z, rs));
}
__device__ __forceinline__ float burley(float ndl, float ndv, float ldh, float rough)
{
    const float fd90 = add(0.5f, mul(mul(mul(2.0f, rough), ldh), ldh));
    const float p1 = sub(1.0f, ndl), p2 = sub(1.0f, ndv);
    const float p1s = mul(p1, p1), p2s = mul(p2, p2);      // pw5 = pw2 * pw2 * pw
    const float a = add(1.0f, mul(sub(fd90, 1.0f), mul(mul(p1s, p1s), p1)));
    const float b = add(1.0f, mul(sub(fd90, 1.0f), mul(mul(p2s, p2s), p2)));
    return mul(a, b);
}
__device__ __forceinline__ float unreal_ratio(const PtSurface& m, float avg)
{
    float integ = mul(mul(2.0f, kPi), avg);
    integ = mul(integ, sub(1.0f, m.mat.x));
    const float specR = add(mul(m.mat.y, sub(1.0f, m.mat.x)), mul(avg, m.mat.x));
    const float total = add(specR, integ);
    return (total == 0.0f) ? 0.0f : __fdiv_rn(integ, total);
}

// Channel values of a colour: RGB (3) or 4 sampled wavelengths.
struct Chan { float v[4]; };

__device__ __forceinline__ Chan chan(float a, float b, float c, float d)
{
    Chan r; r.v[0] = a; r.v[1] = b; r.v[2] = c; r.v[3] = d; return r;
}
__device__ __forceinline__ Chan chan(float4 f) { return chan(f.x, f.y, f.z, f.w); }
__device__ __forceinline__ float4 f4(const Chan& c) { return make_float4(c.v[0], c.v[1], c.v[2], c.v[3]); }

// albedo.Sum() * 0.3333 over the Spectrum's channels (MaterialsDefault.hpp:548)
template<int NC>
__device__ __forceinline__ float avg_albedo(const Chan& a)
{
    float s = add(add(a.v[0], a.v[1]), a.v[2]);
    if(NC == 4) s = add(s, a.v[3]);
    return mul(s, 0.3333f);
}
template<int NC>
__device__ __forceinline__ float specularity(const PtSurface& m, const Chan& alb)
{
    if(m.info.w == kMatReflect || m.info.w == kMatRefract) return 1.0f;
    if(m.info.w == kMatUnreal) return sub(1.0f, unreal_ratio(m, avg_albedo<NC>(alb)));
    return 0.0f;
}
__device__ __forceinline__ float f0_of(const PtSurface& m, float alb)
{
    return add(mul(mul(m.mat.y, 0.08f), sub(1.0f, m.mat.x)), mul(alb, m.mat.x));
}
// UnrealMaterial::Evaluate + Pdf (V, L in the tangent frame).
template<int NC>
__device__ __forceinline__ Chan unreal_eval(const PtSurface& m, const Chan& alb, float3 V, float3 L, float& pdfOut)
{
    const float rough = m.albedo.w;
    const float alpha = mul(rough, rough);
    const float3 H = normalize3(make_float3(add(L.x, V.x), add(L.y, V.y), add(L.z, V.z)));
    const float ldh = fmaxf(0.0f, dot3(L, H));
    const float vdh = fmaxf(0.0f, dot3(V, H));
    const float ndh = fmaxf(0.0f, H.z);
    const float ndv = fmaxf(0.0f, V.z);
    const float D = d_ggx(ndh, alpha);
    const bool dBad = isnan(D) || isinf(D);
    const float Dn = dBad ? 0.0f : D;
    float G = g_correlated(V, L, alpha);
    G = (ldh == 0.0f) ? 0.0f : G;
    G = (vdh == 0.0f) ? 0.0f : G;
    const float ndl = fmaxf(0.0f, L.z);
    const float corr = burley(ndl, ndv, ldh, rough);
    Chan out = chan(0, 0, 0, 0);
#pragma unroll
    for(int k = 0; k < NC; k++)
    {
        const float F = schlick1(vdh, f0_of(m, alb.v[k]));
        const float spec = (ndv == 0.0f) ? 0.0f : __fdiv_rn(mul(mul(mul(Dn, F), G), 0.25f), ndv);
        const float diff = mul(mul(mul(ndl, mul(sub(1.0f, m.mat.x), alb.v[k])), kInvPi), corr);
        out.v[k] = add(diff, spec);
    }
    const float ratio = unreal_ratio(m, avg_albedo<NC>(alb));
    float pd = mul(L.z, kInvPi);
    pd = (pd <= 1.0e-5f) ? 0.0f : pd;
    float ps = vndf_pdf(V, H, alpha);
    ps = dBad ? 0.0f : ps;
    ps = (vdh == 0.0f) ? 0.0f : __fdiv_rn(ps, mul(4.0f, vdh));
    pdfOut = add(mul(pd, ratio), mul(ps, sub(1.0f, ratio)));
    return out;
}
__device__ __forceinline__ float fresnel_dielectric(float cosF, float etaF, float etaB)
{
    const float sinF = sqrt_max(sub(1.0f, mul(cosF, cosF)));
    const float sinB = mul(__fdiv_rn(etaF, etaB), sinF);
    if(sinF >= 1.0f) return 1.0f;
    const float cosB = sqrt_max(sub(1.0f, mul(sinB, sinB)));
    float par = __fdiv_rn(sub(mul(etaB, cosF), mul(etaF, cosB)), add(mul(etaB, cosF), mul(etaF, cosB)));
    par = mul(par, par);
    float per = __fdiv_rn(sub(mul(etaF, cosF), mul(etaB, cosB)), add(mul(etaF, cosF), mul(etaB, cosB)));
    per = mul(per, per);
    return mul(add(par, per), 0.5f);
}

// ---------------------------------------------------------------------------
// Skysphere (LightsDefault.hpp:175-222, 300-420) and its piecewise-constant
// 2D distribution (Distributions.h:128-270).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t wrap_index(int32_t i, int32_t n)
{
    i = i % n;
    return (i < 0) ? i + n : i;
}

// Bilinear, wrap-addressed read with the host texture view's fraction rule
// (a negative texel coordinate keeps the absolute value of its fraction).
__device__ float3 env_read(const PtEnv& E, float u, float v)
{
    const float tx = sub(mul(u, (float)E.width), 0.5f), ty = sub(mul(v, (float)E.height), 0.5f);
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    const int32_t x0 = wrap_index(sx, (int32_t)E.width), x1 = wrap_index(sx + 1, (int32_t)E.width);
    const int32_t y0 = wrap_index(sy, (int32_t)E.height), y1 = wrap_index(sy + 1, (int32_t)E.height);
    const float4 p00 = __ldg(&E.texels[(size_t)y0 * E.width + x0]);
    const float4 p10 = __ldg(&E.texels[(size_t)y0 * E.width + x1]);
    const float4 p01 = __ldg(&E.texels[(size_t)y1 * E.width + x0]);
    const float4 p11 = __ldg(&E.texels[(size_t)y1 * E.width + x1]);
    const float gx = sub(1.0f, fx), gy = sub(1.0f, fy);
    const float ax = add(mul(p00.x, gx), mul(p10.x, fx)), bxx = add(mul(p01.x, gx), mul(p11.x, fx));
    const float ay = add(mul(p00.y, gx), mul(p10.y, fx)), byy = add(mul(p01.y, gx), mul(p11.y, fx));
    const float az = add(mul(p00.z, gx), mul(p10.z, fx)), bzz = add(mul(p01.z, gx), mul(p11.z, fx));
    return make_float3(add(mul(ax, gy), mul(bxx, fy)), add(mul(ay, gy), mul(byy, fy)),
                       add(mul(az, gy), mul(bzz, fy)));
}

__device__ __forceinline__ float2 env_dir_to_uv(float3 d)
{
    // Y-up -> Z-up (z, x, y); azimuth atan2(y, x), inclination acos(z)
    const float az = atan2f(d.x, d.z);
    const float incl = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f));
    return make_float2(__fdiv_rn(mul(add(az, kPi), 0.5f), kPi), sub(1.0f, mul(incl, kInvPi)));
}

__device__ __forceinline__ float env_sa_pdf_sin(float pdf, float sinPhi)
{
    return (sinPhi <= 0.0f) ? 0.0f : __fdiv_rn(pdf, mul(mul(2.0f, mul(kPi, kPi)), sinPhi));
}

__device__ __forceinline__ float3 rows_apply(const float4 (&m)[3], float3 v)
{
    return make_float3(add(add(mul(m[0].x, v.x), mul(m[0].y, v.y)), mul(m[0].z, v.z)),
                       add(add(mul(m[1].x, v.x), mul(m[1].y, v.y)), mul(m[1].z, v.z)),
                       add(add(mul(m[2].x, v.x), mul(m[2].y, v.y)), mul(m[2].z, v.z)));
}

// DistributionPwC<1>::SampleIndex: lower bound, position in the bin, and
// every value >= 1 moved down by one ulp.
__device__ float pwc1_sample_index(const float* __restrict__ cdf, uint32_t n, float xi, float& pdf)
{
    uint32_t lo = 0, cnt = n;
    while(cnt > 0u)
    {
        const uint32_t step = cnt >> 1, mid = lo + step;
        if(__ldg(&cdf[mid]) < xi) { lo = mid + 1u; cnt -= step + 1u; }
        else cnt = step;
    }
    const float prev = (lo == 0u) ? 0.0f : __ldg(&cdf[lo - 1u]);
    const float my = __ldg(&cdf[lo]);
    const float t = __fdiv_rn(sub(xi, prev), sub(my, prev));
    float indexF = add((float)lo, t);
    indexF = (indexF < 1.0f) ? indexF : nextafterf(indexF, -3.402823466e+38f);
    pdf = mul(sub(my, prev), (float)n);
    return indexF;
}

__device__ __forceinline__ float pwc1_pdf_index(const float* __restrict__ cdf, uint32_t n, float index)
{
    const uint32_t i = (uint32_t)index;
    const float prev = (i == 0u) ? 0.0f : __ldg(&cdf[i - 1u]);
    return mul(sub(__ldg(&cdf[i]), prev), (float)n);
}

__device__ __forceinline__ bool env_constant(const PtEnv& E) { return E.width == 1u && E.height == 1u; }

// EmitViaSurfacePoint: radiance arriving along -d (d points away from the
// receiver, into the sky).
__device__ float3 env_emit(const PtEnv& E, float3 d)
{
    const float3 dy = normalize3(rows_apply(E.inv, d));
    const float2 uv = env_constant(E) ? make_float2(0.0f, 0.0f) : env_dir_to_uv(dy);
    return env_read(E, uv.x, uv.y);
}

// PdfSolidAngle(dir)
__device__ float env_pdf(const PtEnv& E, float3 d)
{
    const float3 dy = rows_apply(E.inv, d);
    const float2 uv = env_dir_to_uv(normalize3(dy));
    float pdf = 1.0f;
    if(!env_constant(E))
    {
        float ix = mul(uv.x, (float)E.width), iy = mul(uv.y, (float)E.height);
        ix = (ix < sub((float)E.width, 1.0f)) ? ix : sub((float)E.width, 1.0f);
        iy = (iy < sub((float)E.height, 1.0f)) ? iy : sub((float)E.height, 1.0f);
        const uint32_t row = (uint32_t)iy;
        const float marginal = pwc1_pdf_index(E.cdfY, E.height, iy);
        const float conditional = pwc1_pdf_index(E.cdfX + (size_t)row * E.width, E.width, ix);
        pdf = mul(conditional, marginal);
    }
    return env_sa_pdf_sin(pdf, sinf(acosf(fminf(fmaxf(dy.y, -1.0f), 1.0f))));
}

// SampleSolidAngle: world direction, solid-angle pdf.
__device__ float3 env_sample(const PtEnv& E, float xi0, float xi1, float& pdf)
{
    float2 uv;
    float uvPdf;
    if(env_constant(E)) { uv = make_float2(xi0, xi1); uvPdf = 1.0f; }
    else
    {
        float py, px;
        const float iy = pwc1_sample_index(E.cdfY, E.height, xi1, py);
        const uint32_t row = (uint32_t)iy;
        const float ix = pwc1_sample_index(E.cdfX + (size_t)row * E.width, E.width, xi0, px);
        uv = make_float2(mul(ix, __fdiv_rn(1.0f, (float)E.width)), mul(iy, __fdiv_rn(1.0f, (float)E.height)));
        uvPdf = mul(py, px);
    }
    const float theta = sub(mul(mul(uv.x, kPi), 2.0f), kPi);
    const float phi = mul(sub(1.0f, uv.y), kPi);
    const float sT = sinf(theta), cT = cosf(theta), sP = sinf(phi), cP = cosf(phi);
    pdf = env_sa_pdf_sin(uvPdf, sP);
    return rows_apply(E.m, make_float3(mul(sT, sP), cP, mul(cT, sP)));
}

// ---------------------------------------------------------------------------
// Spectral (SpectrumContext.hpp:36-152, SpectrumContext.cu:40-170): the host
// backend's linear texture reads (texel = uv * n - 0.5, modf with negative
// fractions made absolute, clamp), MRay's arithmetic order.
// ---------------------------------------------------------------------------
constexpr float kCieStart = 360.0f;

__device__ __forceinline__ void tex_axis(float uv, uint32_t n, int32_t& i0, int32_t& i1, float& frac)
{
    const float t = sub(mul(uv, (float)n), 0.5f);
    float b;
    float f = modff(t, &b);
    int32_t s = (int32_t)b;
    if(f < 0.0f) { s -= 1; f = fabsf(f); }
    const int32_t hi = (int32_t)n - 1;
    i0 = s < 0 ? 0 : (s > hi ? hi : s);
    i1 = (s + 1) < 0 ? 0 : ((s + 1) > hi ? hi : (s + 1));
    frac = f;
}
__device__ __forceinline__ float lerp_(float a, float b, float t) { return add(mul(a, sub(1.0f, t)), mul(b, t)); }

__device__ __forceinline__ float tex3d(const PtSpectral& S, uint32_t tex, float u, float v, float w)
{
    const uint32_t n = S.lutRes;
    const float* t = S.lut + (size_t)tex * n * n * n;
    int32_t a0, a1, b0, b1, c0, c1;
    float fx, fy, fz;
    tex_axis(u, n, a0, a1, fx);
    tex_axis(v, n, b0, b1, fy);
    tex_axis(w, n, c0, c1, fz);
    auto T = [&](int32_t x, int32_t y, int32_t z) { return __ldg(&t[((size_t)z * n + (size_t)y) * n + (size_t)x]); };
    const float p0 = lerp_(T(a0, b0, c0), T(a1, b0, c0), fx);
    const float p1 = lerp_(T(a0, b1, c0), T(a1, b1, c0), fx);
    const float p2 = lerp_(T(a0, b0, c1), T(a1, b0, c1), fx);
    const float p3 = lerp_(T(a0, b1, c1), T(a1, b1, c1), fx);
    return lerp_(lerp_(p0, p1, fy), lerp_(p2, p3, fy), fz);
}

__device__ __forceinline__ float inv_smoothstep(float y)
{
    return sub(0.5f, sinf(mul(asinf(sub(1.0f, mul(2.0f, y))), 1.0f / 3.0f)));
}

// SingleSampleSpectrumWavelength, HYPERBOLIC_PBRT (the default mode)
__device__ __forceinline__ void sample_waves(float xi0, float4& waves, float4& pdf)
{
    const float off[4] = { -0.5f, -0.25f, 0.0f, 0.25f };
    float w[4], p[4];
#pragma unroll
    for(int i = 0; i < 4; i++)
    {
        float x = add(xi0, off[i]);
        if(x < 0.0f) x = add(x, 1.0f);
        if(x >= 1.0f) x = sub(x, 1.0f);
        const float a = sub(0.85691062f, mul(1.82750197f, x));
        const float l = sub(538.0f, mul(138.888889f, atanhf(a)));
        float d = coshf(mul(0.0072f, sub(l, 538.0f)));
        d = mul(d, d);
        w[i] = l;
        p[i] = __fdiv_rn(0.0039398042f, d);
    }
    waves = make_float4(w[0], w[1], w[2], w[3]);
    pdf = make_float4(p[0], p[1], p[2], p[3]);
}

__device__ Chan convert_albedo(const PtSpectral& S, float r, float g, float b, const float4& waves)
{
    const float rgb[3] = { r, g, b };
    uint32_t maxI = 0;
    float mx = r;
    if(g > mx) { mx = g; maxI = 1; }
    if(b > mx) { mx = b; maxI = 2; }
    float x = 0.0f, y = 0.0f;
    if(mx > 1.0e-7f)
    {
        const float f = __fdiv_rn(1.0f, mx);
        x = mul(rgb[(maxI + 1) % 3], f);
        y = mul(rgb[(maxI + 2) % 3], f);
    }
    const float slice = mx < 0.0f ? 0.0f : (mx > 1.0f ? 1.0f : mx);
    const float z = inv_smoothstep(inv_smoothstep(slice));
    const float N = (float)S.lutRes;
    const float A = __fdiv_rn(sub(N, 1.0f), N), B = __fdiv_rn(0.5f, N);
    const float u = add(mul(x, A), B), v = add(mul(y, A), B), w = add(mul(z, A), B);
    const float c0 = tex3d(S, 3 * maxI + 0, u, v, w);
    const float c1 = tex3d(S, 3 * maxI + 1, u, v, w);
    const float c2 = tex3d(S, 3 * maxI + 2, u, v, w);
    const float wl[4] = { waves.x, waves.y, waves.z, waves.w };
    Chan out;
#pragma unroll
    for(int i = 0; i < 4; i++)
    {
        const float t = __fmaf_rn(c0, wl[i], c1);
        const float xx = __fmaf_rn(t, wl[i], c2);
        const float dr = __fdiv_rn(1.0f, __fsqrt_rn(__fmaf_rn(xx, xx, 1.0f)));
        out.v[i] = __fmaf_rn(mul(0.5f, xx), dr, 0.5f);
    }
    return out;
}

__device__ __forceinline__ float tex1d(const float* tab, uint32_t n, float coord, uint32_t ch, uint32_t c)
{
    const float uv = __fdiv_rn(coord, (float)n);
    int32_t i0, i1;
    float f;
    tex_axis(uv, n, i0, i1, f);
    return lerp_(__ldg(&tab[(size_t)i0 * ch + c]), __ldg(&tab[(size_t)i1 * ch + c]), f);
}

__device__ Chan convert_radiance(const PtSpectral& S, float r, float g, float b, const float4& waves)
{
    float mx = r;
    if(g > mx) mx = g;
    if(b > mx) mx = b;
    const float scale = mul(mx, 2.0f);
    float c[3] = { 0.0f, 0.0f, 0.0f };
    if(scale != 0.0f) { c[0] = __fdiv_rn(r, scale); c[1] = __fdiv_rn(g, scale); c[2] = __fdiv_rn(b, scale); }
    Chan out = convert_albedo(S, c[0], c[1], c[2], waves);
    const float wl[4] = { waves.x, waves.y, waves.z, waves.w };
#pragma unroll
    for(int i = 0; i < 4; i++)
        out.v[i] = mul(out.v[i], tex1d(S.illuminant, S.cieCount, add(wl[i], 0.5f - kCieStart), 1, 0));
#pragma unroll
    for(int i = 0; i < 4; i++) out.v[i] = mul(out.v[i], scale);
    return out;
}

// ConvertSpectraToRGBSingle (no dispersion)
__device__ float3 spectrum_to_rgb(const PtSpectral& S, const float4& value, const float4& waves, const float4& pdf)
{
    const float val[4] = { value.x, value.y, value.z, value.w };
    const float wl[4] = { waves.x, waves.y, waves.z, waves.w };
    const float pd[4] = { pdf.x, pdf.y, pdf.z, pdf.w };
    float xyz[3] = { 0.0f, 0.0f, 0.0f };
#pragma unroll
    for(int i = 0; i < 4; i++)
    {
        const float coord = add(wl[i], 0.5f - kCieStart);
        const float v = (pd[i] == 0.0f) ? 0.0f : __fdiv_rn(val[i], pd[i]);
#pragma unroll
        for(int k = 0; k < 3; k++) xyz[k] = add(xyz[k], mul(tex1d(S.observer, S.cieCount, coord, 3, k), v));
    }
#pragma unroll
    for(int k = 0; k < 3; k++) xyz[k] = mul(xyz[k], 0.25f);
    float rgb[3];
#pragma unroll
    for(int r = 0; r < 3; r++)
        rgb[r] = __fmaf_rn(S.xyzToRgb[3 * r + 2], xyz[2],
                           __fmaf_rn(S.xyzToRgb[3 * r + 1], xyz[1], mul(S.xyzToRgb[3 * r], xyz[0])));
    return make_float3(rgb[0], rgb[1], rgb[2]);
}

// The colour of an RGB triple on this path: itself, or its spectrum.
template<bool SPEC>
__device__ __forceinline__ Chan albedo_of(const PtSpectral& S, float r, float g, float b, const float4& waves)
{
    if(SPEC) return convert_albedo(S, r, g, b, waves);
    return chan(r, g, b, 0.0f);
}
template<bool SPEC>
__device__ __forceinline__ Chan radiance_of(const PtSpectral& S, float r, float g, float b, const float4& waves)
{
    if(SPEC) return convert_radiance(S, r, g, b, waves);
    return chan(r, g, b, 0.0f);
}

__device__ __forceinline__ uint32_t slot_pixel(const PtLaunch& L, uint32_t i) { return i % (L.width * L.height); }
__device__ __forceinline__ bool training_path(const PtCacheUse& C, uint32_t i, uint32_t sampleBase)
{
    return C.trainStride != 0u && (pcg_hash(i ^ pcg_hash(sampleBase + 0x5BD1E995u)) % C.trainStride) == 0u;
}
__device__ __forceinline__ uint32_t slot_sample(const PtLaunch& L, uint32_t i)
{
    return L.sampleBase + i / (L.width * L.height);
}

// Random number k of bounce b of slot i's path: the counter-based hash, or
// MRay's ZSobol group (sampler 1; sampler 2 with the scramble's bit reversal
// undone, which keeps the stratification) under this dimension plan: the film-filter
// offset (k 6, 7) = Next2D(0), the wavelengths (k 9) = Next(2); bounce b from
// dimension 3 + 7b: k 0..2 (lobe choice and direction) = Next3D(+0), light
// choice (k 3) = Next(+3), light point (k 4, 5) = Next2D(+4), Russian
// roulette (k 8) = Next(+6).
// Kept out of line so the default sampler's kernels keep their registers.
__device__ __noinline__ float rnd_zsobol(const PtLaunch& L, uint32_t i, uint32_t bounce, uint32_t k)
{
    uint32_t dim, size, comp;
    if(k == 6u || k == 7u) { dim = 0u; size = 2u; comp = k - 6u; }
    else if(k == 9u) { dim = 2u; size = 1u; comp = 0u; }
    else
    {
        const uint32_t b = 3u + 7u * bounce;
        if(k <= 2u) { dim = b; size = 3u; comp = k; }
        else if(k == 3u) { dim = b + 3u; size = 1u; comp = 0u; }
        else if(k <= 5u) { dim = b + 4u; size = 2u; comp = k - 4u; }
        else { dim = b + 6u; size = 1u; comp = 0u; }
    }
    const uint32_t pixel = slot_pixel(L, i);
    const ZsGen g = zs_make(pixel % L.width, pixel / L.width, __ldg(L.zsSeeds + pixel), slot_sample(L, i),
                            L.zsMaxSpp, L.zsResBits);
    const uint64_t* perm = reinterpret_cast<const uint64_t*>(L.zsTables + 3 * kZsWidth);
    return zs_to_float01(zs_number(g, L.zsTables, perm, dim, size, comp, L.sampler == 2u));
}

// MRay's independent group (sampler 3; RNGGroupIndependent, Random.cu:661-726):
// the pixel's PCG32 stream (PermutedCG32, Random.h:762-842), its state made
// by GenerateState from the pixel's mt19937 output, read at position
// ((sample * (maxDepth + 1) + bounce) * 16 + k).  The jump there composes the
// affine maps of 2^j LCG steps for the set bits of the position (Brown's
// arbitrary-stride method, as PermutedCG32::Advance does); `count`
// consecutive positions from k0 follow by single steps.
constexpr uint32_t kPcgMult = 747796405u, kPcgInc = 2891336453u;

__device__ __forceinline__ uint32_t pcg_permute(uint32_t s)
{
    const uint32_t x = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    return (x >> 22) ^ x;
}

__device__ __noinline__ float4 rnd_pcg32(const PtLaunch& L, uint32_t i, uint32_t bounce, uint32_t k0, uint32_t count)
{
    const uint32_t pixel = slot_pixel(L, i);
    uint32_t st = (kPcgInc + __ldg(L.zsSeeds + pixel)) * kPcgMult + kPcgInc;   // GenerateState
    uint32_t a = 1u, c = 0u, m = kPcgMult, inc = kPcgInc;
    for(uint32_t n = ((slot_sample(L, i) * (L.maxDepth + 1u) + bounce) << 4) | k0; n; n >>= 1)
    {
        if(n & 1u) { a *= m; c = c * m + inc; }
        inc = (m + 1u) * inc;
        m *= m;
    }
    st = a * st + c;
    float v[3] = { 0.0f, 0.0f, 0.0f };
    #pragma unroll
    for(uint32_t j = 0; j < 3u; j++)
    {
        if(j < count) v[j] = zs_to_float01(pcg_permute(st));
        st = st * kPcgMult + kPcgInc;
    }
    return make_float4(v[0], v[1], v[2], 0.0f);
}

__device__ __forceinline__ float rnd_s(const PtLaunch& L, uint32_t key, uint32_t i, uint32_t bounce, uint32_t k)
{
    if(L.sampler == 0u) return rnd(key, bounce, k);
    if(L.sampler == 3u) return rnd_pcg32(L, i, bounce, k, 1u).x;
    return rnd_zsobol(L, i, bounce, k);
}

// The bounce's numbers k 0..2 (one Next3D request) or k 4, 5 (one Next2D
// request) at once; each equals rnd_s of that k.
__device__ __noinline__ float4 rnd_zsobol_group(const PtLaunch& L, uint32_t i, uint32_t bounce, uint32_t k0)
{
    const uint32_t b = 3u + 7u * bounce;
    const uint32_t dim = (k0 == 0u) ? b : b + 4u, size = (k0 == 0u) ? 3u : 2u;
    const uint32_t pixel = slot_pixel(L, i);
    const ZsGen g = zs_make(pixel % L.width, pixel / L.width, __ldg(L.zsSeeds + pixel), slot_sample(L, i),
                            L.zsMaxSpp, L.zsResBits);
    const uint64_t* perm = reinterpret_cast<const uint64_t*>(L.zsTables + 3 * kZsWidth);
    uint32_t v[3] = { 0u, 0u, 0u };
    zs_numbers(g, L.zsTables, perm, dim, size, v, L.sampler == 2u);
    return make_float4(zs_to_float01(v[0]), zs_to_float01(v[1]), zs_to_float01(v[2]), 0.0f);
}

__device__ __forceinline__ float3 rnd_s3(const PtLaunch& L, uint32_t key, uint32_t i, uint32_t bounce)
{
    if(L.sampler == 0u) return make_float3(rnd(key, bounce, 0), rnd(key, bounce, 1), rnd(key, bounce, 2));
    const float4 r = (L.sampler == 3u) ? rnd_pcg32(L, i, bounce, 0u, 3u) : rnd_zsobol_group(L, i, bounce, 0u);
    return make_float3(r.x, r.y, r.z);
}

__device__ __forceinline__ float2 rnd_s45(const PtLaunch& L, uint32_t key, uint32_t i, uint32_t bounce)
{
    if(L.sampler == 0u) return make_float2(rnd(key, bounce, 4), rnd(key, bounce, 5));
    const float4 r = (L.sampler == 3u) ? rnd_pcg32(L, i, bounce, 4u, 2u) : rnd_zsobol_group(L, i, bounce, 4u);
    return make_float2(r.x, r.y);
}

// ---------------------------------------------------------------------------
// Camera rays: pinhole (CamerasDefault.hpp:94-140), Gaussian film filter
// sampled per axis by inverting its CDF (GaussianFilter::Sample,
// Filters.h:209-219; film weight Evaluate / pdf = 1 per sample); spectral
// paths also draw their 4 wavelengths here.
// ---------------------------------------------------------------------------
// Common::SampleGaussian with mu = 0 (DistributionFunctions.h:686-705):
// sqrt(2) sigma erfinv(2 xi - 1), clamped to 3.5 sigma where erfinv is
// infinite.  MRay's CUDA backend takes Math::InvErrFunc from erfinvf.
__device__ __forceinline__ float gaussian_offset(float xi, float sigma)
{
    const float e = erfinvf(sub(mul(2.0f, xi), 1.0f));
    float x = mul(mul(1.4142135623730950488f, sigma), e);
    if(isinf(e))
    {
        const float mm = mul(3.5f, sigma);
        x = fminf(fmaxf(x, -mm), mm);
    }
    return x;
}

__device__ __forceinline__ void warp_append(bool pred, uint32_t value, uint32_t* list, uint32_t* count)
{
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, pred);
    if(m == 0u) return;
    const uint32_t lane = threadIdx.x & 31u;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if((int)lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if(pred) list[base + __popc(m & ((1u << lane) - 1u))] = value;
}

// throughput * prevPdf / (prevPdf + lightPdf): the balance heuristic with the
// BxDF pdf cancelled (BalanceCancelled, DistributionFunctions.h:957).
template<int NC>
__device__ __forceinline__ Chan mis_weighted(Chan tp, float prevPdf, float lightPdf)
{
    const float misPdf = add(prevPdf, lightPdf);
#pragma unroll
    for(int k = 0; k < NC; k++) tp.v[k] = mul(tp.v[k], prevPdf);
    if(misPdf == 0.0f) return chan(0, 0, 0, 0);
    const float inv = __fdiv_rn(1.0f, misPdf);
#pragma unroll
    for(int k = 0; k < NC; k++) tp.v[k] = mul(tp.v[k], inv);
    return tp;
}

// Albedo texture read: bilinear, wrap addressed, with the host texture view's
// fraction rule; UNORM8 channels as in * (1 / 255) (NormConversion::FromUNorm).
__device__ __forceinline__ float3 texel_rgb(const PtTexture& t, size_t i)
{
    if(t.format == 0u)
    {
        const uchar4 c = __ldg(reinterpret_cast<const uchar4*>(t.texels) + i);
        const float d = 1.0f / 255.0f;
        return make_float3(add(0.0f, mul((float)c.x, d)), add(0.0f, mul((float)c.y, d)), add(0.0f, mul((float)c.z, d)));
    }
    const float4 c = __ldg(reinterpret_cast<const float4*>(t.texels) + i);
    return make_float3(c.x, c.y, c.z);
}

__device__ float3 tex_read(const PtTexture& t, float u, float v)
{
    const float tx = sub(mul(u, (float)t.width), 0.5f), ty = sub(mul(v, (float)t.height), 0.5f);
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    const int32_t x0 = wrap_index(sx, (int32_t)t.width), x1 = wrap_index(sx + 1, (int32_t)t.width);
    const int32_t y0 = wrap_index(sy, (int32_t)t.height), y1 = wrap_index(sy + 1, (int32_t)t.height);
    const float3 p00 = texel_rgb(t, (size_t)y0 * t.width + x0), p10 = texel_rgb(t, (size_t)y0 * t.width + x1);
    const float3 p01 = texel_rgb(t, (size_t)y1 * t.width + x0), p11 = texel_rgb(t, (size_t)y1 * t.width + x1);
    const float gx = sub(1.0f, fx), gy = sub(1.0f, fy);
    const float ax = add(mul(p00.x, gx), mul(p10.x, fx)), bxx = add(mul(p01.x, gx), mul(p11.x, fx));
    const float ay = add(mul(p00.y, gx), mul(p10.y, fx)), byy = add(mul(p01.y, gx), mul(p11.y, fx));
    const float az = add(mul(p00.z, gx), mul(p10.z, fx)), bzz = add(mul(p01.z, gx), mul(p11.z, fx));
    return make_float3(add(mul(ax, gy), mul(bxx, fy)), add(mul(ay, gy), mul(byy, fy)),
                       add(mul(az, gy), mul(bzz, fy)));
}

// The four texels a bilinear read at (u, v) blends and their weights
// (derivative of tex_read's value with respect to each texel).
__device__ __forceinline__ void tex_taps(const PtTexture& t, float u, float v, uint32_t idx[4], float w[4])
{
    const float tx = sub(mul(u, (float)t.width), 0.5f), ty = sub(mul(v, (float)t.height), 0.5f);
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    const int32_t x0 = wrap_index(sx, (int32_t)t.width), x1 = wrap_index(sx + 1, (int32_t)t.width);
    const int32_t y0 = wrap_index(sy, (int32_t)t.height), y1 = wrap_index(sy + 1, (int32_t)t.height);
    const float gx = sub(1.0f, fx), gy = sub(1.0f, fy);
    idx[0] = (uint32_t)y0 * t.width + (uint32_t)x0; w[0] = mul(gx, gy);
    idx[1] = (uint32_t)y0 * t.width + (uint32_t)x1; w[1] = mul(fx, gy);
    idx[2] = (uint32_t)y1 * t.width + (uint32_t)x0; w[2] = mul(gx, fy);
    idx[3] = (uint32_t)y1 * t.width + (uint32_t)x1; w[3] = mul(fx, fy);
}

// Texture coordinates at a hit (GenerateSurface, PrimitiveDefaultTriangle.hpp:
// 472-476: uv = uv0 a + uv1 b + uv2 c with a = hit[0], b = hit[1], c = 1 - a - b).
__device__ __forceinline__ float2 surface_uv(const PtSceneTables& T, uint32_t gprim, float2 mh)
{
    const float4 q0 = T.uvs[2 * (size_t)gprim], q1 = T.uvs[2 * (size_t)gprim + 1];
    const float a = mh.x, b = mh.y, c = sub(sub(1.0f, a), b);
    return make_float2(add(add(mul(q0.x, a), mul(q0.z, b)), mul(q1.x, c)),
                       add(add(mul(q0.y, a), mul(q0.w, b)), mul(q1.y, c)));
}

// ---------------------------------------------------------------------------
// Mip-mapped albedo reads and ray cones.
//   levels      Graphics::TextureMipSize / TextureMipPixelStart
//               (Source/Core/GraphicsFunctions.h:474-525)
//   LOD read    TextureViewCPU::operator()(uv, dpdx, dpdy) and (uv, mipLevel)
//               (Source/Device/CPU/TextureViewCPU.h:405-470), the gradients
//               taken in texels as a GPU's gradient read takes them
//   cones       RayCone::Advance / Project, RayConeSurface::ConeAfterScatter
//               (Source/Tracer/TracerTypes.h:44-66, 323-380); the hit's texture
//               gradients (Triangle::GenerateSurface, PrimitiveDefaultTriangle.hpp:
//               491-569); RefractMaterial::RefractRayCone (MaterialsDefault.hpp:
//               353-462)
// ---------------------------------------------------------------------------
constexpr float kConeEps = 1.0e-5f;          // MathConstants::Epsilon

__device__ __forceinline__ uint32_t mip_dim(uint32_t r, uint32_t m) { return max(r >> m, 1u); }

__device__ __forceinline__ float3 texel_rgb_at(uint32_t format, const void* base, size_t i)
{
    if(format == 0u)
    {
        const uchar4 c = __ldg(reinterpret_cast<const uchar4*>(base) + i);
        const float d = 1.0f / 255.0f;
        return make_float3(add(0.0f, mul((float)c.x, d)), add(0.0f, mul((float)c.y, d)), add(0.0f, mul((float)c.z, d)));
    }
    const float4 c = __ldg(reinterpret_cast<const float4*>(base) + i);
    return make_float3(c.x, c.y, c.z);
}

// Bilinear read of level m (tex_read's arithmetic at the level's size).
__device__ float3 tex_read_level(const PtTexture& t, uint32_t m, float u, float v)
{
    const uint32_t w = mip_dim(t.width, m), h = mip_dim(t.height, m);
    const void* base = t.texels;
    if(m > 0u)
    {
        size_t start = 0;
        for(uint32_t k = 1; k < m; k++) start += (size_t)mip_dim(t.width, k) * mip_dim(t.height, k);
        base = static_cast<const char*>(t.mips) + start * (t.format == 0u ? 4u : 16u);
    }
    const float tx = sub(mul(u, (float)w), 0.5f), ty = sub(mul(v, (float)h), 0.5f);
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    const int32_t x0 = wrap_index(sx, (int32_t)w), x1 = wrap_index(sx + 1, (int32_t)w);
    const int32_t y0 = wrap_index(sy, (int32_t)h), y1 = wrap_index(sy + 1, (int32_t)h);
    const float3 p00 = texel_rgb_at(t.format, base, (size_t)y0 * w + x0);
    const float3 p10 = texel_rgb_at(t.format, base, (size_t)y0 * w + x1);
    const float3 p01 = texel_rgb_at(t.format, base, (size_t)y1 * w + x0);
    const float3 p11 = texel_rgb_at(t.format, base, (size_t)y1 * w + x1);
    const float gx = sub(1.0f, fx), gy = sub(1.0f, fy);
    const float ax = add(mul(p00.x, gx), mul(p10.x, fx)), bxx = add(mul(p01.x, gx), mul(p11.x, fx));
    const float ay = add(mul(p00.y, gx), mul(p10.y, fx)), byy = add(mul(p01.y, gx), mul(p11.y, fx));
    const float az = add(mul(p00.z, gx), mul(p10.z, fx)), bzz = add(mul(p01.z, gx), mul(p11.z, fx));
    return make_float3(add(mul(ax, gy), mul(bxx, fy)), add(mul(ay, gy), mul(byy, fy)),
                       add(mul(az, gy), mul(bzz, fy)));
}

// Level from the uv gradients (in texels), clamped to the chain, and the
// linear blend of the two nearest levels (Math::Lerp).
__device__ float3 tex_read_grad(const PtTexture& t, float u, float v, float2 dx, float2 dy)
{
    const float sx = (float)t.width, sy = (float)t.height;
    const float gxx = mul(dx.x, sx), gxy = mul(dx.y, sy), gyx = mul(dy.x, sx), gyy = mul(dy.y, sy);
    const float maxLenSqr = fmaxf(len2_2(gxx, gxy), len2_2(gyx, gyy));
    float level = mul(0.5f, log2f(maxLenSqr));
    level = fminf(fmaxf(0.0f, level), (float)(t.mipCount - 1u));
    float m0f;
    const float frac = modff(level, &m0f);
    const uint32_t m0 = (uint32_t)m0f, m1 = min(m0 + 1u, t.mipCount - 1u);
    const float3 p0 = tex_read_level(t, m0, u, v);
    if(m0 == m1) return p0;
    const float3 p1 = tex_read_level(t, m1, u, v);
    const float g = sub(1.0f, frac);
    return make_float3(add(mul(p0.x, g), mul(p1.x, frac)), add(mul(p0.y, g), mul(p1.y, frac)),
                       add(mul(p0.z, g), mul(p1.z, frac)));
}

struct Cone
{
    float aperture, width;
};

// RayCone::Advance: the width after distance t (RT Gems I, chapter 20).
__device__ __forceinline__ Cone cone_advance(Cone c, float t)
{
    Cone r;
    r.aperture = c.aperture;
    r.width = fminf(fmaxf(kConeEps, add(c.width, mul(c.aperture, t))), 1.0e6f);
    return r;
}

// RayCone::Project: the cone's footprint axes on the plane with normal f.
__device__ void cone_project(Cone c, float3 f, float3 d, float3& a1, float3& a2)
{
    const float fDotD = dot3(f, d);
    if(fabsf(add(fDotD, 1.0f)) < kConeEps)
        d = make_float3(add(d.x, kConeEps), add(d.y, kConeEps), add(d.z, kConeEps));
    const float3 h1 = make_float3(sub(d.x, mul(fDotD, f.x)), sub(d.y, mul(fDotD, f.y)), sub(d.z, mul(fDotD, f.z)));
    const float3 h2 = cross3(f, h1);
    const float r = mul(c.width, 0.5f);
    const float3 h[2] = { h1, h2 };
    float3 out[2];
#pragma unroll
    for(int k = 0; k < 2; k++)
    {
        const float dh = dot3(d, h[k]);
        const float3 q = make_float3(sub(h[k].x, mul(dh, d.x)), sub(h[k].y, mul(dh, d.y)), sub(h[k].z, mul(dh, d.z)));
        const float denom = fmaxf(kConeEps, __fsqrt_rn(dot3(q, q)));
        const float sc = __fdiv_rn(r, denom);
        out[k] = make_float3(mul(sc, h[k].x), mul(sc, h[k].y), mul(sc, h[k].z));
    }
    a1 = out[0];
    a2 = out[1];
}

// uv gradients of a hit along the cone's footprint axes (GenerateSurface,
// JCGT 2021 Listing 1): P0 and edges E0 = P1 - P0, E1 = P2 - P0 of the
// triangle in world space, f its normal towards the ray.
__device__ void tex_gradients(float3 pos, float3 P0, float3 E0, float3 E1, float3 f, float2 uv0, float2 uv1,
                              float2 uv2, float2 uv, float3 a1, float3 a2, float2& dpdx, float2& dpdy)
{
    const float areaRecip = __fdiv_rn(1.0f, dot3(f, cross3(E0, E1)));
    const float3 off[2] = { a1, a2 };
    float2 out[2];
#pragma unroll
    for(int k = 0; k < 2; k++)
    {
        const float3 eP = make_float3(add(sub(pos.x, P0.x), off[k].x), add(sub(pos.y, P0.y), off[k].y),
                                      add(sub(pos.z, P0.z), off[k].z));
        const float3 c1 = cross3(eP, E1), c2 = cross3(E0, eP);
        const float a = dot3(f, make_float3(mul(c1.x, areaRecip), mul(c1.y, areaRecip), mul(c1.z, areaRecip)));
        const float b = dot3(f, make_float3(mul(c2.x, areaRecip), mul(c2.y, areaRecip), mul(c2.z, areaRecip)));
        const float c = sub(sub(1.0f, a), b);
        const float uo = add(add(mul(uv0.x, c), mul(uv1.x, a)), mul(uv2.x, b));
        const float vo = add(add(mul(uv0.y, c), mul(uv1.y, a)), mul(uv2.y, b));
        out[k] = make_float2(sub(uo, uv.x), sub(vo, uv.y));
    }
    dpdx = out[0];
    dpdy = out[1];
}

__device__ __forceinline__ float dot2(float2 a, float2 b) { return __fmaf_rn(a.y, b.y, __fmaf_rn(a.x, b.x, 0.0f)); }

// Graphics::Refract in the plane z = 0 (RefractRayCone's Refract2D): the
// refracted direction, or on total internal reflection v's component along
// the boundary, normalised.
__device__ float2 refract2d(float2 v, float2 n, float fromEta, float toEta)
{
    const float etaRatio = __fdiv_rn(fromEta, toEta);
    // Vector3(n, 0) . Vector3(-v, 0) with the fma chain over three components
    const float cosIn = __fmaf_rn(0.0f, 0.0f, __fmaf_rn(n.y, -v.y, __fmaf_rn(n.x, -v.x, 0.0f)));
    const float sinInSqr = fmaxf(0.0f, sub(1.0f, mul(cosIn, cosIn)));
    const float sinOutSqr = mul(mul(etaRatio, etaRatio), sinInSqr);
    const float cosOut = sqrt_max(sub(1.0f, sinOutSqr));
    if(sinOutSqr >= 1.0f)
    {
        const float nv = dot2(n, v);
        const float2 q = make_float2(sub(v.x, mul(n.x, nv)), sub(v.y, mul(n.y, nv)));
        const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot2(q, q)));
        return make_float2(mul(q.x, inv), mul(q.y, inv));
    }
    const float k = sub(mul(etaRatio, cosIn), cosOut);
    return make_float2(add(mul(etaRatio, v.x), mul(k, n.x)), add(mul(etaRatio, v.y), mul(k, n.y)));
}

// RefractMaterial::RefractRayCone (RT Gems II, chapter 10): the cone behind a
// smooth dielectric, from the cone in front (aperture, width), the surface's
// curvature term betaN, wo (towards the viewer) and the normal n facing it;
// false (no change) on total internal reflection of wo.
__device__ bool refract_cone(Cone front, float betaN, float3 wo, float3 n, float fromEta, float toEta, Cone& back)
{
    const float etaRatio = __fdiv_rn(fromEta, toEta);
    const float cosIn = dot3(n, wo);
    const float sinInSqr = fmaxf(0.0f, sub(1.0f, mul(cosIn, cosIn)));
    const float sinOutSqr = mul(mul(etaRatio, etaRatio), sinInSqr);
    if(sinOutSqr >= 1.0f) return false;
    const float3 d3 = make_float3(-wo.x, -wo.y, -wo.z);
    // GSOrthonormalize(d3, n) = Normalize(d3 - n Dot(d3, n))
    const float dn = dot3(d3, n);
    const float3 x = normalize3(make_float3(sub(d3.x, mul(n.x, dn)), sub(d3.y, mul(n.y, dn)), sub(d3.z, mul(n.z, dn))));
    const float2 d = make_float2(dot3(x, d3), dot3(n, d3));
    const float wSign = (front.width > 0.0f) ? 1.0f : 0.0f;
    float s, c;
    sincosf(mul(mul(wSign, front.aperture), 0.5f), &s, &c);
    const float2 du = make_float2(sub(mul(d.x, c), mul(d.y, s)), add(mul(d.x, s), mul(d.y, c)));
    const float2 dl = make_float2(add(mul(d.x, c), mul(d.y, s)), add(mul(d.x, -s), mul(d.y, c)));
    float2 orthoD = make_float2(mul(mul(-d.y, front.width), 0.5f), mul(mul(d.x, front.width), 0.5f));
    const float uHitX = add(orthoD.x, mul(du.x, __fdiv_rn(-orthoD.y, du.y)));
    const float lHitX = add(-orthoD.x, mul(dl.x, __fdiv_rn(orthoD.y, dl.y)));
    const float nSign = (uHitX > lHitX) ? 1.0f : -1.0f;
    const float dTheta = mul(mul(-betaN, nSign), 0.5f);
    float ns, nc;
    sincosf(dTheta, &ns, &nc);
    // Rotate2D_UL((0, 1), dTheta)
    const float2 nu = make_float2(sub(mul(0.0f, nc), mul(1.0f, ns)), add(mul(0.0f, ns), mul(1.0f, nc)));
    const float2 nl = make_float2(add(mul(0.0f, nc), mul(1.0f, ns)), add(mul(0.0f, -ns), mul(1.0f, nc)));
    const float2 tu = refract2d(du, nu, fromEta, toEta);
    const float2 tl = refract2d(dl, nl, fromEta, toEta);
    orthoD = make_float2(-d.y, d.x);
    float wl = mul(-uHitX, tu.y);
    wl = __fdiv_rn(wl, dot2(orthoD, make_float2(-tu.y, tu.x)));
    float wu = mul(lHitX, tl.y);
    wu = __fdiv_rn(wu, dot2(orthoD, make_float2(-tl.y, tl.x)));
    const float sgn = copysignf(1.0f, sub(mul(tu.x, tl.y), mul(tu.y, tl.x)));
    const float cosTheta = fminf(fmaxf(-1.0f, dot2(tu, tl)), 1.0f);
    float ap = mul(acosf(cosTheta), sgn);
    ap = fmaxf(ap, kConeEps);
    back.aperture = add(ap, betaN);
    back.width = add(wu, wl);
    return true;
}

// Albedo at a hit: constant, or the texture at the hit's uv.
__device__ __forceinline__ float3 surface_albedo(const PtSceneTables& T, const PtSurface& sf, uint32_t gprim, float2 mh)
{
    if(sf.tex.x == 0u || T.uvs == nullptr || gprim >= T.nTris) return make_float3(sf.albedo.x, sf.albedo.y, sf.albedo.z);
    const float2 uv = surface_uv(T, gprim, mh);
    return tex_read(T.textures[sf.tex.x - 1u], uv.x, uv.y);
}

// The same with a mip-mapped texture read at the level the path's cone
// (advanced to the hit) gives: the cone's footprint on the triangle (f: its
// normal facing the ray, d: the ray's direction) and the uv gradients along
// its axes.  The triangle's corner and edges go to world space with the
// instance transform (edges by its linear part).
__device__ __forceinline__ float3 tex_lod(const PtSceneTables& T, const PtSurface& sf, uint32_t texIdx, uint32_t gprim,
                                       float2 uv, float3 pos, float3 f, float3 d, Cone cone)
{
    const PtTexture tx = T.textures[texIdx - 1u];
    const float4 v0 = T.tris[3 * (size_t)gprim], e0 = T.tris[3 * (size_t)gprim + 1], e1 = T.tris[3 * (size_t)gprim + 2];
    float3 P0, E0, E1;
    P0.x = add(add(add(mul(sf.m[0].x, v0.x), mul(sf.m[0].y, v0.y)), mul(sf.m[0].z, v0.z)), sf.m[0].w);
    P0.y = add(add(add(mul(sf.m[1].x, v0.x), mul(sf.m[1].y, v0.y)), mul(sf.m[1].z, v0.z)), sf.m[1].w);
    P0.z = add(add(add(mul(sf.m[2].x, v0.x), mul(sf.m[2].y, v0.y)), mul(sf.m[2].z, v0.z)), sf.m[2].w);
    E0.x = add(add(mul(sf.m[0].x, e0.x), mul(sf.m[0].y, e0.y)), mul(sf.m[0].z, e0.z));
    E0.y = add(add(mul(sf.m[1].x, e0.x), mul(sf.m[1].y, e0.y)), mul(sf.m[1].z, e0.z));
    E0.z = add(add(mul(sf.m[2].x, e0.x), mul(sf.m[2].y, e0.y)), mul(sf.m[2].z, e0.z));
    E1.x = add(add(mul(sf.m[0].x, e1.x), mul(sf.m[0].y, e1.y)), mul(sf.m[0].z, e1.z));
    E1.y = add(add(mul(sf.m[1].x, e1.x), mul(sf.m[1].y, e1.y)), mul(sf.m[1].z, e1.z));
    E1.z = add(add(mul(sf.m[2].x, e1.x), mul(sf.m[2].y, e1.y)), mul(sf.m[2].z, e1.z));
    float3 a1, a2;
    cone_project(cone, f, normalize3(d), a1, a2);
    const float4 q0 = T.uvs[2 * (size_t)gprim], q1 = T.uvs[2 * (size_t)gprim + 1];
    float2 dpdx, dpdy;
    tex_gradients(pos, P0, E0, E1, f, make_float2(q0.x, q0.y), make_float2(q0.z, q0.w), make_float2(q1.x, q1.y), uv, a1,
                  a2, dpdx, dpdy);
    return tex_read_grad(tx, uv.x, uv.y, dpdx, dpdy);
}

// A texture (index + 1) at the hit's uv: level 0, or the cone's level of a
// mip-mapped one; dflt without a texture or uvs.
__device__ __forceinline__ float3 surface_tex_cone(const PtSceneTables& T, const PtSurface& sf, uint32_t texIdx,
                                                   uint32_t gprim, float2 mh, float3 pos, float3 f, float3 d, Cone cone,
                                                   float3 dflt)
{
    if(texIdx == 0u || T.uvs == nullptr || gprim >= T.nTris) return dflt;
    const float2 uv = surface_uv(T, gprim, mh);
    const PtTexture& tx = T.textures[texIdx - 1u];
    if(tx.mipCount <= 1u) return tex_read(tx, uv.x, uv.y);
    return tex_lod(T, sf, texIdx, gprim, uv, pos, f, d, cone);
}

__device__ __forceinline__ float3 surface_albedo_cone(const PtSceneTables& T, const PtSurface& sf, uint32_t gprim,
                                                      float2 mh, float3 pos, float3 f, float3 d, Cone cone)
{
    return surface_tex_cone(T, sf, sf.tex.x, gprim, mh, pos, f, d, cone,
                            make_float3(sf.albedo.x, sf.albedo.y, sf.albedo.z));
}

// Unreal's texturable roughness, metallic and specular (UnrealMaterial's
// constructor reads each ParamVaryingData<2, Float> at the surface's uv and
// cone gradients, MaterialsDefault.hpp:521-533): the first channel of the
// texture, read like the albedo, replaces the constant in the hit's copy of
// the surface.
__device__ __forceinline__ void unreal_params_cone(const PtSceneTables& T, PtSurface& sf, uint32_t gprim, float2 mh,
                                                   float3 pos, float3 f, float3 d, Cone cone)
{
    if(sf.info.w != kMatUnreal || (sf.tex.y | sf.tex.z | sf.tex.w) == 0u) return;
    if(sf.tex.y) sf.albedo.w = surface_tex_cone(T, sf, sf.tex.y, gprim, mh, pos, f, d, cone, make_float3(0, 0, 0)).x;
    if(sf.tex.z) sf.mat.x = surface_tex_cone(T, sf, sf.tex.z, gprim, mh, pos, f, d, cone, make_float3(0, 0, 0)).x;
    if(sf.tex.w) sf.mat.y = surface_tex_cone(T, sf, sf.tex.w, gprim, mh, pos, f, d, cone, make_float3(0, 0, 0)).x;
}

// The cone a scattered ray leaves with (RefractRayCone, then
// ConeAfterScatter; the surfaces here have no vertex normals, so the
// curvature term betaN is 0): the refracted cone for a dielectric's
// transmission, the incoming one otherwise.
__device__ __forceinline__ Cone cone_after_scatter(const PtSurface& sf, uint32_t mt, bool backSide, Cone cone, float3 wo,
                                                   float3 n, float3 wi)
{
    Cone back = cone;
    if(mt == kMatRefract && dot3(wi, n) <= 0.0f)
    {
        float fromEta = sf.mat.z, toEta = sf.mat.w;
        if(backSide) { const float t = fromEta; fromEta = toEta; toEta = t; }
        Cone r;
        if(refract_cone(cone, 0.0f, wo, n, fromEta, toEta, r)) back = r;
    }
    Cone out;
    if(dot3(wi, n) > 0.0f) { out.aperture = add(cone.aperture, mul(2.0f, 0.0f)); out.width = cone.width; }
    else { out.aperture = sub(back.aperture, 0.0f); out.width = back.width; }
    return out;
}

// Adds an emission-gradient contribution (RGB) to the light instance's FP64
// sums: the active lanes of the warp that share the instance sum their values
// first, and one lane of each group issues the atomics, so a light seen by
// every path costs a few atomics per warp rather than one per lane.  Every
// active lane runs the same number of shuffles (one per active lane).
__device__ void add_emission_grad(double* acc, uint32_t inst, float gx, float gy, float gz)
{
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, inst);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for(unsigned m = act; m != 0u; m &= m - 1u)
    {
        const int src = __ffs(m) - 1;
        const float vx = __shfl_sync(act, gx, src);
        const float vy = __shfl_sync(act, gy, src);
        const float vz = __shfl_sync(act, gz, src);
        if((grp >> src) & 1u) { sx += (double)vx; sy += (double)vy; sz += (double)vz; }
    }
    if((int)(threadIdx.x & 31u) == __ffs(grp) - 1)
    {
        double* a = acc + 4 * (size_t)inst;
        atomicAdd(a + 0, sx);
        atomicAdd(a + 1, sy);
        atomicAdd(a + 2, sz);
    }
}

// A thread's run of emission-gradient terms for one light instance: terms of
// the same instance are summed in registers and reach the FP64 sums (through
// the warp-aggregated add) only when the instance changes and once at the
// end of the thread's work, so a scene with few lights costs few atomics.
constexpr uint32_t kNoEmission = 0xFFFFFFFFu;
struct EmisRun
{
    uint32_t inst;
    float    x, y, z;
};

__device__ __forceinline__ void emis_flush(EmisRun& r, double* acc)
{
    if(r.inst != kNoEmission) add_emission_grad(acc, r.inst, r.x, r.y, r.z);
    r.inst = kNoEmission;
}

__device__ __forceinline__ void emis_push(EmisRun& r, double* acc, uint32_t inst, float gx, float gy, float gz)
{
    if(inst != r.inst)
    {
        emis_flush(r, acc);
        r.inst = inst;
        r.x = 0.0f; r.y = 0.0f; r.z = 0.0f;
    }
    r.x = add(r.x, gx); r.y = add(r.y, gy); r.z = add(r.z, gz);
}

__global__ void k_add_emission_grad(const double* __restrict__ acc, float* __restrict__ out, uint32_t n)
{
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = add(out[i], (float)acc[i]);
}

// Path-replay adjoint at a Lambert vertex whose albedo is the parameter
// texture: every contribution after this vertex is linear in its albedo, so
// d(path radiance)/d(albedo) = (primal radiance - radiance before the vertex)
// / albedo, per channel; scattered to the four texels of the read.
__device__ void adjoint_vertex(const PtLaunch& L, const PtSceneTables& T, const PtSurface& sf, uint32_t slot,
                               uint32_t gprim, float2 mh, float3 alb, const Chan& radBefore)
{
    const float4 tot = L.adj.radTotal[slot];
    const float4 d = L.adj.delta[slot_pixel(L, slot)];
    const float s = L.adj.invSpp;
    const float dd[3] = { d.x, d.y, d.z }, tt[3] = { tot.x, tot.y, tot.z }, aa[3] = { alb.x, alb.y, alb.z };
    float g[3];
#pragma unroll
    for(int k = 0; k < 3; k++)
        g[k] = (aa[k] > 0.0f) ? mul(mul(dd[k], s), __fdiv_rn(sub(tt[k], radBefore.v[k]), aa[k])) : 0.0f;
    const float2 uv = surface_uv(T, gprim, mh);
    uint32_t idx[4];
    float w[4];
    tex_taps(T.textures[sf.tex.x - 1u], uv.x, uv.y, idx, w);
#pragma unroll
    for(int j = 0; j < 4; j++)
#pragma unroll
        for(int k = 0; k < 3; k++)
            atomicAdd(&L.adj.grad[4 * (size_t)idx[j] + k], mul(g[k], w[j]));
}

// Cache inputs of a surface vertex: position, roughness | outgoing direction |
// normal | albedo.
__device__ __forceinline__ void cache_inputs(float4* dst, float3 pos, float rough, float3 wo, float3 nrm, float3 alb)
{
    dst[0] = make_float4(pos.x, pos.y, pos.z, rough);
    dst[1] = make_float4(wo.x, wo.y, wo.z, 0.0f);
    dst[2] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
    dst[3] = make_float4(alb.x, alb.y, alb.z, 0.0f);
}

// A path's hit on area light lt: PdfSolidAngle(hit, ray.pos, ray.dir) times
// the light choice probability invN.
__device__ __forceinline__ float area_light_pdf(const PtLight& lt, float2 mh, float3 org, float3 dir, float invN)
{
    // MRay's hit (a, b) = MetaHit of the world-space light triangle
    // (Triangle::SurfaceFromHit, PrimitiveDefaultTriangle.hpp:320-350)
    float ndl = dot3(f3(lt.n), make_float3(-dir.x, -dir.y, -dir.z));
    ndl = (lt.n.w != 0.0f) ? fabsf(ndl) : fmaxf(0.0f, ndl);
    const float a = mh.x, b = mh.y, c = sub(sub(1.0f, a), b);
    const bool inside = a >= 0.0f && a <= 1.0f && b >= 0.0f && b <= 1.0f &&
                        c >= 0.0f && c <= 1.0f;
    const float3 lpos = make_float3(add(add(mul(lt.p0.x, a), mul(lt.p1.x, b)), mul(lt.p2.x, c)),
                                    add(add(mul(lt.p0.y, a), mul(lt.p1.y, b)), mul(lt.p2.y, c)),
                                    add(add(mul(lt.p0.z, a), mul(lt.p1.z, b)), mul(lt.p2.z, c)));
    const float3 dd = make_float3(sub(org.x, lpos.x), sub(org.y, lpos.y), sub(org.z, lpos.z));
    float lpdf = (ndl == 0.0f) ? 0.0f : __fdiv_rn(__fdiv_rn(1.0f, lt.p0.w), ndl);
    lpdf = inside ? mul(lpdf, dot3(dd, dd)) : 0.0f;
    lpdf = mul(lpdf, invN);
    return lpdf;
}

// MRay's Evaluate and Pdf of the non-specular materials (Lambert, Unreal)
// for a local direction Ls (MaterialsDefault.hpp).
template<int NC>
__device__ __forceinline__ Chan eval_material(const PtSurface& sf, uint32_t mt, const Chan& alb, float3 V, float3 Ls,
                                              float& bpdf)
{
    Chan refl = chan(0, 0, 0, 0);
    if(mt == kMatUnreal) refl = unreal_eval<NC>(sf, alb, V, Ls, bpdf);
    else
    {
        // LambertMaterial::Evaluate: nDotL * albedo * InvPi
        const float ndl = fmaxf(Ls.z, 0.0f);
#pragma unroll
        for(int k = 0; k < NC; k++) refl.v[k] = mul(mul(ndl, alb.v[k]), kInvPi);
        bpdf = mul(Ls.z, kInvPi);
        bpdf = (bpdf <= 1.0e-5f) ? 0.0f : bpdf;
    }
    return refl;
}

// MRay's SampleBxDF of the four materials in the shading frame (V = wO
// local): the local direction, reflectance, pdf, whether it passed through
// (refraction) and the nudged origin for it (MaterialsDefault.hpp).
template<int NC>
__device__ __forceinline__ void sample_material(const PtLaunch& L, uint32_t key, uint32_t i, uint32_t depth,
                                                const PtSurface& sf, uint32_t mt, const Chan& alb, float3 V,
                                                bool backSide, float3 pos, float3 nrm, float3& Ll, Chan& refl,
                                                float& bpdf, bool& passed, float3& pre)
{
    refl = chan(0, 0, 0, 0);
    passed = false;
    pre = pos;
    if(mt == kMatReflect)
    {
        Ll = normalize3(make_float3(-V.x, -V.y, sub(mul(2.0f, V.z), V.z)));
        bpdf = 1.0f;
        refl = chan(1.0f, 1.0f, 1.0f, 1.0f);
    }
    else if(mt == kMatRefract)
    {
        float fromEta = sf.mat.z, toEta = sf.mat.w;
        if(backSide) { const float t = fromEta; fromEta = toEta; toEta = t; }
        const float f = fresnel_dielectric(fabsf(V.z), fromEta, toEta);
        const bool doRefl = rnd_s(L, key, i, depth, 0) < f;
        if(doRefl) Ll = make_float3(-V.x, -V.y, sub(mul(2.0f, V.z), V.z));
        else
        {
            const float eta = __fdiv_rn(fromEta, toEta);
            const float cosIn = V.z;
            const float sin2 = fmaxf(0.0f, sub(1.0f, mul(cosIn, cosIn)));
            const float sinOut2 = mul(mul(eta, eta), sin2);
            const float cosOut = sqrt_max(sub(1.0f, sinOut2));
            Ll = make_float3(mul(eta, -V.x), mul(eta, -V.y),
                             add(mul(eta, -V.z), sub(mul(eta, cosIn), cosOut)));
        }
        bpdf = doRefl ? f : sub(1.0f, f);
        refl = chan(bpdf, bpdf, bpdf, bpdf);
        passed = !doRefl;
        pre = nudge(pos, nrm);
    }
    else if(mt == kMatUnreal)
    {
        const float rough = sf.albedo.w;
        const float alpha = mul(rough, rough);
        const float ratio = unreal_ratio(sf, avg_albedo<NC>(alb));
        const float3 u3 = rnd_s3(L, key, i, depth);
        const float sXi = u3.x, x0 = u3.y, x1 = u3.z;
        float3 H;
        float pd, ps;
        if(sXi < ratio)
        {
            const float ang = mul(mul(2.0f, kPi), x1), sr = __fsqrt_rn(x0);
            Ll.x = mul(sr, cosf(ang)); Ll.y = mul(sr, sinf(ang));
            Ll.z = sqrt_max(sub(1.0f, len2_2(Ll.x, Ll.y)));   // SampleCosDirection
            pd = mul(Ll.z, kInvPi);
            H = normalize3(make_float3(add(Ll.x, V.x), add(Ll.y, V.y), add(Ll.z, V.z)));
            const float vdh = fmaxf(0.0f, dot3(V, H));
            ps = vndf_pdf(V, H, alpha);
            ps = (vdh == 0.0f) ? 0.0f : __fdiv_rn(ps, mul(4.0f, vdh));
        }
        else
        {
            H = vndf_sample(V, alpha, x0, x1);
            const float dv = mul(2.0f, dot3(V, H));
            Ll = make_float3(sub(mul(dv, H.x), V.x), sub(mul(dv, H.y), V.y), sub(mul(dv, H.z), V.z));
            const float vdh = fmaxf(0.0f, dot3(V, H));
            ps = vndf_pdf(V, H, alpha);
            ps = (vdh == 0.0f) ? 0.0f : __fdiv_rn(ps, mul(4.0f, vdh));
            pd = mul(Ll.z, kInvPi);
            pd = (pd <= 1.0e-5f) ? 0.0f : pd;
        }
        const float vdh = fmaxf(0.0f, dot3(V, H));
        const float ldh = fmaxf(0.0f, dot3(Ll, H));
        const float ndh = fmaxf(0.0f, H.z);
        const float ndv = fmaxf(0.0f, V.z);
        const float D = d_ggx(ndh, alpha);
        float G = g_correlated(V, Ll, alpha);
        G = (ldh == 0.0f) ? 0.0f : G;
        G = (vdh == 0.0f) ? 0.0f : G;
        const bool dBad = isinf(D) || isnan(D);
        const float gs = dBad ? g_single(V, alpha) : 1.0f;
        if(dBad) ps = 1.0f;
        const float ndl = fmaxf(0.0f, Ll.z);
        const float corr = burley(ndl, ndv, ldh, rough);
#pragma unroll
        for(int k = 0; k < NC; k++)
        {
            const float F = schlick1(vdh, f0_of(sf, alb.v[k]));
            float spec = (ndv == 0.0f) ? 0.0f : __fdiv_rn(mul(mul(mul(D, F), G), 0.25f), ndv);
            if(dBad) spec = __fdiv_rn(mul(G, F), gs);
            refl.v[k] = add(mul(mul(mul(ndl, mul(sub(1.0f, sf.mat.x), alb.v[k])), kInvPi), corr), spec);
        }
        bpdf = add(mul(pd, ratio), mul(ps, sub(1.0f, ratio)));
    }
    else
    {
        const float3 u3 = rnd_s3(L, key, i, depth);
        const float xi0 = u3.x, xi1 = u3.y;
        const float ang = mul(mul(2.0f, kPi), xi1), sr = __fsqrt_rn(xi0);
        Ll.x = mul(sr, cosf(ang)); Ll.y = mul(sr, sinf(ang));
        Ll.z = sqrt_max(sub(1.0f, len2_2(Ll.x, Ll.y)));   // SampleCosDirection
        bpdf = mul(Ll.z, kInvPi);
        // reflectance = albedo * nDotL * InvPi
        const float ndl = fmaxf(Ll.z, 0.0f);
#pragma unroll
        for(int k = 0; k < NC; k++) refl.v[k] = mul(mul(alb.v[k], ndl), kInvPi);
    }
}

// NEE light choice and sample (DirectLightSamplerUniform::SampleLight,
// LightSampler.hpp:33-76; LightPrim / Skysphere SampleSolidAngle,
// LightsDefault.hpp): the light index, the point on it, its emission
// towards pos and the solid-angle pdf times the choice probability.
template<bool SPEC, int NC>
__device__ __forceinline__ void nee_light(const PtLaunch& L, const PtLight* __restrict__ lights, uint32_t key,
                                          uint32_t i, uint32_t depth, uint32_t nAll, float invN, float3 pos,
                                          const float4& waves, uint32_t& li, float3& lp, Chan& emis,
                                          float& lightPdf)
{
    const float dXi = rnd_s(L, key, i, depth, 3);
    li = (uint32_t)mul(dXi, (float)nAll);
    li = min(li, nAll - 1u);
    emis = chan(0, 0, 0, 0);
    if(li == L.nLights)
    {
        // skysphere: a point sceneDiameter away along the sampled direction
        float spdf;
        const float2 u45 = rnd_s45(L, key, i, depth);
        const float3 wd = env_sample(L.env, u45.x, u45.y, spdf);
        lp = make_float3(add(pos.x, mul(wd.x, L.env.sceneDiameter)),
                         add(pos.y, mul(wd.y, L.env.sceneDiameter)),
                         add(pos.z, mul(wd.z, L.env.sceneDiameter)));
        const float3 sd = normalize3(make_float3(sub(pos.x, lp.x), sub(pos.y, lp.y), sub(pos.z, lp.z)));
        const float3 er = env_emit(L.env, make_float3(-sd.x, -sd.y, -sd.z));
        emis = radiance_of<SPEC>(L.spec, er.x, er.y, er.z, waves);
        lightPdf = mul(invN, spdf);
    }
    else
    {
        const PtLight lt = lights[li];
        const float2 u45 = rnd_s45(L, key, i, depth);
        const float r1 = __fsqrt_rn(u45.x), r2 = u45.y;
        const float a = sub(1.0f, r1), b = mul(sub(1.0f, r2), r1), c = mul(r1, r2);
        lp = make_float3(add(add(mul(lt.p0.x, a), mul(lt.p1.x, b)), mul(lt.p2.x, c)),
                         add(add(mul(lt.p0.y, a), mul(lt.p1.y, b)), mul(lt.p2.y, c)),
                         add(add(mul(lt.p0.z, a), mul(lt.p1.z, b)), mul(lt.p2.z, c)));
        float3 sd = make_float3(sub(pos.x, lp.x), sub(pos.y, lp.y), sub(pos.z, lp.z));
        const float distSq = dot3(sd, sd);
        sd = normalize3(sd);
        float ndl = dot3(f3(lt.n), sd);
        ndl = (lt.n.w != 0.0f) ? fabsf(ndl) : fmaxf(0.0f, ndl);
        float ppdf = (ndl == 0.0f) ? 0.0f : __fdiv_rn(__fdiv_rn(1.0f, lt.p0.w), ndl);
        ppdf = mul(ppdf, distSq);
        lightPdf = mul(invN, ppdf);
        const bool emits = (lt.n.w != 0.0f) || (dot3(f3(lt.n), sd) > 0.0f);
        if(emits) emis = radiance_of<SPEC>(L.spec, lt.radiance.x, lt.radiance.y, lt.radiance.z, waves);
    }
}

} // namespace

} // namespace mrg
