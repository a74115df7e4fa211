// pt_api.cpp -- C ABI of the wavefront path tracer (include/mray_gb300.h,
// "Path tracer" section): surface / light description, camera frame, and the
// host-side enqueue of device-driven render passes.
#include "mrg_ctx.h"
#include "zsobol.cuh"
#include "host_math.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace {

mrg_status cuda_err(cudaError_t e, const char* what)
{
    cudaGetLastError();
    return mrg::set_error(e == cudaErrorMemoryAllocation ? MRG_ERR_OUT_OF_MEMORY : MRG_ERR_CUDA,
                          std::string(what) + ": " + cudaGetErrorString(e));
}
#define PT_TRY(call, what) do { cudaError_t e_ = (call); if(e_ != cudaSuccess) return cuda_err(e_, what); } while(0)

struct DevGuard
{
    int prev = -1;
    explicit DevGuard(int d) { if(cudaGetDevice(&prev) != cudaSuccess) prev = -1; if(prev != d) cudaSetDevice(d); }
    ~DevGuard() { if(prev >= 0) cudaSetDevice(prev); }
};

float dot_fma(const float a[3], const float b[3])
{
    return std::fma(a[2], b[2], std::fma(a[1], b[1], std::fma(a[0], b[0], 0.0f)));
}
void cross_fma(const float a[3], const float b[3], float o[3])
{
    const float x = std::fma(a[1], b[2], -a[2] * b[1]);
    const float y = std::fma(a[2], b[0], -a[0] * b[2]);
    const float z = std::fma(a[0], b[1], -a[1] * b[0]);
    o[0] = x; o[1] = y; o[2] = z;
}
void normalize_fma(float v[3])
{
    const float inv = 1.0f / std::sqrt(dot_fma(v, v));
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
}

// CameraPinhole's constructor (Source/Tracer/CamerasDefault.hpp:6-30).
void camera_frame(const mrg_pt_params& p, mrg::PtCamera& c)
{
    const float wh = std::tan(p.fov[0] * 0.5f) * p.nearFar[0];
    const float hh = std::tan(p.fov[1] * 0.5f) * p.nearFar[0];
    float g[3] = { p.camGaze[0] - p.camPos[0], p.camGaze[1] - p.camPos[1], p.camGaze[2] - p.camPos[2] };
    float r[3], u[3];
    cross_fma(g, p.camUp, r); normalize_fma(r);
    cross_fma(r, g, u); normalize_fma(u);
    cross_fma(u, r, g); normalize_fma(g);
    for(int k = 0; k < 3; k++)
    {
        c.pos[k] = p.camPos[k];
        c.right[k] = r[k];
        c.up[k] = u[k];
        c.bottomLeft[k] = ((p.camPos[k] - r[k] * wh) - u[k] * hh) + g[k] * p.nearFar[0];
    }
    c.planeSize[0] = wh * 2.0f;
    c.planeSize[1] = hh * 2.0f;
    c.nearT = p.nearFar[0];
    c.farT = p.nearFar[1];
}

// Light triangle in world space: ApplyP with MRay's 4-term fma Dot
// (TransformsDefault.hpp:19-23), Triangle::Normal / Area (ShapeFunctions.h:60-73).
void make_light(const float m[12], const float v[9], const float radiance[3], uint32_t twoSided,
                uint32_t instance, mrg::PtLight& out)
{
    float w[3][3];
    for(int c = 0; c < 3; c++)
        for(int r = 0; r < 3; r++)
        {
            float acc = 0.0f;
            acc = std::fma(m[4 * r + 0], v[3 * c + 0], acc);
            acc = std::fma(m[4 * r + 1], v[3 * c + 1], acc);
            acc = std::fma(m[4 * r + 2], v[3 * c + 2], acc);
            acc = std::fma(m[4 * r + 3], 1.0f, acc);
            w[c][r] = acc;
        }
    const float e0[3] = { w[1][0] - w[0][0], w[1][1] - w[0][1], w[1][2] - w[0][2] };
    const float e1[3] = { w[2][0] - w[0][0], w[2][1] - w[0][1], w[2][2] - w[0][2] };
    float cr[3];
    cross_fma(e0, e1, cr);
    const float len = std::sqrt(std::fma(cr[2], cr[2], std::fma(cr[1], cr[1], std::fma(cr[0], cr[0], 0.0f))));
    const float area = len * 0.5f;
    const float inv = 1.0f / len;
    out.p0 = make_float4(w[0][0], w[0][1], w[0][2], area);
    float instBits;
    std::memcpy(&instBits, &instance, sizeof(instBits));
    out.p1 = make_float4(w[1][0], w[1][1], w[1][2], instBits);
    out.p2 = make_float4(w[2][0], w[2][1], w[2][2], 0.0f);
    out.n = make_float4(cr[0] * inv, cr[1] * inv, cr[2] * inv, twoSided ? 1.0f : 0.0f);
    out.radiance = make_float4(radiance[0], radiance[1], radiance[2], 0.0f);
}

// ---- skysphere: luminance and the piecewise-constant 2D distribution ----
// Bilinear, wrap-addressed texel read of the host texture view
// (Device/CPU/TextureViewCPU.h:196-375), used for the luminance at texel centres.
void env_read_host(const float* tex, uint32_t w, uint32_t h, float u, float v, float rgb[3])
{
    const float tx = u * (float)w - 0.5f, ty = v * (float)h - 0.5f;
    float bx, by;
    float fx = std::modf(tx, &bx), fy = std::modf(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = std::fabs(fx); }
    if(fy < 0.0f) { sy -= 1; fy = std::fabs(fy); }
    auto wrap = [](int32_t i, int32_t n) { i %= n; return i < 0 ? i + n : i; };
    const float* p[4];
    for(int j = 0; j < 2; j++)
        for(int i = 0; i < 2; i++)
            p[2 * j + i] = &tex[4 * ((size_t)wrap(sy + j, (int32_t)h) * w + (size_t)wrap(sx + i, (int32_t)w))];
    for(int k = 0; k < 3; k++)
    {
        const float a = p[0][k] * (1.0f - fx) + p[1][k] * fx;
        const float b = p[2][k] * (1.0f - fx) + p[3][k] * fx;
        rgb[k] = a * (1.0f - fy) + b * fy;
    }
}

// KCExtractLuminance (Tracer/ColorConverter.cu:405-475): Y of the Rec.709
// (D65) RGB -> XYZ transform, one texel centre at a time; then
// DistributionGroupPwC2D::Construct (Tracer/Distributions.cu:233-330, host
// backend): double row scans of |f|, a float scan of the row totals, and a
// double normalisation of every row and of the marginal.
void env_distribution(const std::vector<float>& tex, uint32_t w, uint32_t h,
                      std::vector<float>& cdfX, std::vector<float>& cdfY)
{
    cdfX.assign((size_t)w * h, 0.0f);
    cdfY.assign(h, 0.0f);
    const float rx = 1.0f / (float)w, ry = 1.0f / (float)h;
    for(uint32_t y = 0; y < h; y++)
    {
        double sum = 0.0;
        for(uint32_t x = 0; x < w; x++)
        {
            float c[3];
            env_read_host(tex.data(), w, h, ((float)x + 0.5f) * rx, ((float)y + 0.5f) * ry, c);
            const float lum = std::fma(0.0721750f, c[2], std::fma(0.7151522f, c[1], 0.2126729f * c[0]));
            sum += (double)std::fabs(lum);
            cdfX[(size_t)y * w + x] = (float)sum;
        }
    }
    float run = 0.0f;
    for(uint32_t y = 0; y < h; y++) { run += cdfX[(size_t)y * w + (w - 1)]; cdfY[y] = run; }
    for(uint32_t y = 0; y < h; y++)
    {
        float* row = &cdfX[(size_t)y * w];
        const double r = 1.0 / (double)row[w - 1];
        for(uint32_t x = 0; x < w; x++) row[x] = (float)((double)row[x] * r);
    }
    const double r = 1.0 / (double)cdfY[h - 1];
    for(uint32_t y = 0; y < h; y++) cdfY[y] = (float)((double)cdfY[y] * r);
}

mrg_status env_prepare(mrg_ctx* c)
{
    cudaFree(c->dPtEnv);
    c->dPtEnv = nullptr;
    c->ptEnv = mrg::PtEnv{};
    if(!c->ptEnvSet) return MRG_OK;
    const uint32_t w = c->ptEnvW, h = c->ptEnvH;
    std::vector<float> cdfX, cdfY;
    env_distribution(c->ptEnvTexels, w, h, cdfX, cdfY);
    const size_t texBytes = sizeof(float) * c->ptEnvTexels.size();
    const size_t xBytes = (sizeof(float) * cdfX.size() + 255) & ~size_t(255);
    const size_t yBytes = sizeof(float) * cdfY.size();
    PT_TRY(cudaMalloc(&c->dPtEnv, texBytes + xBytes + yBytes), "mrg_pt: skysphere");
    char* base = static_cast<char*>(c->dPtEnv);
    PT_TRY(cudaMemcpy(base, c->ptEnvTexels.data(), texBytes, cudaMemcpyHostToDevice), "mrg_pt: skysphere upload");
    PT_TRY(cudaMemcpy(base + texBytes, cdfX.data(), sizeof(float) * cdfX.size(), cudaMemcpyHostToDevice),
           "mrg_pt: skysphere upload");
    PT_TRY(cudaMemcpy(base + texBytes + xBytes, cdfY.data(), yBytes, cudaMemcpyHostToDevice), "mrg_pt: skysphere upload");
    mrg::PtEnv& E = c->ptEnv;
    E.texels = reinterpret_cast<const float4*>(base);
    E.cdfX = reinterpret_cast<const float*>(base + texBytes);
    E.cdfY = reinterpret_cast<const float*>(base + texBytes + xBytes);
    float inv[12];
    mrg::mat34_inverse(c->ptEnvM, inv, true);
    for(int r = 0; r < 3; r++)
    {
        E.m[r] = make_float4(c->ptEnvM[4 * r], c->ptEnvM[4 * r + 1], c->ptEnvM[4 * r + 2], 0.0f);
        E.inv[r] = make_float4(inv[4 * r], inv[4 * r + 1], inv[4 * r + 2], 0.0f);
    }
    E.width = w; E.height = h;
    // TracerBase.cpp:1650-1664: the diagonal of the scene box over the XZ plane
    const float sx = c->sceneBoxExact[3] - c->sceneBoxExact[0];
    const float sz = c->sceneBoxExact[5] - c->sceneBoxExact[2];
    E.sceneDiameter = std::sqrt(std::fma(sz, sz, sx * sx));
    E.enabled = 1u;
    return MRG_OK;
}

// ZSobol / PCG32 state of a render: the tables (once per context) and the
// per-pixel seeds of (width, height, seed), kept while those stay the same.
// Both groups seed a pixel from the same std::mt19937 output
// (RNGGroupZSobol, Random.cu:1175-1200; RNGGroupIndependent, Random.cu:683-704).
mrg_status pt_zsobol(mrg_ctx* c, const mrg_pt_params& p, mrg::PtLaunch& L, const std::string& w)
{
    if(!c->dZsTables)
    {
        uint32_t t[mrg::kZsTableWords];
        mrg::zsobol_tables(t);
        PT_TRY(cudaMalloc(&c->dZsTables, sizeof(t)), "ZSobol tables");
        PT_TRY(cudaMemcpy(c->dZsTables, t, sizeof(t), cudaMemcpyHostToDevice), "ZSobol tables");
    }
    if(!c->dZsSeeds || c->zsW != p.width || c->zsH != p.height || c->zsSeed != p.seed)
    {
        std::vector<uint32_t> seeds((size_t)p.width * p.height);
        mrg_status s = mrg_zsobol_seeds(p.width, p.height, p.seed, seeds.data());
        if(s != MRG_OK) return s;
        cudaFree(c->dZsSeeds);
        c->dZsSeeds = nullptr;
        PT_TRY(cudaMalloc(&c->dZsSeeds, sizeof(uint32_t) * seeds.size()), "ZSobol seeds");
        PT_TRY(cudaMemcpy(c->dZsSeeds, seeds.data(), sizeof(uint32_t) * seeds.size(), cudaMemcpyHostToDevice),
               "ZSobol seeds");
        c->zsW = p.width; c->zsH = p.height; c->zsSeed = p.seed;
    }
    const uint64_t maxSpp = p.samplerMaxSpp ? p.samplerMaxSpp : (uint64_t)p.sampleStart + p.spp;
    if(maxSpp == 0 || maxSpp > 0x80000000ull) return mrg::set_error(MRG_ERR_INVALID_ARG, w + ": ZSobol sample count");
    const uint32_t m = std::max(p.width, p.height);
    uint32_t pow2 = 1;
    while(pow2 < m) pow2 <<= 1;
    uint32_t bits = 0;
    while((1u << bits) < pow2) bits++;
    L.zsMaxSpp = (uint32_t)maxSpp;
    L.zsResBits = bits;
    L.zsSeeds = c->dZsSeeds;
    L.zsTables = c->dZsTables;
    return MRG_OK;
}

// KCGenerateMipmaps' samples (TextureFilter.cu:62-110, GenerateMipsGeneric
// :1006-1100): 8 x 8 per texel, xi = (k + 0.5) / 8 per axis, in ACCUMULATE mode
// at offset xi 2 r - r pixels, weighted by the Gaussian filter of radius r
// (sigma = 0.285714 r; Math::Gaussian, Core/Math.h:1032-1042).
mrg::MipTaps mip_taps(float r)
{
    mrg::MipTaps t;
    const float sigma = r * 0.285714f;
    const float invSqrt2Pi = (1.0f / 1.4142135623730950488f) * (1.0f / 1.772453850905516027298f);
    for(int k = 0; k < 8; k++)
    {
        const float d = 1.0f / 8.0f;
        const float xi = d * 0.5f + d * (float)k;
        t.off[k] = xi * 2.0f * r - r;
        const float sInv = 1.0f / sigma;
        const float pw = (t.off[k] - 0.0f) * sInv;
        t.g[k] = (invSqrt2Pi * sInv) * std::exp(-0.5f * pw * pw);
    }
    return t;
}

// Uploads surfaces, lights and the primitive-indexed triangle table.
mrg_status pt_prepare(mrg_ctx* c)
{
    if(!c->ptDirty) return MRG_OK;
    const uint32_t ni = (uint32_t)c->insts.size();
    if(c->ptDesc.size() < ni) c->ptDesc.resize(ni);
    std::vector<mrg::PtSurface> surf(ni);
    std::vector<mrg::PtLight> lights;
    uint32_t maxPrim = 0;
    for(const auto& m : c->meshes)
        maxPrim = std::max<uint32_t>(maxPrim, m.primKeyBase + (uint32_t)(m.idx.size() / 3));
    if(maxPrim > (1u << 28))
        return mrg::set_error(MRG_ERR_LIMIT, "mrg_pt: primitive keys must be dense indices below 2^28");
    std::vector<float4> tris(3ull * maxPrim, make_float4(0, 0, 0, 0));
    for(const auto& m : c->meshes)
    {
        const uint32_t nt = (uint32_t)(m.idx.size() / 3);
        for(uint32_t t = 0; t < nt; t++)
        {
            const float* a = &m.pos[3ull * m.idx[3ull * t]];
            const float* b = &m.pos[3ull * m.idx[3ull * t + 1]];
            const float* d = &m.pos[3ull * m.idx[3ull * t + 2]];
            const size_t g = 3ull * (m.primKeyBase + t);
            tris[g] = make_float4(a[0], a[1], a[2], 0.0f);
            tris[g + 1] = make_float4(b[0] - a[0], b[1] - a[1], b[2] - a[2], 0.0f);
            tris[g + 2] = make_float4(d[0] - a[0], d[1] - a[1], d[2] - a[2], 0.0f);
        }
    }
    for(uint32_t i = 0; i < ni; i++)
    {
        const auto& in = c->insts[i];
        const auto& d = c->ptDesc[i];
        const auto& mesh = c->meshes[in.mesh];
        mrg::PtSurface& s = surf[i];
        for(int r = 0; r < 3; r++)
        {
            s.m[r] = make_float4(in.m[4 * r], in.m[4 * r + 1], in.m[4 * r + 2], in.m[4 * r + 3]);
            s.inv[r] = make_float4(in.inv[4 * r], in.inv[4 * r + 1], in.inv[4 * r + 2], in.inv[4 * r + 3]);
        }
        s.albedo = make_float4(d.albedo[0], d.albedo[1], d.albedo[2], d.roughness);
        s.mat = make_float4(d.metallic, d.specular, d.iorFront, d.iorBack);
        s.info = make_uint4(d.kind == 2 ? 1u : 0u, (uint32_t)lights.size(), mesh.primKeyBase, d.material);
        s.tex = d.kind == 1 ? make_uint4(d.texture, d.paramTex[0], d.paramTex[1], d.paramTex[2])
                            : make_uint4(0u, 0u, 0u, 0u);
        if((s.tex.x | s.tex.y | s.tex.z | s.tex.w) && mesh.uv.empty())
            return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt: instance " + std::to_string(i) +
                                  " has a texture but its mesh has no uvs");
        if(d.kind == 2)
        {
            const uint32_t nt = (uint32_t)(mesh.idx.size() / 3);
            for(uint32_t t = 0; t < nt; t++)
            {
                float v[9];
                for(int k = 0; k < 3; k++)
                    for(int q = 0; q < 3; q++) v[3 * k + q] = mesh.pos[3ull * mesh.idx[3ull * t + k] + q];
                mrg::PtLight L;
                make_light(in.m, v, d.radiance, d.twoSided, i, L);
                lights.push_back(L);
            }
        }
    }
    cudaFree(c->dPtSurfaces); cudaFree(c->dPtLights); cudaFree(c->dPtTris);
    c->dPtSurfaces = c->dPtLights = c->dPtTris = nullptr;
    PT_TRY(cudaMalloc(&c->dPtSurfaces, sizeof(mrg::PtSurface) * std::max<size_t>(1, surf.size())), "mrg_pt: surfaces");
    PT_TRY(cudaMalloc(&c->dPtLights, sizeof(mrg::PtLight) * std::max<size_t>(1, lights.size())), "mrg_pt: lights");
    PT_TRY(cudaMalloc(&c->dPtTris, sizeof(float4) * std::max<size_t>(1, tris.size())), "mrg_pt: triangles");
    if(!surf.empty()) PT_TRY(cudaMemcpy(c->dPtSurfaces, surf.data(), sizeof(mrg::PtSurface) * surf.size(), cudaMemcpyHostToDevice), "mrg_pt: upload");
    if(!lights.empty()) PT_TRY(cudaMemcpy(c->dPtLights, lights.data(), sizeof(mrg::PtLight) * lights.size(), cudaMemcpyHostToDevice), "mrg_pt: upload");
    if(!tris.empty()) PT_TRY(cudaMemcpy(c->dPtTris, tris.data(), sizeof(float4) * tris.size(), cudaMemcpyHostToDevice), "mrg_pt: upload");
    c->ptSurfaceCount = ni;
    c->ptLightCount = (uint32_t)lights.size();
    c->ptTriCount = maxPrim;
    // texture coordinates per primitive key, and the texture table
    cudaFree(c->dPtUvs); c->dPtUvs = nullptr;
    bool anyUv = false;
    for(const auto& m : c->meshes) anyUv |= !m.uv.empty();
    if(anyUv)
    {
        std::vector<float4> uvs(2ull * maxPrim, make_float4(0, 0, 0, 0));
        for(const auto& m : c->meshes)
        {
            if(m.uv.empty()) continue;
            const uint32_t nt = (uint32_t)(m.idx.size() / 3);
            for(uint32_t t = 0; t < nt; t++)
            {
                const float* a = &m.uv[2ull * m.idx[3ull * t]];
                const float* b = &m.uv[2ull * m.idx[3ull * t + 1]];
                const float* d = &m.uv[2ull * m.idx[3ull * t + 2]];
                const size_t g = 2ull * (m.primKeyBase + t);
                uvs[g] = make_float4(a[0], a[1], b[0], b[1]);
                uvs[g + 1] = make_float4(d[0], d[1], 0.0f, 0.0f);
            }
        }
        PT_TRY(cudaMalloc(&c->dPtUvs, sizeof(float4) * uvs.size()), "mrg_pt: uvs");
        PT_TRY(cudaMemcpy(c->dPtUvs, uvs.data(), sizeof(float4) * uvs.size(), cudaMemcpyHostToDevice), "mrg_pt: uvs");
    }
    cudaFree(c->dPtTexTable); c->dPtTexTable = nullptr;
    cudaFree(c->dPtTexData); c->dPtTexData = nullptr;
    cudaFree(c->dPtMipData); c->dPtMipData = nullptr;
    if(!c->ptTextures.empty())
    {
        size_t owned = 0;
        for(const auto& t : c->ptTextures) owned += (t.host.size() + 255) & ~size_t(255);
        if(owned) PT_TRY(cudaMalloc(&c->dPtTexData, owned), "mrg_pt: textures");
        std::vector<mrg::PtTexture> table(c->ptTextures.size());
        size_t off = 0;
        for(size_t k = 0; k < c->ptTextures.size(); k++)
        {
            const auto& t = c->ptTextures[k];
            table[k].width = t.width; table[k].height = t.height; table[k].format = t.format;
            table[k].mipCount = 1; table[k].mips = nullptr;
            if(t.borrowed) table[k].texels = t.borrowed;
            else
            {
                char* dst = static_cast<char*>(c->dPtTexData) + off;
                PT_TRY(cudaMemcpy(dst, t.host.data(), t.host.size(), cudaMemcpyHostToDevice), "mrg_pt: textures");
                table[k].texels = dst;
                off += (t.host.size() + 255) & ~size_t(255);
            }
        }
        // mip chains (TextureMemory::GenerateMipmaps): levels 1.. of every
        // texture that has a generation filter or given levels; given levels
        // are copied in place and kept, the others are filtered on the device
        // from their parent
        std::vector<uint32_t> levels(c->ptTextures.size(), 1u);
        size_t mipBytes = 0;
        for(size_t k = 0; k < c->ptTextures.size(); k++)
        {
            const auto& t = c->ptTextures[k];
            uint32_t last = 0;
            for(uint32_t m = 1; m < t.given.size(); m++)
                if(!t.given[m].empty()) last = m;
            if(t.mipRadius > 0.0f) levels[k] = mrg::mip_level_count(t.width, t.height);
            else if(last)
            {
                for(uint32_t m = 1; m < last; m++)
                    if(t.given[m].empty())
                        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt: texture " + std::to_string(k) + " mip " +
                                              std::to_string(m) + " has no data and no generation filter");
                levels[k] = last + 1u;
            }
            if(levels[k] > 1u)
                mipBytes += (mrg::mip_chain_texels(t.width, t.height, levels[k]) * (t.format == MRG_TEX_RGBA8 ? 4u : 16u) +
                             255) & ~size_t(255);
        }
        if(mipBytes)
        {
            PT_TRY(cudaMalloc(&c->dPtMipData, mipBytes), "mrg_pt: mips");
            size_t moff = 0;
            for(size_t k = 0; k < c->ptTextures.size(); k++)
            {
                const auto& t = c->ptTextures[k];
                if(levels[k] <= 1u) continue;
                const size_t bpp = t.format == MRG_TEX_RGBA8 ? 4u : 16u;
                char* dst = static_cast<char*>(c->dPtMipData) + moff;
                uint32_t valid = 0;
                for(uint32_t m = 1; m < levels[k] && m < t.given.size(); m++)
                    if(!t.given[m].empty())
                    {
                        PT_TRY(cudaMemcpy(dst + mrg::mip_chain_texels(t.width, t.height, m) * bpp, t.given[m].data(),
                                          t.given[m].size(), cudaMemcpyHostToDevice), "mrg_pt: mips");
                        valid |= 1u << m;
                    }
                if(t.mipRadius > 0.0f)
                    PT_TRY(mrg::generate_mips(table[k].texels, dst, t.width, t.height, t.format, mip_taps(t.mipRadius),
                                              levels[k], valid), "mrg_pt: mips");
                table[k].mips = dst;
                table[k].mipCount = levels[k];
                moff += (mrg::mip_chain_texels(t.width, t.height, levels[k]) * bpp + 255) & ~size_t(255);
            }
        }
        PT_TRY(cudaMalloc(&c->dPtTexTable, sizeof(mrg::PtTexture) * table.size()), "mrg_pt: textures");
        PT_TRY(cudaMemcpy(c->dPtTexTable, table.data(), sizeof(mrg::PtTexture) * table.size(), cudaMemcpyHostToDevice),
               "mrg_pt: textures");
    }
    uint32_t groups = 0;
    for(uint32_t i = 0; i < ni; i++)
        if(c->ptDesc[i].kind == 1) groups |= 1u << std::min<uint32_t>(c->ptDesc[i].material, 31u);
    c->ptMaterialGroups = (uint32_t)__builtin_popcount(groups);
    mrg_status es = env_prepare(c);
    if(es != MRG_OK) return es;
    c->ptDirty = false;
    return MRG_OK;
}

// Path state of `slots` paths in one allocation (P / mem: one pipeline's).
mrg_status pt_paths_into(mrg::PtPaths& P, void*& mem, uint32_t slots)
{
    if(P.capacity >= slots && mem) return MRG_OK;
    cudaFree(mem);
    mem = nullptr;
    P = mrg::PtPaths{};
    const size_t n = slots;
    const size_t words = (n + 31) / 32;
    // one allocation, every array 256-byte aligned
    const size_t sizes[22] = { n * 32, n * 16, n * 8, n * 16, n * 16, n * 4, n * 32, n * 16,
                               words * 4, n * 4, n * 4, n * 4, 64, n * 4, n * 4, n * 4,
                               4 * mrg::multisplit_hist_words(slots, mrg::kPtWorkKeyBits),
                               n * 4, n * 16, n * 16, n * 4, n * 8 };
    size_t need = 0;
    for(size_t sz : sizes) need += (sz + 255) & ~size_t(255);
    char* base = nullptr;
    PT_TRY(cudaMalloc(&base, need), "mrg_pt: path state");
    mem = base;
    size_t off = 0;
    int k = 0;
    auto take = [&]() { char* q = base + off; off += (sizes[k++] + 255) & ~size_t(255); return q; };
    P.rays = reinterpret_cast<float4*>(take());
    P.hits = reinterpret_cast<uint4*>(take());
    P.meta = reinterpret_cast<float2*>(take());
    P.thr = reinterpret_cast<float4*>(take());
    P.rad = reinterpret_cast<float4*>(take());
    P.state = reinterpret_cast<uint32_t*>(take());
    P.shadowRays = reinterpret_cast<float4*>(take());
    P.shadowRad = reinterpret_cast<float4*>(take());
    P.visBits = reinterpret_cast<uint32_t*>(take());
    P.listA = reinterpret_cast<uint32_t*>(take());
    P.listB = reinterpret_cast<uint32_t*>(take());
    P.shadowList = reinterpret_cast<uint32_t*>(take());
    P.counts = reinterpret_cast<uint32_t*>(take());
    P.workKeys = reinterpret_cast<uint32_t*>(take());
    P.workKeysOut = reinterpret_cast<uint32_t*>(take());
    P.listSorted = reinterpret_cast<uint32_t*>(take());
    P.sortHist = reinterpret_cast<uint32_t*>(take());
    P.prevPdf = reinterpret_cast<float*>(take());
    P.waves = reinterpret_cast<float4*>(take());
    P.wavePdf = reinterpret_cast<float4*>(take());
    P.shadowLight = reinterpret_cast<uint32_t*>(take());
    P.cone = reinterpret_cast<float2*>(take());
    P.capacity = slots;
    return MRG_OK;
}

mrg_status pt_paths(mrg_ctx* c, uint32_t slots) { return pt_paths_into(c->ptPaths, c->ptPathMem, slots); }

} // namespace

extern "C" {

mrg_status mrg_pt_set_lambert(mrg_ctx* c, uint32_t inst, const float albedo[3])
{
    if(!c || !albedo) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_lambert: null pointer");
    if(inst >= c->insts.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_lambert: bad instance id");
    if(c->ptDesc.size() < c->insts.size()) c->ptDesc.resize(c->insts.size());
    auto& d = c->ptDesc[inst];
    d.kind = 1;
    std::memcpy(d.albedo, albedo, sizeof(d.albedo));
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_material(mrg_ctx* c, uint32_t inst, const mrg_pt_material* m)
{
    if(!c || !m) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_material: null pointer");
    if(inst >= c->insts.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_material: bad instance id");
    if(m->type > MRG_MAT_UNREAL) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_material: unknown type");
    if(c->ptDesc.size() < c->insts.size()) c->ptDesc.resize(c->insts.size());
    auto& d = c->ptDesc[inst];
    d.kind = 1;
    d.material = m->type;
    std::memcpy(d.albedo, m->albedo, sizeof(d.albedo));
    d.roughness = m->roughness; d.metallic = m->metallic; d.specular = m->specular;
    d.iorFront = m->iorFront; d.iorBack = m->iorBack;
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_area_light(mrg_ctx* c, uint32_t inst, const float radiance[3], uint32_t twoSided)
{
    if(!c || !radiance) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_area_light: null pointer");
    if(inst >= c->insts.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_area_light: bad instance id");
    if(c->ptDesc.size() < c->insts.size()) c->ptDesc.resize(c->insts.size());
    auto& d = c->ptDesc[inst];
    d.kind = 2;
    std::memcpy(d.radiance, radiance, sizeof(d.radiance));
    d.twoSided = twoSided;
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_env(mrg_ctx* c, uint32_t width, uint32_t height, const float* rgba, const float m3x4[12])
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_env: null context");
    if(width == 0)
    {
        c->ptEnvSet = false;
        c->ptEnvTexels.clear();
        c->ptDirty = true;
        return MRG_OK;
    }
    if(!rgba || height == 0) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_env: null map or zero height");
    if((uint64_t)width * height > (1ull << 26))
        return mrg::set_error(MRG_ERR_LIMIT, "mrg_pt_set_env: more than 2^26 texels");
    const size_t n = 4ull * width * height;
    for(size_t i = 0; i < n; i++)
        if(!std::isfinite(rgba[i])) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_env: non-finite texel");
    c->ptEnvTexels.assign(rgba, rgba + n);
    c->ptEnvW = width; c->ptEnvH = height;
    const float ident[12] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0 };
    std::memcpy(c->ptEnvM, m3x4 ? m3x4 : ident, sizeof(c->ptEnvM));
    c->ptEnvSet = true;
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_spectral(mrg_ctx* c, uint32_t lutRes, const float* lut, uint32_t cieCount,
                               const float* cieXyz, const float integrals[3], const float* spd, float norm,
                               const float xyzToRgb[9])
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_spectral: null context");
    DevGuard g(c->device);
    if(lutRes == 0)
    {
        cudaFree(c->dPtSpec);
        c->dPtSpec = nullptr;
        c->ptSpec = mrg::PtSpectral{};
        return MRG_OK;
    }
    if(!lut || !cieXyz || !integrals || !spd || !xyzToRgb || cieCount < 2)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_spectral: null table or fewer than 2 observer samples");
    if(lutRes < 2 || lutRes > 256) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_spectral: LUT resolution out of [2, 256]");
    const size_t lutN = 9ull * lutRes * lutRes * lutRes;
    // SpectrumContext.cu:400-420: observer / CIE integrals, illuminant * Y / norm
    std::vector<float> obs(3ull * cieCount), ill(cieCount);
    const float w[3] = { 1.0f / integrals[0], 1.0f / integrals[1], 1.0f / integrals[2] };
    const float f = integrals[1] / norm;
    for(uint32_t i = 0; i < cieCount; i++)
    {
        for(int k = 0; k < 3; k++) obs[3ull * i + k] = cieXyz[3ull * i + k] * w[k];
        ill[i] = spd[i] * f;
    }
    const size_t lutBytes = (sizeof(float) * lutN + 255) & ~size_t(255);
    const size_t obsBytes = (sizeof(float) * obs.size() + 255) & ~size_t(255);
    cudaFree(c->dPtSpec);
    c->dPtSpec = nullptr;
    c->ptSpec = mrg::PtSpectral{};
    PT_TRY(cudaMalloc(&c->dPtSpec, lutBytes + obsBytes + sizeof(float) * ill.size()), "mrg_pt_set_spectral");
    char* base = static_cast<char*>(c->dPtSpec);
    PT_TRY(cudaMemcpy(base, lut, sizeof(float) * lutN, cudaMemcpyHostToDevice), "mrg_pt_set_spectral: upload");
    PT_TRY(cudaMemcpy(base + lutBytes, obs.data(), sizeof(float) * obs.size(), cudaMemcpyHostToDevice),
           "mrg_pt_set_spectral: upload");
    PT_TRY(cudaMemcpy(base + lutBytes + obsBytes, ill.data(), sizeof(float) * ill.size(), cudaMemcpyHostToDevice),
           "mrg_pt_set_spectral: upload");
    mrg::PtSpectral& S = c->ptSpec;
    S.lut = reinterpret_cast<const float*>(base);
    S.observer = reinterpret_cast<const float*>(base + lutBytes);
    S.illuminant = reinterpret_cast<const float*>(base + lutBytes + obsBytes);
    std::memcpy(S.xyzToRgb, xyzToRgb, sizeof(S.xyzToRgb));
    S.lutRes = lutRes;
    S.cieCount = cieCount;
    S.enabled = 1u;
    return MRG_OK;
}

mrg_status mrg_pt_add_texture(mrg_ctx* c, uint32_t w, uint32_t h, uint32_t format, const void* texels,
                              uint32_t borrow, uint32_t* outId)
{
    if(!c || !texels || !outId) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_add_texture: null pointer");
    if(w == 0 || h == 0 || format > MRG_TEX_RGBA32F)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_add_texture: empty texture or unknown format");
    if((uint64_t)w * h > (1ull << 28)) return mrg::set_error(MRG_ERR_LIMIT, "mrg_pt_add_texture: more than 2^28 texels");
    mrg_ctx::PtTextureDesc t;
    t.width = w; t.height = h; t.format = format;
    if(borrow) t.borrowed = texels;
    else
    {
        const size_t bytes = (size_t)w * h * (format == MRG_TEX_RGBA8 ? 4u : 16u);
        try { t.host.assign(static_cast<const uint8_t*>(texels), static_cast<const uint8_t*>(texels) + bytes); }
        catch(...) { return mrg::set_error(MRG_ERR_OUT_OF_MEMORY, "mrg_pt_add_texture: host allocation"); }
    }
    c->ptTextures.push_back(std::move(t));
    *outId = (uint32_t)(c->ptTextures.size() - 1);
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_generate_mips(mrg_ctx* c, uint32_t texId, float filterRadius)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_generate_mips: null pointer");
    if(texId >= c->ptTextures.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_generate_mips: unknown texture");
    if(!(filterRadius >= 0.0f) || filterRadius > 64.0f)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_generate_mips: filter radius in [0, 64]");
    c->ptTextures[texId].mipRadius = filterRadius;
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_texture_mip(mrg_ctx* c, uint32_t texId, uint32_t level, const void* texels)
{
    if(!c || !texels) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_texture_mip: null pointer");
    if(texId >= c->ptTextures.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_texture_mip: unknown texture");
    auto& t = c->ptTextures[texId];
    const uint32_t full = mrg::mip_level_count(t.width, t.height);
    if(level == 0 || level >= full)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_texture_mip: level in [1, " + std::to_string(full) + ")");
    const size_t bytes = (size_t)std::max(t.width >> level, 1u) * std::max(t.height >> level, 1u) *
                         (t.format == MRG_TEX_RGBA8 ? 4u : 16u);
    if(t.given.size() < full) t.given.resize(full);
    const uint8_t* b = static_cast<const uint8_t*>(texels);
    t.given[level].assign(b, b + bytes);
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_unreal_textures(mrg_ctx* c, uint32_t inst, uint32_t roughnessTex, uint32_t metallicTex,
                                      uint32_t specularTex)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_unreal_textures: null context");
    if(inst >= c->insts.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_unreal_textures: bad instance");
    const uint32_t ids[3] = { roughnessTex, metallicTex, specularTex };
    for(uint32_t id : ids)
        if(id != 0xFFFFFFFFu && id >= c->ptTextures.size())
            return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_unreal_textures: bad texture id");
    if(c->ptDesc.size() < c->insts.size()) c->ptDesc.resize(c->insts.size());
    for(int k = 0; k < 3; k++) c->ptDesc[inst].paramTex[k] = (ids[k] == 0xFFFFFFFFu) ? 0u : ids[k] + 1u;
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_set_albedo_texture(mrg_ctx* c, uint32_t inst, uint32_t texId)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_albedo_texture: null context");
    if(inst >= c->insts.size()) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_albedo_texture: bad instance");
    if(texId != 0xFFFFFFFFu && texId >= c->ptTextures.size())
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_set_albedo_texture: bad texture id");
    if(c->ptDesc.size() < c->insts.size()) c->ptDesc.resize(c->insts.size());
    c->ptDesc[inst].texture = (texId == 0xFFFFFFFFu) ? 0u : texId + 1u;
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_pt_camera_frame(const mrg_pt_params* p, float out[16])
{
    if(!p || !out) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_camera_frame: null pointer");
    mrg::PtCamera cam;
    camera_frame(*p, cam);
    std::memcpy(out, cam.pos, 12); std::memcpy(out + 3, cam.bottomLeft, 12);
    std::memcpy(out + 6, cam.right, 12); std::memcpy(out + 9, cam.up, 12);
    out[12] = cam.planeSize[0]; out[13] = cam.planeSize[1]; out[14] = cam.nearT; out[15] = cam.farT;
    return MRG_OK;
}

} // extern "C"

namespace {

// One render's launch description, scene tables and switches.
struct PtRun
{
    mrg::PtLaunch       L{};
    mrg::PtSceneTables  T{};
    mrg::TraceScratch   scr{};
    bool                partition = false;
    uint32_t            spp = 1;       // samples per pass
    uint32_t            slots = 0;
};

mrg_status pt_setup(mrg_ctx* c, const mrg_pt_params* p, PtRun& R, const char* who)
{
    const std::string w(who);
    if(!c->built) return mrg::set_error(MRG_ERR_NOT_BUILT, w + ": call mrg_build first");
    if(p->width == 0 || p->height == 0 || p->spp == 0)
        return mrg::set_error(MRG_ERR_INVALID_ARG, w + ": empty image or zero samples");
    if(p->maxDepth == 0 || p->maxDepth > 255 || p->sampleMode > MRG_PT_NEE_MIS || p->partitionByMaterial > 2u)
        return mrg::set_error(MRG_ERR_INVALID_ARG, w + ": maxDepth must be in [1, 255], sampleMode and "
                                                   "partitionByMaterial in [0, 2]");
    const uint64_t wh = (uint64_t)p->width * p->height;
    uint32_t spp = p->samplesPerPass ? p->samplesPerPass
                                     : std::max<uint32_t>(1, (uint32_t)std::min<uint64_t>(p->spp, (1ull << 22) / wh));
    spp = std::min(spp, p->spp);
    if(p->spp % spp != 0) spp = 1;
    if(wh * spp > (1ull << 26)) return mrg::set_error(MRG_ERR_LIMIT, w + ": more than 2^26 paths per pass");
    for(uint32_t i = 0; i < c->insts.size(); i++)
        if(i >= c->ptDesc.size() || c->ptDesc[i].kind == 0)
            return mrg::set_error(MRG_ERR_INVALID_ARG, w + ": instance " + std::to_string(i) + " has no material or light");
    mrg_status s = pt_prepare(c);
    if(s != MRG_OK) return s;
    R.spp = spp;
    R.slots = (uint32_t)(wh * spp);
    if((s = pt_paths(c, R.slots)) != MRG_OK) return s;
    mrg::PtLaunch& L = R.L;
    L.width = p->width; L.height = p->height;
    L.slots = R.slots; L.samplesPerPass = spp;
    L.rrStart = p->rrStart; L.maxDepth = p->maxDepth;
    L.sampleMode = p->sampleMode; L.seed = p->seed;
    L.nLights = c->ptLightCount;
    L.env = c->ptEnv;
    L.spec = c->ptSpec;
    L.filterSigma = p->filterRadius * 0.285714f;
    // CameraPinhole's ray cone (CamerasDefault.hpp:80-86): 2 tan(fovY / 2) / image height
    L.coneAperture = 2.0f * std::tan(p->fov[1] * 0.5f) / (float)p->height;
    if(p->sampler > MRG_PT_SAMPLER_PCG32) return mrg::set_error(MRG_ERR_INVALID_ARG, w + ": unknown sampler");
    // a PCG32 stream holds 2^32 numbers: 16 per bounce, maxDepth + 1 bounces per sample
    if(p->sampler == MRG_PT_SAMPLER_PCG32 &&
       ((uint64_t)p->sampleStart + p->spp) * ((uint64_t)p->maxDepth + 1u) * 16u > 0x100000000ull)
        return mrg::set_error(MRG_ERR_INVALID_ARG, w + ": samples x depth exceed the PCG32 stream");
    L.sampler = p->sampler;
    if(L.sampler != MRG_PT_SAMPLER_INDEPENDENT && (s = pt_zsobol(c, *p, L, w)) != MRG_OK) return s;
    camera_frame(*p, L.cam);
    R.partition = p->partitionByMaterial == 1u ||
                  (p->partitionByMaterial == 2u && (c->ptMaterialGroups > 1u || c->ptEnvSet));
    R.scr.workCounter = c->dScratch;
    R.scr.errorFlag = c->dScratch + 1;
    R.scr.stats = c->dStats;
    R.T.surfaces = static_cast<const mrg::PtSurface*>(c->dPtSurfaces);
    R.T.nSurfaces = c->ptSurfaceCount;
    R.T.lights = static_cast<const mrg::PtLight*>(c->dPtLights);
    R.T.tris = static_cast<const float4*>(c->dPtTris);
    R.T.nTris = c->ptTriCount;
    R.T.uvs = static_cast<const float4*>(c->dPtUvs);
    R.T.textures = static_cast<const mrg::PtTexture*>(c->dPtTexTable);
    return MRG_OK;
}

// raygen + maxDepth bounces of the pass at R.L.sampleBase; leaves each slot's
// radiance in the path state.
// Shadow casts overlap the next closest-hit cast (MRG_PT_OVERLAP=0: one stream).
bool pt_overlap()
{
    const char* v = std::getenv("MRG_PT_OVERLAP");
    return !(v && v[0] == '0');
}

// One pipeline of passes: path state, the stream its closest-hit casts and
// shading run on, the side stream of its shadow casts, their events, and the
// ray-claim counters of its two casts.
struct PtLane
{
    mrg::PtPaths* P;
    cudaStream_t  st;
    cudaStream_t  side;          // == st without overlap
    cudaEvent_t   evShaded, evResolved;
    uint32_t*     closestCounter;
    uint32_t*     shadowCounter;
};

mrg_status pt_lane0(mrg_ctx* c, cudaStream_t st, PtLane& lane)
{
    const bool overlap = pt_overlap();
    if(overlap && !c->ptSideStream)
    {
        PT_TRY(cudaStreamCreateWithFlags(&c->ptSideStream, cudaStreamNonBlocking), "mrg_pt: stream");
        PT_TRY(cudaEventCreateWithFlags(&c->ptEvShaded, cudaEventDisableTiming), "mrg_pt: event");
        PT_TRY(cudaEventCreateWithFlags(&c->ptEvResolved, cudaEventDisableTiming), "mrg_pt: event");
    }
    lane = PtLane{ &c->ptPaths, st, overlap ? c->ptSideStream : st, c->ptEvShaded, c->ptEvResolved,
                   c->dScratch + 0, c->dScratch + (overlap ? 2 : 0) };
    return MRG_OK;
}

// One pass of bounces.  Per bounce: closest-hit cast of the alive paths,
// optional material-key partition, shading (continuations, NEE shadow rays),
// shadow cast and resolve.  The shadow cast and resolve of bounce d run on a
// side stream, beside the closest-hit cast and partition of bounce d + 1;
// shading of bounce d + 1 waits for them, since it rewrites the shadow rays,
// list and count and adds to the same path radiance.  The two casts claim
// rays through separate counters.
cudaError_t pt_bounces(mrg_ctx* c, PtRun& R, const PtLane& lane)
{
    mrg::PtPaths& P = *lane.P;
    const mrg::PtLaunch& L = R.L;
    cudaStream_t st = lane.st, side = lane.side;
    const bool overlap = side != st;
    mrg::TraceScratch closestScr = R.scr, shadowScr = R.scr;
    closestScr.workCounter = lane.closestCounter;
    shadowScr.workCounter = lane.shadowCounter;
    // with the cache every path has ended by vertex recPerPath + 1
    const uint32_t loops = (L.cache.mode == 1u) ? std::min(L.maxDepth, L.cache.recPerPath + 2u) : L.maxDepth;
    cudaError_t e = mrg::pt_raygen(L, P, P.listA, P.counts + 0, c->smCount, st);
    for(uint32_t depth = 0; depth < loops && e == cudaSuccess; depth++)
    {
        uint32_t* alive = (depth & 1u) ? P.listB : P.listA;
        uint32_t* next = (depth & 1u) ? P.listA : P.listB;
        uint32_t* aliveCount = P.counts + ((depth & 1u) ? 1 : 0);
        uint32_t* nextCount = P.counts + ((depth & 1u) ? 0 : 1);
        e = cudaMemsetAsync(nextCount, 0, sizeof(uint32_t), st);
        if(e == cudaSuccess)
            e = mrg::launch_closest(c->scene, closestScr, P.rays, alive, 0, P.hits, P.meta, c->smCount, st, aliveCount);
        const uint32_t* shadeList = alive;
        if(e == cudaSuccess && R.partition)
        {
            mrg::DigitSpec ks;
            ks.batchShift = 0; ks.batchWidth = mrg::kPtWorkKeyBits;
            ks.digitShift = 0; ks.digitBits = mrg::kPtWorkKeyBits;
            e = mrg::pt_work_keys(P, R.T.surfaces, R.T.nSurfaces, alive, aliveCount, c->smCount, st);
            if(e == cudaSuccess)
                e = mrg::multisplit_pass(P.workKeys, alive, P.workKeysOut, P.listSorted, aliveCount, R.slots, ks,
                                         P.sortHist, st);
            shadeList = P.listSorted;
        }
        if(e == cudaSuccess && overlap && depth > 0) e = cudaStreamWaitEvent(st, lane.evResolved, 0);
        if(e == cudaSuccess) e = cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), st);
        if(e == cudaSuccess)
            e = mrg::pt_shade_impl(L, P, R.T, shadeList, aliveCount, next, nextCount, c->smCount, st);
        if(e == cudaSuccess && overlap) e = cudaEventRecord(lane.evShaded, st);
        if(e == cudaSuccess && overlap) e = cudaStreamWaitEvent(side, lane.evShaded, 0);
        if(e == cudaSuccess)
            e = mrg::launch_visibility(c->scene, shadowScr, P.visBits, P.shadowRays, P.shadowList, 0, c->smCount, side,
                                       P.counts + 2);
        if(e == cudaSuccess) e = mrg::pt_resolve(L, P, R.T.lights, depth, c->smCount, side);
        if(e == cudaSuccess && overlap) e = cudaEventRecord(lane.evResolved, side);
    }
    if(e == cudaSuccess && overlap) e = cudaStreamWaitEvent(st, lane.evResolved, 0);
    return e;
}

// Passes of mrg_pt_render and mrg_pt_adjoint run two at a time
// (MRG_PT_PIPELINES=1: one).
bool pt_two_pipelines()
{
    const char* v = std::getenv("MRG_PT_PIPELINES");
    return !(v && v[0] == '1');
}

// The second pipeline: its path state, streams and events (created once),
// counters 3 and 4; it starts after the caller's earlier work on st.
mrg_status pt_lane1(mrg_ctx* c, uint32_t slots, cudaStream_t st, const PtLane& lane0, PtLane& lane1)
{
    mrg_status s = pt_paths_into(c->ptPaths2, c->ptPathMem2, slots);
    if(s != MRG_OK) return s;
    if(!c->ptStream2)
    {
        PT_TRY(cudaStreamCreateWithFlags(&c->ptStream2, cudaStreamNonBlocking), "mrg_pt: stream");
        PT_TRY(cudaStreamCreateWithFlags(&c->ptSideStream2, cudaStreamNonBlocking), "mrg_pt: stream");
        for(cudaEvent_t* q : { &c->ptEvShaded2, &c->ptEvResolved2, &c->ptEvFilm, &c->ptEvStart, &c->ptEvDone2 })
            PT_TRY(cudaEventCreateWithFlags(q, cudaEventDisableTiming), "mrg_pt: event");
    }
    const bool overlap = lane0.side != lane0.st;
    lane1 = PtLane{ &c->ptPaths2, c->ptStream2, overlap ? c->ptSideStream2 : c->ptStream2, c->ptEvShaded2,
                    c->ptEvResolved2, c->dScratch + 3, c->dScratch + (overlap ? 4 : 3) };
    PT_TRY(cudaEventRecord(c->ptEvStart, st), "mrg_pt: event");
    PT_TRY(cudaStreamWaitEvent(c->ptStream2, c->ptEvStart, 0), "mrg_pt: event wait");
    return MRG_OK;
}

// The caller's stream waits for the second pipeline.
mrg_status pt_join(mrg_ctx* c, cudaStream_t st)
{
    PT_TRY(cudaEventRecord(c->ptEvDone2, c->ptStream2), "mrg_pt: event");
    PT_TRY(cudaStreamWaitEvent(st, c->ptEvDone2, 0), "mrg_pt: event wait");
    return MRG_OK;
}

} // namespace

extern "C" {

mrg_status mrg_pt_render(mrg_ctx* c, const mrg_pt_params* p, float* dImage, void* stream)
{
    if(!c || !p || !dImage) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_render: null pointer");
    DevGuard g(c->device);
    PtRun R;
    mrg_status s = pt_setup(c, p, R, "mrg_pt_render");
    if(s != MRG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PtLane lanes[2];
    if((s = pt_lane0(c, st, lanes[0])) != MRG_OK) return s;
    // Two passes at a time: pass k runs on pipeline k mod 2 (own path state,
    // streams and counters), so one pass's casts fill the SMs the other's
    // leave idle.  Film writes stay in pass order (an event chain); the
    // caller's stream waits for both pipelines at the end.
    const uint32_t passes = p->spp / R.spp;
    const bool two = passes >= 2 && pt_two_pipelines();
    if(two && (s = pt_lane1(c, R.slots, st, lanes[0], lanes[1])) != MRG_OK) return s;
    for(uint32_t pass = 0; pass < passes; pass++)
    {
        const PtLane& lane = lanes[two ? (pass & 1u) : 0u];
        R.L.sampleBase = p->sampleStart + pass * R.spp;
        PT_TRY(pt_bounces(c, R, lane), "render pass");
        if(two && pass > 0) PT_TRY(cudaStreamWaitEvent(lane.st, c->ptEvFilm, 0), "film order");
        PT_TRY(mrg::pt_film(R.L, *lane.P, reinterpret_cast<float4*>(dImage), lane.st), "film");
        if(two) PT_TRY(cudaEventRecord(c->ptEvFilm, lane.st), "film order");
    }
    return two ? pt_join(c, st) : MRG_OK;
}

mrg_status mrg_pt_render_cached(mrg_ctx* c, const mrg_pt_params* p, float* dImage, uint32_t trainPaths,
                                float* hLoss, void* stream)
{
    if(!c || !p || !dImage) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_render_cached: null pointer");
    if(!c->cacheOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_pt_render_cached: call mrg_cache_create first");
    constexpr uint32_t kRec = 2;
    DevGuard g(c->device);
    PtRun R;
    mrg_status s = pt_setup(c, p, R, "mrg_pt_render_cached");
    if(s != MRG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // buffers: query in / out / list, per-slot training records, batch, counters
    const size_t slots = R.slots, recs = slots * kRec, cap = c->cache.cap;
    const size_t sizes[8] = { slots * 64, slots * 16, slots * 4, recs * 64, recs * 32, cap * 64, cap * 16, 64 };
    size_t need = 0;
    for(size_t z : sizes) need += (z + 255) & ~size_t(255);
    if(c->ptCacheBufBytes < need)
    {
        cudaFree(c->dPtCacheBuf);
        c->dPtCacheBuf = nullptr;
        c->ptCacheBufBytes = 0;
        PT_TRY(cudaMalloc(&c->dPtCacheBuf, need), "mrg_pt_render_cached: buffers");
        c->ptCacheBufBytes = need;
    }
    char* base = static_cast<char*>(c->dPtCacheBuf);
    size_t off = 0;
    int k = 0;
    auto take = [&]() { char* q = base + off; off += (sizes[k++] + 255) & ~size_t(255); return q; };
    mrg::PtCacheUse& C = R.L.cache;
    C.mode = 1u;
    C.recPerPath = kRec;
    C.queryIn = reinterpret_cast<float4*>(take());
    C.queryOut = reinterpret_cast<float4*>(take());
    C.queryList = reinterpret_cast<uint32_t*>(take());
    C.recIn = reinterpret_cast<float4*>(take());
    C.recAux = reinterpret_cast<float4*>(take());
    float4* batchIn = reinterpret_cast<float4*>(take());
    float4* batchTarget = reinterpret_cast<float4*>(take());
    uint32_t* counters = reinterpret_cast<uint32_t*>(take());   // [0] queries, [1] batch
    C.queryCount = counters;
    // one slot in `stride` trains, for about trainPaths training paths per pass
    C.trainStride = trainPaths ? (uint32_t)std::max<size_t>(1, slots / trainPaths) : 0u;
    C.batchCap = (uint32_t)cap;
    mrg::PtPaths& P = c->ptPaths;
    PtLane lane;
    if((s = pt_lane0(c, st, lane)) != MRG_OK) return s;
    for(uint32_t pass = 0; pass < p->spp / R.spp; pass++)
    {
        R.L.sampleBase = p->sampleStart + pass * R.spp;
        PT_TRY(cudaMemsetAsync(counters, 0, 2 * sizeof(uint32_t), st), "mrg_pt_render_cached: counters");
        if(C.trainStride) PT_TRY(cudaMemsetAsync(C.recAux, 0, sizes[4], st), "mrg_pt_render_cached: records");
        PT_TRY(pt_bounces(c, R, lane), "cached pass");
        PT_TRY(mrg::nrc_query_list(c->cache, C.queryIn, C.queryList, C.queryCount, R.slots, C.queryOut, c->smCount, st),
               "cache query");
        PT_TRY(mrg::pt_cache_apply(P, C, R.L.spec, c->smCount, st), "cache apply");
        if(C.trainStride)
        {
            PT_TRY(mrg::pt_cache_targets(P, C, R.L.spec, R.slots, batchIn, batchTarget, counters + 1, c->smCount, st),
                   "training targets");
            PT_TRY(mrg::nrc_train(c->cache, batchIn, batchTarget, counters + 1, (uint32_t)cap, c->smCount, st),
                   "cache training");
        }
        PT_TRY(mrg::pt_film(R.L, P, reinterpret_cast<float4*>(dImage), st), "film");
    }
    if(hLoss)
    {
        PT_TRY(cudaMemcpyAsync(hLoss, c->cache.loss, sizeof(float), cudaMemcpyDeviceToHost, st), "loss");
        PT_TRY(cudaStreamSynchronize(st), "mrg_pt_render_cached");
    }
    return MRG_OK;
}

mrg_status mrg_pt_adjoint(mrg_ctx* c, const mrg_pt_params* p, uint32_t texId, const float* dImageAdjoint,
                          float* dGrad, float* dGradEmission, float* dImage, void* stream)
{
    const bool texParam = texId != MRG_PT_NO_TEXTURE;
    if(!c || !p || !dImageAdjoint || (texParam && !dGrad))
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_adjoint: null pointer");
    if(!texParam && !dGradEmission)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_adjoint: no parameter (no texture and no emission gradient)");
    if(texParam && (texId >= c->ptTextures.size() || c->ptTextures[texId].format != MRG_TEX_RGBA32F))
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_adjoint: the parameter must be an f32 texture");
    if(texParam && (c->ptTextures[texId].mipRadius > 0.0f ||
                    std::any_of(c->ptTextures[texId].given.begin(), c->ptTextures[texId].given.end(),
                                [](const std::vector<uint8_t>& v) { return !v.empty(); })))
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_adjoint: the parameter texture must have no mip chain");
    if(c->ptSpec.enabled) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_adjoint: RGB rendering only");
    for(uint32_t i = 0; i < c->insts.size() && i < c->ptDesc.size(); i++)
        if(texParam && c->ptDesc[i].kind == 1 && c->ptDesc[i].texture == texId + 1 &&
           c->ptDesc[i].material != MRG_MAT_LAMBERT)
            return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_adjoint: the parameter texture must feed Lambert albedos");
    DevGuard g(c->device);
    PtRun R;
    mrg_status s = pt_setup(c, p, R, "mrg_pt_adjoint");
    if(s != MRG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if(c->ptRadTotalCap < R.slots)
    {
        cudaFree(c->dPtRadTotal);
        c->dPtRadTotal = nullptr;
        c->ptRadTotalCap = 0;
        PT_TRY(cudaMalloc(&c->dPtRadTotal, sizeof(float4) * (size_t)R.slots), "mrg_pt_adjoint: primal radiance");
        c->ptRadTotalCap = R.slots;
    }
    mrg::PtAdjoint& A = R.L.adj;
    A.delta = reinterpret_cast<const float4*>(dImageAdjoint);
    A.grad = dGrad;
    A.texIndex = texParam ? texId + 1u : 0u;
    A.gradEmission = nullptr;
    const uint32_t nInst = (uint32_t)c->insts.size();
    if(dGradEmission)
    {
        if(c->ptGradEmissionCap < nInst)
        {
            cudaFree(c->dPtGradEmission);
            c->dPtGradEmission = nullptr;
            c->ptGradEmissionCap = 0;
            PT_TRY(cudaMalloc(&c->dPtGradEmission, sizeof(double) * 4 * (size_t)nInst), "mrg_pt_adjoint: emission sums");
            c->ptGradEmissionCap = nInst;
        }
        PT_TRY(cudaMemsetAsync(c->dPtGradEmission, 0, sizeof(double) * 4 * (size_t)nInst, st), "emission sums");
        A.gradEmission = c->dPtGradEmission;
    }
    A.invSpp = 1.0f / (float)p->spp;
    // passes (primal + replay each) on two pipelines as in mrg_pt_render; the
    // gradient is a sum of atomic adds, so its value does not depend on it
    PtLane lanes[2];
    if((s = pt_lane0(c, st, lanes[0])) != MRG_OK) return s;
    const uint32_t passes = p->spp / R.spp;
    const bool two = passes >= 2 && pt_two_pipelines();
    if(two)
    {
        if(c->ptRadTotalCap2 < R.slots)
        {
            cudaFree(c->dPtRadTotal2);
            c->dPtRadTotal2 = nullptr;
            c->ptRadTotalCap2 = 0;
            PT_TRY(cudaMalloc(&c->dPtRadTotal2, sizeof(float4) * (size_t)R.slots), "mrg_pt_adjoint: primal radiance");
            c->ptRadTotalCap2 = R.slots;
        }
        if((s = pt_lane1(c, R.slots, st, lanes[0], lanes[1])) != MRG_OK) return s;
    }
    for(uint32_t pass = 0; pass < passes; pass++)
    {
        const uint32_t li = two ? (pass & 1u) : 0u;
        const PtLane& lane = lanes[li];
        float4* radTotal = static_cast<float4*>(li ? c->dPtRadTotal2 : c->dPtRadTotal);
        R.L.sampleBase = p->sampleStart + pass * R.spp;
        A.radTotal = radTotal;
        A.enabled = 0u;
        PT_TRY(pt_bounces(c, R, lane), "primal pass");
        if(dImage)
        {
            if(two && pass > 0) PT_TRY(cudaStreamWaitEvent(lane.st, c->ptEvFilm, 0), "film order");
            PT_TRY(mrg::pt_film(R.L, *lane.P, reinterpret_cast<float4*>(dImage), lane.st), "film");
            if(two) PT_TRY(cudaEventRecord(c->ptEvFilm, lane.st), "film order");
        }
        PT_TRY(cudaMemcpyAsync(radTotal, lane.P->rad, sizeof(float4) * (size_t)R.slots,
                               cudaMemcpyDeviceToDevice, lane.st), "primal radiance");
        A.enabled = 1u;
        PT_TRY(pt_bounces(c, R, lane), "replay pass");
    }
    if(two && (s = pt_join(c, st)) != MRG_OK) return s;
    if(dGradEmission)
        PT_TRY(mrg::pt_add_emission_grad(c->dPtGradEmission, dGradEmission, 4 * nInst, st), "emission gradient");
    return MRG_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Guided path tracing (GuidedPTRenderer): the hash grid, its per-slot path
// state and the bounce loop (see mrg_guide.h for the kernel order).
// ---------------------------------------------------------------------------
namespace {

uint32_t next_pow2(uint32_t v)
{
    uint32_t p = 1;
    while(p < v) p <<= 1;
    return p;
}

// HashGrid::Reset's table size: NextPowerOfTwo(uint32(entries * (1 / 0.6))).
uint32_t guide_table_size(uint32_t entryLimit)
{
    const float mult = 1.0f / 0.6f;
    return next_pow2((uint32_t)((float)entryLimit * mult));
}

// HashGrid::View (HashGrid.h:436-460) over the scene box.
void guide_view(mrg_ctx* c)
{
    mrg::GuideGrid& G = c->guide;
    const mrg_guide_params& p = c->guidePrm;
    const uint32_t base = 1u << p.posBits;
    double size[3];
    int mx = 0;
    for(int k = 0; k < 3; k++) size[k] = (double)(c->sceneBoxExact[3 + k] - c->sceneBoxExact[k]);
    for(int k = 1; k < 3; k++)
        if(size[k] > size[mx]) mx = k;
    G.baseDelta = (float)((double)base / size[mx]);
    G.baseDim = base;
    G.normalDim = 1u << p.normalBits;
    G.normalDelta = (float)G.normalDim;
    G.maxLevelOffset = p.maxLevelOffset;
    const float aperture = (3.1415926535897932384626433f / 180.0f) * p.coneAperture;   // DegToRadCoef
    G.tanConeHalfTimes2 = std::tan(aperture * 0.5f) * 2.0f;
    G.maxEntryLimit = (uint32_t)((float)(G.tableMask + 1u) * 0.6f);
    G.rmin = make_float3(c->sceneBoxExact[0], c->sceneBoxExact[1], c->sceneBoxExact[2]);
    G.lobeProb = p.lobeProbability;
    G.fixZeroWeight = p.fixZeroWeight ? 1u : 0u;
}

mrg_status guide_clear(mrg_ctx* c)
{
    const mrg::GuideGrid& G = c->guide;
    const size_t T = (size_t)G.tableMask + 1u;
    PT_TRY(cudaMemset(G.codes, 0xFF, sizeof(unsigned long long) * T), "mrg_guide: clear");
    PT_TRY(cudaMemset(G.counter, 0, sizeof(uint32_t)), "mrg_guide: clear");
    PT_TRY(cudaMemset(G.mcA, 0, sizeof(float4) * T), "mrg_guide: clear");
    PT_TRY(cudaMemset(G.mcW, 0, sizeof(float) * T), "mrg_guide: clear");
    PT_TRY(cudaMemset(G.mcN, 0, sizeof(uint32_t) * T), "mrg_guide: clear");
    PT_TRY(cudaMemset(G.irr, 0, sizeof(float2) * T), "mrg_guide: clear");
    c->guideCamSet = false;
    c->guideBkValid = false;
    return MRG_OK;
}

// Per-slot guided state for `slots` paths (one allocation, 256-byte aligned
// arrays); the record keys start empty.
mrg_status guide_paths(mrg_ctx* c, uint32_t slots)
{
    mrg::GuidePaths& Q = c->guideQ;
    uint32_t lg = 0;
    while((1u << lg) < c->guide.tableMask + 1u) lg++;
    if(c->guideCap < slots || !c->dGuidePaths)
    {
        cudaFree(c->dGuidePaths);
        c->dGuidePaths = nullptr;
        c->guideCap = 0;
        Q = mrg::GuidePaths{};
        const size_t n = slots;
        const size_t sizes[17] = { n * 4, n * 4, n * 4, n * 4, n * 8, n * 4, n * 16, n * 8, n * 8, n * 8,
                                   n * 8, n * 8, n * 8, n * 8, 4 * mrg::multisplit_hist_words(2u * slots, 8),
                                   8 * ((2 * n) / 32 + 1), 4 };
        size_t need = 0;
        for(size_t sz : sizes) need += (sz + 255) & ~size_t(255);
        char* base = nullptr;
        PT_TRY(cudaMalloc(&base, need), "mrg_pt_render_guided: path state");
        c->dGuidePaths = base;
        size_t off = 0;
        int k = 0;
        auto take = [&]() { char* q = base + off; off += (sizes[k++] + 255) & ~size_t(255); return q; };
        Q.bk = reinterpret_cast<uint32_t*>(take());
        Q.lifted = reinterpret_cast<uint32_t*>(take());
        Q.prevRefl = reinterpret_cast<float*>(take());
        Q.scoreSum = reinterpret_cast<float*>(take());
        Q.prevNormal = reinterpret_cast<float2*>(take());
        Q.shadowOut = reinterpret_cast<float*>(take());
        Q.tmpA = reinterpret_cast<float4*>(take());
        Q.tmpB = reinterpret_cast<float2*>(take());
        Q.recKey = reinterpret_cast<uint32_t*>(take());
        Q.recVal = reinterpret_cast<float*>(take());
        Q.sortKeysA = reinterpret_cast<uint32_t*>(take());
        Q.sortIdxA = reinterpret_cast<uint32_t*>(take());
        Q.sortKeysB = reinterpret_cast<uint32_t*>(take());
        Q.sortIdxB = reinterpret_cast<uint32_t*>(take());
        Q.sortHist = reinterpret_cast<uint32_t*>(take());
        Q.longRuns = reinterpret_cast<uint2*>(take());
        Q.longCount = reinterpret_cast<uint32_t*>(take());
        c->guideCap = slots;
        c->guideBkValid = false;
        // every bounce leaves the records empty again (guide_apply)
        PT_TRY(cudaMemset(Q.recKey, 0xFF, sizeof(uint32_t) * 2u * n), "mrg_pt_render_guided: records");
    }
    if(Q.slots != slots) c->guideBkValid = false;
    Q.slots = slots;
    Q.keyBits = lg + 2u;
    return MRG_OK;
}

// Backup streams: slot i starts at PermutedCG32::GenerateState of output
// width * height + i of std::mt19937(seed) (the outputs before it seed the
// pixels' main streams, as RNGGroupIndependent::Seed orders them,
// Random.cu:683-724).
mrg_status guide_backup_streams(mrg_ctx* c, const mrg_pt_params* p, uint32_t slots)
{
    if(c->guideBkValid && c->guideBkSeed == p->seed && c->guideBkW == p->width && c->guideBkH == p->height)
        return MRG_OK;
    PT_TRY(cudaDeviceSynchronize(), "mrg_pt_render_guided: earlier work");
    std::mt19937 rng(p->seed);
    rng.discard((unsigned long long)p->width * p->height);
    std::vector<uint32_t> st(slots);
    for(uint32_t i = 0; i < slots; i++)
        st[i] = ((uint32_t)rng() + mrg::kBackupPcgInc) * mrg::kBackupPcgMult + mrg::kBackupPcgInc;
    PT_TRY(cudaMemcpy(c->guideQ.bk, st.data(), sizeof(uint32_t) * slots, cudaMemcpyHostToDevice),
           "mrg_pt_render_guided: backup streams");
    c->guideBkValid = true;
    c->guideBkSeed = p->seed; c->guideBkW = p->width; c->guideBkH = p->height;
    return MRG_OK;
}

// One pass: raygen, then per bounce closest-hit cast, backprop, chain
// writes, shade, and on the side stream the shadow cast, resolve and the
// irradiance records' application.  The next bounce's backprop waits for that
// application (it reads the averages); its closest-hit cast does not.
cudaError_t guided_bounces(mrg_ctx* c, PtRun& R, const PtLane& lane)
{
    mrg::PtPaths& P = *lane.P;
    const mrg::PtLaunch& L = R.L;
    const mrg::GuideGrid& G = c->guide;
    const mrg::GuidePaths& Q = c->guideQ;
    cudaStream_t st = lane.st, side = lane.side;
    const bool overlap = side != st;
    mrg::TraceScratch closestScr = R.scr, shadowScr = R.scr;
    closestScr.workCounter = lane.closestCounter;
    shadowScr.workCounter = lane.shadowCounter;
    const size_t T = (size_t)G.tableMask + 1u;
    cudaError_t e = mrg::pt_raygen(L, P, P.listA, P.counts + 0, c->smCount, st);
    if(e == cudaSuccess) e = cudaMemsetAsync(Q.lifted, 0xFF, sizeof(uint32_t) * (size_t)R.slots, st);
    for(uint32_t depth = 0; depth < L.maxDepth && e == cudaSuccess; depth++)
    {
        uint32_t* alive = (depth & 1u) ? P.listB : P.listA;
        uint32_t* next = (depth & 1u) ? P.listA : P.listB;
        uint32_t* aliveCount = P.counts + ((depth & 1u) ? 1 : 0);
        uint32_t* nextCount = P.counts + ((depth & 1u) ? 0 : 1);
        e = cudaMemsetAsync(nextCount, 0, sizeof(uint32_t), st);
        if(e == cudaSuccess) e = cudaMemsetAsync(G.lock, 0xFF, sizeof(uint32_t) * T, st);
        if(e == cudaSuccess)
            e = mrg::launch_closest(c->scene, closestScr, P.rays, alive, 0, P.hits, P.meta, c->smCount, st, aliveCount);
        const uint32_t* shadeList = alive;
        if(e == cudaSuccess && R.partition)
        {
            mrg::DigitSpec ks;
            ks.batchShift = 0; ks.batchWidth = mrg::kPtWorkKeyBits;
            ks.digitShift = 0; ks.digitBits = mrg::kPtWorkKeyBits;
            e = mrg::pt_work_keys(P, R.T.surfaces, R.T.nSurfaces, alive, aliveCount, c->smCount, st);
            if(e == cudaSuccess)
                e = mrg::multisplit_pass(P.workKeys, alive, P.workKeysOut, P.listSorted, aliveCount, R.slots, ks,
                                         P.sortHist, st);
            shadeList = P.listSorted;
        }
        if(e == cudaSuccess && overlap && depth > 0) e = cudaStreamWaitEvent(st, lane.evResolved, 0);
        if(e == cudaSuccess) e = mrg::guide_backprop(L, P, G, Q, R.T, alive, aliveCount, c->smCount, st);
        if(e == cudaSuccess) e = mrg::guide_write_mc(P, G, Q, R.T, alive, aliveCount, c->smCount, st);
        if(e == cudaSuccess) e = cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), st);
        if(e == cudaSuccess)
            e = mrg::guide_shade(L, P, G, Q, R.T, shadeList, aliveCount, next, nextCount, c->smCount, st);
        if(e == cudaSuccess && overlap) e = cudaEventRecord(lane.evShaded, st);
        if(e == cudaSuccess && overlap) e = cudaStreamWaitEvent(side, lane.evShaded, 0);
        if(e == cudaSuccess)
            e = mrg::launch_visibility(c->scene, shadowScr, P.visBits, P.shadowRays, P.shadowList, 0, c->smCount, side,
                                       P.counts + 2);
        if(e == cudaSuccess) e = mrg::guide_resolve(P, Q, c->smCount, side);
        if(e == cudaSuccess) e = mrg::guide_apply(G, Q, c->smCount, side);
        if(e == cudaSuccess && overlap) e = cudaEventRecord(lane.evResolved, side);
    }
    if(e == cudaSuccess && overlap) e = cudaStreamWaitEvent(st, lane.evResolved, 0);
    return e;
}

} // namespace

extern "C" {

mrg_status mrg_guide_defaults(mrg_guide_params* out)
{
    if(!out) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_defaults: null pointer");
    *out = mrg_guide_params{};
    out->entryLimit = 2000000u;
    out->posBits = 14u;
    out->normalBits = 2u;
    out->maxLevelOffset = 3u;
    out->coneAperture = 0.6f;
    out->lobeProbability = 0.75f;
    return MRG_OK;
}

mrg_status mrg_guide_create(mrg_ctx* c, const mrg_guide_params* p)
{
    if(!c || !p) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_create: null pointer");
    if(!c->built) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_guide_create: call mrg_build first");
    // HashGrid::Reset's limits (HashGrid.cu:22-36): SpatioDirCode holds 3 normal
    // bits per axis and levels up to 15
    if(p->normalBits > 3u || p->posBits > 15u)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_create: normalBits > 3 or posBits > 15");
    if(p->entryLimit == 0u || p->entryLimit > (1u << 27) || !(p->lobeProbability >= 0.0f && p->lobeProbability <= 1.0f) ||
       !(p->coneAperture >= 0.0f))
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_create: entryLimit in [1, 2^27], lobeProbability "
                                                   "in [0, 1], coneAperture >= 0");
    DevGuard g(c->device);
    PT_TRY(cudaDeviceSynchronize(), "mrg_guide_create: earlier work");
    const uint32_t T = guide_table_size(p->entryLimit);
    cudaFree(c->dGuideGrid);
    c->dGuideGrid = nullptr;
    c->guideOn = false;
    const size_t t = T;
    const size_t sizes[7] = { t * 8, 256, t * 16, t * 4, t * 4, t * 4, t * 8 };
    size_t need = 0;
    for(size_t sz : sizes) need += (sz + 255) & ~size_t(255);
    char* base = nullptr;
    PT_TRY(cudaMalloc(&base, need), "mrg_guide_create: grid");
    c->dGuideGrid = base;
    size_t off = 0;
    int k = 0;
    auto take = [&]() { char* q = base + off; off += (sizes[k++] + 255) & ~size_t(255); return q; };
    mrg::GuideGrid& G = c->guide;
    G = mrg::GuideGrid{};
    G.codes = reinterpret_cast<unsigned long long*>(take());
    G.counter = reinterpret_cast<uint32_t*>(take());
    G.mcA = reinterpret_cast<float4*>(take());
    G.mcW = reinterpret_cast<float*>(take());
    G.mcN = reinterpret_cast<uint32_t*>(take());
    G.lock = reinterpret_cast<uint32_t*>(take());
    G.irr = reinterpret_cast<float2*>(take());
    G.tableMask = T - 1u;
    c->guidePrm = *p;
    guide_view(c);
    mrg_status s = guide_clear(c);
    if(s != MRG_OK) return s;
    c->guideOn = true;
    return MRG_OK;
}

mrg_status mrg_guide_clear(mrg_ctx* c)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_clear: null pointer");
    if(!c->guideOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_guide_clear: call mrg_guide_create first");
    DevGuard g(c->device);
    PT_TRY(cudaDeviceSynchronize(), "mrg_guide_clear: earlier work");
    return guide_clear(c);
}

mrg_status mrg_guide_destroy(mrg_ctx* c)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_destroy: null pointer");
    DevGuard g(c->device);
    PT_TRY(cudaDeviceSynchronize(), "mrg_guide_destroy: earlier work");
    cudaFree(c->dGuideGrid);
    cudaFree(c->dGuidePaths);
    c->dGuideGrid = nullptr;
    c->dGuidePaths = nullptr;
    c->guideCap = 0;
    c->guideQ = mrg::GuidePaths{};
    c->guide = mrg::GuideGrid{};
    c->guideOn = false;
    c->guideBkValid = false;
    return MRG_OK;
}

mrg_status mrg_guide_stats(mrg_ctx* c, uint32_t* used, uint32_t* tableSize)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_stats: null pointer");
    if(!c->guideOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_guide_stats: call mrg_guide_create first");
    DevGuard g(c->device);
    if(used) PT_TRY(cudaMemcpy(used, c->guide.counter, sizeof(uint32_t), cudaMemcpyDeviceToHost), "mrg_guide_stats");
    if(tableSize) *tableSize = c->guide.tableMask + 1u;
    return MRG_OK;
}

mrg_status mrg_guide_read(mrg_ctx* c, uint64_t* hCodes, float* hChain6, float* hIrr2)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_guide_read: null pointer");
    if(!c->guideOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_guide_read: call mrg_guide_create first");
    DevGuard g(c->device);
    const mrg::GuideGrid& G = c->guide;
    const size_t T = (size_t)G.tableMask + 1u;
    PT_TRY(cudaDeviceSynchronize(), "mrg_guide_read");
    if(hCodes) PT_TRY(cudaMemcpy(hCodes, G.codes, 8 * T, cudaMemcpyDeviceToHost), "mrg_guide_read: codes");
    if(hChain6)
    {
        std::vector<float4> a(T);
        std::vector<float> w(T);
        std::vector<uint32_t> n(T);
        PT_TRY(cudaMemcpy(a.data(), G.mcA, 16 * T, cudaMemcpyDeviceToHost), "mrg_guide_read: chains");
        PT_TRY(cudaMemcpy(w.data(), G.mcW, 4 * T, cudaMemcpyDeviceToHost), "mrg_guide_read: chains");
        PT_TRY(cudaMemcpy(n.data(), G.mcN, 4 * T, cudaMemcpyDeviceToHost), "mrg_guide_read: chains");
        for(size_t i = 0; i < T; i++)
        {
            float* o = hChain6 + 6 * i;
            o[0] = a[i].x; o[1] = a[i].y; o[2] = a[i].z; o[3] = a[i].w; o[4] = w[i]; o[5] = (float)n[i];
        }
    }
    if(hIrr2)
    {
        std::vector<float2> r(T);
        PT_TRY(cudaMemcpy(r.data(), G.irr, 8 * T, cudaMemcpyDeviceToHost), "mrg_guide_read: irradiance");
        for(size_t i = 0; i < T; i++)
        {
            uint32_t cnt;
            std::memcpy(&cnt, &r[i].y, 4);
            hIrr2[2 * i] = r[i].x;
            hIrr2[2 * i + 1] = (float)cnt;
        }
    }
    return MRG_OK;
}

mrg_status mrg_pt_render_guided(mrg_ctx* c, const mrg_pt_params* p, float* dImage, void* stream)
{
    if(!c || !p || !dImage) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_render_guided: null pointer");
    if(!c->guideOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_pt_render_guided: call mrg_guide_create first");
    if(p->sampler != MRG_PT_SAMPLER_INDEPENDENT && p->sampler != MRG_PT_SAMPLER_PCG32)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_pt_render_guided: samplers INDEPENDENT and PCG32 only");
    DevGuard g(c->device);
    PtRun R;
    mrg_status s = pt_setup(c, p, R, "mrg_pt_render_guided");
    if(s != MRG_OK) return s;
    if((s = guide_paths(c, R.slots)) != MRG_OK) return s;
    if((s = guide_backup_streams(c, p, R.slots)) != MRG_OK) return s;
    if(!c->guideCamSet)
    {
        // GenCameraPosition of the pinhole camera: its position
        c->guide.cam = make_float3(p->camPos[0], p->camPos[1], p->camPos[2]);
        c->guideCamSet = true;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PtLane lane;
    if((s = pt_lane0(c, st, lane)) != MRG_OK) return s;
    const uint32_t passes = p->spp / R.spp;
    for(uint32_t pass = 0; pass < passes; pass++)
    {
        R.L.sampleBase = p->sampleStart + pass * R.spp;
        PT_TRY(guided_bounces(c, R, lane), "guided pass");
        PT_TRY(mrg::pt_film(R.L, *lane.P, reinterpret_cast<float4*>(dImage), lane.st), "film");
    }
    return MRG_OK;
}

} // extern "C"
