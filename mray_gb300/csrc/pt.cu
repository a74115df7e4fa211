// pt.cu -- wavefront path tracer kernels (RGB or 4-wavelength spectral, NEE +
// MIS, Russian roulette).
//
// The estimator is MRay's (Source/TracerDLL/PathTracerRendererShaders.h:
// 203-300 BxDF sample + RR, 354-445 NEE, 450-517 light hits with MIS;
// Source/TracerDLL/PathTracerRenderer.cu:13-31 shadow accumulation).  The
// structure is GB300-first: one pass is
//     raygen -> [closest hit -> shade -> any hit -> resolve] x maxDepth -> film
// where every kernel is a fixed-size persistent grid that reads its work count
// from device memory, so the host enqueues a pass without a single
// synchronisation (MRay waits on the host at least four times per bounce).
// Live paths are compacted with warp ballots; NEE and the BxDF sample of a
// surface hit run in one fused shade kernel; the film is resolved per pixel
// without atomics, so images are bit-reproducible run to run.
//
// Random numbers are a counter-based hash of (seed, pixel, sample, bounce,
// dimension): no per-path RNG state is stored or advanced.
//
// Arithmetic that the CPU oracle mirrors uses the _rn intrinsics (no fused
// multiply-add), so both render the same paths up to the library's sin / cos
// / log, which differ between CUDA and the host C library by a few ulps.
#include "pt_device.cuh"

#include <algorithm>

namespace mrg {

namespace {

template<bool SPEC>
__global__ void __launch_bounds__(kPtTPB)
k_raygen(PtLaunch L, PtPaths P, uint32_t* aliveList, uint32_t* aliveCount)
{
    if(blockIdx.x == 0 && threadIdx.x == 0) *aliveCount = L.slots;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L.slots; i += gridDim.x * blockDim.x)
    {
        const uint32_t pixel = slot_pixel(L, i);
        const uint32_t x = pixel % L.width, y = pixel / L.width;
        const uint32_t key = path_key(L.seed, pixel, slot_sample(L, i));
        const float ox = gaussian_offset(rnd_s(L, key, i, 0, 6), L.filterSigma);
        const float oy = gaussian_offset(rnd_s(L, key, i, 0, 7), L.filterSigma);
        const float dx = __fdiv_rn(L.cam.planeSize[0], (float)L.width);
        const float dy = __fdiv_rn(L.cam.planeSize[1], (float)L.height);
        const float sx = mul(add((float)x, add(ox, 0.5f)), dx);
        const float sy = mul(add((float)y, add(oy, 0.5f)), dy);
        float3 d;
        d.x = sub(add(add(L.cam.bottomLeft[0], mul(sx, L.cam.right[0])), mul(sy, L.cam.up[0])), L.cam.pos[0]);
        d.y = sub(add(add(L.cam.bottomLeft[1], mul(sx, L.cam.right[1])), mul(sy, L.cam.up[1])), L.cam.pos[1]);
        d.z = sub(add(add(L.cam.bottomLeft[2], mul(sx, L.cam.right[2])), mul(sy, L.cam.up[2])), L.cam.pos[2]);
        d = normalize3(d);
        P.rays[2 * (size_t)i] = make_float4(L.cam.pos[0], L.cam.pos[1], L.cam.pos[2], L.cam.nearT);
        P.rays[2 * (size_t)i + 1] = make_float4(d.x, d.y, d.z, L.cam.farT);
        P.hits[i].x = kMissMark;
        P.thr[i] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        P.cone[i] = make_float2(L.coneAperture, 0.0f);     // CameraPinhole: RT Gems I ch. 20 eq. 30
        P.rad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        P.prevPdf[i] = 0.0f;
        P.state[i] = 0u;
        if(SPEC)
        {
            float4 w, p;
            sample_waves(rnd_s(L, key, i, 0, 9), w, p);
            P.waves[i] = w;
            P.wavePdf[i] = p;
        }
        aliveList[i] = i;
    }
}

// ---------------------------------------------------------------------------
// Shade: light hits (emission with MIS), misses (skysphere with MIS), surface
// hits (NEE + BxDF sample + Russian roulette).  Live paths and shadow rays
// are appended to their lists with one atomic per warp.  NC colour channels:
// 3 (RGB) or 4 (wavelengths).
// ---------------------------------------------------------------------------

template<bool SPEC, bool ADJ, int CM>
__global__ void __launch_bounds__(kPtTPB)
k_shade(PtLaunch L, PtPaths P, PtSceneTables T,
        const uint32_t* __restrict__ aliveList, const uint32_t* __restrict__ aliveCount,
        uint32_t* nextList, uint32_t* nextCount)
{
    constexpr int NC = SPEC ? 4 : 3;
    const PtSurface* __restrict__ surfaces = T.surfaces;
    const uint32_t nSurfaces = T.nSurfaces;
    const PtLight* __restrict__ lights = T.lights;
    const float4* __restrict__ tris = T.tris;
    const uint32_t nTris = T.nTris;
    const uint32_t n = *aliveCount;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t nAll = L.nLights + (L.env.enabled ? 1u : 0u);
    const float invN = nAll ? __fdiv_rn(1.0f, (float)nAll) : 0.0f;
    EmisRun emis{ kNoEmission, 0.0f, 0.0f, 0.0f };
    // warp-uniform trip count so every lane reaches the ballots
    const uint32_t first = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    for(uint32_t base = first; base < n; base += stride)
    {
        const uint32_t idx = base + (threadIdx.x & 31u);
        bool alive = false, shadow = false, query = false;
        uint32_t i = 0;
        if(idx < n)
        {
            i = aliveList[idx];
            const uint4 hk = P.hits[i];
            uint32_t st = P.state[i];
            uint32_t depth = st & 0xFFu;
            uint32_t type = (st >> 8) & 3u;
            const uint32_t key = path_key(L.seed, slot_pixel(L, i), slot_sample(L, i));
            const uint32_t surfIdx = hk.z & 0x00FFFFFFu;
            const float4 waves = SPEC ? P.waves[i] : make_float4(0, 0, 0, 0);
            if(hk.x != kMissMark && surfIdx < nSurfaces)
            {
                const float4 r0 = P.rays[2 * (size_t)i], r1 = P.rays[2 * (size_t)i + 1];
                const float3 org = f3(r0), dir = f3(r1);
                PtSurface sf = surfaces[surfIdx];
                const uint32_t gprim = hk.x;
                const uint32_t localPrim = gprim - sf.info.z;
                const float2 mh = P.meta[i];
                const float bu = mh.y;
                const float bv = sub(sub(1.0f, mh.x), mh.y);
                float4 v0 = make_float4(0, 0, 0, 0), e0 = v0, e1 = v0;
                if(gprim < nTris)
                {
                    v0 = tris[3 * (size_t)gprim]; e0 = tris[3 * (size_t)gprim + 1]; e1 = tris[3 * (size_t)gprim + 2];
                }
                const float3 pl = make_float3(add(add(v0.x, mul(e0.x, bu)), mul(e1.x, bv)),
                                              add(add(v0.y, mul(e0.y, bu)), mul(e1.y, bv)),
                                              add(add(v0.z, mul(e0.z, bu)), mul(e1.z, bv)));
                float3 pos;
                pos.x = add(add(add(mul(sf.m[0].x, pl.x), mul(sf.m[0].y, pl.y)), mul(sf.m[0].z, pl.z)), sf.m[0].w);
                pos.y = add(add(add(mul(sf.m[1].x, pl.x), mul(sf.m[1].y, pl.y)), mul(sf.m[1].z, pl.z)), sf.m[1].w);
                pos.z = add(add(add(mul(sf.m[2].x, pl.x), mul(sf.m[2].y, pl.y)), mul(sf.m[2].z, pl.z)), sf.m[2].w);
                const float3 nl = cross3(f3(e0), f3(e1));
                float3 gn;
                gn.x = add(add(mul(sf.inv[0].x, nl.x), mul(sf.inv[1].x, nl.y)), mul(sf.inv[2].x, nl.z));
                gn.y = add(add(mul(sf.inv[0].y, nl.x), mul(sf.inv[1].y, nl.y)), mul(sf.inv[2].y, nl.z));
                gn.z = add(add(mul(sf.inv[0].z, nl.x), mul(sf.inv[1].z, nl.y)), mul(sf.inv[2].z, nl.z));
                gn = normalize3(gn);
                Chan thr = chan(P.thr[i]);
                const float prevPdf = P.prevPdf[i];
                Chan rad = chan(P.rad[i]);

                if(sf.info.x)
                {
                    // ---- light hit (LightWorkFunction[WithNEE]) ----
                    const PtLight lt = lights[sf.info.y + localPrim];
                    const bool neeOnly = (L.sampleMode == 1u && type == 1u);
                    if(!neeOnly)
                    {
                        Chan tp = thr;
                        if(L.sampleMode == 2u && type == 1u)
                        {
                            const float lpdf = area_light_pdf(lt, mh, org, dir, invN);
                            tp = mis_weighted<NC>(tp, prevPdf, lpdf);
                        }
                        const float3 wo = make_float3(-dir.x, -dir.y, -dir.z);
                        const bool emits = (lt.n.w != 0.0f) || (dot3(f3(lt.n), wo) > 0.0f);
                        if(emits && depth + 1u <= L.maxDepth)
                        {
                            const Chan lr = radiance_of<SPEC>(L.spec, lt.radiance.x, lt.radiance.y, lt.radiance.z, waves);
#pragma unroll
                            for(int k = 0; k < NC; k++) rad.v[k] = add(rad.v[k], mul(lr.v[k], tp.v[k]));
                            if(ADJ && L.adj.gradEmission)
                            {
                                // the emission enters linearly: d(contribution) / d(radiance) = tp
                                const float4 d = L.adj.delta[slot_pixel(L, i)];
                                const float sc = L.adj.invSpp;
                                emis_push(emis, L.adj.gradEmission, __float_as_uint(lt.p1.w),
                                          mul(mul(d.x, sc), tp.v[0]), mul(mul(d.y, sc), tp.v[1]),
                                          mul(mul(d.z, sc), tp.v[2]));
                            }
                        }
                    }
                }
                else
                {
                    // GenerateSurface flips the normal towards the ray
                    // (PrimitiveDefaultTriangle.hpp:480-486).
                    const bool backSide = dot3(gn, dir) > 0.0f;
                    if(backSide) gn = make_float3(-gn.x, -gn.y, -gn.z);
                    const float3 nrm = gn;
                    float3 tng, btg;
                    onb(nrm, tng, btg);
                    const float3 wo = make_float3(-dir.x, -dir.y, -dir.z);
                    const float3 V = make_float3(dot3(wo, tng), dot3(wo, btg), dot3(wo, nrm));
                    const float2 cn = P.cone[i];
                    const Cone cone = cone_advance(Cone{ cn.x, cn.y }, r1.w);
                    const float3 a3 = surface_albedo_cone(T, sf, gprim, mh, pos, nrm, dir, cone);
                    unreal_params_cone(T, sf, gprim, mh, pos, nrm, dir, cone);
                    const Chan alb = albedo_of<SPEC>(L.spec, a3.x, a3.y, a3.z, waves);
                    if(ADJ && L.adj.texIndex != 0u && sf.tex.x == L.adj.texIndex && sf.info.w == kMatLambert &&
                       T.uvs != nullptr && gprim < nTris)
                        adjoint_vertex(L, T, sf, i, gprim, mh, a3, rad);
                    const bool isSpec = specularity<NC>(sf, alb) >= kSpecularThreshold;
                    const uint32_t mt = sf.info.w;
                    const float crough = (mt == kMatLambert) ? 1.0f : ((mt == kMatUnreal) ? sf.albedo.w : 0.0f);
                    const bool trainer = (CM == 1) && training_path(L.cache, i, L.sampleBase);
                    if(trainer && depth >= 1u && depth <= L.cache.recPerPath)
                    {
                        const size_t rec = (size_t)i * L.cache.recPerPath + (depth - 1u);
                        cache_inputs(L.cache.recIn + 4 * rec, pos, crough, wo, nrm, a3);
                        // throughput and radiance so far: RGB (w = 1 marks the record),
                        // or the 4 wavelengths (a zero marks nothing to learn from)
                        L.cache.recAux[2 * rec] = make_float4(thr.v[0], thr.v[1], thr.v[2], SPEC ? thr.v[3] : 1.0f);
                        L.cache.recAux[2 * rec + 1] = make_float4(rad.v[0], rad.v[1], rad.v[2], SPEC ? rad.v[3] : 0.0f);
                    }
                    const bool terminal = (CM == 1) && depth == (trainer ? L.cache.recPerPath + 1u : 1u);
                    if(terminal)
                    {
                        // the cache stands for the rest of the path
                        cache_inputs(L.cache.queryIn + 4 * (size_t)i, pos, crough, wo, nrm, a3);
                        query = true;
                    }
                    else
                    {
                    // ---- NEE (WorkFunctionNEE); specular materials cast none ----
                    if(L.sampleMode != 0u && nAll > 0u && !isSpec && depth + 2u <= L.maxDepth)
                    {
                        uint32_t li;
                        float3 lp;
                        Chan emis;
                        float lightPdf;
                        nee_light<SPEC, NC>(L, lights, key, i, depth, nAll, invN, pos, waves, li, lp, emis, lightPdf);
                        const float3 sdir = normalize3(make_float3(sub(lp.x, pos.x), sub(lp.y, pos.y), sub(lp.z, pos.z)));
                        const float3 lpn = nudge(lp, make_float3(-sdir.x, -sdir.y, -sdir.z));
                        const float3 seg = make_float3(sub(lpn.x, pos.x), sub(lpn.y, pos.y), sub(lpn.z, pos.z));
                        const float length = __fsqrt_rn(dot3(seg, seg));
                        const float3 Ls = make_float3(dot3(sdir, tng), dot3(sdir, btg), dot3(sdir, nrm));
                        float bpdf;
                        const Chan refl = eval_material<NC>(sf, mt, alb, V, Ls, bpdf);
                        const float pdf = (L.sampleMode == 2u) ? add(bpdf, lightPdf) : lightPdf;
                        Chan srad = chan(0, 0, 0, 0);
                        if(pdf != 0.0f)
                        {
                            const float inv = __fdiv_rn(1.0f, pdf);
#pragma unroll
                            for(int k = 0; k < NC; k++) srad.v[k] = mul(mul(mul(thr.v[k], refl.v[k]), emis.v[k]), inv);
                        }
                        const float3 so = nudge(pos, nrm);
                        P.shadowRays[2 * (size_t)i] = make_float4(so.x, so.y, so.z, 1.0e-5f);
                        P.shadowRays[2 * (size_t)i + 1] = make_float4(sdir.x, sdir.y, sdir.z,
                                                                      mul(length, sub(1.0f, 1.0e-4f)));
                        P.shadowRad[i] = f4(srad);
                        if(ADJ) P.shadowLight[i] = (li < L.nLights) ? li : 0xFFFFFFFFu;
                        shadow = true;
                    }
                    // ---- BxDF sample + Russian roulette (WorkFunction) ----
                    float3 Ll;
                    Chan refl;
                    float bpdf;
                    bool passed;
                    float3 pre;
                    sample_material<NC>(L, key, i, depth, sf, mt, alb, V, backSide, pos, nrm, Ll, refl, bpdf, passed, pre);
                    float3 wi = make_float3(add(add(mul(tng.x, Ll.x), mul(btg.x, Ll.y)), mul(nrm.x, Ll.z)),
                                            add(add(mul(tng.y, Ll.x), mul(btg.y, Ll.y)), mul(nrm.y, Ll.z)),
                                            add(add(mul(tng.z, Ll.x), mul(btg.z, Ll.y)), mul(nrm.z, Ll.z)));
                    wi = normalize3(wi);
#pragma unroll
                    for(int k = 0; k < NC; k++) thr.v[k] = mul(thr.v[k], refl.v[k]);
                    depth += 1u;
                    bool dead = depth >= L.maxDepth;
                    if(!dead && depth >= L.rrStart && !isSpec)
                    {
                        // throughput.Sum() * ChannelCountInv (PathTracerRendererShaders.h:250-256)
                        float pr = add(add(thr.v[0], thr.v[1]), thr.v[2]);
                        pr = (NC == 4) ? mul(add(pr, thr.v[3]), 0.25f) : mul(pr, 0.33333333f);
                        pr = fminf(fmaxf(pr, 0.1f), 1.0f);
                        const float xr = rnd_s(L, key, i, depth - 1u, 8);
                        if(xr >= pr) dead = true;
                        else
                        {
                            const float inv = __fdiv_rn(1.0f, pr);
#pragma unroll
                            for(int k = 0; k < NC; k++) thr.v[k] = mul(thr.v[k], inv);
                        }
                    }
                    type = isSpec ? 2u : 1u;
                    if(!dead)
                    {
                        if(bpdf == 0.0f) thr = chan(0, 0, 0, 0);
                        else
                        {
                            const float inv = __fdiv_rn(1.0f, bpdf);
#pragma unroll
                            for(int k = 0; k < NC; k++) thr.v[k] = mul(thr.v[k], inv);
                        }
                        const float3 nn = passed ? make_float3(-nrm.x, -nrm.y, -nrm.z) : nrm;
                        const float3 no = nudge(pre, nn);
                        P.rays[2 * (size_t)i] = make_float4(no.x, no.y, no.z, 1.0e-4f);
                        P.rays[2 * (size_t)i + 1] = make_float4(wi.x, wi.y, wi.z, 3.402823466e+38f);
                        const Cone co = cone_after_scatter(sf, mt, backSide, cone, wo, nrm, wi);
                        P.cone[i] = make_float2(co.aperture, co.width);
                        P.hits[i].x = kMissMark;
                        P.thr[i] = f4(thr);
                        P.prevPdf[i] = bpdf;
                        P.state[i] = depth | (type << 8);
                        alive = true;
                    }
                    }   // not terminal
                }
                P.rad[i] = f4(rad);
            }
            else if(hk.x == kMissMark && L.env.enabled)
            {
                // ---- miss: skysphere emission (LightWorkFunction[WithNEE]) ----
                const bool neeOnly = (L.sampleMode == 1u && type == 1u);
                if(!neeOnly && depth + 1u <= L.maxDepth)
                {
                    const float3 dir = f3(P.rays[2 * (size_t)i + 1]);
                    Chan tp = chan(P.thr[i]);
                    Chan rad = chan(P.rad[i]);
                    if(L.sampleMode == 2u && type == 1u)
                        tp = mis_weighted<NC>(tp, P.prevPdf[i], mul(env_pdf(L.env, dir), invN));
                    const float3 er = env_emit(L.env, dir);
                    const Chan em = radiance_of<SPEC>(L.spec, er.x, er.y, er.z, waves);
#pragma unroll
                    for(int k = 0; k < NC; k++) rad.v[k] = add(rad.v[k], mul(em.v[k], tp.v[k]));
                    P.rad[i] = f4(rad);
                }
            }
        }
        warp_append(alive, i, nextList, nextCount);
        warp_append(shadow, i, P.shadowList, P.counts + 2);
        if(CM == 1) warp_append(query, i, L.cache.queryList, L.cache.queryCount);
    }
    if(ADJ && L.adj.gradEmission) emis_flush(emis, L.adj.gradEmission);
}

// The cache's RGB radiance, times the path's throughput, ends the path.  A
// spectral path takes it at its 4 wavelengths through the radiance
// conversion that emission uses.
template<bool SPEC>
__global__ void __launch_bounds__(kPtTPB)
k_cache_apply(PtPaths P, PtCacheUse C, PtSpectral S)
{
    const uint32_t n = *C.queryCount;
    for(uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const uint32_t i = C.queryList[k];
        const float4 q = C.queryOut[i], t = P.thr[i];
        float4 r = P.rad[i];
        const Chan lc = radiance_of<SPEC>(S, fmaxf(q.x, 0.0f), fmaxf(q.y, 0.0f), fmaxf(q.z, 0.0f),
                                          SPEC ? P.waves[i] : make_float4(0, 0, 0, 0));
        r.x = add(r.x, mul(t.x, lc.v[0]));
        r.y = add(r.y, mul(t.y, lc.v[1]));
        r.z = add(r.z, mul(t.z, lc.v[2]));
        if(SPEC) r.w = add(r.w, mul(t.w, lc.v[3]));
        P.rad[i] = r;
    }
}

// Training targets: the radiance the path gathered after a recorded vertex,
// over the throughput up to it.  A spectral path's 4-wavelength estimate is
// turned into RGB as the film turns a sample (divided by the wavelength
// pdfs, through the observer), an unbiased RGB target.
template<bool SPEC>
__global__ void __launch_bounds__(kPtTPB)
k_cache_targets(PtPaths P, PtCacheUse C, PtSpectral S, uint32_t paths, float4* batchIn, float4* batchTarget,
                uint32_t* batchCount)
{
    const uint32_t total = paths * C.recPerPath;
    const uint32_t first = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    for(uint32_t base = first; base < total; base += gridDim.x * blockDim.x)
    {
        const uint32_t r = base + (threadIdx.x & 31u);
        bool ok = false;
        float4 tgt = make_float4(0, 0, 0, 0);
        if(r < total)
        {
            const float4 th = C.recAux[2 * (size_t)r], before = C.recAux[2 * (size_t)r + 1];
            if(th.w > 0.0f && th.x > 0.0f && th.y > 0.0f && th.z > 0.0f)
            {
                const uint32_t path = r / C.recPerPath;
                const float4 tot = P.rad[path];
                tgt = make_float4(__fdiv_rn(sub(tot.x, before.x), th.x), __fdiv_rn(sub(tot.y, before.y), th.y),
                                  __fdiv_rn(sub(tot.z, before.z), th.z), 0.0f);
                if(SPEC)
                {
                    tgt.w = __fdiv_rn(sub(tot.w, before.w), th.w);
                    const float3 rgb = spectrum_to_rgb(S, tgt, P.waves[path], P.wavePdf[path]);
                    tgt = make_float4(rgb.x, rgb.y, rgb.z, 0.0f);
                }
                ok = isfinite(tgt.x) && isfinite(tgt.y) && isfinite(tgt.z);
            }
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        if(m == 0u) continue;
        const uint32_t lane = threadIdx.x & 31u;
        const int leader = __ffs(m) - 1;
        uint32_t b = 0;
        if((int)lane == leader) b = atomicAdd(batchCount, (uint32_t)__popc(m));
        b = __shfl_sync(0xFFFFFFFFu, b, leader);
        if(ok)
        {
            const uint32_t o = b + __popc(m & ((1u << lane) - 1u));
            if(o < C.batchCap)
            {
                for(int j = 0; j < 4; j++) batchIn[4 * (size_t)o + j] = C.recIn[4 * (size_t)r + j];
                batchTarget[o] = tgt;
            }
        }
    }
}

// Work key of every alive path (KCGenerateSurfaceWorkKeysIndirect,
// RendererCommon.h:14): 0 miss (boundary light), 1 area light, 2 + material
// group.
__global__ void __launch_bounds__(kPtTPB)
k_work_keys(PtPaths P, const PtSurface* __restrict__ surfaces, uint32_t nSurfaces,
            const uint32_t* __restrict__ aliveList, const uint32_t* __restrict__ aliveCount)
{
    const uint32_t n = *aliveCount;
    for(uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const uint4 hk = P.hits[aliveList[k]];
        const uint32_t s = hk.z & 0x00FFFFFFu;
        uint32_t key = 0u;
        if(hk.x != kMissMark && s < nSurfaces)
        {
            const uint4 info = surfaces[s].info;
            key = info.x ? 1u : 2u + min(info.w, 5u);
        }
        P.workKeys[k] = key;
    }
}

// Adds the radiance of every shadow ray that reached its light
// (KCAccumulateShadowRaysPT; the depth limit was applied when it was cast).
// Resolve: visible NEE samples add their radiance.  In an adjoint replay with
// emission gradients (ADJ) each also adds delta / spp * (its radiance / the
// light's radiance), its derivative by the light's radiance, to the light's
// instance.
template<bool ADJ>
__global__ void __launch_bounds__(kPtTPB)
k_resolve(PtPaths P, PtLaunch L, const PtLight* __restrict__ lights)
{
    const uint32_t n = P.counts[2];
    EmisRun emis{ kNoEmission, 0.0f, 0.0f, 0.0f };
    for(uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const uint32_t i = P.shadowList[k];
        if((P.visBits[i >> 5] >> (i & 31u)) & 1u)
        {
            const float4 s = P.shadowRad[i];
            float4 r = P.rad[i];
            r.x = add(r.x, s.x); r.y = add(r.y, s.y); r.z = add(r.z, s.z); r.w = add(r.w, s.w);
            P.rad[i] = r;
            if(ADJ)
            {
                const uint32_t li = P.shadowLight[i];
                if(li < L.nLights)
                {
                    const PtLight lt = lights[li];
                    const float4 d = L.adj.delta[slot_pixel(L, i)];
                    const float sc = L.adj.invSpp;
                    emis_push(emis, L.adj.gradEmission, __float_as_uint(lt.p1.w),
                        (lt.radiance.x > 0.0f) ? mul(mul(d.x, sc), __fdiv_rn(s.x, lt.radiance.x)) : 0.0f,
                        (lt.radiance.y > 0.0f) ? mul(mul(d.y, sc), __fdiv_rn(s.y, lt.radiance.y)) : 0.0f,
                        (lt.radiance.z > 0.0f) ? mul(mul(d.z, sc), __fdiv_rn(s.z, lt.radiance.z)) : 0.0f);
                }
            }
        }
    }
    if(ADJ) emis_flush(emis, L.adj.gradEmission);
}

// Film: every pixel sums its samples of the pass (slots p, p + WH, ...);
// spectral samples are converted to RGB first (KCConvertSpectrumToRGBIndirect).
template<bool SPEC>
__global__ void __launch_bounds__(kPtTPB)
k_film(PtLaunch L, PtPaths P, float4* __restrict__ image)
{
    const uint32_t wh = L.width * L.height;
    for(uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < wh; p += gridDim.x * blockDim.x)
    {
        float4 acc = image[p];
        for(uint32_t k = 0; k < L.samplesPerPass; k++)
        {
            const size_t slot = p + (size_t)k * wh;
            const float4 r = P.rad[slot];
            const float3 c = SPEC ? spectrum_to_rgb(L.spec, r, P.waves[slot], P.wavePdf[slot]) : f3(r);
            acc.x = add(acc.x, c.x); acc.y = add(acc.y, c.y); acc.z = add(acc.z, c.z);
            acc.w = add(acc.w, 1.0f);
        }
        image[p] = acc;
    }
}

inline unsigned grid_for(uint32_t n, int smCount)
{
    const uint32_t want = (n + kPtTPB - 1) / kPtTPB;
    const uint32_t cap = (uint32_t)smCount * 8u;
    return (unsigned)(want < cap ? (want ? want : 1u) : cap);
}

// One level of a mip chain from the one above it (KCGenerateMipmaps with
// FilterPixel in ACCUMULATE mode, TextureFilter.cu:62-110, 124-192): per
// texel the 8 x 8 weighted samples of the parent, each the parent texel
// nearest to ConvertPixelIndices of the sample point (GraphicsFunctions.h:
// 527-538), summed in row order and divided by the weight sum.  Texels are
// read as stored (UNORM8 as 0..255, GenericRead) and written back rounded and
// clamped (GenericWrite).
__global__ void __launch_bounds__(kPtTPB)
k_gen_mip(const void* __restrict__ src, void* __restrict__ dst, uint32_t format, uint32_t pw, uint32_t ph, uint32_t w,
          uint32_t h, MipTaps taps)
{
    const float rx = __fdiv_rn((float)pw, (float)w), ry = __fdiv_rn((float)ph, (float)h);
    const uint32_t n = w * h;
    for(uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x)
    {
        const uint32_t x = idx % w, y = idx / w;
        float acc[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
        float wsum = 0.0f;
        for(int sy = 0; sy < 8; sy++)
        {
            float py = sub(mul(add(add((float)y, taps.off[sy]), 0.5f), ry), 0.5f);
            py = fminf(fmaxf(0.0f, py), (float)(ph - 1u));
            const uint32_t iy = (uint32_t)lroundf(py);
            for(int sx = 0; sx < 8; sx++)
            {
                float px = sub(mul(add(add((float)x, taps.off[sx]), 0.5f), rx), 0.5f);
                px = fminf(fmaxf(0.0f, px), (float)(pw - 1u));
                const uint32_t ix = (uint32_t)lroundf(px);
                const float wgt = mul(taps.g[sx], taps.g[sy]);
                const size_t t = (size_t)iy * pw + ix;
                float v[4];
                if(format == 0u)
                {
                    const uchar4 c = reinterpret_cast<const uchar4*>(src)[t];
                    v[0] = (float)c.x; v[1] = (float)c.y; v[2] = (float)c.z; v[3] = (float)c.w;
                }
                else
                {
                    const float4 c = reinterpret_cast<const float4*>(src)[t];
                    v[0] = c.x; v[1] = c.y; v[2] = c.z; v[3] = c.w;
                }
#pragma unroll
                for(int k = 0; k < 4; k++) acc[k] = add(acc[k], mul(wgt, v[k]));
                wsum = add(wsum, wgt);
            }
        }
        float o[4];
#pragma unroll
        for(int k = 0; k < 4; k++) o[k] = __fdiv_rn(acc[k], wsum);
        if(format == 0u)
        {
            uchar4 c;
            c.x = (unsigned char)fminf(fmaxf(roundf(o[0]), 0.0f), 255.0f);
            c.y = (unsigned char)fminf(fmaxf(roundf(o[1]), 0.0f), 255.0f);
            c.z = (unsigned char)fminf(fmaxf(roundf(o[2]), 0.0f), 255.0f);
            c.w = (unsigned char)fminf(fmaxf(roundf(o[3]), 0.0f), 255.0f);
            reinterpret_cast<uchar4*>(dst)[idx] = c;
        }
        else reinterpret_cast<float4*>(dst)[idx] = make_float4(o[0], o[1], o[2], o[3]);
    }
}

} // namespace

cudaError_t generate_mips(const void* texels, void* mips, uint32_t w, uint32_t h, uint32_t format, const MipTaps& taps,
                          uint32_t levels, uint32_t validMask)
{
    const size_t bpp = (format == 0u) ? 4u : 16u;
    char* chain = static_cast<char*>(mips);
    for(uint32_t m = 1; m < levels; m++)
    {
        if(validMask & (1u << m)) continue;
        const uint32_t pw = (w >> (m - 1)) ? (w >> (m - 1)) : 1u, ph = (h >> (m - 1)) ? (h >> (m - 1)) : 1u;
        const uint32_t cw = (w >> m) ? (w >> m) : 1u, ch = (h >> m) ? (h >> m) : 1u;
        const uint32_t n = cw * ch;
        const void* src = (m == 1) ? texels : chain + mip_chain_texels(w, h, m - 1) * bpp;
        void* out = chain + mip_chain_texels(w, h, m) * bpp;
        k_gen_mip<<<std::min<uint32_t>((n + kPtTPB - 1) / kPtTPB, 65535u), kPtTPB>>>(src, out, format, pw, ph, cw, ch,
                                                                                    taps);
        cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess) return e;
    }
    return cudaDeviceSynchronize();
}

cudaError_t pt_raygen(const PtLaunch& L, const PtPaths& P, uint32_t* aliveList, uint32_t* aliveCount,
                      int smCount, cudaStream_t st)
{
    if(L.spec.enabled) k_raygen<true><<<grid_for(L.slots, smCount), kPtTPB, 0, st>>>(L, P, aliveList, aliveCount);
    else k_raygen<false><<<grid_for(L.slots, smCount), kPtTPB, 0, st>>>(L, P, aliveList, aliveCount);
    return cudaGetLastError();
}

cudaError_t pt_shade_impl(const PtLaunch& L, const PtPaths& P, const PtSceneTables& T,
                          const uint32_t* aliveList, const uint32_t* aliveCount,
                          uint32_t* nextList, uint32_t* nextCount, int smCount, cudaStream_t st)
{
    const unsigned grid = (unsigned)smCount * 8u;
    if(L.cache.mode == 1u && L.spec.enabled)
        k_shade<true, false, 1><<<grid, kPtTPB, 0, st>>>(L, P, T, aliveList, aliveCount, nextList, nextCount);
    else if(L.cache.mode == 1u)
        k_shade<false, false, 1><<<grid, kPtTPB, 0, st>>>(L, P, T, aliveList, aliveCount, nextList, nextCount);
    else if(L.adj.enabled)
        k_shade<false, true, 0><<<grid, kPtTPB, 0, st>>>(L, P, T, aliveList, aliveCount, nextList, nextCount);
    else if(L.spec.enabled)
        k_shade<true, false, 0><<<grid, kPtTPB, 0, st>>>(L, P, T, aliveList, aliveCount, nextList, nextCount);
    else
        k_shade<false, false, 0><<<grid, kPtTPB, 0, st>>>(L, P, T, aliveList, aliveCount, nextList, nextCount);
    return cudaGetLastError();
}

cudaError_t pt_work_keys(const PtPaths& P, const PtSurface* surfaces, uint32_t nSurfaces,
                         const uint32_t* aliveList, const uint32_t* aliveCount, int smCount, cudaStream_t st)
{
    k_work_keys<<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, surfaces, nSurfaces, aliveList, aliveCount);
    return cudaGetLastError();
}

cudaError_t pt_cache_apply(const PtPaths& P, const PtCacheUse& C, const PtSpectral& S, int smCount,
                           cudaStream_t st)
{
    if(S.enabled) k_cache_apply<true><<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, C, S);
    else k_cache_apply<false><<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, C, S);
    return cudaGetLastError();
}

cudaError_t pt_cache_targets(const PtPaths& P, const PtCacheUse& C, const PtSpectral& S, uint32_t slots,
                             float4* batchIn, float4* batchTarget, uint32_t* batchCount, int smCount,
                             cudaStream_t st)
{
    if(S.enabled)
        k_cache_targets<true><<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, C, S, slots, batchIn, batchTarget,
                                                                           batchCount);
    else
        k_cache_targets<false><<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, C, S, slots, batchIn, batchTarget,
                                                                            batchCount);
    return cudaGetLastError();
}

cudaError_t pt_add_emission_grad(const double* acc, float* out, uint32_t n, cudaStream_t st)
{
    if(n == 0) return cudaSuccess;
    k_add_emission_grad<<<(n + 255u) / 256u, 256, 0, st>>>(acc, out, n);
    return cudaGetLastError();
}

cudaError_t pt_resolve(const PtLaunch& L, const PtPaths& P, const PtLight* lights, uint32_t, int smCount,
                       cudaStream_t st)
{
    if(L.adj.enabled && L.adj.gradEmission) k_resolve<true><<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, L, lights);
    else k_resolve<false><<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, L, lights);
    return cudaGetLastError();
}

cudaError_t pt_film(const PtLaunch& L, const PtPaths& P, float4* image, cudaStream_t st)
{
    if(L.spec.enabled) k_film<true><<<grid_for(L.width * L.height, 152), kPtTPB, 0, st>>>(L, P, image);
    else k_film<false><<<grid_for(L.width * L.height, 152), kPtTPB, 0, st>>>(L, P, image);
    return cudaGetLastError();
}

} // namespace mrg
