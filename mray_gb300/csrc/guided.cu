// guided.cu -- guided path tracing kernels (MRay's GuidedPTRenderer:
// Markov-chain mixtures after Alber et al. 2025 on the spatio-directional
// hash grid), bounce by bounce in the order mrg_guide.h lays out.
//   backprop   KCBackpropagateHashGridPath     Source/TracerDLL/GuidedPTRenderer.cu:164-311
//   write MC   KCWriteMarkovChains             GuidedPTRenderer.cu:313-344
//   shade      WorkFunction::Call              Source/TracerDLL/GuidedPTRendererShaders.h:588-848
//              LightWorkFunction::Call         GuidedPTRendererShaders.h:853-931
//              GaussLobeMixtureT               GuidedPTRendererShaders.h:381-450
//   resolve    KCAccumulateShadowRaysGPT       GuidedPTRenderer.cu:13-33
//   apply      KCBackpropagateIrradNEE / Light GuidedPTRenderer.cu:346-430
// Materials, lights and the sampler are the plain path tracer's
// (pt_device.cuh).  Random numbers of bounce b: mixture or material sample
// k 0..2, light choice k 3, light point k 4, 5, Russian roulette k 8 and the
// mixture / material choice k 10; the grid's stochastic codes and choices draw
// from the slot's backup PCG32 state, as MRay's BackupRNG does.
#include "mrg_guide.h"
#include "pt_device.cuh"
#include "guide.cuh"
#include "mrg_partition.h"

namespace mrg {

namespace {

constexpr uint32_t kRnMis = 10u;
constexpr float kInf = __builtin_huge_valf();

// Surface point and geometric normal of a triangle hit (as k_shade forms them).
__device__ __forceinline__ void hit_point(const PtSceneTables& T, const PtSurface& sf, uint32_t gprim, float2 mh,
                                          float3& pos, float3& gn)
{
    const float bu = mh.y;
    const float bv = sub(sub(1.0f, mh.x), mh.y);
    float4 v0 = make_float4(0, 0, 0, 0), e0 = v0, e1 = v0;
    if(gprim < T.nTris)
    {
        v0 = T.tris[3 * (size_t)gprim]; e0 = T.tris[3 * (size_t)gprim + 1]; e1 = T.tris[3 * (size_t)gprim + 2];
    }
    const float3 pl = make_float3(add(add(v0.x, mul(e0.x, bu)), mul(e1.x, bv)),
                                  add(add(v0.y, mul(e0.y, bu)), mul(e1.y, bv)),
                                  add(add(v0.z, mul(e0.z, bu)), mul(e1.z, bv)));
    pos.x = add(add(add(mul(sf.m[0].x, pl.x), mul(sf.m[0].y, pl.y)), mul(sf.m[0].z, pl.z)), sf.m[0].w);
    pos.y = add(add(add(mul(sf.m[1].x, pl.x), mul(sf.m[1].y, pl.y)), mul(sf.m[1].z, pl.z)), sf.m[1].w);
    pos.z = add(add(add(mul(sf.m[2].x, pl.x), mul(sf.m[2].y, pl.y)), mul(sf.m[2].z, pl.z)), sf.m[2].w);
    const float3 nl = cross3(f3(e0), f3(e1));
    gn.x = add(add(mul(sf.inv[0].x, nl.x), mul(sf.inv[1].x, nl.y)), mul(sf.inv[2].x, nl.z));
    gn.y = add(add(mul(sf.inv[0].y, nl.x), mul(sf.inv[1].y, nl.y)), mul(sf.inv[2].y, nl.z));
    gn.z = add(add(mul(sf.inv[0].z, nl.x), mul(sf.inv[1].z, nl.y)), mul(sf.inv[2].z, nl.z));
    gn = normalize3(gn);
}

// A hit the light work handles: a miss (the boundary light) or an emitting
// surface (IS_LIGHT_KEY_FLAG).  Invalid surfaces end their path silently.
__device__ __forceinline__ bool light_hit(const PtSceneTables& T, const uint4& hk)
{
    if(hk.x == kMissMark) return true;
    const uint32_t s = hk.z & 0x00FFFFFFu;
    return s < T.nSurfaces && T.surfaces[s].info.x != 0u;
}

template<int NC>
__device__ __forceinline__ float chan_avg(const Chan& c)
{
    // Spectrum::Sum() * SpectrumCountInv (4 wavelengths); RGB: the 3 channels' mean
    float s = add(add(c.v[0], c.v[1]), c.v[2]);
    return (NC == 4) ? mul(add(s, c.v[3]), 0.25f) : mul(s, 0.33333333f);
}

__device__ __forceinline__ void put_record(const GuidePaths& Q, uint32_t pos, uint32_t cell, uint32_t light, float v)
{
    Q.recKey[pos] = (cell << 1) | light;
    Q.recVal[pos] = isfinite(v) ? v : 0.0f;
}

// ---------------------------------------------------------------------------
// KCBackpropagateHashGridPath: for a path that left vertex prev (its lifted
// chain) and hit a surface, the irradiance at the hit's cell times the
// reflectance stored at prev is prev's irradiance sample; the chain of prev,
// moved by its EMA towards the hit, lifts to a stochastic neighbour cell and
// competes for it (smallest slot wins).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPtTPB)
k_guide_backprop(GuideGrid G, GuidePaths Q, PtPaths P, PtSceneTables T,
                 const uint32_t* __restrict__ aliveList, const uint32_t* __restrict__ aliveCount)
{
    const uint32_t n = *aliveCount;
    for(uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const uint32_t i = aliveList[k];
        const uint4 hk = P.hits[i];
        if(light_hit(T, hk)) continue;
        if((hk.z & 0x00FFFFFFu) >= T.nSurfaces) continue;
        const uint32_t prev = Q.lifted[i];
        if(prev == guide::kInvalid) continue;
        const float4 r0 = P.rays[2 * (size_t)i], r1 = P.rays[2 * (size_t)i + 1];
        const float3 org = f3(r0), dir = f3(r1);
        const float t = r1.w;
        // Ray::AdvancedPos: pos + t * dir
        const float3 nextPos = make_float3(add(org.x, mul(t, dir.x)), add(org.y, mul(t, dir.y)),
                                           add(org.z, mul(t, dir.z)));
        const float3 wdir = normalize3(make_float3(-dir.x, -dir.y, -dir.z));
        const uint32_t loc = guide::search(G, guide::gen_code(G, nextPos, wdir));
        if(loc == guide::kInvalid) continue;
        float out = mul(Q.prevRefl[i], G.irr[loc].x);
        if(!isfinite(out)) out = 0.0f;
        put_record(Q, i, prev, 0u, out);

        uint32_t rng = Q.bk[i];
        const float score = Q.scoreSum[i];
        if(score != kInf && mul(guide::next_float(rng), score) > mul(out, (float)guide::kLobes))
        {
            Q.bk[i] = rng;
            continue;
        }
        const float2 pn = Q.prevNormal[i];
        const uint64_t mcCode = guide::gen_code_stochastic(G, org, guide::conc_octa_to_dir(pn), rng);
        Q.bk[i] = rng;
        uint32_t ni = guide::search(G, mcCode);
        if(ni == guide::kInvalid) ni = prev;
        Q.lifted[i] = ni;
        const uint32_t old = atomicMin(&G.lock[ni], i + 1u);
        if(old < i + 1u) continue;
        guide::Chain s;
        uint32_t cnt;
        if(score == kInf)
        {
            s.target = make_float3(0.0f, 0.0f, 0.0f);
            s.cosine = 0.0f;
            s.weight = 0.0f;
            cnt = 0u;
        }
        else
        {
            const float4 a = G.mcA[prev];
            s.target = f3(a);
            s.cosine = a.w;
            s.weight = G.mcW[prev];
            cnt = guide::chain_ema(s, org, nextPos, out, G.mcN[prev]);
        }
        if(!isfinite(s.cosine)) s.cosine = 0.0f;
        if(!isfinite(s.target.x) || !isfinite(s.target.y) || !isfinite(s.target.z))
            s.target = make_float3(0.0f, 0.0f, 0.0f);
        if(!isfinite(s.weight)) s.weight = 0.0f;
        Q.tmpA[i] = make_float4(s.target.x, s.target.y, s.target.z, s.cosine);
        Q.tmpB[i] = make_float2(s.weight, __uint_as_float(cnt));
    }
}

// KCWriteMarkovChains: the lock winners write the chains they carried.
__global__ void __launch_bounds__(kPtTPB)
k_guide_write_mc(GuideGrid G, GuidePaths Q, PtPaths P, PtSceneTables T,
                 const uint32_t* __restrict__ aliveList, const uint32_t* __restrict__ aliveCount)
{
    const uint32_t n = *aliveCount;
    for(uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const uint32_t i = aliveList[k];
        if(light_hit(T, P.hits[i])) continue;
        const uint32_t w = Q.lifted[i];
        if(w == guide::kInvalid) continue;
        if(G.lock[w] != i + 1u) continue;
        const float4 a = Q.tmpA[i];
        const float2 b = Q.tmpB[i];
        G.mcA[w] = a;
        G.mcW[w] = b.x;
        G.mcN[w] = __float_as_uint(b.y);
    }
}

// A thread's mixture (GaussLobeMixtureSharedT's layout idea,
// GuidedPTRendererShaders.h:191-214): per lobe its direction, kappa, alpha,
// weight, code, slot and pdf scratch, one shared-memory word per field, lobe
// and thread (thread-contiguous, so bank-conflict free).  Kept off the local
// stack, which spilled to L2 at this occupancy.
constexpr uint32_t kMixFields = 10;
constexpr size_t kMixSmem = (size_t)kMixFields * guide::kLobes * kPtTPB * sizeof(float);
enum : uint32_t { kMxDx = 0, kMxDy, kMxDz, kMxKappa, kMxAlpha, kMxW, kMxCodeLo, kMxCodeHi, kMxSlot, kMxPdf };

struct Mix
{
    float* p;
    __device__ __forceinline__ float& f(uint32_t field, uint32_t j) const
    {
        return p[(field * guide::kLobes + j) * kPtTPB + threadIdx.x];
    }
    __device__ __forceinline__ uint32_t& u(uint32_t field, uint32_t j) const
    {
        return reinterpret_cast<uint32_t&>(f(field, j));
    }
    __device__ __forceinline__ guide::Lobe lobe(uint32_t j) const
    {
        guide::Lobe l;
        l.dir = make_float3(f(kMxDx, j), f(kMxDy, j), f(kMxDz, j));
        l.kappa = f(kMxKappa, j);
        l.alpha = f(kMxAlpha, j);
        return l;
    }
    __device__ __forceinline__ void set(uint32_t j, const guide::Lobe& l, float w) const
    {
        f(kMxDx, j) = l.dir.x; f(kMxDy, j) = l.dir.y; f(kMxDz, j) = l.dir.z;
        f(kMxKappa, j) = l.kappa; f(kMxAlpha, j) = l.alpha; f(kMxW, j) = w;
    }
    __device__ __forceinline__ bool same_code(uint32_t a, uint32_t b) const
    {
        return u(kMxCodeLo, a) == u(kMxCodeLo, b) && u(kMxCodeHi, a) == u(kMxCodeHi, b);
    }
};

// GaussLobeMixtureT::Pdf; a repeated code's lobe pdf is the earlier one's.
__device__ __noinline__ float mixture_pdf(Mix m, float sumW, float3 d)
{
    if(sumW == 0.0f) return 0.0f;
    float pdf = 0.0f;
#pragma unroll 1
    for(uint32_t j = 0; j < guide::kLobes; j++)
    {
        const float w = m.f(kMxW, j);
        if(w == 0.0f) continue;
        uint32_t q = 0;
        while(q < j && !m.same_code(q, j)) q++;
        const float lp = (q < j) ? m.f(kMxPdf, q) : guide::lobe_pdf(m.lobe(j), d);
        m.f(kMxPdf, j) = lp;
        pdf = add(pdf, mul(w, lp));
    }
    return __fdiv_rn(pdf, sumW);
}

// ---------------------------------------------------------------------------
// Shade (WorkFunction / LightWorkFunction of the guided renderer).
// ---------------------------------------------------------------------------
template<bool SPEC>
__global__ void __launch_bounds__(kPtTPB)
k_shade_guided(PtLaunch L, PtPaths P, GuideGrid G, GuidePaths Q, PtSceneTables T,
               const uint32_t* __restrict__ aliveList, const uint32_t* __restrict__ aliveCount,
               uint32_t* nextList, uint32_t* nextCount)
{
    constexpr int NC = SPEC ? 4 : 3;
    extern __shared__ float gmix[];
    const PtLight* __restrict__ lights = T.lights;
    const uint32_t n = *aliveCount;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t nAll = L.nLights + (L.env.enabled ? 1u : 0u);
    const float invN = nAll ? __fdiv_rn(1.0f, (float)nAll) : 0.0f;
    const uint32_t first = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    for(uint32_t base = first; base < n; base += stride)
    {
        const uint32_t idx = base + (threadIdx.x & 31u);
        bool alive = false, shadow = false;
        uint32_t i = 0;
        if(idx < n)
        {
            i = aliveList[idx];
            const uint4 hk = P.hits[i];
            const uint32_t st = P.state[i];
            uint32_t depth = st & 0xFFu;
            const uint32_t type = (st >> 8) & 3u;
            const uint32_t key = path_key(L.seed, slot_pixel(L, i), slot_sample(L, i));
            const uint32_t surfIdx = hk.z & 0x00FFFFFFu;
            const float4 waves = SPEC ? P.waves[i] : make_float4(0, 0, 0, 0);
            const float4 r0 = P.rays[2 * (size_t)i], r1 = P.rays[2 * (size_t)i + 1];
            const float3 org = f3(r0), dir = f3(r1);
            const bool isMiss = hk.x == kMissMark;
            if(light_hit(T, hk))
            {
                // ---- LightWorkFunction: emission (MIS for path rays), the
                // light-cache radiance of the previous vertex ----
                Chan tp = chan(P.thr[i]);
                Chan rad = chan(P.rad[i]);
                float lcRefl = Q.prevRefl[i];
                float lpdf = 0.0f;
                Chan em = chan(0, 0, 0, 0);
                if(!isMiss)
                {
                    const PtSurface sf = T.surfaces[surfIdx];
                    const PtLight lt = lights[sf.info.y + (hk.x - sf.info.z)];
                    if(type == 1u) lpdf = area_light_pdf(lt, P.meta[i], org, dir, invN);
                    const float3 wo = make_float3(-dir.x, -dir.y, -dir.z);
                    const bool emits = (lt.n.w != 0.0f) || (dot3(f3(lt.n), wo) > 0.0f);
                    if(emits) em = radiance_of<SPEC>(L.spec, lt.radiance.x, lt.radiance.y, lt.radiance.z, waves);
                }
                else if(L.env.enabled)
                {
                    if(type == 1u) lpdf = mul(env_pdf(L.env, dir), invN);
                    const float3 er = env_emit(L.env, dir);
                    em = radiance_of<SPEC>(L.spec, er.x, er.y, er.z, waves);
                }
                if(type == 1u)
                {
                    const float p0 = P.prevPdf[i];
                    const float misPdf = add(p0, lpdf);
                    tp = mis_weighted<NC>(tp, p0, lpdf);
                    lcRefl = mul(lcRefl, p0);
                    lcRefl = (misPdf == 0.0f) ? 0.0f : __fdiv_rn(lcRefl, misPdf);
                }
                float lcRad = 0.0f;
                if(depth + 1u <= L.maxDepth)
                {
#pragma unroll
                    for(int k = 0; k < NC; k++) rad.v[k] = add(rad.v[k], mul(em.v[k], tp.v[k]));
                    lcRad = mul(lcRefl, chan_avg<NC>(em));
                }
                P.rad[i] = f4(rad);
                const uint32_t lm = Q.lifted[i];
                if(lm != guide::kInvalid) put_record(Q, Q.slots + i, lm, 1u, lcRad);
            }
            else if(surfIdx < T.nSurfaces)
            {
                PtSurface sf = T.surfaces[surfIdx];
                const uint32_t gprim = hk.x;
                const float2 mh = P.meta[i];
                float3 pos, gn;
                hit_point(T, sf, gprim, mh, pos, gn);
                Chan thr = chan(P.thr[i]);
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
                const float specv = specularity<NC>(sf, alb);
                const bool isSpec = specv >= kSpecularThreshold;
                const uint32_t mt = sf.info.w;
                const float3 woW = normalize3(wo);

                // ---- GaussLobeMixtureT::LoadStochastic ----
                // A code drawn again gives the slot and lobe it gave before
                // (nothing writes chains while paths shade), so repeats reuse them.
                const Mix mx{ gmix };
                float sumW = 0.0f;
                uint32_t sIdx = guide::kInvalid;
                uint32_t rng = Q.bk[i];
                const float3 codeN = normalize3(woW);
                const guide::CodeBase cb = guide::code_base(G, pos, codeN);
#pragma unroll 1
                for(uint32_t j = 0; j < guide::kLobes; j++)
                {
                    const uint64_t code = guide::gen_code_stochastic(G, cb, pos, rng);
                    mx.u(kMxCodeLo, j) = (uint32_t)code;
                    mx.u(kMxCodeHi, j) = (uint32_t)(code >> 32);
                    uint32_t q = 0;
                    while(q < j && !mx.same_code(q, j)) q++;
                    uint32_t slot;
                    float w;
                    if(q < j)
                    {
                        slot = mx.u(kMxSlot, q);
                        w = mx.f(kMxW, q);
                        mx.set(j, mx.lobe(q), w);
                    }
                    else
                    {
                        slot = guide::try_insert(G, code);
                        guide::Lobe l;
                        l.dir = make_float3(0, 0, 0); l.kappa = 0.0f; l.alpha = 0.0f;
                        w = 0.0f;
                        if(slot != guide::kInvalid)
                        {
                            guide::Chain c;
                            const float4 a = G.mcA[slot];
                            c.target = f3(a);
                            c.cosine = a.w;
                            c.weight = G.mcW[slot];
                            l = guide::chain_to_lobe(c, G.mcN[slot], pos);
                            w = c.weight;
                        }
                        mx.set(j, l, w);
                    }
                    mx.u(kMxSlot, j) = slot;
                    if(slot == guide::kInvalid) continue;
                    sumW = add(sumW, w);
                    const float ratio = (sumW != 0.0f) ? __fdiv_rn(w, sumW) : 1.0f;
                    if(guide::next_float(rng) < ratio) sIdx = j;
                }
                const uint32_t liftedMC = (sIdx != guide::kInvalid) ? mx.u(kMxSlot, sIdx) : guide::kInvalid;
                Q.bk[i] = rng;
                const float2 coN = guide::dir_to_conc_octa(woW);

                // ---- mixture or material sample, balance-heuristic pdf ----
                float mw0 = 0.0f;
                if(!isSpec)
                {
                    const float t = fminf(fmaxf(sub(1.0f, specv), 0.0f), 1.0f);
                    mw0 = add(mul(0.0f, sub(1.0f, t)), mul(G.lobeProb, t));     // Math::Lerp(0, p, t)
                    if(G.fixZeroWeight && (sIdx == guide::kInvalid || mx.f(kMxW, sIdx) == 0.0f)) mw0 = 0.0f;
                }
                const float mw1 = sub(1.0f, mw0);
                Chan refl;
                float pdf0, pdf1;
                bool passed = false, lobeSampled = false;
                float3 wdir, orgOut = pos;
                if(rnd_s(L, key, i, depth, kRnMis) < mw0)
                {
                    // GaussLobeMixtureT::Sample: a zero-weight choice (or none) is the
                    // Y axis with pdf 0
                    float3 v = make_float3(0.0f, 1.0f, 0.0f);
                    float mpdf = 0.0f;
                    if(sIdx != guide::kInvalid && mx.f(kMxW, sIdx) != 0.0f)
                    {
                        const float3 u3 = rnd_s3(L, key, i, depth);
                        v = guide::lobe_sample(mx.lobe(sIdx), u3.x, u3.y);
                        mpdf = mixture_pdf(mx, sumW, v);
                    }
                    wdir = v;
                    const float3 vn = normalize3(v);
                    const float3 Ls = make_float3(dot3(vn, tng), dot3(vn, btg), dot3(vn, nrm));
                    float bpdf;
                    refl = eval_material<NC>(sf, mt, alb, V, Ls, bpdf);
                    pdf0 = mpdf;
                    pdf1 = bpdf;
                    lobeSampled = true;
                }
                else
                {
                    float3 Ll, pre;
                    float bpdf;
                    sample_material<NC>(L, key, i, depth, sf, mt, alb, V, backSide, pos, nrm, Ll, refl, bpdf, passed,
                                        pre);
                    wdir = normalize3(make_float3(add(add(mul(tng.x, Ll.x), mul(btg.x, Ll.y)), mul(nrm.x, Ll.z)),
                                                  add(add(mul(tng.y, Ll.x), mul(btg.y, Ll.y)), mul(nrm.y, Ll.z)),
                                                  add(add(mul(tng.z, Ll.x), mul(btg.z, Ll.y)), mul(nrm.z, Ll.z))));
                    orgOut = pre;
                    pdf0 = mixture_pdf(mx, sumW, wdir);
                    pdf1 = bpdf;
                }
                const float pdfPath = add(mul(pdf0, mw0), mul(pdf1, mw1));     // BalanceCancelled<2>

                // ---- Russian roulette on the throughput before this vertex ----
                const uint32_t bounce = depth;
                depth += 1u;
                bool dead = depth >= L.maxDepth;
                if(!dead && depth >= L.rrStart && !isSpec)
                {
                    const float pr = fminf(fmaxf(chan_avg<NC>(thr), 0.1f), 1.0f);
                    if(rnd_s(L, key, i, bounce, 8) >= pr) dead = true;
                    else
                    {
                        const float inv = __fdiv_rn(1.0f, pr);
#pragma unroll
                        for(int k = 0; k < NC; k++) thr.v[k] = mul(thr.v[k], inv);
                    }
                }
                const float avgRefl = chan_avg<NC>(refl);
                if(!dead)
                {
                    Chan pthr;
#pragma unroll
                    for(int k = 0; k < NC; k++) pthr.v[k] = mul(thr.v[k], refl.v[k]);
                    if(pdfPath == 0.0f) pthr = chan(0, 0, 0, 0);
                    else
                    {
                        const float inv = __fdiv_rn(1.0f, pdfPath);
#pragma unroll
                        for(int k = 0; k < NC; k++) pthr.v[k] = mul(pthr.v[k], inv);
                    }
                    const float3 nn = passed ? make_float3(-nrm.x, -nrm.y, -nrm.z) : nrm;
                    const float3 no = nudge(orgOut, nn);
                    P.rays[2 * (size_t)i] = make_float4(no.x, no.y, no.z, 1.0e-4f);
                    P.rays[2 * (size_t)i + 1] = make_float4(wdir.x, wdir.y, wdir.z, 3.402823466e+38f);
                    const Cone co = cone_after_scatter(sf, mt, backSide, cone, wo, nrm, wdir);
                    P.cone[i] = make_float2(co.aperture, co.width);
                    P.hits[i].x = kMissMark;
                    P.thr[i] = f4(pthr);
                    P.prevPdf[i] = pdfPath;
                    P.state[i] = depth | ((isSpec ? 2u : 1u) << 8);
                    Q.prevRefl[i] = __fdiv_rn(avgRefl, fmaxf(pdfPath, 10.0f));
                    Q.scoreSum[i] = lobeSampled ? sumW : kInf;
                    Q.lifted[i] = liftedMC;
                    Q.prevNormal[i] = coN;
                    alive = true;
                }
                // ---- NEE with the mixture / material MIS, then with the light ----
                if(!dead && !isSpec && nAll > 0u)
                {
                    uint32_t li;
                    float3 lp;
                    Chan emis;
                    float lightPdf;
                    nee_light<SPEC, NC>(L, lights, key, i, bounce, nAll, invN, pos, waves, li, lp, emis, lightPdf);
                    const float3 sdir = normalize3(make_float3(sub(lp.x, pos.x), sub(lp.y, pos.y), sub(lp.z, pos.z)));
                    const float3 lpn = nudge(lp, make_float3(-sdir.x, -sdir.y, -sdir.z));
                    const float3 seg = make_float3(sub(lpn.x, pos.x), sub(lpn.y, pos.y), sub(lpn.z, pos.z));
                    const float length = __fsqrt_rn(dot3(seg, seg));
                    const float3 Ls = make_float3(dot3(sdir, tng), dot3(sdir, btg), dot3(sdir, nrm));
                    float bpdf;
                    const Chan srefl = eval_material<NC>(sf, mt, alb, V, Ls, bpdf);
                    float pdfS = add(mul(mixture_pdf(mx, sumW, sdir), mw0), mul(bpdf, mw1));
                    pdfS = add(pdfS, lightPdf);
                    Chan srad = chan(0, 0, 0, 0);
                    if(pdfS != 0.0f)
                    {
                        const float inv = __fdiv_rn(1.0f, pdfS);
#pragma unroll
                        for(int k = 0; k < NC; k++) srad.v[k] = mul(mul(mul(thr.v[k], srefl.v[k]), emis.v[k]), inv);
                    }
                    const float3 so = nudge(pos, nrm);
                    P.shadowRays[2 * (size_t)i] = make_float4(so.x, so.y, so.z, 1.0e-5f);
                    P.shadowRays[2 * (size_t)i + 1] = make_float4(sdir.x, sdir.y, sdir.z,
                                                                  mul(length, sub(1.0f, 1.0e-4f)));
                    P.shadowRad[i] = f4(srad);
                    const float se = mul(chan_avg<NC>(srefl), chan_avg<NC>(emis));
                    Q.shadowOut[i] = __fdiv_rn(se, fmaxf(pdfS, 10.0f));
                    shadow = true;
                }
            }
        }
        warp_append(alive, i, nextList, nextCount);
        warp_append(shadow, i, P.shadowList, P.counts + 2);
    }
}

// KCAccumulateShadowRaysGPT and KCBackpropagateIrradNEE's records.
__global__ void __launch_bounds__(kPtTPB)
k_guide_resolve(PtPaths P, GuidePaths Q)
{
    const uint32_t n = P.counts[2];
    for(uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const uint32_t i = P.shadowList[k];
        if(!((P.visBits[i >> 5] >> (i & 31u)) & 1u)) continue;
        const float4 s = P.shadowRad[i];
        float4 r = P.rad[i];
        r.x = add(r.x, s.x); r.y = add(r.y, s.y); r.z = add(r.z, s.z); r.w = add(r.w, s.w);
        P.rad[i] = r;
        const uint32_t lm = Q.lifted[i];
        if(lm != guide::kInvalid) put_record(Q, Q.slots + i, lm, 0u, Q.shadowOut[i]);
    }
}

// MCIrradiance::AtomicEMA's update of record k of a run, split into the part
// that does not depend on the average (known once the count before the run,
// n0, and k are): n = min(n0 + k + 1, 128), t = max(1 / n, 0.01),
// a = 1 - t, b = r t; the average then steps x = x a + b, exactly
// Math::Lerp(x, r, t) = x (1 - t) + r t.
__device__ __forceinline__ void ema_terms(uint32_t n0, uint32_t k, float r, float& a, float& b)
{
    const uint32_t nn = min(n0 + k + 1u, 128u);
    const float t = fmaxf(__fdiv_rn(1.0f, (float)nn), 0.01f);
    a = __fsub_rn(1.0f, t);
    b = __fmul_rn(r, t);
}

// The sorted records of a bounce, one warp per window of 32 sorted
// positions.  Each lane holding a cell's first record applies that cell's
// records in order, all such cells of the window at once: every lane forms
// its record's (a, b) terms in parallel, and the first lane of each cell runs
// the dependent steps x = x a + b, taking the terms by shuffle.  A cell whose
// records run past the window goes to the long-run list instead, whole.
__global__ void __launch_bounds__(kPtTPB)
k_guide_apply(GuideGrid G, const uint32_t* __restrict__ keys, const float* __restrict__ vals, uint32_t n,
              uint2* __restrict__ longRuns, uint32_t* longCount)
{
    const uint32_t tableSize = G.tableMask + 1u;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for(uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c * 32u < n; c += warps)
    {
        const uint32_t j = c * 32u + lane;
        const uint32_t key = (j < n) ? keys[j] : 0xFFFFFFFFu;
        uint32_t prevKey = __shfl_up_sync(0xFFFFFFFFu, key, 1);
        if(lane == 0u) prevKey = (j > 0u && j - 1u < n) ? keys[j - 1u] : 0xFFFFFFFFu;
        const uint32_t cell = key >> 1;
        const bool ok = cell < tableSize;
        const bool head = ok && (j == 0u || (prevKey >> 1) != cell);
        const uint32_t headMask = __ballot_sync(0xFFFFFFFFu, head);
        if(headMask == 0u) continue;
        // my cell's first lane in this window (none: a run from an earlier window)
        const uint32_t mine = headMask & ((lane == 31u) ? 0xFFFFFFFFu : ((2u << lane) - 1u));
        const uint32_t hl = mine ? 31u - (uint32_t)__clz(mine) : 32u;
        // the record after the last one of my cell in this window: the next
        // first record or empty record, else 32
        const uint32_t okMask = __ballot_sync(0xFFFFFFFFu, ok);
        const uint32_t bounds = (headMask | ~okMask) & ((lane == 31u) ? 0u : (0xFFFFFFFFu << (lane + 1u)));
        const uint32_t segEnd = bounds ? (uint32_t)(__ffs(bounds) - 1) : 32u;
        const uint32_t hlEnd = __shfl_sync(0xFFFFFFFFu, segEnd, hl & 31u);
        const bool shortRun = hl < 32u && hlEnd < 32u;        // my record belongs to a run ending here
        const float r = (ok && shortRun) ? vals[j] : 0.0f;
        float v = 0.0f;
        uint32_t cnt = 0;
        if(head && segEnd < 32u)
        {
            const float2 e = G.irr[cell];
            v = e.x;
            cnt = __float_as_uint(e.y);
        }
        const uint32_t n0 = __shfl_sync(0xFFFFFFFFu, cnt, hl & 31u);
        float a = 1.0f, b = 0.0f;
        if(ok && shortRun) ema_terms(n0, lane - hl, r, a, b);
#pragma unroll
        for(uint32_t k = 0; k < 32u; k++)
        {
            const float ak = __shfl_sync(0xFFFFFFFFu, a, (lane + k) & 31u);
            const float bk = __shfl_sync(0xFFFFFFFFu, b, (lane + k) & 31u);
            if(head && lane + k < segEnd) v = __fadd_rn(__fmul_rn(v, ak), bk);
        }
        if(head && segEnd < 32u) G.irr[cell] = make_float2(v, __uint_as_float(min(cnt + (segEnd - lane), 128u)));
        if(head && segEnd == 32u) longRuns[atomicAdd(longCount, 1u)] = make_uint2(j, cell);
    }
}

// Runs longer than a window, one block per run: the block forms the (a, b)
// terms of the next 256 records (and whether they are still the run's) into
// shared memory while thread 0 runs the dependent chain over the previous 256.
__global__ void __launch_bounds__(kPtTPB)
k_guide_apply_long(GuideGrid G, const uint32_t* __restrict__ keys, const float* __restrict__ vals, uint32_t n,
                   const uint2* __restrict__ longRuns, const uint32_t* longCount)
{
    __shared__ __align__(16) float sA[2][kPtTPB];
    __shared__ __align__(16) float sB[2][kPtTPB];
    const uint32_t runs = *longCount;
    for(uint32_t e = blockIdx.x; e < runs; e += gridDim.x)
    {
        const uint2 run = longRuns[e];
        const uint32_t start = run.x, cell = run.y;
        const float2 e0 = G.irr[cell];
        const uint32_t n0 = __float_as_uint(e0.y);
        float v = e0.x;
        uint32_t total = 0;
        // terms of chunk ch into buffer ch & 1; returns how many of its records are the run's
        auto terms = [&](uint32_t ch) -> uint32_t {
            const uint32_t q = start + ch * kPtTPB + threadIdx.x;
            const bool in = q < n && (keys[q] >> 1) == cell;
            float a = 1.0f, b = 0.0f;
            if(in) ema_terms(n0, q - start, vals[q], a, b);
            sA[ch & 1u][threadIdx.x] = a;
            sB[ch & 1u][threadIdx.x] = b;
            return (uint32_t)__syncthreads_count(in);       // sorted: a prefix of the chunk
        };
        uint32_t len = terms(0);
        for(uint32_t ch = 0;; ch++)
        {
            const uint32_t cur = ch & 1u;
            // the next chunk's terms go into the other buffer meanwhile
            uint32_t next = 0;
            if(threadIdx.x == 0)
            {
                // four terms per shared-memory load, loads unrolled ahead of the chain
                const float4* A4 = reinterpret_cast<const float4*>(sA[cur]);
                const float4* B4 = reinterpret_cast<const float4*>(sB[cur]);
                const uint32_t quads = len >> 2;
#pragma unroll 8
                for(uint32_t k = 0; k < quads; k++)
                {
                    const float4 a = A4[k], b = B4[k];
                    v = __fadd_rn(__fmul_rn(v, a.x), b.x);
                    v = __fadd_rn(__fmul_rn(v, a.y), b.y);
                    v = __fadd_rn(__fmul_rn(v, a.z), b.z);
                    v = __fadd_rn(__fmul_rn(v, a.w), b.w);
                }
                for(uint32_t k = quads << 2; k < len; k++) v = __fadd_rn(__fmul_rn(v, sA[cur][k]), sB[cur][k]);
            }
            total += len;
            if(len < (uint32_t)kPtTPB) break;           // block-uniform
            next = terms(ch + 1u);
            len = next;
        }
        if(threadIdx.x == 0) G.irr[cell] = make_float2(v, __uint_as_float(min(n0 + total, 128u)));
        __syncthreads();
    }
}

} // namespace

cudaError_t guide_backprop(const PtLaunch&, const PtPaths& P, const GuideGrid& G, const GuidePaths& Q,
                           const PtSceneTables& T, const uint32_t* aliveList, const uint32_t* aliveCount,
                           int smCount, cudaStream_t st)
{
    k_guide_backprop<<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(G, Q, P, T, aliveList, aliveCount);
    return cudaGetLastError();
}

cudaError_t guide_write_mc(const PtPaths& P, const GuideGrid& G, const GuidePaths& Q, const PtSceneTables& T,
                           const uint32_t* aliveList, const uint32_t* aliveCount, int smCount, cudaStream_t st)
{
    k_guide_write_mc<<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(G, Q, P, T, aliveList, aliveCount);
    return cudaGetLastError();
}

cudaError_t guide_shade(const PtLaunch& L, const PtPaths& P, const GuideGrid& G, const GuidePaths& Q,
                        const PtSceneTables& T, const uint32_t* aliveList, const uint32_t* aliveCount,
                        uint32_t* nextList, uint32_t* nextCount, int smCount, cudaStream_t st)
{
    static bool attr = false;
    if(!attr)
    {
        cudaError_t e = cudaFuncSetAttribute(k_shade_guided<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kMixSmem);
        if(e == cudaSuccess)
            e = cudaFuncSetAttribute(k_shade_guided<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kMixSmem);
        if(e != cudaSuccess) return e;
        attr = true;
    }
    const unsigned grid = (unsigned)smCount * 2u;
    if(L.spec.enabled)
        k_shade_guided<true><<<grid, kPtTPB, kMixSmem, st>>>(L, P, G, Q, T, aliveList, aliveCount, nextList,
                                                             nextCount);
    else
        k_shade_guided<false><<<grid, kPtTPB, kMixSmem, st>>>(L, P, G, Q, T, aliveList, aliveCount, nextList,
                                                              nextCount);
    return cudaGetLastError();
}

cudaError_t guide_resolve(const PtPaths& P, const GuidePaths& Q, int smCount, cudaStream_t st)
{
    k_guide_resolve<<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(P, Q);
    return cudaGetLastError();
}

cudaError_t guide_apply(const GuideGrid& G, const GuidePaths& Q, int smCount, cudaStream_t st)
{
    const uint32_t n = 2u * Q.slots;
    const uint32_t passes = (Q.keyBits + 7u) / 8u;
    // the records' values ride along as the sort's payload, so the sorted
    // values are read in order
    const uint32_t* kIn = Q.recKey;
    const uint32_t* iIn = reinterpret_cast<const uint32_t*>(Q.recVal);
    for(uint32_t p = 0; p < passes; p++)
    {
        uint32_t* kOut = (p & 1u) ? Q.sortKeysB : Q.sortKeysA;
        uint32_t* iOut = (p & 1u) ? Q.sortIdxB : Q.sortIdxA;
        DigitSpec s;
        s.batchShift = 0; s.batchWidth = Q.keyBits;
        s.dataShift = 0; s.dataWidth = 0;
        s.digitShift = 8u * p;
        s.digitBits = min(8u, Q.keyBits - 8u * p);
        cudaError_t e = multisplit_pass(kIn, iIn, kOut, iOut, nullptr, n, s, Q.sortHist, st);
        if(e != cudaSuccess) return e;
        kIn = kOut;
        iIn = iOut;
    }
    cudaError_t e = cudaMemsetAsync(Q.longCount, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    const float* vals = reinterpret_cast<const float*>(iIn);
    k_guide_apply<<<(unsigned)smCount * 4u, kPtTPB, 0, st>>>(G, kIn, vals, n, Q.longRuns, Q.longCount);
    k_guide_apply_long<<<(unsigned)smCount * 2u, kPtTPB, 0, st>>>(G, kIn, vals, n, Q.longRuns, Q.longCount);
    e = cudaGetLastError();
    if(e != cudaSuccess) return e;
    return cudaMemsetAsync(Q.recKey, 0xFF, sizeof(uint32_t) * n, st);
}

} // namespace mrg
