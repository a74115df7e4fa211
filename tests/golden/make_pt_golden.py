"""Writes tests/golden/pt_math.npz: seeded inputs and the outputs of MRay's
OWN path-tracer building blocks on them, computed by MRay's code compiled from
its source tree (oracle/ref_pt_driver.cpp through oracle/build.py:
build_ref_pt).  Run where the MRay source tree is present; the fixture is
committed and checked against the project's restatement by
tests/test_oracle_pt_golden.py.

Covered (MRay file:line):
  materials      Lambert / Reflect / Refract / Unreal SampleBxDF, Evaluate,
                 Pdf, Specularity (Tracer/MaterialsDefault.hpp) on a surface
                 whose shading rotation is the identity
  fresnel        BxDF::FresnelDielectric (Tracer/DistributionFunctions.h:382)
  vndf           BxDF::VNDFGGXSmithSample (:529)
  cos            Common::SampleCosDirection (:847)
  rr             Common::RussianRoulette (:943)
  balance        MIS::BalanceCancelled<2> (:957)
  filter         GaussianFilter::Sample / Evaluate (Tracer/Filters.h:195-233)
  light          LightPrim<Triangle<TransformContextSingle>> SampleSolidAngle,
                 PdfSolidAngle, EmitViaHit, EmitViaSurfacePoint, area
                 (Tracer/LightsDefault.hpp:14-165)
  sph            SphericalCoordConverter (Tracer/LightsDefault.hpp:174-215)
  pwc            DistributionPwC<2>::SampleUV / PdfUV (Tracer/Distributions.h)
  camera         CameraPinhole + EvaluateRay (Tracer/CamerasDefault.hpp)
  waves          SingleSampleSpectrumWavelength (Tracer/SpectrumContext.cu:9)
  zsobol         ZSobolDetail::ZSobol Next / Next2D / Next3D (Tracer/Random.cu:265-425)
                 and the group's per-pixel seeds (Random.cu:1175-1200)
  pcg32          PermutedCG32 GenerateState / Advance / Next (Tracer/Random.h:762-842),
                 the independent group's generator
  guide          the guided path tracer's blocks: Distribution::GaussianLobe
                 (Tracer/DistributionFunctions.h:230-380), concentric octahedral mapping
                 (Core/GraphicsFunctions.h:318-384), HashGridView GenCode /
                 GenCodeStochastic / TryInsert / Search (Tracer/HashGrid.h:230-400)
  cone           RayCone::Advance / Project, RayConeSurface::ConeAfterScatter
                 (Tracer/TracerTypes.h:323-380), RefractMaterial::RefractRayCone
                 (Tracer/MaterialsDefault.hpp:353-462)
  pix            Graphics::ConvertPixelIndices (Core/GraphicsFunctions.h:529-538)

Usage: python tests/golden/make_pt_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_pt  # noqa: E402

N = 1024


def unit(v):
    return (v / np.linalg.norm(v, axis=-1, keepdims=True)).astype(np.float32)


def upper_dirs(rng, n, grazing=0.1):
    """Unit directions in the upper hemisphere, a share of them grazing,
    some exactly along the normal."""
    d = rng.normal(size=(n, 3))
    d[:, 2] = np.abs(d[:, 2])
    k = int(n * grazing)
    d[:k, 2] = rng.uniform(1e-4, 2e-2, k)
    d[k:k + 8] = (0.0, 0.0, 1.0)
    return unit(d)


def materials(rng):
    out = {}
    for kind in ("lambert", "reflect", "refract", "unreal"):
        rec = np.zeros(N, ref_pt.MAT_IN)
        rec["albedo"] = rng.uniform(0.0, 1.0, (N, 3))
        rec["albedo"][:16] = 0.0
        rough = rng.uniform(0.05, 0.5, N)
        rough[:32] = rng.choice([0.0, 1e-3, 0.02, 1.0], 32)
        rec["rough"] = rough
        rec["metal"] = rng.choice([0.0, 1.0, 0.5], N) if kind == "unreal" else 0.0
        rec["metal"][N // 2:] = rng.uniform(0, 1, N - N // 2)
        rec["spec"] = rng.uniform(0.0, 1.0, N)
        rec["iorF"] = 1.0
        rec["iorB"] = rng.choice([1.5, 1.33, 2.4], N)
        rec["backSide"] = rng.integers(0, 2, N)
        rec["pos"] = rng.uniform(-50, 50, (N, 3))
        rec["pos"][:64] = rng.uniform(-0.02, 0.02, (64, 3))      # Nudge's small-coordinate branch
        rec["wo"] = upper_dirs(rng, N)
        ev = rng.normal(size=(N, 3))
        ev[: N // 8, 2] = -np.abs(ev[: N // 8, 2])                # some below the surface
        rec["wiEval"] = unit(ev)
        rec["xi"] = rng.integers(0, 2 ** 32, (N, 3), dtype=np.uint64).astype(np.uint32)
        rec["xi"][:8] = 0
        rec["xi"][8:16] = 0xFFFFFFFF
        out["mat_%s_in" % kind] = rec
        out["mat_%s_out" % kind] = ref_pt.material(kind, rec)
    return out


def building_blocks(rng):
    out = {}
    cosF = rng.uniform(0, 1, N).astype(np.float32)
    cosF[:4] = (0.0, 1.0, 1e-6, 0.5)
    etas = rng.choice([1.0, 1.5, 1.33, 2.4], (N, 2)).astype(np.float32)
    f_in = np.stack([cosF, etas[:, 0], etas[:, 1]], 1)
    out["fresnel_in"], out["fresnel_out"] = f_in, ref_pt.fresnel_dielectric(f_in)

    v_in = np.zeros((N, 6), np.float32)
    v_in[:, :3] = upper_dirs(rng, N)
    v_in[:, 3] = rng.uniform(0.0025, 0.25, N)
    v_in[:, 4:6] = rng.uniform(0, 1, (N, 2))
    out["vndf_in"], out["vndf_out"] = v_in, ref_pt.vndf_sample(v_in)

    c_in = rng.uniform(0, 1, (N, 2)).astype(np.float32)
    c_in[:4] = ((0, 0), (0.999999, 0.5), (0.25, 0.999), (1e-9, 0.3))
    out["cos_in"], out["cos_out"] = c_in, ref_pt.cos_sample(c_in)

    r_in = np.zeros((N, 6), np.float32)
    r_in[:, :4] = rng.uniform(0, 3, (N, 4))
    r_in[:, 4] = rng.uniform(-0.2, 1.5, N)
    r_in[:, 5] = rng.uniform(0, 1, N)
    out["rr_in"], out["rr_out"] = r_in, ref_pt.russian_roulette(r_in)

    b_in = rng.uniform(0, 4, (N, 4)).astype(np.float32)
    b_in[:, 3] = 1.0 - b_in[:, 2] / 4.0
    b_in[:, 2] = b_in[:, 2] / 4.0
    out["balance_in"], out["balance_out"] = b_in, ref_pt.balance_cancelled(b_in)

    g_in = np.zeros((N, 3), np.float32)
    g_in[:, 0] = rng.choice([1.0, 0.5, 2.0], N)
    g_in[:, 1:] = rng.uniform(0, 1, (N, 2))
    g_in[:4, 1:] = ((0, 0.5), (0.5, 0), (0.999999, 0.5), (0.5, 0.5))
    out["filter_in"], out["filter_out"] = g_in, ref_pt.gaussian_filter(g_in)

    s_in = np.zeros((N, 6), np.float32)
    s_in[:, :3] = unit(rng.normal(size=(N, 3)))
    s_in[:4, :3] = ((0, 1, 0), (0, -1, 0), (1, 0, 0), (0, 0, -1))
    s_in[:, 3:5] = rng.uniform(0, 1, (N, 2))
    s_in[:4, 3:5] = ((0, 0), (1, 1), (0.5, 0.5), (0.25, 1))
    s_in[:, 5] = rng.uniform(0, 3, N)
    out["sph_in"], out["sph_out"] = s_in, ref_pt.spherical_coords(s_in)
    return out


def lights(rng):
    rec = np.zeros(N, ref_pt.LIGHT_IN)
    for i in range(N):
        a, b = rng.uniform(0, 2 * np.pi, 2)
        s = rng.choice([1.0, 0.5, 3.0])
        rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
        ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
        m = np.zeros((3, 4))
        m[:, :3] = rz @ ry * s
        m[:, 3] = rng.uniform(-10, 10, 3)
        rec["m"][i] = m.reshape(12)
    rec["v9"] = rng.uniform(-1, 1, (N, 9))
    rec["twoSided"] = rng.integers(0, 2, N)
    rec["radiance"] = rng.uniform(0, 20, (N, 3))
    rec["distant"] = rng.uniform(-15, 15, (N, 3))
    rec["xi"] = rng.integers(0, 2 ** 32, (N, 2), dtype=np.uint64).astype(np.uint32)
    ab = rng.uniform(0, 1, (N, 2))
    swap = ab.sum(1) > 1
    ab[swap] = 1 - ab[swap]
    rec["hit"] = ab
    rec["hit"][:4] = ((1, 0), (0, 1), (0, 0), (0.5, 0.5))
    rec["dir"] = unit(rng.normal(size=(N, 3)))
    rec["wo"] = unit(rng.normal(size=(N, 3)))
    return {"light_in": rec, "light_out": ref_pt.tri_light(rec)}


def distributions(rng):
    h, w = 16, 32
    f = rng.uniform(0, 1, (h, w)).astype(np.float32) ** 3
    # (a row of zeros is left out: MRay's construction divides by the row's
    # zero total, Distributions.cu KCNormalizeXY, and its CDF is NaN)
    f[3] = 1e-6                    # a nearly empty row
    f[7, 5] = 40.0                 # a sun
    # the CDFs as the oracle builds them (MRay builds them in its device
    # layer); the sampling over them is MRay's
    import oracle
    d = oracle.Pwc2D(f)
    xi = rng.uniform(0, 1, (N, 2)).astype(np.float32)
    xi[:4] = ((0, 0), (0.999999, 0.999999), (0.5, 0.0), (0.0, 0.5))
    uvq = rng.uniform(0, 1, (N, 2)).astype(np.float32)
    uvq[:4] = ((1, 1), (0, 0), (1, 0), (0.999999, 1))
    s, p = ref_pt.pwc2d(d.cdf_x, d.cdf_y, xi, uvq)
    return {"pwc_func": f, "pwc_cdfx": d.cdf_x, "pwc_cdfy": d.cdf_y, "pwc_xi": xi, "pwc_uvq": uvq,
            "pwc_sample": s, "pwc_pdf": p}


def cameras(rng):
    out = {}
    cam = np.array([0.0, 1.0, 3.5, 0.0, 0.9, 0.0, 0.0, 1.0, 0.0, 0.9, 0.7, 0.01, 100.0], np.float32)
    res = np.array([256, 192], np.uint32)
    pix = np.stack([rng.integers(0, 256, N), rng.integers(0, 192, N)], 1).astype(np.uint32)
    pix[:4] = ((0, 0), (255, 191), (0, 191), (255, 0))
    off = np.zeros((N, 4), np.float32)
    off[:, :2] = rng.normal(0, 0.3, (N, 2))
    off[:, 2:] = 2.0
    out["cam_params"], out["cam_res"], out["cam_pix"], out["cam_off"] = cam, res, pix, off
    out["cam_out"] = ref_pt.camera(cam, res, pix, off)
    return out


def waves(rng):
    xi = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32)
    xi[:4] = (0, 0xFFFFFFFF, 0x80000000, 0x40000000)
    w, p = ref_pt.sample_waves(2, xi)
    return {"waves_xi": xi, "waves_out": w, "waves_pdf": p}


def zsobol(rng):
    q = np.zeros((N, 8), np.uint32)
    q[:, 0] = rng.integers(0, 1920, N)
    q[:, 1] = rng.integers(0, 1080, N)
    q[:, 2] = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32)
    q[:, 3] = rng.integers(0, 300, N)
    q[:, 4] = rng.choice([1, 4, 16, 64], N)
    q[:, 5] = rng.choice([6, 8, 11], N)
    q[:, 6] = rng.integers(0, 90, N)
    q[:, 7] = rng.integers(1, 4, N)
    seeds = ref_pt.zsobol_seeds(0x123456789ABCDEF0, 4096)
    return {"zs_in": q, "zs_out": ref_pt.zsobol(q), "zs_seed64": np.uint64(0x123456789ABCDEF0), "zs_seeds": seeds}


def pcg32(rng):
    seeds = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32)
    delta = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32)
    delta[:8] = [0, 1, 2, 15, 16, 1 << 20, 0x7FFFFFFF, 0xFFFFFFFF]
    return {"pcg_seeds": seeds, "pcg_delta": delta, "pcg_out": ref_pt.pcg32_jump(seeds, delta),
            "pcg_seq_seed": np.uint32(0x9E3779B9), "pcg_seq": ref_pt.pcg32_seq(0x9E3779B9, 4096)}


def guide(rng):
    n = N
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    kap = np.concatenate([np.zeros(8), np.full(8, 1e-8), rng.uniform(0, 0.5, 250), rng.uniform(0.5, 50, 500),
                          10 ** rng.uniform(1.7, 4, n - 766)]).astype(np.float32)
    xi = rng.random((n, 2)).astype(np.float32)
    xi[:4] = [[0, 0], [0.99999994, 0.99999994], [0.5, 0], [0, 0.5]]
    in7 = np.concatenate([d, kap[:, None], xi, np.zeros((n, 1), np.float32)], 1).astype(np.float32)
    w = rng.normal(size=(n, 3)).astype(np.float32)
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    st = rng.random((n, 2)).astype(np.float32)
    dd = d.copy()
    dd[:4] = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, -1, 0]]
    octa_st, octa_dir = ref_pt.conc_octa(dd, st)
    # a grid over [-1, 2] x [-1, 2.5] x [-1, 3], 2^14 base cells, 4 x 4 normals,
    # 3 level offsets, a 0.6 degree cone (the guided renderer's defaults)
    view = np.array([0.5, 0.5, -1.4, -1, -1, -1, 2, 2.5, 3, 16384 / 4.0, 16384, 4, 4, 3, 0], np.float32)
    view[14] = np.float32(np.tan(np.float32(np.float32(np.pi) / np.float32(180)) * np.float32(0.6) *
                                 np.float32(0.5))) * np.float32(2)
    pos = rng.uniform(-1.2, 3.2, (n, 3)).astype(np.float32)
    in6 = np.concatenate([pos, dd], 1).astype(np.float32)
    rs = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    codes, rs_after = ref_pt.guide_codes(view, in6, rs)
    tcodes = rng.integers(0, 2 ** 63, 600, dtype=np.uint64)
    probe = np.concatenate([tcodes[::3], rng.integers(0, 2 ** 63, 200, dtype=np.uint64)])
    slots, found = ref_pt.guide_table(tcodes, probe, 1024)
    return {"gl_in": in7, "gl_w": w, "gl_out": ref_pt.guide_lobe(in7, w), "go_dir": dd, "go_st": st,
            "go_st_out": octa_st, "go_dir_out": octa_dir, "gc_view": view, "gc_in": in6, "gc_rng": rs,
            "gc_out": codes, "gc_rng_out": rs_after, "gt_codes": tcodes, "gt_probe": probe, "gt_slots": slots,
            "gt_found": found}


def cones(rng):
    """Ray cones: Advance, Project, the refracted cone and ConeAfterScatter,
    on the tangent surface (normal +z), and the parent-texel lookup of the
    mip generation."""
    n = N
    q = np.zeros((n, 20), np.float32)
    q[:, 0] = rng.uniform(-0.05, 0.05, n)
    q[:, 1] = rng.uniform(0.0, 0.2, n)
    q[:, 2] = rng.uniform(0.0, 30.0, n)
    q[:16, 1] = 0.0                                  # a camera cone (width 0) ...
    q[16:32, 2] = 1e8                                # ... and widths past the clamp
    q[:, 3:6] = unit(rng.normal(size=(n, 3)))
    q[:, 6:9] = unit(rng.normal(size=(n, 3)))
    q[:, 9] = rng.choice([0.0, 0.01, -0.02], n)
    wo = rng.normal(size=(n, 3))
    wo[:, 2] = np.abs(wo[:, 2]) * rng.choice([1.0, -1.0], n)
    q[:, 10:13] = unit(wo)
    q[:, 13] = 1.0
    q[:, 14] = rng.choice([1.5, 1.33, 2.4], n)
    q[:, 15] = rng.integers(0, 2, n)
    q[:, 16:19] = unit(rng.normal(size=(n, 3)))
    p = np.zeros((n, 6), np.float32)
    fr = rng.integers(1, 512, (n, 2)).astype(np.float32)
    p[:, 2:4] = np.maximum(1.0, np.floor(fr / 2))
    p[:, 4:6] = fr
    p[:, 0:2] = rng.uniform(-3.0, fr + 3.0)
    return {"cone_in": q, "cone_out": ref_pt.cone(q), "pix_in": p, "pix_out": ref_pt.pixel_indices(p)}


def main():
    if ref_pt.load() is None:
        sys.exit("the MRay source tree and fmt headers are needed (MRAY_REFERENCE_SRC)")
    rng = np.random.default_rng(20261204)
    out = {}
    for f in (materials, building_blocks, lights, distributions, cameras, waves, zsobol, pcg32, guide, cones):
        out.update(f(rng))
    path = os.path.join(HERE, "pt_math.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
