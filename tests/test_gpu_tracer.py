"""The TracerI interface on the GPU: scenes pushed through the tracer calls
(include/mray_gb300_tracer.h) render bit-identically to the same scenes
given straight to the path tracer -- from Python (mray_gb300.tracer), from
the scene-JSON reader and from a C++ client (tests/tracer_driver.cpp) --
for RGB and spectral renderers; plus render-work accounting, camera
transforms and ClearAll."""
import os
import struct
import subprocess

import numpy as np
import pytest

from mray_gb300 import _native as N
from mray_gb300 import scene_json, scenes
from mray_gb300.pt import PathTracer, load_box_scene
from mray_gb300.tracer import INDEX, POSITION, UV0, Tracer

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.join(ROOT, "tests", "scenes")
GOLD = os.path.join(ROOT, "tests", "golden")
_MAT = {"lambert": "(Mt)Lambert", "reflect": "(Mt)Reflect", "refract": "(Mt)Refract", "unreal": "(Mt)Unreal"}
_MAT_CODE = {"lambert": N.MRG_MAT_LAMBERT, "reflect": N.MRG_MAT_REFLECT, "refract": N.MRG_MAT_REFRACT,
             "unreal": N.MRG_MAT_UNREAL}


def push_surfaces(t, surfaces, camera):
    """The dict-form scene (mray_gb300.scenes) through the tracer calls:
    a batch and a (T)Single transform per surface, a material group per
    type, primitive-backed lights, a pinhole camera.  Returns the camera
    surface id (the surfaces are not committed)."""
    pg = t.create_primitive_group("(P)Triangle")
    batches = t.reserve_primitive_batches(pg, [(s["idx"].shape[0], s["pos"].shape[0]) for s in surfaces])
    t.commit_prim_reservations(pg)
    for s, b in zip(surfaces, batches):
        t.push_prim_attribute(pg, b, POSITION, s["pos"])
        t.push_prim_attribute(pg, b, INDEX, s["idx"])
        if s.get("uv") is not None:
            t.push_prim_attribute(pg, b, UV0, s["uv"])
    tg = t.create_transform_group("(T)Single")
    trans = t.reserve_transformations(tg, len(surfaces))
    t.commit_trans_reservations(tg)
    for s, tid in zip(surfaces, trans):
        m = np.eye(4, dtype=np.float32)
        m[:3, :] = np.asarray(s["m34"], np.float32).reshape(3, 4)
        t.push_trans_attribute(tg, (tid, tid), 0, m)
    tex = {}
    mats = {}
    for kind in _MAT:
        members = [i for i, s in enumerate(surfaces) if s["kind"] != "light" and s.get("material", "lambert") == kind]
        if not members:
            continue
        g = t.create_material_group(_MAT[kind])
        ids = t.reserve_materials(g, len(members))
        t.commit_mat_reservations(g)
        for i, mid in zip(members, ids):
            s, r = surfaces[i], (mid, mid)
            mats[i] = mid
            if kind in ("lambert", "unreal"):
                if s.get("texture") is not None:
                    key = id(s["texture"])
                    if key not in tex:
                        given = s.get("mips_given") or {}
                        tex[key] = (t.create_texture_2d(s["texture"].shape[1], s["texture"].shape[0],
                                                        1 + max(given, default=0),
                                                        "rgba8_unorm" if s["texture"].dtype == np.uint8
                                                        else "rgba_float"), s["texture"], given)
                    t.push_mat_attribute(g, r, 0, None, [tex[key][0]])
                else:
                    t.push_mat_attribute(g, r, 0, s["albedo"], [None])
            if kind == "unreal":
                for k, name in enumerate(("roughness", "specular", "metallic")):
                    pt_tex = s.get(name + "_texture")
                    if pt_tex is not None:
                        key = id(pt_tex)
                        if key not in tex:
                            kind4 = "rgba8_unorm" if pt_tex.dtype == np.uint8 else "rgba_float"
                            kind1 = "r8_unorm" if pt_tex.dtype == np.uint8 else "r_float"
                            tex[key] = (t.create_texture_2d(pt_tex.shape[1], pt_tex.shape[0], 1,
                                                            kind1 if pt_tex.ndim == 2 else kind4), pt_tex, {})
                        t.push_mat_attribute(g, r, 2 + k, None, [tex[key][0]])
                    else:
                        t.push_mat_attribute(g, r, 2 + k, [s.get(name, 0.5 if name == "specular" else 0.0)], [None])
            if kind == "refract":
                front, back = s.get("ior", (1.0, 1.5))
                t.push_mat_attribute(g, r, 0, [back, 0, 0])
                t.push_mat_attribute(g, r, 1, [front, 0, 0])
    lights = [i for i, s in enumerate(surfaces) if s["kind"] == "light"]
    lids = {}
    if lights:
        g = t.create_light_group("(L)Prim(P)Triangle", pg)
        ids = t.reserve_lights(g, len(lights), [batches[i] for i in lights])
        t.commit_light_reservations(g)
        for i, lid in zip(lights, ids):
            lids[i] = lid
            t.push_light_attribute(g, (lid, lid), 0, surfaces[i]["radiance"], [None])
            t.push_light_attribute(g, (lid, lid), 1, [0], dtype=np.uint8)
    cg = t.create_camera_group("(C)Pinhole")
    (cid,) = t.reserve_cameras(cg, 1)
    t.commit_cam_reservations(cg)
    t.push_cam_attribute(cg, (cid, cid), 0, list(camera["fov"]) + list(camera["near_far"]))
    t.push_cam_attribute(cg, (cid, cid), 1, camera["gaze"])
    t.push_cam_attribute(cg, (cid, cid), 2, camera["pos"])
    t.push_cam_attribute(cg, (cid, cid), 3, camera["up"])
    t.commit_textures()
    for tid, data, given in tex.values():
        t.push_texture_data(tid, 0, data)
        for lv, texels in sorted(given.items()):
            t.push_texture_data(tid, lv, texels)
    for i, s in enumerate(surfaces):
        if s["kind"] != "light":
            t.create_surface([batches[i]], [mats[i]], trans[i], [s.get("cull", True)])
    for i in lights:
        t.create_light_surface(lids[i], trans[i])
    t.set_boundary_surface(0)
    return t.create_camera_surface(cid)


def tracer_render(t, cs, w, h, total, burst, mode="WithNEEAndMIS", rr=(3, 8), renderer="(R)PathTracerRGB"):
    r = t.create_renderer(renderer)
    t.push_renderer_attribute(r, 0, total)
    t.push_renderer_attribute(r, 1, burst)
    t.push_renderer_attribute(r, 3, mode)
    t.push_renderer_attribute(r, 4, rr)
    info = t.start_render(r, cs, w, h)
    assert info["total_spp"] == total and info["d_film"]
    works = []
    while True:
        o = t.do_render_work()
        works.append(o)
        if o["finished"]:
            break
    assert [o["samples_done"] for o in works] == [min(total, burst * (k + 1)) for k in range(len(works))]
    return t.read_film(), works


def direct_render(pt, camera, w, h, total, burst, seed, mode=N.MRG_PT_NEE_MIS, rr=(3, 8)):
    img = None
    for s in range(0, total, burst):
        p = PathTracer.params(w, h, min(burst, total - s), camera, max_depth=rr[1], rr_start=rr[0], sample_mode=mode,
                              seed=seed, sample_start=s, sampler="pcg32")
        img = pt.render(p, image=img)
    return img.cpu().numpy()


def _lights_unculled(surfaces):
    # light surfaces are never back-face culled behind TracerI
    return [dict(s, cull=False) if s["kind"] == "light" else s for s in surfaces]


@pytest.mark.parametrize("scene_fn", [scenes.box_scene, scenes.box_scene_mixed])
def test_tracer_matches_direct_path(scene_fn):
    surf = _lights_unculled(scene_fn(0))
    cam = scenes.box_camera()
    with Tracer(seed=21) as t:
        cs = push_surfaces(t, surf, cam)
        res = t.commit_surfaces()
        assert res["instance_count"] == len(surf) and res["accelerator_count"] == len(surf)
        film, works = tracer_render(t, cs, 64, 48, 12, 4)
        assert all(o["paths_per_second"] > 0 for o in works)
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    want = direct_render(pt, cam, 64, 48, 12, 4, seed=21)
    pt.close()
    assert film[..., 3].min() > 0
    assert np.array_equal(film, want)


@pytest.mark.parametrize("gen_mips", [True, False])
def test_tracer_texture_mips_match_direct_path(gen_mips):
    """TracerParameters::genMips (every texture's full chain, Gaussian
    mipGenFilter of radius 1.5) and mip levels pushed by PushTextureData:
    the tracer's film equals the direct path tracer's with the same chains."""
    surf = _lights_unculled(scenes.box_scene_textured(0, size=64))
    tex = surf[2]["texture"]
    surf[2]["mips_given"] = {1: np.ascontiguousarray(tex[::2, ::2]),
                             2: np.full((16, 16, 4), (30, 200, 90, 255), np.uint8)}
    if gen_mips:
        scenes.mipmapped(surf, 1.5)
    cam = scenes.box_camera()
    with Tracer(seed=23, gen_mips=gen_mips, mip_filter_radius=1.5) as t:
        cs = push_surfaces(t, surf, cam)
        t.commit_surfaces()
        film, _ = tracer_render(t, cs, 64, 48, 8, 4)
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    want = direct_render(pt, cam, 64, 48, 8, 4, seed=23)
    pt.close()
    assert np.array_equal(film, want)


def test_tracer_unreal_parameter_textures_match_direct_path():
    """Textured roughness / specular / metallic pushed through TracerI (with
    genMips) render as the direct path tracer's Unreal parameter textures."""
    surf = scenes.mipmapped(_lights_unculled(scenes.box_scene_unreal_textured(0, size=64)), 2.0)
    cam = scenes.box_camera()
    with Tracer(seed=29, gen_mips=True) as t:
        cs = push_surfaces(t, surf, cam)
        t.commit_surfaces()
        film, _ = tracer_render(t, cs, 64, 48, 8, 4)
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    want = direct_render(pt, cam, 64, 48, 8, 4, seed=29)
    pt.close()
    assert np.array_equal(film, want)


def test_tracer_single_channel_textures():
    """R8 UNORM and R float textures (MRay's usual roughness / metallic maps)
    read as (r, r, r, 1): the film equals the direct path's with the RGBA
    expansions."""
    surf = _lights_unculled(scenes.box_scene_unreal_textured(0, size=32))
    r8 = np.ascontiguousarray(surf[0]["roughness_texture"][..., 0])
    rf = np.ascontiguousarray(surf[0]["metallic_texture"][..., 0].astype(np.float32) / 255.0)
    r8x = np.repeat(r8[..., None], 4, axis=2)
    r8x[..., 3] = 255
    rfx = np.concatenate([np.repeat(rf[..., None], 3, axis=2), np.ones(rf.shape + (1,), np.float32)], axis=2)
    single, want = [dict(s) for s in surf], [dict(s) for s in surf]
    for s1, s2 in zip(single, want):
        if s1.get("material") == "unreal":
            s1["roughness_texture"], s1["metallic_texture"] = r8, rf      # 2D: single channel
            s2["roughness_texture"], s2["metallic_texture"] = r8x, rfx
    cam = scenes.box_camera()
    with Tracer(seed=31) as t:
        cs = push_surfaces(t, single, cam)
        t.commit_surfaces()
        film, _ = tracer_render(t, cs, 48, 32, 4, 4)
    pt = PathTracer(0)
    load_box_scene(pt, want)
    ref = direct_render(pt, cam, 48, 32, 4, 4, seed=31)
    pt.close()
    assert np.array_equal(film, ref)


def test_scene_json_through_tracer_matches_reader():
    path = os.path.join(HERE, "open_box.json")
    with Tracer(seed=3) as t:
        out = scene_json.load_tracer(t, path)
        assert out["commit"]["instance_count"] == 5
        assert out["commit"]["accelerator_count"] == 4            # the floor's batch is shared
        total, used = t.device_memory()
        assert total > used > 0
        film, _ = tracer_render(t, out["camera_surfaces"][0], 48, 48, 8, 8)
    pt = PathTracer(0)
    cam, _ = scene_json.load(pt, path)
    want = direct_render(pt, cam, 48, 48, 8, 8, seed=3)
    pt.close()
    assert np.array_equal(film, want)


def test_spectral_renderer_matches_direct_path():
    from mray_gb300 import spectral
    res, lut = spectral.read_mrspectra(os.path.join(GOLD, "REC_709_r32.mrspectra"))
    tables = spectral.load_tables(os.path.join(GOLD, "spectral_rec709.npz"))
    surf = _lights_unculled(scenes.box_scene_mixed(0))
    cam = scenes.box_camera()
    with Tracer(seed=4) as t:
        t.set_spectral_data(res, lut, tables)
        cs = push_surfaces(t, surf, cam)
        t.commit_surfaces()
        film, _ = tracer_render(t, cs, 40, 32, 8, 4, renderer="(R)PathTracerSpectral")
        rgb, _ = tracer_render(t, cs, 40, 32, 8, 4)                # and back to RGB on the same scene
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    pt.set_spectral(res, lut, tables)
    want = direct_render(pt, cam, 40, 32, 8, 4, seed=4)
    pt.set_spectral(0, None, None)
    want_rgb = direct_render(pt, cam, 40, 32, 8, 4, seed=4)
    pt.close()
    assert np.array_equal(film, want)
    assert np.array_equal(rgb, want_rgb)


def test_guided_renderer_matches_direct_path():
    """(R)GuidedPathTracerSpectral through the tracer calls: the grid is reset
    at StartRender and learns across the render-work calls, as
    mrg_guide_create and successive mrg_pt_render_guided calls do."""
    from mray_gb300 import spectral
    res, lut = spectral.read_mrspectra(os.path.join(GOLD, "REC_709_r32.mrspectra"))
    tables = spectral.load_tables(os.path.join(GOLD, "spectral_rec709.npz"))
    surf = _lights_unculled(scenes.box_scene_mixed(0))
    cam = scenes.box_camera()
    total, burst = 12, 4
    with Tracer(seed=6) as t:
        t.set_spectral_data(res, lut, tables)
        cs = push_surfaces(t, surf, cam)
        t.commit_surfaces()
        r = t.create_renderer("(R)GuidedPathTracerSpectral")
        t.push_renderer_attribute(r, 5, (2, 8))
        t.push_renderer_attribute(r, 6, total)
        t.push_renderer_attribute(r, 8, "Latency")
        t.push_renderer_attribute(r, 9, burst)
        t.push_renderer_attribute(r, 11, "Render")
        t.start_render(r, cs, 40, 32)
        while not t.do_render_work()["finished"]:
            pass
        film = t.read_film()
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    pt.set_spectral(res, lut, tables)
    pt.guide_create()
    img = None
    for s0 in range(0, total, burst):
        img = pt.render_guided(PathTracer.params(40, 32, burst, cam, max_depth=8, rr_start=2, seed=6,
                                                 sample_start=s0, sampler="pcg32"), image=img)
    pt.close()
    assert np.isfinite(film).all() and film[..., 3].min() == total
    assert np.array_equal(film, img.cpu().numpy())


def test_spectral_renderer_needs_its_data():
    with Tracer() as t:
        cs = push_surfaces(t, scenes.box_scene(0), scenes.box_camera())
        t.commit_surfaces()
        r = t.create_renderer("(R)PathTracerSpectral")
        with pytest.raises(N.MRGError, match="spectral data"):
            t.start_render(r, cs, 16, 16)


def test_camera_transform_and_clear_all():
    surf, cam = _lights_unculled(scenes.box_scene(0)), scenes.box_camera()
    with Tracer(seed=8) as t:
        cs = push_surfaces(t, surf, cam)
        t.commit_surfaces()
        assert np.allclose(t.get_cam_transform(cs), list(cam["pos"]) + list(cam["gaze"]) + list(cam["up"]))
        r = t.create_renderer("(R)PathTracerRGB")
        t.push_renderer_attribute(r, 0, 4)
        t.push_renderer_attribute(r, 1, 4)
        t.start_render(r, cs, 32, 32)
        t.do_render_work()
        moved = np.array(list(cam["pos"]) + list(cam["gaze"]) + list(cam["up"]), np.float32)
        moved[0] += 0.1
        t.set_camera_transform(r, moved)                          # restarts the accumulation
        o = t.do_render_work()
        assert o["samples_done"] == 4 and o["finished"]
        assert t.do_render_work()["samples_done"] == 4            # nothing more once finished
        film = t.read_film()
        t.stop_render()
        with pytest.raises(N.MRGError, match="already committed"):
            t.commit_surfaces()
        t.clear_all()
        cs = push_surfaces(t, surf, cam)                          # the tracer is reusable
        t.commit_surfaces()
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    c2 = dict(cam, pos=tuple(float(x) for x in moved[:3]))
    want = pt.render(PathTracer.params(32, 32, 4, c2, max_depth=20, rr_start=4, sample_mode=N.MRG_PT_PURE,
                                       seed=8, sampler="pcg32")).cpu().numpy()
    pt.close()
    assert np.array_equal(film, want)


def _dump(path, surfaces, camera, w, h, total, burst, mode, rr, seed):
    with open(path, "wb") as f:
        f.write(struct.pack("<I", len(surfaces)))
        for s in surfaces:
            light = s["kind"] == "light"
            mat = _MAT_CODE[s.get("material", "lambert")]
            pos = np.ascontiguousarray(s["pos"], np.float32)
            idx = np.ascontiguousarray(s["idx"], np.uint32)
            f.write(struct.pack("<5I", 1 if light else 0, mat, 1 if s.get("cull", True) else 0, pos.shape[0],
                                idx.shape[0]))
            f.write(pos.tobytes() + idx.tobytes() + np.asarray(s["m34"], np.float32).tobytes())
            col = s["radiance"] if light else s["albedo"]
            ior = s.get("ior", (1.0, 1.5))
            f.write(np.array(list(col) + [s.get("roughness", 0.0), s.get("metallic", 0.0), s.get("specular", 0.5),
                                          ior[0], ior[1]], np.float32).tobytes())
        f.write(np.array(list(camera["pos"]) + list(camera["gaze"]) + list(camera["up"]) + list(camera["fov"]) +
                         list(camera["near_far"]), np.float32).tobytes())
        f.write(struct.pack("<7IQ", w, h, total, burst, mode, rr[0], rr[1], seed))


def test_cpp_client_matches_direct_path(tmp_path):
    """A C++ program drives the tracer calls in TracerI order (the way MRay's
    scene loader does) and renders the same film as the direct path."""
    from mray_gb300 import build as B
    exe = str(tmp_path / "tracer_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "tracer_driver.cpp"), "-o", exe, B.LIB,
                    "-Wl,-rpath," + os.path.dirname(B.LIB)], check=True, capture_output=True, text=True)
    surf = _lights_unculled(scenes.box_scene_mixed(0))
    cam = scenes.box_camera()
    _dump(str(tmp_path / "scene.bin"), surf, cam, 56, 40, 12, 4, N.MRG_PT_NEE_MIS, (3, 8), 77)
    r = subprocess.run([exe, str(tmp_path / "scene.bin"), str(tmp_path / "film.bin")], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "instances 8 works 3 samples 12" in r.stdout
    film = np.fromfile(str(tmp_path / "film.bin"), np.float32).reshape(40, 56, 4)
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    want = direct_render(pt, cam, 56, 40, 12, 4, seed=77)
    pt.close()
    assert np.array_equal(film, want)
