"""The TracerI interface (include/mray_gb300_tracer.h, mray_gb300/tracer.py)
without a GPU: type lists and attribute information as MRay declares them,
MRay's id layouts and implicit groups, the reservation / commit / push
order MRay enforces, renderer options, and the scene-JSON reader pushing
through it (everything before the surface commit).  CPU only."""
import os
import threading

import numpy as np
import pytest

from mray_gb300 import _native as N
from mray_gb300 import scene_json
from mray_gb300.tracer import INDEX, POSITION, UV0, Tracer

HERE = os.path.join(os.path.dirname(__file__), "scenes")


@pytest.fixture
def tr(cuda_lib):
    t = Tracer(seed=5)
    yield t
    t.close()


def test_type_lists(tr):
    assert tr.primitive_groups() == ["(P)Triangle"]
    assert tr.material_groups() == ["(Mt)Lambert", "(Mt)Reflect", "(Mt)Refract", "(Mt)Unreal"]
    assert tr.transform_groups() == ["(T)Single"]
    assert tr.camera_groups() == ["(C)Pinhole"]
    assert tr.medium_groups() == []
    assert tr.light_groups() == ["(L)Prim(P)Triangle", "(L)Skysphere_Spherical"]
    assert tr.renderers() == ["(R)PathTracerRGB", "(R)PathTracerSpectral", "(R)GuidedPathTracerSpectral"]


def test_attribute_info_follows_mray(tr):
    # MatGroupLambert::AttributeInfo (MaterialsDefault.cpp:38-53)
    lam = tr.attribute_info("material", "(Mt)Lambert")
    assert [a["name"] for a in lam] == ["albedo", "normalMap"]
    assert lam[0]["data_type"] == "VECTOR_3" and lam[0]["texturable"] == N.MRG_ATTR_TEXTURE_OR_CONSTANT
    assert lam[0]["is_color"] and not lam[0]["optional"]
    assert lam[1]["optional"] and lam[1]["texturable"] == N.MRG_ATTR_TEXTURE_ONLY
    # MatGroupUnreal (:382-402), MatGroupRefract (:236-251)
    assert [a["name"] for a in tr.attribute_info("material", "(Mt)Unreal")] == [
        "albedo", "normalMap", "roughness", "specular", "metallic"]
    assert [a["name"] for a in tr.attribute_info("material", "(Mt)Refract")] == ["cauchyBack", "cauchyFront"]
    assert tr.attribute_info("material", "(Mt)Reflect") == []
    # PrimGroupTriangle (PrimitiveDefaultTriangle.cu:169-184)
    tri = tr.attribute_info("prim", "(P)Triangle")
    assert [a["data_type"] for a in tri] == ["VECTOR_3", "QUATERNION", "VECTOR_2", "VECTOR_3UI"]
    # CameraGroupPinhole (CamerasDefault.cpp:37-50), TransformGroupSingle (TransformsDefault.cu:27-37)
    assert [a["name"] for a in tr.attribute_info("camera", "(C)Pinhole")] == ["FovAndPlanes", "gaze", "position", "up"]
    assert tr.attribute_info("transform", "(T)Single")[0]["data_type"] == "MATRIX_4x4"
    assert tr.attribute_info("transform", "(T)Identity") == []
    # LightGroupPrim (LightsDefault.hpp:547-561)
    pl = tr.attribute_info("light", "(L)Prim(P)Triangle")
    assert [(a["name"], a["data_type"]) for a in pl] == [("radiance", "VECTOR_3"), ("isTwoSided", "BOOL")]
    # PathTracerRendererT::StaticAttributeInfo (PathTracerRenderer.cu:1386-1400)
    r = tr.attribute_info("renderer", "(R)PathTracerRGB")
    assert [(a["name"], a["data_type"], a["optional"]) for a in r] == [
        ("totalSPP", "UINT32", False), ("burstSize", "UINT32", True), ("renderMode", "STRING", False),
        ("sampleMode", "STRING", False), ("rrRange", "VECTOR_2UI", False), ("neeSamplerType", "STRING", False)]
    # GuidedPTRenderer::StaticAttributeInfo (GuidedPTRenderer.cu:1273-1292)
    g = tr.attribute_info("renderer", "(R)GuidedPathTracerSpectral")
    assert [(a["name"], a["data_type"], a["optional"]) for a in g] == [
        ("cacheEntryLimit", "UINT32", True), ("cachePosBits", "UINT32", True), ("cacheNormalBits", "UINT32", True),
        ("cacheMaxLvlOffset", "UINT32", True), ("cacheConeAperture", "FLOAT", True),
        ("rrRange", "VECTOR_2UI", False), ("totalSPP", "UINT32", False), ("lightSampler", "STRING", True),
        ("renderMode", "STRING", False), ("burstSize", "UINT32", True), ("lobeProbability", "FLOAT", True),
        ("displayMode", "STRING", False)]
    with pytest.raises(N.MRGError, match="Unable to find type"):
        tr.attribute_info("material", "(Mt)Nope")


def test_ids_and_implicit_groups(tr):
    # implicit groups 0 (TracerBase.cpp:579-600, 905-925, 1010-1035)
    assert tr.create_primitive_group("(P)Empty") == 0
    assert tr.create_transform_group("(T)Identity") == 0
    assert tr.create_light_group("(L)Null") == 0
    assert tr.create_material_group("(Mt)Passthrough") == 0
    pg = tr.create_primitive_group("(P)Triangle")
    assert pg == 1
    b = tr.reserve_primitive_batches(pg, [(2, 4), (12, 8)])
    assert b == [(1 << 28) | 0, (1 << 28) | 1]                 # PrimBatchKey: 4 group bits
    mg = tr.create_material_group("(Mt)Lambert")
    assert mg == 1 and tr.reserve_materials(mg, 3) == [(1 << 21) | i for i in range(3)]   # MaterialKey: 11
    mg2 = tr.create_material_group("(Mt)Unreal")
    assert tr.reserve_materials(mg2, 1) == [2 << 21]
    tg = tr.create_transform_group("(T)Single")
    assert tr.reserve_transformations(tg, 2) == [1 << 24, (1 << 24) | 1]                   # TransformKey: 8
    cg = tr.create_camera_group("(C)Pinhole")
    assert cg == 0 and tr.reserve_cameras(cg, 1) == [0]
    lg = tr.create_light_group("(L)Prim(P)Triangle", pg)
    assert tr.reserve_lights(lg, 1, [b[0]]) == [1 << 21]
    assert tr.type_name("material", mg2) == "(Mt)Unreal"
    assert tr.type_name("light", 0) == "(L)Null"
    r = tr.create_renderer("(R)PathTracerRGB")
    assert r == 0 and tr.type_name("renderer", r) == "(R)PathTracerRGB"
    t0 = tr.create_texture_2d(4, 4)
    assert t0 == 1                                              # 0 = TracerConstants::InvalidTexture


def test_order_rules(tr):
    with pytest.raises(N.MRGError, match="Unable to find generator"):
        tr.create_material_group("(Mt)Disney")
    pg = tr.create_primitive_group("(P)Triangle")
    (b,) = tr.reserve_primitive_batches(pg, [(1, 3)])
    tri = np.zeros((3, 3), np.float32)
    with pytest.raises(N.MRGError, match="not committed"):
        tr.push_prim_attribute(pg, b, POSITION, tri)
    assert not tr.is_prim_committed(pg)
    tr.commit_prim_reservations(pg)
    assert tr.is_prim_committed(pg)
    with pytest.raises(N.MRGError, match="no more reservations"):
        tr.reserve_primitive_batches(pg, [(1, 3)])
    with pytest.raises(N.MRGError, match="already committed"):
        tr.commit_prim_reservations(pg)
    with pytest.raises(N.MRGError, match="wants 36 bytes"):
        tr.push_prim_attribute(pg, b, POSITION, tri[:2])
    with pytest.raises(N.MRGError, match="unknown attribute index"):
        tr.push_prim_attribute(pg, b, 7, tri)
    tr.push_prim_attribute(pg, b, POSITION, tri[:2], sub_range=(0, 2))        # sub-batch pushes
    tr.push_prim_attribute(pg, b, POSITION, tri[2:], sub_range=(2, 3))
    with pytest.raises(N.MRGError, match="outside the batch"):
        tr.push_prim_attribute(pg, b, POSITION, tri[2:], sub_range=(3, 4))
    tr.push_prim_attribute(pg, b, INDEX, np.array([[0, 1, 2]], np.uint32))
    tr.push_prim_attribute(pg, b, UV0, np.zeros((3, 2), np.float32))

    mg = tr.create_material_group("(Mt)Lambert")
    ids = tr.reserve_materials(mg, 2)
    with pytest.raises(N.MRGError, match="not committed"):
        tr.push_mat_attribute(mg, (ids[0], ids[1]), 0, np.ones((2, 3)), [None, None])
    tr.commit_mat_reservations(mg)
    tr.push_mat_attribute(mg, (ids[0], ids[1]), 0, np.ones((2, 3)), [None, None])   # inclusive range
    with pytest.raises(N.MRGError, match="outside the reservations"):
        tr.push_mat_attribute(mg, (ids[0], ids[1] + 1), 0, np.ones((3, 3)), [None] * 3)
    with pytest.raises(N.MRGError, match="takes textures only"):
        tr.push_mat_attribute(mg, (ids[0], ids[0]), 1, np.ones(3))
    with pytest.raises(N.MRGError, match="unknown texture"):
        tr.push_mat_attribute(mg, (ids[0], ids[0]), 0, None, [9])
    rg = tr.create_material_group("(Mt)Refract")
    (rid,) = tr.reserve_materials(rg, 1)
    tr.commit_mat_reservations(rg)
    with pytest.raises(N.MRGError, match="not texturable"):
        tr.push_mat_attribute(rg, (rid, rid), 0, np.ones(3), [None])
    with pytest.raises(N.MRGError, match="outside the group"):
        tr.push_mat_attribute(rg, (ids[0], ids[0]), 0, np.ones(3))

    t = tr.create_texture_2d(2, 2, 1, "rgba8_unorm")
    t8 = tr.create_texture_2d(4, 2, 2, "r8_unorm")
    tf = tr.create_texture_2d(4, 2, 1, "r_float")
    with pytest.raises(N.MRGError, match="before CommitTextures"):
        tr.push_texture_data(t, 0, np.zeros((2, 2, 4), np.uint8))
    tr.commit_textures()
    with pytest.raises(N.MRGError, match="wants 16 bytes"):
        tr.push_texture_data(t, 0, np.zeros((2, 2, 2), np.uint8))
    tr.push_texture_data(t, 0, np.zeros((2, 2, 4), np.uint8))
    # single-channel types: one byte / one float per texel, per level
    with pytest.raises(N.MRGError, match="wants 8 bytes"):
        tr.push_texture_data(t8, 0, np.zeros((2, 4, 4), np.uint8))
    tr.push_texture_data(t8, 0, np.zeros((2, 4), np.uint8))
    tr.push_texture_data(t8, 1, np.zeros((1, 2), np.uint8))
    with pytest.raises(N.MRGError, match="wants 32 bytes"):
        tr.push_texture_data(tf, 0, np.zeros((2, 4), np.uint8))
    tr.push_texture_data(tf, 0, np.zeros((2, 4), np.float32))
    with pytest.raises(N.MRGError, match="no more textures"):
        tr.create_texture_2d(2, 2)

    with pytest.raises(N.MRGError, match="1 to 8"):
        tr.create_surface([b] * 9, [ids[0]] * 9)
    with pytest.raises(N.MRGError, match="alpha maps"):
        tr.create_surface([b], [ids[0]], alpha_maps=[t])
    with pytest.raises(N.MRGError, match="was not reserved"):
        tr.create_surface([b], [ids[1] + 5])
    assert tr.create_surface([b], [ids[0]]) == 0
    pg2 = tr.create_primitive_group("(P)Triangle")
    (b2,) = tr.reserve_primitive_batches(pg2, [(1, 3)])
    with pytest.raises(N.MRGError, match="same type"):
        tr.create_surface([b, b2], [ids[0], ids[1]])
    with pytest.raises(N.MRGError, match="Unable to locate PrimitiveGroup"):
        tr.create_light_group("(L)Prim(P)Triangle", 0)


def test_renderer_options(tr):
    r = tr.create_renderer("(R)PathTracerSpectral")
    tr.push_renderer_attribute(r, 0, 64)
    tr.push_renderer_attribute(r, 1, 4)
    for mode in ("Throughput", "Latency"):
        tr.push_renderer_attribute(r, 2, mode)
    for mode in ("Pure", "WithNextEventEstimation", "WithNEEAndMIS"):
        tr.push_renderer_attribute(r, 3, mode)
    tr.push_renderer_attribute(r, 4, (3, 12))
    tr.push_renderer_attribute(r, 5, "Uniform")
    for idx, bad, msg in ((3, "NEE", "unknown sampleMode"), (2, "Fast", "unknown renderMode"),
                          (5, "PowerWeighted", "Uniform only"), (0, 0, "positive"), (4, (9, 3), "rrRange"),
                          (6, 1, "Unknown attribute index")):
        with pytest.raises(N.MRGError, match=msg):
            tr.push_renderer_attribute(r, idx, bad)
    with pytest.raises(N.MRGError, match="before CommitSurfaces"):
        tr.start_render(r, 0, 16, 16)
    with pytest.raises(N.MRGError, match="without StartRender"):
        tr.do_render_work()
    tr.destroy_renderer(r)
    with pytest.raises(N.MRGError, match="unknown renderer"):
        tr.push_renderer_attribute(r, 0, 1)


def test_guided_renderer_options(tr):
    r = tr.create_renderer("(R)GuidedPathTracerSpectral")
    for idx, v in ((0, 500000), (1, 12), (2, 3), (3, 2), (4, 1.5), (5, (2, 12)), (6, 64), (7, "Uniform"),
                   (8, "Throughput"), (8, "Latency"), (9, 4), (10, 0.5), (11, "Render")):
        tr.push_renderer_attribute(r, idx, v)
    for idx, bad, msg in ((1, 16, "cachePosBits"), (2, 4, "cacheNormalBits"), (0, 0, "cacheEntryLimit"),
                          (4, -1.0, "cacheConeAperture"), (10, 1.5, "lobeProbability"), (5, (9, 3), "rrRange"),
                          (6, 0, "positive"), (7, "PowerWeighted", "Uniform only"), (11, "MCTarget", "only Render"),
                          (8, "Fast", "unknown renderMode"), (12, 1, "Unknown attribute index")):
        with pytest.raises(N.MRGError, match=msg):
            tr.push_renderer_attribute(r, idx, bad)


def test_parameters_and_memory(cuda_lib):
    with Tracer(seed=(7 << 32) | 9, sampler="zsobol", film_filter_radius=1.5, watertight=True) as t:
        p = t.parameters()
        assert p.seed == (7 << 32) | 9 and p.samplerType == N.MRG_TRACER_SAMPLER_ZSOBOL
        assert p.triangleTest == N.MRG_TRI_WATERTIGHT and p.filmFilterRadius == 1.5
        assert t.device_memory() == (0, 0)                       # no device use before the commit
        assert not t.context()
    with Tracer(gen_mips=True, mip_filter_radius=3.0) as t:
        p = t.parameters()
        assert p.genMips == 1 and p.mipGenFilterRadius == 3.0
    with pytest.raises(N.MRGError, match="mip generation filter"):
        Tracer(gen_mips=True, mip_filter_radius=100.0)


def test_scene_json_through_the_tracer(tr):
    """The open-box scene pushed as MRay's loader would: every type and
    attribute accepted, the camera surface's camera equal to the reader's."""
    out = scene_json.load_tracer(tr, os.path.join(HERE, "open_box.json"), commit=False)
    assert out["commit"] is None and out["camera_surfaces"] == [0]
    _, cam, _ = scene_json.read_scene(os.path.join(HERE, "open_box.json"))
    got = tr.get_cam_transform(0)
    want = np.array(list(cam["pos"]) + list(cam["gaze"]) + list(cam["up"]), np.float32)
    assert np.array_equal(got, want)


def test_concurrent_pushes(tr):
    """MRay's loader pushes attributes from its thread pool: pushes of many
    batches from several threads all land."""
    pg = tr.create_primitive_group("(P)Triangle")
    batches = tr.reserve_primitive_batches(pg, [(1, 3)] * 64)
    tr.commit_prim_reservations(pg)
    errs = []

    def work(bs):
        try:
            for b in bs:
                tr.push_prim_attribute(pg, b, POSITION, np.eye(3, dtype=np.float32))
                tr.push_prim_attribute(pg, b, INDEX, np.array([[0, 1, 2]], np.uint32))
        except Exception as e:                                  # pragma: no cover
            errs.append(e)
    th = [threading.Thread(target=work, args=(batches[i::4],)) for i in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errs


def test_commit_without_gpu_fails_cleanly(tr):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    scene_json.load_tracer(tr, os.path.join(HERE, "open_box.json"), commit=False)
    with pytest.raises(N.MRGError):
        tr.commit_surfaces()
    assert not tr.context()
    tr.clear_all()                                              # and the tracer is reusable
    assert tr.create_primitive_group("(P)Triangle") == 1
