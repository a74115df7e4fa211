"""Reader of MRay's JSON scene format (Docs/markdown/scene/mrayScene.md;
loader SceneLoaderMRay.cpp) for the path tracer.

Supported: cameras "Pinhole" (fov in degrees, isFovX, aspect, planes, gaze,
position, up; SceneLoaderMRay.cpp:595-655); transforms "Identity" and
"Single" with layout "matrix" (row-major 4x4) or "trs" (translate * rotZ *
rotY * rotX * scale, degrees; :478-560); primitives "Triangle" with tag
"nodeTriangle" or "nodeTriangleIndexed" (position, optional uv, index);
materials "Lambert" (albedo), "Reflect", "Refract" (cauchyFront /
cauchyBack without dispersion: the A coefficient is the index), "Unreal"
(albedo, roughness, specular, metallic); albedo textures given as numpy
files; lights "Primitive" (radiance), "Null", and boundary skyspheres
"Skysphere_Spherical" with a constant radiance or a numpy radiance map;
surfaces (transform, material / primitive pairs, cullFace), light surfaces
and camera surfaces.  Comments (// and /* */) are stripped; trailing commas
are rejected as MRay does.

Not supported (raises SceneError): sphere primitives (the accelerator holds
triangles), file-backed meshes (assimp / gfg), image textures, media,
normal and alpha maps, multi-transforms.
"""
import json
import math
import os

import numpy as np


class SceneError(ValueError):
    pass


def strip_comments(text):
    """Removes // and /* */ comments outside of strings."""
    out, i, n = [], 0, len(text)
    in_str = False
    while i < n:
        ch = text[i]
        if in_str:
            out.append(ch)
            if ch == "\\" and i + 1 < n:
                out.append(text[i + 1])
                i += 2
                continue
            if ch == '"':
                in_str = False
            i += 1
        elif ch == '"':
            in_str = True
            out.append(ch)
            i += 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            if j < 0:
                raise SceneError("unterminated /* comment")
            i = j + 2
        else:
            out.append(ch)
            i += 1
    return "".join(out)


def load_jsonc(path_or_text):
    text = path_or_text
    if os.path.exists(str(path_or_text)):
        with open(path_or_text) as f:
            text = f.read()
    try:
        return json.loads(strip_comments(text))
    except json.JSONDecodeError as e:
        raise SceneError("scene JSON: %s" % e) from None


def _items(group):
    """Expands a type-group list into {id: (type, attributes)}; arrayed
    structs (id arrays) spread their attribute arrays."""
    out = {}
    for st in group:
        ids, typ = st.get("id"), st.get("type")
        if ids is None or typ is None:
            raise SceneError("every struct needs an 'id' and a 'type'")
        if isinstance(ids, list):
            for k, i in enumerate(ids):
                attrs = {}
                for key, val in st.items():
                    if key in ("id", "type"):
                        continue
                    attrs[key] = val[k] if isinstance(val, list) and len(val) == len(ids) and key not in (
                        "position", "uv", "index", "normal") else val
                out[int(i)] = (typ, attrs)
        else:
            out[int(ids)] = (typ, {k: v for k, v in st.items() if k not in ("id", "type")})
    return out


def _rot(axis, deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4)
    if axis == 0:
        m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, -s, s, c
    elif axis == 1:
        m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    else:
        m[0, 0], m[0, 1], m[1, 0], m[1, 1] = c, -s, s, c
    return m


def _transform(transforms, tid):
    if tid is None:
        return np.eye(4)
    if int(tid) not in transforms:
        raise SceneError("unknown transform %s" % tid)
    typ, a = transforms[int(tid)]
    if typ == "Identity":
        return np.eye(4)
    if typ != "Single":
        raise SceneError("transform type %s is not supported" % typ)
    layout = a.get("layout")
    if layout == "matrix":
        m = np.asarray(a["matrix"], np.float64).reshape(4, 4)
        return m
    if layout == "trs":
        t = np.asarray(a.get("translate", [0, 0, 0]), np.float64)
        r = np.asarray(a.get("rotate", [0, 0, 0]), np.float64)
        s = np.asarray(a.get("scale", [1, 1, 1]), np.float64)
        m = np.diag([s[0], s[1], s[2], 1.0])
        m = _rot(0, r[0]) @ m
        m = _rot(1, r[1]) @ m
        m = _rot(2, r[2]) @ m
        tr = np.eye(4)
        tr[:3, 3] = t
        return tr @ m
    raise SceneError("transform layout %s is not supported" % layout)


def _mesh(prims, pid, base_dir):
    if int(pid) not in prims:
        raise SceneError("unknown primitive %s" % pid)
    typ, a = prims[int(pid)]
    if typ != "Triangle":
        raise SceneError("primitive type %s is not supported (triangles only)" % typ)
    tag = a.get("tag")
    pos = np.asarray(a.get("position", []), np.float32).reshape(-1, 3)
    uv = np.asarray(a["uv"], np.float32).reshape(-1, 2) if "uv" in a else None
    if tag == "nodeTriangleIndexed":
        idx = np.asarray(a["index"], np.uint32).reshape(-1, 3)
    elif tag == "nodeTriangle":
        if pos.shape[0] % 3:
            raise SceneError("nodeTriangle positions must come in threes")
        idx = np.arange(pos.shape[0], dtype=np.uint32).reshape(-1, 3)
    else:
        raise SceneError("primitive tag %s is not supported" % tag)
    if idx.size and idx.max() >= pos.shape[0]:
        raise SceneError("primitive %s: index out of range" % pid)
    return pos, idx, uv


def _texture(textures, ref, base_dir):
    tid = int(ref["texture"])
    if tid not in textures:
        raise SceneError("unknown texture %d" % tid)
    _, a = textures[tid]
    f = a.get("file", "")
    if not f.endswith(".npy"):
        raise SceneError("texture %d: only numpy (.npy) textures are supported" % tid)
    t = np.load(os.path.join(base_dir, f))
    if t.ndim != 3 or t.shape[2] != 4:
        raise SceneError("texture %d must be (h, w, 4)" % tid)
    return np.ascontiguousarray(t)


def _material(materials, textures, mid, base_dir):
    if int(mid) not in materials:
        raise SceneError("unknown material %s" % mid)
    typ, a = materials[int(mid)]
    d = dict(kind="lambert", albedo=[0.5, 0.5, 0.5])
    alb = a.get("albedo", [0.5, 0.5, 0.5])
    if isinstance(alb, dict):
        d["texture"] = _texture(textures, alb, base_dir)
    elif alb != "-":
        d["albedo"] = [float(x) for x in alb]
    if typ == "Lambert":
        d["material"] = "lambert"
    elif typ == "Reflect":
        d["material"] = "reflect"
    elif typ == "Refract":
        front = a.get("cauchyFront", [1.0, 0.0, 0.0])
        back = a.get("cauchyBack", [1.0, 0.0, 0.0])
        if front[1] or front[2] or back[1] or back[2]:
            raise SceneError("material %s: dispersive Cauchy coefficients are not supported" % mid)
        d.update(material="refract", ior=(float(front[0]), float(back[0])))
    elif typ == "Unreal":
        d.update(material="unreal", roughness=float(a.get("roughness", 0.5)), metallic=float(a.get("metallic", 0.0)),
                 specular=float(a.get("specular", 0.5)))
    else:
        raise SceneError("material type %s is not supported" % typ)
    return d


def _m34(m):
    return np.asarray(m[:3, :4], np.float32).reshape(12)


def read_scene(path_or_text, base_dir=None):
    """Returns (surfaces, camera, env): surfaces in the dict form the path
    tracer and its oracle load (one per material / primitive pair and light
    surface), the first camera surface as a camera dict, and the boundary
    skysphere as {"texels": (h, w, 4) float32} or None."""
    j = load_jsonc(path_or_text)
    base_dir = base_dir or (os.path.dirname(os.path.abspath(path_or_text)) if os.path.exists(str(path_or_text))
                            else os.getcwd())
    for key in ("Cameras", "Lights", "Mediums", "Transforms", "Textures", "Materials", "Primitives", "Boundary",
                "Surfaces", "LightSurfaces", "CameraSurfaces"):
        if key not in j:
            raise SceneError("scene JSON lacks '%s'" % key)
    cams, lights = _items(j["Cameras"]), _items(j["Lights"])
    transforms, textures = _items(j["Transforms"]), _items(j["Textures"])
    materials, prims = _items(j["Materials"]), _items(j["Primitives"])
    surfaces = []
    for s in j["Surfaces"]:
        m = _transform(transforms, s.get("transform"))
        mats = s["material"] if isinstance(s["material"], list) else [s["material"]]
        pids = s["primitive"] if isinstance(s["primitive"], list) else [s["primitive"]]
        if len(mats) != len(pids):
            raise SceneError("surface material / primitive counts differ")
        culls = s.get("cullFace", True)
        culls = culls if isinstance(culls, list) else [culls] * len(pids)
        if "alphaMap" in s and any(x != "-" for x in (s["alphaMap"] if isinstance(s["alphaMap"], list)
                                                       else [s["alphaMap"]])):
            raise SceneError("alpha maps are not supported")
        for mid, pid, cull in zip(mats, pids, culls):
            pos, idx, uv = _mesh(prims, pid, base_dir)
            d = _material(materials, textures, mid, base_dir)
            if "texture" in d and uv is None:
                raise SceneError("primitive %s has a textured material but no uv" % pid)
            d.update(pos=pos, idx=idx, m34=_m34(m), cull=bool(cull))
            if uv is not None:
                d["uv"] = uv
            surfaces.append(d)
    for ls in j["LightSurfaces"]:
        lid = int(ls["light"])
        if lid not in lights:
            raise SceneError("unknown light %d" % lid)
        typ, a = lights[lid]
        if typ != "Primitive":
            raise SceneError("light surface type %s is not supported" % typ)
        pos, idx, _ = _mesh(prims, a["primitive"], base_dir)
        rad = a.get("radiance", [1, 1, 1])
        if isinstance(rad, dict):
            raise SceneError("textured area-light radiance is not supported")
        m = _transform(transforms, ls.get("transform"))
        # light surfaces are not back-face culled (AcceleratorCommon.cu:345-365)
        surfaces.append(dict(pos=pos, idx=idx, m34=_m34(m), kind="light", radiance=[float(x) for x in rad],
                             cull=False))
    # boundary light
    env = None
    b = j["Boundary"]
    btyp, ba = lights.get(int(b["light"]), (None, None))
    if btyp is None:
        raise SceneError("unknown boundary light")
    if btyp.startswith("Skysphere"):
        if btyp not in ("Skysphere_Spherical", "Skysphere"):
            raise SceneError("boundary light %s is not supported (spherical mapping only)" % btyp)
        rad = ba.get("radiance", [1, 1, 1])
        if isinstance(rad, dict):
            tex = _texture(textures, rad, base_dir)
            tex = tex.astype(np.float32) / 255.0 if tex.dtype == np.uint8 else tex.astype(np.float32)
        else:
            tex = np.ones((1, 1, 4), np.float32)
            tex[0, 0, :3] = [float(x) for x in rad]
        bm = _transform(transforms, b.get("transform"))
        env = dict(texels=tex, m34=_m34(bm))
    elif btyp != "Null":
        raise SceneError("boundary light %s is not supported" % btyp)
    # camera
    cs = j["CameraSurfaces"][0]
    ctyp, ca = cams.get(int(cs["camera"]), (None, None))
    if ctyp != "Pinhole":
        raise SceneError("camera type %s is not supported" % ctyp)
    fx, fy, near, far = _camera_fnp(ca)
    cm = _transform(transforms, cs.get("transform"))
    pos = cm @ np.append(np.asarray(ca["position"], np.float64), 1.0)
    gaze = cm @ np.append(np.asarray(ca["gaze"], np.float64), 1.0)
    up = cm[:3, :3] @ np.asarray(ca["up"], np.float64)
    camera = dict(pos=tuple(pos[:3]), gaze=tuple(gaze[:3]), up=tuple(up), fov=(fx, fy), near_far=(near, far))
    return surfaces, camera, env


def _camera_fnp(ca):
    """FovAndPlanes of a pinhole camera node (SceneLoaderMRay.cpp:626-644):
    fov in radians on both axes from fov, isFovX and aspect, then the planes."""
    fov = math.radians(float(ca["fov"]))
    aspect = float(ca.get("aspect", 1.0))
    if ca.get("isFovX", True):
        fx, fy = fov, 2.0 * math.atan(math.tan(fov * 0.5) / aspect)
    else:
        fy, fx = fov, 2.0 * math.atan(math.tan(fov * 0.5) * aspect)
    planes = ca.get("planes", [0.01, 1000.0])
    return [fx, fy, float(planes[0]), float(planes[1])]


def load_tracer(tracer, path_or_text, base_dir=None, commit=True):
    """Pushes a scene through the TracerI calls of a mray_gb300.tracer.Tracer
    the way MRay's SceneLoaderMRay does (SceneLoaderMRay.cpp: one group per
    type, reservations, commits, attribute pushes, then surfaces, light
    surfaces, the boundary and camera surfaces) and commits the surfaces.
    Only what the surfaces reference is loaded.  The type mapping (materials,
    lights, defaults) happens behind the tracer's C ABI.  Returns
    {"camera_surfaces": [ids], "commit": commit result or None}; commit=False
    stops before the surface commit (the first call that needs the device)."""
    j = load_jsonc(path_or_text)
    base_dir = base_dir or (os.path.dirname(os.path.abspath(path_or_text)) if os.path.exists(str(path_or_text))
                            else os.getcwd())
    for key in ("Cameras", "Lights", "Mediums", "Transforms", "Textures", "Materials", "Primitives", "Boundary",
                "Surfaces", "LightSurfaces", "CameraSurfaces"):
        if key not in j:
            raise SceneError("scene JSON lacks '%s'" % key)
    cams, lights = _items(j["Cameras"]), _items(j["Lights"])
    transforms, textures = _items(j["Transforms"]), _items(j["Textures"])
    materials, prims = _items(j["Materials"]), _items(j["Primitives"])

    def lst(v):
        return v if isinstance(v, list) else [v]

    # what the surfaces reference
    used_mats, used_prims, used_trans = set(), set(), set()
    for sf in j["Surfaces"]:
        used_mats.update(int(m) for m in lst(sf["material"]))
        used_prims.update(int(p) for p in lst(sf["primitive"]))
        used_trans.add(int(sf.get("transform", 0)))
        if "alphaMap" in sf and any(x != "-" for x in lst(sf["alphaMap"])):
            raise SceneError("alpha maps are not supported")
    used_lights = [int(ls["light"]) for ls in j["LightSurfaces"]]
    used_trans.update(int(ls.get("transform", 0)) for ls in j["LightSurfaces"])
    b = j["Boundary"]
    used_trans.add(int(b.get("transform", 0)))
    used_trans.update(int(cs.get("transform", 0)) for cs in j["CameraSurfaces"])
    for lid in used_lights:
        if lid not in lights:
            raise SceneError("unknown light %d" % lid)
        if lights[lid][0] != "Primitive":
            raise SceneError("light surface type %s is not supported" % lights[lid][0])
        used_prims.add(int(lights[lid][1]["primitive"]))

    # textures: created now, their data pushed after CommitTextures
    tex_pending, tex_map = [], {}

    def texture(ref):
        tid = int(ref["texture"])
        if tid not in tex_map:
            t = _texture(textures, ref, base_dir)
            kind = "rgba8_unorm" if t.dtype == np.uint8 else "rgba_float"
            tex_map[tid] = tracer.create_texture_2d(t.shape[1], t.shape[0], 1, kind)
            tex_pending.append((tex_map[tid], np.ascontiguousarray(t if t.dtype == np.uint8 else t.astype(np.float32))))
        return tex_map[tid]

    # transforms: (T)Identity is the implicit transform 0
    trans_ids, singles = {}, []
    for tid in sorted(used_trans):
        if tid not in transforms:
            raise SceneError("unknown transform %s" % tid)
        typ = transforms[tid][0]
        if typ == "Identity":
            trans_ids[tid] = 0
        elif typ == "Single":
            singles.append(tid)
        else:
            raise SceneError("transform type %s is not supported" % typ)
    if singles:
        g = tracer.create_transform_group("(T)Single")
        for tid, nid in zip(singles, tracer.reserve_transformations(g, len(singles))):
            trans_ids[tid] = nid
        tracer.commit_trans_reservations(g)
        for tid in singles:
            m = np.asarray(_transform(transforms, tid), np.float32).reshape(16)
            tracer.push_trans_attribute(g, (trans_ids[tid], trans_ids[tid]), 0, m)

    # primitives: one (P)Triangle group, a batch per primitive
    from .tracer import INDEX, POSITION, UV0
    meshes = {pid: _mesh(prims, pid, base_dir) for pid in sorted(used_prims)}
    pg = tracer.create_primitive_group("(P)Triangle")
    order = sorted(meshes)
    batch = dict(zip(order, tracer.reserve_primitive_batches(
        pg, [(meshes[p][1].shape[0], meshes[p][0].shape[0]) for p in order])))
    tracer.commit_prim_reservations(pg)
    for pid in order:
        pos, idx, uv = meshes[pid]
        tracer.push_prim_attribute(pg, batch[pid], POSITION, pos)
        tracer.push_prim_attribute(pg, batch[pid], INDEX, idx)
        if uv is not None:
            tracer.push_prim_attribute(pg, batch[pid], UV0, uv)

    # materials: a group per type
    by_type = {}
    for mid in sorted(used_mats):
        if mid not in materials:
            raise SceneError("unknown material %s" % mid)
        by_type.setdefault(materials[mid][0], []).append(mid)
    mat_ids = {}
    for typ, mids in by_type.items():
        if typ not in ("Lambert", "Reflect", "Refract", "Unreal"):
            raise SceneError("material type %s is not supported" % typ)
        g = tracer.create_material_group("(Mt)" + typ)
        for mid, nid in zip(mids, tracer.reserve_materials(g, len(mids))):
            mat_ids[mid] = nid
        tracer.commit_mat_reservations(g)
        for mid in mids:
            a, r = materials[mid][1], (mat_ids[mid], mat_ids[mid])
            if typ in ("Lambert", "Unreal"):
                alb = a.get("albedo", [0.5, 0.5, 0.5])
                if isinstance(alb, dict):
                    tracer.push_mat_attribute(g, r, 0, None, [texture(alb)])
                else:
                    tracer.push_mat_attribute(g, r, 0, [0.5, 0.5, 0.5] if alb == "-" else alb, [None])
            if typ == "Unreal":
                for k, (name, dflt) in enumerate((("roughness", 0.5), ("specular", 0.5), ("metallic", 0.0))):
                    v = a.get(name, dflt)
                    if isinstance(v, dict):
                        raise SceneError("material %s: textured %s is not supported" % (mid, name))
                    tracer.push_mat_attribute(g, r, 2 + k, [float(v)], [None])
            if typ == "Refract":
                tracer.push_mat_attribute(g, r, 0, a.get("cauchyBack", [1.0, 0.0, 0.0]))
                tracer.push_mat_attribute(g, r, 1, a.get("cauchyFront", [1.0, 0.0, 0.0]))

    # lights: primitive-backed ones in one group, the boundary light
    light_ids = {}
    prim_lights = sorted(set(used_lights))
    if prim_lights:
        g = tracer.create_light_group("(L)Prim(P)Triangle", pg)
        ids = tracer.reserve_lights(g, len(prim_lights), [batch[int(lights[l][1]["primitive"])] for l in prim_lights])
        light_ids.update(zip(prim_lights, ids))
        tracer.commit_light_reservations(g)
        for lid in prim_lights:
            a = lights[lid][1]
            rad = a.get("radiance", [1, 1, 1])
            if isinstance(rad, dict):
                raise SceneError("textured area-light radiance is not supported")
            r = (light_ids[lid], light_ids[lid])
            tracer.push_light_attribute(g, r, 0, rad, [None])
            tracer.push_light_attribute(g, r, 1, [1 if a.get("isTwoSided", False) else 0], dtype=np.uint8)
    blid = int(b["light"])
    if blid not in lights:
        raise SceneError("unknown boundary light")
    btyp, ba = lights[blid]
    if btyp == "Null":
        boundary_light = 0
    elif btyp in ("Skysphere_Spherical", "Skysphere"):
        g = tracer.create_light_group("(L)Skysphere_Spherical")
        boundary_light = tracer.reserve_lights(g, 1)[0]
        tracer.commit_light_reservations(g)
        rad = ba.get("radiance", [1, 1, 1])
        r = (boundary_light, boundary_light)
        if isinstance(rad, dict):
            tracer.push_light_attribute(g, r, 0, None, [texture(rad)])
        else:
            tracer.push_light_attribute(g, r, 0, rad, [None])
    else:
        raise SceneError("boundary light %s is not supported" % btyp)

    # cameras
    cam_used = sorted({int(cs["camera"]) for cs in j["CameraSurfaces"]})
    cam_ids = {}
    if cam_used:
        for cid in cam_used:
            if cams.get(cid, (None,))[0] != "Pinhole":
                raise SceneError("camera type %s is not supported" % cams.get(cid, (None,))[0])
        g = tracer.create_camera_group("(C)Pinhole")
        cam_ids = dict(zip(cam_used, tracer.reserve_cameras(g, len(cam_used))))
        tracer.commit_cam_reservations(g)
        for cid in cam_used:
            ca, r = cams[cid][1], (cam_ids[cid], cam_ids[cid])
            tracer.push_cam_attribute(g, r, 0, _camera_fnp(ca))
            tracer.push_cam_attribute(g, r, 1, ca["gaze"])
            tracer.push_cam_attribute(g, r, 2, ca["position"])
            tracer.push_cam_attribute(g, r, 3, ca["up"])

    tracer.commit_textures()
    for tid, data in tex_pending:
        tracer.push_texture_data(tid, 0, data)

    # surfaces, light surfaces, boundary, camera surfaces
    for sf in j["Surfaces"]:
        mats, pids = lst(sf["material"]), lst(sf["primitive"])
        if len(mats) != len(pids):
            raise SceneError("surface material / primitive counts differ")
        culls = sf.get("cullFace", True)
        culls = culls if isinstance(culls, list) else [culls] * len(pids)
        tracer.create_surface([batch[int(p)] for p in pids], [mat_ids[int(m)] for m in mats],
                              trans_ids[int(sf.get("transform", 0))], culls)
    for ls in j["LightSurfaces"]:
        tracer.create_light_surface(light_ids[int(ls["light"])], trans_ids[int(ls.get("transform", 0))])
    tracer.set_boundary_surface(boundary_light, trans_ids[int(b.get("transform", 0))])
    cam_surfaces = [tracer.create_camera_surface(cam_ids[int(cs["camera"])], trans_ids[int(cs.get("transform", 0))])
                    for cs in j["CameraSurfaces"]]
    return {"camera_surfaces": cam_surfaces, "commit": tracer.commit_surfaces() if commit else None}


def load(pt, path_or_text, base_dir=None):
    """Reads a scene into a mray_gb300.pt.PathTracer (built); returns the
    camera and the surface list."""
    from .pt import load_box_scene
    surfaces, camera, env = read_scene(path_or_text, base_dir)
    load_box_scene(pt, surfaces)
    if env is not None:
        pt.set_env(env["texels"], env["m34"])
    return camera, surfaces
