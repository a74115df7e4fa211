"""Seeded synthetic workloads (numpy front end of libmrg_scenes.so).

``bvh_stress_scene`` is the 1.31M-triangle displaced icosphere instanced 64
times with rigid transforms inside a 100^3 cube; ``primary_rays`` /
``bounce_rays`` build its 1920x1080 primary + one-diffuse-bounce ray set.
All generators use only IEEE basic operations, so the same seed gives the same
bits on every host.
"""
import ctypes as C

import numpy as np

from . import _native as N

FLT_MAX = np.float32(3.4028235e38)

# 1.31M-triangle stress scene
STRESS_LEVEL = 8              # 20 * 4^8 = 1,310,720 triangles
STRESS_RADIUS = 11.0
STRESS_NOISE_AMP = 0.05       # relative to the radius, 3-octave value noise
STRESS_NOISE_FREQ = 4.0
STRESS_INSTANCES = 64
STRESS_BOX = 100.0
STRESS_JITTER = 1.5
STRESS_EYE = (0.0, 0.0, -90.0)
STRESS_TARGET = (0.0, 0.0, 0.0)
STRESS_UP = (0.0, 1.0, 0.0)
STRESS_TAN_HALF_FOV = 0.5


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


def icosphere(level, radius=1.0, noise_amp=0.0, noise_freq=4.0, seed=0):
    s = N.scenes_lib()
    nv, nt = C.c_uint32(), C.c_uint32()
    s.mrgs_icosphere_counts(level, C.byref(nv), C.byref(nt))
    pos = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.uint32)
    rc = s.mrgs_icosphere(level, radius, noise_amp, noise_freq, seed, _vp(pos), _vp(idx))
    if rc != 0:
        raise RuntimeError("icosphere generation failed (%d)" % rc)
    return pos, idx


def instance_field(count, seed=0, box=STRESS_BOX, jitter=STRESS_JITTER):
    m = np.empty((count, 12), np.float32)
    N.scenes_lib().mrgs_instance_field(count, seed, box, jitter, _vp(m))
    return m


def bvh_stress_scene(level=STRESS_LEVEL, instances=STRESS_INSTANCES, seed=0):
    """(pos, idx, transforms) of the displaced-icosphere instance field."""
    pos, idx = icosphere(level, STRESS_RADIUS, STRESS_NOISE_AMP, STRESS_NOISE_FREQ, seed)
    m = instance_field(instances, seed)
    return pos, idx, m


def primary_rays(width, height, seed=0, eye=STRESS_EYE, target=STRESS_TARGET, up=STRESS_UP,
                 tan_half_fov=STRESS_TAN_HALF_FOV):
    rays = np.empty((width * height, 8), np.float32)
    N.scenes_lib().mrgs_primary_rays(width, height, _d3(eye), _d3(target), _d3(up),
                                     tan_half_fov, seed, _vp(rays))
    return rays


def bounce_rays(primary, hit_inst, hit_prim, hit_t, pos, idx, m34, seed=0):
    """One cosine-weighted diffuse ray per primary hit.  Returns (rays, src)."""
    n = primary.shape[0]
    out = np.empty((n, 8), np.float32)
    src = np.empty(n, np.uint32)
    hi = np.ascontiguousarray(hit_inst, np.uint32)
    hp = np.ascontiguousarray(hit_prim, np.uint32)
    ht = np.ascontiguousarray(hit_t, np.float32)
    m = N.scenes_lib().mrgs_bounce_rays(n, _vp(primary), _vp(hi), _vp(hp), _vp(ht),
                                        _vp(np.ascontiguousarray(pos, np.float32)),
                                        _vp(np.ascontiguousarray(idx, np.uint32)),
                                        _vp(np.ascontiguousarray(m34, np.float32)),
                                        seed, _vp(out), _vp(src))
    return out[:m].copy(), src[:m].copy()


def shadow_rays(origins, light):
    out = np.empty_like(origins)
    N.scenes_lib().mrgs_shadow_rays(origins.shape[0], _vp(origins), _d3(light), _vp(out))
    return out


# ---------------------------------------------------------------------------
# Box scene (the small path-tracing configuration): five inward-facing walls
# of the unit cube, two boxes rotated about y by seeded angles, one ceiling
# quad light with radiance 15, Lambert albedos uniform in [0.1, 0.8]^3.
# ---------------------------------------------------------------------------
def _hash32(x):
    x &= 0xFFFFFFFF
    x ^= x >> 16; x = (x * 0x7feb352d) & 0xFFFFFFFF
    x ^= x >> 15; x = (x * 0x846ca68b) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def _u01(seed, i):
    return _hash32(_hash32(seed * 0x9E3779B9 + 0x1234567) ^ (i * 0x85EBCA6B)) / 4294967296.0


def _quad(o, u, v):
    o, u, v = (np.asarray(a, np.float64) for a in (o, u, v))
    pos = np.array([o, o + u, o + u + v, o + v], np.float64)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    return pos, idx


def _box(w, h, d):
    faces = [((0.5, -0.5, -0.5), (0, 1, 0), (0, 0, 1)), ((-0.5, -0.5, -0.5), (0, 0, 1), (0, 1, 0)),
             ((-0.5, 0.5, -0.5), (0, 0, 1), (1, 0, 0)), ((-0.5, -0.5, -0.5), (1, 0, 0), (0, 0, 1)),
             ((-0.5, -0.5, 0.5), (1, 0, 0), (0, 1, 0)), ((-0.5, -0.5, -0.5), (0, 1, 0), (1, 0, 0))]
    P, I = [], []
    for k, (o, u, v) in enumerate(faces):
        p, i = _quad(o, u, v)
        P.append(p)
        I.append(i + 4 * k)
    s = np.array([w, h, d], np.float64)
    return np.vstack(P) * s, np.vstack(I)


def box_scene(seed=0):
    """Surfaces of the box scene: list of dicts with pos, idx, m34, kind
    ("lambert" / "light"), albedo or radiance.  36 triangles in total."""
    I34 = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    walls = [((0, 0, 0), (0, 0, 1), (1, 0, 0)),      # floor, +y
             ((0, 1, 0), (1, 0, 0), (0, 0, 1)),      # ceiling, -y
             ((0, 0, 1), (0, 1, 0), (1, 0, 0)),      # back, -z
             ((0, 0, 0), (0, 1, 0), (0, 0, 1)),      # left, +x
             ((1, 0, 0), (0, 0, 1), (0, 1, 0))]      # right, -x
    out = []
    k = 0
    for o, u, v in walls:
        p, i = _quad(o, u, v)
        alb = [0.1 + 0.7 * _u01(seed, 3 * k + j) for j in range(3)]
        out.append(dict(pos=p.astype(np.float32), idx=i, m34=I34.copy(), kind="lambert", albedo=alb))
        k += 1
    # boxes float 1e-3 above the floor: coplanar faces would make exact-t ties
    # whose winner depends on traversal order
    for size, at in (((0.28, 0.6, 0.28), (0.33, 0.301, 0.62)), ((0.28, 0.28, 0.28), (0.68, 0.141, 0.35))):
        p, i = _box(*size)
        t = 2.0 * _u01(seed, 100 + k) - 1.0
        c, s = (1 - t * t) / (1 + t * t), 2 * t / (1 + t * t)
        m = np.array([c, 0, s, at[0], 0, 1, 0, at[1], -s, 0, c, at[2]], np.float32)
        alb = [0.1 + 0.7 * _u01(seed, 3 * k + j) for j in range(3)]
        out.append(dict(pos=p.astype(np.float32), idx=i, m34=m, kind="lambert", albedo=alb))
        k += 1
    p, i = _quad((0.35, 0.999, 0.35), (0.3, 0, 0), (0, 0, 0.3))
    out.append(dict(pos=p.astype(np.float32), idx=i, m34=I34.copy(), kind="light",
                    radiance=[15.0, 15.0, 15.0]))
    return out


def box_scene_mixed(seed=0):
    """Box scene with every material group: the tall box GGX metal (Unreal,
    metallic 1, roughness 0.3), the short box glass (Refract, IoR 1.5, no
    back-face culling), the back wall a rough dielectric-coated Unreal
    surface (metallic 0, roughness 0.5), the left wall a mirror."""
    s = box_scene(seed)
    s[2].update(material="unreal", roughness=0.5, metallic=0.0, specular=0.5)
    s[3].update(material="reflect")
    s[5].update(material="unreal", roughness=0.3, metallic=1.0, specular=0.5)
    s[6].update(material="refract", ior=(1.0, 1.5), cull=False)
    return s


def sky_map(width=64, height=32, seed=0, sun=(0.3, 0.8), sun_radiance=40.0):
    """Seeded lat-long sky radiance, (height, width, 4) float32 RGBA rounded
    through float16 (a half-float HDR map): a blue gradient above the horizon,
    dim ground below, a small bright sun disc at uv = sun and +-10% value
    noise.  Every texel is positive, so no row of the sampling distribution is
    empty.  Row 0 is v = 0 (straight down)."""
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    V, U = np.meshgrid(v, u, indexing="ij")
    up = np.clip((V - 0.5) * 2.0, 0.0, 1.0)
    rgb = np.empty((height, width, 3), np.float64)
    sky = np.stack([0.35 + 0.25 * (1 - up), 0.55 + 0.2 * (1 - up), 0.95 + 0.0 * up], -1) * 1.5
    ground = np.stack([0.25 + 0 * V, 0.2 + 0 * V, 0.15 + 0 * V], -1)
    rgb[:] = np.where((V >= 0.5)[..., None], sky, ground)
    du = np.minimum(np.abs(U - sun[0]), 1.0 - np.abs(U - sun[0]))
    d2 = (du * 2.0) ** 2 + (V - sun[1]) ** 2
    rgb += sun_radiance * np.exp(-d2 / (2 * 0.03 ** 2))[..., None] * np.array([1.0, 0.9, 0.75])
    noise = np.array([_u01(seed, 7919 + i) for i in range(height * width)]).reshape(height, width)
    rgb *= (0.9 + 0.2 * noise)[..., None]
    rgb = np.maximum(rgb, 0.02)
    out = np.ones((height, width, 4), np.float32)
    out[..., :3] = rgb.astype(np.float16).astype(np.float32)
    return out


def sky_scene(seed=0):
    """Open variant of the box scene lit by a sky: floor, left wall, the GGX
    metal tall box, the Lambert short box and the ceiling light quad; the
    ceiling, back and right walls are left out, so paths leave the scene and
    camera rays see the sky."""
    s = box_scene(seed)
    s[5].update(material="unreal", roughness=0.3, metallic=1.0, specular=0.5)
    return [s[0], s[3], s[5], s[6], s[7]]


def value_noise_texture(size=256, seed=0, octaves=4, base=0.15, span=0.7, dtype=np.uint8):
    """Seeded RGBA texture of fractal gradient ("Perlin") noise, one
    independent field per colour channel, mapped to [base, base + span];
    uint8 (RGBA8, alpha 255) or float32 (alpha 1).  Tileable (wraps)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((size, size, 3), np.float64)
    y, x = np.meshgrid(np.arange(size) / size, np.arange(size) / size, indexing="ij")
    for c in range(3):
        acc = np.zeros((size, size))
        amp, total = 1.0, 0.0
        for o in range(octaves):
            cells = 4 << o
            ang = rng.random((cells, cells)) * 2 * np.pi
            gx, gy = np.cos(ang), np.sin(ang)
            fx, fy = x * cells, y * cells
            ix, iy = np.floor(fx).astype(np.int64), np.floor(fy).astype(np.int64)
            tx, ty = fx - ix, fy - iy

            def dot(ox, oy):
                cx, cy = (ix + ox) % cells, (iy + oy) % cells
                return gx[cy, cx] * (tx - ox) + gy[cy, cx] * (ty - oy)
            sx = tx * tx * tx * (tx * (tx * 6 - 15) + 10)
            sy = ty * ty * ty * (ty * (ty * 6 - 15) + 10)
            top = dot(0, 0) * (1 - sx) + dot(1, 0) * sx
            bot = dot(0, 1) * (1 - sx) + dot(1, 1) * sx
            acc += amp * (top * (1 - sy) + bot * sy)
            total += amp
            amp *= 0.5
        out[..., c] = np.clip(0.5 + acc / total, 0.0, 1.0)
    val = base + span * out
    if dtype == np.uint8:
        t = np.full((size, size, 4), 255, np.uint8)
        t[..., :3] = np.round(val * 255.0).astype(np.uint8)
        return t
    t = np.ones((size, size, 4), np.float32)
    t[..., :3] = val.astype(np.float32)
    return t


def quad_uv():
    """Texture coordinates of _quad's four corners."""
    return np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)


def box_scene_textured(seed=0, size=256):
    """Box scene with RGBA8 noise textures on the floor, back and left walls
    (two textures, one shared) and per-vertex uvs on every quad."""
    s = box_scene(seed)
    t0 = value_noise_texture(size, seed)
    t1 = value_noise_texture(size, seed + 1)
    for k, tex in ((0, t0), (2, t1), (3, t0)):
        s[k]["uv"] = quad_uv() * 2.0            # two repeats: exercises wrapping
        s[k]["texture"] = tex
    return s


def box_scene_unreal_textured(seed=0, size=64):
    """The textured box with its back wall and floor made Unreal (GGX) with
    textured roughness, metallic and specular (RGBA8 noise, first channel
    used) beside their textured albedos."""
    s = box_scene_textured(seed, size)
    rough = value_noise_texture(size, seed + 7, base=0.05, span=0.6)
    metal = value_noise_texture(size, seed + 8, base=0.0, span=1.0)
    spec = value_noise_texture(size, seed + 9, base=0.2, span=0.6)
    for k in (0, 2):
        s[k].update(material="unreal", roughness=0.3, metallic=0.2, specular=0.5, roughness_texture=rough,
                    metallic_texture=metal, specular_texture=spec)
    return s


def mipmapped(surf, radius=2.0):
    """Marks every textured surface's texture for a mip chain of the given
    filter radius (MRay's texture-load option, read at the ray cone's level
    of detail); returns the surface list."""
    for s in surf:
        if s.get("texture") is not None:
            s["mip_radius"] = float(radius)
    return surf


def uv_sphere(n_theta=128, n_phi=256, radius=1.0, noise=0.0, seed=0):
    """Latitude-longitude sphere with (n_theta - 1) * n_phi * 2 triangles
    plus the pole fans (2 * n_phi), uv = (phi / 2pi, theta / pi); optional
    smooth radial displacement of amplitude noise * radius."""
    th = np.linspace(0.0, np.pi, n_theta + 1)
    ph = np.linspace(0.0, 2 * np.pi, n_phi + 1)
    T, Pp = np.meshgrid(th, ph, indexing="ij")
    rng = np.random.default_rng(seed)
    r = np.full(T.shape, radius)
    if noise:
        for k in range(1, 4):
            a, b, c = rng.random(3) * 2 * np.pi
            r += noise * radius / k * np.sin(k * 3 * T + a) * np.cos(k * 2 * Pp + b + c)
        r[:, -1] = r[:, 0]
    pos = np.stack([r * np.sin(T) * np.cos(Pp), r * np.cos(T), r * np.sin(T) * np.sin(Pp)], -1).reshape(-1, 3)
    uv = np.stack([Pp / (2 * np.pi), T / np.pi], -1).reshape(-1, 2)
    W = n_phi + 1
    idx = []
    for i in range(n_theta):
        for j in range(n_phi):
            a, b, c, d = i * W + j, i * W + j + 1, (i + 1) * W + j + 1, (i + 1) * W + j
            if i != 0:
                idx.append((a, c, b))
            if i != n_theta - 1:
                idx.append((a, d, c))
    return pos.astype(np.float32), np.array(idx, np.uint32), uv.astype(np.float32)


def adjoint_scene(texture, seed=0, n_theta=128, n_phi=256, noise=0.03):
    """The box scene plus a displaced lat-long sphere (radius 0.15 at
    (0.35, 0.2, 0.25), clear of both boxes; 65,024 triangles at the default
    resolution) whose Lambert albedo is `texture` (an f32 RGBA array or
    tensor): the differentiable-rendering workload."""
    s = box_scene(seed)
    pos, idx, uv = uv_sphere(n_theta, n_phi, 0.15, noise=noise, seed=seed)
    m = np.array([1, 0, 0, 0.35, 0, 1, 0, 0.2, 0, 0, 1, 0.25], np.float32)
    s.insert(len(s) - 1, dict(pos=pos, idx=idx, uv=uv, m34=m, kind="lambert", albedo=[0.5, 0.5, 0.5],
                              texture=texture, cull=False))
    return s


def c2_scene(seed=0, texture_size=2048, sphere_level=2, spheres=500, ground_quads=141):
    """The spectral production workload: a displaced ground grid (2 x 141^2 =
    39,762 triangles) and 500 level-2 icospheres (320 triangles each) --
    199,762 triangles; half the spheres and the ground Lambert with seeded
    RGBA8 noise textures (texture_size^2, two textures), a quarter GGX metal
    (Unreal, metallic 1, roughness ~ U[0.05, 0.5]), a quarter glass (Refract,
    IoR 1.5); 8 quad area lights.  Returns (surfaces, camera); pair it with
    sky_map(1024, 512) as the skysphere."""
    rng = np.random.default_rng(seed)
    tex = [value_noise_texture(texture_size, seed + 17 + k) for k in range(2)]
    out = []
    # ground
    n = ground_quads
    g = np.linspace(-20.0, 20.0, n + 1)
    X, Z = np.meshgrid(g, g, indexing="ij")
    Y = 0.25 * np.sin(X * 0.45 + 0.3) * np.cos(Z * 0.37 - 0.2) + 0.08 * np.sin(X * 1.9) * np.sin(Z * 2.3)
    pos = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack([X / 8.0, Z / 8.0], -1).reshape(-1, 2).astype(np.float32)
    W = n + 1
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (ii * W + jj).ravel()
    idx = np.concatenate([np.stack([a, a + 1, a + W + 1], 1), np.stack([a, a + W + 1, a + W], 1)]).astype(np.uint32)
    I34 = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    out.append(dict(pos=pos, idx=idx, uv=uv, m34=I34.copy(), kind="lambert", albedo=[0.5, 0.5, 0.5],
                    texture=tex[0]))
    # spheres
    sp, si = icosphere(sphere_level, 1.0)
    d = sp / np.linalg.norm(sp, axis=1, keepdims=True)
    suv = np.stack([np.arctan2(d[:, 2], d[:, 0]) / (2 * np.pi) + 0.5, np.arccos(np.clip(d[:, 1], -1, 1)) / np.pi],
                   1).astype(np.float32)
    side = int(np.ceil(np.sqrt(spheres)))
    cells = np.linspace(-18.0, 18.0, side)
    k = 0
    for ix in range(side):
        for iz in range(side):
            if k == spheres:
                break
            r = 0.35 + 0.5 * rng.random()
            x = cells[ix] + (rng.random() - 0.5) * 0.6
            z = cells[iz] + (rng.random() - 0.5) * 0.6
            m = np.array([r, 0, 0, x, 0, r, 0, r + 0.35, 0, 0, r, z], np.float32)
            kind = k % 4
            srf = dict(pos=sp, idx=si, m34=m, kind="lambert", albedo=[0.5, 0.5, 0.5])
            if kind in (0, 1):
                srf.update(uv=suv, texture=tex[k % 2])
            elif kind == 2:
                srf.update(material="unreal", metallic=1.0, roughness=float(0.05 + 0.45 * rng.random()),
                           specular=0.5, albedo=[float(0.6 + 0.35 * rng.random()) for _ in range(3)])
            else:
                srf.update(material="refract", ior=(1.0, 1.5), cull=False)
            out.append(srf)
            k += 1
    # lights
    for l in range(8):
        x = -15.0 + 30.0 * (l % 4) / 3.0
        z = -8.0 + 16.0 * (l // 4)
        p, i = _quad((x - 0.75, 9.0, z - 0.75), (1.5, 0, 0), (0, 0, 1.5))
        out.append(dict(pos=p.astype(np.float32), idx=i, m34=I34.copy(), kind="light",
                        radiance=[40.0, 38.0, 34.0]))
    f = 50.0 * np.pi / 180.0
    cam = dict(pos=(0.0, 7.0, -26.0), gaze=(0.0, 0.5, 0.0), up=(0.0, 1.0, 0.0), fov=(f, f * 9.0 / 16.0),
               near_far=(0.05, 500.0))
    return out, cam


def box_camera():
    """Pinhole camera of the box scene (position, gaze point, up, fov radians, near/far)."""
    f = 40.0 * np.pi / 180.0
    return dict(pos=(0.5, 0.5, -1.4), gaze=(0.5, 0.5, 0.5), up=(0.0, 1.0, 0.0), fov=(f, f),
                near_far=(0.05, 100.0))
