"""Seeded synthetic workloads (no public dataset is involved).

  cornell_box()           10-triangle Cornell box, 20x20 area light (emission 12),
                          mirror and glass spheres r=16.5; 256x256, ss=8 (64 spp)
  icosphere_in_box()      level-6 displaced icosphere (81,920 triangles, radius 25,
                          0.1 * fBm of 4 octaves), Lambert 0.8 with a Phong lobe of
                          exponent 64 on half the faces, in the Cornell box;
                          1024x768, ss=16 (256 spp), max depth 10
  terrain_ibl()           1024x512-cell heightfield (1,048,576 triangles) with
                          fBm heights in [0, 50], 64 glass spheres, 2048x1024
                          float sky (gradient + 0.5 degree sun of 1e4 + log-normal
                          background) sampled through its CDF (next-event
                          estimation on); 1920x1080, ss=32 (1024 spp), max depth 12
  cornell_lens()          the Cornell box through a thin lens (CircleAperture)
  textured_scene()        textured Lambert quad and sphere under a white background
  reference_cornell()     the reference's own built-in CornellBoxScene
                          (src/scenes/CornellBoxScene.cpp:10-36): axis floors,
                          a two-layer sphere, a SphereLight
Each returns (SceneDesc, Camera, render settings dict).  Also:
  sphere_light_box(), sky_floor()   small next-event-estimation scenes (SceneDesc, Camera)
  batched_jobs()                    64 uneven render jobs for the batched form
  served_pool(), served_request()   resident scenes and Poisson requests for the served form
"""
import math

import numpy as np

from . import abi
from .scene import Camera, SceneDesc, fbm3, icosphere, quad, vertex_normals


def _box_walls(sd, white, red, blue):
    L = 100.0
    walls = [
        ([[0, 0, 0], [L, 0, 0], [L, 0, L], [0, 0, L]], (0, 1, 0), white),      # floor
        ([[0, L, 0], [L, L, 0], [L, L, L], [0, L, L]], (0, -1, 0), white),     # ceiling
        ([[0, 0, 0], [L, 0, 0], [L, L, 0], [0, L, 0]], (0, 0, 1), white),      # back
        ([[0, 0, 0], [0, L, 0], [0, L, L], [0, 0, L]], (1, 0, 0), red),        # left
        ([[L, 0, 0], [L, L, 0], [L, L, L], [L, 0, L]], (-1, 0, 0), blue),      # right
    ]
    for corners, facing, mat in walls:
        sd.add_triangles(quad(corners, facing), sd.layers(mat))


def _box_light(sd, light):
    y = 99.9
    sd.add_triangles(quad([[40, y, 40], [60, y, 40], [60, y, 60], [40, y, 60]], (0, -1, 0)), sd.layers(light))


def cornell_camera(width, height):
    # pinhole at (50, 50, 250) looking down -z with a 40 degree vertical field of view
    return Camera(width, height, (50.0, 50.0, 250.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0),
                  2.0 * 40.0 * math.tan(math.radians(20.0)), 40.0, 300.0, 0.0)


def cornell_box(width=256, height=256):
    sd = SceneDesc()
    white = sd.material(abi.OR3_LAMBERT, (0.75, 0.75, 0.75))
    red = sd.material(abi.OR3_LAMBERT, (0.75, 0.25, 0.25))
    blue = sd.material(abi.OR3_LAMBERT, (0.25, 0.25, 0.75))
    light = sd.material(abi.OR3_LAMBERT, (0.0, 0.0, 0.0), emission=(12.0, 12.0, 12.0))
    mirror = sd.material(abi.OR3_SPECULAR, (0.99, 0.99, 0.99))
    glass = sd.material(abi.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    _box_walls(sd, white, red, blue)
    _box_light(sd, light)
    sd.add_sphere((30.0, 16.5, 40.0), 16.5, sd.layers(mirror))
    sd.add_sphere((70.0, 16.5, 60.0), 16.5, sd.layers(glass))
    settings = dict(supersamples=8, min_samples=1, max_samples=1, step_samples=1, rr_min_depth=3, max_depth=8)
    return sd, cornell_camera(width, height), settings


def cornell_lens(width=128, height=128, aperture=1.3, focal=300.0):
    """The Cornell box seen through a thin lens: CircleAperture(radius) with
    the focal plane `focal` along z from the eye (Camera.h:65-93,
    Aperture.h:23-35).  The reference's main() always installs
    CircleAperture(1.3) with focal distance 300 (src/main.cpp:98-99)."""
    sd, cam, settings = cornell_box(width, height)
    cam.aperture_radius = float(aperture)
    cam.focal_distance = float(focal)
    return sd, cam, settings


def textured_scene(width=96, height=64, seed=9):
    """Textured Lambert layers under a constant white background: a quad whose
    uv runs past [0, 1] on every side (the clamp and the x0.99999 rule of
    Image::GetPixelByUV, src/tools/Image.h:21-31) and a sphere with the
    reference's lat-long uv (Sphere.h:61-75).  The sphere lies behind the
    quad's plane and the quad is single-sided, so no bounce from one reaches
    the other: every camera path's radiance is exactly colour x texel
    (GetTexturedColor, src/renderer/PathTracer.cpp:327-346) and pixel means
    have no Monte Carlo noise.  Textures are 37x23 and 29x16 texels of seeded
    colours."""
    rng = np.random.default_rng(seed)
    sd = SceneDesc()
    t0 = sd.add_texture(rng.uniform(0.05, 1.0, (23, 37, 3)))
    t1 = sd.add_texture(rng.uniform(0.05, 1.0, (16, 29, 3)))
    mq = sd.material(abi.OR3_LAMBERT, (0.9, 0.8, 0.7), texture=t0)
    ms = sd.material(abi.OR3_LAMBERT, (0.85, 0.9, 0.95), texture=t1)
    c0, c1, c2, c3 = (-60.0, -25.0, 0.0), (-5.0, -25.0, 0.0), (-5.0, 25.0, 0.0), (-60.0, 25.0, 0.0)
    u0, u1, v0, v1 = -0.2, 1.15, 1.25, -0.1  # uv at x = -60 / -5 and y = -25 / 25
    uv = {c0: (u0, v0), c1: (u1, v0), c2: (u1, v1), c3: (u0, v1)}
    tris = [(c0, c1, c2), (c0, c2, c3)]  # face normal +z, toward the camera
    sd.add_triangles([list(t) for t in tris], sd.layers(mq), uvs=[[uv[c] for c in t] for t in tris])
    sd.add_sphere((35.0, 0.0, -30.0), 22.0, sd.layers(ms))
    sd.background = (1.0, 1.0, 1.0)
    cam = Camera.from_fov(width, height, (0.0, 0.0, 150.0), (0.0, 0.0, 0.0), 34.0)
    settings = dict(supersamples=2, min_samples=1, max_samples=1, step_samples=1, rr_min_depth=5, max_depth=0)
    return sd, cam, settings


def sphere_light_box(width=64, height=64):
    """The Cornell walls lit only by an emissive sphere flagged as a SphereLight
    (radius 6, radiance 40), with a Phong sphere (exponent 20) and a mirror
    sphere: next-event estimation with a sphere light and a glossy lobe."""
    sd = SceneDesc()
    white = sd.material(abi.OR3_LAMBERT, (0.75, 0.75, 0.75))
    red = sd.material(abi.OR3_LAMBERT, (0.75, 0.25, 0.25))
    blue = sd.material(abi.OR3_LAMBERT, (0.25, 0.25, 0.75))
    lamp = sd.material(abi.OR3_LAMBERT, (0.0, 0.0, 0.0), emission=(40.0, 40.0, 40.0))
    glossy = sd.material(abi.OR3_PHONG, (0.7, 0.7, 0.7), phong_exponent=20.0)
    mirror = sd.material(abi.OR3_SPECULAR, (0.95, 0.95, 0.95))
    _box_walls(sd, white, red, blue)
    sd.add_sphere((50.0, 80.0, 50.0), 6.0, sd.layers(lamp), light=True)
    sd.add_sphere((32.0, 15.0, 45.0), 15.0, sd.layers(glossy))
    sd.add_sphere((72.0, 12.0, 65.0), 12.0, sd.layers(mirror))
    return sd, cornell_camera(width, height)


def sky_floor(width=64, height=64, env=(256, 128), seed=3, constant=None):
    """A Lambert floor and an axis-aligned Lambert box under the synthetic sky
    (sun of radiance 1e4), or under a constant background when `constant` is an
    RGB triple: next-event estimation of the environment."""
    sd = SceneDesc()
    white = sd.material(abi.OR3_LAMBERT, (0.7, 0.7, 0.7))
    tan = sd.material(abi.OR3_LAMBERT, (0.6, 0.5, 0.35))
    sd.add_triangles(quad([[-200, 0, -200], [200, 0, -200], [200, 0, 200], [-200, 0, 200]], (0, 1, 0)),
                     sd.layers(white))
    x0, x1, y1, z0, z1 = -20.0, 20.0, 30.0, -20.0, 20.0
    box = [
        ([[x0, y1, z0], [x1, y1, z0], [x1, y1, z1], [x0, y1, z1]], (0, 1, 0)),
        ([[x0, 0, z1], [x1, 0, z1], [x1, y1, z1], [x0, y1, z1]], (0, 0, 1)),
        ([[x0, 0, z0], [x1, 0, z0], [x1, y1, z0], [x0, y1, z0]], (0, 0, -1)),
        ([[x1, 0, z0], [x1, y1, z0], [x1, y1, z1], [x1, 0, z1]], (1, 0, 0)),
        ([[x0, 0, z0], [x0, y1, z0], [x0, y1, z1], [x0, 0, z1]], (-1, 0, 0)),
    ]
    for corners, facing in box:
        sd.add_triangles(quad(corners, facing), sd.layers(tan))
    if constant is None:
        sky, _ = sky_image(env[0], env[1], seed=seed)
        sd.set_env(sky)
    else:
        sd.background = tuple(float(c) for c in constant)
    cam = Camera.from_fov(width, height, (60.0, 70.0, 140.0), (0.0, 10.0, 0.0), 45.0)
    return sd, cam


def icosphere_in_box(width=1024, height=768, level=6, seed=2, glossy_faces=True):
    """glossy_faces False: every face Lambert 0.8 (a scene the reference's own
    integrator can render, which has no glossy lobe)."""
    rng = np.random.default_rng(seed)
    sd = SceneDesc()
    white = sd.material(abi.OR3_LAMBERT, (0.75, 0.75, 0.75))
    red = sd.material(abi.OR3_LAMBERT, (0.75, 0.25, 0.25))
    blue = sd.material(abi.OR3_LAMBERT, (0.25, 0.25, 0.75))
    light = sd.material(abi.OR3_LAMBERT, (0.0, 0.0, 0.0), emission=(12.0, 12.0, 12.0))
    diffuse = sd.material(abi.OR3_LAMBERT, (0.8, 0.8, 0.8))
    gloss = sd.material(abi.OR3_PHONG, (0.8, 0.8, 0.8), phong_exponent=64.0)
    _box_walls(sd, white, red, blue)
    _box_light(sd, light)
    v, f = icosphere(level)
    disp = 1.0 + 0.1 * fbm3(v * 2.0, seed)
    center = np.array([50.0, 45.0, 50.0])
    pos = v * (25.0 * disp)[:, None] + center
    vn = vertex_normals(pos, f)
    lam = sd.layers(diffuse)
    mix = sd.layers([(diffuse, 0.5), (gloss, 0.5)])
    glossy = rng.random(len(f)) < 0.5
    if not glossy_faces:
        glossy[:] = False
    lay = np.where(glossy[:, None], np.array(mix, np.uint32), np.array(lam, np.uint32)).astype(np.uint32)
    sd.add_triangles(pos[f], lay, normals=vn[f])
    settings = dict(supersamples=16, min_samples=1, max_samples=1, step_samples=1, rr_min_depth=5, max_depth=10)
    return sd, cornell_camera(width, height), settings


def sky_image(width=2048, height=1024, seed=3, sun_dir=(0.5, 0.55, -0.3), sun_radiance=1.0e4,
              sun_radius_deg=0.5, sigma=1.0):
    """Equirect float sky in the reference IBL's mapping (src/renderer/IBL.h:30-45):
    row = theta / pi (theta from +y), column = phi / 2pi (phi from +x toward +z)."""
    rng = np.random.default_rng(seed)
    th = (np.arange(height) + 0.5) / height * math.pi
    ph = (np.arange(width) + 0.5) / width * 2.0 * math.pi
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    d = np.stack(np.broadcast_arrays(st * np.cos(ph)[None, :], ct, st * np.sin(ph)[None, :]), -1)
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    cosg = np.clip((d * s).sum(-1), -1.0, 1.0)
    gamma = np.arccos(cosg)
    up = np.clip(d[..., 1], 0.0, 1.0)
    # Preetham-like: zenith darkening + circumsolar brightening (Perez-style shape)
    zen = 1.0 + 2.0 * np.exp(-3.0 / (up + 0.08))
    circ = 1.0 + 8.0 * np.exp(-3.0 * gamma) + 0.45 * cosg ** 2
    base = np.stack([0.25 * zen * circ, 0.35 * zen * circ, 0.65 * zen * circ], -1) * 0.5
    base[d[..., 1] < 0] = 0.05
    noise = np.exp(sigma * rng.standard_normal((height, width)) - 0.5 * sigma * sigma)
    img = base * noise[..., None]
    img[gamma < math.radians(sun_radius_deg)] = sun_radiance
    return img.astype(np.float32), s


def terrain_ibl(width=1920, height=1080, cells_x=1024, cells_z=512, seed=3, spheres=64):
    rng = np.random.default_rng(seed)
    sd = SceneDesc()
    ground = sd.material(abi.OR3_LAMBERT, (0.45, 0.42, 0.38))
    glass = sd.material(abi.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    ex, ez = 2000.0, 1000.0
    xs = np.linspace(-ex / 2, ex / 2, cells_x + 1)
    zs = np.linspace(-ez / 2, ez / 2, cells_z + 1)
    X, Z = np.meshgrid(xs, zs)  # (cells_z+1, cells_x+1)
    h = fbm3(np.stack([X / 250.0, np.zeros_like(X), Z / 250.0], -1), seed)
    h = (h - h.min()) / (h.max() - h.min()) * 50.0
    P = np.stack([X, h, Z], -1).reshape(-1, 3)
    idx = np.arange((cells_z + 1) * (cells_x + 1)).reshape(cells_z + 1, cells_x + 1)
    a, b = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel()
    c, d = idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
    f = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)])
    nrm = np.cross(P[f[:, 1]] - P[f[:, 0]], P[f[:, 2]] - P[f[:, 0]])
    flip = nrm[:, 1] < 0
    f[flip] = f[flip][:, ::-1]
    vn = vertex_normals(P, f)
    sd.add_triangles(P[f], sd.layers(ground), normals=vn[f])
    gl = sd.layers(glass)
    for _ in range(spheres):
        r = rng.uniform(3.0, 10.0)
        x, z = rng.uniform(-300, 300), rng.uniform(-150, 250)
        ix = int(round((x + ex / 2) / ex * cells_x))
        iz = int(round((z + ez / 2) / ez * cells_z))
        y = h[iz, ix] + r
        sd.add_sphere((x, y, z), r, gl)
    sky, _ = sky_image(seed=seed)
    sd.set_env(sky)
    cam = Camera.from_fov(width, height, (0.0, 140.0, 520.0), (0.0, 20.0, 0.0), 45.0)
    # the sky is importance-sampled: next-event estimation on
    settings = dict(supersamples=32, min_samples=1, max_samples=1, step_samples=1, rr_min_depth=5, max_depth=12,
                    next_event_estimation=True)
    return sd, cam, settings


def reference_cornell(width=160, height=120):
    """The reference's built-in CornellBoxScene, object for object
    (src/scenes/CornellBoxScene.cpp:10-36, floors from src/scenes/Scene.cpp:88-200),
    camera from settings.txt (position 50,55,230; direction ~(0,-0.15,-1))."""
    sd = SceneDesc()
    L = abi.OR3_LAMBERT

    def floor(kind, sx, sy, pos, mat):
        # Scene::AddFloor* vertex lists, translated by `pos`
        hx, hy = sx / 2.0, sy / 2.0
        p = np.asarray(pos, np.float64)
        tbl = {
            "YZ_xUp": ([(0, hx, -hy), (0, hx, hy), (0, -hx, hy)], [(0, -hx, -hy), (0, hx, -hy), (0, -hx, hy)],
                       (1, 0, 0)),
            "YZ_xDown": ([(0, -hx, hy), (0, hx, hy), (0, hx, -hy)], [(0, -hx, hy), (0, hx, -hy), (0, -hx, -hy)],
                         (-1, 0, 0)),
            "XY_zUp": ([(-hx, hy, 0), (-hx, -hy, 0), (hx, -hy, 0)], [(hx, hy, 0), (-hx, hy, 0), (hx, -hy, 0)],
                       (0, 0, 1)),
            "XY_zDown": ([(hx, -hy, 0), (-hx, -hy, 0), (-hx, hy, 0)], [(hx, -hy, 0), (-hx, hy, 0), (hx, hy, 0)],
                         (0, 0, -1)),
            "XZ_yUp": ([(-hx, 0, -hy), (-hx, 0, hy), (hx, 0, -hy)], [(hx, 0, -hy), (-hx, 0, hy), (hx, 0, hy)],
                       (0, 1, 0)),
            "XZ_yDown": ([(hx, 0, -hy), (-hx, 0, hy), (-hx, 0, -hy)], [(hx, 0, hy), (-hx, 0, hy), (hx, 0, -hy)],
                         (0, -1, 0)),
        }
        t0, t1, n = tbl[kind]
        tris = np.asarray([t0, t1], np.float64) + p
        normals = np.broadcast_to(np.asarray(n, np.float64), (2, 3, 3))
        sd.add_triangles(tris, sd.layers(mat), normals=normals)

    red = sd.material(L, (0.75, 0.25, 0.25))
    blue = sd.material(L, (0.25, 0.25, 0.75))
    back = sd.material(L, (1, 1, 1))
    front = sd.material(L, (0.75, 0.75, 0.75))
    white = sd.material(L, (0.75, 0.75, 0.75))
    floor("YZ_xUp", 200, 200, (1, 40.8, 81.6), red)
    floor("YZ_xDown", 200, 200, (99, 40.8, 81.6), blue)
    floor("XY_zUp", 150, 150 / 1.77777777777, (50, 40.8, 0), back)
    floor("XY_zDown", 150, 150 / 1.77777777777, (50, 40.8, 250), front)
    floor("XZ_yUp", 2000, 2000, (50, 0, 81.6), white)
    floor("XZ_yDown", 200, 200, (50, 81.6, 81.6), white)
    green = sd.material(L, (0.25, 0.75, 0.25))
    spec = sd.material(abi.OR3_SPECULAR, (0.99, 0.99, 0.99))
    glass = sd.material(abi.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    lightm = sd.material(L, (0, 0, 0), emission=(36, 36, 36))
    # first layer rate 1.0, then AddMaterial(spec, 0.1) normalises to 1/1.1, 0.1/1.1
    sd.add_sphere((50, 20, 50), 20, sd.layers([(green, 1.0 / 1.1), (spec, 0.1 / 1.1)]))
    sd.add_sphere((19, 16.5, 25), 16.5, sd.layers(spec))
    sd.add_sphere((77, 16.5, 78), 16.5, sd.layers(glass))
    sd.add_sphere((50.0, 90, 81.6), 15, sd.layers(lightm), light=True)
    cam = Camera(width, height, (50.0, 55.0, 230.0), (0.00001, -0.15, -1.0), (0.0, 1.0, 0.0), 30.0, 40.0, 300.0, 0.0)
    settings = dict(supersamples=4, min_samples=1, max_samples=4, step_samples=1, rr_min_depth=5, max_depth=0)
    return sd, cam, settings


def _mesh_scene(rng, tris, kind, env_size=(512, 256)):
    """One seeded scene of about `tris` triangles: a displaced icosphere in the
    Cornell box (kind 0) or a heightfield under a sky (kind 1); the main
    surface is Lambertian, mirror or glass, with a few mirror/glass spheres."""
    sd = SceneDesc()
    pick = rng.random()
    albedo = tuple(rng.uniform(0.4, 0.85, 3))
    if pick < 0.6:
        main = sd.material(abi.OR3_LAMBERT, albedo)
    elif pick < 0.8:
        main = sd.material(abi.OR3_SPECULAR, (0.95, 0.95, 0.95))
    else:
        main = sd.material(abi.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    mirror = sd.material(abi.OR3_SPECULAR, (0.95, 0.95, 0.95))
    glass = sd.material(abi.OR3_REFRACTION, (0.99, 0.99, 0.99), ior=1.5)
    seed = int(rng.integers(1 << 30))
    if kind == 0:
        white = sd.material(abi.OR3_LAMBERT, (0.75, 0.75, 0.75))
        red = sd.material(abi.OR3_LAMBERT, (0.75, 0.25, 0.25))
        blue = sd.material(abi.OR3_LAMBERT, (0.25, 0.25, 0.75))
        light = sd.material(abi.OR3_LAMBERT, (0.0, 0.0, 0.0), emission=(12.0, 12.0, 12.0))
        _box_walls(sd, white, red, blue)
        _box_light(sd, light)
        level = int(np.clip(np.round(np.log(max(tris, 80) / 20.0) / np.log(4.0)), 2, 9))
        v, f = icosphere(level)
        pos = v * (22.0 * (1.0 + 0.1 * fbm3(v * 2.0, seed)))[:, None] + np.array([50.0, 40.0, 50.0])
        sd.add_triangles(pos[f], sd.layers(main), normals=vertex_normals(pos, f)[f])
        for k in range(3):
            sd.add_sphere((15.0 + 35.0 * k, 8.0, 85.0), 7.0, sd.layers(mirror if k % 2 else glass))
        cam = None
    else:
        cells = max(tris // 2, 8)
        cx = max(int(np.sqrt(cells * 2)), 2)
        cz = max(cells // cx, 2)
        ex, ez = 400.0, 400.0 * cz / cx
        xs, zs = np.linspace(-ex / 2, ex / 2, cx + 1), np.linspace(-ez / 2, ez / 2, cz + 1)
        X, Z = np.meshgrid(xs, zs)
        h = fbm3(np.stack([X / 80.0, np.zeros_like(X), Z / 80.0], -1), seed) * 15.0
        P = np.stack([X, h, Z], -1).reshape(-1, 3)
        idx = np.arange((cz + 1) * (cx + 1)).reshape(cz + 1, cx + 1)
        a, b = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel()
        c, d = idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
        f = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)])
        sd.add_triangles(P[f], sd.layers(main), normals=vertex_normals(P, f)[f])
        for k in range(4):
            sd.add_sphere((rng.uniform(-60, 60), 25.0, rng.uniform(-60, 60)), rng.uniform(5, 12),
                          sd.layers(mirror if k % 2 else glass))
        sky, _ = sky_image(env_size[0], env_size[1], seed=seed % 1000)
        sd.set_env(sky)
        cam = (0.0, 90.0, 260.0)
    return sd, cam


def batched_jobs(n=64, seed=4, scale=1.0, small=False):
    """Batched workload: n seeded scenes, triangle counts log-uniform in [1k, 2M] (x scale),
    alternating displaced icospheres and heightfields, mixed Lambert/mirror/glass,
    square images with sides uniform in [128, 1024], spp uniform in [16, 512]
    (a 4x4 sub-pixel grid times spp/16 samples), next-event estimation on (the
    box's light quad, or the sky through its CDF).  small: sides in [64, 256] and
    spp in {16, 32, 48, 64} instead (the jobs a single render cannot fill the GPU
    with).  Returns [(SceneDesc, Camera, settings)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        tris = int(np.exp(rng.uniform(np.log(1e3), np.log(2e6))) * scale)
        sd, eye = _mesh_scene(rng, tris, i % 2)
        side = int(rng.integers(128, 1025))
        spp = int(rng.integers(16, 513)) // 16 * 16 or 16
        if small:
            side = 64 + side * 192 // 1024
            spp = 16 * (1 + spp * 4 // 528)
        if eye is None:
            cam = cornell_camera(side, side)
        else:
            cam = Camera.from_fov(side, side, eye, (0.0, 0.0, 0.0), 50.0)
        st = dict(supersamples=4, min_samples=spp // 16, max_samples=spp // 16, step_samples=1,
                  rr_min_depth=5, max_depth=8, seed=1000 + i, next_event_estimation=True)
        out.append((sd, cam, st))
    return out


SERVED_RES = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
SERVED_SPP = [16, 64, 256, 1024]


def served_pool(n=32, seed=5, scale=1.0, env=(2048, 1024)):
    """Served workload: n resident scenes of 10k-4M triangles (log-uniform, x scale), each
    with its own float32 equirect sky of `env` size.  Returns [(SceneDesc, eye)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        tris = int(np.exp(rng.uniform(np.log(1e4), np.log(4e6))) * scale)
        sd, eye = _mesh_scene(rng, tris, 1, env_size=env)
        out.append((sd, eye))
    return out


def served_request(rng, pool_size, eye_of):
    """One request: a resident scene, a resolution from SERVED_RES and an spp from SERVED_SPP."""
    s = int(rng.integers(pool_size))
    w, h = SERVED_RES[int(rng.integers(len(SERVED_RES)))]
    spp = SERVED_SPP[int(rng.integers(len(SERVED_SPP)))]
    cam = Camera.from_fov(w, h, eye_of(s), (0.0, 0.0, 0.0), 50.0)
    st = dict(supersamples=4, min_samples=spp // 16, max_samples=spp // 16, step_samples=1, rr_min_depth=5,
              max_depth=8, seed=int(rng.integers(1 << 31)), layout=abi.OR3_LAYOUT_COMPACT,
              next_event_estimation=True)
    return s, cam, st


def random_triangles(n=2000, seed=7, extent=100.0, size=8.0):
    """Triangle soup for closest-hit parity (random orientation, both windings)."""
    rng = np.random.default_rng(seed)
    sd = SceneDesc()
    m = sd.material(abi.OR3_LAMBERT, (0.5, 0.5, 0.5))
    c = rng.uniform(0, extent, (n, 1, 3))
    v = c + rng.uniform(-size, size, (n, 3, 3))
    sd.add_triangles(v, sd.layers(m))
    cen = rng.uniform(0, extent, (max(1, n // 100), 3))
    for p in cen:
        sd.add_sphere(p, rng.uniform(1.0, 6.0), sd.layers(m))
    return sd


def random_rays(n, seed, lo=-20.0, hi=120.0, target_lo=0.0, target_hi=100.0):
    """Seeded rays from a box around the scene toward random points inside it (FP64, unit)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    t = rng.uniform(target_lo, target_hi, (n, 3))
    d = t - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d
