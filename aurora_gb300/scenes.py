"""Seeded synthetic scenes with the shapes of the benchmark configurations, plus the host-side
packing of camera and options into the renderer's frame data.

Everything here is deterministic for a given seed (numpy's PCG64 generator), so the CUDA renderer
and the CPU oracle render byte-identical inputs on any machine.

  config_small      : plain method, small (512x512, 16 spp, 5 bounces): ground quad + 8x8 grid of
                      UV spheres (32x16 segments), Standard Surface per sphere with base_color
                      U[0.1,0.9]^3, metalness {0,1} (p = 0.5), specular_roughness U[0.05,0.8],
                      constant-radiance 64x32 RGB32F lat-long environment.
  config_large      : plain method, large (1920x1080, 64 spp, 8 bounces): one icosphere BLAS at
                      subdivision 8 (1,310,720 triangles) with radial displacement N(0, 0.02),
                      instanced 64x with random rigid transforms in a 100^3 box; coat ~ U[0,1],
                      transmission 1 (IOR 1.5) on 10% of instances; 2048x1024 RGB32F environment
                      with log-normal(0, 2) texels plus 4 sun-like hot spots.
  config_layered    : layered materials at small sizes (parity tests): distinct BLASes instanced
                      several times, each instance with a base material and an alpha-masked decal
                      layer (RGBA8 noise texture).
  config_stress     : plain method, stress with layered materials and accumulation (3840x2160,
                      progressive to 4096 spp): 16 BLAS of 10K-500K triangles, 1000 instances with
                      a decal layer each (1024^2 RGBA8 noise texture).
"""
import math

import numpy as np

from . import _abi

# ------------------------------------------------------------------------------ materials

# Standard Surface defaults (MaterialBase.cpp:109-167).
_DEFAULTS = {
    "base": 0.8, "base_color": (1.0, 1.0, 1.0), "diffuse_roughness": 0.0, "metalness": 0.0,
    "specular": 1.0, "specular_color": (1.0, 1.0, 1.0), "specular_roughness": 0.2,
    "specular_IOR": 1.5, "specular_anisotropy": 0.0, "specular_rotation": 0.0,
    "transmission": 0.0, "transmission_color": (1.0, 1.0, 1.0), "subsurface": 0.0,
    "subsurface_color": (1.0, 1.0, 1.0), "subsurface_radius": (1.0, 1.0, 1.0),
    "subsurface_scale": 1.0, "subsurface_anisotropy": 0.0, "sheen": 0.0,
    "sheen_color": (1.0, 1.0, 1.0), "sheen_roughness": 0.3, "coat": 0.0,
    "coat_color": (1.0, 1.0, 1.0), "coat_roughness": 0.1, "coat_anisotropy": 0.0,
    "coat_rotation": 0.0, "coat_IOR": 1.5, "coat_affect_color": 0.0,
    "coat_affect_roughness": 0.0, "emission": 0.0, "emission_color": (1.0, 1.0, 1.0),
    "opacity": (1.0, 1.0, 1.0), "thin_walled": 0,
}
_TEX_PREFIXES = ("base_color", "specular_roughness", "emission_color", "opacity", "normal")


def materials(n, **overrides):
    """n Standard Surface blocks at the reference defaults, with per-field overrides (scalars or
    arrays of n)."""
    m = np.zeros(n, dtype=_abi.MATERIAL_DTYPE)
    for k, v in _DEFAULTS.items():
        m[k] = v
    for p in _TEX_PREFIXES:
        m[p + "_image_scale"] = (1.0, 1.0)
    for k, v in overrides.items():
        m[k] = v
    return m


def no_textures(n):
    t = np.zeros(n, dtype=_abi.MATERIAL_TEXTURES_DTYPE)
    t["image"] = -1
    return t


# -------------------------------------------------------------------------------- meshes

def uv_sphere(segments=32, rings=16, radius=1.0):
    """UV sphere: `segments` around the axis, `rings` from pole to pole, pole caps as fans."""
    verts, norms, uvs = [], [], []
    for r in range(rings + 1):
        v = r / rings
        theta = v * math.pi
        for s in range(segments + 1):
            u = s / segments
            phi = u * 2.0 * math.pi
            n = (math.sin(theta) * math.cos(phi), math.cos(theta), math.sin(theta) * math.sin(phi))
            verts.append([radius * c for c in n])
            norms.append(n)
            uvs.append((u, v))
    idx = []
    row = segments + 1
    for r in range(rings):
        for s in range(segments):
            a = r * row + s
            b = a + row
            if r != 0:
                idx.append((a, b, a + 1))
            if r != rings - 1:
                idx.append((a + 1, b, b + 1))
    return (np.asarray(verts, np.float32), np.asarray(norms, np.float32),
            np.asarray(uvs, np.float32), np.asarray(idx, np.uint32).reshape(-1))


def quad(half=1.0):
    p = np.array([[-half, 0, -half], [half, 0, -half], [half, 0, half], [-half, 0, half]], np.float32)
    n = np.array([[0, 1, 0]] * 4, np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    i = np.array([0, 2, 1, 0, 3, 2], np.uint32)
    return p, n, uv, i


def icosphere(level, radius=1.0, displacement=0.0, seed=0):
    """Icosphere with 20 * 4^level triangles: each icosahedron face is split into a
    2^level grid and projected to the sphere; shared vertices are merged.  Vertices are displaced
    radially by radius * N(0, displacement) and normals are area-weighted face normals."""
    t = (1.0 + 5 ** 0.5) / 2.0
    base = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                     [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                    np.float64)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                      [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                      [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                      [8, 6, 7], [9, 8, 1]], np.int64)
    n = 1 << level
    # Lattice points (i, j) with i + j <= n on each face: P = A + (B - A) i/n + (C - A) j/n.
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = ii + jj <= n
    ii, jj = ii[keep], jj[keep]
    local = {(a, b): k for k, (a, b) in enumerate(zip(ii.tolist(), jj.tolist()))}
    tri_local = []
    for a in range(n):
        for b in range(n - a):
            tri_local.append((local[(a, b)], local[(a + 1, b)], local[(a, b + 1)]))
            if a + b + 1 < n:
                tri_local.append((local[(a + 1, b)], local[(a + 1, b + 1)], local[(a, b + 1)]))
    tri_local = np.asarray(tri_local, np.int64)
    npts = len(ii)
    A = base[faces[:, 0]][:, None, :]
    B = base[faces[:, 1]][:, None, :]
    C = base[faces[:, 2]][:, None, :]
    pts = A + (B - A) * (ii[None, :, None] / n) + (C - A) * (jj[None, :, None] / n)
    pts = pts.reshape(-1, 3)
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    # Merge the copies of edge and corner vertices that neighbouring faces produce.  Distinct
    # lattice points are >= 1e-3 apart at level 8, far above the 2^-16 quantisation step.
    key = np.round(pts * (1 << 16)).astype(np.int64)
    _, first, inverse = np.unique(key, axis=0, return_index=True, return_inverse=True)
    inverse = inverse.reshape(-1)
    assert len(first) == 10 * 4 ** level + 2, "icosphere vertex merge failed" 
    dirs = pts[first]
    tris = (tri_local[None, :, :] + (np.arange(20) * npts)[:, None, None]).reshape(-1, 3)
    tris = inverse[tris]
    rng = np.random.default_rng(seed)
    r = radius * (1.0 + rng.normal(0.0, displacement, len(dirs))) if displacement else \
        np.full(len(dirs), radius)
    pos = dirs * r[:, None]
    # Outward winding.
    e1 = pos[tris[:, 1]] - pos[tris[:, 0]]
    e2 = pos[tris[:, 2]] - pos[tris[:, 0]]
    fn = np.cross(e1, e2)
    flip = np.einsum("ij,ij->i", fn, pos[tris[:, 0]]) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    fn[flip] = -fn[flip]
    nrm = np.zeros_like(pos)
    for k in range(3):
        np.add.at(nrm, tris[:, k], fn)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    u = np.arctan2(dirs[:, 0], -dirs[:, 2]) / (2 * math.pi) + 0.5
    v = -np.arcsin(np.clip(dirs[:, 1], -1, 1)) / math.pi + 0.5
    uv = np.stack([u, v], axis=1)
    return (pos.astype(np.float32), nrm.astype(np.float32), uv.astype(np.float32),
            tris.astype(np.uint32).reshape(-1))


def lumpy_sphere(target_triangles, radius=1.0, displacement=0.0, seed=0):
    """UV sphere of about `target_triangles` triangles (segments = 2 x rings), vertices displaced
    radially by radius * N(0, displacement) (the seam column and each pole share one value, so the
    surface stays closed); normals are area-weighted face normals.  Vectorised: 500K triangles in
    well under a second."""
    seg = max(8, int(round(math.sqrt(target_triangles) + 1.0)))
    seg += seg % 2
    rings = seg // 2
    v = np.arange(rings + 1) / rings
    u = np.arange(seg + 1) / seg
    theta = v[:, None] * math.pi
    phi = u[None, :] * 2.0 * math.pi
    dirs = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta) * np.ones_like(phi),
                     np.sin(theta) * np.sin(phi)], axis=-1)
    rng = np.random.default_rng(seed)
    d = rng.normal(0.0, displacement, (rings + 1, seg)) if displacement else np.zeros((rings + 1, seg))
    d[0, :] = d[0, 0]
    d[-1, :] = d[-1, 0]
    d = np.concatenate([d, d[:, :1]], axis=1)
    pos = (dirs * (radius * (1.0 + d))[..., None]).reshape(-1, 3)
    uv = np.stack(np.broadcast_arrays(u[None, :], v[:, None]), axis=-1).reshape(-1, 2)
    row = seg + 1
    r, c = np.meshgrid(np.arange(rings), np.arange(seg), indexing="ij")
    a = r * row + c
    b = a + row
    t1 = np.stack([a, b, a + 1], axis=-1)[r != 0]
    t2 = np.stack([a + 1, b, b + 1], axis=-1)[r != rings - 1]
    tris = np.concatenate([t1, t2]).astype(np.int64)
    e1 = pos[tris[:, 1]] - pos[tris[:, 0]]
    e2 = pos[tris[:, 2]] - pos[tris[:, 0]]
    fn = np.cross(e1, e2)
    nrm = np.zeros_like(pos)
    for k in range(3):
        np.add.at(nrm, tris[:, k], fn)
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(ln > 0, nrm / np.maximum(ln, 1e-30), dirs.reshape(-1, 3))
    return (pos.astype(np.float32), nrm.astype(np.float32), uv.astype(np.float32),
            tris.astype(np.uint32).reshape(-1))


# -------------------------------------------------------------------------------- camera

def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    """World-to-camera matrix (right-handed, camera looks down -Z), as glm::lookAt."""
    eye, target, up = (np.asarray(x, np.float64) for x in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def perspective(fovy_deg, aspect, near=0.1, far=1000.0):
    """OpenGL-style perspective matrix, as glm::perspective."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[2, 3] = 2 * far * near / (near - far)
    m[3, 2] = -1.0
    return m


def denoising_range(view, scene_bounds):
    """RendererBase::denoisingRange (RendererBase.cpp:206-224): farthest view-space depth of the
    scene box, +10 %, clamped to [1, 5e8]; FP32 like glm."""
    if scene_bounds is None:
        return np.float32(1.0)
    lo, hi = np.asarray(scene_bounds[0], np.float32), np.asarray(scene_bounds[1], np.float32)
    v = np.asarray(view, np.float32)
    zs = []
    for c in range(8):
        p = np.array([hi[0] if c & 1 else lo[0], hi[1] if c & 2 else lo[1],
                      hi[2] if c & 4 else lo[2], 1.0], np.float32)
        zs.append(np.float32(v[2] @ p))
    depth = -np.float32(min(zs))
    return np.float32(min(max(depth * np.float32(1.1), np.float32(1.0)), np.float32(5.0e8)))


def frame_data(view, proj, trace_depth=5, max_luminance=1000.0, russian_roulette=True,
               rr_start_depth=3, lights=(), force_opaque_shadows=True, focal_distance=1.0,
               lens_radius=0.0, display_errors=False, scene_bounds=None, aovs=False, jitter=None,
               prev=None):
    """Packs camera and options like RendererBase::updateFrameDataGPUStruct
    (RendererBase.cpp:225-295).  view / proj are math-convention 4x4 arrays (column vectors);
    lights: (direction, color, intensity, angular_diameter) tuples packed as HGIScene.cpp:118-132
    (direction negated, cos of half the angular diameter).  aovs: denoising AOVs on; jitter:
    temporal camera jitter in pixels (PTRenderer.cpp:1149-1194); prev: (view, proj, jitter) of the
    previous frame for motion vectors (default: this frame)."""
    f = np.zeros((), dtype=_abi.FRAME_DTYPE)
    view = np.asarray(view, np.float64)
    proj = np.asarray(proj, np.float64)
    inv = np.linalg.inv(view)
    # Bytes of glm transpose(inverse(view)) = camera-to-world stored row-major.
    f["camera_view_proj"] = (proj @ view).T.reshape(-1)
    f["camera_inv_view"] = inv.reshape(-1)
    if prev is None:
        f["camera_view_proj_prev"] = f["camera_view_proj"]
        f["camera_inv_view_prev"] = f["camera_inv_view"]
    else:
        pv, pp = np.asarray(prev[0], np.float64), np.asarray(prev[1], np.float64)
        f["camera_view_proj_prev"] = (pp @ pv).T.reshape(-1)
        f["camera_inv_view_prev"] = np.linalg.inv(pv).reshape(-1)
        if len(prev) > 2 and prev[2] is not None:
            f["camera_jitter_prev"] = prev[2]
    if jitter is not None:
        f["camera_jitter"] = jitter
        f["is_temporal_jitter_enabled"] = 1
        if prev is None:
            f["camera_jitter_prev"] = jitter
    f["is_denoising_aovs_enabled"] = 1 if aovs else 0
    f["sky_view_z"] = -denoising_range(view, scene_bounds) * np.float32(2.0)
    f["view_size"] = (2.0 / proj[0, 0], 2.0 / proj[1, 1])
    f["is_ortho_projection"] = 1 if proj[3, 3] == 1.0 else 0
    f["focal_distance"] = focal_distance
    f["lens_radius"] = lens_radius
    f["time_delta_ms"] = 1000.0 / 60.0
    if scene_bounds is not None:
        lo, hi = np.asarray(scene_bounds[0]), np.asarray(scene_bounds[1])
        f["scene_size"] = float(np.linalg.norm(hi - lo))
    f["is_force_opaque_shadows_enabled"] = 1 if force_opaque_shadows else 0
    f["is_display_errors_enabled"] = 1 if display_errors else 0
    f["trace_depth"] = max(1, min(10, trace_depth))
    f["max_luminance"] = max_luminance
    f["is_russian_roulette_enabled"] = 1 if russian_roulette else 0
    f["russian_roulette_start_depth"] = max(0, rr_start_depth)
    lights = list(lights)[:4]
    f["distant_light_count"] = len(lights)
    for k, (direction, color, intensity, diameter) in enumerate(lights):
        f["distant_lights"][k]["color_and_intensity"] = (*color, intensity)
        f["distant_lights"][k]["direction"] = [-float(x) for x in direction]
        f["distant_lights"][k]["cos_radius"] = math.cos(0.5 * diameter)
    return f


def environment(light_top=(1, 1, 1), light_bottom=(0, 0, 0),
                background_top=(0.02, 0.25, 0.60), background_bottom=(0.32, 0.79, 1.0)):
    """EnvironmentData with the reference defaults (EnvironmentBase.cpp:33-45), identity
    transforms."""
    e = np.zeros((), dtype=_abi.ENV_DTYPE)
    e["light_top"], e["light_bottom"] = light_top, light_bottom
    e["background_top"], e["background_bottom"] = background_top, background_bottom
    eye = np.eye(4, dtype=np.float32).reshape(-1)
    e["light_transform"] = eye
    e["light_transform_inv"] = eye
    e["background_transform"] = eye
    return e


def translation(x, y, z):
    m = np.zeros(12, np.float32)
    m[0] = m[5] = m[10] = 1.0
    m[3], m[7], m[11] = x, y, z
    return m


def random_rigid(rng, box):
    """3x4 row-major transform: uniform random rotation and a translation in [-box/2, box/2]^3."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    t = rng.uniform(-box / 2, box / 2, 3)
    m = np.zeros((3, 4))
    m[:, :3], m[:, 3] = R, t
    return m.astype(np.float32).reshape(-1)


# --------------------------------------------------------------------------------- scenes

class SceneDesc:
    """A complete scene: meshes, instances, materials, images, environment, camera, options."""

    def __init__(self, name):
        self.name = name
        self.meshes = []        # dicts: positions, normals, texcoords, indices
        self.instances = []     # dicts: mesh, material, xform (12), layers [(material, uv)]
        self.materials = None   # MATERIAL_DTYPE array
        self.textures = None    # MATERIAL_TEXTURES_DTYPE array or None
        # Material node-graph programs or None: dict(first, count (int32 per material), ops
        # (GRAPH_OP_DTYPE), consts (float32, 4 per constant)); image operands index self.images.
        self.graphs = None
        self.images = []        # dicts: pixels, width, height, format, linear
        self.env = environment()
        self.env_light = -1     # image index
        self.env_background = -1
        self.ground_plane = None  # GROUND_PLANE_DTYPE record (_abi.ground_plane()) or None
        self.frame = None
        self.width = 0
        self.height = 0
        self.spp = 1

    @property
    def triangle_count(self):
        return sum(len(self.meshes[i["mesh"]]["indices"]) // 3 for i in self.instances)

    @property
    def unique_triangles(self):
        return sum(len(m["indices"]) // 3 for m in self.meshes)

    def add_mesh(self, positions, normals, texcoords, indices):
        self.meshes.append(dict(positions=np.ascontiguousarray(positions, np.float32),
                                normals=None if normals is None else np.ascontiguousarray(normals, np.float32),
                                texcoords=None if texcoords is None else np.ascontiguousarray(texcoords, np.float32),
                                indices=np.ascontiguousarray(indices, np.uint32)))
        return len(self.meshes) - 1

    def add_image(self, pixels, fmt, linear=False):
        h, w = pixels.shape[:2]
        self.images.append(dict(pixels=np.ascontiguousarray(pixels), width=w, height=h,
                                format=fmt, linear=1 if linear else 0))
        return len(self.images) - 1

    def bounds(self):
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        for inst in self.instances:
            p = self.meshes[inst["mesh"]]["positions"]
            m = np.asarray(inst["xform"], np.float64).reshape(3, 4)
            w = p @ m[:, :3].T + m[:, 3]
            lo, hi = np.minimum(lo, w.min(0)), np.maximum(hi, w.max(0))
        return lo, hi


def constant_env(width, height, value):
    return np.full((height, width, 3), value, np.float32)


def hdr_env(width, height, seed, sigma=2.0, suns=4, sun_radiance=5.0e4, sun_radius=4.0):
    """Log-normal(0, sigma) texels plus `suns` disc-shaped hot spots in the upper hemisphere."""
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(0.0, sigma, (height, width, 3))).astype(np.float32)
    yy, xx = np.mgrid[0:height, 0:width]
    for _ in range(suns):
        cx = rng.uniform(0, width)
        cy = rng.uniform(0.1, 0.45) * height
        d2 = np.minimum(np.abs(xx - cx), width - np.abs(xx - cx)) ** 2 + (yy - cy) ** 2
        img[d2 <= sun_radius ** 2] = sun_radiance * np.array([1.0, 0.95, 0.85], np.float32)
    return img


def config_small(seed=0, width=512, height=512, spp=16, trace_depth=5):
    s = SceneDesc("small: 8x8 UV spheres + quad, 64x32 constant env")
    rng = np.random.default_rng(seed)
    sphere = s.add_mesh(*uv_sphere(32, 16, 1.0))
    plane = s.add_mesh(*quad(12.0))
    n = 64
    s.materials = materials(n + 1)
    s.materials["base_color"][:n] = rng.uniform(0.1, 0.9, (n, 3))
    s.materials["metalness"][:n] = (rng.uniform(size=n) < 0.5).astype(np.float32)
    s.materials["specular_roughness"][:n] = rng.uniform(0.05, 0.8, n)
    for k in range(n):
        gx, gz = k % 8, k // 8
        s.instances.append(dict(mesh=sphere, material=k,
                                xform=translation(2.5 * (gx - 3.5), 1.0, 2.5 * (gz - 3.5)), layers=[]))
    s.instances.append(dict(mesh=plane, material=n, xform=translation(0, 0, 0), layers=[]))
    img = s.add_image(constant_env(64, 32, 1.0), _abi.FORMAT_RGB32F)
    s.env_light = img
    s.env_background = img
    s.width, s.height, s.spp = width, height, spp
    view = look_at((0.0, 14.0, 22.0), (0.0, 0.0, 0.0))
    proj = perspective(45.0, width / height)
    s.frame = frame_data(view, proj, trace_depth=trace_depth, scene_bounds=s.bounds())
    return s


def config_large(seed=0, width=1920, height=1080, spp=64, trace_depth=8, level=8, instances=64,
                 env_size=(2048, 1024)):
    s = SceneDesc(f"large: icosphere level {level} x{instances}, {env_size[0]}x{env_size[1]} HDR env")
    rng = np.random.default_rng(seed)
    ico = s.add_mesh(*icosphere(level, radius=6.0, displacement=0.02, seed=seed + 1))
    s.materials = materials(instances)
    s.materials["base_color"] = rng.uniform(0.1, 0.9, (instances, 3))
    s.materials["coat"] = rng.uniform(0.0, 1.0, instances)
    s.materials["specular_roughness"] = rng.uniform(0.05, 0.6, instances)
    glass = rng.permutation(instances)[: max(1, instances // 10)]
    s.materials["transmission"][glass] = 1.0
    s.materials["specular_IOR"][glass] = 1.5
    for k in range(instances):
        s.instances.append(dict(mesh=ico, material=k, xform=random_rigid(rng, 100.0), layers=[]))
    img = s.add_image(hdr_env(env_size[0], env_size[1], seed + 2), _abi.FORMAT_RGB32F)
    s.env_light = img
    s.env_background = img
    s.width, s.height, s.spp = width, height, spp
    view = look_at((0.0, 40.0, 150.0), (0.0, 0.0, 0.0))
    proj = perspective(45.0, width / height)
    s.frame = frame_data(view, proj, trace_depth=trace_depth, scene_bounds=s.bounds())
    return s


def noise_decal(size, seed):
    """RGBA8 noise texture whose alpha (replicated into RGB for the opacity slot) is a mask."""
    rng = np.random.default_rng(seed)
    coarse = rng.uniform(size=(size // 16 + 1, size // 16 + 1))
    up = np.kron(coarse, np.ones((16, 16)))[:size, :size]
    mask = (up > 0.55).astype(np.float32)
    rgba = np.zeros((size, size, 4), np.uint8)
    rgba[..., 0] = rng.integers(0, 256, (size, size))
    rgba[..., 1] = 255 - rgba[..., 0]
    rgba[..., 2] = 128
    rgba[..., 3] = (mask * 255).astype(np.uint8)
    opacity = np.repeat((mask * 255).astype(np.uint8)[..., None], 4, axis=2)
    return rgba, opacity


def config_layered(seed=0, width=960, height=540, spp=64, trace_depth=5, blas=4, instances=64,
                   tri_range=(2000, 20000), decal_size=256):
    """Layered-material stress at parameterised sizes (the full-size run uses 16 BLAS of
    10K-500K triangles, 1000 instances, 3840x2160 and a 1024^2 decal)."""
    s = SceneDesc(f"layered: {blas} BLAS x {instances} instances with decal layers")
    rng = np.random.default_rng(seed)
    meshes = []
    for b in range(blas):
        target = rng.integers(tri_range[0], tri_range[1] + 1)
        level = max(1, int(round(math.log(max(target / 20, 1), 4))))
        meshes.append(s.add_mesh(*icosphere(level, radius=2.0, displacement=0.02, seed=seed + 10 + b)))
    rgba, opacity = noise_decal(decal_size, seed + 3)
    color_img = s.add_image(rgba, _abi.FORMAT_RGBA8, linear=True)
    mask_img = s.add_image(opacity, _abi.FORMAT_RGBA8, linear=True)
    s.materials = materials(instances + 1)
    s.materials["base_color"][:instances] = rng.uniform(0.1, 0.9, (instances, 3))
    s.materials["specular_roughness"][:instances] = rng.uniform(0.05, 0.6, instances)
    decal = instances
    s.materials["has_base_color_image"][decal] = 1
    s.materials["has_opacity_image"][decal] = 1
    s.textures = no_textures(instances + 1)
    s.textures["image"][decal, _abi.TEX_BASE_COLOR] = color_img
    s.textures["image"][decal, _abi.TEX_OPACITY] = mask_img
    for k in range(instances):
        mesh = meshes[k % blas]
        uv = s.meshes[mesh]["texcoords"] * np.float32(3.0)
        s.instances.append(dict(mesh=mesh, material=k, xform=random_rigid(rng, 40.0),
                                layers=[(decal, np.ascontiguousarray(uv, np.float32))]))
    img = s.add_image(hdr_env(256, 128, seed + 4, sigma=1.0, suns=2, sun_radiance=500.0,
                              sun_radius=2.0), _abi.FORMAT_RGB32F)
    s.env_light = img
    s.env_background = img
    s.width, s.height, s.spp = width, height, spp
    view = look_at((0.0, 15.0, 60.0), (0.0, 0.0, 0.0))
    proj = perspective(45.0, width / height)
    s.frame = frame_data(view, proj, trace_depth=trace_depth, scene_bounds=s.bounds())
    return s


def config_stress(seed=0, width=3840, height=2160, spp=4096, trace_depth=5, blas=16, instances=1000,
                  tri_range=(10_000, 500_000), decal_size=1024, box=120.0):
    """Plain method, stress with layered materials and accumulation, at the stated shape by
    default: `blas` distinct BLASes whose triangle counts are evenly spaced over `tri_range`
    (16 x 10K-500K: 4.08M unique triangles -- the per-BLAS range caps the total at 8M, below the
    "~20M" the configuration also names), `instances` instances with random rigid transforms in a
    `box`^3 volume, each with a base Standard Surface material and an alpha-masked decal layer (a
    `decal_size`^2 RGBA8 noise colour texture and its mask), 3840x2160, accumulated progressively
    to `spp` samples (Kahan-compensated sums).  Smaller sizes keep the same structure for tests."""
    s = SceneDesc(f"stress: {blas} BLAS x {instances} instances with decal layers, {width}x{height}")
    rng = np.random.default_rng(seed)
    counts = np.linspace(tri_range[0], tri_range[1], blas).round().astype(int) if blas > 1 else \
        np.array([tri_range[0]])
    meshes = [s.add_mesh(*lumpy_sphere(int(c), radius=2.0, displacement=0.005, seed=seed + 100 + b))
              for b, c in enumerate(counts)]
    rgba, opacity = noise_decal(decal_size, seed + 3)
    color_img = s.add_image(rgba, _abi.FORMAT_RGBA8, linear=True)
    mask_img = s.add_image(opacity, _abi.FORMAT_RGBA8, linear=True)
    s.materials = materials(instances + 1)
    s.materials["base_color"][:instances] = rng.uniform(0.1, 0.9, (instances, 3))
    s.materials["metalness"][:instances] = (rng.uniform(size=instances) < 0.3).astype(np.float32)
    s.materials["specular_roughness"][:instances] = rng.uniform(0.05, 0.6, instances)
    decal = instances
    s.materials["has_base_color_image"][decal] = 1
    s.materials["has_opacity_image"][decal] = 1
    s.textures = no_textures(instances + 1)
    s.textures["image"][decal, _abi.TEX_BASE_COLOR] = color_img
    s.textures["image"][decal, _abi.TEX_OPACITY] = mask_img
    layer_uv = [np.ascontiguousarray(s.meshes[m]["texcoords"] * np.float32(3.0), np.float32) for m in meshes]
    for k in range(instances):
        b = int(rng.integers(0, blas))
        s.instances.append(dict(mesh=meshes[b], material=k, xform=random_rigid(rng, box),
                                layers=[(decal, layer_uv[b])]))
    img = s.add_image(hdr_env(256, 128, seed + 4, sigma=1.0, suns=2, sun_radiance=500.0,
                              sun_radius=2.0), _abi.FORMAT_RGB32F)
    s.env_light = img
    s.env_background = img
    s.width, s.height, s.spp = width, height, spp
    view = look_at((0.0, 0.25 * box, 1.4 * box), (0.0, 0.0, 0.0))
    proj = perspective(45.0, width / height)
    s.frame = frame_data(view, proj, trace_depth=trace_depth, scene_bounds=s.bounds())
    return s


def config_tiny(seed=0, width=32, height=24, spp=4, trace_depth=4, lights=True):
    """A few triangles with every material feature switched on somewhere: parity-test size."""
    s = SceneDesc("tiny")
    rng = np.random.default_rng(seed)
    sphere = s.add_mesh(*uv_sphere(8, 6, 1.0))
    plane = s.add_mesh(*quad(4.0))
    s.materials = materials(5)
    s.materials["base_color"] = rng.uniform(0.2, 0.9, (5, 3))
    s.materials["metalness"][1] = 1.0
    s.materials["coat"][2] = 0.7
    s.materials["sheen"][2] = 0.5
    s.materials["transmission"][3] = 1.0
    s.materials["subsurface"][0] = 0.3
    s.materials["emission"][4] = 0.5
    s.materials["diffuse_roughness"][4] = 0.4
    s.instances.append(dict(mesh=sphere, material=0, xform=translation(-1.2, 1.0, 0), layers=[]))
    s.instances.append(dict(mesh=sphere, material=1, xform=translation(1.2, 1.0, 0), layers=[]))
    s.instances.append(dict(mesh=sphere, material=2, xform=translation(0, 1.0, -1.5), layers=[]))
    s.instances.append(dict(mesh=sphere, material=3, xform=translation(0, 0.8, 1.2), layers=[]))
    s.instances.append(dict(mesh=plane, material=4, xform=translation(0, 0, 0), layers=[]))
    img = s.add_image(hdr_env(32, 16, seed + 1, sigma=1.0, suns=1, sun_radiance=200.0,
                              sun_radius=1.5), _abi.FORMAT_RGB32F)
    s.env_light = img
    s.env_background = img
    s.width, s.height, s.spp = width, height, spp
    view = look_at((0.0, 3.0, 7.0), (0.0, 0.8, 0.0))
    proj = perspective(45.0, width / height)
    lt = [((0.3, -1.0, -0.2), (1.0, 0.95, 0.9), 2.0, 0.05)] if lights else []
    s.frame = frame_data(view, proj, trace_depth=trace_depth, lights=lt, scene_bounds=s.bounds())
    return s
