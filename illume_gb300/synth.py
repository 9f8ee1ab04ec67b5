"""Seeded synthetic scenes for the benchmark configurations.

* Geodesic icosphere of frequency f (20 f^2 triangles), vertices displaced radially by
  4-octave value noise: r' = r (1 + amp * n(p)), n in [-1, 1], lattice values from
  Philox4x32-10 keyed by the seed, trilinear interpolation with a smoothstep fade, base
  frequency 2, each octave doubling the frequency and halving the amplitude.
* Equirectangular environment map in the reference's (u, v) convention
  (src/renderer.cu:380-381): sky gradient from 0.2 at the horizon to 1.0 at the zenith,
  0.2 below the horizon, plus a Gaussian sun lobe of peak 5000 and 0.5 degree width at a
  seeded direction (azimuth U[0, 2 pi), elevation U[15, 60] degrees).
* Scene builders: the triangle-heavy traversal scene (displaced icosphere with a rough
  gold conductor over a checkerboard ground quad, environment lighting), the Cornell box,
  and the subsurface scene (displaced mesh with a scattering medium in the Cornell box).
"""
from __future__ import annotations

import math

import numpy as np

from . import _capi as C
from .scenedata import Material, Mesh, SceneData, Texture

GOLD_ETA = (0.143, 0.374, 1.442)
GOLD_K = (3.983, 2.385, 1.603)
COPPER_ETA = (0.200, 0.924, 1.102)
COPPER_K = (3.912, 2.452, 2.142)


# ---------------------------------------------------------------- Philox (numpy)
def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 on uint32 arrays; returns the four output words."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) & 0xFFFFFFFF for x in (c0, c1, c2, c3))
    k0 = np.uint64(k0) & np.uint64(0xFFFFFFFF)
    k1 = np.uint64(k1) & np.uint64(0xFFFFFFFF)
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    mask = np.uint64(0xFFFFFFFF)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(0x9E3779B9)) & mask
            k1 = (k1 + np.uint64(0xBB67AE85)) & mask
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & mask, lo1, (hi0 ^ c3 ^ k1) & mask, lo0
    return tuple(x.astype(np.uint32) for x in (c0, c1, c2, c3))


# ---------------------------------------------------------------- geometry
def icosahedron():
    t = (1 + 5 ** 0.5) / 2
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
                  (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    return v, f


def icosphere(freq: int):
    """Geodesic sphere of frequency `freq`: 20 * freq^2 triangles, unit radius."""
    v, faces = icosahedron()
    pts, tris = [], []
    base = 0
    idx = {}
    ij = [(i, j) for i in range(freq + 1) for j in range(freq + 1 - i)]
    for (i, j) in ij:
        idx[(i, j)] = len(idx)
    ii = np.array([p[0] for p in ij], np.float64)
    jj = np.array([p[1] for p in ij], np.float64)
    local = []
    for i in range(freq):
        for j in range(freq - i):
            local.append((idx[(i, j)], idx[(i + 1, j)], idx[(i, j + 1)]))
            if i + j + 1 < freq:
                local.append((idx[(i + 1, j)], idx[(i + 1, j + 1)], idx[(i, j + 1)]))
    local = np.array(local, np.int64)
    for a, b, c in faces:
        A, B, Cc = v[a], v[b], v[c]
        P = A[None] + (B - A)[None] * (ii / freq)[:, None] + (Cc - A)[None] * (jj / freq)[:, None]
        P /= np.linalg.norm(P, axis=1, keepdims=True)
        pts.append(P)
        tris.append(local + base)
        base += len(P)
    P = np.concatenate(pts)
    T = np.concatenate(tris)
    # merge the vertices shared by neighbouring faces
    key = np.round(P * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)
    remap = np.empty_like(order)
    remap[order] = np.arange(len(order))
    P = P[first[order]]
    T = remap[inv.reshape(-1)[T]]
    # outward winding
    n = np.cross(P[T[:, 1]] - P[T[:, 0]], P[T[:, 2]] - P[T[:, 0]])
    flip = (n * P[T].mean(1)).sum(1) < 0
    T[flip] = T[flip][:, [0, 2, 1]]
    return P, T.astype(np.int32)


def freq_for_tris(n: int) -> int:
    return max(1, int(round(math.sqrt(n / 20.0))))


def value_noise(p: np.ndarray, seed: int, octaves: int = 4, base_freq: float = 2.0) -> np.ndarray:
    """4-octave value noise on points p (N, 3), normalised to [-1, 1]."""
    total = np.zeros(len(p))
    amp_sum = 0.0
    freq, amp = base_freq, 1.0
    for o in range(octaves):
        q = p * freq
        q0 = np.floor(q).astype(np.int64)
        f = q - q0
        s = f * f * (3 - 2 * f)
        acc = np.zeros(len(p))
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    c = q0 + np.array([dx, dy, dz])
                    w0, _, _, _ = philox4x32_10(c[:, 0] & 0xFFFFFFFF, c[:, 1] & 0xFFFFFFFF, c[:, 2] & 0xFFFFFFFF,
                                                np.full(len(p), o, np.uint64), seed, 0x6E6F6973)
                    val = w0.astype(np.float64) / 4294967295.0 * 2.0 - 1.0
                    wx = s[:, 0] if dx else 1 - s[:, 0]
                    wy = s[:, 1] if dy else 1 - s[:, 1]
                    wz = s[:, 2] if dz else 1 - s[:, 2]
                    acc += wx * wy * wz * val
        total += amp * acc
        amp_sum += amp
        freq *= 2.0
        amp *= 0.5
    return total / amp_sum


def displaced_icosphere(freq: int, seed: int, amp: float = 0.15, radius: float = 1.0):
    P, T = icosphere(freq)
    n = value_noise(P, seed)
    P = P * (radius * (1.0 + amp * n))[:, None]
    return P.astype(np.float32), T


def quad(size: float, y: float):
    s = size / 2
    P = np.array([(-s, y, -s), (s, y, -s), (s, y, s), (-s, y, s)], np.float32)
    UV = np.array([(0, 0), (1, 0), (1, 1), (0, 1)], np.float32)
    T = np.array([(0, 2, 1), (0, 3, 2)], np.int32)
    return P, T, UV


# ---------------------------------------------------------------- environment
def sun_direction(seed: int):
    w = philox4x32_10(np.array([0]), np.array([0]), np.array([0]), np.array([0]), seed, 0x73756E)
    az = 2 * math.pi * (float(w[0][0]) / 4294967296.0)
    el = math.radians(15 + 45 * (float(w[1][0]) / 4294967296.0))
    return np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)]), az, el


def environment_map(seed: int = 1, width: int = 2048, height: int = 1024, sun_peak: float = 5000.0,
                    sun_sigma_deg: float = 0.5) -> np.ndarray:
    """RGBA float32 (height, width, 4) equirectangular map, reference uv convention."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = (u - 0.5) * 2 * math.pi                   # atan2(d.z, d.x)
    elev = (0.5 - v) * math.pi                      # asin(d.y)
    se = np.sin(elev)
    tint = np.array([0.75, 0.85, 1.0])
    out = np.ones((height, width, 4), np.float32)
    # sky: a function of elevation only
    row = np.where(se[:, None] > 0, (0.2 + 0.8 * np.clip(se, 0.0, 1.0))[:, None] * tint[None, :], 0.2)
    out[:, :, :3] = row[:, None, :].astype(np.float32)
    # sun lobe: rows within 12 sigma of the sun's elevation
    sdir, _, sun_el = sun_direction(seed)
    sig = math.radians(sun_sigma_deg)
    rows = np.nonzero(np.abs(elev - sun_el) < 12 * sig)[0]
    if len(rows):
        ce, se_r = np.cos(elev[rows])[:, None], se[rows][:, None]
        cosang = ce * np.cos(phi)[None, :] * sdir[0] + se_r * sdir[1] + ce * np.sin(phi)[None, :] * sdir[2]
        ang = np.arccos(np.clip(cosang, -1.0, 1.0))
        sun = sun_peak * np.exp(-0.5 * (ang / sig) ** 2)
        out[rows, :, :3] += (sun[..., None] * np.array([1.0, 0.95, 0.85])).astype(np.float32)
    return out


def lookat(pos, target):
    """Rows of the reference's lookat camera matrix (src/math/matrix4.cu:55-67), float64."""
    pos = np.asarray(pos, np.float64)
    f = np.asarray(target, np.float64) - pos
    f /= np.linalg.norm(f)
    r = np.cross([0.0, 1.0, 0.0], f)
    r /= np.linalg.norm(r)
    u = np.cross(f, r)
    u /= np.linalg.norm(u)
    return np.array([[r[0], u[0], f[0], pos[0]], [r[1], u[1], f[1], pos[1]], [r[2], u[2], f[2], pos[2]]], np.float32)


# ---------------------------------------------------------------- scenes
def traversal_scene(tris: int = 100_000, seed: int = 1, width: int = 1024, height: int = 1024,
                    env_size=(2048, 1024), alpha: float = 0.2) -> SceneData:
    """Displaced icosphere (~tris triangles) in rough gold (GGX, alpha), 20 x 20 ground quad
    at y = -1.2 with a 16 x 16 checkerboard lambert, synthetic environment map."""
    s = SceneData()
    P, T = displaced_icosphere(freq_for_tris(tris), seed)
    m_sphere = s.add_mesh(Mesh(P, T, leaf_size=4))
    GP, GT, GUV = quad(20.0, -1.2)
    m_ground = s.add_mesh(Mesh(GP, GT, texcoords=GUV, leaf_size=4))
    tiny = s.constant((alpha, alpha, alpha))
    gold = s.add_material(Material(C.MAT_ROUGHCONDUCTOR, s.constant((0, 0, 0)), tiny, eta=GOLD_ETA, k=GOLD_K,
                                   distribution=C.DIST_GGX))
    checker = s.add_texture(Texture(C.TEX_CHECKERBOARD, color=(0.8, 0.8, 0.8), off=(0.2, 0.2, 0.2), scale=(16.0, 16.0)))
    ground = s.add_material(Material(C.MAT_LAMBERT, checker, s.constant((1e-4, 1e-4, 1e-4))))
    s.add_instance(m_sphere, gold)
    s.add_instance(m_ground, ground)
    s.env_tex = s.add_texture(Texture(C.TEX_BITMAP, texels=environment_map(seed, *env_size), hdr=1))
    s.camera_transform = lookat((0.0, 0.8, -4.2), (0.0, -0.15, 0.0))
    s.camera_fov, s.camera_dof, s.camera_aperture = 40.0, 1.0, 0.0
    s.width, s.height = width, height
    s.ray_bias = 1e-4
    s.tonemapper = C.TONE_LINEAR
    return s


def cornell_scene(width: int = 256, height: int = 256, light=(17.0, 12.0, 4.0), spheres=True) -> SceneData:
    """555-unit Cornell box from 5 wall quads and a 130 x 105 ceiling light."""
    s = SceneData()
    qP = np.array([(-0.5, -0.5, 0), (0.5, -0.5, 0), (0.5, 0.5, 0), (-0.5, 0.5, 0)], np.float32)
    qT = np.array([(0, 1, 2), (0, 2, 3)], np.int32)
    qm = s.add_mesh(Mesh(qP, qT))
    rough = s.constant((1e-4, 1e-4, 1e-4))
    white = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.725, 0.71, 0.68)), rough))
    red = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.63, 0.065, 0.05)), rough))
    green = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.14, 0.45, 0.091)), rough))
    lamp = s.add_material(Material(C.MAT_EMISSIVE, s.constant(light), rough))

    def place(t, sc, rot_x=0.0, rot_y=0.0):
        rx, ry = math.radians(rot_x), math.radians(rot_y)
        Rx = np.array([[1, 0, 0], [0, math.cos(rx), -math.sin(rx)], [0, math.sin(rx), math.cos(rx)]])
        Ry = np.array([[math.cos(ry), 0, math.sin(ry)], [0, 1, 0], [-math.sin(ry), 0, math.cos(ry)]])
        M = np.zeros((3, 4))
        M[:, :3] = Rx @ Ry @ np.diag(sc)
        M[:, 3] = t
        return M

    s.add_instance(qm, white, place((277.5, 0, 277.5), (555, 555, 555), rot_x=90))
    s.add_instance(qm, white, place((277.5, 555, 277.5), (555, 555, 555), rot_x=90))
    s.add_instance(qm, white, place((277.5, 277.5, 555), (555, 555, 555)))
    s.add_instance(qm, red, place((0, 277.5, 277.5), (555, 555, 555), rot_y=90))
    s.add_instance(qm, green, place((555, 277.5, 277.5), (555, 555, 555), rot_y=90))
    s.add_instance(qm, lamp, place((277.5, 554.99, 277.5), (130, 105, 1), rot_x=90))
    if spheres:
        mirror = s.add_material(Material(C.MAT_REFLECTIVE, s.constant((1, 1, 1)), rough))
        glass = s.add_material(Material(C.MAT_REFRACTIVE, s.constant((1, 1, 1)), rough, ior=1.5))
        s.add_sphere((185.0, 90.0, 370.0), 90.0, mirror)
        s.add_sphere((370.0, 90.0, 185.0), 90.0, glass)
    M = np.zeros((3, 4), np.float32)
    M[:, :3] = np.eye(3)
    M[:, 3] = (278.0, 273.0, -800.0)
    s.camera_transform = M
    s.camera_fov, s.camera_dof, s.camera_aperture = 40.0, 1.0, 0.0
    s.width, s.height = width, height
    s.ray_bias = 0.01
    return s


def sss_scene(tris: int = 700_000, seed: int = 3, width: int = 960, height: int = 720, exact_hg=False) -> SceneData:
    """Displaced mesh with a smooth dielectric boundary (ior 1.3) enclosing a homogeneous
    medium (sigma_a = (0.01, 0.08, 0.3), sigma_s = 1, g = 0.7) in the Cornell box."""
    s = cornell_scene(width, height, spheres=False)
    P, T = displaced_icosphere(freq_for_tris(tris), seed)
    m = s.add_mesh(Mesh(P, T))
    sigma_a = np.array([0.01, 0.08, 0.3])
    med = s.add_medium(sigma_a, 1.0, 0.7)   # JSON absorption = 1 - sigma_a, stored as sigma_a
    glass = s.add_material(Material(C.MAT_REFRACTIVE, s.constant((1, 1, 1)), s.constant((1e-4,) * 3), ior=1.3,
                                    medium=med))
    M = np.zeros((3, 4), np.float32)
    M[:, :3] = np.eye(3) * 120.0
    M[:, 3] = (277.5, 140.0, 277.5)
    s.add_instance(m, glass, M)
    return s


# ---------------------------------------------------------------- batched and served workloads
def random_rotation(rng) -> np.ndarray:
    """Uniform random rotation (unit quaternion from four normals)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def mixed_material(s: SceneData, rng) -> int:
    """One of: lambert (albedo U[0.1, 0.9]), GGX rough dielectric (alpha U[0.05, 0.5],
    ior 1.5), smooth plastic (ior 1.5, diffuse U[0.1, 0.9]), rough copper (GGX alpha
    U[0.05, 0.5])."""
    kind = int(rng.integers(4))
    if kind == 0:
        return s.add_material(Material(C.MAT_LAMBERT, s.constant(rng.uniform(0.1, 0.9, 3)), s.constant((1e-4,) * 3)))
    if kind == 1:
        a = float(rng.uniform(0.05, 0.5))
        return s.add_material(Material(C.MAT_ROUGHREFRACTIVE, s.constant((1, 1, 1)), s.constant((a, a, a)), ior=1.5,
                                       distribution=C.DIST_GGX))
    if kind == 2:
        return s.add_material(Material(C.MAT_PLASTIC, s.constant(rng.uniform(0.1, 0.9, 3)), s.constant((1e-4,) * 3),
                                       ior=1.5))
    a = float(rng.uniform(0.05, 0.5))
    return s.add_material(Material(C.MAT_ROUGHCONDUCTOR, s.constant((0, 0, 0)), s.constant((a, a, a)),
                                   eta=COPPER_ETA, k=COPPER_K, distribution=C.DIST_GGX))


class MeshPool:
    """Displaced icospheres of `count` sizes log-uniformly spaced in [lo, hi] triangles
    (distinct seeds); instances draw a log-uniform size and take the nearest pool mesh."""

    def __init__(self, count: int = 16, lo: int = 5_000, hi: int = 700_000, seed: int = 2):
        self.sizes = np.exp(np.linspace(math.log(lo), math.log(hi), count))
        self.lo, self.hi, self.seed = lo, hi, seed
        self.meshes = {}

    def get(self, k: int):
        if k not in self.meshes:
            self.meshes[k] = displaced_icosphere(freq_for_tris(int(self.sizes[k])), self.seed * 1000 + k)
        return self.meshes[k]

    def draw(self, rng) -> int:
        n = math.exp(rng.uniform(math.log(self.lo), math.log(self.hi)))
        return int(np.argmin(np.abs(np.log(self.sizes) - math.log(n))))


def scene_bounds(s: SceneData):
    lo, hi = np.full(3, np.inf), np.full(3, -np.inf)
    for (m, _, M, _, _) in s.instances:
        P = s.meshes[m].positions.astype(np.float64) @ M[:, :3].T.astype(np.float64) + M[:, 3]
        lo, hi = np.minimum(lo, P.min(0)), np.maximum(hi, P.max(0))
    for (c, r, _) in s.spheres:
        lo, hi = np.minimum(lo, np.array(c) - r), np.maximum(hi, np.array(c) + r)
    return lo, hi


def batch_jobs(n: int = 64, seed: int = 2, pool: MeshPool = None, env=None, depth: int = 15,
               resolutions=(128, 256, 512, 1024), spp_range=(64, 1024)):
    """Uneven jobs: resolution uniform in `resolutions` (square), spp uniform in spp_range,
    1-8 displaced icospheres (5k-700k triangles, log-uniform, from a mesh pool) with random
    affine transforms (uniform rotation, scale U[0.5, 2], translation in a 10-unit box),
    mixed materials, the traversal scene's environment map. Returns [(SceneData, dict)]
    with the render settings of each job (width, height, spp, max_depth, seed, job)."""
    rng = np.random.default_rng(seed)
    pool = pool or MeshPool(seed=seed)
    env = environment_map(1) if env is None else env
    out = []
    for j in range(n):
        s = SceneData()
        res = int(rng.choice(resolutions))
        spp = int(rng.integers(spp_range[0], spp_range[1] + 1))
        ninst = int(rng.integers(1, 9))
        used = {}
        for _ in range(ninst):
            k = pool.draw(rng)
            if k not in used:
                P, T = pool.get(k)
                used[k] = s.add_mesh(Mesh(P, T))
            M = np.zeros((3, 4))
            M[:, :3] = random_rotation(rng) * rng.uniform(0.5, 2.0)
            M[:, 3] = rng.uniform(-5.0, 5.0, 3)
            s.add_instance(used[k], mixed_material(s, rng), M.astype(np.float32))
        s.env_tex = s.add_texture(Texture(C.TEX_BITMAP, texels=env, hdr=1))
        lo, hi = scene_bounds(s)
        c = 0.5 * (lo + hi)
        radius = 0.5 * float(np.linalg.norm(hi - lo))
        s.camera_transform = lookat(c + np.array([0.0, 0.35, -1.0]) / np.linalg.norm([0.0, 0.35, -1.0]) * 2.6 * radius, c)
        s.camera_fov, s.camera_dof, s.camera_aperture = 40.0, 1.0, 0.0
        s.width = s.height = res
        s.ray_bias = 1e-3
        s.tonemapper = C.TONE_LINEAR
        out.append((s, dict(width=res, height=res, spp=spp, max_depth=depth, seed=seed, job=j)))
    return out


def instanced_scene(count: int = 16, tris: int = 125_000, seed: int = 5, env=None) -> SceneData:
    """`count` distinct displaced icospheres of ~`tris` triangles each on a 4-wide grid
    (spacing 3, uniform random rotations), mixed materials, environment lighting."""
    rng = np.random.default_rng(seed)
    s = SceneData()
    f = freq_for_tris(tris)
    for i in range(count):
        P, T = displaced_icosphere(f, seed * 1000 + i)
        m = s.add_mesh(Mesh(P, T))
        M = np.zeros((3, 4))
        M[:, :3] = random_rotation(rng)
        M[:, 3] = (3.0 * (i % 4) - 4.5, 0.0, 3.0 * (i // 4) - 4.5)
        s.add_instance(m, mixed_material(s, rng), M.astype(np.float32))
    s.env_tex = s.add_texture(Texture(C.TEX_BITMAP, texels=environment_map(1) if env is None else env, hdr=1))
    s.camera_transform = lookat((0.0, 8.0, -14.0), (0.0, 0.0, 0.0))
    s.width, s.height = 1024, 1024
    s.ray_bias = 1e-3
    return s


def orbit_camera(s: SceneData, rng, fov: float = 40.0) -> np.ndarray:
    """15 floats (camera rows, fov, dof, aperture) of a camera on an orbit around the
    scene: azimuth U[0, 2 pi), elevation U[5, 60] degrees, radius 3x the scene radius."""
    lo, hi = scene_bounds(s)
    c = 0.5 * (lo + hi)
    radius = 0.5 * float(np.linalg.norm(hi - lo))
    az = rng.uniform(0.0, 2 * math.pi)
    el = math.radians(rng.uniform(5.0, 60.0))
    pos = c + 3.0 * radius * np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    out = np.zeros(15, np.float32)
    out[:12] = lookat(pos, c).reshape(-1)
    out[12], out[13], out[14] = fov, 1.0, 0.0
    return out


def request_stream(n: int, scenes: int, seed: int = 4, rate: float = 40.0, max_res=(1920, 1080), min_res=64,
                   spp_range=(16, 4096), depth_range=(10, 25)):
    """Seeded Poisson arrivals (mean `rate` per second). Each request: scene index,
    resolution log-uniform between min_res^2 and max_res (one draw scales both sides),
    spp log-uniform in spp_range, depth uniform in depth_range, an orbit-pose seed."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        a = rng.uniform()
        w = int(round(min_res * (max_res[0] / min_res) ** a))
        h = int(round(min_res * (max_res[1] / min_res) ** a))
        spp = int(round(math.exp(rng.uniform(math.log(spp_range[0]), math.log(spp_range[1])))))
        depth = int(rng.integers(depth_range[0], depth_range[1] + 1))
        out.append(dict(arrival=t, scene=int(rng.integers(scenes)), width=w, height=h, spp=spp, max_depth=depth,
                        pose_seed=int(rng.integers(1 << 30)), job=i))
    return out
