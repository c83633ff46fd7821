"""Seeded synthetic scenes and ray batches for the ray-batch intersection path.

The reference ships no benchmark scenes for its GPU accelerators (its
``scenes/conference`` and ``scenes/sibenik`` geometry is missing), so the
workloads are generated here from fixed seeds.  All geometry is float32 in
world space, one record of nine floats per triangle (v0.xyz v1.xyz v2.xyz),
which is the layout the reference packs for its kernels
(accelerators/naive.cpp:59-101, ``vertices[9*n]``).

Ray batches are SoA float32 arrays of shape [8, n]: rows ox, oy, oz, dx, dy,
dz, mint, maxt (core/geometry.h:314-336, ``Ray::o, d, mint, maxt``).
"""
from __future__ import annotations

import math

import numpy as np

F32 = np.float32


# ----------------------------------------------------------------- meshes

def uv_sphere(radius: float = 1.0, nseg: int = 64, nring: int = 32,
              center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """UV sphere: nring latitude bands x nseg quads, two triangles per quad.

    The 64 zero-area triangles of the north-pole band are dropped and those
    of the south-pole band kept, which gives 32*64*2 - 64 = 4,032 triangles
    for the 64x32 sphere of the small naive workload.  The kept pole
    triangles have two coincident vertices and exercise pbrt's
    ``divisor == 0`` rejection (shapes/trianglemesh.cpp:131).
    """
    th = np.pi * np.arange(nring + 1, dtype=np.float64) / nring
    ph = 2.0 * np.pi * np.arange(nseg + 1, dtype=np.float64) / nseg
    st, ct = np.sin(th), np.cos(th)
    st[0] = 0.0
    st[-1] = 0.0
    ct[0], ct[-1] = 1.0, -1.0
    sp, cp = np.sin(ph), np.cos(ph)
    sp[-1], cp[-1] = sp[0], cp[0]
    x = radius * st[:, None] * cp[None, :] + center[0]
    y = radius * ct[:, None] * np.ones_like(cp)[None, :] + center[1]
    z = radius * st[:, None] * sp[None, :] + center[2]
    V = np.stack([x, y, z], -1).astype(F32)  # [nring+1, nseg+1, 3]
    tris = []
    for i in range(nring):
        a = V[i, :-1]
        b = V[i + 1, :-1]
        c = V[i + 1, 1:]
        d = V[i, 1:]
        ta = np.concatenate([a, b, c], -1)
        tb = np.concatenate([a, c, d], -1)
        if i == 0:
            tris.append(ta)  # tb has a == d at the north pole
        else:
            q = np.stack([ta, tb], 1).reshape(-1, 9)
            tris.append(q)
    return np.ascontiguousarray(np.concatenate(tris, 0), dtype=F32)


def ground_quad(y: float = -1.0, half: float = 10.0) -> np.ndarray:
    """Two triangles spanning [-half, half]^2 at height y."""
    p = np.array([[-half, y, -half], [half, y, -half], [half, y, half], [-half, y, half]], F32)
    return np.stack([np.concatenate([p[0], p[1], p[2]]),
                     np.concatenate([p[0], p[2], p[3]])]).astype(F32)


def icosphere(subdiv: int = 3) -> np.ndarray:
    """Unit icosphere with 20*4^subdiv triangles (1,280 at subdivision 3)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
         (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts)
    Fi = np.array(faces)
    return V, Fi


def _rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _value_noise_fbm(x: np.ndarray, z: np.ndarray, rng: np.random.Generator, octaves=6,
                     lacunarity=2.0, gain=0.5, lattice=256) -> np.ndarray:
    """fBm over a seeded value-noise lattice with smoothstep interpolation."""
    table = rng.random((lattice, lattice))
    out = np.zeros_like(x)
    amp, freq = 1.0, 1.0
    norm = 0.0
    for _ in range(octaves):
        fx, fz = x * freq, z * freq
        ix, iz = np.floor(fx).astype(np.int64), np.floor(fz).astype(np.int64)
        tx, tz = fx - ix, fz - iz
        tx = tx * tx * (3 - 2 * tx)
        tz = tz * tz * (3 - 2 * tz)
        a = table[ix % lattice, iz % lattice]
        b = table[(ix + 1) % lattice, iz % lattice]
        c = table[ix % lattice, (iz + 1) % lattice]
        d = table[(ix + 1) % lattice, (iz + 1) % lattice]
        v = (a * (1 - tx) + b * tx) * (1 - tz) + (c * (1 - tx) + d * tx) * tz
        out += amp * (2 * v - 1)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return out / norm


def terrain_icospheres(seed: int = 2, grid: int = 256, extent: float = 16.0,
                       amplitude: float = 2.0, n_spheres: int = 40) -> dict:
    """Height field of (grid-1)^2*2 triangles plus icospheres at subdivision 3.

    256x256 grid -> 130,050 terrain triangles; 40 icospheres x 1,280 ->
    51,200; 181,250 in all.  Heights are 6-octave fBm (lacunarity 2, gain
    0.5) scaled to the amplitude; sphere radii are U[0.2, 1.5] with random
    rotations and positions spread over the terrain, resting on it.
    """
    rng = np.random.default_rng(seed)
    n = grid
    xs = np.linspace(-extent / 2, extent / 2, n)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    H = amplitude * _value_noise_fbm(X / extent * 8.0, Z / extent * 8.0, rng)
    P = np.stack([X, H, Z], -1).astype(F32)
    a = P[:-1, :-1].reshape(-1, 3)
    b = P[1:, :-1].reshape(-1, 3)
    c = P[1:, 1:].reshape(-1, 3)
    d = P[:-1, 1:].reshape(-1, 3)
    t1 = np.concatenate([a, c, b], -1)
    t2 = np.concatenate([a, d, c], -1)
    terrain = np.stack([t1, t2], 1).reshape(-1, 9)
    V, Fi = icosphere(3)
    spheres = []
    for _ in range(n_spheres):
        r = rng.uniform(0.2, 1.5)
        R = _rotation(rng)
        cx, cz = rng.uniform(-extent / 2 + 1.5, extent / 2 - 1.5, size=2)
        gi = int(round((cx + extent / 2) / extent * (n - 1)))
        gk = int(round((cz + extent / 2) / extent * (n - 1)))
        cy = H[gi, gk] + r
        W = (V @ R.T) * r + np.array([cx, cy, cz])
        spheres.append(W[Fi].reshape(-1, 9))
    tris = np.concatenate([terrain] + spheres, 0).astype(F32)
    light = np.array([[-0.5, 12.0, -0.5], [0.5, 12.0, -0.5], [0.5, 12.0, 0.5], [-0.5, 12.0, 0.5]], F32)
    return {"tris": np.ascontiguousarray(tris), "area_light_quad": light,
            "n_terrain": int(terrain.shape[0]), "seed": seed}


def displaced_icospheres(seed: int = 3, n_inst: int = 800, box: float = 40.0,
                         displacement: float = 0.1) -> dict:
    """800 seeded displaced icospheres (1,280 triangles each) in a 40^3 box.

    Each instance perturbs every vertex radially by amplitude*U[-1,1]
    (a per-instance noise field), then applies a log-uniform scale in
    [0.3, 3], a random rotation and a uniform position: 1,024,000 triangles.
    """
    rng = np.random.default_rng(seed)
    V, Fi = icosphere(3)
    out = []
    for _ in range(n_inst):
        disp = 1.0 + displacement * rng.uniform(-1, 1, size=(V.shape[0], 1))
        s = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
        R = _rotation(rng)
        c = rng.uniform(-box / 2, box / 2, size=3)
        W = ((V * disp) @ R.T) * s + c
        out.append(W[Fi].reshape(-1, 9))
    tris = np.concatenate(out, 0).astype(F32)
    return {"tris": np.ascontiguousarray(tris), "seed": seed}


# ------------------------------------------------------------------ rays

def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(np.asarray(up, np.float64), f)
    r /= np.linalg.norm(r)
    u = np.cross(f, r)
    return eye, r, u, f


def pinhole_rays(width: int, height: int, eye, target, fov_deg: float, spp: int = 1,
                 jitter_seed: int | None = None, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Primary rays in breadth-first order: scanlines, spp consecutive samples
    per pixel (renderers/breadth-first.cpp:43-62).  Directions are normalised
    (cameras/perspective.cpp:79); mint = 0, maxt = inf."""
    eye, r, u, f = look_at(eye, target, up)
    n = width * height * spp
    pix = np.arange(width * height)
    px = np.repeat(pix % width, spp).astype(np.float64)
    py = np.repeat(pix // width, spp).astype(np.float64)
    if jitter_seed is None:
        jx = np.full(n, 0.5)
        jy = np.full(n, 0.5)
    else:
        g = np.random.default_rng(jitter_seed)  # PCG64
        jx = g.random(n)
        jy = g.random(n)
    aspect = width / height
    scale = math.tan(math.radians(fov_deg) / 2)
    sx = (2 * (px + jx) / width - 1) * scale * (aspect if aspect > 1 else 1)
    sy = (1 - 2 * (py + jy) / height) * scale / (aspect if aspect < 1 else 1)
    d = sx[:, None] * r[None] + sy[:, None] * u[None] + f[None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.empty((8, n), F32)
    rays[0:3] = eye.astype(F32)[:, None]
    rays[3:6] = d.T.astype(F32)
    rays[6] = 0.0
    rays[7] = np.inf
    return rays


def random_rays(n: int, lo, hi, seed: int, maxt: float = np.inf) -> np.ndarray:
    """Incoherent rays: origins uniform in the box [lo, hi], directions
    uniform on the sphere."""
    g = np.random.default_rng(seed)
    o = g.uniform(lo, hi, size=(n, 3))
    d = g.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.empty((8, n), F32)
    rays[0:3] = o.T
    rays[3:6] = d.T
    rays[6] = 0.0
    rays[7] = maxt
    return rays


def shadow_rays_to_point(points: np.ndarray, light, eps: float = 1e-3) -> np.ndarray:
    """Shadow segments from surface points to a point light, built like
    VisibilityTester::SetSegment (core/light.h:79-84): normalised direction,
    mint = eps, maxt = dist * (1 - eps)."""
    light = np.asarray(light, np.float32)
    d = (light[None, :] - points).astype(F32)
    dist = np.sqrt((d.astype(np.float64) ** 2).sum(1)).astype(F32)
    dn = (d / dist[:, None]).astype(F32)
    rays = np.empty((8, points.shape[0]), F32)
    rays[0:3] = points.T
    rays[3:6] = dn.T
    rays[6] = eps
    rays[7] = dist * (1 - eps)
    return rays


def config_small_naive() -> dict:
    """The small naive workload: 256x256, 1 spp at pixel centres, camera at
    (0,1,-4) looking at the origin with 45 degree fov; UV sphere r=1
    (4,032 triangles) + ground quad at y=-1 (+-10); point light (2,4,-2)."""
    tris = np.concatenate([uv_sphere(), ground_quad()], 0)
    rays = pinhole_rays(256, 256, (0.0, 1.0, -4.0), (0.0, 0.0, 0.0), 45.0, 1)
    return {"tris": tris, "rays": rays, "light": np.array([2.0, 4.0, -2.0], F32)}


# ------------------------------------------------------- many-scene batch

def surface_points(tris: np.ndarray, n: int, rng: np.random.Generator, eps: float = 1e-3):
    """n uniform points on uniformly chosen triangles, lifted by eps along
    the geometric normal (turned towards +y), and that normal."""
    idx = rng.integers(0, tris.shape[0], n)
    v = tris[idx].astype(np.float64).reshape(n, 3, 3)
    su = np.sqrt(rng.random(n))
    b = rng.random(n)
    p = (1 - su)[:, None] * v[:, 0] + (su * (1 - b))[:, None] * v[:, 1] + (su * b)[:, None] * v[:, 2]
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(ln > 0, nrm / np.maximum(ln, 1e-30), np.array([0.0, 1.0, 0.0]))
    nrm *= np.where(nrm[:, 1:2] < 0, -1.0, 1.0)
    return p + eps * nrm, nrm


def _cosine_dirs(nrm: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """Cosine-weighted directions about each normal (Malley's method)."""
    n = nrm.shape[0]
    r = np.sqrt(rng.random(n))
    phi = 2 * np.pi * rng.random(n)
    lx, ly = r * np.cos(phi), r * np.sin(phi)
    lz = np.sqrt(np.maximum(0.0, 1 - lx * lx - ly * ly))
    a = np.where(np.abs(nrm[:, 0:1]) > 0.9, np.array([0.0, 1.0, 0.0]), np.array([1.0, 0.0, 0.0]))
    t = np.cross(nrm, a)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    s = np.cross(nrm, t)
    d = lx[:, None] * t + ly[:, None] * s + lz[:, None] * nrm
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _rays(o: np.ndarray, d: np.ndarray, mint, maxt) -> np.ndarray:
    rays = np.empty((8, o.shape[0]), F32)
    rays[0:3] = o.T
    rays[3:6] = d.T
    rays[6] = mint
    rays[7] = maxt
    return rays


def many_scenes(seed: int = 5, n_scenes: int = 64, median_tris: int = 20000, sigma: float = 1.0,
                tri_range=(1000, 500000), ray_range=(4096, 1 << 20), split=(0.4, 0.3, 0.3)) -> list:
    """Independent scenes for the batched many-scene pipeline.

    Triangle counts are log-normal (median 20k, sigma 1, clipped to
    [1k, 500k]); each scene is a terrain + icospheres scene of that size
    (half terrain, half subdivision-3 icospheres, as terrain_icospheres
    builds them).  Rays per scene are uniform in [4k, 1M] and mixed:
    primary camera rays (nearest hit), path rays from surface points in
    cosine-weighted directions (nearest hit; what bounce-3 rays look like:
    incoherent, leaving surfaces) and shadow segments from surface points to
    seeded points on the area light (any hit).  Each entry: tris, near
    ([8, n] rays), shadow ([8, m] rays), kinds (counts of primary / path /
    shadow)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        target = int(np.clip(round(math.exp(rng.normal(math.log(median_tris), sigma))),
                             tri_range[0], tri_range[1]))
        n_sph = max(1, int(round(target / 2 / 1280)))
        grid = max(8, int(round(math.sqrt(max(target - n_sph * 1280, 128) / 2))) + 1)
        sc = terrain_icospheres(seed=1000 + k, grid=grid, n_spheres=n_sph)
        tris = sc["tris"]
        nr = int(rng.integers(ray_range[0], ray_range[1] + 1))
        n_prim = int(nr * split[0])
        n_path = int(nr * split[1])
        n_shad = nr - n_prim - n_path
        side = int(math.ceil(math.sqrt(n_prim)))
        prim = pinhole_rays(side, side, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, 1,
                            jitter_seed=2000 + k)[:, :n_prim]
        p, nrm = surface_points(tris, n_path, rng)
        path = _rays(p, _cosine_dirs(nrm, rng), 0.0, np.inf)
        q, _ = surface_points(tris, n_shad, rng)
        quad = sc["area_light_quad"].astype(np.float64)
        u, v = rng.random(n_shad), rng.random(n_shad)
        lp = quad[0] + u[:, None] * (quad[1] - quad[0]) + v[:, None] * (quad[3] - quad[0])
        d = lp - q
        dist = np.linalg.norm(d, axis=1)
        shad = _rays(q, d / dist[:, None], 1e-3, (dist * (1 - 1e-3)).astype(F32))
        near = np.ascontiguousarray(np.concatenate([prim, path], 1))
        out.append({"tris": tris, "near": near, "shadow": np.ascontiguousarray(shad),
                    "kinds": (n_prim, n_path, n_shad)})
    return out
