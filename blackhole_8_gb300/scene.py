"""Python mirror of the reference's scene API and the synthetic workloads.

The classes follow the reference's C++ types one to one (FP64), so a scene is
built the way the reference's main() builds it and then resolved to the
``bh_scene`` POD of the C ABI:

- ``Object``          object/object.h:23-118 (vertex list whose [0] is the
                      position; Rotate*/Move* about the object's own axes via
                      RotationMatrixForAxis, matrix.h:342-356)
- ``Camera``          camera.h:21-71 (axes (1,0,0), (0,-1,0), (0,0,-1); fov
                      clamp and focus length W / (2 tan(fov/2)))
- ``StaticBlackhole`` blackhole_solution.h:16-96
- ``Annulus``         object/vector_object.h:306-356 (the default (0,0,0)
                      vertex is kept and the four quad corners follow it; the
                      normal is fixed at construction)

Every pose operation is also logged in ``ops`` so the same sequence can be
replayed on the reference's own objects.

Textures are generated by integer hashing, so they are identical on every
machine and numpy version.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import capi


def normalize(v) -> np.ndarray:
    """cv::normalize semantics: v * (1/|v|), zero vector stays zero."""
    v = np.asarray(v, dtype=np.float64)
    n = math.sqrt(float(v @ v))
    return v * (1.0 / n if n != 0 else 0.0)


def rotation_matrix_for_axis(v, theta: float) -> np.ndarray:
    """Rodrigues rotation about axis v by theta (matrix.h:342-356)."""
    ux, uy, uz = normalize(v)
    c = math.cos(theta)
    c2 = 1 - c
    s = math.sin(theta)
    return np.array([
        [c + ux * ux * c2, ux * uy * c2 - uz * s, ux * uz * c2 + uy * s],
        [uy * ux * c2 + uz * s, c + uy * uy * c2, uy * uz * c2 - ux * s],
        [uz * ux * c2 - uy * s, uz * uy * c2 + ux * s, c + uz * uz * c2],
    ])


class Object:
    """Object<T> (object/object.h:23-118)."""

    def __init__(self, vertices=((0.0, 0.0, 0.0),), vx=(1, 0, 0), vy=(0, 1, 0), vz=(0, 0, 1)):
        self._v = [np.array(p, dtype=np.float64) for p in vertices]
        self._vx = normalize(vx)
        self._vy = normalize(vy)
        self._vz = normalize(vz)
        self.ops: list[tuple] = []

    def _rotate(self, r: np.ndarray) -> None:
        pos = self._v[0].copy()
        self._v = [r @ (v - pos) + pos for v in self._v]

    def RotateZ(self, rad: float) -> None:
        r = rotation_matrix_for_axis(self._vz, rad)
        self._vx = normalize(r @ self._vx)
        self._vy = normalize(r @ self._vy)
        self._rotate(r)
        self.ops.append(("RotateZ", float(rad)))

    def RotateY(self, rad: float) -> None:
        r = rotation_matrix_for_axis(self._vy, rad)
        self._vx = normalize(r @ self._vx)
        self._vz = normalize(r @ self._vz)
        self._rotate(r)
        self.ops.append(("RotateY", float(rad)))

    def RotateX(self, rad: float) -> None:
        r = rotation_matrix_for_axis(self._vx, rad)
        self._vy = normalize(r @ self._vy)
        self._vz = normalize(r @ self._vz)
        self._rotate(r)
        self.ops.append(("RotateX", float(rad)))

    def MoveTo(self, x, y=None, z=None) -> None:
        p = np.array(x if y is None else (x, y, z), dtype=np.float64)
        self._v[0] = p
        self.ops.append(("MoveTo", *map(float, p)))

    def Move(self, dx: float, dy: float, dz: float) -> None:
        self.MoveX(dx)
        self.MoveY(dy)
        self.MoveZ(dz)

    def MoveX(self, d: float) -> None:
        self._v = [v + self._vx * d for v in self._v]
        self.ops.append(("MoveX", float(d)))

    def MoveY(self, d: float) -> None:
        self._v = [v + self._vy * d for v in self._v]
        self.ops.append(("MoveY", float(d)))

    def MoveZ(self, d: float) -> None:
        self._v = [v + self._vz * d for v in self._v]
        self.ops.append(("MoveZ", float(d)))

    def position(self) -> np.ndarray:
        return self._v[0]

    def vector_x(self) -> np.ndarray:
        return self._vx

    def vector_y(self) -> np.ndarray:
        return self._vy

    def vector_z(self) -> np.ndarray:
        return self._vz

    def vertex(self) -> list[np.ndarray]:
        return self._v


class Camera(Object):
    """Camera<T> (camera.h:21-71)."""

    def __init__(self, width: int, height: int, fov_x: float):
        super().__init__(((0.0, 0.0, 0.0),), (1, 0, 0), (0, -1, 0), (0, 0, -1))
        self._w = int(width)
        self._h = int(height)
        self._fov = math.pi / 2
        self._focus_len = 1.0
        self._set_fov(fov_x)

    def _set_fov(self, fov_x: float) -> None:
        fov_x = min(max(0.0, float(fov_x)), math.nextafter(math.pi, 0.0))
        self._fov = fov_x
        self._focus_len = self._w / (2 * math.tan(fov_x / 2.0))

    def fov(self, fov_x: float | None = None):
        """fov() reads; fov(x) clamps to [0, pi) and sets the focus length."""
        if fov_x is None:
            return self._fov
        self._set_fov(fov_x)
        self.ops.append(("Fov", float(fov_x)))
        return None

    def width(self) -> int:
        return self._w

    def height(self) -> int:
        return self._h

    def focus(self) -> np.ndarray:
        return self.position()

    def focus_len(self) -> float:
        return self._focus_len

    def focus_vector(self) -> np.ndarray:
        return self._vx * self._focus_len

    def PixelVector(self, x: int, y: int, focus_v=None) -> np.ndarray:
        fv = self.focus_vector() if focus_v is None else focus_v
        return fv - self._vy * (self._w / 2.0 - x) - self._vz * (self._h / 2.0 - y)

    def to_c(self) -> capi.Camera:
        c = capi.Camera()
        c.position[:] = list(self.position())
        c.axis_x[:] = list(self._vx)
        c.axis_y[:] = list(self._vy)
        c.axis_z[:] = list(self._vz)
        c.focus_len = self._focus_len
        c.width = self._w
        c.height = self._h
        return c


class StaticBlackhole(Object):
    """StaticBlackhole<T> (blackhole_solution.h:16-96)."""

    def __init__(self, position, mass: float):
        super().__init__((position,))
        self._mass = float(mass)
        self._b_c = 3.0 * math.sqrt(3) * self._mass

    def mass(self) -> float:
        return self._mass

    def b_c(self) -> float:
        return self._b_c

    def radius(self) -> float:
        return 2 * self._mass

    def center(self) -> np.ndarray:
        return self.position()

    def G(self, u: float, b: float) -> float:
        return (u * u * (2.0 * self._mass * u - 1.0)) + (1.0 / (b * b))

    def InvSqrtG(self, u: float, b: float) -> float:
        return 1.0 / math.sqrt(self.G(u, b))

    def to_c(self) -> capi.Hole:
        h = capi.Hole()
        h.position[:] = list(self.position())
        h.mass = self._mass
        return h


class Annulus(Object):
    """Annulus<T> (vector_object.h:306-356): quad corners p1..p4 follow the
    default (0,0,0) vertex, which is the disc centre."""

    def __init__(self, p1, p2, p3, p4, r_outer: float, r_inner: float):
        super().__init__(((0.0, 0.0, 0.0), p1, p2, p3, p4))
        self.construction = tuple(np.array(p, dtype=np.float64) for p in (p1, p2, p3, p4))
        p1, p2, p3 = (np.asarray(p, dtype=np.float64) for p in (p1, p2, p3))
        self._norm = normalize(np.cross(p3 - p1, p2 - p1))
        self._r_inner = float(r_inner)
        self._r_outer = float(r_outer)
        self.texture: Texture | None = None
        self.mapping = capi.DISC_MAP_REF_PLANAR

    def SetTexture(self, texture: "Texture") -> None:
        if texture is None or texture.empty():
            raise ValueError("empty texture (the reference terminates here, material.h:30-33)")
        self.texture = texture

    def center(self) -> np.ndarray:
        return self._v[0]

    def norm(self) -> np.ndarray:
        return self._norm

    def r_inner(self) -> float:
        return self._r_inner

    def r_outer(self) -> float:
        return self._r_outer

    def to_c(self, texture_id: int) -> capi.Disc:
        d = capi.Disc()
        v = self._v
        d.center[:] = list(v[0])
        d.normal[:] = list(self._norm)
        d.corner[:] = list(v[1])
        d.edge_s1[:] = list(v[2] - v[1])
        d.edge_s2[:] = list(v[4] - v[1])
        d.r_inner = self._r_inner
        d.r_outer = self._r_outer
        d.texture = texture_id
        d.mapping = self.mapping
        d.enabled = 1
        return d


class Rectangle(Object):
    """Rectangle<T> (vector_object.h:80-183): corners p1..p4 follow the
    default (0,0,0) vertex; drawn by Rectangle::color from its texture."""

    def __init__(self, p1, p2, p3, p4):
        super().__init__(((0.0, 0.0, 0.0), p1, p2, p3, p4))
        self.construction = tuple(np.array(p, dtype=np.float64) for p in (p1, p2, p3, p4))
        self.texture: Texture | None = None

    def SetTexture(self, texture: "Texture") -> None:
        if texture is None or texture.empty():
            raise ValueError("empty texture (the reference terminates here, material.h:30-33)")
        self.texture = texture

    def to_c(self, texture_ids: dict) -> capi.Object:
        o = capi.Object()
        o.type = capi.OBJECT_RECTANGLE
        o.texture = texture_ids[id(self.texture)] if self.texture is not None else -1
        for k in range(4):
            o.v[k][:] = list(self._v[k + 1])
        return o


class Triangle(Object):
    """Triangle<T> (vector_object.h:18-77): vertices v1..v3 follow the default
    (0,0,0) vertex; it has no colour of its own (black, material.h:54)."""

    def __init__(self, v1, v2, v3):
        super().__init__(((0.0, 0.0, 0.0), v1, v2, v3))

    def to_c(self, texture_ids: dict) -> capi.Object:
        o = capi.Object()
        o.type = capi.OBJECT_TRIANGLE
        o.texture = -1
        for k in range(3):
            o.v[k][:] = list(self._v[k + 1])
        return o


class ChessPattern2D:
    """ChessPattern2D<T> (pattern.h:14-50): black and white cells of
    `pattern_size`."""

    def __init__(self, pattern_size: float = 1):
        self.pattern_size = float(pattern_size)


class InfinitePlane(Object):
    """InfinitePlane<T> (vector_object.h:187-238): the plane through
    position() normal to vector_z(), coloured by a ChessPattern2D (or black)."""

    def __init__(self, p, pattern: ChessPattern2D | None = None):
        super().__init__((p,))
        self.construction = (np.array(p, dtype=np.float64),)
        self.pattern = pattern

    def to_c(self, texture_ids: dict) -> capi.Object:
        o = capi.Object()
        o.type = capi.OBJECT_PLANE
        o.texture = -1
        o.v[0][:] = list(self._v[0])
        o.axis_x[:] = list(self._vx)
        o.axis_y[:] = list(self._vy)
        o.axis_z[:] = list(self._vz)
        o.pattern_size = self.pattern.pattern_size if self.pattern is not None else 0.0
        return o


class Texture:
    """Host texture (H, W, C) uint8 with a channel layout (capi.TEXEL_*)."""

    def __init__(self, texels: np.ndarray, layout: int):
        self.texels = np.ascontiguousarray(texels, dtype=np.uint8)
        self.layout = layout

    def empty(self) -> bool:
        return self.texels.size == 0

    @property
    def width(self) -> int:
        return self.texels.shape[1]

    @property
    def height(self) -> int:
        return self.texels.shape[0]

    def bgra(self) -> np.ndarray:
        """The texels as BGRA8 (the device layout)."""
        t = self.texels
        out = np.empty(t.shape[:2] + (4,), dtype=np.uint8)
        if self.layout == capi.TEXEL_BGR8:
            out[..., :3] = t[..., :3]
            out[..., 3] = 255
        elif self.layout == capi.TEXEL_RGB8:
            out[..., :3] = t[..., 2::-1]
            out[..., 3] = 255
        elif self.layout == capi.TEXEL_BGRA8:
            out[...] = t
        else:
            out[..., :3] = t[..., 2::-1]
            out[..., 3] = t[..., 3]
        return out


@dataclass
class Scene:
    camera: Camera
    hole: StaticBlackhole
    disc: Annulus | None = None
    background: Texture | None = None
    meta: dict = field(default_factory=dict)
    objects: list = field(default_factory=list)  # Rectangle / Triangle / InfinitePlane, in table order
    extra_holes: list = field(default_factory=list)  # further StaticBlackholes (MULTI integrator)

    def textures(self) -> list:
        """Every texture the scene draws with."""
        out = [t for t in (self.disc.texture if self.disc is not None else None, self.background) if t is not None]
        out += [o.texture for o in self.objects if getattr(o, "texture", None) is not None]
        return out

    def to_c(self, texture_ids: dict) -> capi.Scene:
        """The C scene; its object and extra-hole tables live in the returned
        struct's `_keep` attribute, which the caller keeps alive while the C
        ABI reads it."""
        s = capi.Scene()
        s.camera = self.camera.to_c()
        s.hole = self.hole.to_c()
        if self.disc is not None:
            s.disc = self.disc.to_c(texture_ids[id(self.disc.texture)])
        else:
            s.disc.enabled = 0
            s.disc.texture = -1
        s.background = texture_ids[id(self.background)] if self.background is not None else -1
        keep = []
        if self.objects:
            arr = (capi.Object * len(self.objects))(*[o.to_c(texture_ids) for o in self.objects])
            s.objects = C.cast(arr, C.POINTER(capi.Object))
            s.n_objects = len(self.objects)
            keep.append(arr)
        if self.extra_holes:
            harr = (capi.Hole * len(self.extra_holes))(*[h.to_c() for h in self.extra_holes])
            s.extra_holes = C.cast(harr, C.POINTER(capi.Hole))
            s.n_extra_holes = len(self.extra_holes)
            keep.append(harr)
        s._keep = keep or None
        return s


# ---------------------------------------------------------------------------
# deterministic procedural textures (integer hashing, no RNG streams)
_M32 = np.uint64(0xFFFFFFFF)


def _hash32(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.uint64) & _M32
    x ^= x >> np.uint64(16)
    x = (x * np.uint64(0x7FEB352D)) & _M32
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x846CA68B)) & _M32
    x ^= x >> np.uint64(16)
    return x


def hash_u01(*keys) -> np.ndarray:
    """Uniform [0, 1) from integer keys (broadcasting arrays)."""
    h = np.uint64(0x9E3779B9)
    for k in keys:
        h = _hash32(np.asarray(k, dtype=np.uint64) ^ h)
    return h.astype(np.float64) / 4294967296.0


def disc_ring_texture(seed: int, width: int = 1024, height: int = 64) -> Texture:
    """4-colour radial-ring RGBA8 texture for the polar disc mapping: x is the
    radius, y the azimuth. Ring boundaries and the 4-colour palette come from
    the seed; the colour of a ring shifts by one palette entry per azimuthal
    quarter, so the disc's rotation stays visible. No texel is black."""
    pal = np.stack([40 + (hash_u01(seed, 1, i, np.arange(3)) * 215).astype(np.int64) for i in range(4)])
    n_rings = 12 + int(hash_u01(seed, 2) * 9)
    widths = 0.5 + hash_u01(seed, 3, np.arange(n_rings))
    edges = np.cumsum(widths) / widths.sum() * width
    x = np.arange(width) + 0.5
    ring = np.searchsorted(edges, x, side="right")
    quarter = (np.arange(height) * 4) // height
    idx = (ring[None, :] + quarter[:, None]) % 4
    rgb = pal[idx]
    out = np.empty((height, width, 4), dtype=np.uint8)
    out[..., :3] = rgb.astype(np.uint8)
    out[..., 3] = 255
    return Texture(out, capi.TEXEL_RGBA8)


def value_noise_background(seed: int, width: int = 2048, height: int = 1024, octaves: int = 4,
                           base_cells: int = 8) -> Texture:
    """Equirectangular RGB8 sky: seeded value noise (smoothstep-interpolated
    lattice, wrapping in longitude) plus sparse white stars."""
    ys = (np.arange(height) + 0.5) / height
    xs = (np.arange(width) + 0.5) / width
    out = np.zeros((height, width, 3), dtype=np.float64)
    for ch in range(3):
        acc = np.zeros((height, width))
        amp, norm = 1.0, 0.0
        for o in range(octaves):
            cx = base_cells * (2 ** o)
            cy = max(1, cx // 2)
            fx = xs * cx
            fy = ys * cy
            ix = np.floor(fx).astype(np.int64)
            iy = np.floor(fy).astype(np.int64)
            tx = fx - ix
            ty = fy - iy
            tx = tx * tx * (3 - 2 * tx)
            ty = ty * ty * (3 - 2 * ty)
            ix0, ix1 = ix % cx, (ix + 1) % cx
            iy0, iy1 = np.minimum(iy, cy), np.minimum(iy + 1, cy)
            # lattice values, hashed once per lattice point
            lattice = hash_u01(seed, 10 + ch, o, np.arange(cy + 1)[:, None], np.arange(cx)[None, :])
            def lat(a, b):
                return lattice[b[:, None], a[None, :]]
            v00, v10 = lat(ix0, iy0), lat(ix1, iy0)
            v01, v11 = lat(ix0, iy1), lat(ix1, iy1)
            top = v00 + (v10 - v00) * tx[None, :]
            bot = v01 + (v11 - v01) * tx[None, :]
            acc += amp * (top + (bot - top) * ty[:, None])
            norm += amp
            amp *= 0.5
        out[..., ch] = acc / norm
    rgb = np.clip(out * 255.0, 0, 255).astype(np.uint8)
    stars = hash_u01(seed, 99, np.arange(height)[:, None], np.arange(width)[None, :]) < 0.002
    rgb[stars] = 255
    return Texture(rgb, capi.TEXEL_RGB8)


# ---------------------------------------------------------------------------
# synthetic workloads (geometric units, M = 1 unless stated)
def aimed_camera(width: int, height: int, fov: float, radius: float, inclination: float,
                 azimuth: float = 0.0, center=(0.0, 0.0, 0.0)) -> Camera:
    """Camera at `radius` from `center`, `inclination` from the +z disc
    normal, looking at the centre: RotateZ(-azimuth), RotateY(incl - pi/2),
    MoveTo(position) on the reference's Camera."""
    cam = Camera(width, height, fov)
    cam.RotateZ(-azimuth)
    cam.RotateY(inclination - math.pi / 2)
    s, c = math.sin(inclination), math.cos(inclination)
    pos = np.asarray(center, dtype=np.float64) + radius * np.array(
        [-s * math.cos(azimuth), -s * math.sin(azimuth), c])
    cam.MoveTo(*pos)
    return cam


def equatorial_disc(r_inner: float, r_outer: float, texture: Texture,
                    mapping: int = capi.DISC_MAP_POLAR) -> Annulus:
    """Annulus in the z = 0 plane centred on the origin; the quad is the
    disc's bounding square (as in the reference's main(), which spans
    +-r_outer)."""
    R = r_outer
    d = Annulus((R, R, 0.0), (-R, R, 0.0), (-R, -R, 0.0), (R, -R, 0.0), r_outer, r_inner)
    d.SetTexture(texture)
    d.mapping = mapping
    return d


_TEXTURE_CACHE: dict = {}


def _cached(key, fn):
    if key not in _TEXTURE_CACHE:
        _TEXTURE_CACHE[key] = fn()
    return _TEXTURE_CACHE[key]


def standard_textures(seed: int = 0):
    """The single-scene disc (1024x64 RGBA8) and background (2048x1024 RGB8)."""
    disc = _cached(("disc", seed, 1024, 64), lambda: disc_ring_texture(seed, 1024, 64))
    bg = _cached(("bg", seed, 2048, 1024), lambda: value_noise_background(seed + 1, 2048, 1024))
    return disc, bg


def single_scene(width: int = 640, height: int = 360, seed: int = 0) -> Scene:
    """Plain single-scene render: M = 1, camera at r = 20 M, 80 degrees from
    the disc normal, FoV 60 degrees; disc 6 M - 20 M; value-noise sky."""
    disc_tex, bg = standard_textures(seed)
    cam = aimed_camera(width, height, math.radians(60), 20.0, math.radians(80))
    return Scene(cam, StaticBlackhole((0.0, 0.0, 0.0), 1.0), equatorial_disc(6.0, 20.0, disc_tex), bg,
                 {"workload": f"single {width}x{height}"})


def binary_scene(width: int = 640, height: int = 360, seed: int = 0, separation: float = 6.0,
                 mass_ratio: float = 1.0, inclination_deg: float = 80.0, radius: float = 30.0) -> Scene:
    """Two holes for the MULTI integrator (isotropic coordinates): total mass
    1 split m1 : m2 = 1 : mass_ratio, on the y axis `separation` apart about
    their centre of mass at the origin; a circumbinary disc from
    1.4 separation to 20 in the z = 0 plane (polar map); the camera at
    `radius` from the origin, `inclination_deg` from the disc normal, in the
    x-z plane (an equal-mass scene is mirror symmetric in y)."""
    disc_tex, bg = standard_textures(seed)
    m1 = 1.0 / (1.0 + mass_ratio)
    m2 = 1.0 - m1
    h1 = StaticBlackhole((0.0, -separation * m2, 0.0), m1)
    h2 = StaticBlackhole((0.0, separation * m1, 0.0), m2)
    cam = aimed_camera(width, height, math.radians(60), radius, math.radians(inclination_deg))
    return Scene(cam, h1, equatorial_disc(1.4 * separation, 20.0, disc_tex), bg,
                 {"workload": f"binary {width}x{height}"}, extra_holes=[h2])


def binary_orbit(frames: int = 8, width: int = 1920, height: int = 1080, seed: int = 0,
                 separation: float = 6.0) -> list[Scene]:
    """The equal-mass binary_scene at `frames` phases of one orbit: the holes
    turned about the disc normal by 2 pi k / frames."""
    out = []
    for k in range(frames):
        sc = binary_scene(width, height, seed, separation)
        a = 2 * math.pi * k / frames
        c, s = math.cos(a), math.sin(a)
        for h in [sc.hole] + sc.extra_holes:
            x, y, z = h.position()
            h.MoveTo(c * x - s * y, s * x + c * y, z)
        sc.meta = {"workload": f"binary orbit {width}x{height}", "frame": k}
        out.append(sc)
    return out


def panel_texture(seed: int, width: int = 160, height: int = 120) -> Texture:
    """A hash-noise BGR8 picture for a Rectangle (no black texels)."""
    def make():
        t = value_noise_background(seed, width, height, octaves=2, base_cells=8).bgra()[..., :3].copy()
        t[t.sum(-1) == 0] = 1
        return Texture(t, capi.TEXEL_BGR8)
    return _cached(("panel", seed, width, height), make)


def flat_demo_scene(width: int = 800, height: int = 450, seed: int = 0) -> Scene:
    """The reference's flat RayTracer scene (ray_tracer_test.cc:50-98):
    Camera(W, H, pi/2) moved to (-400, 120, 100), RotateY(-pi/24),
    RotateZ(pi/12); three textured Rectangles (hash pictures stand in for
    the photos) and an InfinitePlane through the origin with
    ChessPattern2D{10}. The hole takes no part in the FLAT integrator."""
    cam = Camera(width, height, math.pi / 2)
    cam.MoveTo(-400, 120, 100)
    cam.RotateY(-math.pi / 24)
    cam.RotateZ(math.pi / 12)
    rects = [
        ((100, 120, 100), (100, 0, 100), (100, 0, 0), (100, 120, 0)),
        ((100, 0, 150), (100, -100, 150), (100, -100, 0), (100, 0, 0)),
        ((-100, 50, 100), (-100, -50, 100), (-100, -50, 0), (-100, 50, 0)),
    ]
    objects = []
    for k, corners in enumerate(rects):
        r = Rectangle(*corners)
        r.SetTexture(panel_texture(seed + 10 + k))
        objects.append(r)
    objects.append(InfinitePlane((0.0, 0.0, 0.0), ChessPattern2D(10)))
    return Scene(cam, StaticBlackhole((0.0, 0.0, 0.0), 1.0), None, None,
                 {"workload": f"flat demo {width}x{height}"}, objects)


def objects_scene(width: int = 640, height: int = 360, seed: int = 0) -> Scene:
    """The single-scene workload with ordinary objects inside the camera's
    radius: a chess plane 6 M below the disc (ChessPattern2D{2}), a textured
    panel standing behind the hole at x = 12 M and one beside it at
    y = -10 M. The disc takes the reference's planar map."""
    sc = single_scene(width, height, seed)
    sc.disc.mapping = capi.DISC_MAP_REF_PLANAR
    back = Rectangle((12, 8, 8), (12, -8, 8), (12, -8, -4), (12, 8, -4))
    back.SetTexture(panel_texture(seed + 20))
    side = Rectangle((-8, -10, 6), (8, -10, 6), (8, -10, -2), (-8, -10, -2))
    side.SetTexture(panel_texture(seed + 21))
    sc.objects = [InfinitePlane((0.0, 0.0, -6.0), ChessPattern2D(2)), back, side]
    sc.meta = {"workload": f"objects {width}x{height}"}
    return sc


def flythrough(frames: int = 120, width: int = 1920, height: int = 1080, seed: int = 0) -> list[Scene]:
    """Fly-through: camera on an inward spiral from r = 30 M to 8 M (one turn
    in azimuth), inclination swept 60 -> 89 degrees, FoV 60 degrees; the
    single-scene disc and sky."""
    disc_tex, bg = standard_textures(seed)
    hole = StaticBlackhole((0.0, 0.0, 0.0), 1.0)
    disc = equatorial_disc(6.0, 20.0, disc_tex)
    out = []
    for f in range(frames):
        t = f / max(1, frames - 1)
        r = 30.0 + (8.0 - 30.0) * t
        inc = math.radians(60.0 + 29.0 * t)
        az = 2 * math.pi * t
        cam = aimed_camera(width, height, math.radians(60), r, inc, az)
        out.append(Scene(cam, hole, disc, bg, {"frame": f}))
    return out


def batched_scenes(count: int = 256, seed: int = 7, min_side: int = 64, max_side: int = 1024,
                   bg_size=(512, 256)) -> list[Scene]:
    """Batched uneven scenes: square sides log-uniform in [min_side,
    max_side], M ~ U[0.5, 2], camera radius ~ U[6M, 50M], inclination
    ~ U[0, 90] deg, FoV ~ U[20, 90] deg, disc 6M .. U[12M, 30M]; disc and sky
    textures from a per-scene seed."""
    out = []
    for i in range(count):
        u = hash_u01(seed, i, np.arange(8))
        side = int(round(math.exp(math.log(min_side) + u[0] * (math.log(max_side) - math.log(min_side)))))
        M = 0.5 + 1.5 * u[1]
        r_cam = (6.0 + 44.0 * u[2]) * M
        inc = math.radians(90.0 * u[3])
        fov = math.radians(20.0 + 70.0 * u[4])
        r_out = (12.0 + 18.0 * u[5]) * M
        sseed = int(seed * 100003 + i)
        disc_tex = disc_ring_texture(sseed, 1024, 64)
        bg = value_noise_background(sseed + 1, bg_size[0], bg_size[1])
        cam = aimed_camera(side, side, fov, r_cam, inc, 2 * math.pi * u[6])
        out.append(Scene(cam, StaticBlackhole((0.0, 0.0, 0.0), M), equatorial_disc(6.0 * M, r_out, disc_tex),
                         bg, {"scene": i, "side": side}))
    return out


def photon_ring_scene(side: int = 4096, fov_deg: float = 0.5, radius: float = 20.0, seed: int = 0) -> Scene:
    """Near-critical stress: narrow FoV aimed at the photon ring. The camera
    at `radius` looks at the point of the ring on the image's centre row,
    so the image spans impact parameters around 3 sqrt(3) M."""
    disc_tex, bg = standard_textures(seed)
    b_c = 3.0 * math.sqrt(3.0)
    cam = aimed_camera(side, side, math.radians(fov_deg), radius, math.radians(80))
    # turn the view from the hole toward the critical impact parameter
    cam.RotateZ(math.asin(b_c / radius))
    return Scene(cam, StaticBlackhole((0.0, 0.0, 0.0), 1.0), equatorial_disc(6.0, 20.0, disc_tex), bg,
                 {"workload": f"photon ring {side}x{side}"})


def ref_impact_parameter(scene: Scene, xs, ys) -> np.ndarray:
    """b / M of the ray of pixels (xs, ys) under REF ray generation: the
    reference forms the ray direction e = F - pv from the camera focus F and
    the point pv = PixelVector(x, y) - hole (blackhole_solution_test.cc:
    167-170), and the orbit's impact parameter is b = |F x e| / |e| with F
    relative to the hole. Vectorised over the pixels, FP64."""
    cam, hole = scene.camera, scene.hole
    a = cam.width() / 2.0 - np.asarray(xs, dtype=np.float64)
    c = cam.height() / 2.0 - np.asarray(ys, dtype=np.float64)
    F = cam.position() - hole.center()
    E0 = cam.position() - cam.focus_vector()
    e = E0[None, :] + a.reshape(-1, 1) * cam.vector_y()[None, :] + c.reshape(-1, 1) * cam.vector_z()[None, :]
    fe = np.cross(F[None, :], e)
    b = np.sqrt((fe * fe).sum(1) / (e * e).sum(1)) / hole.mass()
    return b.reshape(np.shape(xs))


def impact_grid_scene(side: int = 4096, window: float = 1e-4, radius: float = 20.0, seed: int = 0) -> Scene:
    """Near-critical stress set: a side x side image whose rays have impact
    parameters spread uniformly over 3 sqrt(3) M +- window M, every pixel a
    different value. The camera at `radius` has a field of view of ~1e-5 rad
    aimed at the photon ring, so b changes linearly along the image rows; it
    is turned about its view axis by atan(1 / side) so that the rows also
    step b by 1/side of a column: b follows the pixel's raster index
    x * side + y. Same hole, disc and sky as the single scene."""
    b_c = 3.0 * math.sqrt(3.0)
    base = photon_ring_scene(side, 0.5, radius, seed)
    cam = base.camera
    mid = side / 2.0
    ends = np.array([0.0, side - 1.0])

    def b_at(xs, ys):
        return ref_impact_parameter(base, np.asarray(xs, dtype=np.float64), np.asarray(ys, dtype=np.float64))

    # narrow the field of view until a row spans 2 window (b is linear in the
    # column to ~1e-9 at these angles), then aim the centre at b_c
    for _ in range(3):
        lo, hi = b_at(ends, [mid, mid])
        want = 2.0 * window * (side - 1.0) / side
        cam.fov(2.0 * math.atan(math.tan(cam.fov() / 2.0) * want / abs(hi - lo)))
    for _ in range(4):
        bc0 = float(b_at([mid], [mid])[0])
        d = 1e-9
        cam.RotateZ(d)
        bc1 = float(b_at([mid], [mid])[0])
        cam.RotateZ((b_c - bc1) * d / (bc1 - bc0))
    cam.RotateX(math.atan(1.0 / side))
    base.meta = {"workload": f"impact-parameter grid {side}x{side}, b = 3 sqrt(3) M +- {window:g} M"}
    return base
