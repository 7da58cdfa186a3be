"""Seeded synthetic scenes in the flattened form the C-ABI takes.

A scene is what RenderToy's ``World`` holds once flattened (RenderToy
include/RenderToy/world.h:13-43): world-space triangle vertices in
``World::triangles`` order, per-vertex normals, the mesh of each triangle, each
mesh's material index and smooth flag, the material table
(``PrincipledBSDF``, include/RenderToy/material.h:14-30) and the sky / ground
emission.  The camera is a ``Camera`` (include/RenderToy/object.h:69-95): an
object-to-world matrix, focal length in mm and gate in inches.

Workloads (sizes and seeds fixed):

* ``cornell_box()`` — 555-unit Cornell box: 5 walls (10 triangles), a short
  and a tall rotated box (12 triangles each) and a 130 x 105 ceiling light
  quad (2 triangles): 36 triangles.  Pinhole camera, 40 degree vertical field
  of view.
* ``cornell_mixed()`` — the same room with a smooth-shaded icosphere and
  boxes of glass, metal, clearcoat, sheen and subsurface materials, so that
  every lobe of the principled BSDF is exercised.
* ``displaced_icosphere()`` — an icosphere subdivided 8 times (1,310,720
  triangles) displaced along its normal by seeded Perlin noise of amplitude
  0.05 r, inside the Cornell room; principled parameters drawn per object.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

MAT_FLOATS = 24  # material record: see include/rtx.h


@dataclasses.dataclass
class Scene:
    verts: np.ndarray        # (n, 9) float32: v0, v1, v2 world space
    norms: np.ndarray        # (n, 9) float32: per-vertex normals
    tri_mesh: np.ndarray     # (n,) int32
    mesh_mat: np.ndarray     # (m,) int32
    mesh_smooth: np.ndarray  # (m,) uint8
    mats: np.ndarray         # (k, 24) float32
    sky: np.ndarray          # (3,) float32
    ground: np.ndarray       # (3,) float32
    camera: np.ndarray       # (21,) float32
    name: str = ""

    @property
    def n_tris(self) -> int:
        return int(self.verts.shape[0])

    def emitters(self) -> np.ndarray:
        """World::PrepareDirectLightSampling order (RenderToy src/world.cpp:24-37):
        meshes in order, each emissive mesh's triangles in id order."""
        out = []
        order = np.argsort(self.tri_mesh, kind="stable")
        for m in range(len(self.mesh_mat)):
            em = self.mats[self.mesh_mat[m], 3:6]
            if np.any(np.abs(em) > np.float32(1e-7)):
                out.append(order[self.tri_mesh[order] == m])
        if not out:
            return np.zeros(0, np.int32)
        return np.concatenate(out).astype(np.int32)


def material(base_color=(1.0, 1.0, 1.0), emission=(0.0, 0.0, 0.0), roughness=0.5,
             metallic=0.0, anisotropic=0.0, subsurface=0.0, specular_tint=0.0,
             sheen=0.0, sheen_tint=0.5, clearcoat=0.0, clearcoat_roughness=0.03,
             spec_trans=0.0, ior=1.45, at_distance=1.0, extinction=(1.0, 1.0, 1.0)):
    """One 24-float material record; defaults are PrincipledBSDF's member
    initialisers (RenderToy include/RenderToy/material.h:16-30)."""
    m = np.zeros(MAT_FLOATS, np.float32)
    m[0:3] = base_color
    m[3:6] = emission
    m[6:18] = (roughness, metallic, anisotropic, subsurface, specular_tint, sheen,
               sheen_tint, clearcoat, clearcoat_roughness, spec_trans, ior, at_distance)
    m[18:21] = extinction
    return m


def camera(o2w, focal_mm, gate_in=(1.0, 1.0), near=0.1, far=1000.0):
    c = np.zeros(21, np.float32)
    c[:16] = np.asarray(o2w, np.float32).reshape(16)
    c[16] = focal_mm
    c[17:19] = gate_in
    c[19] = near
    c[20] = far
    return c


def fov_camera(eye, forward_sign_z=+1.0, vfov_deg=40.0, near=0.1, far=1000.0):
    """Pinhole camera at ``eye`` looking along world +z (camera -z) with +y up.
    Gate 1 x 1 inch, focal length chosen so that tan(vfov/2) = top."""
    ex, ey, ez = eye
    s = forward_sign_z
    o2w = [[-s, 0, 0, ex], [0, 1, 0, ey], [0, 0, -s, ez], [0, 0, 0, 1]]
    focal = 25.4 * 1.0 / 2.0 / math.tan(math.radians(vfov_deg) / 2.0)
    return camera(o2w, focal, (1.0, 1.0), near, far)


class _Builder:
    def __init__(self):
        self.tris = []     # list of (3,3) arrays
        self.norms = []
        self.tri_mesh = []
        self.mesh_mat = []
        self.mesh_smooth = []
        self.mats = []

    def add_material(self, m) -> int:
        self.mats.append(np.asarray(m, np.float32))
        return len(self.mats) - 1

    def add_mesh(self, tris, mat, smooth=False, norms=None):
        tris = np.asarray(tris, np.float64).reshape(-1, 3, 3)
        mid = len(self.mesh_mat)
        self.mesh_mat.append(mat)
        self.mesh_smooth.append(1 if smooth else 0)
        if norms is None:
            e1 = tris[:, 1] - tris[:, 0]
            e2 = tris[:, 2] - tris[:, 0]
            n = np.cross(e1, e2)
            n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
            norms = np.repeat(n[:, None, :], 3, axis=1)
        self.tris.append(tris)
        self.norms.append(np.asarray(norms, np.float32).reshape(-1, 3, 3))
        self.tri_mesh.append(np.full(len(tris), mid, np.int32))
        return mid

    def add_quad(self, a, b, c, d, mat):
        # two triangles (a, b, c) and (a, c, d)
        return self.add_mesh([[a, b, c], [a, c, d]], mat)

    def finish(self, cam, name, sky=(0, 0, 0), ground=(0, 0, 0)) -> Scene:
        # The room is modelled in the classic [0, 555]^3 coordinates and then
        # centred on the world origin, where RenderToy's own demo scenes sit:
        # its octree refits every node box starting from a box at the origin
        # (src/bvh.cpp:9-12, 197-228), so a room in the positive octant would
        # leave it nearly unable to cull.
        verts = np.concatenate(self.tris).reshape(-1, 9).astype(np.float64) - ROOM_CENTER
        cam = np.asarray(cam, np.float32).copy()
        cam[3] -= ROOM_CENTER
        cam[7] -= ROOM_CENTER
        cam[11] -= ROOM_CENTER
        # -0.0 -> +0.0, as the identity object-to-world transform of a Mesh does
        verts = (verts + np.float32(0.0)).astype(np.float32)
        return Scene(
            verts=np.ascontiguousarray(verts),
            norms=np.ascontiguousarray(np.concatenate(self.norms).reshape(-1, 9).astype(np.float32)),
            tri_mesh=np.concatenate(self.tri_mesh).astype(np.int32),
            mesh_mat=np.asarray(self.mesh_mat, np.int32),
            mesh_smooth=np.asarray(self.mesh_smooth, np.uint8),
            mats=np.ascontiguousarray(np.stack(self.mats).astype(np.float32)),
            sky=np.asarray(sky, np.float32), ground=np.asarray(ground, np.float32),
            camera=np.asarray(cam, np.float32), name=name)


def _box_tris(center, size, rot_y_deg):
    """12 triangles of an axis-aligned box rotated about +y.  Boxes standing on
    the floor are sunk 1 unit into it so that no face is coplanar with (and
    overlapping) another: overlapping coplanar faces make the closest hit a
    tie that RenderToy resolves by its traversal order."""
    cx, cy, cz = center
    sx, sy, sz = (s / 2.0 for s in size)
    a = math.radians(rot_y_deg)
    ca, sa = math.cos(a), math.sin(a)

    def p(x, y, z):
        return (cx + ca * x + sa * z, cy + y, cz - sa * x + ca * z)

    c = [p(-sx, -sy, -sz), p(sx, -sy, -sz), p(sx, -sy, sz), p(-sx, -sy, sz),
         p(-sx, sy, -sz), p(sx, sy, -sz), p(sx, sy, sz), p(-sx, sy, sz)]
    faces = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (3, 0, 4, 7)]
    tris = []
    for f in faces:
        tris.append([c[f[0]], c[f[1]], c[f[2]]])
        tris.append([c[f[0]], c[f[2]], c[f[3]]])
    return tris


RED = (0.63, 0.065, 0.05)
GREEN = (0.14, 0.45, 0.091)
WHITE = (0.725, 0.725, 0.725)
LIGHT_LE = (17.0, 12.0, 4.0)
CORNELL_EYE = (278.0, 273.0, -800.0)
ROOM_CENTER = 277.5  # subtracted from every coordinate (see _Builder.finish)


def _cornell_room(b: _Builder, white, red, green, light):
    L = 555.0
    b.add_quad((0, 0, 0), (L, 0, 0), (L, 0, L), (0, 0, L), white)          # floor
    b.add_quad((0, L, 0), (0, L, L), (L, L, L), (L, L, 0), white)          # ceiling
    b.add_quad((0, 0, L), (L, 0, L), (L, L, L), (0, L, L), white)          # back
    b.add_quad((L, 0, 0), (L, L, 0), (L, L, L), (L, 0, L), red)            # left (x = 555)
    b.add_quad((0, 0, 0), (0, 0, L), (0, L, L), (0, L, 0), green)          # right (x = 0)


def _cornell_light(b: _Builder, light):
    # 130 x 105 quad, 1 unit below the ceiling (not coplanar with it)
    y = 554.0
    x0, x1, z0, z1 = 213.0, 343.0, 227.0, 332.0
    b.add_quad((x0, y, z0), (x1, y, z0), (x1, y, z1), (x0, y, z1), light)


def cornell_box() -> Scene:
    """The 36-triangle Cornell box (34 room/box triangles + 2 light triangles)."""
    b = _Builder()
    white = b.add_material(material(WHITE, roughness=1.0, metallic=0.0))
    red = b.add_material(material(RED, roughness=1.0, metallic=0.0))
    green = b.add_material(material(GREEN, roughness=1.0, metallic=0.0))
    light = b.add_material(material((0.78, 0.78, 0.78), emission=LIGHT_LE, roughness=1.0))
    _cornell_room(b, white, red, green, light)
    b.add_mesh(_box_tris((185.5, 81.5, 169.0), (165.0, 165.0, 165.0), -18.0), white)
    b.add_mesh(_box_tris((368.5, 164.0, 351.5), (165.0, 330.0, 165.0), 15.0), white)
    _cornell_light(b, light)
    cam = fov_camera(CORNELL_EYE, vfov_deg=40.0, near=700.0, far=1500.0)
    return b.finish(cam, "cornell_box")


def icosphere(subdiv: int):
    """Unit icosphere: (V, 3) float64 vertices and (F, 3) int64 faces."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(v) + 1) + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a = uk // (len(v) + 1)
        c = uk % (len(v) + 1)
        mid = v[a] + v[c]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def perlin3(p: np.ndarray, seed: int) -> np.ndarray:
    """Improved gradient noise (Perlin, SIGGRAPH 2002) with a seeded permutation;
    returns values in about [-1, 1] for points p (N, 3)."""
    rng = np.random.RandomState(seed)
    perm = rng.permutation(256).astype(np.int64)
    perm = np.concatenate([perm, perm])
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    pi &= 255
    u = pf * pf * pf * (pf * (pf * 6 - 15) + 10)

    def grad(h, x, y, z):
        h = h & 15
        a = np.where(h < 8, x, y)
        b = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
        return np.where(h & 1, -a, a) + np.where(h & 2, -b, b)

    X, Y, Z = pi[:, 0], pi[:, 1], pi[:, 2]
    x, y, z = pf[:, 0], pf[:, 1], pf[:, 2]
    A = perm[X] + Y
    AA = perm[A] + Z
    AB = perm[A + 1] + Z
    B = perm[X + 1] + Y
    BA = perm[B] + Z
    BB = perm[B + 1] + Z

    def lerp(t, a, b):
        return a + t * (b - a)

    return lerp(u[:, 2],
                lerp(u[:, 1], lerp(u[:, 0], grad(perm[AA], x, y, z), grad(perm[BA], x - 1, y, z)),
                     lerp(u[:, 0], grad(perm[AB], x, y - 1, z), grad(perm[BB], x - 1, y - 1, z))),
                lerp(u[:, 1], lerp(u[:, 0], grad(perm[AA + 1], x, y, z - 1), grad(perm[BA + 1], x - 1, y, z - 1)),
                     lerp(u[:, 0], grad(perm[AB + 1], x, y - 1, z - 1), grad(perm[BB + 1], x - 1, y - 1, z - 1))))


def _vertex_normals(v, f):
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    vn = np.zeros_like(v)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    return vn


def specular_to_ior(s: float) -> float:
    """Disney 'specular' in [0, 1] -> index of refraction through F0 = 0.08 s
    (PrincipledBSDF has no specular parameter; this mapping is an extension),
    clamped to [1.05, 2.0]."""
    f0 = 0.08 * s
    r = math.sqrt(max(f0, 1e-8))
    return float(min(max((1.0 + r) / (1.0 - r), 1.05), 2.0))


def random_principled(rng: np.random.RandomState) -> np.ndarray:
    """Principled parameters drawn uniformly: base colour [0,1]^3, metallic,
    roughness [0.05, 1], specular, clearcoat, sheen in [0, 1]."""
    return material(base_color=tuple(rng.uniform(0, 1, 3)), metallic=rng.uniform(0, 1),
                    roughness=rng.uniform(0.05, 1.0), ior=specular_to_ior(rng.uniform(0, 1)),
                    clearcoat=rng.uniform(0, 1), sheen=rng.uniform(0, 1),
                    clearcoat_roughness=0.03)


def displaced_icosphere(subdiv: int = 8, radius: float = 150.0, seed: int = 1,
                        center=(278.0, 165.0, 278.0)) -> Scene:
    """Icosphere (20 * 4**subdiv triangles) displaced by 0.05 r * Perlin noise
    along the normal, smooth shaded, in the Cornell room with its light."""
    b = _Builder()
    white = b.add_material(material(WHITE, roughness=1.0))
    red = b.add_material(material(RED, roughness=1.0))
    green = b.add_material(material(GREEN, roughness=1.0))
    light = b.add_material(material((0.78, 0.78, 0.78), emission=LIGHT_LE, roughness=1.0))
    _cornell_room(b, white, red, green, light)
    rng = np.random.RandomState(seed)
    sphere_mat = b.add_material(random_principled(rng))
    v, f = icosphere(subdiv)
    n0 = v.copy()
    disp = 0.05 * radius * perlin3(v * 4.0 + 17.0, seed)
    v = v * radius + n0 * disp[:, None] + np.asarray(center)
    vn = _vertex_normals(v, f)
    tris = v[f].astype(np.float32)
    norms = vn[f].astype(np.float32)
    b.add_mesh(tris, sphere_mat, smooth=True, norms=norms)
    _cornell_light(b, light)
    cam = fov_camera(CORNELL_EYE, vfov_deg=40.0, near=700.0, far=1500.0)
    return b.finish(cam, f"displaced_icosphere_s{subdiv}")


def cornell_mixed() -> Scene:
    """Cornell room with materials covering every BSDF lobe: a smooth glass
    icosphere, a metal box, a clearcoat + sheen box and a subsurface sphere."""
    b = _Builder()
    white = b.add_material(material(WHITE, roughness=1.0))
    red = b.add_material(material(RED, roughness=0.7, sheen=0.5, sheen_tint=0.3))
    green = b.add_material(material(GREEN, roughness=0.3, specular_tint=0.6))
    light = b.add_material(material((0.78, 0.78, 0.78), emission=LIGHT_LE, roughness=1.0))
    glass = b.add_material(material((0.95, 0.95, 0.95), roughness=0.05, spec_trans=1.0, ior=1.33))
    rough_glass = b.add_material(material((0.9, 0.8, 0.7), roughness=0.4, spec_trans=0.8, ior=1.5,
                                          metallic=0.1))
    metal = b.add_material(material((0.9, 0.9, 0.9), roughness=0.05, metallic=1.0, anisotropic=1.0))
    coat = b.add_material(material((0.2, 0.4, 0.8), roughness=0.5, clearcoat=1.0,
                                   clearcoat_roughness=0.1, sheen=1.0, sheen_tint=0.5))
    sss = b.add_material(material((0.8, 0.6, 0.5), roughness=0.6, subsurface=1.0,
                                  clearcoat=0.3, clearcoat_roughness=1.0))
    _cornell_room(b, white, red, green, light)
    b.add_mesh(_box_tris((185.5, 81.5, 169.0), (165.0, 165.0, 165.0), -18.0), metal)
    b.add_mesh(_box_tris((368.5, 164.0, 351.5), (165.0, 330.0, 165.0), 15.0), coat)
    v, f = icosphere(2)
    vn = v.copy()
    tris = (v * 70.0 + np.array([200.0, 240.0, 160.0]))[f].astype(np.float32)
    b.add_mesh(tris, glass, smooth=True, norms=vn[f].astype(np.float32))
    v2, f2 = icosphere(1)
    tris2 = (v2 * 60.0 + np.array([420.0, 390.0, 250.0]))[f2].astype(np.float32)
    b.add_mesh(tris2, sss, smooth=True, norms=v2[f2].astype(np.float32))
    b.add_mesh(_box_tris((120.0, 39.0, 420.0), (80.0, 80.0, 80.0), 30.0), rough_glass)
    _cornell_light(b, light)
    cam = fov_camera(CORNELL_EYE, vfov_deg=40.0, near=700.0, far=1500.0)
    return b.finish(cam, "cornell_mixed")


# ---------------------------------------------------------------------------
# Procedural scenes (batched-scene and denoiser-training workloads)
# ---------------------------------------------------------------------------

# Material texture slots (floats 21..23 of the record, padding in RenderToy's
# PrincipledBSDF): [21] kind, [22] the texture's own parameter, [23] texture
# units per world unit.  The texture is sampled at the hit point's two world
# coordinates across the shading normal's dominant axis, times [23], and
# scales base_color by 0.25 + 0.75 s.  RenderToy's textures (src/procedural.cpp)
# only rasterise to an image: this binding is an extension.
TEX_NONE, TEX_CHECKER, TEX_WAVE, TEX_PERLIN = 0, 1, 2, 3


def blackbody_rgb(t_kelvin: float) -> np.ndarray:
    """Convert::BlackBody (RenderToy src/rtmath.cpp:34-56): Krystek's
    approximation of the Planckian locus in CIE 1960 UCS, to xyY (Y = 1), XYZ
    and linear sRGB (Lindbloom's D65 matrix), normalised by the largest
    channel.  Evaluated in float64 (scene construction only)."""
    t = float(t_kelvin)
    tt = t * t
    u = (0.860117757 + 1.54118254e-4 * t + 1.28641212e-7 * tt) / (1.0 + 8.42420235e-4 * t + 7.08145163e-7 * tt)
    v = (0.317398726 + 4.22806245e-5 * t + 4.20481691e-8 * tt) / (1.0 - 2.89741816e-5 * t + 1.61456053e-7 * tt)
    d = 2.0 * u - 8.0 * v + 4.0
    x, y = 3.0 * u / d, 2.0 * v / d
    xyz = np.array([x / y, 1.0, (1.0 - x - y) / y])
    m = np.array([[3.2404542, -1.5371385, -0.4985314],
                  [-0.9692660, 1.8760108, 0.0415560],
                  [0.0556434, -0.2040259, 1.0572252]])
    rgb = m @ xyz
    return rgb / rgb.max()


def _grid_tris(n: int, size: float, amp: float, seed: int, center, rot_y_deg: float):
    """A displaced n x n grid (2 n^2 triangles) of side `size`, heights
    amp * perlin, lying on y = center.y, rotated about +y."""
    g = np.linspace(-size / 2, size / 2, n + 1)
    X, Z = np.meshgrid(g, g, indexing="ij")
    pts = np.stack([X.ravel() / size * 6.0, Z.ravel() / size * 6.0, np.full(X.size, 0.5)], 1)
    Y = amp * perlin3(pts, seed).reshape(X.shape)
    a = math.radians(rot_y_deg)
    ca, sa = math.cos(a), math.sin(a)
    P = np.stack([center[0] + ca * X + sa * Z, center[1] + Y, center[2] - sa * X + ca * Z], -1)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    i, j = i.ravel(), j.ravel()
    p00, p10, p01, p11 = P[i, j], P[i + 1, j], P[i, j + 1], P[i + 1, j + 1]
    t1 = np.stack([p00, p01, p11], 1)
    t2 = np.stack([p00, p11, p10], 1)
    return np.stack([t1, t2], 1).reshape(-1, 3, 3)


def _sphere_tris(subdiv: int, radius: float, center, amp: float = 0.0, seed: int = 0):
    v, f = icosphere(subdiv)
    if amp:
        v = v * (1.0 + amp * perlin3(v * 3.0, seed))[:, None]
    v = v * radius + np.asarray(center, np.float64)
    vn = _vertex_normals(v, f)
    return v[f], vn[f]


def procedural_scene(seed: int, n_tris=None, textures: bool = True, tri_range=(1e3, 2e6)):
    """One seeded procedural scene and its render job.

    Geometry: a 555-unit room (5 walls) holding 2-8 objects (boxes, smooth
    icospheres, Perlin-displaced grids) whose sizes share a triangle budget
    drawn log-uniformly from `tri_range` (or `n_tris`).  Materials: principled
    parameters drawn as ``random_principled``, each object with a checkerboard,
    wave or Perlin texture (or none) when `textures`.  Lights: 1-4 ceiling
    quads with blackbody emission, 2500-9000 K.  Job: resolution drawn from
    256^2, 512^2, 1280x720, 1920x1080 and spp uniform in [1, 64].
    Returns (Scene, {"W", "H", "spp", "n_lights", "target_tris"})."""
    rng = np.random.RandomState(1_000_003 + seed)
    draw = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
    target = int(n_tris if n_tris is not None else round(draw))
    b = _Builder()

    def tex(m):
        if textures:
            kind = rng.randint(0, 4)
            m[21] = kind
            m[22] = (rng.randint(2, 9) if kind == TEX_CHECKER else
                     rng.uniform(1.0, 6.0) if kind == TEX_WAVE else 10.0 if kind == TEX_PERLIN else 0.0)
            m[23] = rng.uniform(1.0 / 400.0, 1.0 / 100.0) if kind else 0.0
        return m

    walls = [b.add_material(tex(material(tuple(rng.uniform(0.3, 0.85, 3)), roughness=rng.uniform(0.5, 1.0))))
             for _ in range(3)]
    _cornell_room(b, walls[0], walls[1], walls[2], None)
    budget = max(target - 10, 12)
    n_obj = int(rng.randint(2, 9))
    kinds = rng.choice(["box", "sphere", "grid"], size=n_obj, p=[0.3, 0.4, 0.3])
    if not (kinds != "box").any():
        kinds[0] = "sphere"
    shares = rng.dirichlet(np.ones(int((kinds != "box").sum())))
    si = 0
    for k in kinds:
        mat = b.add_material(tex(random_principled(rng)))
        cx, cz = rng.uniform(110, 445), rng.uniform(140, 440)
        if k == "box":
            sx, sy, sz = rng.uniform(50, 160, 3)
            b.add_mesh(_box_tris((cx, sy / 2 - 1.0, cz), (sx, sy, sz), rng.uniform(-45, 45)), mat)
            continue
        share = budget * shares[si]
        si += 1
        if k == "sphere":
            s = int(np.clip(round(math.log(max(share, 80) / 20.0, 4)), 1, 8))
            r = rng.uniform(40, 110)
            tris, nrm = _sphere_tris(s, r, (cx, r + rng.uniform(-10, 60), cz), amp=rng.uniform(0, 0.08),
                                     seed=int(rng.randint(1 << 30)))
            b.add_mesh(tris, mat, smooth=True, norms=nrm)
        else:
            n = max(2, int(round(math.sqrt(max(share, 8) / 2.0))))
            size = rng.uniform(150, 400)
            tris = _grid_tris(n, size, rng.uniform(5, 60), int(rng.randint(1 << 30)),
                              (cx, rng.uniform(20, 200), cz), rng.uniform(0, 90))
            b.add_mesh(tris, mat)
    n_lights = int(rng.randint(1, 5))
    for _ in range(n_lights):
        w, d = rng.uniform(60, 160, 2)
        x0, z0 = rng.uniform(20, 535 - w), rng.uniform(20, 535 - d)
        power = 17.0 * 130 * 105 / (w * d) / n_lights * rng.uniform(0.7, 1.4)
        le = blackbody_rgb(rng.uniform(2500, 9000)) * power
        light = b.add_material(material((0.78, 0.78, 0.78), emission=tuple(le), roughness=1.0))
        y = 554.0  # 1 unit below the ceiling, as the Cornell light
        b.add_quad((x0, y, z0), (x0 + w, y, z0), (x0 + w, y, z0 + d), (x0, y, z0 + d), light)
    eye = (278.0 + rng.uniform(-60, 60), 273.0 + rng.uniform(-60, 60), -800.0 + rng.uniform(-100, 100))
    cam = fov_camera(eye, vfov_deg=rng.uniform(35, 50), near=700.0, far=1500.0)
    W, H = [(256, 256), (512, 512), (1280, 720), (1920, 1080)][rng.randint(4)]
    spp = int(rng.randint(1, 65))
    scene = b.finish(cam, f"procedural_{seed}")
    return scene, {"W": W, "H": H, "spp": spp, "n_lights": n_lights, "target_tris": target}
