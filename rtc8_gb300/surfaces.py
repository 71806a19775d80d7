"""Triangle-mesh surfaces of a scene (the reference's surface path without OptiX).

A scene is a list of materials, a list of meshes (geometry instances: object-space vertices
with shading normal and tangent, triangles, one material each) and a list of instances, each
placing a contiguous range of meshes (a geometry group) with a 3x4 transform, as the
reference's scene loader builds them (renderer/renderer_scene.h, renderer_scene.cpp:1286-1620).
Materials carry the immediate values of the reference's 1x1 textures (see include/rtc8_vpt.h,
VptSurfaceMaterial).

The builders below make procedural stand-ins for the reference's loaded meshes: the reference
ships no mesh assets, so scenes are boxes and rectangles (`rectangle` follows the reference's
`rect` command, renderer_scene.cpp:1554-1618).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SIMPLE_PBR = 0
LAMBERT = 1


@dataclass
class Material:
    kind: int = SIMPLE_PBR
    base_color: tuple = (0.8, 0.8, 0.8)
    roughness: float = 0.5
    metallic: float = 0.0
    emittance: tuple = (0.0, 0.0, 0.0)


@dataclass
class Mesh:
    vertices: np.ndarray   # (n, 9) float32: position, shading normal, tangent
    triangles: np.ndarray  # (m, 3) uint32
    material: int = 0


@dataclass
class Instance:
    first_geometry: int
    num_geometries: int = 1
    transform: np.ndarray = field(default_factory=lambda: np.eye(3, 4, dtype=np.float32))
    uniform_scale: float = 1.0


@dataclass
class SurfaceScene:
    materials: list
    meshes: list
    instances: list

    def add(self, mesh: Mesh, transform=None, uniform_scale: float = 1.0) -> int:
        """Adds a mesh in an instance of its own; returns the instance index."""
        self.meshes.append(mesh)
        t = np.eye(3, 4, dtype=np.float32) if transform is None else np.asarray(transform, dtype=np.float32)
        self.instances.append(Instance(len(self.meshes) - 1, 1, t, uniform_scale))
        return len(self.instances) - 1

    @property
    def num_triangles(self) -> int:
        return sum(len(self.meshes[i.first_geometry + k].triangles) for i in self.instances for k in range(i.num_geometries))


def translation(x: float, y: float, z: float, scale: float = 1.0) -> np.ndarray:
    """Row-major 3x4 transform: uniform scale, then translation."""
    t = np.zeros((3, 4), dtype=np.float32)
    t[0, 0] = t[1, 1] = t[2, 2] = scale
    t[:, 3] = (x, y, z)
    return t


def rotation_y(deg: float, x: float = 0.0, y: float = 0.0, z: float = 0.0) -> np.ndarray:
    c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    t = np.zeros((3, 4), dtype=np.float32)
    t[:, :3] = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], dtype=np.float32)
    t[:, 3] = (x, y, z)
    return t


def _quad(corners, normal, tangent) -> tuple[np.ndarray, np.ndarray]:
    v = np.zeros((4, 9), dtype=np.float32)
    v[:, 0:3] = corners
    v[:, 3:6] = normal
    v[:, 6:9] = tangent
    return v, np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32)


def rectangle(width: float, depth: float, material: int) -> Mesh:
    """The reference's rectangle: in the y = 0 plane, shading normal -y, tangent +x, facing down
    (renderer_scene.cpp:1580-1589)."""
    hw, hd = 0.5 * width, 0.5 * depth
    v, t = _quad([(-hw, 0, -hd), (hw, 0, -hd), (hw, 0, hd), (-hw, 0, hd)], (0, -1, 0), (1, 0, 0))
    return Mesh(v, t, material)


def box(size, material: int, inward: bool = False, skip=()) -> Mesh:
    """An axis-aligned box of half-extents `size` centred at the origin, one quad per face
    (faces named -x, +x, -y, +y, -z, +z; `skip` leaves faces out). Normals point out, or in
    for a room (`inward`)."""
    hx, hy, hz = size
    faces = {
        "-x": ([(-hx, -hy, -hz), (-hx, -hy, hz), (-hx, hy, hz), (-hx, hy, -hz)], (-1, 0, 0), (0, 0, 1)),
        "+x": ([(hx, -hy, -hz), (hx, hy, -hz), (hx, hy, hz), (hx, -hy, hz)], (1, 0, 0), (0, 1, 0)),
        "-y": ([(-hx, -hy, -hz), (hx, -hy, -hz), (hx, -hy, hz), (-hx, -hy, hz)], (0, -1, 0), (1, 0, 0)),
        "+y": ([(-hx, hy, -hz), (-hx, hy, hz), (hx, hy, hz), (hx, hy, -hz)], (0, 1, 0), (0, 0, 1)),
        "-z": ([(-hx, -hy, -hz), (-hx, hy, -hz), (hx, hy, -hz), (hx, -hy, -hz)], (0, 0, -1), (0, 1, 0)),
        "+z": ([(-hx, -hy, hz), (hx, -hy, hz), (hx, hy, hz), (-hx, hy, hz)], (0, 0, 1), (1, 0, 0)),
    }
    verts, tris = [], []
    for name, (corners, n, t) in faces.items():
        if name in skip:
            continue
        if inward:
            corners = corners[::-1]
            n = tuple(-c for c in n)
        v, tr = _quad(corners, n, t)
        tris.append(tr + 4 * len(verts))
        verts.append(v)
    return Mesh(np.concatenate(verts), np.concatenate(tris).astype(np.uint32), material)


def room_scene(light_emittance: float = 40.0, light_size: float = 0.5) -> SurfaceScene:
    """A room around the unit volume box [-0.5, 0.5]^3: grey floor and ceiling, a grey back wall,
    a red left wall and a green right wall (Lambert; the front stays open to the environment),
    a glossy SimplePBR block and a metallic one on the floor, and a rectangle light under the
    ceiling (SimplePBR with an emittance, as the reference's `rect` + `emittance` commands)."""
    mats = [
        Material(LAMBERT, (0.75, 0.75, 0.75)),                       # 0 white walls
        Material(LAMBERT, (0.75, 0.15, 0.12)),                       # 1 red
        Material(LAMBERT, (0.15, 0.65, 0.18)),                       # 2 green
        Material(SIMPLE_PBR, (0.9, 0.9, 0.9), 1.0, 0.0, (light_emittance,) * 3),  # 3 light
        Material(SIMPLE_PBR, (0.55, 0.6, 0.8), 0.3, 0.0),            # 4 glossy dielectric
        Material(SIMPLE_PBR, (0.95, 0.75, 0.45), 0.2, 1.0),          # 5 metal
    ]
    sc = SurfaceScene(mats, [], [])
    h = 0.9
    sc.add(box((h, 0.75, h), 0, inward=True, skip=("-x", "+x", "+z")), translation(0, 0.15, 0))
    left = box((h, 0.75, h), 1, inward=True, skip=("+x", "-y", "+y", "-z", "+z"))
    right = box((h, 0.75, h), 2, inward=True, skip=("-x", "-y", "+y", "-z", "+z"))
    sc.add(left, translation(0, 0.15, 0))
    sc.add(right, translation(0, 0.15, 0))
    sc.add(rectangle(light_size, light_size, 3), translation(0, 0.88, 0))
    sc.add(box((0.17, 0.25, 0.17), 4), rotation_y(20.0, -0.42, -0.35, -0.35))
    sc.add(box((0.14, 0.14, 0.14), 5), rotation_y(-30.0, 0.45, -0.46, 0.3))
    return sc


def sphere(radius: float, material: int, segments: int = 16, rings: int = 8) -> Mesh:
    """A UV sphere centred at the origin (y up): `rings` bands of `segments` quads, triangles at the
    poles, smooth shading normals, tangents along the azimuth, every triangle wound so that its
    geometric normal points outwards."""
    verts = []
    for r in range(rings + 1):
        th = math.pi * r / rings
        for s in range(segments + 1):
            ph = 2 * math.pi * s / segments
            n = (math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph))
            verts.append((*[radius * c for c in n], *n, -math.sin(ph), 0.0, math.cos(ph)))
    v = np.array(verts, dtype=np.float32)

    def idx(r, s):
        return r * (segments + 1) + s

    tris = []
    for r in range(rings):
        for s in range(segments):
            a, b, c, d = idx(r, s), idx(r + 1, s), idx(r + 1, s + 1), idx(r, s + 1)
            if r > 0:
                tris.append((a, b, d))
            if r < rings - 1:
                tris.append((b, c, d))
    t = np.array(tris, dtype=np.uint32)
    p = v[:, 0:3]
    gn = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    inward = np.einsum("ij,ij->i", gn, p[t].mean(axis=1)) < 0
    t[inward] = t[inward][:, ::-1]
    return Mesh(v, t, material)
