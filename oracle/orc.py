"""ctypes binding of the oracle library (test infrastructure only; see oracle/vpt_oracle.h)."""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import build as _build

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)


class OrcScene(C.Structure):
    _fields_ = [
        ("voxels", f32p), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("inv_voxel_size", C.c_float), ("origin", C.c_float * 3),
        ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3),
        ("global_majorant", C.c_float), ("cell_majorant", f32p),
        ("cx", C.c_int32), ("cy", C.c_int32), ("cz", C.c_int32),
        ("density_coeff", C.c_float), ("albedo", C.c_float),
        ("phase_kind", C.c_int32), ("phase_param", C.c_float),
        ("env_enabled", C.c_int32), ("env_rgb", f32p), ("env_w", C.c_int32), ("env_h", C.c_int32),
        ("env_power", C.c_float), ("env_rotation", C.c_float),
        ("imp_mips", f32p), ("imp_offsets", i64p), ("map_w", C.c_int32), ("map_h", C.c_int32),
        ("num_mips", C.c_int32), ("imp_integral", C.c_float),
        ("sun_enabled", C.c_int32), ("sun_dir", C.c_float * 3), ("sun_irradiance", C.c_float * 3),
        ("sun_prob", C.c_float),
        ("world_radius", C.c_float), ("world_min", C.c_float * 3), ("world_max", C.c_float * 3),
        ("cam_aspect", C.c_float), ("cam_fovy", C.c_float), ("cam_pos", C.c_float * 3), ("cam_quat", C.c_float * 4),
        ("width", C.c_int32), ("height", C.c_int32),
        ("max_bounces", C.c_int32), ("rr_start", C.c_int32), ("majorant_mode", C.c_int32), ("max_steps", C.c_int32),
        ("stream_mode", C.c_int32), ("maj_shift", C.c_int32), ("shadow_rr", C.c_float),
        ("surfaces", C.c_void_p), ("volume_disabled", C.c_int32),
    ]


class OrcSurfMaterial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("base_color", C.c_float * 3), ("roughness", C.c_float),
                ("metallic", C.c_float), ("emittance", C.c_float * 3)]


class OrcSurfGeometry(C.Structure):
    _fields_ = [("vertices", f32p), ("num_vertices", C.c_uint32), ("triangles", u32p), ("num_triangles", C.c_uint32),
                ("material", C.c_uint32)]


class OrcSurfInstance(C.Structure):
    _fields_ = [("first_geometry", C.c_uint32), ("num_geometries", C.c_uint32), ("transform", C.c_float * 12),
                ("uniform_scale", C.c_float)]


_FUNCS = {
    "orc_version": (C.c_int, []),
    "orc_seed_states": (None, [C.c_int32, C.c_int32, C.c_uint64, u64p]),
    "orc_pcg_floats": (None, [C.c_uint64, C.c_int32, f32p, u64p]),
    "orc_imp_map_size": (C.c_int64, [C.c_int32, C.c_int32, i32p, i32p, i32p, i64p]),
    "orc_build_imp_map": (C.c_float, [f32p, C.c_int32, C.c_int32, f32p]),
    "orc_majorants": (C.c_float, [f32p, C.c_int32, C.c_int32, C.c_int32, f32p]),
    "orc_sample_density": (None, [C.POINTER(OrcScene), f32p, C.c_int32, f32p]),
    "orc_srgb_gamma": (None, [f32p, C.c_int32, f32p]),
    "orc_tonemap": (None, [f32p, C.c_int32, C.c_float, C.c_int32, f32p, C.POINTER(C.c_uint8)]),
    "orc_clip_rays": (None, [C.POINTER(OrcScene), f32p, f32p, C.c_int32, f32p, f32p, i32p]),
    "orc_env_sample": (None, [C.POINTER(OrcScene), f32p, C.c_int32, f32p, f32p, f32p]),
    "orc_env_evaluate": (None, [C.POINTER(OrcScene), f32p, C.c_int32, f32p, f32p]),
    "orc_imp_sample": (None, [C.POINTER(OrcScene), f32p, C.c_int32, f32p]),
    "orc_surfaces_create": (C.c_void_p, [C.POINTER(OrcSurfMaterial), C.c_uint32, C.POINTER(OrcSurfGeometry),
                                         C.c_uint32, C.POINTER(OrcSurfInstance), C.c_uint32, f32p]),
    "orc_surfaces_destroy": (None, [C.c_void_p]),
    "orc_surface_closest": (None, [C.c_void_p, f32p, f32p, C.c_int32, C.c_float, i32p, f32p]),
    "orc_surface_any": (None, [C.c_void_p, f32p, f32p, f32p, C.c_int32, i32p]),
    "orc_bsdf_eval": (None, [C.POINTER(OrcSurfMaterial), f32p, f32p, C.c_int32, f32p, f32p]),
    "orc_bsdf_sample": (None, [C.POINTER(OrcSurfMaterial), f32p, f32p, C.c_int32, f32p]),
    "orc_offset_origin": (None, [f32p, C.c_int32, f32p]),
    "orc_phase_sample": (None, [C.c_int32, C.c_float, f32p, C.c_int32, f32p, f32p]),
    "orc_phase_eval": (None, [C.c_int32, C.c_float, f32p, C.c_int32, f32p]),
    "orc_polar_yup": (None, [f32p, C.c_int32, f32p]),
    "orc_coordinate_system": (None, [f32p, C.c_int32, f32p]),
    "orc_quat_to_matrix": (None, [f32p, f32p]),
    "orc_render_plain": (C.c_int64, [C.POINTER(OrcScene), u64p, C.c_int32, C.c_int32, f64p, f32p, u32p, C.c_int32,
                                     C.c_int32, C.c_int32]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        for name, (res, args) in _FUNCS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def seed_states(width: int, height: int, seed: int) -> np.ndarray:
    out = np.empty(width * height, dtype=np.uint64)
    lib().orc_seed_states(width, height, C.c_uint64(seed), p(out, C.c_uint64))
    return out


def pcg_floats(state: int, n: int) -> tuple[np.ndarray, int]:
    out = np.empty(n, dtype=np.float32)
    st = C.c_uint64()
    lib().orc_pcg_floats(C.c_uint64(state), n, p(out, C.c_float), C.byref(st))
    return out, st.value


def importance_map(env_rgb: np.ndarray) -> tuple[np.ndarray, np.ndarray, dict]:
    img = np.ascontiguousarray(env_rgb, dtype=np.float32)
    h, w, _ = img.shape
    mw, mh, nm = C.c_int32(), C.c_int32(), C.c_int32()
    offs = np.zeros(32, dtype=np.int64)
    total = lib().orc_imp_map_size(w, h, C.byref(mw), C.byref(mh), C.byref(nm), p(offs, C.c_int64))
    mips = np.zeros(total, dtype=np.float32)
    integral = lib().orc_build_imp_map(p(img, C.c_float), w, h, p(mips, C.c_float))
    return mips, offs, {"map_w": mw.value, "map_h": mh.value, "num_mips": nm.value, "integral": float(integral)}


def majorants(vox: np.ndarray) -> tuple[np.ndarray, float]:
    v = np.ascontiguousarray(vox, dtype=np.float32)
    nx, ny, nz = v.shape
    cells = np.zeros(((nx + 7) // 8, (ny + 7) // 8, (nz + 7) // 8), dtype=np.float32)
    g = lib().orc_majorants(p(v, C.c_float), nx, ny, nz, p(cells, C.c_float))
    return cells, float(g)


def srgb_gamma(v: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(v, dtype=np.float32)
    out = np.zeros_like(a)
    lib().orc_srgb_gamma(p(a, C.c_float), a.size, p(out, C.c_float))
    return out


def tonemap(mean_rgb: np.ndarray, brightness: float = 1.0, srgb: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """Tone-mapped float RGB and 8-bit RGBA of a mean image (..., 3)."""
    m = np.ascontiguousarray(mean_rgb, dtype=np.float32)
    n = m.size // 3
    out = np.zeros(m.shape, dtype=np.float32)
    rgba = np.zeros(m.shape[:-1] + (4,), dtype=np.uint8)
    lib().orc_tonemap(p(m, C.c_float), n, brightness, int(srgb), p(out, C.c_float), p(rgba, C.c_uint8))
    return out, rgba


def fbm_volume(spec) -> np.ndarray:
    """Dense fBm volume of a rtc8_gb300.configs.VolumeSpec built on the host (oracle/scene_oracle.cpp),
    bit-identical to the device generator."""
    L = lib()
    fn = L.orc_fbm_volume
    fn.restype = None
    fn.argtypes = [C.c_int32, C.c_uint32, C.c_int64, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float, f32p,
                   f32p]
    n = spec.n
    out = np.empty((n, n, n), dtype=np.float32)
    scratch = np.empty((n, n, n), dtype=np.float32) if spec.union_seed is not None else None
    fn(n, spec.seed & 0xFFFFFFFF, -1 if spec.union_seed is None else int(spec.union_seed), spec.octaves,
       spec.lacunarity, spec.gain, spec.base_frequency, spec.threshold, p(out, C.c_float),
       p(scratch, C.c_float) if scratch is not None else None)
    return out


def pool_cells(cells: np.ndarray, factor: int) -> np.ndarray:
    """Majorant cells of `factor`^3 times the volume (max-pooling, ragged edges included)."""
    cx, cy, cz = cells.shape
    mx, my, mz = (-(-cx // factor), -(-cy // factor), -(-cz // factor))
    pad = np.zeros((mx * factor, my * factor, mz * factor), dtype=np.float32)
    pad[:cx, :cy, :cz] = cells
    return pad.reshape(mx, factor, my, factor, mz, factor).max(axis=(1, 3, 5))


@dataclass
class OracleScene:
    """Keeps the arrays referenced by an OrcScene alive."""
    scene: OrcScene
    keep: list

    @property
    def ref(self):
        return C.byref(self.scene)


def make_scene(*, voxels: np.ndarray, voxel_size: float, origin, density_coeff: float, albedo: float,
               phase_kind: int, phase_param: float, env_rgb: np.ndarray | None, width: int, height: int,
               cam_aspect: float, cam_fovy: float, cam_pos, cam_quat, sun_dir=None, sun_irradiance=0.0,
               sun_prob=0.5, max_bounces=0, rr_start=1, majorant_mode=0, max_steps=0, stream_mode=0, maj_shift=3,
               env_power=1.0,
               env_rotation=0.0, cells: np.ndarray | None = None, global_majorant: float | None = None,
               shadow_rr: float = 0.0) -> OracleScene:
    s = OrcScene()
    v = np.ascontiguousarray(voxels, dtype=np.float32)
    keep = [v]
    s.voxels = p(v, C.c_float)
    s.nx, s.ny, s.nz = v.shape
    s.inv_voxel_size = float(np.float32(1.0 / float(voxel_size)))
    o = np.asarray(origin, dtype=np.float32)
    n = np.array(v.shape, dtype=np.float64)
    bmax = (o.astype(np.float64) + n * float(np.float32(voxel_size))).astype(np.float32)
    for a in range(3):
        s.origin[a] = float(o[a])
        s.bbox_min[a] = float(o[a])
        s.bbox_max[a] = float(bmax[a])
        s.world_min[a] = float(o[a])
        s.world_max[a] = float(bmax[a])
    center = (o + bmax) * np.float32(0.5)
    d = (bmax - center).astype(np.float32)
    s.world_radius = float(np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])))
    if cells is None or global_majorant is None:
        cells, global_majorant = majorants(v)
    if maj_shift > 3:
        cells = pool_cells(cells, 1 << (maj_shift - 3))
    s.maj_shift = max(maj_shift, 3)
    cells = np.ascontiguousarray(cells, dtype=np.float32)
    keep.append(cells)
    s.global_majorant = global_majorant
    s.cell_majorant = p(cells, C.c_float)
    s.cx, s.cy, s.cz = cells.shape
    s.density_coeff = density_coeff
    s.albedo = albedo
    s.phase_kind = phase_kind
    s.phase_param = phase_param
    if env_rgb is not None:
        img = np.ascontiguousarray(env_rgb, dtype=np.float32)
        mips, offs, info = importance_map(img)
        keep += [img, mips, offs]
        s.env_enabled = 1
        s.env_rgb = p(img, C.c_float)
        s.env_h, s.env_w = img.shape[:2]
        s.env_power = env_power
        s.env_rotation = env_rotation
        s.imp_mips = p(mips, C.c_float)
        s.imp_offsets = p(offs, C.c_int64)
        s.map_w, s.map_h, s.num_mips = info["map_w"], info["map_h"], info["num_mips"]
        s.imp_integral = info["integral"]
    if sun_dir is not None:
        s.sun_enabled = 1
        for a in range(3):
            s.sun_dir[a] = float(sun_dir[a])
            s.sun_irradiance[a] = float(sun_irradiance)
        s.sun_prob = sun_prob if env_rgb is not None else 1.0
    s.cam_aspect = cam_aspect
    s.cam_fovy = cam_fovy
    for a in range(3):
        s.cam_pos[a] = float(cam_pos[a])
    for a in range(4):
        s.cam_quat[a] = float(cam_quat[a])
    s.width, s.height = width, height
    s.max_bounces, s.rr_start, s.majorant_mode, s.max_steps = max_bounces, rr_start, majorant_mode, max_steps
    s.stream_mode = stream_mode
    s.shadow_rr = shadow_rr if 0.0 < shadow_rr < 1.0 else 0.0
    return OracleScene(s, keep)


def scene_from_config(cfg, voxels: np.ndarray, env_rgb: np.ndarray | None, **over) -> OracleScene:
    """OrcScene for a rtc8_gb300.configs.SceneConfig (same camera, lights and path rules)."""
    from rtc8_gb300.configs import camera_for, sun_direction, volume_box
    vs, origin = volume_box(cfg.volume)
    cam = camera_for(cfg)
    sun = None if cfg.sun_elevation_deg is None else sun_direction(cfg.sun_elevation_deg, cfg.sun_azimuth_deg)
    kw = dict(voxels=voxels, voxel_size=vs, origin=origin, density_coeff=cfg.volume.sigma_t_max, albedo=cfg.albedo,
              phase_kind=cfg.phase_kind, phase_param=cfg.phase_param, env_rgb=env_rgb, width=cfg.width,
              height=cfg.height, cam_aspect=cam.aspect, cam_fovy=cam.fovy,
              cam_pos=np.asarray(cam.position, dtype=np.float32), cam_quat=np.asarray(cam.orientation, np.float32),
              sun_dir=None if sun is None else sun.astype(np.float32), sun_irradiance=cfg.sun_irradiance,
              sun_prob=cfg.sun_select_prob, max_bounces=cfg.max_bounces, rr_start=cfg.rr_start_vertex,
              majorant_mode=cfg.majorant_mode, max_steps=cfg.max_steps_per_segment,
              stream_mode=cfg.rng_stream_mode, maj_shift=cfg.majorant_cell_log2,
              shadow_rr=cfg.shadow_rr_threshold)
    kw.update(over)
    return make_scene(**kw)


def _material(m) -> OrcSurfMaterial:
    o = OrcSurfMaterial()
    o.kind = m.kind
    o.base_color[:] = [float(x) for x in m.base_color]
    o.roughness, o.metallic = float(m.roughness), float(m.metallic)
    o.emittance[:] = [float(x) for x in m.emittance]
    return o


class OracleSurfaces:
    """The oracle's prepared copy of a rtc8_gb300.surfaces.SurfaceScene (freed on close)."""

    def __init__(self, scene):
        L = lib()
        mats = (OrcSurfMaterial * len(scene.materials))(*[_material(m) for m in scene.materials])
        self.keep = []
        geoms = (OrcSurfGeometry * len(scene.meshes))()
        for g, mesh in zip(geoms, scene.meshes):
            v = np.ascontiguousarray(mesh.vertices, dtype=np.float32)
            t = np.ascontiguousarray(mesh.triangles, dtype=np.uint32)
            self.keep += [v, t]
            g.vertices, g.num_vertices = p(v, C.c_float), len(v)
            g.triangles, g.num_triangles, g.material = p(t, C.c_uint32), len(t), mesh.material
        insts = (OrcSurfInstance * len(scene.instances))()
        for d, src in zip(insts, scene.instances):
            d.first_geometry, d.num_geometries = src.first_geometry, src.num_geometries
            d.transform[:] = [float(x) for x in np.asarray(src.transform, dtype=np.float32).reshape(12)]
            d.uniform_scale = float(src.uniform_scale)
        box = np.zeros(6, dtype=np.float32)
        self.handle = L.orc_surfaces_create(mats, len(mats), geoms, len(geoms), insts, len(insts), p(box, C.c_float))
        if not self.handle:
            raise ValueError("orc_surfaces_create rejected the scene")
        self.box = box

    def closest(self, org: np.ndarray, d: np.ndarray, tmax: float = 1e10):
        org = np.ascontiguousarray(org, dtype=np.float32)
        d = np.ascontiguousarray(d, dtype=np.float32)
        n = len(org)
        tri = np.zeros(n, dtype=np.int32)
        tb = np.zeros((n, 3), dtype=np.float32)
        lib().orc_surface_closest(self.handle, p(org, C.c_float), p(d, C.c_float), n, tmax, p(tri, C.c_int32),
                                  p(tb, C.c_float))
        return tri, tb

    def close(self):
        if self.handle:
            lib().orc_surfaces_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def attach_surfaces(sc: OracleScene, scene, volume_enabled: bool = True) -> OracleSurfaces:
    """Adds a surface scene to an oracle scene and widens its world box to the union of the
    volume's box (unless disabled) and the instances' boxes (compute_light_probs.cu:139-157)."""
    surf = OracleSurfaces(scene)
    s = sc.scene
    s.surfaces = surf.handle
    s.volume_disabled = 0 if volume_enabled else 1
    lo = surf.box[:3].copy()
    hi = surf.box[3:].copy()
    if volume_enabled:
        lo = np.minimum(lo, np.array(s.bbox_min[:], dtype=np.float32))
        hi = np.maximum(hi, np.array(s.bbox_max[:], dtype=np.float32))
    center = (lo + hi) * np.float32(0.5)
    d = (hi - center).astype(np.float32)
    r2 = np.float32(0)
    for a in range(3):
        r2 = np.float32(r2 + np.float32(d[a] * d[a]))
        s.world_min[a] = float(lo[a])
        s.world_max[a] = float(hi[a])
    s.world_radius = float(np.sqrt(r2))
    sc.keep.append(surf)
    return surf


def bsdf_eval(material, q: np.ndarray, v: np.ndarray):
    q = np.ascontiguousarray(q, dtype=np.float32)
    v = np.ascontiguousarray(v, dtype=np.float32)
    val = np.zeros((len(q), 3), dtype=np.float32)
    pdf = np.zeros(len(q), dtype=np.float32)
    lib().orc_bsdf_eval(C.byref(_material(material)), p(q, C.c_float), p(v, C.c_float), len(q), p(val, C.c_float),
                        p(pdf, C.c_float))
    return val, pdf


def bsdf_sample(material, q: np.ndarray, u: np.ndarray) -> np.ndarray:
    q = np.ascontiguousarray(q, dtype=np.float32)
    u = np.ascontiguousarray(u, dtype=np.float32)
    out = np.zeros((len(q), 7), dtype=np.float32)
    lib().orc_bsdf_sample(C.byref(_material(material)), p(q, C.c_float), p(u, C.c_float), len(q), p(out, C.c_float))
    return out


def offset_origin(pn: np.ndarray) -> np.ndarray:
    pn = np.ascontiguousarray(pn, dtype=np.float32)
    out = np.zeros((len(pn), 3), dtype=np.float32)
    lib().orc_offset_origin(p(pn, C.c_float), len(pn), p(out, C.c_float))
    return out


def render_plain(sc: OracleScene, rng: np.ndarray, spp: int, accum_base: int = 0, rows=None, threads: int = 0,
                 sum_rgb=None, mean_rgb=None, log: bool = False):
    s = sc.scene
    r0, r1 = (0, s.height) if rows is None else rows
    if sum_rgb is None:
        sum_rgb = np.zeros((s.height, s.width, 3), dtype=np.float64)
    if mean_rgb is None:
        mean_rgb = np.zeros((s.height, s.width, 3), dtype=np.float32)
    dlog = np.zeros((s.height * s.width, spp, 4), dtype=np.uint32) if log else None
    n = lib().orc_render_plain(sc.ref, p(rng, C.c_uint64), accum_base, spp, p(sum_rgb, C.c_double),
                               p(mean_rgb, C.c_float), p(dlog, C.c_uint32) if log else None, r0, r1, threads)
    return {"sum": sum_rgb, "mean": mean_rgb, "log": dlog, "lookups": int(n)}


# ------------------------------------------------------------------------------ radiance cache
_NRC_FUNCS = {
    "orc_nrc_in_dim": (C.c_int, [C.c_int]),
    "orc_nrc_num_params": (C.c_int64, [C.c_int, C.c_int]),
    "orc_nrc_encode": (None, [C.c_int, f32p, C.c_int, f32p, f32p]),
    "orc_nrc_grid_params": (C.c_int64, []),
    "orc_nrc_forward": (None, [C.c_int, C.c_int, C.c_int, f32p, f32p, C.c_int, f32p]),
    "orc_nrc_loss_grad": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_float, f32p, f32p, f32p, C.c_int, f32p]),
    "orc_adam": (None, [f32p, f32p, f32p, f32p, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                        C.c_int]),
}


def nrc_lib():
    L = lib()
    for name, (res, args) in _NRC_FUNCS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def nrc_encode(encoding: int, queries: np.ndarray, grid: np.ndarray | None = None) -> np.ndarray:
    """Encoded inputs; `grid` = the hash-grid tables (encoding 2: the parameters after the MLP's)."""
    q = np.ascontiguousarray(queries, np.float32)
    n = len(q)
    d = nrc_lib().orc_nrc_in_dim(encoding)
    out = np.zeros((n, d), np.float32)
    g = None if grid is None else np.ascontiguousarray(grid, np.float32)
    nrc_lib().orc_nrc_encode(encoding, p(q, C.c_float), n, p(out, C.c_float), None if g is None else p(g, C.c_float))
    return out


def nrc_grid_params() -> int:
    return int(nrc_lib().orc_nrc_grid_params())


def nrc_forward(encoding: int, hidden: int, out_act: int, params: np.ndarray, queries: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(params, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    out = np.zeros((len(q), 3), np.float32)
    nrc_lib().orc_nrc_forward(encoding, hidden, out_act, p(w, C.c_float), p(q, C.c_float), len(q), p(out, C.c_float))
    return out


def nrc_loss_grad(encoding: int, hidden: int, out_act: int, loss_scale: float, params: np.ndarray,
                  queries: np.ndarray, targets: np.ndarray):
    w = np.ascontiguousarray(params, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    t = np.ascontiguousarray(targets, np.float32)
    g = np.zeros_like(w)
    loss = nrc_lib().orc_nrc_loss_grad(encoding, hidden, out_act, loss_scale, p(w, C.c_float), p(q, C.c_float),
                                       p(t, C.c_float), len(q), p(g, C.c_float))
    return float(loss), g


def adam(w, m, v, grad, lr, beta1, beta2, eps, l2, step):
    w, m, v = (np.ascontiguousarray(a, np.float32).copy() for a in (w, m, v))
    g = np.ascontiguousarray(grad, np.float32)
    nrc_lib().orc_adam(p(w, C.c_float), p(m, C.c_float), p(v, C.c_float), p(g, C.c_float), len(w), lr, beta1, beta2,
                       eps, l2, step)
    return w, m, v


# ------------------------------------------------------------------------------ radiance-cache passes
class OrcNrcSink(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("density_query", C.c_int32),
        ("img_w", C.c_uint32),
        ("img_h", C.c_uint32),
        ("unbiased_offset", C.c_uint32),
        ("termination", C.c_float),
        ("train_termination", C.c_float),
        ("infer_query", f32p),
        ("terminal_tp", f32p),
        ("terminal_bits", u32p),
        ("frame_contribution", f32p),
        ("train_suffix", u32p),
        ("train_query", f32p),
        ("train_target", f32p),
        ("train_local_tp", f32p),
        ("train_bits", u32p),
        ("num_train", u32p),
    ]


TRAIN_BUFFER_SIZE = 131072
TRAIN_PER_FRAME = 65536
INVALID_VERTEX = 0x3FFFFF

_PASS_FUNCS = {
    "orc_nrc_pass": (C.c_int64, [C.POINTER(OrcScene), u64p, C.POINTER(OrcNrcSink), u32p]),
    "orc_nrc_shufflers": (None, [u32p]),
    "orc_nrc_prepare": (None, [u32p, f32p, u32p, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_int32]),
    "orc_nrc_propagate": (None, [C.c_uint32, u32p, f32p, f32p, f32p, f32p, f32p, C.c_float]),
    "orc_nrc_shuffle": (None, [C.c_uint32, f32p, u32p, f32p, f32p, f32p, f32p, C.c_float, u32p]),
    "orc_nrc_accumulate": (None, [C.c_uint32, f32p, f32p, f32p, f32p, C.c_float, C.c_uint32, f64p, f32p]),
}


def pass_lib():
    L = lib()
    for name, (res, args) in _PASS_FUNCS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def nrc_pass(sc: OracleScene, rng: np.ndarray, mode: int, img_w: int, img_h: int, unbiased_offset: int = 0,
             density_query: bool = False, log: bool = False, termination: float = 0.0,
             train_termination: float = 0.0) -> dict:
    """One radiance-cache pass (mode 1 render, 2 training) on the pass image img_w x img_h;
    `rng` (the full image's per-pixel states) is advanced in place."""
    n = img_w * img_h
    out = {
        "infer_query": np.zeros((n, 14), np.float32),
        "terminal_tp": np.zeros((n, 3), np.float32),
        "terminal_bits": np.zeros(n, np.uint32),
        "frame_contribution": np.zeros((n, 3), np.float32),
        "train_suffix": np.full(n, INVALID_VERTEX, np.uint32),
        "train_query": np.zeros((TRAIN_BUFFER_SIZE, 14), np.float32),
        "train_target": np.zeros((TRAIN_BUFFER_SIZE, 3), np.float32),
        "train_local_tp": np.zeros((TRAIN_BUFFER_SIZE, 3), np.float32),
        "train_bits": np.zeros(TRAIN_BUFFER_SIZE, np.uint32),
        "num_train": np.zeros(1, np.uint32),
    }
    k = OrcNrcSink()
    k.mode, k.density_query, k.img_w, k.img_h = mode, int(density_query), img_w, img_h
    k.unbiased_offset = unbiased_offset & 0xFFFFFFFF
    k.termination = termination
    k.train_termination = train_termination
    for name, t in (("infer_query", C.c_float), ("terminal_tp", C.c_float), ("terminal_bits", C.c_uint32),
                    ("frame_contribution", C.c_float), ("train_suffix", C.c_uint32), ("train_query", C.c_float),
                    ("train_target", C.c_float), ("train_local_tp", C.c_float), ("train_bits", C.c_uint32),
                    ("num_train", C.c_uint32)):
        setattr(k, name, p(out[name], t))
    dlog = np.zeros((n, 4), np.uint32) if log else None
    out["lookups"] = int(pass_lib().orc_nrc_pass(sc.ref, p(rng, C.c_uint64), C.byref(k),
                                                 p(dlog, C.c_uint32) if log else None))
    out["log"] = dlog
    return out


def nrc_shufflers() -> np.ndarray:
    out = np.zeros(TRAIN_PER_FRAME, np.uint32)
    pass_lib().orc_nrc_shufflers(p(out, C.c_uint32))
    return out


def nrc_prepare(counters: np.ndarray, stats: np.ndarray, train_suffix: np.ndarray, width: int, height: int,
                buf: int, offset: int, new_sequence: bool) -> None:
    pass_lib().orc_nrc_prepare(p(counters, C.c_uint32), p(stats, C.c_float), p(train_suffix, C.c_uint32), width,
                               height, buf, offset & 0xFFFFFFFF, int(new_sequence))


def nrc_propagate(num_suffixes: int, train_suffix, inferred, infer_query, vertex, train_query0, train_target0,
                  radiance_scale: float = 0.0) -> None:
    """vertex: (M, 4) float32 records (local throughput rgb + bits reinterpreted)."""
    pass_lib().orc_nrc_propagate(num_suffixes, p(train_suffix, C.c_uint32), p(inferred, C.c_float),
                                 p(infer_query, C.c_float), p(vertex, C.c_float), p(train_query0, C.c_float),
                                 p(train_target0, C.c_float), radiance_scale)


def nrc_shuffle(num_training: int, stats_buf, shufflers, train_query0, train_target0, train_query1, train_target1,
                radiance_scale: float = 0.0) -> np.ndarray:
    writers = np.zeros(TRAIN_PER_FRAME, np.uint32)
    pass_lib().orc_nrc_shuffle(num_training, p(stats_buf, C.c_float), p(shufflers, C.c_uint32),
                               p(train_query0, C.c_float), p(train_target0, C.c_float), p(train_query1, C.c_float),
                               p(train_target1, C.c_float), radiance_scale, p(writers, C.c_uint32))
    return writers


def nrc_accumulate(num_pixels: int, terminal, frame_contribution, inferred, infer_query, radiance_scale: float,
                   accum_frames: int, sum_rgb, mean_rgb) -> None:
    pass_lib().orc_nrc_accumulate(num_pixels, p(terminal, C.c_float), p(frame_contribution, C.c_float),
                                  p(inferred, C.c_float), p(infer_query, C.c_float), radiance_scale, accum_frames,
                                  p(sum_rgb, C.c_double), p(mean_rgb, C.c_float))


def suffix_chains(train_suffix: np.ndarray, bits: np.ndarray, n_items: int) -> list:
    """Per pass pixel, the list of training-vertex indices from the first vertex to the last
    (walking the prev links back from the suffix terminal)."""
    chains = []
    for i in range(n_items):
        idx = int(train_suffix[i]) & INVALID_VERTEX
        chain = []
        while idx != INVALID_VERTEX and len(chain) < TRAIN_BUFFER_SIZE:
            chain.append(idx)
            idx = int(bits[idx]) & INVALID_VERTEX
        chains.append(chain[::-1])
    return chains
