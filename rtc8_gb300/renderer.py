"""Host-side driver of the GB300 volumetric path tracer over the C ABI.

:class:`Renderer` owns one ``VptContext`` and mirrors the reference's headless frame loop
(renderer/renderer_main.cpp:1444-1667): scene set-up (volume, environment, camera, medium
parameters) followed by per-frame launches of the path-tracing entry points.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import VptFrameParams, check, ptr
from .configs import SceneConfig, camera_for, sun_direction, volume_box


TRAIN_BUFFER_SIZE = 131072  # VPT_NRC_TRAIN_BUFFER_SIZE
TRAIN_PER_FRAME = 65536     # VPT_NRC_TRAIN_DATA_PER_FRAME


class _DeviceArray:
    """Exposes a raw device allocation through __cuda_array_interface__ (version 3)."""

    def __init__(self, ptr: int, shape: tuple, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_view(ptr: int, shape: tuple, typestr: str):
    """A torch tensor aliasing `shape` elements of type `typestr` at device address `ptr`."""
    import torch

    if not ptr:
        raise ValueError("null device pointer")
    return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device="cuda")


class Renderer:
    def __init__(self, width: int, height: int):
        self.lib = _lib.load()
        self.width, self.height = width, height
        h = C.c_void_p()
        check(self.lib.vpt_create(width, height, C.byref(h)), "vpt_create")
        self.ctx = h
        self.params = VptFrameParams()

    # ------------------------------------------------------------------ lifetime
    def close(self) -> None:
        if self.ctx:
            self.lib.vpt_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ scene
    def seed_rng(self, seed: int) -> None:
        check(self.lib.vpt_seed_rng(self.ctx, C.c_uint64(seed)), "vpt_seed_rng")

    def rng_states(self) -> np.ndarray:
        out = np.empty(self.width * self.height, dtype=np.uint64)
        check(self.lib.vpt_get_rng_states(self.ctx, ptr(out, C.c_uint64)), "vpt_get_rng_states")
        return out

    def set_volume_dense(self, voxels: np.ndarray, voxel_size: float, origin) -> None:
        v = np.ascontiguousarray(voxels, dtype=np.float32)
        o = np.ascontiguousarray(origin, dtype=np.float32)
        nx, ny, nz = v.shape
        check(self.lib.vpt_set_volume_dense(self.ctx, ptr(v, C.c_float), nx, ny, nz, voxel_size, ptr(o, C.c_float)),
              "vpt_set_volume_dense")

    def generate_fbm_volume(self, spec, voxel_size: float, origin) -> None:
        o = np.ascontiguousarray(origin, dtype=np.float32)
        if spec.union_seed is not None:
            check(self.lib.vpt_generate_fbm_union(self.ctx, spec.n, spec.seed, spec.union_seed, spec.octaves,
                                                  spec.lacunarity, spec.gain, spec.base_frequency, spec.threshold,
                                                  voxel_size, ptr(o, C.c_float)), "vpt_generate_fbm_union")
            return
        check(self.lib.vpt_generate_fbm_volume(self.ctx, spec.n, spec.seed, spec.octaves, spec.lacunarity, spec.gain,
                                               spec.base_frequency, spec.threshold, voxel_size, ptr(o, C.c_float)),
              "vpt_generate_fbm_volume")

    def set_volume_nanovdb(self, grid: bytes) -> dict:
        """Density volume from an in-memory NanoVDB float grid (Scene::allocateVolumeGrid,
        renderer/renderer_scene.cpp:491-537); returns the grid's metadata."""
        from . import nvdb

        info = nvdb.grid_info(grid)
        check(self.lib.vpt_set_volume_nanovdb(self.ctx, grid, len(grid)), "vpt_set_volume_nanovdb")
        self._dims = tuple(8 * (hi - lo) // 8 for lo, hi in zip(info["extent_min"], info["extent_max"]))
        return info

    def load_nvdb(self, path, grid: int | str = 0) -> dict:
        """Density volume from grid `grid` (index or name) of an .nvdb file (nanovdb::io::readGrid +
        allocateVolumeGrid, renderer/renderer_scene.cpp:2468-2469); ZIP-coded grids are inflated
        on the host first."""
        from . import nvdb

        return self.set_volume_nanovdb(nvdb.read_grid(path, grid))

    def download_volume(self) -> np.ndarray:
        info = self.volume_info()
        n = info["dims"]
        out = np.empty(n, dtype=np.float32)
        check(self.lib.vpt_download_volume_dense(self.ctx, ptr(out, C.c_float)), "vpt_download_volume_dense")
        return out

    def volume_info(self) -> dict:
        a, t, b = C.c_int64(), C.c_int64(), C.c_int64()
        m = C.c_float()
        check(self.lib.vpt_get_volume_info(self.ctx, C.byref(a), C.byref(t), C.byref(m), C.byref(b)),
              "vpt_get_volume_info")
        tot = t.value
        return {"active_leaves": a.value, "total_leaves": tot, "global_majorant": m.value, "grid_bytes": b.value,
                "dims": self._dims}

    def cell_majorants(self) -> np.ndarray:
        info = self.volume_info()
        out = np.empty(info["total_leaves"], dtype=np.float32)
        check(self.lib.vpt_download_cell_majorants(self.ctx, ptr(out, C.c_float)), "vpt_download_cell_majorants")
        return out

    def load_environment_exr(self, path) -> np.ndarray:
        """Image-based environment from an OpenEXR file (the scene's `envmap`,
        renderer/renderer_scene.cpp:1140-1165, 1765-1790): rows are the polar angle from +y.
        Returns the RGB image that was uploaded."""
        from . import image

        rgb = np.ascontiguousarray(image.read_exr(path)[..., :3])
        self.set_environment_rgb(rgb)
        return rgb

    def set_surfaces(self, scene) -> None:
        """Uploads a rtc8_gb300.surfaces.SurfaceScene (None removes the surfaces): the BVH and
        the emitters' light distributions are built on the host by vpt_set_surfaces."""
        from . import _lib as L

        if scene is None or not scene.instances:
            check(self.lib.vpt_set_surfaces(self.ctx, None, 0, None, 0, None, 0), "vpt_set_surfaces")
            return
        mats = (L.VptSurfaceMaterial * len(scene.materials))()
        for m, src in zip(mats, scene.materials):
            m.kind = src.kind
            m.base_color[:] = [float(x) for x in src.base_color]
            m.roughness, m.metallic = float(src.roughness), float(src.metallic)
            m.emittance[:] = [float(x) for x in src.emittance]
        keep = []
        geoms = (L.VptSurfaceGeometry * len(scene.meshes))()
        for g, mesh in zip(geoms, scene.meshes):
            v = np.ascontiguousarray(mesh.vertices, dtype=np.float32)
            t = np.ascontiguousarray(mesh.triangles, dtype=np.uint32)
            if v.ndim != 2 or v.shape[1] != 9 or t.ndim != 2 or t.shape[1] != 3:
                raise ValueError("set_surfaces: vertices must be (n, 9) and triangles (m, 3)")
            keep += [v, t]
            g.vertices = ptr(v, C.c_float)
            g.num_vertices = len(v)
            g.triangles = ptr(t, C.c_uint32)
            g.num_triangles = len(t)
            g.material = mesh.material
        insts = (L.VptSurfaceInstance * len(scene.instances))()
        for d, src in zip(insts, scene.instances):
            d.first_geometry, d.num_geometries = src.first_geometry, src.num_geometries
            d.transform[:] = [float(x) for x in np.asarray(src.transform, dtype=np.float32).reshape(12)]
            d.uniform_scale = float(src.uniform_scale)
        check(self.lib.vpt_set_surfaces(self.ctx, mats, len(mats), geoms, len(geoms), insts, len(insts)),
              "vpt_set_surfaces")

    def surface_info(self) -> dict:
        tri, nodes, em = C.c_uint32(), C.c_uint32(), C.c_uint32()
        box = (C.c_float * 6)()
        check(self.lib.vpt_get_surface_info(self.ctx, C.byref(tri), C.byref(nodes), C.byref(em), box),
              "vpt_get_surface_info")
        return {"triangles": tri.value, "bvh_nodes": nodes.value, "emitters": em.value, "world_box": list(box)}

    def clear_volume(self) -> None:
        check(self.lib.vpt_clear_volume(self.ctx), "vpt_clear_volume")

    def set_environment_rgb(self, rgb: np.ndarray) -> None:
        img = np.ascontiguousarray(rgb, dtype=np.float32)
        h, w, _ = img.shape
        check(self.lib.vpt_set_environment_rgb(self.ctx, ptr(img, C.c_float), w, h), "vpt_set_environment_rgb")

    def generate_sky(self, width: int, height: int, states: np.ndarray, solar: np.ndarray, cmf: np.ndarray,
                     sun_dir, include_solar_disc: bool) -> None:
        from . import sky as _sky

        s = np.ascontiguousarray(states, dtype=np.float32)
        so = np.ascontiguousarray(solar, dtype=np.float32)
        if s.size != _sky.BANDS * _sky.STATE_FLOATS or so.size != _sky.SOLAR_FLOATS:
            raise ValueError("generate_sky: states must hold 16 x 122 floats and solar SOLAR_FLOATS floats")
        cm = np.ascontiguousarray(cmf, dtype=np.float32)
        d = np.ascontiguousarray(sun_dir, dtype=np.float32)
        check(self.lib.vpt_generate_sky(self.ctx, width, height, ptr(s, C.c_float), ptr(so, C.c_float),
                                        ptr(cm, C.c_float), ptr(d, C.c_float), int(include_solar_disc)),
              "vpt_generate_sky")

    def importance_map(self) -> tuple[np.ndarray, dict]:
        mw, mh, nm = C.c_int32(), C.c_int32(), C.c_int32()
        tot, integ = C.c_int64(), C.c_float()
        check(self.lib.vpt_get_importance_map_info(self.ctx, C.byref(mw), C.byref(mh), C.byref(nm), C.byref(tot),
                                                   C.byref(integ)), "vpt_get_importance_map_info")
        out = np.empty(tot.value, dtype=np.float32)
        check(self.lib.vpt_download_importance_map(self.ctx, ptr(out, C.c_float)), "vpt_download_importance_map")
        return out, {"map_w": mw.value, "map_h": mh.value, "num_mips": nm.value, "integral": integ.value}

    def download_environment(self, width: int, height: int) -> np.ndarray:
        out = np.empty((height, width, 3), dtype=np.float32)
        check(self.lib.vpt_download_environment(self.ctx, ptr(out, C.c_float)), "vpt_download_environment")
        return out

    # ------------------------------------------------------------------ frame
    def set_frame(self, p: VptFrameParams) -> None:
        self.params = p
        check(self.lib.vpt_set_frame_params(self.ctx, C.byref(p)), "vpt_set_frame_params")

    def set_tracker(self, kind: int = 0, slots_per_sm: int = 0, pass_steps: int = 0, track_ctas_per_sm: int = 0) -> None:
        """0 = persistent megakernel (default), 1 = wavefront; see vpt_set_tracker."""
        check(self.lib.vpt_set_tracker(self.ctx, kind, slots_per_sm, pass_steps, track_ctas_per_sm), "vpt_set_tracker")

    def set_leaf_staging(self, min_lanes: int) -> None:
        """Per-warp leaf staging in shared memory (0 = off); see vpt_set_leaf_staging."""
        check(self.lib.vpt_set_leaf_staging(self.ctx, min_lanes), "vpt_set_leaf_staging")

    def set_launch_shape(self, ctas_per_sm: int = 0, threads: int = 0, park_threshold: int = 0) -> None:
        check(self.lib.vpt_set_launch_shape(self.ctx, ctas_per_sm, threads, park_threshold), "vpt_set_launch_shape")

    def launch_plain(self, spp: int, stream: int | None = None) -> None:
        check(self.lib.vpt_launch_plain(self.ctx, C.c_void_p(stream or 0), spp), "vpt_launch_plain")

    def launch_plain_logged(self, spp: int, dev_log_ptr: int, stream: int | None = None) -> None:
        check(self.lib.vpt_launch_plain_logged(self.ctx, C.c_void_p(stream or 0), spp, C.c_void_p(dev_log_ptr)),
              "vpt_launch_plain_logged")

    def synchronize(self, stream: int | None = None) -> None:
        check(self.lib.vpt_synchronize(self.ctx, C.c_void_p(stream or 0)), "vpt_synchronize")

    def reset_accumulation(self) -> None:
        check(self.lib.vpt_reset_accumulation(self.ctx), "vpt_reset_accumulation")

    def download_sum(self) -> tuple[np.ndarray, int]:
        out = np.empty((self.height, self.width, 3), dtype=np.float64)
        n = C.c_uint32()
        check(self.lib.vpt_download_sum(self.ctx, ptr(out, C.c_double), C.byref(n)), "vpt_download_sum")
        return out, n.value

    def download_mean(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), dtype=np.float32)
        check(self.lib.vpt_download_mean(self.ctx, ptr(out, C.c_float)), "vpt_download_mean")
        return out

    def image(self) -> np.ndarray:
        s, n = self.download_sum()
        return s / max(n, 1)

    def image_rgba8(self, brightness: float = 1.0, srgb: bool = True, flip_y: bool = False) -> np.ndarray:
        """The frame the headless loop saves: tone map + sRGB + 8-bit conversion on the device
        (vpt_download_image_rgba8), as an (h, w, 4) uint8 array."""
        out = np.empty((self.height, self.width), dtype=np.uint32)
        flags = (_lib.VPT_SDR_SRGB if srgb else 0) | (_lib.VPT_SDR_FLIP_Y if flip_y else 0)
        check(self.lib.vpt_download_image_rgba8(self.ctx, brightness, flags, ptr(out, C.c_uint32)),
              "vpt_download_image_rgba8")
        return out.view(np.uint8).reshape(self.height, self.width, 4)

    def save_png(self, path, brightness: float = 1.0) -> None:
        """Writes the current frame as the reference's headless loop does ("%03u.png")."""
        from . import image

        image.write_png(path, self.image_rgba8(brightness))

    def save_exr(self, path, brightness: float = 1.0, flip_y: bool = False) -> None:
        """Writes the mean image as saveImageHDR does (half-float A, B, G, R channels)."""
        from . import image

        image.write_exr(path, self.download_mean().reshape(self.height, self.width, 3), brightness, flip_y)

    def counters(self) -> dict:
        a, b, c, d = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(self.lib.vpt_get_counters(self.ctx, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "vpt_get_counters")
        return {"lookups": a.value, "vertices": b.value, "samples": c.value, "cell_steps": d.value}

    def reset_counters(self) -> None:
        check(self.lib.vpt_reset_counters(self.ctx), "vpt_reset_counters")

    def device_errors(self) -> int:
        return int(self.lib.vpt_get_device_errors(self.ctx))

    # ------------------------------------------------------------------ radiance cache
    # The entry points of the reference's NRC frame (renderer_main.cpp:1553-1637).
    def nrc_buffers(self) -> _lib.VptNrcBuffers:
        b = _lib.VptNrcBuffers()
        check(self.lib.vpt_nrc_get_buffers(self.ctx, C.byref(b)), "vpt_nrc_get_buffers")
        return b

    def nrc_views(self) -> dict:
        """torch tensors aliasing the context's radiance-cache buffers (no copies)."""
        b = self.nrc_buffers()
        n = self.width * self.height * b.render_spp
        cap = b.infer_capacity
        tb = TRAIN_BUFFER_SIZE
        return {
            "infer_query": device_view(b.infer_query, (cap, 14), "<f4"),
            "infer_terminal": device_view(b.infer_terminal, (n, 4), "<f4"),
            "train_suffix": device_view(b.train_suffix, (self.width * self.height,), "<i4"),
            "inferred": device_view(b.inferred, (cap, 3), "<f4"),
            "frame_contribution": device_view(b.frame_contribution, (n, 3), "<f4"),
            "train_query0": device_view(b.train_query[0], (tb, 14), "<f4"),
            "train_query1": device_view(b.train_query[1], (tb, 14), "<f4"),
            "train_target0": device_view(b.train_target[0], (tb, 3), "<f4"),
            "train_target1": device_view(b.train_target[1], (tb, 3), "<f4"),
            "train_vertex": device_view(b.train_vertex, (tb, 4), "<f4"),
            "train_end_query": device_view(b.train_end_query, (self.width * self.height, 14), "<f4"),
            "train_end_inferred": device_view(b.train_end_inferred, (self.width * self.height, 3), "<f4"),
            "train_rng": device_view(b.train_rng, (self.width * self.height,), "<i8"),
            "shufflers": device_view(b.shufflers, (TRAIN_PER_FRAME,), "<i4"),
            "counters": device_view(b.counters, (16,), "<i4"),
            "stats": device_view(b.stats, (18,), "<f4"),
        }

    def nrc_set_termination_factor(self, render_factor: float, train_factor: float = 0.0) -> None:
        check(self.lib.vpt_nrc_set_termination_factor(self.ctx, render_factor, train_factor),
              "vpt_nrc_set_termination_factor")

    def nrc_set_combined_pass(self, on: bool) -> None:
        check(self.lib.vpt_nrc_set_combined_pass(self.ctx, int(on)), "vpt_nrc_set_combined_pass")

    def nrc_set_query_density(self, on: bool) -> None:
        check(self.lib.vpt_nrc_set_query_density(self.ctx, int(on)), "vpt_nrc_set_query_density")

    def prepare_nrc(self, buffer_index: int, offset: int, new_sequence: bool, stream: int | None = None) -> None:
        check(self.lib.vpt_prepare_nrc(self.ctx, C.c_void_p(stream or 0), buffer_index, offset & 0xFFFFFFFF,
                                       int(new_sequence)), "vpt_prepare_nrc")

    def launch_generate_training(self, buffer_index: int, stream: int | None = None) -> None:
        check(self.lib.vpt_launch_generate_training(self.ctx, C.c_void_p(stream or 0), buffer_index),
              "vpt_launch_generate_training")

    def propagate(self, stream: int | None = None) -> None:
        check(self.lib.vpt_propagate(self.ctx, C.c_void_p(stream or 0)), "vpt_propagate")

    def shuffle(self, buffer_index: int, stream: int | None = None) -> None:
        check(self.lib.vpt_shuffle(self.ctx, C.c_void_p(stream or 0), buffer_index), "vpt_shuffle")

    def launch_render_nrc(self, stream: int | None = None) -> None:
        check(self.lib.vpt_launch_render_nrc(self.ctx, C.c_void_p(stream or 0)), "vpt_launch_render_nrc")

    def accumulate_inferred(self, accum_frames: int, stream: int | None = None) -> None:
        check(self.lib.vpt_accumulate_inferred(self.ctx, C.c_void_p(stream or 0), accum_frames),
              "vpt_accumulate_inferred")

    def launch_render_nrc_batch(self, spp: int, stream: int | None = None) -> None:
        check(self.lib.vpt_launch_render_nrc_batch(self.ctx, C.c_void_p(stream or 0), spp),
              "vpt_launch_render_nrc_batch")

    def accumulate_inferred_batch(self, accum_frames: int, spp: int, stream: int | None = None) -> None:
        check(self.lib.vpt_accumulate_inferred_batch(self.ctx, C.c_void_p(stream or 0), accum_frames, spp),
              "vpt_accumulate_inferred_batch")

    def nrc_frame(self, cache, train_iterations: int, spp: int, new_sequence: bool,
                  stream: int | None = None) -> None:
        """One frame with the radiance cache `cache` (a :class:`rtc8_gb300.nrc.NeuralRadianceCache`)."""
        check(self.lib.vpt_nrc_frame(self.ctx, cache.h, C.c_void_p(stream or 0), train_iterations, spp,
                                     int(new_sequence)), "vpt_nrc_frame")

    _dims = (0, 0, 0)


def frame_params(cfg: SceneConfig, env_enabled: bool = True) -> VptFrameParams:
    """Per-frame launch parameters of a configuration (renderer_main.cpp:1466-1469 defaults
    are reproduced by SceneConfig's reference-mode values)."""
    cam = camera_for(cfg)
    p = VptFrameParams()
    p.cam_aspect = cam.aspect
    p.cam_fovy = cam.fovy
    p.cam_position[:] = [float(x) for x in cam.position]
    p.cam_orientation[:] = [float(x) for x in cam.orientation]
    p.density_coeff = cfg.volume.sigma_t_max
    p.scattering_albedo = cfg.albedo
    p.phase_kind = cfg.phase_kind
    p.phase_param = cfg.phase_param
    p.radiance_scale = 0.0
    p.env_enabled = int(env_enabled and (cfg.env_constant is not None or cfg.sky is not None))
    p.env_power = 1.0
    p.env_rotation = 0.0
    if cfg.sun_elevation_deg is not None:
        p.sun_enabled = 1
        p.sun_direction[:] = [float(x) for x in sun_direction(cfg.sun_elevation_deg, cfg.sun_azimuth_deg)]
        p.sun_irradiance[:] = [cfg.sun_irradiance] * 3
        p.sun_select_prob = cfg.sun_select_prob if p.env_enabled else 1.0
    p.max_bounces = cfg.max_bounces
    p.rr_start_vertex = cfg.rr_start_vertex
    p.majorant_mode = cfg.majorant_mode
    p.max_steps_per_segment = cfg.max_steps_per_segment
    p.rng_stream_mode = cfg.rng_stream_mode
    p.majorant_cell_log2 = cfg.majorant_cell_log2
    p.shadow_rr_threshold = cfg.shadow_rr_threshold
    return p


def constant_environment(value: float, width: int = 64, height: int = 32) -> np.ndarray:
    return np.full((height, width, 3), value, dtype=np.float32)


def setup_scene(r: Renderer, cfg: SceneConfig, volume: np.ndarray | None = None) -> None:
    """Builds the configuration's scene on the device: volume (generated on the device unless
    `volume` is given), environment, frame parameters, RNG seeds."""
    vs, origin = volume_box(cfg.volume)
    if volume is None:
        r.generate_fbm_volume(cfg.volume, vs, origin)
        r._dims = (cfg.volume.n,) * 3
    else:
        r.set_volume_dense(volume, vs, origin)
        r._dims = tuple(volume.shape)
    if cfg.sky is not None:
        from . import sky as _sky
        d = sun_direction(cfg.sun_elevation_deg, cfg.sun_azimuth_deg)
        st = _sky.load_sky_state(cfg.sky, cfg.sun_elevation_deg, d)
        r.generate_sky(cfg.sky.width, cfg.sky.height, st["states"], st["solar"], st["cmf"], d,
                       cfg.sky.include_solar_disc)
    elif cfg.env_constant is not None:
        r.set_environment_rgb(constant_environment(cfg.env_constant))
    if cfg.surfaces is not None:
        from . import surfaces as _surf
        if cfg.surfaces != "room":
            raise ValueError(f"unknown surface scene {cfg.surfaces!r}")
        r.set_surfaces(_surf.room_scene())
    if not cfg.volume_enabled:
        r.clear_volume()
    r.set_frame(frame_params(cfg))
    r.seed_rng(cfg.rng_seed)
