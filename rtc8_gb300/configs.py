"""Scene configurations of the volumetric workloads, with their seeded synthetic inputs.

Reference defaults (renderer/renderer_main.cpp:1466-1469, renderer_shared.h:10-13): density
coefficient 0.3 over a NanoVDB grid, albedo 0.99, Schlick forwardness 0, Russian roulette at
every vertex, no bounce cap, a single global majorant, RNG seeds from
std::mt19937_64(591842031321323413). The GB300 workloads below add a directional sun, the
Henyey-Greenstein phase function, bounce caps and the majorant grid; their volumes are
seeded fBm value noise generated on the device.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field

import numpy as np

REFERENCE_RNG_SEED = 591842031321323413


@dataclass(frozen=True)
class VolumeSpec:
    n: int                      # voxels per axis
    seed: int = 1
    octaves: int = 4
    lacunarity: float = 2.0
    gain: float = 0.5
    base_frequency: float = 4.0  # lattice cells across the grid at the first octave
    threshold: float = 0.0       # > 0: sparse cloud, density = max(0, (r - t) / (1 - t))
    sigma_t_max: float = 20.0    # density coefficient (grid values lie in [0, 1])
    union_seed: int | None = None  # a second cloud (same parameters, this seed) unioned by max


@dataclass(frozen=True)
class SkySpec:
    turbidity: float = 3.0
    ground_albedo: float = 0.3
    width: int = 3200
    height: int = 1600
    include_solar_disc: bool = False


@dataclass(frozen=True)
class SceneConfig:
    name: str
    width: int
    height: int
    spp: int
    volume: VolumeSpec
    albedo: float = 0.99
    phase_kind: int = 1          # 0 = Schlick (reference), 1 = Henyey-Greenstein
    phase_param: float = 0.8
    sun_elevation_deg: float | None = 30.0
    sun_azimuth_deg: float = 120.0
    sun_irradiance: float = 10.0
    sun_select_prob: float = 0.5
    env_constant: float | None = 0.5
    sky: SkySpec | None = None
    max_bounces: int = 64
    rr_start_vertex: int = 9     # "Russian roulette after 8" bounces
    majorant_mode: int = 1       # 1 = 8^3 majorant grid with DDA
    max_steps_per_segment: int = 1 << 20
    rng_stream_mode: int = 1       # 0 = reference per-pixel sequential streams, 1 = sample-parallel
    majorant_cell_log2: int = 3    # majorant-grid cell = 2^k voxels (3: one cell per 8^3 leaf)
    # Russian roulette on NEE shadow-ray visibility below this threshold (unbiased; 0 = off, the
    # reference's plain ratio tracking). About 85% of the density lookups of these scenes are
    # shadow-ray steps, most of them where the visibility is already near zero.
    shadow_rr_threshold: float = 0.1
    fov_deg: float = 40.0
    cam_distance_diagonals: float = 2.5
    cam_direction: tuple = (0.55, 0.3, 1.0)   # from the grid centre towards the camera
    rng_seed: int = REFERENCE_RNG_SEED
    # Triangle meshes around the volume: the name of a procedural scene of
    # rtc8_gb300.surfaces ("room"), or None; volume_enabled = False renders the surfaces alone.
    surfaces: str | None = None
    volume_enabled: bool = True

    def replace(self, **kw) -> "SceneConfig":
        return dataclasses.replace(self, **kw)

    @property
    def paths_per_frame(self) -> int:
        return self.width * self.height


# Dense workload: plain tracer, 256^2 x 16 spp, dense 64^3 fBm, sigma_t max 20.
C1 = SceneConfig(name="c1_dense64_256px", width=256, height=256, spp=16,
                 volume=VolumeSpec(n=64, seed=1, octaves=4, sigma_t_max=20.0),
                 albedo=0.99, phase_kind=1, phase_param=0.8, sun_elevation_deg=30.0, env_constant=0.5,
                 max_bounces=64, rr_start_vertex=9)

# The same scene rendered with the reference's own path rules: single global majorant,
# Schlick phase function, no bounce cap, Russian roulette at every vertex, environment only.
C1_REFERENCE_MODE = C1.replace(name="c1_reference_mode", phase_kind=0, phase_param=0.0, sun_elevation_deg=None,
                               max_bounces=0, rr_start_vertex=1, majorant_mode=0, rng_stream_mode=0,
                               shadow_rr_threshold=0.0)

# Sparse workload at scale: 1024^2 x 64 spp, sparse 512^3 fBm (6 octaves, threshold 0.55),
# sigma_t max 200, albedo 0.999, HG g = 0.85, <= 256 bounces, sun at 20 degrees + Hosek sky.
C2 = SceneConfig(name="c2_sparse512_1024px", width=1024, height=1024, spp=64,
                 volume=VolumeSpec(n=512, seed=2, octaves=6, threshold=0.55, sigma_t_max=200.0),
                 albedo=0.999, phase_kind=1, phase_param=0.85, sun_elevation_deg=20.0, env_constant=None,
                 sky=SkySpec(turbidity=3.0, ground_albedo=0.3), max_bounces=256, rr_start_vertex=9,
                 majorant_cell_log2=5)

# Stress workload: 2048^2, sparse 1024^3 made of two fBm clouds unioned
# (threshold 0.78: about 8% of the leaves hold density), sigma_t max 400, albedo 0.9995, g = 0.9,
# <= 1024 bounces.
C5 = SceneConfig(name="c5_sparse1024_2048px", width=2048, height=2048, spp=16,
                 volume=VolumeSpec(n=1024, seed=5, octaves=6, threshold=0.78, sigma_t_max=400.0, union_seed=6),
                 albedo=0.9995, phase_kind=1, phase_param=0.9, sun_elevation_deg=20.0, env_constant=None,
                 sky=SkySpec(turbidity=3.0, ground_albedo=0.3), max_bounces=1024, rr_start_vertex=9,
                 majorant_cell_log2=6)

# Mixed surface + volume workload (the reference's scenes put clouds among meshes): the dense
# 64^3 cloud of C1 inside an open room with coloured Lambert walls, a glossy and a metallic
# SimplePBR block and a rectangle light under the ceiling, 512^2, seen from the open side.
C_ROOM = C1.replace(name="room_cloud64_512px", width=512, height=512, surfaces="room", cam_direction=(0.0, 0.12, 1.0),
                    cam_distance_diagonals=1.55, fov_deg=48.0, sun_azimuth_deg=20.0)
# The same with the reference's own path rules.
C_ROOM_REFERENCE_MODE = C_ROOM.replace(name="room_reference_mode", phase_kind=0, phase_param=0.0,
                                       sun_elevation_deg=None, max_bounces=0, rr_start_vertex=1, majorant_mode=0,
                                       rng_stream_mode=0, shadow_rr_threshold=0.0)

CONFIGS = {c.name: c for c in (C1, C1_REFERENCE_MODE, C2, C5, C_ROOM, C_ROOM_REFERENCE_MODE)}


# ------------------------------------------------------------------------------ geometry
def sun_direction(elevation_deg: float, azimuth_deg: float) -> np.ndarray:
    """Unit vector towards the sun, y up; azimuth measured from +z towards +x."""
    e, a = math.radians(elevation_deg), math.radians(azimuth_deg)
    return np.array([math.cos(e) * math.sin(a), math.sin(e), math.cos(e) * math.cos(a)], dtype=np.float64)


def quat_from_matrix(m: np.ndarray) -> np.ndarray:
    """Quaternion (x, y, z, w) of a rotation matrix whose columns are the rotated axes."""
    t = m[0, 0] + m[1, 1] + m[2, 2]
    if t > 0:
        s = math.sqrt(t + 1.0) * 2
        w, x, y, z = 0.25 * s, (m[2, 1] - m[1, 2]) / s, (m[0, 2] - m[2, 0]) / s, (m[1, 0] - m[0, 1]) / s
    elif m[0, 0] > m[1, 1] and m[0, 0] > m[2, 2]:
        s = math.sqrt(1.0 + m[0, 0] - m[1, 1] - m[2, 2]) * 2
        w, x, y, z = (m[2, 1] - m[1, 2]) / s, 0.25 * s, (m[0, 1] + m[1, 0]) / s, (m[0, 2] + m[2, 0]) / s
    elif m[1, 1] > m[2, 2]:
        s = math.sqrt(1.0 + m[1, 1] - m[0, 0] - m[2, 2]) * 2
        w, x, y, z = (m[0, 2] - m[2, 0]) / s, (m[0, 1] + m[1, 0]) / s, 0.25 * s, (m[1, 2] + m[2, 1]) / s
    else:
        s = math.sqrt(1.0 + m[2, 2] - m[0, 0] - m[1, 1]) * 2
        w, x, y, z = (m[1, 0] - m[0, 1]) / s, (m[0, 2] + m[2, 0]) / s, (m[1, 2] + m[2, 1]) / s, 0.25 * s
    q = np.array([x, y, z, w])
    return q / np.linalg.norm(q)


def look_at(position, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Orientation of a camera at `position` looking at `target`; the camera looks down its
    local -z axis (optix_pathtracing_kernels.cu:52), local +y is up."""
    p, t, u = (np.asarray(v, dtype=np.float64) for v in (position, target, up))
    back = p - t
    back /= np.linalg.norm(back)
    right = np.cross(u, back)
    right /= np.linalg.norm(right)
    up2 = np.cross(back, right)
    return quat_from_matrix(np.stack([right, up2, back], axis=1))


@dataclass
class Camera:
    aspect: float
    fovy: float            # radians
    position: np.ndarray
    orientation: np.ndarray  # quaternion x, y, z, w


def volume_box(spec: VolumeSpec) -> tuple[float, np.ndarray]:
    """Voxel size and origin that place the grid in the unit cube [-0.5, 0.5]^3."""
    return 1.0 / spec.n, np.array([-0.5, -0.5, -0.5], dtype=np.float32)


def camera_for(cfg: SceneConfig) -> Camera:
    diag = math.sqrt(3.0)
    d = np.asarray(cfg.cam_direction, dtype=np.float64)
    d /= np.linalg.norm(d)
    pos = d * cfg.cam_distance_diagonals * diag
    q = look_at(pos, (0.0, 0.0, 0.0))
    return Camera(aspect=cfg.width / cfg.height, fovy=math.radians(cfg.fov_deg), position=pos, orientation=q)
