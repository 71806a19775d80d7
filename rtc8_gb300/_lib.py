"""ctypes binding of ``librtc8_gb300.so`` (the C ABI in include/rtc8_vpt.h and rtc8_nrc.h).

The library is built in-tree by :func:`rtc8_gb300.build.build`. Loading fails loudly when it
is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "librtc8_gb300.so"

VPT_SDR_SRGB = 0x1  # include/rtc8_vpt.h
VPT_SDR_FLIP_Y = 0x2

c_float_p = C.POINTER(C.c_float)
c_double_p = C.POINTER(C.c_double)
c_u32_p = C.POINTER(C.c_uint32)
c_u64_p = C.POINTER(C.c_uint64)
c_i32_p = C.POINTER(C.c_int32)
c_i64_p = C.POINTER(C.c_int64)


class VptFrameParams(C.Structure):
    """Mirror of ``VptFrameParams`` (include/rtc8_vpt.h)."""

    _fields_ = [
        ("cam_aspect", C.c_float),
        ("cam_fovy", C.c_float),
        ("cam_position", C.c_float * 3),
        ("cam_orientation", C.c_float * 4),
        ("density_coeff", C.c_float),
        ("scattering_albedo", C.c_float),
        ("phase_kind", C.c_int32),
        ("phase_param", C.c_float),
        ("radiance_scale", C.c_float),
        ("env_enabled", C.c_int32),
        ("env_power", C.c_float),
        ("env_rotation", C.c_float),
        ("sun_enabled", C.c_int32),
        ("sun_direction", C.c_float * 3),
        ("sun_irradiance", C.c_float * 3),
        ("sun_select_prob", C.c_float),
        ("max_bounces", C.c_int32),
        ("rr_start_vertex", C.c_int32),
        ("majorant_mode", C.c_int32),
        ("max_steps_per_segment", C.c_int32),
        ("rng_stream_mode", C.c_int32),
        ("majorant_cell_log2", C.c_int32),
        ("shadow_rr_threshold", C.c_float),
    ]


class VptNoAllocTrace(C.Structure):
    """Mirror of ``VptNoAllocTrace`` (include/rtc8_vpt.h): arguments of the allocation-free launch."""

    _fields_ = [
        ("frame", VptFrameParams),
        ("width", C.c_int32), ("height", C.c_int32),
        ("spp", C.c_uint32), ("accum_base", C.c_uint32), ("stream_base", C.c_uint32),
        ("leaf_table", C.c_void_p), ("leaf_values", C.c_void_p), ("majorants", C.c_void_p),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("mx", C.c_int32), ("my", C.c_int32), ("mz", C.c_int32),
        ("voxel_size", C.c_float), ("origin", C.c_float * 3), ("global_majorant", C.c_float),
        ("env_texels", C.c_void_p), ("env_w", C.c_int32), ("env_h", C.c_int32),
        ("imp_mips", C.c_void_p), ("map_w", C.c_int32), ("map_h", C.c_int32), ("num_mips", C.c_int32),
        ("imp_integral", C.c_float),
        ("rng", C.c_void_p), ("sum_rgb", C.c_void_p), ("mean_rgb", C.c_void_p),
        ("device_errors", C.c_void_p),
    ]


class VptNanoVdbInfo(C.Structure):
    """Mirror of ``VptNanoVdbInfo`` (include/rtc8_vpt.h)."""

    _fields_ = [
        ("name", C.c_char * 256),
        ("grid_type", C.c_uint32), ("grid_class", C.c_uint32),
        ("grid_bytes", C.c_uint64), ("file_bytes", C.c_uint64), ("active_voxels", C.c_uint64),
        ("index_min", C.c_int32 * 3), ("index_max", C.c_int32 * 3),
        ("world_min", C.c_double * 3), ("world_max", C.c_double * 3), ("voxel_size", C.c_double * 3),
        ("map_mat_f", C.c_float * 9), ("map_inv_mat_f", C.c_float * 9), ("map_vec_f", C.c_float * 3),
        ("map_mat_d", C.c_double * 9), ("map_vec_d", C.c_double * 3),
        ("background", C.c_float),
        ("node_count", C.c_uint32 * 3), ("tile_count", C.c_uint32 * 3),
        ("codec", C.c_uint32), ("grid_count", C.c_uint32), ("payload_offset", C.c_uint64),
        ("extent_min", C.c_int32 * 3), ("extent_max", C.c_int32 * 3), ("flat_leaves", C.c_int64),
    ]


class VptSurfaceMaterial(C.Structure):
    """Mirror of ``VptSurfaceMaterial`` (include/rtc8_vpt.h)."""

    _fields_ = [
        ("kind", C.c_int32), ("base_color", C.c_float * 3), ("roughness", C.c_float), ("metallic", C.c_float),
        ("emittance", C.c_float * 3),
    ]


class VptSurfaceGeometry(C.Structure):
    """Mirror of ``VptSurfaceGeometry`` (include/rtc8_vpt.h)."""

    _fields_ = [
        ("vertices", c_float_p), ("num_vertices", C.c_uint32),
        ("triangles", C.POINTER(C.c_uint32)), ("num_triangles", C.c_uint32), ("material", C.c_uint32),
    ]


class VptSurfaceInstance(C.Structure):
    """Mirror of ``VptSurfaceInstance`` (include/rtc8_vpt.h)."""

    _fields_ = [
        ("first_geometry", C.c_uint32), ("num_geometries", C.c_uint32), ("transform", C.c_float * 12),
        ("uniform_scale", C.c_float),
    ]


# name -> (restype, argtypes)
_VPT = {
    "vpt_create": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "vpt_destroy": (C.c_int, [C.c_void_p]),
    "vpt_last_error": (C.c_char_p, []),
    "vpt_seed_rng": (C.c_int, [C.c_void_p, C.c_uint64]),
    "vpt_set_rng_states": (C.c_int, [C.c_void_p, c_u64_p]),
    "vpt_get_rng_states": (C.c_int, [C.c_void_p, c_u64_p]),
    "vpt_set_volume_dense": (C.c_int, [C.c_void_p, c_float_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, c_float_p]),
    "vpt_set_volume_dense_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float,
                                              c_float_p]),
    "vpt_generate_fbm_volume": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32, C.c_int32, C.c_float, C.c_float, C.c_float,
                                          C.c_float, C.c_float, c_float_p]),
    "vpt_download_volume_dense": (C.c_int, [C.c_void_p, c_float_p]),
    "vpt_get_volume_info": (C.c_int, [C.c_void_p, c_i64_p, c_i64_p, c_float_p, c_i64_p]),
    "vpt_download_cell_majorants": (C.c_int, [C.c_void_p, c_float_p]),
    "vpt_nvdb_file_info": (C.c_int, [C.c_char_p, C.c_uint64, C.POINTER(VptNanoVdbInfo)]),
    "vpt_nanovdb_grid_info": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(VptNanoVdbInfo)]),
    "vpt_nanovdb_decode_leaves": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int64, c_i32_p, c_float_p, c_i64_p]),
    "vpt_set_volume_nanovdb": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "vpt_set_volume_nvdb_file": (C.c_int, [C.c_void_p, C.c_char_p, C.c_uint64]),
    "vpt_set_surfaces": (C.c_int, [C.c_void_p, C.POINTER(VptSurfaceMaterial), C.c_uint32,
                                   C.POINTER(VptSurfaceGeometry), C.c_uint32, C.POINTER(VptSurfaceInstance),
                                   C.c_uint32]),
    "vpt_get_surface_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint32), c_float_p]),
    "vpt_clear_volume": (C.c_int, [C.c_void_p]),
    "vpt_set_environment_rgb": (C.c_int, [C.c_void_p, c_float_p, C.c_int32, C.c_int32]),
    "vpt_get_importance_map_info": (C.c_int, [C.c_void_p, c_i32_p, c_i32_p, c_i32_p, c_i64_p, c_float_p]),
    "vpt_download_importance_map": (C.c_int, [C.c_void_p, c_float_p]),
    "vpt_generate_sky": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, c_float_p, c_float_p, c_float_p, c_float_p,
                                   C.c_int32]),
    "vpt_download_environment": (C.c_int, [C.c_void_p, c_float_p]),
    "vpt_set_frame_params": (C.c_int, [C.c_void_p, C.POINTER(VptFrameParams)]),
    "vpt_launch_plain": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vpt_launch_plain_logged": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vpt_launch_plain_noalloc": (C.c_int, [C.POINTER(VptNoAllocTrace), C.c_void_p]),
    "vpt_set_leaf_staging": (C.c_int, [C.c_void_p, C.c_int32]),
    "vpt_nrc_set_combined_pass": (C.c_int, [C.c_void_p, C.c_int32]),
    "vpt_tonemap": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_uint32, C.c_void_p, C.c_void_p]),
    "vpt_download_image_rgba8": (C.c_int, [C.c_void_p, C.c_float, C.c_uint32, c_u32_p]),
    "vpt_reset_accumulation": (C.c_int, [C.c_void_p]),
    "vpt_download_sum": (C.c_int, [C.c_void_p, c_double_p, c_u32_p]),
    "vpt_download_mean": (C.c_int, [C.c_void_p, c_float_p]),
    "vpt_get_accum_device_ptrs": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "vpt_get_counters": (C.c_int, [C.c_void_p, c_u64_p, c_u64_p, c_u64_p, c_u64_p]),
    "vpt_reset_counters": (C.c_int, [C.c_void_p]),
    "vpt_get_device_errors": (C.c_uint32, [C.c_void_p]),
    "vpt_synchronize": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vpt_set_launch_shape": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "vpt_set_tracker": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "vpt_generate_fbm_union": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, C.c_int32, C.c_float, C.c_float,
                                         C.c_float, C.c_float, C.c_float, c_float_p]),
    "vpt_nrc_enable": (C.c_int, [C.c_void_p]),
    "vpt_nrc_get_buffers": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vpt_nrc_set_query_density": (C.c_int, [C.c_void_p, C.c_int32]),
    "vpt_nrc_set_termination_factor": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "vpt_prepare_nrc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32]),
    "vpt_launch_generate_training": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vpt_propagate": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vpt_shuffle": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vpt_launch_render_nrc": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vpt_accumulate_inferred": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vpt_launch_render_nrc_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vpt_accumulate_inferred_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    "vpt_nrc_frame": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32]),
}

class VptNrcBuffers(C.Structure):
    """Device pointers of the radiance-cache buffers of a context (rtc8_vpt.h)."""

    _fields_ = [
        ("infer_query", C.c_void_p),
        ("infer_terminal", C.c_void_p),
        ("train_suffix", C.c_void_p),
        ("inferred", C.c_void_p),
        ("frame_contribution", C.c_void_p),
        ("train_query", C.c_void_p * 2),
        ("train_target", C.c_void_p * 2),
        ("train_vertex", C.c_void_p),
        ("train_end_query", C.c_void_p),
        ("train_end_inferred", C.c_void_p),
        ("train_rng", C.c_void_p),
        ("shufflers", C.c_void_p),
        ("counters", C.c_void_p),
        ("stats", C.c_void_p),
        ("infer_capacity", C.c_uint32),
        ("buffer_index", C.c_uint32),
        ("render_spp", C.c_uint32),
    ]


class NrcConfig(C.Structure):
    _fields_ = [
        ("encoding", C.c_int32), ("num_hidden_layers", C.c_int32), ("output_activation", C.c_int32),
        ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
        ("l2_reg", C.c_float), ("ema_decay", C.c_float), ("loss_scale", C.c_float), ("seed", C.c_uint32),
    ]


_NRC = {
    "nrc_default_config": (None, [C.c_int32, C.POINTER(NrcConfig)]),
    "nrc_create": (C.c_int, [C.POINTER(NrcConfig), C.POINTER(C.c_void_p)]),
    "nrc_destroy": (C.c_int, [C.c_void_p]),
    "nrc_last_error": (C.c_char_p, []),
    "nrc_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "nrc_infer_device_count": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "nrc_infer_indexed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.c_void_p]),
    "nrc_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, c_float_p]),
    "nrc_get_layout": (C.c_int, [C.c_void_p, c_i32_p, c_i32_p, c_i32_p, c_i64_p]),
    "nrc_get_params": (C.c_int, [C.c_void_p, c_float_p]),
    "nrc_set_params": (C.c_int, [C.c_void_p, c_float_p]),
    "nrc_get_gradients": (C.c_int, [C.c_void_p, c_float_p]),
    "nrc_encode": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "nrc_step_count": (C.c_uint64, [C.c_void_p]),
    "nrc_device_errors": (C.c_uint32, [C.c_void_p]),
    "nrc_selftest_mma": (C.c_int, [c_float_p, c_float_p, C.c_int32, C.c_int32, c_float_p]),
    "nrc_selftest_mma_rate": (C.c_int, [C.c_int32, C.c_uint32, c_double_p]),
}



EXPORTS: dict[str, tuple] = dict(_VPT)
EXPORTS.update(_NRC)

_lib: C.CDLL | None = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads the product library and declares every exported entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(rtc8_gb300 has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class VptError(RuntimeError):
    pass


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = load().vpt_last_error()
        raise VptError(f"{what} failed with code {rc}: {msg.decode() if msg else ''}")


def ptr(arr, ctype):
    """Pointer to a contiguous numpy array."""
    return arr.ctypes.data_as(C.POINTER(ctype))
