"""ctypes binding of libvradgpu.so (the C ABI in include/vradgpu.h).

There is no fallback: if the library is missing or fails to load, every
entry point raises.  ``load(build=True)`` compiles it in-tree first.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

VRG_OK = 0
ERRORS = {-1: "invalid argument", -2: "out of memory", -3: "CUDA error", -4: "timeout",
          -5: "call out of order", -6: "unsupported"}

_lock = threading.Lock()
_lib = None

P = C.c_void_p
F = C.c_float
I32 = C.c_int32
I64 = C.c_int64
U64 = C.c_uint64

SIGNATURES = {
    "vrg_ctx_create": (C.c_int, [C.c_int, P]),
    "vrg_ctx_destroy": (None, [P]),
    "vrg_last_error": (C.c_char_p, [P]),
    "vrg_ctx_set_stream": (C.c_int, [P, P]),
    "vrg_ctx_synchronize": (C.c_int, [P]),
    "vrg_ctx_set_timing": (C.c_int, [P, C.c_int]),
    "vrg_ctx_kernel_stats": (C.c_int, [P, C.c_char_p, P, P]),
    "vrg_ctx_reset_stats": (C.c_int, [P]),
    "vrg_ctx_launch_count": (I64, [P]),
    "vrg_ctx_set_autotune": (C.c_int, [P, C.c_int]),
    "vrg_ctx_autotune_choice": (C.c_int, [P, C.c_char_p, P, P, I32]),
    "vrg_ctx_autotune_save": (C.c_int, [P, C.c_char_p]),
    "vrg_ctx_autotune_load": (C.c_int, [P, C.c_char_p]),
    "vrg_ctx_set_hbm_reserve": (C.c_int, [P, U64]),
    "vrg_env_create": (C.c_int, [P, P]),
    "vrg_env_destroy": (None, [P]),
    "vrg_env_add_triangle": (C.c_int, [P, I32, P, P, P, P, C.c_uint16, I32]),
    "vrg_env_add_quad": (C.c_int, [P, I32, P, P, P, P, P]),
    "vrg_env_add_axis_aligned_rectangular_solid": (C.c_int, [P, I32, P, P, P]),
    "vrg_env_add_triangles": (C.c_int, [P, P, P, I64]),
    "vrg_env_setup_acceleration_structure": (C.c_int, [P]),
    "vrg_env_num_triangles": (I64, [P]),
    "vrg_env_tree_info": (C.c_int, [P, P, P, P]),
    "vrg_env_get_tree": (C.c_int, [P, P, P, P]),
    "vrg_env_set_walk_tree_costs": (C.c_int, [P, F, F, F, I32]),
    "vrg_env_walk_tree_info": (C.c_int, [P, P, P, P]),
    "vrg_env_set_walk_tree_builder": (C.c_int, [P, I32]),
    "vrg_env_wall_slots": (C.c_int, [P, P, P]),
    "vrg_env_set_wall_slots": (C.c_int, [P, I32]),
    "vrg_env_get_walk_tree": (C.c_int, [P, P, P, P]),
    "vrg_env_get_triangle": (C.c_int, [P, I64, P]),
    "vrg_env_bounds": (C.c_int, [P, P, P]),
    "vrg_env_trace4_rays": (C.c_int, [P, P, P, P, P, I32, P, P, P]),
    "vrg_env_trace_closest": (C.c_int, [P, P, P, P, P, I64, I32, P, P]),
    "vrg_env_trace_closest_d": (C.c_int, [P, P, P, P, P, I64, I32, P, P]),
    "vrg_env_test_line_does_hit_sky": (C.c_int, [P, P, P, I64, I32, P]),
    "vrg_env_occlusion_mask": (C.c_int, [P, P, P, I64, I32, P, P, P]),
    "vrg_env_trace_coverage": (C.c_int, [P, P, P, P, P, I64, I32, P, P, P]),
    "vrg_env_test_line_coverage": (C.c_int, [P, P, P, I64, I32, P]),
    "vrg_env_set_triangle_flags": (C.c_int, [P, I64, I64, P, P]),
    "vrg_env_occlusion_mask_d": (C.c_int, [P, P, P, I64, I32, P, P, P]),
    "vrg_env_add_to_ray_stream": (C.c_int, [P, P, P, I32]),
    "vrg_env_flush_stream_entry": (C.c_int, [P]),
    "vrg_env_finish_ray_stream": (C.c_int, [P, P, I64, P]),
    "vrg_light_set_falloff_params": (C.c_int, [P, P]),
    "vrg_light_parse_spot": (C.c_int, [P, P]),
    "vrg_light_parse_point": (C.c_int, [P, P]),
    "vrg_env_set_lights": (C.c_int, [P, P, I32]),
    "vrg_env_set_faces": (C.c_int, [P, I32, P, P, P, P, P, P, P, P, P, P]),
    "vrg_env_num_luxels": (I64, [P]),
    "vrg_env_gather_direct_light": (C.c_int, [P, I32, U64, P, P]),
    "vrg_env_gather_direct_light_d": (C.c_int, [P, I32, U64, P, P]),
    "vrg_env_gather_points": (C.c_int, [P, P, P, I64, P, P]),
    "vrg_env_make_patches": (C.c_int, [P, F, F, P, P]),
    "vrg_env_get_patches": (C.c_int, [P, P, P, P, P, P, P, P, P, P, P, P]),
    "vrg_env_make_transfers": (C.c_int, [P, P, I32, P]),
    "vrg_env_get_transfers": (C.c_int, [P, P, P, P]),
    "vrg_env_transfer_info": (C.c_int, [P, P, P, P]),
    "vrg_ctx_set_transfer_table_limit": (C.c_int, [P, I32]),
    "vrg_env_gather_patch_direct": (C.c_int, [P, P]),
    "vrg_env_bounce_light": (C.c_int, [P, I32, F, P, P, P]),
    "vrg_env_bounce_light_noalloc": (C.c_int, [P, I32, F, P, P, P]),
    "vrg_env_bake": (C.c_int, [P, I32, U64, I32, F, P]),
    "vrg_env_get_bake": (C.c_int, [P, P, P, P, P, P]),
    "vrg_calc_face_extents": (C.c_int, [P, I32, P, P, P, P]),
    "vrg_env_get_lightmap": (C.c_int, [P, P, P]),
    "vrg_env_add_bsp_world": (C.c_int, [P, P, P, P]),
    "vrg_base_winding_for_plane": (C.c_int, [P, F, P]),
    "vrg_chop_winding": (C.c_int, [P, I32, P, F, F, P, P]),
    "vrg_env_get_triangle_vertices": (C.c_int, [P, I64, I64, P, P]),
    "vrg_env_can_leaf_trace_to_sky": (C.c_int, [P, P, P, I64, P]),
    "vrg_leaf_sky_lines": (C.c_int, [P, P, I64, P, P]),
    "vrg_bsp_open": (C.c_int, [P, C.c_size_t, P]),
    "vrg_bsp_close": (None, [P]),
    "vrg_bsp_get_world": (C.c_int, [P, P]),
    "vrg_bsp_use_hdr_faces": (C.c_int, [P, I32]),
    "vrg_bsp_info": (C.c_int, [P, P, P, P]),
    "vrg_batch_create": (C.c_int, [P, P]),
    "vrg_batch_destroy": (None, [P]),
    "vrg_batch_add": (C.c_int, [P, P]),
    "vrg_batch_size": (I32, [P]),
    "vrg_batch_bake": (C.c_int, [P, I32, U64, I32, F, P]),
    "vrg_env_relight_prepare": (C.c_int, [P, I32, U64, I32, F]),
    "vrg_env_relight": (C.c_int, [P, P, I32, I32, F, P, P]),
    "vrg_server_create": (C.c_int, [P, I32, I32, F, P]),
    "vrg_server_destroy": (None, [P]),
    "vrg_server_add_scene": (C.c_int, [P, P, P]),
    "vrg_server_submit": (C.c_int, [P, I32, P, I32, P]),
    "vrg_server_wait": (C.c_int, [P, I64, C.c_double]),
    "vrg_server_drain": (C.c_int, [P, C.c_double]),
    "vrg_server_result": (C.c_int, [P, I64, P, P, P, P, P]),
}


def header_symbols():
    """Function names declared in include/vradgpu.h."""
    import re

    text = (_build.PKG.parent / "include" / "vradgpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(vrg_\w+)\s*\(", text, re.M)))


def load(build: bool = True):
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build() if build else _build.LIB
            if not path.exists():
                raise RuntimeError(f"libvradgpu.so not built ({path}); run vrad_gb300.build.build()")
            lib = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


class VrgError(RuntimeError):
    pass


def check(rc: int, ctx=None, what: str = ""):
    if rc != VRG_OK:
        msg = ""
        if ctx is not None:
            raw = load().vrg_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise VrgError(f"{what}: {ERRORS.get(rc, rc)} ({rc}) {msg}".strip())
