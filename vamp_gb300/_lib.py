"""ctypes binding of libvamp_gb300.so (the C ABI in include/vamp_gb300.h).

The shared library is built in tree (python -m vamp_gb300.build).  There is no fallback: if the
library is missing, importing vamp_gb300 raises, and if no GPU is usable every check raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvamp_gb300.so"

VG_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "invalid state", -5: "limit exceeded"}
SQRT_X86, SQRT_EXACT = 0, 1

_p = ctypes.c_void_p
_f = ctypes.c_float
_i = ctypes.c_int
_sz = ctypes.c_size_t
_s = ctypes.c_char_p


class VampError(RuntimeError):
    pass


def _load() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA library first (python -m vamp_gb300.build). "
            "vamp_gb300 has no CPU fallback."
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    sig = {
        "vg_last_error": ([], _s),
        "vg_version": ([], _s),
        "vg_robot_info": ([_s, _p, _p, _p, _p, _p], _i),
        "vg_robot_limits": ([_s, _p, _p], _i),
        "vg_env_create": ([], _p),
        "vg_env_destroy": ([_p], None),
        "vg_env_add_sphere": ([_p, _p], _i),
        "vg_env_add_capsule": ([_p, _p], _i),
        "vg_env_add_cuboid": ([_p, _p], _i),
        "vg_env_add_pointcloud": ([_p, _p, _sz, _f, _f, _f], _i),
        "vg_env_add_pointcloud_device": ([_p, _p, _sz, _f, _f, _f, _p], _i),
        "vg_env_add_heightfield": ([_p, _p, _p, _sz, _sz, _p], _i),
        "vg_validate_vectors_device": ([ctypes.c_char_p, _p, _p, _p, _p, _sz, _i, _p, _p, _p], _i),
        "vg_validate_vectors": ([ctypes.c_char_p, _p, _p, _p, _p, _sz, _i, _p], _i),
        "vg_filter_self_from_pointcloud_device": ([ctypes.c_char_p, _p, _p, _sz, _f, _p, _p, _p, _p], _i),
        "vg_filter_self_from_pointcloud": ([ctypes.c_char_p, _p, _p, _sz, _f, _p, _p, _p], _i),
        "vg_env_attach": ([_p, _p, _p, _sz], _i),
        "vg_env_detach": ([_p], _i),
        "vg_eefk_device": ([ctypes.c_char_p, _p, _sz, _p, _p], _i),
        "vg_eefk": ([ctypes.c_char_p, _p, _sz, _p], _i),
        "vg_filter_pointcloud_device": ([_p, _sz, _f, _f, _p, _p, _p, _i, _p, _p, _p], _i),
        "vg_filter_pointcloud": ([_p, _sz, _f, _f, _p, _p, _p, _i, _p, _p, _p], _i),
        "vg_env_pointcloud_layout": ([_p, _i, _p, _p, _p, _p, _p, _p], _i),
        "vg_env_set_mode": ([_p, _i, _i], _i),
        "vg_env_set_schedule": ([_p, _i], _i),
        "vg_mlp_set_wait_limit": ([_p, ctypes.c_longlong], _i),
        "vg_env_add_primitive": ([_p, _i, _p, _f], _i),
        "vg_env_add_pointcloud_layout": ([_p, _i, _p, _p, _p, _p, _sz, _p, _f, _f, _f], _i),
        "vg_env_add_heightfield_fields": ([_p, _p, _sz, _sz, _p], _i),
        "vg_fkcc_blocks_device": ([_s, _p, _p, _sz, _p, _p], _i),
        "vg_fkcc_blocks": ([_s, _p, _p, _sz, _p], _i),
        "vg_env_count": ([_p, _i, _p], _i),
        "vg_env_get": ([_p, _i, _sz, _p], _i),
        "vg_validate_states_device": ([_s, _p, _p, _sz, _p, _p], _i),
        "vg_validate_motions_device": ([_s, _p, _p, _p, _sz, _i, _p, _p, _p], _i),
        "vg_validate_motions_device_noalloc": ([_s, _p, _p, _p, _sz, _i, _p, _p, _p], _i),
        "vg_sphere_fk_device": ([_s, _p, _sz, _p, _p], _i),
        "vg_validate_states": ([_s, _p, _p, _sz, _p], _i),
        "vg_validate_motions": ([_s, _p, _p, _p, _sz, _i, _p], _i),
        "vg_sphere_fk": ([_s, _p, _sz, _p], _i),
        "vg_gemm_bf16_device": ([_p, _p, _p, _i, _i, _i, _p, _p], _i),
        "vg_mlp_create": ([_i, ctypes.c_uint64], _p),
        "vg_mlp_destroy": ([_p], None),
        "vg_mlp_param_count": ([_i], _sz),
        "vg_mlp_get_params": ([_p, _p], _i),
        "vg_mlp_set_params": ([_p, _p], _i),
        "vg_mlp_train_device": ([_p, _p, _p, _sz, _i, _i, _f, _p, _p], _i),
        "vg_mlp_gradients": ([_p, _p, _p, _sz, _p, _p, _p], _i),
        "vg_mlp_predict_device": ([_p, _p, _sz, _p, _p], _i),
        "vg_mlp_infer_device": ([_p, _p, _sz, _p, _p], _i),
        "vg_mlp_score_edges_device": ([_p, _p, _p, _sz, _i, _p, _p], _i),
        "vg_mlp_error": ([_p], _i),
        "vg_validate_motions_scored_device": ([_s, _p, _p, _p, _sz, _i, _p, _i, _p, _p, _p], _i),
        "vg_validate_motions_learned_device": ([_s, _p, _p, _p, _p, _sz, _i, _i, _p, _p, _p], _i),
        "vg_autotune_motions": ([_s, _p, _p, _p, _sz, _i, _p, _p, _p, _p], _i),
        "vg_debug_sizes": ([_s, _p, _p, _p, _p], _i),
        "vg_debug_device": ([_s, _p, _p, _sz, _p, _p, _p], _i),
        "vg_debug": ([_s, _p, _p, _sz, _p, _p], _i),
        "vg_batch_create": ([], _p),
        "vg_batch_destroy": ([_p], None),
        "vg_batch_add_motions": ([_p, _s, _p, _p, _p, _sz, _i, _p, _i, _p, _p], _i),
        "vg_batch_launch": ([_p, _p], _i),
        "vg_host_alloc": ([_sz], _p),
        "vg_host_free": ([_p], None),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = _load()


def check(rc: int) -> None:
    if rc != VG_OK:
        msg = lib.vg_last_error().decode(errors="replace")
        raise VampError(f"{ERRORS.get(rc, 'error')} ({rc}): {msg}")


# Symbols declared in include/vamp_gb300.h (the C-ABI test checks that each one is exported).
EXPORTED = (
    "vg_last_error",
    "vg_version",
    "vg_robot_info",
    "vg_robot_limits",
    "vg_env_create",
    "vg_env_destroy",
    "vg_env_add_sphere",
    "vg_env_add_capsule",
    "vg_env_add_cuboid",
    "vg_env_add_pointcloud",
    "vg_env_add_pointcloud_device",
    "vg_env_add_heightfield",
    "vg_validate_vectors_device",
    "vg_validate_vectors",
    "vg_filter_self_from_pointcloud_device",
    "vg_filter_self_from_pointcloud",
    "vg_env_attach",
    "vg_env_detach",
    "vg_eefk_device",
    "vg_eefk",
    "vg_filter_pointcloud_device",
    "vg_filter_pointcloud",
    "vg_env_pointcloud_layout",
    "vg_env_set_mode",
    "vg_env_set_schedule",
    "vg_env_add_primitive",
    "vg_env_add_pointcloud_layout",
    "vg_env_add_heightfield_fields",
    "vg_fkcc_blocks_device",
    "vg_fkcc_blocks",
    "vg_env_count",
    "vg_env_get",
    "vg_validate_states_device",
    "vg_validate_motions_device",
    "vg_validate_motions_device_noalloc",
    "vg_sphere_fk_device",
    "vg_validate_states",
    "vg_validate_motions",
    "vg_sphere_fk",
    "vg_gemm_bf16_device",
    "vg_mlp_create",
    "vg_mlp_destroy",
    "vg_mlp_param_count",
    "vg_mlp_get_params",
    "vg_mlp_set_params",
    "vg_mlp_train_device",
    "vg_mlp_gradients",
    "vg_mlp_predict_device",
    "vg_mlp_infer_device",
    "vg_mlp_score_edges_device",
    "vg_mlp_error",
    "vg_mlp_set_wait_limit",
    "vg_validate_motions_scored_device",
    "vg_validate_motions_learned_device",
    "vg_autotune_motions",
    "vg_debug_sizes",
    "vg_debug_device",
    "vg_debug",
    "vg_batch_create",
    "vg_batch_destroy",
    "vg_batch_add_motions",
    "vg_batch_launch",
    "vg_host_alloc",
    "vg_host_free",
)
