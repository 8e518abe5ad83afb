"""ctypes binding of libmrmg_gb300.so (the C ABI declared in include/mrmg_gb300.h).

The library is the only compute path: if it is missing, importing a GPU entry
point raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libmrmg_gb300.so"

MRMG_OK = 0
MRMG_ERR_ARG = -1
MRMG_ERR_CUDA = -2
MRMG_ERR_TIMEOUT = -3
MRMG_ERR_UNSUPPORTED = -4
MRMG_ERR_N_START = -5
MRMG_ERR_HOST = -6
MRMG_MAX_STORE_MODES = 1 << 20

MRMG_F32 = 0
MRMG_F64 = 1
MRMG_FLAG_ASYNC = 1
MRMG_FLAG_FULL_EVAL = 2
MRMG_FLAG_BATCH_FORM = 4
MRMG_NOALLOC_MAX_EDGES = 16384

METRICS = {"euclidean": 0, "sum_euclidean": 1, "max_euclidean": 2, "max": 3}
COST_METRICS = {"euclidean": 0, "max": 1}
REDUCTIONS = {"max": 0, "sum": 1}

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
f64 = C.c_double
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_f64 = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol of include/mrmg_gb300.h
SIGNATURES: dict[str, tuple] = {
    "mrmg_version": (C.c_char_p, []),
    "mrmg_last_error": (C.c_char_p, []),
    "mrmg_abstract_scene_create": (i32, [i32, i32, i32, vp, vp, vp, vp, i32, vp, vp, i32, vp, vp, vp, C.POINTER(vp)]),
    "mrmg_arm_scene_create": (i32, [i32, i32, vp, vp, vp, vp, vp, i32, vp, vp, vp, vp, i32, vp, vp, f64, C.POINTER(vp)]),
    "mrmg_scene_destroy": (i32, [vp]),
    "mrmg_scene_info": (i32, [vp, vp, vp]),
    "mrmg_table_stage_timeouts": (i32, [vp]),
    "mrmg_host_access": (i32, [vp]),
    "mrmg_serving_gather": (i32, [vp, i32, i32, i64, i64, vp, vp, vp, vp, vp]),
    "mrmg_arm_total_penetration": (i32, [vp, vp, i32, i64, vp, vp]),
    "mrmg_scene_set_tuning": (i32, [vp, i32, i32, i32, i32]),
    "mrmg_scene_get_tuning": (i32, [vp, vp]),
    "mrmg_scene_set_launch": (i32, [vp, i32, i32]),
    "mrmg_arm_scene_tune_order": (i32, [vp, vp, i32, i64, vp, vp]),
    "mrmg_is_collision_free_batch": (i32, [vp, vp, i32, i64, vp, vp, i32]),
    "mrmg_is_collision_free_batch_robots": (i32, [vp, vp, i32, i64, C.c_uint32, vp, vp, i32]),
    "mrmg_is_edge_collision_free_batch": (i32, [vp, vp, vp, i32, i64, f64, i32, vp, i64, i64, vp, vp, i32]),
    "mrmg_is_edge_collision_free_batch_noalloc": (i32, [vp, vp, vp, i32, i64, f64, i32, vp, i64, i64, vp, vp, i32]),
    "mrmg_is_collision_free_host": (i32, [vp, vp, i32, i64, C.c_uint32, vp, i32]),
    "mrmg_is_edge_collision_free_host": (i32, [vp, vp, vp, i32, i64, f64, i32, vp, i64, i64, vp, i32]),
    "mrmg_arm_sphere_centers": (i32, [vp, vp, i32, i64, vp, vp, vp]),
    "mrmg_path_penetration": (i32, [vp, vp, i64, i32, vp, vp, vp, vp, vp, i32, vp, i32]),
    "mrmg_penetration_info": (i32, [vp, vp]),
    "mrmg_last_call_stats": (i32, [vp, vp]),
    "mrmg_scene_error_word": (i32, [vp, vp]),
    "mrmg_scene_reserve": (i32, [vp, i64, vp]),
    "mrmg_status_from_error_bits": (i32, [i32]),
    "mrmg_arm_slot_map": (i32, [vp, vp, i64]),
    "mrmg_binary_search_indices": (i32, [i64, vp, i32, vp]),
    "mrmg_config_dist_matrix": (i32, [vp, i64, vp, i64, i32, vp, i32, i32, vp, vp, i32]),
    "mrmg_batch_config_cost": (i32, [vp, vp, i64, i32, vp, i32, i32, i32, f64, i32, vp, vp, i32]),
    "mrmg_microbench_fma": (i32, [i32, i64, vp, vp]),
    "mrmg_knn_exact": (i32, [vp, i64, vp, vp, vp, i32, vp, i32, i32, i32, vp, vp, vp, i32]),
    "mrmg_selftest_umma": (i32, [vp, vp, i32, vp, vp]),
    "mrmg_node_store_create": (i32, [vp, i64, i32, vp, i32, vp, i32, i32, C.POINTER(vp), vp]),
    "mrmg_node_store_destroy": (i32, [vp]),
    "mrmg_knn": (i32, [vp, vp, i64, vp, i32, vp, vp, vp, vp]),
    "mrmg_near": (i32, [vp, vp, i64, vp, vp, f64, vp, vp, vp, i64, vp, vp]),
    "mrmg_near_fetch": (i32, [vp, vp, vp, i64, vp]),
    "mrmg_arm_scene_set_modes": (i32, [vp, i32, vp, vp, vp, vp, vp]),
    "mrmg_scene_set_mode": (i32, [vp, i32]),
    "mrmg_arm_scene_set_joint_offsets": (i32, [vp, vp]),
    "mrmg_node_store_append": (i32, [vp, i32, vp, i64, vp]),
    "mrmg_node_store_info": (i32, [vp, i32, vp]),
    "mrmg_node_store_set_path": (i32, [vp, i32]),
    "mrmg_node_store_remove": (i32, [vp, i32, i64, vp]),
}


class Gb300Error(RuntimeError):
    """A CUDA or library failure reported by libmrmg_gb300."""


_lib = None


def load() -> C.CDLL:
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH.name} is not built; run __graft_entry__.build() (nvcc, sm_103a). "
            "There is no CPU fallback for the GB300 backend."
        )
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(SIGNATURES)


def check(rc: int, what: str = "") -> int:
    """Map a status code to the reference's exception types."""
    if rc >= 0:
        return rc
    msg = load().mrmg_last_error().decode(errors="replace")
    if what:
        msg = f"{what}: {msg}"
    if rc == MRMG_ERR_N_START:
        raise AssertionError(msg)          # abstract_env.py:325-326 asserts
    if rc == MRMG_ERR_ARG:
        raise ValueError(msg)
    if rc == MRMG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == MRMG_ERR_HOST:
        raise MemoryError(msg)
    raise Gb300Error(msg)


def ptr(t) -> int:
    """Device (or host) address of a torch tensor / numpy array."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


_raw_stream = None


def stream_handle(stream=None) -> int:
    """The cudaStream_t of `stream`, or of the current device's current
    stream.  The current one comes from torch's raw-stream accessor (no
    Python stream object is built: 0.1 us against 3 us for
    torch.cuda.current_stream() on a GB300 host), where torch has it."""
    global _raw_stream
    if stream is not None:
        return stream.cuda_stream
    import torch

    if _raw_stream is None:
        _raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", False)
    if _raw_stream:
        return _raw_stream(torch.cuda.current_device())
    return torch.cuda.current_stream().cuda_stream
