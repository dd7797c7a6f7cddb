"""ctypes declarations of the jcde C ABI (include/jcde.h)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)
# JCDE_LIBRARY names another build of the same library (e.g. one compiled with other launch-shape
# defaults); there is no fallback to anything but a libjcde build.
LIB_PATH = os.environ.get("JCDE_LIBRARY") or os.path.join(PKG_DIR, "libjcde.so")

OK, ERR_ARG, ERR_CUDA, ERR_CAPACITY, ERR_NOT_FOUND, ERR_TIMEOUT, ERR_STATE = 0, -1, -2, -3, -4, -5, -6


class JcdeError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {_lib_status_string(status)} ({status})")


class jcde_rect(C.Structure):
    _fields_ = [("x_min", C.c_float), ("y_min", C.c_float), ("x_max", C.c_float), ("y_max", C.c_float)]


class jcde_resident_config(C.Structure):
    _fields_ = [("max_nodes", C.c_uint32), ("max_entries", C.c_uint32), ("max_edges", C.c_uint32),
                ("max_hazard_vertices", C.c_uint32), ("max_keys", C.c_uint32), ("max_tasks", C.c_uint32)]


class jcde_lbf_params(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_candidates", C.c_uint32), ("n_types", C.c_uint32),
                ("remove_every", C.c_uint32), ("max_steps", C.c_uint32), ("verdict_log_steps", C.c_uint32),
                ("uniform_rounds", C.c_uint32), ("sample_box", jcde_rect), ("ls_rounds", C.c_uint32),
                ("ls_candidates", C.c_uint32), ("ls_sigma_t", C.c_float * 8), ("ls_sigma_turns", C.c_double * 8),
                ("item_sequence", C.POINTER(C.c_uint32)), ("n_sequence", C.c_uint32),
                ("n_orientation_items", C.c_uint32), ("orientation_offsets", C.POINTER(C.c_uint32)),
                ("orientation_cs", C.POINTER(C.c_float))]


class jcde_tuning(C.Structure):
    _fields_ = [("surrogate_warp_max", C.c_uint32), ("leaf_table_max", C.c_uint32), ("poly_chunk", C.c_uint32),
                ("order_min_batch", C.c_uint32), ("surrogate_lanes", C.c_uint32), ("edge_tile", C.c_uint32),
                ("staging_depth", C.c_uint32)]


class jcde_config(C.Structure):
    _fields_ = [
        ("quadtree_depth", C.c_uint8),
        ("cd_threshold", C.c_uint8),
        ("reserved", C.c_uint8 * 2),
        ("n_pole_limits", C.c_uint32),
        ("pole_limit_n", C.c_uint32 * 3),
        ("pole_limit_coverage", C.c_float * 3),
        ("n_ff_poles", C.c_uint32),
        ("n_ff_piers", C.c_uint32),
    ]


class jcde_hazard(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("dynamic", C.c_int32),
        ("xy", C.POINTER(C.c_float)),
        ("n_vertices", C.c_uint32),
        ("poi", C.c_float * 3),
        ("tag", C.c_uint64),
    ]


class jcde_filter(C.Structure):
    _fields_ = [("ignored", C.POINTER(C.c_uint32)), ("n_ignored", C.c_uint32)]


P = C.c_void_p
f32p = C.POINTER(C.c_float)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
u8p = C.POINTER(C.c_uint8)

SIGNATURES = {
    "jcde_status_string": (C.c_char_p, [C.c_int32]),
    "jcde_default_config": (None, [C.POINTER(jcde_config)]),
    "jcde_create": (C.c_int32, [C.POINTER(jcde_config), jcde_rect, C.POINTER(jcde_hazard), C.c_uint32, C.POINTER(P)]),
    "jcde_destroy": (None, [P]),
    "jcde_bbox": (C.c_int32, [P, C.POINTER(jcde_rect)]),
    "jcde_register_hazard": (C.c_int32, [P, C.POINTER(jcde_hazard), u32p]),
    "jcde_deregister_hazard": (C.c_int32, [P, C.c_uint32]),
    "jcde_deregister_hazard_by_entity": (C.c_int32, [P, C.c_int32, C.c_uint64, u32p]),
    "jcde_n_hazard_slots": (C.c_int32, [P, u32p]),
    "jcde_register_item": (C.c_int32, [P, f32p, C.c_uint32, f32p, f32p, C.c_uint32, f32p, C.c_uint32, u32p]),
    "jcde_detect_batch": (C.c_int32, [P, P, C.c_uint32, C.POINTER(jcde_filter), P, P]),
    "jcde_detect_surrogate_batch": (C.c_int32, [P, P, C.c_uint32, C.POINTER(jcde_filter), P, P]),
    "jcde_detect_poly_batch": (C.c_int32, [P, P, C.c_uint32, C.POINTER(jcde_filter), P, P]),
    "jcde_detect_batch_host": (C.c_int32, [P, P, C.c_uint32, C.POINTER(jcde_filter), P]),
    "jcde_collect_batch": (C.c_int32, [P, P, C.c_uint32, C.POINTER(jcde_filter), P, P, P, C.c_uint32, P, P]),
    "jcde_detect_batch_noalloc": (C.c_int32, [P, P, C.c_uint32, C.POINTER(jcde_filter), P, P]),
    "jcde_detect_poly": (C.c_int32, [P, f32p, C.c_uint32, f32p, C.POINTER(jcde_filter), u8p]),
    "jcde_detect_surrogate": (C.c_int32, [P, C.c_uint32, f32p, C.POINTER(jcde_filter), u8p]),
    "jcde_collect_poly": (C.c_int32, [P, f32p, C.c_uint32, f32p, C.POINTER(jcde_filter), u32p, C.c_uint32, u32p]),
    "jcde_collect_surrogate": (C.c_int32, [P, C.c_uint32, f32p, C.POINTER(jcde_filter), u32p, C.c_uint32, u32p]),
    "jcde_save": (C.c_int32, [P, C.POINTER(P)]),
    "jcde_restore": (C.c_int32, [P, P]),
    "jcde_snapshot_free": (None, [P]),
    "jcde_spolygon_new": (C.c_int32, [f32p, C.c_uint32, f32p, f32p, f32p, f32p]),
    "jcde_surrogate_poles": (C.c_int32, [f32p, C.c_uint32, C.c_float, f32p, C.POINTER(jcde_config), f32p, C.c_uint32, u32p]),
    "jcde_close_concavities": (C.c_int32, [f32p, C.c_uint32, C.c_int, C.c_float, f32p, u32p]),
    "jcde_spolygon_batch": (C.c_int32, [f32p, u32p, C.c_uint32, f32p, f32p, f32p, P, P, C.c_uint32]),
    "jcde_simplify_batch": (C.c_int32, [P, P, C.c_uint32, C.c_uint32, P, C.c_int, C.c_float, P, P, P, P]),
    "jcde_gen_candidates": (C.c_int32, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, jcde_rect, P, C.c_uint32, P, P, P]),
    "jcde_gen_candidates_segments": (C.c_int32, [C.c_uint64, P, P, C.c_uint32, C.c_uint32, C.c_uint32, P, C.c_uint32, P,
                                                 P, P]),
    "jcde_lbf_select_segments": (C.c_int32, [P, P, P, C.c_uint32, C.c_uint32, P, P]),
    "jcde_poles_workspace_bytes": (C.c_uint64, [C.c_uint32, C.c_uint32, C.c_int]),
    "jcde_poi_batch": (C.c_int32, [P, P, C.c_uint32, C.c_uint32, P, P, P, P, C.c_uint64, P]),
    "jcde_surrogate_poles_batch": (C.c_int32, [P, P, C.c_uint32, C.c_uint32, P, P, C.POINTER(jcde_config), P, C.c_uint32,
                                               P, P, P, P, C.c_uint64, P]),
    "jcde_tree_dump": (C.c_int32, [P, u32p, C.c_uint64, u64p]),
    "jcde_device_stats": (C.c_int32, [P, u64p]),
    "jcde_kernel_launches": (C.c_uint64, [P]),
    "jcde_l2_read_peak": (C.c_int32, [C.c_uint64, C.c_uint32, C.POINTER(C.c_double)]),
    "jcde_profile_enable": (C.c_int32, [P, C.c_int]),
    "jcde_multi_create": (C.c_int32, [C.POINTER(P), C.c_uint32, C.POINTER(P)]),
    "jcde_set_hazard_poles": (C.c_int32, [P, C.c_uint32, f32p, C.c_uint32]),
    "jcde_resident_default_config": (None, [P]),
    "jcde_resident_create": (C.c_int32, [P, P, P]),
    "jcde_resident_destroy": (None, [P]),
    "jcde_resident_reset": (C.c_int32, [P, C.POINTER(C.c_uint64)]),
    "jcde_resident_register_placed": (C.c_int32, [P, P, P, P]),
    "jcde_resident_deregister": (C.c_int32, [P, P, P]),
    "jcde_resident_detect_batch": (C.c_int32, [P, P, C.c_uint32, P, P]),
    "jcde_resident_status": (C.c_int32, [P, u32p]),
    "jcde_resident_tree_dump": (C.c_int32, [P, u32p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "jcde_resident_kernel_launches": (C.c_uint64, [P]),
    "jcde_lbf_begin": (C.c_int32, [P, P]),
    "jcde_lbf_steps": (C.c_int32, [P, C.c_uint32, C.c_uint32, P]),
    "jcde_lbf_read": (C.c_int32, [P, u32p, u32p, C.c_uint32, u32p, C.c_uint32, u32p, C.c_uint32, P, C.c_uint64]),
    "jcde_lbf_select": (C.c_int32, [P, P, P, C.c_uint32, P, P]),
    "jcde_get_tuning": (C.c_int32, [P, P]),
    "jcde_set_tuning": (C.c_int32, [P, P]),
    "jcde_autotune": (C.c_int32, [P, P, C.c_uint32, P, P, P, C.POINTER(C.c_double)]),
    "jcde_multi_autotune": (C.c_int32, [P, P, u32p, P, P, P, u32p, C.POINTER(C.c_double)]),
    "jcde_proxy_forward": (C.c_int32, [P, P, P, C.c_uint32, P, P, P]),
    "jcde_proxy_backward": (C.c_int32, [P, P, P, C.c_uint32, P, P, P, P]),
    "jcde_proxy_batch": (C.c_int32, [P, P, P, C.c_uint32, C.POINTER(jcde_filter), P, P, P]),
    "jcde_separate_batch": (C.c_int32, [P, P, P, C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, C.POINTER(jcde_filter), P, P, P]),
    "jcde_resample_batch": (C.c_int32, [P, P, P, C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_uint32, P, P]),
    "jcde_multi_destroy": (None, [P]),
    "jcde_multi_detect": (C.c_int32, [P, P, u32p, C.POINTER(jcde_filter), P, P]),
    "jcde_multi_detect_graph": (C.c_int32, [P, P, u32p, C.POINTER(jcde_filter), P, P]),
    "jcde_multi_kernel_launches": (C.c_uint64, [P]),
    "jcde_profile_read": (C.c_int32, [P, C.POINTER(C.c_double), u64p, C.c_int]),
}

_lib = None


def build(force: bool = False, jobs: int = 3) -> str:
    """Compile libjcde.so in-tree with the package Makefile (nvcc for sm_103a + g++)."""
    args = ["make", "-s", f"-j{jobs}", "-C", ROOT_DIR]
    if force:
        subprocess.run(["make", "-s", "-C", ROOT_DIR, "clean"], check=True)
    subprocess.run(args, check=True)
    return LIB_PATH


def lib():
    """The loaded jcde library.  Raises if it was not built: there is no fallback path."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libjcde.so not built ({LIB_PATH}); run jcde.build() or `make -C jagua-rs_gb300`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _lib_status_string(s: int) -> str:
    try:
        return lib().jcde_status_string(s).decode()
    except Exception:  # library not loadable: only the numeric code is known
        return "status"


def check(status: int, what: str) -> None:
    if status != OK:
        raise JcdeError(status, what)
