"""The C ABI: library loads, exports every declared entry point, rejects bad arguments.

Only host-side entry points run here (no GPU is needed to create an engine, register hazards or
prepare shapes); every query entry point is exercised by the GPU tests.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO


def declared_functions():
    src = open(os.path.join(REPO, "include", "jcde.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jcde_[a-z0-9_]+)\s*\(", src)))


def test_header_parses():
    names = declared_functions()
    assert "jcde_detect_batch" in names and "jcde_create" in names and len(names) >= 25


def test_exports_every_declared_symbol(jcde_mod):
    L = C.CDLL(os.path.join(REPO, "jagua-rs_gb300", "jcde", "libjcde.so"))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(jcde_mod):
    from jcde import _ffi

    assert set(declared_functions()) == set(_ffi.SIGNATURES), set(declared_functions()) ^ set(_ffi.SIGNATURES)


def test_status_strings(jcde_mod):
    L = jcde_mod.lib()
    assert L.jcde_status_string(0) == b"ok"
    assert L.jcde_status_string(-4) == b"not found"


def test_bad_arguments(jcde_mod):
    from jcde import _ffi

    L = jcde_mod.lib()
    cfg = _ffi.jcde_config()
    L.jcde_default_config(C.byref(cfg))
    h = C.c_void_p()
    # empty box
    assert L.jcde_create(C.byref(cfg), _ffi.jcde_rect(0, 0, 0, 1), None, 0, C.byref(h)) == _ffi.ERR_ARG
    # depth beyond the 15 levels the kernels track
    cfg.quadtree_depth = 16
    assert L.jcde_create(C.byref(cfg), _ffi.jcde_rect(0, 0, 1, 1), None, 0, C.byref(h)) == _ffi.ERR_ARG
    cfg.quadtree_depth = 5
    assert L.jcde_create(C.byref(cfg), _ffi.jcde_rect(0, 0, 1, 1), None, 0, C.byref(h)) == _ffi.OK
    # a hazard needs >= 3 vertices; unknown keys are reported, never abort
    hz = _ffi.jcde_hazard()
    hz.kind = 0
    hz.n_vertices = 2
    xy = np.zeros(4, np.float32)
    hz.xy = xy.ctypes.data_as(C.POINTER(C.c_float))
    k = C.c_uint32()
    assert L.jcde_register_hazard(h, C.byref(hz), C.byref(k)) == _ffi.ERR_ARG
    assert L.jcde_deregister_hazard(h, 7) == _ffi.ERR_NOT_FOUND
    assert L.jcde_detect_batch(None, None, 0, None, None, None) == _ffi.ERR_ARG
    L.jcde_destroy(h)


def test_engine_default_config_matches_lbf(jcde_mod):
    """lbf/src/config.rs:37-45."""
    from jcde import _ffi

    cfg = _ffi.jcde_config()
    jcde_mod.lib().jcde_default_config(C.byref(cfg))
    assert (cfg.quadtree_depth, cfg.cd_threshold, cfg.n_ff_poles, cfg.n_ff_piers) == (5, 16, 2, 0)
    assert list(cfg.pole_limit_n) == [100, 20, 10]
    assert [round(v, 2) for v in cfg.pole_limit_coverage] == [0.0, 0.75, 0.9]


def test_python_engine_errors(jcde_mod):
    eng = jcde_mod.CDEngine((0, 0, 10, 10))
    with pytest.raises(KeyError):
        eng.deregister_hazard_by_key(3)
    with pytest.raises(KeyError):
        eng.deregister_hazard_by_entity(0, 12345)


def test_tuning_round_trip(jcde_mod):
    eng = jcde_mod.CDEngine((0.0, 0.0, 100.0, 100.0))
    t = eng.get_tuning()
    assert t["surrogate_warp_max"] == 1 << 17 and t["poly_chunk"] == 2
    eng.set_tuning(poly_chunk=4, order_min_batch=0xFFFFFFFF)
    t2 = eng.get_tuning()
    assert t2["poly_chunk"] == 4 and t2["order_min_batch"] == 0xFFFFFFFF
    assert t2["surrogate_warp_max"] == t["surrogate_warp_max"]


def test_batch_prep_and_generator_arguments(jcde_mod):
    """The device batch entry points of item preparation, simplification and candidate generation
    check their arguments before any CUDA call: null buffers and bad sizes are JCDE_ERR_ARG, empty
    batches succeed without touching the device."""
    from jcde._ffi import jcde_config, jcde_rect, lib

    L = lib()
    ARG = -1
    cfg = jcde_config()
    L.jcde_default_config(C.byref(cfg))
    # empty batches
    assert L.jcde_poi_batch(None, None, 0, 3, None, None, None, None, 0, None) == 0
    assert L.jcde_surrogate_poles_batch(None, None, 0, 3, None, None, C.byref(cfg), None, 1, None, None, None, None, 0,
                                        None) == 0
    assert L.jcde_simplify_batch(None, None, 0, 3, None, 0, 0.001, None, None, None, None) == 0
    assert L.jcde_gen_candidates(1, 2, 0, 0, jcde_rect(0, 0, 1, 1), None, 0, None, None, None) == 0
    assert L.jcde_poles_workspace_bytes(0, 8, 1) == 0
    # null buffers, bad sizes, bad config
    assert L.jcde_poi_batch(None, None, 4, 8, None, None, None, None, 0, None) == ARG
    assert L.jcde_surrogate_poles_batch(None, None, 4, 8, None, None, None, None, 1, None, None, None, None, 0,
                                        None) == ARG
    bad = jcde_config()
    L.jcde_default_config(C.byref(bad))
    bad.n_pole_limits = 4
    assert L.jcde_surrogate_poles_batch(None, None, 0, 3, None, None, C.byref(bad), None, 1, None, None, None, None, 0,
                                        None) == ARG
    assert L.jcde_simplify_batch(None, None, 4, 8, None, 0, 0.001, None, None, None, None) == ARG
    assert L.jcde_gen_candidates(1, 2, 16, 0, jcde_rect(0, 0, 1, 1), None, 0, None, None, None) == ARG
    assert L.jcde_gen_candidates(1, 2, 16, 0, jcde_rect(1, 0, 1, 1), None, 0, 1024, None, None) == ARG   # empty box
    assert L.jcde_gen_candidates(1, 2, 16, 0, jcde_rect(0, 0, 1, 1), None, 3, 1024, None, None) == ARG   # no table
    # the host batch of SPolygon::new: status per shape, no CUDA
    xy = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [0, 0], [1, 0], [0, 0]], np.float32)
    off = np.array([0, 4, 7], np.uint32)
    out = np.zeros_like(xy)
    bb = np.zeros((2, 4), np.float32)
    ad = np.zeros((2, 2), np.float32)
    st = np.zeros(2, np.int32)
    f32p, u32p = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
    assert L.jcde_spolygon_batch(xy.ctypes.data_as(f32p), off.ctypes.data_as(u32p), 2, out.ctypes.data_as(f32p),
                                 bb.ctypes.data_as(f32p), ad.ctypes.data_as(f32p), None, C.c_void_p(st.ctypes.data),
                                 1) == 0
    assert st.tolist() == [0, ARG] and ad[0, 0] == 1.0


def test_tuning_values_are_checked(jcde_mod):
    """jcde_set_tuning rejects edge tiles, lane counts and staging depths outside the allowed sets."""
    import jcde

    eng = jcde.CDEngine((0.0, 0.0, 100.0, 100.0), (), jcde.CDEConfig())
    t = eng.get_tuning()
    assert t["edge_tile"] == 8 and t["surrogate_lanes"] == 32 and t["staging_depth"] == 0
    for bad in ({"edge_tile": 5}, {"surrogate_lanes": 4}, {"staging_depth": 5}):
        with pytest.raises(jcde.JcdeError):
            eng.set_tuning(**bad)
    eng.set_tuning(edge_tile=16, surrogate_lanes=8, staging_depth=3)
    assert eng.get_tuning()["edge_tile"] == 16
