"""jcde — GB300-native collision detection engine for 2D irregular nesting.

A drop-in for the query path of jagua-rs's ``CDEngine``: the quadtree of hazards is mirrored into
GPU memory and detect / collect queries run as hand-written sm_103a kernels behind the C ABI of
``include/jcde.h``.  This package is the Python host side over that ABI.

Submodules: ``engine`` (CDEngine, MultiEngine, ResidentEngine), ``workload`` (seeded layouts and the
importer), ``prep`` (item preparation on the device), ``lbf`` (the LBF build, host and device
drivers), ``instance`` (strip-packing instances), ``bpp`` (bin packing), ``shards`` (replicas on
several ranks).
"""
from ._ffi import JcdeError, build, lib
from .engine import (CDEConfig, CDEngine, GpuBackend, GpuEngine, Hazard, MultiEngine, ResidentEngine, pole_overlap,
                     spolygon_new, surrogate_poles)
from .workload import QUERY_DTYPE

__all__ = [
    "CDEConfig",
    "CDEngine",
    "GpuBackend",
    "GpuEngine",
    "Hazard",
    "MultiEngine",
    "pole_overlap",
    "ResidentEngine",
    "JcdeError",
    "QUERY_DTYPE",
    "build",
    "lib",
    "spolygon_new",
    "surrogate_poles",
]
