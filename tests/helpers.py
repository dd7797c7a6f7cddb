"""Helpers shared by the test modules: a GPU engine holding a layout, batch calls on the GPU
engine, and CSR key lists as per-query lists."""
import os

import numpy as np

import jcde
from jcde import workload as W


# The reference's own instance files (its assets/ directory), read in place by a few CPU tests when
# this variable names that directory; the tests skip otherwise.
REFERENCE_ASSETS = os.environ.get("JCDE_REFERENCE_ASSETS", "")


def reference_asset(name: str) -> str:
    """Path of one of the reference's asset files, or "" when the directory is not given."""
    return os.path.join(REFERENCE_ASSETS, name) if REFERENCE_ASSETS else ""


def torch_queries(q):
    import torch

    return torch.from_numpy(np.ascontiguousarray(q, dtype=W.QUERY_DTYPE).view(np.uint8).copy()).cuda()


def gpu_engine(lay):
    """A fresh GPU engine with the layout's item types and hazards (keys checked against the layout)."""
    eng = jcde.CDEngine(lay.cde_bbox, (), jcde.CDEConfig(quadtree_depth=lay.depth, cd_threshold=lay.cd_threshold))
    for it in lay.items:
        eng.register_item(it.xy, it.poi, it.poles)
    for hz in lay.hazards:
        assert eng.register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag)) == hz.key
    return eng


def gpu_detect(eng, q, filter=None, mode="both"):
    import torch

    out = eng.detect_batch(torch_queries(q), filter=filter, mode=mode)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def gpu_collect(eng, q, filter=None):
    off, cnt, ids, total = eng.collect_batch(torch_queries(q), filter=filter)
    off, cnt, ids = off.cpu().numpy(), cnt.cpu().numpy(), ids.cpu().numpy()
    return [ids[o : o + c].tolist() for o, c in zip(off, cnt)]


def csr_lists(counts, ids):
    """(counts, ids) CSR -> list of per-query key lists."""
    out, o = [], 0
    ids = np.asarray(ids)
    for c in np.asarray(counts):
        out.append(ids[o : o + c].tolist())
        o += int(c)
    return out
