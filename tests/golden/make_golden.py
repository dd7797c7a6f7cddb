"""Writes the golden fixtures of tests/golden/ from the oracle (the CPU restatement of the
reference CDE): small seeded cases whose expected outputs the CUDA path must reproduce without the
oracle at hand, and that pin the oracle itself against regressions.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "jagua-rs_gb300")]

from jcde import bpp, lbf  # noqa: E402
from jcde import workload as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

N_QUERIES = 65536
N_COLLECT = 4096
SIMPLIFY_TOLS = (0.01, 0.05)


def prep_shapes():
    """Six star items of 8-200 vertices, a rectangle and an L: the shapes of the preparation cases."""
    st = W.Stream(0x601D, 1)
    out = [W.star_polygon(st, int(st.randint(8, 200, 1)[0]), 20.0, 60.0) for _ in range(6)]
    out.append(W.rect_polygon(5.0, -3.0, 45.0, 22.0))
    out.append(np.array([[0, 0], [60, 0], [60, 20], [20, 20], [20, 50], [0, 50]], np.float32))
    return out


def lbf_spec():
    return lbf.LbfSpec(n_types=12, n_cand=512, steps=60, remove_every=20, uniform_rounds=1)


def bpp_case():
    return bpp.load_bpp(bpp.synthetic_instance(n_types=6, n_bins=2)), bpp.BppSpec(n_cand=512)


def tree_hash(dump: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(dump, dtype=np.uint32).tobytes()).hexdigest()


def main():
    O.build()
    B = O.OracleBackend
    out = {}
    # the CPU-runnable strip layout (seed 0xC0): placements, verdicts of 65,536 queries, collect sets
    lay, eng = W.strip_layout(B)
    pl = [h.placement for h in lay.hazards if h.placement is not None]
    out["strip_placements"] = np.array([[p[0], *[np.float32(x).view(np.uint32) for x in p[1:]]] for p in pl],
                                       dtype=np.uint32)
    q = W.queries_for(lay, N_QUERIES, 0xC0)
    out["strip_verdicts"] = np.packbits(eng.detect_batch(q))
    counts, ids = eng.collect_batch(q[:N_COLLECT])
    out["strip_collect_counts"] = counts.astype(np.uint32)
    out["strip_collect_ids"] = ids.astype(np.uint32)
    out["strip_tree_sha256"] = np.frombuffer(bytes.fromhex(tree_hash(eng.tree_dump())), dtype=np.uint8)
    # item preparation: poi, surrogate poles, simplification (both modes)
    for i, raw in enumerate(prep_shapes()):
        it = W.import_item(B, raw)
        out[f"prep{i}_poi"] = it.poi
        out[f"prep{i}_poles"] = it.poles
        xy, _, area, _, _ = B.spolygon_new(raw)
        for tol in SIMPLIFY_TOLS:
            for deflate in (0, 1):
                out[f"simp{i}_{tol}_{deflate}"] = B.simplify_shape(xy, area, bool(deflate), tol)
    # a short LBF build (removals every 20 steps)
    spec = lbf_spec()
    lay_l, eng_l = lbf.setup(B, spec)
    log = lbf.run_host(lay_l, eng_l, spec)
    out["lbf_placements"], out["lbf_removals"], out["lbf_free_counts"] = log.placements, log.removals, log.free_counts
    # a small bin-packing solve
    inst, bspec = bpp_case()
    blog = bpp.run_bpp(B, bpp.setup_bpp(B, inst), bspec)
    out["bpp_placements"] = blog.placements
    out["bpp_layouts"] = np.array(blog.layouts, dtype=np.uint32)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(out)} arrays to tests/golden/golden.npz")


if __name__ == "__main__":
    main()
