"""Regenerate the golden fixtures in this directory.

tess_table.json : digest and sizes of the committed table blob, which
                  data/make_tess_table.py produces by compiling the reference's
                  src/tessellation_table_nv_raw.hpp unchanged (oracle/Makefile `ref`).
oracle_frames.json : digests of the oracle's outputs for small seeded frames
                  (plain, and with PN + ripple, transient builds and raster
                  batching), pinning the CPU restatement against accidental drift.

Usage: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def table_digest():
    from vk_tessellated_clusters_gb300.table import TABLE_PATH, load_raw_table
    raw = load_raw_table()
    with open(TABLE_PATH, "rb") as f:
        d = hashlib.sha256(f.read()).hexdigest()
    return {"sha256": d, "max_edge_segments": raw.max_edge_segments, "num_vertices": int(raw.vertices.size),
            "num_triangles": int(raw.triangles.size), "num_configs": raw.num_configs}


def frame_digests():
    from tests.golden.cases import CASES, VARIANTS, run_case_digest, run_variant_digest
    d = {name: run_case_digest(name) for name in CASES}
    d.update({name: run_variant_digest(name) for name in VARIANTS})
    return d


if __name__ == "__main__":
    with open(os.path.join(HERE, "tess_table.json"), "w") as f:
        json.dump(table_digest(), f, indent=1)
    with open(os.path.join(HERE, "oracle_frames.json"), "w") as f:
        json.dump(frame_digests(), f, indent=1, sort_keys=True)
    print("written")
