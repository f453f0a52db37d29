"""The tessellation table: pinned to the reference's generated header and its
documented facts (README.md:30-92), and the 16^3 lookup expansion
(src/tessellation_table.cpp:52-83)."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300.table import TABLE_PATH, load_raw_table, lookup_entries, lookup_index

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "tess_table.json")
REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_table_dump")


@pytest.fixture(scope="module")
def raw():
    return load_raw_table()


def test_blob_matches_golden_digest(raw):
    with open(GOLDEN) as f:
        g = json.load(f)
    with open(TABLE_PATH, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == g["sha256"]
    assert raw.max_edge_segments == g["max_edge_segments"] == 11
    assert raw.vertices.size == g["num_vertices"] == 7059
    assert raw.triangles.size == g["num_triangles"] == 8398
    assert raw.num_configs == g["num_configs"] == 286


def test_blob_equals_reference_header_compiled(tmp_path):
    """Compile the reference's own header unchanged (oracle/Makefile target
    `ref`; skipped where the reference checkout is absent) and compare its arrays."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, capture_output=True)
    if not os.path.exists(REF_DUMP):
        pytest.skip("reference checkout absent: oracle/_ref/ref_table_dump not built")
    out = tmp_path / "ref.bin"
    subprocess.check_call([REF_DUMP, str(out)], stdout=subprocess.DEVNULL)
    with open(TABLE_PATH, "rb") as f:
        assert out.read_bytes() == f.read()


def test_readme_facts(raw):
    # README.md:41-46: the first (unsubdivided) triangle's uvs (0,0),(1,0),(0,1)
    assert list(raw.vertices[:3]) == [0x00000000, 0x00008000, 0x80000000]
    # README.md:52-53: the first triangle's indices [0,1,2]
    assert raw.triangles[0] == 0x00020100
    cfg = raw.configs.reshape(-1, 4)
    # README.md:83-85: all configs <= (2,2,2) have <= 4 triangles / <= 6 vertices
    small = [lookup_entries(raw)[lookup_index(x, y, z)] for x, y, z in [(1, 1, 1), (2, 1, 1), (2, 2, 1), (2, 2, 2)]]
    assert all(e["numTriangles"] <= 4 and e["numVertices"] <= 6 for e in small)
    # tessellation_table_nv_raw.hpp:2309-2310: config 285 (11,11,11) has 121 triangles / 78 vertices
    assert tuple(cfg[285][2:]) == (121, 78)
    # config 3 is (2,2,2): 4 triangles / 6 vertices
    assert tuple(cfg[3][2:]) == (4, 6)


def test_configs_partition_the_arrays(raw):
    cfg = raw.configs.reshape(-1, 4).astype(np.int64)
    assert cfg[0, 0] == 0 and cfg[0, 1] == 0
    assert np.all(cfg[1:, 0] == cfg[:-1, 0] + cfg[:-1, 2])
    assert np.all(cfg[1:, 1] == cfg[:-1, 1] + cfg[:-1, 3])
    assert cfg[-1, 0] + cfg[-1, 2] == raw.triangles.size
    assert cfg[-1, 1] + cfg[-1, 3] == raw.vertices.size


def test_pattern_geometry(raw):
    """Every pattern indexes its own vertices, covers the unit triangle exactly
    (signed areas in 2^-15 units sum to the whole) and keeps its corners."""
    cfg = raw.configs.reshape(-1, 4)
    for ft, fv, nt, nv in cfg:
        v = raw.vertices[fv:fv + nv]
        u, w = (v & 0xFFFF).astype(np.int64), (v >> 16).astype(np.int64)
        assert np.all(u + w <= L.TESSTABLE_COORD_MAX)
        t = raw.triangles[ft:ft + nt]
        idx = np.stack([t & 0xFF, (t >> 8) & 0xFF, (t >> 16) & 0xFF], 1).astype(np.int64)
        assert idx.max() < nv
        a = (u[idx[:, 1]] - u[idx[:, 0]]) * (w[idx[:, 2]] - w[idx[:, 0]]) - (w[idx[:, 1]] - w[idx[:, 0]]) * (
            u[idx[:, 2]] - u[idx[:, 0]])
        assert np.all(a > 0)  # counter-clockwise, non-degenerate
        assert a.sum() == L.TESSTABLE_COORD_MAX ** 2
        corners = set(zip(u.tolist(), w.tolist()))
        assert {(0, 0), (L.TESSTABLE_COORD_MAX, 0), (0, L.TESSTABLE_COORD_MAX)} <= corners


def test_lookup_expansion_matches_oracle(raw, oracle):
    np_entries = lookup_entries(raw)
    assert np.array_equal(np_entries, oracle.table_entries())
    # every factor triple in [1,11]^3 reaches a filled entry after the config rotation
    from oracle.binding import lib
    import ctypes
    for x in range(1, 12):
        for y in range(1, 12):
            for z in range(1, 12):
                f = (ctypes.c_uint32 * 3)(x, y, z)
                tv = (ctypes.c_uint32 * 3)(0, 1, 2)
                c = lib().tco_get_config(f, tv)
                e = np_entries[c & 0x7FFF]
                assert e["numTriangles"] > 0, (x, y, z)


def test_lookup_permuted_entries(raw):
    e = lookup_entries(raw)
    cfg = raw.configs.reshape(-1, 4)
    ci = 0
    for x in range(1, 12):
        for y in range(1, x + 1):
            for z in range(1, y + 1):
                assert tuple(e[lookup_index(x, y, z)]) == tuple(cfg[ci])
                if z != y and x > 1:
                    assert tuple(e[lookup_index(x, z, y)]) == tuple(cfg[ci])
                ci += 1
    filled = np.count_nonzero(e["numTriangles"])
    assert filled == 286 + sum(1 for x in range(2, 12) for y in range(1, x + 1) for z in range(1, y) if z != y)
