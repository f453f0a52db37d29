"""The NVIDIA tessellation table (11 segments per edge) used by the pipeline.

``data/tess_table_nv.bin`` holds the reference's generated table
(src/tessellation_table_nv_raw.hpp) in a small binary container
(see data/make_tess_table.py): 7059 packed barycentric vertices, 8398 packed
triangles and 286 configs. The lookup expansion (src/tessellation_table.cpp:36-83)
is done by the C ABI (tc_table_init); ``lookup_entries`` restates it in numpy
for host-side bookkeeping.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

from . import layouts as L

TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tess_table_nv.bin")
MAGIC = 0x42544354


@dataclass
class RawTable:
    max_edge_segments: int
    vertices: np.ndarray  # uint32
    triangles: np.ndarray  # uint32
    configs: np.ndarray  # uint16, 4 per config

    @property
    def num_configs(self) -> int:
        return self.configs.size // 4


def load_raw_table(path: str = TABLE_PATH) -> RawTable:
    with open(path, "rb") as f:
        data = f.read()
    hdr = np.frombuffer(data, "<u4", 6)
    if hdr[0] != MAGIC or hdr[1] != 1:
        raise ValueError(f"{path}: not a tessellation table container")
    mes, nv, nt, nc = (int(x) for x in hdr[2:6])
    off = 24
    verts = np.frombuffer(data, "<u4", nv, off).copy()
    off += 4 * nv
    tris = np.frombuffer(data, "<u4", nt, off).copy()
    off += 4 * nt
    cfgs = np.frombuffer(data, "<u2", 4 * nc, off).copy()
    off += 8 * nc
    if off != len(data):
        raise ValueError(f"{path}: trailing bytes")
    return RawTable(mes, verts, tris, cfgs)


def lookup_index(x: int, y: int, z: int) -> int:
    Ls = L.TESSTABLE_LOOKUP_SIZE
    return x + y * Ls + z * Ls * Ls - (1 + Ls + Ls * Ls)


def lookup_entries(raw: RawTable) -> np.ndarray:
    """16^3 lookup of TessTableEntry including the permuted (flipped) configs."""
    e = np.zeros(L.TESSTABLE_LOOKUP_ENTRIES, L.TessTableEntry)
    c = raw.configs.reshape(-1, 4)
    ci = 0
    for x in range(1, raw.max_edge_segments + 1):
        for y in range(1, x + 1):
            for z in range(1, y + 1):
                rec = tuple(int(v) for v in c[ci])
                e[lookup_index(x, y, z)] = rec
                if z != y and x > 1:
                    e[lookup_index(x, z, y)] = rec
                ci += 1
    return e


def synthetic_templates(entries: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Per lookup entry CLAS template address and worst-case instantiation size.
    In the reference these come from building one CLAS template per config
    (src/tessellation_table.cpp:102-404), which is outside the tessellation
    path; deterministic stand-ins keep the instantiation arguments checkable."""
    idx = np.arange(L.TESSTABLE_LOOKUP_ENTRIES, dtype=np.uint64)
    addr = np.uint64(0x7E00_0000_0000) + idx * np.uint64(4096)
    nt = entries["numTriangles"].astype(np.uint32)
    size = np.where(nt > 0, 128 + 40 * nt, 0).astype(np.uint32)
    return addr, size
