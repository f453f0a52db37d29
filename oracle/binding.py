"""ctypes binding of the CPU oracle (oracle/tc_oracle.h).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker. It runs the C++
restatement of the reference's shaders on host-memory copies of exactly the
inputs the CUDA library receives.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300.frame import FrameState, HostMemory
from vk_tessellated_clusters_gb300.scene import Camera, Scene, frame_constants
from vk_tessellated_clusters_gb300.table import load_raw_table, lookup_entries, synthetic_templates

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libtc_oracle.so")

N = L.TESSTABLE_LOOKUP_ENTRIES


class TcoTable(ctypes.Structure):
    _fields_ = [("entries", ctypes.c_uint16 * (4 * N)), ("templateAddresses", ctypes.c_uint64 * N),
                ("templateInstantiationSizes", ctypes.c_uint32 * N), ("vertices", ctypes.c_void_p),
                ("triangles", ctypes.c_void_p), ("numVertices", ctypes.c_uint32), ("numTriangles", ctypes.c_uint32),
                ("maxVertices", ctypes.c_uint32), ("maxTriangles", ctypes.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.check_call(["make", "-s", "-C", HERE])
        l = ctypes.CDLL(LIB)
        vp, u32, f = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float
        P = ctypes.POINTER
        l.tco_table_init.argtypes = [P(TcoTable), vp, u32, vp, u32, vp, u32, u32]
        l.tco_encode_barycentrics.argtypes = [f, f, f]
        l.tco_encode_barycentrics.restype = u32
        l.tco_decode_barycentrics.argtypes = [u32, P(ctypes.c_float)]
        l.tco_tess_factors.argtypes = [P(f), P(f), P(f), P(f), f, f, f, P(u32)]
        l.tco_get_config.argtypes = [P(u32), P(u32)]
        l.tco_get_config.restype = u32
        l.tco_split_factor.argtypes = [u32, u32]
        l.tco_split_factor.restype = u32
        l.tco_split_pass_count.argtypes = [u32]
        l.tco_split_pass_count.restype = u32
        l.tco_frame_build.argtypes = [P(TcoTable), P(L.FrameArgs), ctypes.c_int, P(u32)]
        for name in ("tco_frame_begin", "tco_instances_classify", "tco_clusters_cull", "tco_blas_setup_insertion",
                     "tco_blas_clusters_insert"):
            getattr(l, name).argtypes = [P(L.FrameArgs)]
        l.tco_build_setup.argtypes = [P(L.FrameArgs), u32]
        for name in ("tco_cluster_classify", "tco_triangle_split_pass", "tco_triangle_instantiate"):
            getattr(l, name).argtypes = [P(TcoTable), P(L.FrameArgs), ctypes.c_int]
        l.tco_generate_vertices_f64.argtypes = [P(TcoTable), P(L.FrameArgs), vp, ctypes.c_int]
        l.tco_generate_vertices_f64.restype = ctypes.c_uint64
        l.tco_generate_vertices_f64_params.argtypes = [P(TcoTable), P(L.FrameArgs), vp, vp, vp, vp]
        l.tco_generate_vertices_f64_params.restype = ctypes.c_uint64
        l.tco_backward_f64.argtypes = [P(TcoTable), P(L.FrameArgs), vp, vp, vp, vp]
        l.tco_decode_hits.argtypes = [P(TcoTable), P(L.FrameArgs), vp, u32, vp]
        l.tco_raster_batches.argtypes = [P(TcoTable), P(L.FrameArgs), P(L.RasterOutputs)]
        _lib = l
    return _lib


class Oracle:
    """The CPU restatement with the standard table and synthetic CLAS templates."""

    def __init__(self):
        self.lib = lib()
        self.raw = load_raw_table()
        self.entries = lookup_entries(self.raw)
        self.table = TcoTable()
        rc = self.lib.tco_table_init(ctypes.byref(self.table), self.raw.vertices.ctypes.data, self.raw.vertices.size,
                                     self.raw.triangles.ctypes.data, self.raw.triangles.size,
                                     self.raw.configs.ctypes.data, self.raw.num_configs, self.raw.max_edge_segments)
        if rc != 0:
            raise RuntimeError(f"tco_table_init failed ({rc})")
        addr, size = synthetic_templates(self.entries)
        ctypes.memmove(self.table.templateAddresses, addr.ctypes.data, addr.nbytes)
        ctypes.memmove(self.table.templateInstantiationSizes, size.ctypes.data, size.nbytes)

    def table_entries(self) -> np.ndarray:
        return np.frombuffer(bytes(self.table.entries), L.TessTableEntry)

    def new_state(self, scene: Scene, caps: dict, flags: int) -> FrameState:
        return FrameState(scene, HostMemory(), caps, flags)

    def frame(self, scene: Scene, camera: Camera | np.ndarray, caps: dict, flags: int = L.FLAG_CULLING,
              threads: int = 0, camera_last=None, state: FrameState | None = None):
        """Run one frame; returns (FrameState, run starts)."""
        st = state or self.new_state(scene, caps, flags)
        fc = camera if isinstance(camera, np.ndarray) else frame_constants(camera)
        fl = fc if camera_last is None else (camera_last if isinstance(camera_last, np.ndarray)
                                             else frame_constants(camera_last))
        st.set_cameras(fc, fl)
        runs = (ctypes.c_uint32 * 20)()
        rc = self.lib.tco_frame_build(ctypes.byref(self.table), ctypes.byref(st.args), threads or os.cpu_count(), runs)
        if rc != 0:
            raise RuntimeError(f"tco_frame_build failed ({rc})")
        return st, list(runs)

    def decode_hits(self, state: FrameState, hits: np.ndarray) -> np.ndarray:
        """tc_decode_hits restated on the CPU for the frame in `state`."""
        hits = np.ascontiguousarray(hits, dtype=L.Hit)
        out = np.zeros(len(hits), L.BaseHit)
        self.lib.tco_decode_hits(ctypes.byref(self.table), ctypes.byref(state.args), hits.ctypes.data, len(hits),
                                 out.ctypes.data)
        return out

    def raster_batches(self, state: FrameState) -> dict:
        """tc_raster_batches restated on the CPU for the frame in `state`."""
        ro, _ = state.raster_outputs()
        self.lib.tco_raster_batches(ctypes.byref(self.table), ctypes.byref(state.args), ctypes.byref(ro))
        return state.raster_results()

    def vertices_f64(self, state: FrameState, count: int) -> np.ndarray:
        out = np.zeros((count, 3), np.float64)
        self.lib.tco_generate_vertices_f64(ctypes.byref(self.table), ctypes.byref(state.args), out.ctypes.data, 1)
        return out
