"""ctypes binding of the C ABI (include/tc_tessellation.h) of libtc_gb300.so.

This is the Python-side stub a maintainer would bind the library with; it
fails loudly when the library was not built (there is no CPU fallback for the
product path).
"""
from __future__ import annotations

import ctypes
import os

from . import layouts as L

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libtc_gb300.so")

_lib = None


class TcError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        msg = lib().tc_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})")


def _bind(lib):
    u32, u64, vp = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p
    st = ctypes.c_int
    sig = {
        "tc_version": (ctypes.c_char_p, []),
        "tc_status_string": (ctypes.c_char_p, [st]),
        "tc_context_create": (st, [ctypes.POINTER(L.ContextDesc), ctypes.POINTER(vp)]),
        "tc_context_destroy": (st, [vp]),
        "tc_table_init": (st, [vp, vp, u32, vp, u32, vp, u32, u32, ctypes.POINTER(L.TableInfoC)]),
        "tc_table_set_templates": (st, [vp, vp, vp, vp]),
        "tc_set_schedule": (st, [vp, ctypes.POINTER(L.Schedule)]),
        "tc_get_schedule": (st, [vp, ctypes.POINTER(L.Schedule)]),
        "tc_frame_build": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_frame_build_graph": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_frame_build_graph_host": (st, [vp, ctypes.POINTER(L.FrameArgs), vp, u64, u64, vp, vp]),
        "tc_frame_build_plain": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_frame_begin": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_instances_classify": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_clusters_cull": (st, [vp, ctypes.POINTER(L.FrameArgs), u32, u32, vp]),
        "tc_build_setup": (st, [vp, ctypes.POINTER(L.FrameArgs), u32, vp]),
        "tc_cluster_classify": (st, [vp, ctypes.POINTER(L.FrameArgs), u32, u32, vp]),
        "tc_triangle_split": (st, [vp, ctypes.POINTER(L.FrameArgs), u32, u32, vp]),
        "tc_triangle_split_all": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_triangle_instantiate": (st, [vp, ctypes.POINTER(L.FrameArgs), u32, u32, vp]),
        "tc_triangle_instantiate_run": (st, [vp, ctypes.POINTER(L.FrameArgs), u32, u32, u32, vp]),
        "tc_blas_setup_insertion": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_blas_clusters_insert": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_blas_setup_insertion_noalloc": (st, [ctypes.POINTER(L.FrameArgs), vp, vp]),
        "tc_split_pass_count": (u32, [u32]),
        "tc_instantiate_backward": (st, [vp, ctypes.POINTER(L.FrameArgs), u64, u64, u64, vp]),
        "tc_generate_vertices": (st, [vp, ctypes.POINTER(L.FrameArgs), vp]),
        "tc_decode_hits": (st, [vp, ctypes.POINTER(L.FrameArgs), vp, u32, vp, vp]),
        "tc_raster_batches": (st, [vp, ctypes.POINTER(L.FrameArgs), ctypes.POINTER(L.RasterOutputs), vp]),
        "tc_read_device_errors": (st, [vp, ctypes.POINTER(u32), vp]),
        "tc_launch_count": (u64, [vp]),
        "tc_lookback_probe": (st, [vp, u32, ctypes.POINTER(u64), vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def exported_symbols() -> list[str]:
    """Every entry point declared in include/tc_tessellation.h."""
    return [
        "tc_version", "tc_status_string", "tc_context_create", "tc_context_destroy", "tc_table_init",
        "tc_table_set_templates", "tc_set_schedule", "tc_get_schedule", "tc_frame_build", "tc_frame_build_graph",
        "tc_frame_build_graph_host", "tc_frame_build_plain", "tc_frame_begin", "tc_instances_classify", "tc_clusters_cull", "tc_build_setup",
        "tc_cluster_classify", "tc_triangle_split", "tc_triangle_split_all", "tc_triangle_instantiate", "tc_triangle_instantiate_run",
        "tc_blas_setup_insertion", "tc_blas_clusters_insert", "tc_blas_setup_insertion_noalloc",
        "tc_split_pass_count", "tc_instantiate_backward",
        "tc_generate_vertices", "tc_decode_hits", "tc_raster_batches",
        "tc_read_device_errors", "tc_launch_count", "tc_lookback_probe",
    ]


def lib():
    """Load libtc_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -m vk_tessellated_clusters_gb300.build_lib` (requires nvcc)")
        _lib = _bind(ctypes.CDLL(LIB_PATH))
    return _lib


def check(status: int, what: str) -> None:
    if status != L.TC_OK:
        raise TcError(status, what)
