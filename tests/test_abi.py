"""The C ABI: the library loads and exports every entry point declared in
include/tc_tessellation.h; the Python layouts agree with the header; calls
that need no GPU behave. No compute calls here."""
import ctypes
import os
import re
import subprocess

import pytest

from tests.conftest import cuda_available
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tc_tessellation.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:tc_status|const char\*|uint32_t|uint64_t)\s+(tc_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(native.LIB_PATH):
        from vk_tessellated_clusters_gb300 import build_lib
        build_lib.build()
    return native.lib()


def test_header_declares_the_bound_entry_points():
    assert declared_functions() == sorted(native.exported_symbols())


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (tc_\w+)$", out, re.M))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_header_static_asserts_and_python_layouts(tmp_path):
    """Compile the header as C++ (its static_asserts pin the reference sizes) and
    check every numpy layout against sizeof/offsetof."""
    probe = tmp_path / "probe.cpp"
    fields = {
        "tc_SceneBuilding": (L.SceneBuilding, ["genClusterDataCounter", "instanceStates", "partTriangles",
                                               "positionTruncateBitCount", "genVertices", "blasBuildInfos",
                                               "numBlasReservedSizes"]),
        "tc_RenderInstance": (L.RenderInstance, ["geometryID", "displacementIndex", "geoLo", "positions",
                                                 "clusterTemplateInstantiatonSizes"]),
        "tc_FrameConstants": (L.FrameConstants, ["viewProjMatrix", "viewport", "viewportf", "tessRate",
                                                 "displacementScale", "nearPlane", "hizSizeFactors",
                                                 "visFilterClusterID"]),
        "tc_Readback": (L.Readback, ["numGenDatas", "numBlasReservedSizes", "debugU64", "debugA", "debugC"]),
        "tc_TemplateInstantiateInfo": (L.TemplateInstantiateInfo, ["clusterTemplateAddress", "vertexBufferStride"]),
        "tc_BlasBuildInfo": (L.BlasBuildInfo, ["clusterReferences"]),
        "tc_DisplacementTexture": (L.DisplacementTexture, ["format"]),
    }
    lines = ['#include <cstdio>', '#include <cstddef>', '#include "tc_tessellation.h"', "int main(){"]
    for st, (_, fs) in fields.items():
        lines.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fs:
            lines.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    lines += ['printf("tc_TessTriangleInfo %zu\\n", sizeof(tc_TessTriangleInfo));', "return 0;}"]
    probe.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(probe), "-o", str(exe)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)], text=True).splitlines())
    for st, (dt, fs) in fields.items():
        assert int(got[st]) == dt.itemsize, st
        for f in fs:
            assert int(got[f"{st}.{f}"]) == dt.fields[f][1], (st, f)
    assert int(got["tc_TessTriangleInfo"]) == L.TessTriangleInfo.itemsize == 24


def test_header_is_c_and_links_from_c(tmp_path, lib):
    """The ABI as a C consumer (a cgo or N-API shim) sees it: the header
    compiles as C11 and a C program links against the library and calls it."""
    prog = tmp_path / "consumer.c"
    prog.write_text('#include <stdio.h>\n#include "tc_tessellation.h"\n'
                    "int main(void) {\n"
                    "  tc_context* ctx = 0;\n"
                    '  printf("%s|%s|%u|%d\\n", tc_version(), tc_status_string(TC_ERR_CAPACITY),\n'
                    "         tc_split_pass_count(8), (int)tc_context_create(0, &ctx));\n"
                    "  return sizeof(tc_SceneBuilding) == 368 && sizeof(tc_schedule) == 40 ? 0 : 1;\n"
                    "}\n")
    exe = tmp_path / "consumer"
    libdir = os.path.dirname(native.LIB_PATH)
    subprocess.check_call(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(prog),
                           "-L", libdir, "-ltc_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).strip().split("|")
    assert "sm_103a" in out[0]
    assert out[1] == "request exceeds the context's capacity"
    assert out[2] == "4"
    assert int(out[3]) == L.TC_ERR_INVALID_ARG  # no descriptor


def test_calls_without_gpu(lib):
    assert b"sm_103a" in lib.tc_version()
    assert lib.tc_status_string(L.TC_ERR_CAPACITY) == b"request exceeds the context's capacity"
    assert [lib.tc_split_pass_count(s) for s in (2, 8, 11)] == [14, 4, 4]
    assert lib.tc_launch_count(None) == 0
    # argument validation happens before any CUDA call
    assert lib.tc_context_create(None, None) == L.TC_ERR_INVALID_ARG
    assert lib.tc_frame_build(None, None, None) == L.TC_ERR_INVALID_ARG
    assert lib.tc_frame_build_graph(None, None, None) == L.TC_ERR_INVALID_ARG
    assert lib.tc_frame_build_graph_host(None, None, None, 0, 0, None, None) == L.TC_ERR_INVALID_ARG
    assert lib.tc_context_destroy(None) == L.TC_ERR_INVALID_ARG


@pytest.mark.skipif(cuda_available(), reason="checks the no-GPU failure path")
def test_context_create_reports_cuda_error_without_gpu(lib):
    desc = L.ContextDesc()
    desc.maxInstances = 1
    desc.maxTotalClusters = 1
    desc.caps = L.caps_from(L.default_caps(visible_bits=4, part_bits=4, split_bits=4, vertex_bits=8, megs=1))
    ctx = ctypes.c_void_p()
    assert lib.tc_context_create(ctypes.byref(desc), ctypes.byref(ctx)) == L.TC_ERR_CUDA
    assert not ctx.value


def test_noalloc_source_names_no_allocation_call():
    """tc_blas_setup_insertion_noalloc's translation unit calls no device
    allocator: its scratch is a file-scope __device__ array."""
    src = open(os.path.join(ROOT, "vk_tessellated_clusters_gb300", "csrc", "tc_noalloc.cu")).read()
    code = "\n".join(line.split("//")[0] for line in src.splitlines())
    for name in ("cudaMalloc", "cudaFree", "cudaMallocAsync", "cudaFreeAsync", "cudaMallocManaged", "cudaMallocHost",
                 "cuMemAlloc", "cuMemCreate", "malloc(", "new "):
        assert name not in code, name
    assert "static __device__ __align__(256)" in code
    assert "cudaGetSymbolAddress" in code
