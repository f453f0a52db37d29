"""tc_blas_setup_insertion_noalloc, the blas_setup_insertion entry point for
callers that cannot allocate device memory (its look-back scratch is a fixed
__device__ array of the library): through the C ABI its output equals the
context entry point's, on two calls in a row (the shared scratch is reused),
and at the largest instance count it accepts it equals the exclusive scan of
the per-instance counts. Collected last on purpose: it must pass both alone in
a fresh process (its first call sets the scratch address up) and after the
other GPU tests."""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from tests.conftest import cuda_available
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import native
from vk_tessellated_clusters_gb300 import scene as S

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

MAX_INSTANCES = 1 << 20  # TC_NOALLOC_MAX_INSTANCES


def _noalloc(args, errors, stream):
    return native.lib().tc_blas_setup_insertion_noalloc(ctypes.byref(args), errors, stream)


def _stages_until_blas_setup(pipe):
    n = pipe.args.numInstances
    pipe.stage("frame_begin")
    pipe.stage("instances_classify")
    pipe.stage("clusters_cull", 0, n)
    pipe.stage("build_setup", L.BUILD_SETUP_CLASSIFY)
    pipe.stage("cluster_classify", 0, n)
    pipe.stage("build_setup", L.BUILD_SETUP_SPLIT)
    passes = pipe.split_passes()
    for p in range(passes):
        pipe.stage("triangle_split", 0, n)
        if p + 1 < passes:
            pipe.stage("build_setup", L.BUILD_SETUP_SPLIT_PASS)
    pipe.stage("build_setup", L.BUILD_SETUP_INSTANTIATE_TESS)
    pipe.stage("triangle_instantiate", 0, 0xFFFFFFFF)
    pipe.stage("build_setup", L.BUILD_SETUP_BUILD_BLAS)


def test_matches_context_entry_point_on_two_calls_in_a_row():
    import torch
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    # 1500 instances: six look-back tiles of 256
    sc = S.scene_batched(num_instances=1500, map_size=64)
    caps = L.default_caps(visible_bits=20, part_bits=20, split_bits=16, vertex_bits=24, megs=1024)
    pipe = TessellationPipeline(sc, caps, L.FLAG_CULLING)
    try:
        pipe.set_cameras(S.camera_orbit(0))
        _stages_until_blas_setup(pipe)
        st = pipe.state
        bufs = (st.build, st.blas_build_infos, st.readback)
        torch.cuda.synchronize()
        before = [b.handle.clone() for b in bufs]
        counts = before[1].cpu().numpy().view(L.BlasBuildInfo)["clusterReferencesCount"]
        assert (counts[:256] > 0).any() and (counts[256:] > 0).any()  # real counts in several tiles

        pipe.stage("blas_setup_insertion")
        torch.cuda.synchronize()
        want = [b.handle.cpu().numpy().tobytes() for b in bufs]
        assert want[1] != before[1].cpu().numpy().tobytes()

        errors = torch.zeros(1, dtype=torch.int32, device="cuda")
        for call in range(2):
            for b, snap in zip(bufs, before):
                b.handle.copy_(snap)
            status = _noalloc(pipe.args, errors.data_ptr(), pipe.stream())
            assert status == L.TC_OK, (call, status)
            torch.cuda.synchronize()
            got = [b.handle.cpu().numpy().tobytes() for b in bufs]
            for name, g, w in zip(("SceneBuilding", "BlasBuildInfo", "Readback"), got, want):
                assert g == w, (call, name)
            assert int(errors.item()) == 0

        # the rest of the frame runs on from the no-alloc output
        pipe.stage("blas_clusters_insert")
        assert pipe.device_errors() == 0
    finally:
        pipe.close()


def _standalone_buffers(torch, n, rng, base_counter):
    counts = rng.integers(0, 200, n).astype(np.uint32)
    counts[rng.random(n) < 0.3] = 0
    infos = np.zeros(n, L.BlasBuildInfo)
    infos["clusterReferencesCount"] = counts
    d_infos = torch.from_numpy(infos.view(np.uint8).copy()).cuda()
    sizes = rng.integers(0, 1 << 12, n).astype(np.uint32)
    d_sizes = torch.from_numpy(sizes.view(np.uint8).copy()).cuda()
    sb = np.zeros(1, L.SceneBuilding)
    sb["numRenderInstances"] = n
    sb["blasClusterCounter"] = base_counter
    sb["blasBuildInfos"] = d_infos.data_ptr()
    sb["blasBuildSizes"] = d_sizes.data_ptr()
    sb["blasClusterAddresses"] = 0x500000000000  # only used to form addresses
    d_sb = torch.from_numpy(sb.view(np.uint8).copy()).cuda()
    d_rb = torch.zeros(L.Readback.itemsize, dtype=torch.uint8, device="cuda")
    args = L.FrameArgs()
    args.build = d_sb.data_ptr()
    args.readback = d_rb.data_ptr()
    args.numInstances = n
    return counts, sizes, d_infos, d_sb, d_rb, args


def test_largest_instance_count_is_the_exclusive_scan():
    import torch
    rng = np.random.default_rng(3)
    stream = torch.cuda.current_stream().cuda_stream
    errors = torch.zeros(1, dtype=torch.int32, device="cuda")
    for call, n in enumerate((MAX_INSTANCES, 1000)):
        base = 17 + call
        counts, sizes, d_infos, d_sb, d_rb, args = _standalone_buffers(torch, n, rng, base)
        assert _noalloc(args, errors.data_ptr(), stream) == L.TC_OK
        torch.cuda.synchronize()
        infos = d_infos.cpu().numpy().view(L.BlasBuildInfo)
        offsets = base + np.concatenate([[0], np.cumsum(counts.astype(np.uint64))[:-1]])
        assert (infos["clusterReferencesCount"] == 0).all()
        assert (infos["clusterReferencesStride"] == 8).all()
        assert np.array_equal(infos["clusterReferences"], 0x500000000000 + offsets.astype(np.uint64) * 8)
        sb = d_sb.cpu().numpy().view(L.SceneBuilding)[0]
        assert int(sb["blasClusterCounter"]) == base + int(counts.sum())
        rb = d_rb.cpu().numpy().view(L.Readback)[0]
        assert int(rb["numBlasActualSizes"]) == int(sizes.astype(np.uint64).sum() % (1 << 32))
        assert int(errors.item()) == 0


def test_rejects_sizes_beyond_the_maximum_and_missing_buffers():
    import torch
    args = L.FrameArgs()
    args.build = 0x1000
    args.readback = 0x2000
    args.numInstances = MAX_INSTANCES + 1
    stream = torch.cuda.current_stream().cuda_stream
    assert _noalloc(args, None, stream) == L.TC_ERR_CAPACITY  # rejected before any launch
    args.numInstances = 1
    args.build = 0
    assert _noalloc(args, None, stream) == L.TC_ERR_INVALID_ARG
    assert native.lib().tc_blas_setup_insertion_noalloc(None, None, stream) == L.TC_ERR_INVALID_ARG


_FRESH = textwrap.dedent("""
    import sys
    sys.path.insert(0, {root!r})
    import numpy as np
    import torch
    from tests.test_zz_no_alloc import _noalloc, _standalone_buffers
    from vk_tessellated_clusters_gb300 import layouts as L
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    errors = torch.zeros(1, dtype=torch.int32, device="cuda")
    n, base = 70000, 5
    counts, sizes, d_infos, d_sb, d_rb, args = _standalone_buffers(torch, n, rng, base)
    snap = d_infos.clone()
    torch.cuda.synchronize()
    want = base + np.concatenate([[0], np.cumsum(counts.astype(np.uint64))[:-1]])
    # the first call in this process's context: it looks the scratch array up
    assert _noalloc(args, errors.data_ptr(), stream) == L.TC_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2):
        d_infos.copy_(snap)
        sb = d_sb.cpu().numpy().view(L.SceneBuilding)
        sb["blasClusterCounter"] = base
        d_sb.copy_(torch.from_numpy(sb.view(np.uint8).copy()))
        assert _noalloc(args, errors.data_ptr(), stream) == L.TC_OK
        torch.cuda.synchronize()
        infos = d_infos.cpu().numpy().view(L.BlasBuildInfo)
        assert np.array_equal(infos["clusterReferences"], 0x500000000000 + want.astype(np.uint64) * 8), call
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    assert int(errors.item()) == 0
    print("fresh-process no-alloc ok")
""")


def test_first_call_in_a_fresh_process_and_no_device_allocation():
    """The set-up path (the first call in a new CUDA context) runs in a child
    process of its own, and the calls after it leave the device's free memory
    unchanged: nothing is allocated."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", _FRESH.format(root=root)], capture_output=True, text=True,
                         timeout=600, cwd=root)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-4000:]
    assert "fresh-process no-alloc ok" in out.stdout
