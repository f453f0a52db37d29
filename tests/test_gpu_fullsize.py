"""GPU path against the oracle at the sizes the bench measures.

- the batched scene (256 instances of four meshes, 512² fp32 maps, orbit
  camera, culling on) on the frames the bench's timed steps start with, through
  the CUDA graph like the bench, and one frame from host buffers like the
  bench's end-to-end figure;
- the terrain (1024² quads, 4096² fp16 fBm map of 8 octaves, grazing camera at
  3840x2160, the bench's terrain capacities): the split passes fire and the
  fp16 texel path samples every vertex;
- maps in the other texel formats and sizes: unorm16, and fp32 / fp16 /
  unorm16 maps whose sizes are not powers of two (the wrap by modulo instead
  of a mask).
Integer outputs bit-exact; positions within 1e-5 x the smallest mesh diagonal
of the oracle's, and within 1e-5 x the scene diagonal of the FP64 twin (max and
RMS error printed)."""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.parity import assert_same, max_position_error, scene_diagonal, vertex_tolerance
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import scene as S

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]


def terrain_caps():
    # the bench's terrain capacities (bench.terrain_caps)
    return L.default_caps(visible_bits=16, part_bits=21, split_bits=18, vertex_bits=25, megs=2048)


def fp64_error(oracle, pipe, scene, cam, caps, flags, cam_last=None):
    """(max, rms) |GPU - FP64 twin| of a frame built with the full-cluster list."""
    flags |= L.FLAG_WRITE_FULLCLUSTERS
    pipe_flags = pipe.state.args.flags
    pipe.state.args.flags = flags
    pipe.set_cameras(cam, cam_last)
    pipe.build("graph")
    got = pipe.outputs()
    pipe.state.args.flags = pipe_flags
    st, _ = oracle.frame(scene, cam, caps, flags, camera_last=cam_last)
    ref64 = oracle.vertices_f64(st, len(got["genVertices"]))
    d = np.abs(got["genVertices"].astype(np.float64) - ref64)
    return float(d.max()), float(np.sqrt((d ** 2).mean()))


@pytest.fixture(scope="module")
def batched():
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(256)
    pipe = TessellationPipeline(sc, L.default_caps(), L.FLAG_CULLING)
    yield sc, pipe
    pipe.close()


@pytest.mark.parametrize("frame", [0, 5, 17, 31])
def test_batched_scene_full_size_bit_exact(oracle, batched, frame):
    """Frame 5 is the bench's first timed frame (warm-up 5)."""
    sc, pipe = batched
    cam, last = S.camera_orbit(frame), S.camera_orbit(frame - 1)
    pipe.set_cameras(cam, last)
    pipe.build("graph")
    got = pipe.outputs()
    assert pipe.device_errors() == 0
    st, _ = oracle.frame(sc, cam, L.default_caps(), L.FLAG_CULLING, camera_last=last)
    want = st.outputs(oracle.entries)
    assert int(want["readback"]["numTotalTriangles"]) > 3_000_000
    states = want["instanceStates"]
    assert (states & L.INSTANCE_VISIBLE_BIT).any() and not (states & L.INSTANCE_VISIBLE_BIT).all()
    assert_same(got, want, f"batched frame {frame}", vertex_tol=vertex_tolerance(sc))


def test_batched_scene_from_host_buffers_bit_exact(oracle, batched):
    """The bench's end-to-end form at full size: frame 5 through
    tc_frame_build_graph_host (frame constants and instance records from a
    pinned staging block, the Readback to pinned host memory) matches the
    oracle, and the host Readback equals the device one."""
    import torch
    sc, pipe = batched
    FC = L.FrameConstants.itemsize
    rec = pipe.state.res.instance_records.view(np.uint8).reshape(-1)
    blk = 2 * FC + rec.size
    stage = torch.empty(blk, dtype=torch.uint8, pin_memory=True)
    sn = stage.numpy()
    cam, last = S.camera_orbit(5), S.camera_orbit(4)
    sn[:FC] = np.frombuffer(S.frame_constants(cam).tobytes(), np.uint8)
    sn[FC:2 * FC] = np.frombuffer(S.frame_constants(last).tobytes(), np.uint8)
    sn[2 * FC:] = rec
    dev_block = torch.empty(blk + 256, dtype=torch.uint8, device="cuda")
    base = (dev_block.data_ptr() + 255) // 256 * 256
    rb_host = torch.zeros(L.Readback.itemsize, dtype=torch.uint8, pin_memory=True)
    fa = pipe.args
    saved = (fa.view, fa.viewLast, fa.instances)
    fa.view, fa.viewLast, fa.instances = base, base + FC, base + 2 * FC
    try:
        pipe.build_host(stage.data_ptr(), base, blk, rb_host.data_ptr())
        torch.cuda.synchronize()
        got = pipe.outputs()
    finally:
        fa.view, fa.viewLast, fa.instances = saved
    assert pipe.device_errors() == 0
    assert np.array_equal(rb_host.numpy(), pipe.state.readback.handle[:L.Readback.itemsize].cpu().numpy())
    st, _ = oracle.frame(sc, cam, L.default_caps(), L.FLAG_CULLING, camera_last=last)
    assert_same(got, st.outputs(oracle.entries), "batched frame 5 from host buffers", vertex_tol=vertex_tolerance(sc))


def test_batched_scene_full_size_fp64_error(oracle, batched):
    sc, pipe = batched
    mx, rms = fp64_error(oracle, pipe, sc, S.camera_orbit(5), L.default_caps(), L.FLAG_CULLING, S.camera_orbit(4))
    print(f"batched scene frame 5: |GPU - FP64| max {mx:.3e} rms {rms:.3e} (scene diagonal {scene_diagonal(sc):.3f})")
    assert mx <= 1e-5 * scene_diagonal(sc), mx


@pytest.fixture(scope="module")
def terrain():
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_terrain()
    pipe = TessellationPipeline(sc, terrain_caps(), L.FLAG_CULLING)
    yield sc, pipe
    pipe.close()


def test_terrain_fp16_map_with_splits_bit_exact(oracle, terrain):
    sc, pipe = terrain
    assert sc.textures[0].format == L.TEXEL_F16 and sc.textures[0].texels.shape == (4096, 4096)
    cam = S.camera_terrain()
    pipe.set_cameras(cam)
    pipe.build("graph")
    got = pipe.outputs()
    assert pipe.device_errors() == 0
    st, _ = oracle.frame(sc, cam, terrain_caps(), L.FLAG_CULLING)
    want = st.outputs(oracle.entries)
    rb = want["readback"]
    assert int(rb["numSplitTriangles"]) > 1000  # the split passes fire
    assert int(rb["numTotalTriangles"]) > 20_000_000
    assert int(rb["numGenVertices"]) > 20_000_000
    assert_same(got, want, "terrain", vertex_tol=vertex_tolerance(sc))
    # and the same frame through per-stage launches equals the graph's
    pipe.build("batched")
    assert_same(pipe.outputs(), got, "terrain batched vs graph")


def test_terrain_fp64_error(oracle, terrain):
    sc, pipe = terrain
    mx, rms = fp64_error(oracle, pipe, sc, S.camera_terrain(), terrain_caps(), L.FLAG_CULLING)
    print(f"terrain: |GPU - FP64| max {mx:.3e} rms {rms:.3e} (scene diagonal {scene_diagonal(sc):.3f})")
    assert mx <= 1e-5 * scene_diagonal(sc), mx


def _noise(h, w, seed):
    """Seeded fBm of an h x w map (tileable value noise resampled to h x w)."""
    n = S.value_noise(max(h, w), 4, seed)
    return np.ascontiguousarray(n[:h, :w])


MAP_CASES = {
    "unorm16_pow2": lambda: S.Texture((np.round(_noise(512, 512, 21) * 65535)).astype(np.uint16), L.TEXEL_UNORM16),
    "fp32_npot": lambda: S.Texture(_noise(300, 517, 22).astype(np.float32), L.TEXEL_F32),
    "fp16_npot": lambda: S.Texture(_noise(1000, 333, 23).astype(np.float16), L.TEXEL_F16),
    "unorm16_npot": lambda: S.Texture((np.round(_noise(257, 129, 24) * 65535)).astype(np.uint16), L.TEXEL_UNORM16),
}


@pytest.mark.parametrize("case", sorted(MAP_CASES))
@pytest.mark.parametrize("mode", ["graph", "plain"])
def test_map_formats_and_sizes_bit_exact(oracle, case, mode):
    """Two icospheres (subdivision 5) on one map: a close one whose triangles
    split and become parts, and one 100 units behind it whose clusters stay
    whole, so split parts, parts and full clusters all sample the map."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    base = S.scene_icosphere()
    far = np.eye(4)
    far[2, 3] = -100.0
    insts = [base.instances[0], S.Instance(0, far, 0, 0.05, 0.0)]
    sc = S.Scene(f"icosphere {case}", base.geometries, insts, [MAP_CASES[case]()])
    cam = S.Camera(eye=(0.0, 0.0, 1.3), center=(0.0, 0.0, 0.0), tess_rate_pixels=2.0, far=1000.0)
    caps = L.default_caps(visible_bits=16, part_bits=20, split_bits=16, vertex_bits=23, megs=1024)
    flags = L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS
    pipe = TessellationPipeline(sc, caps, flags)
    try:
        pipe.set_cameras(cam)
        pipe.build(mode)
        got = pipe.outputs()
        assert pipe.device_errors() == 0
        st, _ = oracle.frame(sc, cam, caps, flags)
        want = st.outputs(oracle.entries)
        rb = want["readback"]
        assert int(rb["numSplitTriangles"]) > 0 and int(rb["numPartTriangles"]) > 0 and int(rb["numFullClusters"]) > 0
        assert_same(got, want, f"{case} {mode}", vertex_tol=vertex_tolerance(sc))
        ref64 = oracle.vertices_f64(st, len(got["genVertices"]))
        assert max_position_error(got["genVertices"], ref64) <= 1e-5 * scene_diagonal(sc)
    finally:
        pipe.close()
