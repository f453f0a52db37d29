"""GPU path (through the C ABI) against the CPU oracle on the same seeded inputs."""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.parity import assert_same, max_position_error, scene_diagonal, vertex_tolerance
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import scene as S

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

FLAGS = L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS


def small_caps(**kw):
    caps = L.default_caps(visible_bits=16, part_bits=18, split_bits=14, vertex_bits=21, megs=256)
    caps.update(kw)
    return caps


def run_both(oracle, scene, cam, caps, flags=FLAGS, mode="batched", cam_last=None):
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    ref_state, runs = oracle.frame(scene, cam, caps, flags, camera_last=cam_last)
    ref = ref_state.outputs(oracle.entries)
    pipe = TessellationPipeline(scene, caps, flags)
    pipe.set_cameras(cam, cam_last)
    pipe.build(mode)
    out = pipe.outputs()
    return pipe, out, ref, ref_state


@pytest.fixture(scope="module")
def icosphere():
    return S.scene_icosphere()


def test_icosphere_batched_bit_exact(oracle, icosphere):
    pipe, out, ref, ref_state = run_both(oracle, icosphere, S.camera_icosphere(), small_caps())
    assert pipe.device_errors() == 0
    assert int(ref["readback"]["numPartTriangles"]) > 10000
    assert_same(out, ref, "icosphere batched", vertex_tol=vertex_tolerance(icosphere))
    # the 1e-5 x diagonal bar and the error against the FP64 twin
    ref64 = oracle.vertices_f64(ref_state, len(ref["genVertices"]))
    err = max_position_error(out["genVertices"], ref64)
    d = np.abs(out["genVertices"].astype(np.float64) - ref64)
    print(f"icosphere 20,480 tris: |GPU - FP64| max {err:.3e} rms {np.sqrt((d ** 2).mean()):.3e} "
          f"(scene diagonal {scene_diagonal(icosphere):.3f})")
    assert err <= 1e-5 * scene_diagonal(icosphere), err
    pipe.close()


@pytest.mark.parametrize("mode", ["graph", "plain"])
def test_icosphere_modes_identical(oracle, icosphere, mode):
    pipe, out, ref, _ = run_both(oracle, icosphere, S.camera_icosphere(), small_caps(), mode=mode)
    assert pipe.device_errors() == 0
    assert_same(out, ref, f"icosphere {mode}", vertex_tol=vertex_tolerance(icosphere))
    pipe.close()


def test_close_camera_splits_bit_exact(oracle):
    """Camera just above the surface at 1 px per segment: factors in the
    hundreds, several split passes."""
    sc = S.scene_icosphere(subdivisions=3, map_size=256)
    cam = S.Camera(eye=(0.0, 0.0, 1.08), center=(0.0, 0.0, 0.0), tess_rate_pixels=1.0, near=0.01, far=10.0)
    pipe, out, ref, _ = run_both(oracle, sc, cam, small_caps(maxSplitTriangles=1 << 17, maxPartTriangles=1 << 19,
                                                             maxGeneratedVertices=1 << 23))
    b = ref["build"]
    assert int(b["splitWriteCounter"]) > 0 and int(b["splitPass"]) >= 1
    assert pipe.device_errors() == 0
    assert_same(out, ref, "close camera", vertex_tol=vertex_tolerance(sc))
    pipe.close()


@pytest.mark.parametrize("mode", ["batched", "plain", "graph"])
def test_batched_scene_culling_bit_exact(oracle, mode):
    sc = S.scene_batched(num_instances=24, map_size=128)
    cam = S.camera_orbit(5)
    last = S.camera_orbit(4)
    pipe, out, ref, _ = run_both(oracle, sc, cam, small_caps(), mode=mode, cam_last=last)
    states = ref["instanceStates"]
    assert (states & L.INSTANCE_VISIBLE_BIT).any() and not (states & L.INSTANCE_VISIBLE_BIT).all()
    assert pipe.device_errors() == 0
    assert_same(out, ref, f"batched scene {mode}", vertex_tol=vertex_tolerance(sc))
    pipe.close()


@pytest.mark.parametrize("mode", ["batched", "plain", "graph"])
def test_raster_cull_bit_exact(oracle, mode):
    """Raster semantics: clusters_cull drops clusters, so classify reads the
    compacted visible list (the RT path reads it from the instances' cluster
    prefix instead)."""
    sc = S.scene_batched(num_instances=24, map_size=128)
    cam, last = S.camera_orbit(5), S.camera_orbit(4)
    flags = FLAGS | L.FLAG_RASTER_CULL
    pipe, out, ref, _ = run_both(oracle, sc, cam, small_caps(), flags=flags, mode=mode, cam_last=last)
    assert int(ref["readback"]["numVisibleClusters"]) < sc.total_clusters  # something was culled
    assert pipe.device_errors() == 0
    assert_same(out, ref, f"raster cull {mode}", vertex_tol=vertex_tolerance(sc))
    pipe.close()


def test_many_instances_batched_matches_plain():
    """More instances than the fused BLAS set-up takes (4096): the batched
    frame launches the multi-block set-up, and its output equals the plain
    per-instance path's byte for byte (vertices included)."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(num_instances=4160, map_size=32, box=160.0)
    cam = S.camera_orbit(3, radius=120.0, center=(80.0, 80.0, 80.0), height=40.0)
    outs = {}
    for mode in ("graph", "plain"):
        pipe = TessellationPipeline(sc, L.default_caps(), FLAGS)
        pipe.set_cameras(cam)
        pipe.build(mode)
        outs[mode] = pipe.outputs()
        assert pipe.device_errors() == 0
        pipe.close()
    assert int(outs["graph"]["readback"]["numBlasClusters"]) > 0
    assert_same(outs["graph"], outs["plain"], "4160 instances graph vs plain")


@pytest.mark.parametrize("which", ["parts", "splits", "vertices", "clusters", "megs", "visible"])
def test_capacity_overflow_matches_reference_semantics(oracle, which):
    """Tiny caps: the reference drops work past each cap and lets the raw
    counters run on (cluster_classify.comp.glsl:351-360, build_setup.comp.glsl:108-117)."""
    sc = S.scene_icosphere(subdivisions=3, map_size=128)
    cam = S.Camera(eye=(0.0, 0.0, 1.3), center=(0.0, 0.0, 0.0), tess_rate_pixels=2.0)
    kw = {"parts": dict(maxPartTriangles=300), "splits": dict(maxSplitTriangles=40),
          "vertices": dict(maxGeneratedVertices=5000), "clusters": dict(maxGeneratedClusters=200),
          "megs": dict(maxGeneratedClusterMegs=0), "visible": dict(maxVisibleClusters=7)}[which]
    caps = small_caps(**kw)
    pipe, out, ref, _ = run_both(oracle, sc, cam, caps)
    assert pipe.device_errors() == 0
    assert_same(out, ref, f"overflow {which}", vertex_tol=vertex_tolerance(sc))
    pipe.close()


def test_split_factor_variants(oracle):
    sc = S.scene_icosphere(subdivisions=2, map_size=64)
    cam = S.Camera(eye=(0.0, 0.0, 1.02), center=(0.0, 0.0, 0.0), tess_rate_pixels=1.0)
    for sf in (2, 5, 11):
        pipe, out, ref, _ = run_both(oracle, sc, cam, small_caps(splitFactor=sf))
        assert pipe.device_errors() == 0
        assert_same(out, ref, f"split factor {sf}", vertex_tol=vertex_tolerance(sc))
        pipe.close()


@pytest.mark.parametrize("split", ["per_pass", "all_passes"])
@pytest.mark.parametrize("camera", ["far", "close"])
def test_per_stage_entry_points_match_frame(oracle, icosphere, split, camera):
    """Driving the stages one by one through the C ABI equals the fused frame,
    with the split passes one call each (and the SPLIT_PASS set-ups between
    them) or all in one tc_triangle_split_all call; the close camera makes
    the split passes fire."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    caps = small_caps()
    sc = icosphere
    cam = S.camera_icosphere()
    if camera == "close":
        sc = S.scene_icosphere(subdivisions=3, map_size=256)
        cam = S.Camera(eye=(0.0, 0.0, 1.08), center=(0.0, 0.0, 0.0), tess_rate_pixels=1.0, near=0.01, far=10.0)
    pipe = TessellationPipeline(sc, caps, FLAGS)
    pipe.set_cameras(cam)
    pipe.build("batched")
    want = pipe.outputs()
    if camera == "close":
        assert int(want["readback"]["numSplitTriangles"]) > 0
    pipe.stage("frame_begin")
    pipe.stage("instances_classify")
    pipe.stage("clusters_cull", 0, 1)
    pipe.stage("build_setup", L.BUILD_SETUP_CLASSIFY)
    pipe.stage("cluster_classify", 0, 1)
    pipe.stage("build_setup", L.BUILD_SETUP_SPLIT)
    passes = pipe.split_passes()
    if split == "all_passes":
        pipe.stage("triangle_split_all")
    else:
        for p in range(passes):
            pipe.stage("triangle_split", 0, 1)
            if p + 1 < passes:
                pipe.stage("build_setup", L.BUILD_SETUP_SPLIT_PASS)
    pipe.stage("build_setup", L.BUILD_SETUP_INSTANTIATE_TESS)
    pipe.stage("triangle_instantiate", 0, 0xFFFFFFFF)
    pipe.stage("build_setup", L.BUILD_SETUP_BUILD_BLAS)
    pipe.stage("blas_setup_insertion")
    pipe.stage("blas_clusters_insert")
    got = pipe.outputs()
    assert pipe.device_errors() == 0
    assert_same(got, want, "per-stage vs frame")
    pipe.close()


def test_repeated_frames_are_stable(oracle, icosphere):
    """Scratch reuse across frames (memset or self-clean) leaves no residue."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    caps = small_caps()
    pipe = TessellationPipeline(icosphere, caps, FLAGS)
    pipe.set_cameras(S.camera_icosphere())
    outs = []
    for mode in ("batched", "plain", "batched", "graph", "graph", "plain"):
        pipe.build(mode)
        outs.append(pipe.outputs())
    for o in outs[1:]:
        assert_same(o, outs[0], "repeat")
    assert pipe.device_errors() == 0
    pipe.close()


def test_schedules_change_timing_only(oracle):
    """Every valid launch schedule (what the autotuner searches) gives the
    oracle's output; out-of-range schedules are rejected."""
    from vk_tessellated_clusters_gb300 import native
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(num_instances=24, map_size=128)
    cam, last = S.camera_orbit(5), S.camera_orbit(4)
    caps = small_caps()
    ref_state, _ = oracle.frame(sc, cam, caps, FLAGS, camera_last=last)
    ref = ref_state.outputs(oracle.entries)
    pipe = TessellationPipeline(sc, caps, FLAGS)
    pipe.set_cameras(cam, last)
    schedules = [
        dict(classifyBlocksPerSM=4, scanBlocksPerSM=2, splitBlockSize=128, blocksPerSM=2, vertexBlocksPerSM=2,
             vertexGridPerSM=1),
        dict(classifyBlocksPerSM=16, scanBlocksPerSM=16, splitBlockSize=512, blocksPerSM=4, vertexBlocksPerSM=5,
             fullVertexBlocksPerSM=8, frameShape=1, splitPerPass=1),
        dict(classifyBlocksPerSM=6, scanBlocksPerSM=1, splitBlockSize=256, blocksPerSM=1, vertexBlocksPerSM=1,
             fullVertexBlocksPerSM=1),
        dict(classifyBlocksPerSM=1, scanBlocksPerSM=4, splitBlockSize=256, blocksPerSM=1, vertexBlocksPerSM=6,
             vertexGridPerSM=32, frameShape=0),
    ]
    for sched in schedules:
        pipe.set_schedule(sched)
        assert pipe.schedule() == {**pipe.schedule(), **sched}
        for mode in ("batched", "graph"):
            pipe.build(mode)
            assert_same(pipe.outputs(), ref, f"schedule {sched} {mode}", vertex_tol=vertex_tolerance(sc))
    assert pipe.device_errors() == 0
    for bad in (dict(splitBlockSize=64), dict(vertexBlocksPerSM=0), dict(scanBlocksPerSM=65),
                dict(fullVertexBlocksPerSM=65), dict(vertexGridPerSM=65), dict(frameShape=2), dict(splitPerPass=2)):
        with pytest.raises(native.TcError):
            pipe.set_schedule(bad)
    pipe.close()


@pytest.mark.parametrize("case", ["splits", "transient"])
def test_frame_shapes_identical(oracle, case):
    """Both frame-graph shapes (the first part run allocated beside the split
    passes, or every run after them) and both split forms (one launch for all
    passes, or one per pass) give the oracle's output, on a split-heavy frame
    and on one with 1X + 2X transient builds."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_icosphere(subdivisions=3, map_size=256)
    cam = S.Camera(eye=(0.0, 0.0, 1.08), center=(0.0, 0.0, 0.0), tess_rate_pixels=1.0, near=0.01, far=10.0)
    flags = FLAGS | ((L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X) if case == "transient" else 0)
    if case == "transient":
        sc, cam = S.scene_icosphere(), S.camera_icosphere()
    caps = small_caps()
    ref_state, _ = oracle.frame(sc, cam, caps, flags)
    ref = ref_state.outputs(oracle.entries)
    if case == "splits":
        assert int(ref["readback"]["numSplitTriangles"]) > 0
    pipe = TessellationPipeline(sc, caps, flags)
    pipe.set_cameras(cam)
    for shape, per_pass in ((1, 0), (0, 1), (1, 1), (0, 0)):
        pipe.set_schedule({"frameShape": shape, "splitPerPass": per_pass})
        for mode in ("batched", "graph"):
            pipe.build(mode)
            assert_same(pipe.outputs(), ref, f"{case} shape {shape} {mode}", vertex_tol=vertex_tolerance(sc))
    assert pipe.device_errors() == 0
    pipe.close()


def test_animated_instances_replay_bit_exact(oracle):
    """Per-frame rigid motion written into the instance buffer in place: the
    replayed frame graph sees the new transforms and matches the oracle run
    on the moved scene."""
    import dataclasses
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(num_instances=32, map_size=64)
    motion = S.animation_motion(len(sc.instances))
    caps = small_caps()
    cam = S.camera_orbit(7)
    pipe = TessellationPipeline(sc, caps, FLAGS)
    pipe.set_cameras(cam)
    counts = []
    for t in (0.0, 1.5, 4.0):
        W = S.animated_worlds(sc, motion, t)
        pipe.state.res.set_world_matrices(W)
        pipe.build("graph")
        out = pipe.outputs()
        moved = S.Scene(sc.name, sc.geometries,
                        [dataclasses.replace(i, world=w) for i, w in zip(sc.instances, W)], sc.textures)
        ref_state, _ = oracle.frame(moved, cam, caps, FLAGS)
        assert_same(out, ref_state.outputs(oracle.entries), f"animated t={t}", vertex_tol=vertex_tolerance(sc))
        counts.append(int(out["readback"]["numTotalTriangles"]))
    assert len(set(counts)) > 1  # the motion changes the work
    assert pipe.device_errors() == 0
    pipe.close()


@pytest.mark.parametrize("visualize", [0, L.VISUALIZE_TRIANGLES])
def test_hit_decode_matches_oracle(oracle, visualize):
    """tc_decode_hits on the GPU equals the oracle's restatement field for
    field (base cluster, triangle, vertices, barycentric bits, part id,
    status) on seeded hits of a built frame, malformed hits included."""
    from vk_tessellated_clusters_gb300.hits import sample_hits
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(num_instances=24, map_size=128)
    fc, last = S.frame_constants(S.camera_orbit(5)), S.frame_constants(S.camera_orbit(4))
    fc["visualize"] = visualize
    caps = small_caps()
    ref_state, _ = oracle.frame(sc, fc, caps, FLAGS, camera_last=last)
    pipe = TessellationPipeline(sc, caps, FLAGS)
    pipe.set_cameras(fc, last)
    pipe.build("graph")
    out = pipe.outputs()
    hits = sample_hits(out, sc, pipe.entries, 20000, seed=11, bad=200)
    got = pipe.decode_hits(hits)
    want = oracle.decode_hits(ref_state, hits)
    assert pipe.device_errors() == 0
    assert (got["status"][:20000] == L.HIT_OK).all()
    assert got.tobytes() == want.tobytes()
    pipe.close()


def _ripple_constants(cam, amplitude=0.02):
    fc = S.frame_constants(cam)
    fc["animationRippleAmplitude"] = amplitude
    fc["animationRippleFrequency"] = 8.0
    fc["animationRippleSpeed"] = 1.5
    fc["animationState"] = 0.7
    return fc


@pytest.mark.parametrize("mode", ["batched", "plain", "graph"])
def test_pn_and_ripple_bit_exact(oracle, mode):
    """PN-triangle displacement of part vertices (displacement.glsl:47-104)
    and the ripple on every generated vertex (:106-120): integer outputs
    bit-exact, positions within the vertex tolerance, on a curved mesh seen
    close up (parts everywhere) and on the culled batched scene."""
    ico = S.scene_icosphere(subdivisions=2, map_size=64)
    near = S.Camera(eye=(0.0, 0.0, 1.3), center=(0.0, 0.0, 0.0), tess_rate_pixels=2.0)
    sc = S.scene_batched(num_instances=24, map_size=128)
    cases = [(ico, _ripple_constants(near), None, FLAGS | L.FLAG_PN),
             (ico, _ripple_constants(near), None, FLAGS | L.FLAG_PN | L.FLAG_RIPPLE),
             (sc, _ripple_constants(S.camera_orbit(5)), S.camera_orbit(4), FLAGS | L.FLAG_PN | L.FLAG_RIPPLE)]
    for scene, fc, last, flags in cases:
        pipe, out, ref, _ = run_both(oracle, scene, fc, small_caps(), flags=flags, mode=mode, cam_last=last)
        assert int(ref["readback"]["numPartTriangles"]) > 1000
        assert pipe.device_errors() == 0
        assert_same(out, ref, f"pn/ripple flags={flags} {mode}", vertex_tol=vertex_tolerance(scene))
        pipe.close()


def test_pn_ripple_entry_point_matches_frame(oracle):
    """The stages driven one by one through the C ABI with PN and ripple set
    write the same vertices as the frame path."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    ico = S.scene_icosphere(subdivisions=2, map_size=64)
    fc = _ripple_constants(S.Camera(eye=(0.0, 0.0, 1.3), center=(0.0, 0.0, 0.0), tess_rate_pixels=2.0))
    pipe = TessellationPipeline(ico, small_caps(), FLAGS | L.FLAG_PN | L.FLAG_RIPPLE)
    pipe.set_cameras(fc, None)
    pipe.build("graph")
    want = pipe.outputs()
    pipe.stage("frame_begin")
    pipe.stage("instances_classify")
    pipe.stage("clusters_cull", 0, 1)
    pipe.stage("build_setup", L.BUILD_SETUP_CLASSIFY)
    pipe.stage("cluster_classify", 0, 1)
    pipe.stage("build_setup", L.BUILD_SETUP_SPLIT)
    passes = pipe.split_passes()
    for p in range(passes):
        pipe.stage("triangle_split", 0, 1)
        if p + 1 < passes:
            pipe.stage("build_setup", L.BUILD_SETUP_SPLIT_PASS)
    pipe.stage("build_setup", L.BUILD_SETUP_INSTANTIATE_TESS)
    pipe.stage("triangle_instantiate", 0, 0xFFFFFFFF)
    got = pipe.outputs()
    assert pipe.device_errors() == 0
    assert len(want["genVertices"]) > 1000
    assert got["genVertices"].tobytes() == want["genVertices"].tobytes()
    pipe.close()


TRANSIENT = L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X


@pytest.mark.parametrize("mode", ["batched", "plain", "graph"])
def test_transient_builds_bit_exact(oracle, mode):
    """1X subset and 2X batch transient builds (cluster_classify.comp.glsl:
    254-905): ClasBuildInfos, instance IDs, CLAS addresses, the back slots of
    partTriangles, the index bytes, the two-sided counter and every other
    output bit-exact; positions within the vertex tolerance. Each flag alone
    and both, on the icosphere and the culled batched scene, and with PN and
    the ripple."""
    ico = S.scene_icosphere()
    sc = S.scene_batched(num_instances=24, map_size=128)
    cases = [(ico, S.camera_icosphere(), None, FLAGS | L.FLAG_TRANSIENT_1X),
             (ico, S.camera_icosphere(), None, FLAGS | L.FLAG_TRANSIENT_2X),
             (ico, S.camera_icosphere(), None, FLAGS | TRANSIENT),
             (sc, S.camera_orbit(0), S.camera_orbit(59), FLAGS | TRANSIENT),
             (sc, _ripple_constants(S.camera_orbit(5)), S.camera_orbit(4), FLAGS | TRANSIENT | L.FLAG_PN | L.FLAG_RIPPLE)]
    for scene, cam, last, flags in cases:
        pipe, out, ref, _ = run_both(oracle, scene, cam, small_caps(), flags=flags, mode=mode, cam_last=last)
        assert len(ref["transBuilds"]) > 10
        assert pipe.device_errors() == 0
        assert_same(out, ref, f"transient flags={flags} {mode}", vertex_tol=vertex_tolerance(scene))
        pipe.close()


@pytest.mark.parametrize("which", ["parts", "clusters", "vertices"])
def test_transient_builds_capacity_overflow(oracle, which):
    """Capacity overflow with transient builds: the two-sided part counter
    running out (front chunks and back slots rejected as wholes), generated
    clusters and vertices running out; outputs equal the oracle's."""
    sc = S.scene_batched(num_instances=24, map_size=128)
    kw = {"parts": {"maxPartTriangles": 3000}, "clusters": {"maxGeneratedClusters": 4000},
          "vertices": {"maxGeneratedVertices": 150000}}[which]
    pipe, out, ref, _ = run_both(oracle, sc, S.camera_orbit(0), small_caps(**kw), flags=FLAGS | TRANSIENT,
                                 cam_last=S.camera_orbit(59))
    assert pipe.device_errors() == 0
    assert_same(out, ref, f"transient overflow {which}", vertex_tol=vertex_tolerance(sc))
    pipe.close()


def test_transient_hit_decode_matches_oracle(oracle):
    """tc_decode_hits with 1X subset and 2X batch hits (rchit.glsl:150-180)
    equals the oracle's restatement field for field."""
    from vk_tessellated_clusters_gb300.hits import sample_hits
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(num_instances=24, map_size=128)
    flags = FLAGS | TRANSIENT
    for visualize in (0, L.VISUALIZE_TRIANGLES):
        fc, last = S.frame_constants(S.camera_orbit(0)), S.frame_constants(S.camera_orbit(59))
        fc["visualize"] = visualize
        ref_state, _ = oracle.frame(sc, fc, small_caps(), flags, camera_last=last)
        pipe = TessellationPipeline(sc, small_caps(), flags)
        pipe.set_cameras(fc, last)
        pipe.build("graph")
        out = pipe.outputs()
        hits = sample_hits(out, sc, pipe.entries, 20000, seed=5, bad=200)
        assert ((hits["clusterID"][:20000] >> 30) >= 2).sum() > 1000
        got = pipe.decode_hits(hits)
        want = oracle.decode_hits(ref_state, hits)
        assert pipe.device_errors() == 0
        assert (got["status"][:20000] == L.HIT_OK).all()
        assert got.tobytes() == want.tobytes()
        pipe.close()


@pytest.mark.parametrize("case", ["icosphere", "batched_pn_ripple", "close_splits", "transient"])
def test_raster_batches_match_oracle(oracle, case):
    """tc_raster_batches (render_raster_clusters_batched task + mesh shaders as
    compute): batch records, counts, batch-local indices and primitive IDs
    bit-exact; world and clip positions within the vertex tolerance (scaled
    by the instances' transforms)."""
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    flags, last = FLAGS, None
    if case == "icosphere":
        sc, cam = S.scene_icosphere(), S.frame_constants(S.camera_icosphere())
    elif case == "batched_pn_ripple":
        sc, cam, last = S.scene_batched(num_instances=24, map_size=128), _ripple_constants(S.camera_orbit(5)), S.camera_orbit(4)
        cam["visualize"] = L.VISUALIZE_TRIANGLES
        flags |= L.FLAG_PN | L.FLAG_RIPPLE
    elif case == "close_splits":
        sc = S.scene_icosphere(subdivisions=3, map_size=256)
        cam = S.frame_constants(S.Camera(eye=(0.0, 0.0, 1.08), center=(0.0, 0.0, 0.0), tess_rate_pixels=1.0,
                                         near=0.01, far=10.0))
    else:
        sc, cam, last = S.scene_batched(num_instances=24, map_size=128), S.frame_constants(S.camera_orbit(0)), S.camera_orbit(59)
        flags |= TRANSIENT
    caps = small_caps(maxSplitTriangles=1 << 17, maxPartTriangles=1 << 19, maxGeneratedVertices=1 << 23)
    ref_state, _ = oracle.frame(sc, cam, caps, flags, camera_last=last)
    want = oracle.raster_batches(ref_state)
    pipe = TessellationPipeline(sc, caps, flags)
    pipe.set_cameras(cam, last)
    pipe.build("graph")
    got = pipe.raster_batches()
    assert pipe.device_errors() == 0
    assert got["counts"] == want["counts"] and want["counts"][0] > 100
    for f in ("batches", "indices", "primitiveIDs"):
        assert got[f].tobytes() == want[f].tobytes(), f
    scale = max(float(np.abs(np.asarray(i.world)[:3, :3]).sum(axis=1).max()) for i in sc.instances)
    tol = vertex_tolerance(sc) * max(1.0, scale)
    assert np.abs(got["worldPositions"].astype(np.float64) - want["worldPositions"]).max() <= tol
    cm = float(np.abs(want["clipPositions"]).max())
    assert np.abs(got["clipPositions"].astype(np.float64) - want["clipPositions"]).max() <= 1e-5 * cm + 1e-4
    pipe.close()


def test_host_io_frames_match_oracle(oracle):
    """tc_frame_build_graph_host: each frame's inputs (its frame constants,
    the previous frame's, the instance records) read from a pinned host block
    and its Readback written to pinned host memory by kernels of the frame
    graph; per orbit frame the outputs match the oracle and the host Readback
    equals the device one. Unpinned or misaligned host buffers are argument
    errors that launch nothing and leave the context usable."""
    import torch
    from vk_tessellated_clusters_gb300 import native
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    from vk_tessellated_clusters_gb300.scene import frame_constants
    sc = S.scene_batched(num_instances=32, map_size=64)
    caps = small_caps()
    pipe = TessellationPipeline(sc, caps, FLAGS)
    FC = L.FrameConstants.itemsize
    RB = L.Readback.itemsize
    rec = pipe.state.res.instance_records.view(np.uint8).reshape(-1)
    frames = (3, 4, 9)
    blk = 2 * FC + rec.size
    assert blk % 16 == 0
    # rows of blk + 16 bytes: the second frame also uploads a 4-byte tail
    # (inputBytes not a multiple of 16) into slack past the frame's inputs
    host = torch.zeros((len(frames), blk + 16), dtype=torch.uint8, pin_memory=True)
    for k, f in enumerate(frames):
        host[k, :FC] = torch.from_numpy(np.frombuffer(frame_constants(S.camera_orbit(f)).tobytes(), np.uint8).copy())
        host[k, FC:2 * FC] = torch.from_numpy(
            np.frombuffer(frame_constants(S.camera_orbit(f - 1)).tobytes(), np.uint8).copy())
        host[k, 2 * FC:blk] = torch.from_numpy(rec.copy())
    tail = torch.tensor([0xA5, 0x5A, 0x3C, 0x77], dtype=torch.uint8)
    host[1, blk:blk + 4] = tail
    rb_host = torch.zeros(RB, dtype=torch.uint8, pin_memory=True)
    dev_block = torch.zeros(blk + 512, dtype=torch.uint8, device="cuda")
    base = (dev_block.data_ptr() + 255) // 256 * 256
    off = base - dev_block.data_ptr()
    fa = pipe.args
    saved = (fa.view, fa.viewLast, fa.instances)
    fa.view, fa.viewLast, fa.instances = base, base + FC, base + 2 * FC
    for k, f in enumerate(frames):
        rb_host.zero_()
        pipe.build_host(host[k].data_ptr(), base, blk + (4 if k == 1 else 0), rb_host.data_ptr())
        torch.cuda.synchronize()
        if k == 1:
            assert torch.equal(dev_block[off + blk:off + blk + 4].cpu(), tail)
        out = pipe.outputs()
        ref_state, _ = oracle.frame(sc, S.camera_orbit(f), caps, FLAGS, camera_last=S.camera_orbit(f - 1))
        assert_same(out, ref_state.outputs(oracle.entries), f"host-io frame {f}", vertex_tol=vertex_tolerance(sc))
        assert np.array_equal(rb_host.numpy(), pipe.state.readback.handle[:RB].cpu().numpy()), f"frame {f}"
        assert int(rb_host.numpy().view(L.Readback)[0]["numTotalTriangles"]) > 0

    # argument errors: a pageable host block, a misaligned one, a misaligned Readback buffer
    pageable = np.zeros(blk + 64, np.uint8)
    p_addr = (pageable.ctypes.data + 15) // 16 * 16
    for hin, hrb in ((p_addr, rb_host.data_ptr()), (host[0].data_ptr() + 4, rb_host.data_ptr()),
                     (host[0].data_ptr(), rb_host.data_ptr() + 4)):
        with pytest.raises(native.TcError) as e:
            pipe.build_host(hin, base, blk, hrb)
        assert e.value.status == L.TC_ERR_INVALID_ARG

    # the context still replays: the last frame again, then the Readback alone
    # with the frame reading the resident buffers
    pipe.build_host(host[2].data_ptr(), base, blk, rb_host.data_ptr())
    torch.cuda.synchronize()
    last = pipe.outputs()
    fa.view, fa.viewLast, fa.instances = saved
    pipe.set_cameras(S.camera_orbit(frames[2]), S.camera_orbit(frames[2] - 1))
    rb_host.zero_()
    pipe.build_host(0, 0, 0, rb_host.data_ptr())
    torch.cuda.synchronize()
    assert_same(pipe.outputs(), last, "readback-only frame")
    assert np.array_equal(rb_host.numpy(), pipe.state.readback.handle[:RB].cpu().numpy())

    # the frame constants from the uploaded block, the instance records from the
    # resident buffer: the upload runs as its own kernel before the frame
    # (the frame's first kernel reads its inputs from the host block only when
    # all of them lie in it)
    fa.view, fa.viewLast = base, base + FC
    rb_host.zero_()
    pipe.build_host(host[0].data_ptr(), base, blk, rb_host.data_ptr())
    torch.cuda.synchronize()
    ref_state, _ = oracle.frame(sc, S.camera_orbit(frames[0]), caps, FLAGS, camera_last=S.camera_orbit(frames[0] - 1))
    assert_same(pipe.outputs(), ref_state.outputs(oracle.entries), "separate upload", vertex_tol=vertex_tolerance(sc))
    assert np.array_equal(rb_host.numpy(), pipe.state.readback.handle[:RB].cpu().numpy())
    fa.view, fa.viewLast = saved[0], saved[1]
    assert pipe.device_errors() == 0
    pipe.close()
