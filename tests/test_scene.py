"""Synthetic scenes and the clusterizer produce valid reference-layout clusters."""
import numpy as np
import pytest

from vk_tessellated_clusters_gb300 import scene as S


@pytest.mark.parametrize("make", [lambda: S.icosphere(3), lambda: S.torus(1.0, 0.3, 32, 12), lambda: S.grid(16, 8),
                                  lambda: S.subdivided_cube(4, 2)])
def test_clusterizer_preserves_the_mesh(make):
    mesh = make()
    g = S.clusterize(mesh, 3)
    cl = g.clusters
    assert (cl["numTriangles"] <= 64).all() and (cl["numVertices"] <= 64).all()
    assert (cl["numTriangles"] > 0).all()
    assert int(cl["numTriangles"].sum()) == mesh.triangles.shape[0] == g.num_triangles
    assert np.array_equal(cl["firstLocalTriangle"], np.concatenate([[0], np.cumsum(cl["numTriangles"].astype(int) * 3)[:-1]]))
    assert np.array_equal(cl["firstLocalVertex"], np.concatenate([[0], np.cumsum(cl["numVertices"].astype(int))[:-1]]))
    # every original triangle appears once, with the same positions
    tris = []
    for c in cl:
        lt = g.local_triangles[c["firstLocalTriangle"]:c["firstLocalTriangle"] + 3 * c["numTriangles"]].reshape(-1, 3)
        assert lt.max() < c["numVertices"]
        p = g.positions[c["firstLocalVertex"] + lt.astype(int)]
        tris.append(p)
    got = np.concatenate(tris).round(5)
    want = mesh.positions[mesh.triangles].astype(np.float32).round(5)
    key = lambda a: sorted(map(lambda t: tuple(t.reshape(-1)), a))
    assert key(got) == key(want)
    # bounding boxes contain their cluster's vertices
    for i, c in enumerate(cl[:50]):
        p = g.positions[c["firstLocalVertex"]:c["firstLocalVertex"] + c["numVertices"]]
        assert (p >= g.bboxes[i]["lo"] - 1e-6).all() and (p <= g.bboxes[i]["hi"] + 1e-6).all()
    assert len(np.unique(g.template_addresses)) == len(cl)


def test_sizes_of_the_benchmark_meshes():
    assert S.icosphere(5).triangles.shape[0] == 20480
    assert S.icosphere(4).triangles.shape[0] == 5120
    assert S.torus(1.0, 0.3, 128, 48).triangles.shape[0] == 12288
    assert S.grid(128, 128).triangles.shape[0] == 32768
    assert S.subdivided_cube(16, 8).triangles.shape[0] == 1536
    g = S.clusterize(S.grid(1024, 1024, 1024.0, 1024.0))
    assert g.num_triangles == 2097152 and g.num_clusters == 32768


def test_value_noise_is_seeded_tileable_and_normalised():
    a = S.value_noise(64, 4, seed=5)
    b = S.value_noise(64, 4, seed=5)
    c = S.value_noise(64, 4, seed=6)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() == 0.0 and a.max() == 1.0 and a.dtype == np.float32
    # periodic lattice: the wrap-around neighbours differ as little as interior neighbours do
    assert np.abs(a[:, 0] - a[:, -1]).max() < 4 * np.abs(np.diff(a, axis=1)).max()
    h = S.value_noise(64, 8, seed=1, dtype=np.float16)
    assert h.dtype == np.float16


def test_camera_matrices_follow_glm_conventions():
    cam = S.camera_icosphere()
    fc = S.frame_constants(cam)
    vp = fc["viewProjMatrix"].reshape(4, 4).T.astype(np.float64)  # back to row-major
    # the origin projects to the screen centre, in front of the camera (depth in [0,1])
    h = vp @ np.array([0, 0, 0, 1.0])
    assert abs(h[0] / h[3]) < 1e-6 and abs(h[1] / h[3]) < 1e-6 and 0 < h[2] / h[3] < 1
    assert np.allclose(fc["viewPos"][:3], cam.eye)
    assert fc["tessRate"] == np.float32(1 / 8) and tuple(fc["viewportf"]) == (1920.0, 1080.0)
