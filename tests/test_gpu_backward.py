"""Differentiable path on the GPU: the frozen-frame forward reproduces the build,
and the hand-written backward matches the FP64 adjoint of the oracle and
central finite differences (FP64, h = 1e-3) on 64 random parameters."""
import ctypes

import numpy as np
import pytest

from tests.conftest import cuda_available
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import scene as S

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

FLAGS = L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS


def caps():
    return L.default_caps(visible_bits=14, part_bits=17, split_bits=14, vertex_bits=21, megs=256)


# reduced: subdivision 4, 256² map, a far camera mixing 59 full clusters and
# 1344 part triangles; icosphere_20480: the small plain frame at full size
# (icosphere of 20,480 triangles, 1024² fp32 map of 4 octaves, camera at
# distance 3, 8 px per segment), the frame the backward is specified on
CASES = {
    "reduced": dict(subdivisions=4, map_size=256,
                    cam=S.Camera(eye=(0.0, 0.0, 8.0), center=(0.0, 0.0, 0.0), tess_rate_pixels=8.0)),
    "icosphere_20480": dict(subdivisions=5, map_size=1024, cam=S.camera_icosphere()),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def setup(oracle, request):
    import torch
    from vk_tessellated_clusters_gb300.autograd import FrozenFrame, tessellate
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    case = CASES[request.param]
    sc = S.scene_icosphere(subdivisions=case["subdivisions"], map_size=case["map_size"])
    if request.param == "icosphere_20480":
        assert sc.total_triangles == 20480 and sc.textures[0].texels.shape == (1024, 1024)
    cam = case["cam"]
    pipe = TessellationPipeline(sc, caps(), FLAGS)
    pipe.set_cameras(cam)
    pipe.build("batched")
    built = pipe.outputs()
    frozen = FrozenFrame(pipe)
    # targets: same frame, displacement map of another seed
    tex = frozen.texels[0]
    orig = tex.detach().clone()
    with torch.no_grad():
        tex.copy_(torch.from_numpy(S.value_noise(case["map_size"], 4, seed=11)).to(tex.device))
    target = frozen.generate()
    with torch.no_grad():
        tex.copy_(orig)
    ref_state, _ = oracle.frame(sc, cam, caps(), FLAGS)
    return dict(sc=sc, pipe=pipe, frozen=frozen, built=built, target=target, ref_state=ref_state,
                tessellate=tessellate)


def test_frozen_forward_reproduces_the_build(setup):
    f = setup["frozen"]
    v = f.generate().cpu().numpy()
    assert v.shape == setup["built"]["genVertices"].shape
    assert v.tobytes() == setup["built"]["genVertices"].tobytes()
    assert (setup["built"]["tempInstantiations"]["clusterIdOffset"] >> 30 == 0).any()  # full clusters covered too


def _gpu_grads(setup):
    import torch
    f = setup["frozen"]
    for p in f.parameters():
        p.grad = None
    v = setup["tessellate"](f)
    loss = ((v - setup["target"]) ** 2).sum()
    loss.backward()
    return loss, v


def _fp64_adjoint(oracle, setup, grad_v):
    from oracle.binding import lib as olib
    st = setup["ref_state"]
    g = setup["sc"].geometries[0]
    dP = np.zeros(g.positions.shape)
    dN = np.zeros(g.normals.shape)
    dT = np.zeros(setup["sc"].textures[0].texels.shape)
    olib().tco_backward_f64(ctypes.byref(oracle.table), ctypes.byref(st.args), grad_v.ctypes.data,
                            (ctypes.c_void_p * 1)(dP.ctypes.data), (ctypes.c_void_p * 1)(dN.ctypes.data),
                            (ctypes.c_void_p * 1)(dT.ctypes.data))
    return dP, dN, dT


def test_gradients_match_fp64_adjoint(setup, oracle):
    """L = sum |v - t|^2 with t from a map of another seed: relative error of the
    whole FP32 gradient (positions, normals, texels) against the FP64 adjoint.
    (With this target v - t is parallel to the displacement direction, so the
    normal gradient is nearly zero; the next test checks every group alone.)"""
    _gpu_grads(setup)
    f, st = setup["frozen"], setup["ref_state"]
    v64 = oracle.vertices_f64(st, f.num_vertices)
    grad_v = 2 * (v64 - setup["target"].double().cpu().numpy())
    want = np.concatenate([a.reshape(-1) for a in _fp64_adjoint(oracle, setup, grad_v)])
    got = np.concatenate([x.grad.double().cpu().numpy().reshape(-1)
                          for x in (f.positions[0], f.normals[0], f.texels[0])])
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= 1e-4, rel


def test_each_gradient_group_matches_fp64_adjoint(setup, oracle):
    """A target offset by seeded noise gives every group (positions, normals,
    texels) a well-conditioned gradient; each must match the FP64 adjoint."""
    import torch
    f, st = setup["frozen"], setup["ref_state"]
    for p in f.parameters():
        p.grad = None
    v = setup["tessellate"](f)
    rng = np.random.default_rng(5)
    target = v.detach() + torch.from_numpy(rng.normal(0, 0.01, tuple(v.shape)).astype(np.float32)).to(v.device)
    ((v - target) ** 2).sum().backward()
    v64 = oracle.vertices_f64(st, f.num_vertices)
    grad_v = 2 * (v64 - target.double().cpu().numpy())
    for name, got, want in zip(("positions", "normals", "texels"), (f.positions[0], f.normals[0], f.texels[0]),
                               _fp64_adjoint(oracle, setup, grad_v)):
        got = got.grad.double().cpu().numpy()
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel <= 1e-4, (name, rel)


def test_gradients_match_central_differences(setup, oracle):
    """64 random parameters, central differences in FP64 on the frozen frame."""
    from oracle.binding import lib as olib
    _gpu_grads(setup)
    f, st = setup["frozen"], setup["ref_state"]
    g = setup["sc"].geometries[0]
    P = g.positions.astype(np.float64).copy()
    N = g.normals.astype(np.float64).copy()
    T = setup["sc"].textures[0].texels.astype(np.float64).copy()
    t64 = setup["target"].double().cpu().numpy()
    pp, nn, tt = ((ctypes.c_void_p * 1)(a.ctypes.data) for a in (P, N, T))

    def loss():
        v = np.zeros((f.num_vertices, 3))
        olib().tco_generate_vertices_f64_params(ctypes.byref(oracle.table), ctypes.byref(st.args), pp, nn, tt,
                                                v.ctypes.data)
        return ((v - t64) ** 2).sum()

    gp, gn, gt = (x.grad.double().cpu().numpy().reshape(-1) for x in (f.positions[0], f.normals[0], f.texels[0]))
    rng = np.random.default_rng(7)
    touched_t = np.flatnonzero(gt)
    picks = [(P, gp, i) for i in rng.choice(P.size, 22, replace=False)]
    picks += [(N, gn, i) for i in rng.choice(N.size, 21, replace=False)]
    picks += [(T, gt, i) for i in rng.choice(touched_t, 21, replace=False)]
    assert len(picks) == 64
    h = 1e-3
    worst = 0.0
    for arr, grad, i in picks:
        flat = arr.reshape(-1)
        old = flat[i]
        flat[i] = old + h
        lp = loss()
        flat[i] = old - h
        lm = loss()
        flat[i] = old
        fd = (lp - lm) / (2 * h)
        worst = max(worst, abs(grad[i] - fd) / max(abs(fd), 1e-2))
    assert worst <= 1e-3, worst
