"""The CPU oracle: known answers of the shader math, whole-frame invariants,
golden digests, and its FP64 adjoint against finite differences."""
import ctypes
import json
import math
import os

import numpy as np
import pytest

from tests.golden.cases import CASES, VARIANTS, outputs_digest, run_case, run_variant_digest
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ONE = L.TESSTABLE_COORD_MAX


def lib():
    from oracle.binding import lib as _lib
    return _lib()


def encode(w, u, v):
    return lib().tco_encode_barycentrics(w, u, v)


def decode(e):
    out = (ctypes.c_float * 3)()
    lib().tco_decode_barycentrics(e, out)
    return tuple(out)


def factors(a, b, c, eye=(0, 0, 0), near=0.01, h=1080.0, rate=0.25):
    f3 = ctypes.c_float * 3
    out = (ctypes.c_uint32 * 3)()
    lib().tco_tess_factors(f3(*a), f3(*b), f3(*c), f3(*eye), near, h, rate, out)
    return tuple(out)


def get_config(f, tv=(0, 1, 2)):
    ff = (ctypes.c_uint32 * 3)(*f)
    t = (ctypes.c_uint32 * 3)(*tv)
    c = lib().tco_get_config(ff, t)
    return c, tuple(t)


# ---------------------------------------------------------------------------
# tessellation.glsl known answers
# ---------------------------------------------------------------------------

def test_encode_corners_and_midpoints():
    assert encode(1, 0, 0) == 0
    assert encode(0, 1, 0) == ONE
    assert encode(0, 0, 1) == ONE << 16
    assert encode(0.5, 0.5, 0) == ONE // 2
    assert encode(0, 0.5, 0.5) == (ONE // 2) | ((ONE // 2) << 16)
    # largest component is fixed up so the three sum to exactly 1 (tessellation.glsl:51-57)
    e = encode(0.2, 0.7, 0.1)
    u, v = e & 0xFFFF, e >> 16
    assert v == int(0.1 * ONE + 0.5) and u == ONE - int(0.2 * ONE + 0.5) - v


def test_decode_is_exact_and_inverts_encode():
    rng = np.random.default_rng(0)
    for _ in range(200):
        u = int(rng.integers(0, ONE + 1))
        v = int(rng.integers(0, ONE - u + 1))
        w = decode(u | (v << 16))
        assert w[1] == u / ONE and w[2] == v / ONE and w[0] == (1 - u / ONE) - v / ONE
        assert encode(*w) == u | (v << 16)


def test_tess_factor_known_answers():
    # edge length 1 at distance 10: round(1/10 * 1080 * 0.25) = 27
    assert factors((0, 0, 10), (1, 0, 10), (0, 1, 10), rate=0.25)[0] == 27
    # clamped to [1, 32768]
    assert factors((0, 0, 1000), (1e-4, 0, 1000), (0, 1e-4, 1000)) == (1, 1, 1)
    assert factors((0, 0, 0.0), (5, 0, 0), (0, 5, 0), near=0.01)[0] == 32768
    # distance uses the nearer endpoint of each edge and the near plane
    f = factors((0, 0, 2), (1, 0, 20), (0, 1, 20), rate=1.0, h=100.0)
    assert f[0] == round(math.dist((0, 0, 2), (1, 0, 20)) / 2 * 100)
    # round half to even: 2.5 -> 2
    assert factors((0, 0, 1), (0.025, 0, 1), (0, 0.025, 1), rate=1.0, h=100.0)[0] == 2


def test_get_config_rotation_and_flip():
    lk = lambda x, y, z: x + 16 * y + 256 * z - 273
    c, tv = get_config((3, 2, 1))
    assert c == lk(3, 2, 1) and tv == (0, 1, 2)
    c, tv = get_config((1, 3, 2))   # max at y -> .yzx
    assert c == lk(3, 2, 1) and tv == (1, 2, 0)
    c, tv = get_config((2, 1, 3))   # max at z -> .zxy
    assert c == lk(3, 2, 1) and tv == (2, 0, 1)
    c, tv = get_config((3, 1, 2))   # z > y -> flipped
    assert c == lk(3, 1, 2) | 0x8000
    c, _ = get_config((2, 2, 1))    # tie: y checked first -> (2,1,2), flipped
    assert c == lk(2, 1, 2) | 0x8000


def test_split_factor_and_pass_count():
    sf = lambda f, s: lib().tco_split_factor(f, s)
    assert sf(12, 8) == 2 and sf(11, 8) == 1 and sf(100, 8) == 8 and sf(32768, 11) == 11 and sf(30, 2) == 2
    for s in range(2, 12):
        coord, n = ONE, 0
        while coord > s:
            coord //= s
            n += 1
        assert lib().tco_split_pass_count(s) == n
    assert lib().tco_split_pass_count(8) == 4


# ---------------------------------------------------------------------------
# whole frames
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_frame_digests(name, oracle):
    with open(os.path.join(ROOT, "tests", "golden", "oracle_frames.json")) as f:
        want = json.load(f)[name]
    assert run_case(name, oracle) and outputs_digest(run_case(name, oracle)[2]) == want


@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_golden_variant_digests(name, oracle):
    """PN + ripple, transient builds and raster batching outputs pinned by digest."""
    with open(os.path.join(ROOT, "tests", "golden", "oracle_frames.json")) as f:
        want = json.load(f)[name]
    assert run_variant_digest(name, oracle) == want


@pytest.mark.parametrize("name", sorted(CASES))
def test_frame_invariants(name, oracle):
    sc, st, out = run_case(name, oracle)
    e = oracle.entries
    rb, b = out["readback"], out["build"]
    ti = out["tempInstantiations"]
    full = (ti["clusterIdOffset"] >> 30) == 0
    parts = out["partTriangles"]
    # every instantiation is accounted for; instantiation slots follow generation order
    assert len(ti) == int(rb["numTempInstantiations"]) == int(b["tempInstantiateCounter"])
    pidx = ti["clusterIdOffset"][~full] & 0x3FFFFFFF
    assert np.array_equal(pidx, np.arange(len(pidx)))
    # vertex ranges are contiguous and ordered
    nvs = []
    for j in range(len(ti)):
        if full[j]:
            fc = out["fullClusters"][j]
            g = sc.geometries[sc.instances[fc["instanceID"]].geometry]
            nvs.append(int(g.clusters[fc["clusterID"]]["numVertices"]))
        else:
            p = parts[ti["clusterIdOffset"][j] & 0x3FFFFFFF]
            nvs.append(int(e[(p["triangleID_config"] >> 16) & 0x7FFF]["numVertices"]))
    starts = ti["vertexBufferAddress"] // 12
    assert np.array_equal(starts, np.concatenate([[0], np.cumsum(nvs)[:-1]]).astype(np.uint64))
    assert len(out["genVertices"]) == sum(nvs) == int(rb["numGenVertices"])
    # tessellated triangles = full cluster triangles + part pattern triangles
    tris = sum(int(sc.geometries[sc.instances[fc["instanceID"]].geometry].clusters[fc["clusterID"]]["numTriangles"])
               for fc in out["fullClusters"])
    tris += int(e[(parts["triangleID_config"] >> 16) & 0x7FFF]["numTriangles"].astype(np.int64).sum())
    assert tris == int(rb["numTotalTriangles"])
    # BLAS lists: per-instance sections holding exactly that instance's CLAS, in instantiation order
    bi = out["blasBuildInfos"]
    refs = out["blasClusterAddresses"]
    for i in range(len(sc.instances)):
        mine = out["tempClusterAddresses"][out["tempInstanceIDs"] == i]
        off = int(bi[i]["clusterReferences"]) // 8
        assert bi[i]["clusterReferencesCount"] == len(mine) and bi[i]["clusterReferencesStride"] == 8
        assert np.array_equal(refs[off:off + len(mine)], mine)
    # part triangles: positively oriented sub-triangles inside the unit triangle
    v = parts["vtxEncoded"].astype(np.int64)
    u_, w_ = v & 0xFFFF, v >> 16
    assert np.all(u_ + w_ <= ONE)
    area = (u_[:, 1] - u_[:, 0]) * (w_[:, 2] - w_[:, 0]) - (w_[:, 1] - w_[:, 0]) * (u_[:, 2] - u_[:, 0])
    assert np.all(area > 0)
    # the split tree tiles each base triangle (up to the 2^-15 quantisation of deep levels)
    key = parts["instanceID"].astype(np.int64) << 40 | parts["clusterID"].astype(np.int64) << 16 | (
        parts["triangleID_config"] & 0xFFFF).astype(np.int64)
    if int(b["splitWriteCounter"]) == 0:
        # no splits: every part triangle is a whole base triangle
        assert np.all(area == ONE * ONE)
    sums = {}
    for k_, a_ in zip(key.tolist(), area.tolist()):
        sums[k_] = sums.get(k_, 0) + a_
    rel = np.abs(np.array(list(sums.values())) / (ONE * ONE) - 1.0)
    nothing_dropped = (int(rb["numPartTriangles"]) == len(parts)
                       and int(rb["numSplitTriangles"]) <= st.caps["maxSplitTriangles"])
    if nothing_dropped and len(parts):
        assert rel.max() < 2e-3, rel.max()


def test_fp32_vertices_close_to_fp64_twin(oracle):
    sc, st, out = run_case("icosphere2_split", oracle)
    ref = oracle.vertices_f64(st, len(out["genVertices"]))
    err = np.abs(out["genVertices"].astype(np.float64) - ref).max()
    assert err < 1e-5 * 2.1  # bounding-box diagonal of a unit sphere with displacement


# ---------------------------------------------------------------------------
# FP64 adjoint vs central differences (tessellation decisions frozen)
# ---------------------------------------------------------------------------

def test_fp64_adjoint_matches_finite_differences(oracle):
    from oracle.binding import lib as olib
    sc, st, out = run_case("icosphere2_split", oracle)
    g = sc.geometries[0]
    tex = sc.textures[0].texels.astype(np.float64)
    P = g.positions.astype(np.float64).copy()
    N = g.normals.astype(np.float64).copy()
    T = tex.copy()
    nverts = len(out["genVertices"])
    rng = np.random.default_rng(3)
    target = out["genVertices"].astype(np.float64) + rng.normal(0, 0.01, (nverts, 3))
    pp = (ctypes.c_void_p * 1)(P.ctypes.data)
    nn = (ctypes.c_void_p * 1)(N.ctypes.data)
    tt = (ctypes.c_void_p * 1)(T.ctypes.data)

    def loss():
        v = np.zeros((nverts, 3))
        olib().tco_generate_vertices_f64_params(ctypes.byref(oracle.table), ctypes.byref(st.args), pp, nn, tt,
                                                v.ctypes.data)
        return float(((v - target) ** 2).sum()), v

    L0, v0 = loss()
    grad_v = 2 * (v0 - target)
    dP = np.zeros_like(P)
    dN = np.zeros_like(N)
    dT = np.zeros_like(T)
    olib().tco_backward_f64(ctypes.byref(oracle.table), ctypes.byref(st.args), grad_v.ctypes.data,
                            (ctypes.c_void_p * 1)(dP.ctypes.data), (ctypes.c_void_p * 1)(dN.ctypes.data),
                            (ctypes.c_void_p * 1)(dT.ctypes.data))
    h = 1e-3
    picks = [("P", P, dP, i) for i in rng.choice(P.size, 8, replace=False)]
    picks += [("N", N, dN, i) for i in rng.choice(N.size, 8, replace=False)]
    touched = np.flatnonzero(dT.reshape(-1))
    picks += [("T", T, dT, i) for i in rng.choice(touched, 8, replace=False)]
    for name, arr, grad, i in picks:
        flat = arr.reshape(-1)
        old = flat[i]
        flat[i] = old + h
        lp, _ = loss()
        flat[i] = old - h
        lm, _ = loss()
        flat[i] = old
        fd = (lp - lm) / (2 * h)
        an = grad.reshape(-1)[i]
        assert abs(fd - an) <= 1e-4 * max(1.0, abs(fd)), (name, i, fd, an)


def test_hit_decode_properties(oracle):
    """Hit-time decode (render_raytrace_clusters.rchit.glsl:131-214): full-
    cluster hits keep their barycentrics, part-triangle hits land on the base
    triangle (weights in [0, 1] summing to 1), a hit on a table vertex maps to
    that vertex composed with the part's corners, and malformed hits report
    their status."""
    from vk_tessellated_clusters_gb300.hits import sample_hits
    sc = S.scene_batched(num_instances=8, map_size=64)
    caps = L.default_caps(visible_bits=14, part_bits=17, split_bits=14, vertex_bits=20, megs=64)
    st, _ = oracle.frame(sc, S.camera_orbit(7), caps, L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS)
    out = st.outputs(oracle.entries)
    hits = sample_hits(out, sc, oracle.entries, 2000, seed=5, bad=40)
    got = oracle.decode_hits(st, hits)
    ok = got["status"] == L.HIT_OK
    assert ok[:2000].all() and (got["status"][2000:] != L.HIT_OK).all()
    assert set(np.unique(got["status"][2000:])) == {L.HIT_UNSUPPORTED_MODE, L.HIT_OUT_OF_RANGE}
    mode = hits["clusterID"] >> 30
    fullh = ok & (mode == 0)
    parth = ok & (mode == 1)
    assert fullh.any() and parth.any()
    w = np.stack([(np.float32(1) - hits["barycentrics"][:, 0]) - hits["barycentrics"][:, 1],
                  hits["barycentrics"][:, 0], hits["barycentrics"][:, 1]], 1).astype(np.float32)
    assert (got["barycentrics"][fullh] == w[fullh]).all()
    assert (got["clusterID"][fullh] == hits["clusterID"][fullh]).all()
    b = got["barycentrics"][parth].astype(np.float64)
    assert (b > -1e-6).all() and (b < 1 + 1e-6).all() and np.abs(b.sum(1) - 1).max() < 1e-5
    # vertex indices are the base triangle's
    for h in np.flatnonzero(ok)[:200]:
        geo = sc.geometries[sc.instances[int(hits["instanceID"][h])].geometry]
        cl = geo.clusters[got["clusterID"][h]]
        tri = geo.local_triangles[cl["firstLocalTriangle"] + 3 * got["triangleID"][h]:][:3].astype(np.int64)
        assert list(got["vertexIndices"][h]) == list(tri + int(cl["firstLocalVertex"]))
    # a hit on the micro-triangle's first corner is that table vertex in the part's corners
    p = int(np.flatnonzero(parth)[0])
    h1 = hits[p:p + 1].copy()
    h1["barycentrics"] = (0.0, 0.0)
    g1 = oracle.decode_hits(st, h1)[0]
    part = out["partTriangles"][int(h1["clusterID"][0]) & 0x3FFFFFFF]
    cfg = int(part["triangleID_config"]) >> 16
    e = oracle.entries[cfg & 0x7FFF]
    tri = int(oracle.raw.triangles[int(e["firstTriangle"]) + int(h1["triangleID"][0])])
    idx = [tri & 0xFF, (tri >> 8) & 0xFF, (tri >> 16) & 0xFF]
    if cfg & 0x8000:
        idx[1], idx[2] = idx[2], idx[1]
    vtx = int(oracle.raw.vertices[int(e["firstVertex"]) + idx[0]])
    a, bb = (vtx & 0xFFFF) / 32768.0, (vtx >> 16) / 32768.0
    sub = np.array([1 - a - bb, a, bb]) if not cfg & 0x8000 else np.array([a, 1 - a - bb, bb])
    corners = np.array([[1 - ((c & 0xFFFF) + (c >> 16)) / 32768.0, (c & 0xFFFF) / 32768.0, (c >> 16) / 32768.0]
                        for c in (int(x) for x in part["vtxEncoded"])])
    assert np.allclose(g1["barycentrics"], sub @ corners, atol=1e-6)



def _ripple_constants(cam, amplitude=0.02):
    fc = S.frame_constants(cam)
    fc["animationRippleAmplitude"] = amplitude
    fc["animationRippleFrequency"] = 8.0
    fc["animationRippleSpeed"] = 1.5
    fc["animationState"] = 0.7
    return fc


def test_pn_and_ripple_restatement(oracle):
    """PN displacement (displacement.glsl:47-104) and the ripple
    (:106-120) change generated vertices only: every integer output equals
    the plain frame's; PN moves part vertices of a curved mesh by a fraction
    of its size (flat meshes and full clusters keep theirs); a zero-amplitude
    ripple changes nothing and a small one moves vertices by at most
    amplitude x geometry size."""
    caps = L.default_caps(visible_bits=14, part_bits=17, split_bits=14, vertex_bits=21, megs=64)
    flags = L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS
    ints = ("visibleClusters", "partTriangles", "tempInstantiations", "tempInstanceIDs", "blasBuildInfos")
    # PN on a curved mesh close up (every vertex of the frame is a part vertex)
    ico = S.scene_icosphere(subdivisions=2, map_size=64)
    near = S.Camera(eye=(0.0, 0.0, 1.3), center=(0.0, 0.0, 0.0), tess_rate_pixels=2.0)
    base = oracle.frame(ico, near, caps, flags)[0].outputs(oracle.entries)
    pn = oracle.frame(ico, near, caps, flags | L.FLAG_PN)[0].outputs(oracle.entries)
    for f in ints:
        assert pn[f].tobytes() == base[f].tobytes(), f
    d = np.abs(pn["genVertices"].astype(np.float64) - base["genVertices"]).max(axis=1)
    assert (d > 0).mean() > 0.5 and d.max() < 0.05 * float(np.linalg.norm(ico.geometries[0].hi - ico.geometries[0].lo))
    # ripple on the batched scene (full clusters and parts)
    sc = S.scene_batched(num_instances=8, map_size=64)
    cam = S.camera_orbit(7)
    base = oracle.frame(sc, cam, caps, flags)[0].outputs(oracle.entries)
    size = max(float(np.linalg.norm(g.hi - g.lo)) for g in sc.geometries)
    for amp in (0.0, 0.02):
        out = oracle.frame(sc, _ripple_constants(cam, amp), caps, flags | L.FLAG_RIPPLE)[0].outputs(oracle.entries)
        for f in ints:
            assert out[f].tobytes() == base[f].tobytes(), (amp, f)
        d = np.abs(out["genVertices"].astype(np.float64) - base["genVertices"]).max()
        assert (d == 0) if amp == 0 else (0 < d <= amp * size * 1.001)


@pytest.mark.parametrize("which", ["icosphere", "batched"])
def test_transient_builds_restatement(oracle, which):
    """cluster_classify with 1X and 2X transient builds
    (cluster_classify.comp.glsl:254-905) against the same frame without them:
    the tessellated triangle total is unchanged; every 2X batch's vertices
    equal the part instantiation's vertices of the same base triangle; a 1X
    subset lists the cluster's untessellated triangles with their local
    indices; ClasBuildInfo fields follow the shader; BLAS lists hold every
    template instantiation, then the transient builds."""
    if which == "icosphere":
        sc, cam, last = S.scene_icosphere(), S.camera_icosphere(), None
    else:
        sc, cam, last = S.scene_batched(num_instances=24, map_size=64), S.camera_orbit(0), S.camera_orbit(59)
    caps = L.default_caps(visible_bits=16, part_bits=18, split_bits=14, vertex_bits=21, megs=256)
    flags = L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS
    base = oracle.frame(sc, cam, caps, flags, camera_last=last)[0].outputs(oracle.entries)
    st, _ = oracle.frame(sc, cam, caps, flags | L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X, camera_last=last)
    out = st.outputs(oracle.entries)
    rb, b = out["readback"], out["build"]
    assert int(rb["numTotalTriangles"]) == int(base["readback"]["numTotalTriangles"])
    tb = out["transBuilds"]
    modes = tb["clusterID"] >> 30
    assert (modes == L.RT_CLUSTER_MODE_1X_SUBSET_CLUSTER).any() and (modes == L.RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED).any()
    assert int(rb["numTransBuilds"]) == len(tb) == int(b["transBuildCounter"])
    assert int(rb["numBlasClusters"]) == len(tb) + len(out["tempInstantiations"])
    assert int(b["dualPartTriangleCounter"]) & 0xFFFFFFFF == int(b["partTriangleCounter"])
    assert int(rb["numTransPartTriangles"]) == int(b["dualPartTriangleCounter"]) >> 32
    assert (tb["baseGeometryIndexAndFlags"] == 4 << 29).all() and (tb["indexBufferStride"] == 1).all()
    assert (tb["vertexBufferStride"] == 12).all() and ((tb["packed"] >> 24) == 1).all()
    nv = (tb["packed"] >> 9) & 0x1FF
    assert (tb["indexBuffer"] == tb["vertexBuffer"] + nv * 12).all()
    # the base frame's part instantiations by (instance, cluster, triangle)
    ti, parts, gvb = base["tempInstantiations"], base["partTriangles"], base["genVertices"]
    part_verts = {}
    for j in np.flatnonzero((ti["clusterIdOffset"] >> 30) == L.RT_CLUSTER_MODE_SINGLE_TESSELLATED):
        p = parts[int(ti[j]["clusterIdOffset"]) & 0x3FFFFFFF]
        cfg = (int(p["triangleID_config"]) >> 16) & 0x7FFF
        key = (int(p["instanceID"]), int(p["clusterID"]), int(p["triangleID_config"]) & 0xFFFF)
        v0 = int(ti[j]["vertexBufferAddress"]) // 12
        part_verts[key] = gvb[v0:v0 + int(oracle.entries[cfg]["numVertices"])]
    gv, raw, idx = out["genVertices"], out["transParts"], out["transIndices"]
    ppos = ipos = 0
    checked = 0
    for r, inst in zip(tb, out["transInstanceIDs"]):
        mode, ntri = int(r["clusterID"]) >> 30, int(r["packed"]) & 0x1FF
        slots = 3 if mode == L.RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED else (8 + ntri + 23) // 24
        rec = raw[ppos:ppos + 24 * slots]
        ppos += 24 * slots
        nidx = 96 if mode == L.RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED else (ntri * 3 + 11) // 12 * 12
        ib = idx[ipos:ipos + nidx]
        ipos += nidx
        hdr = rec[:8].view(np.uint32)
        assert int(hdr[0]) == int(inst)
        geo = sc.geometries[sc.instances[int(inst)].geometry]
        cl = geo.clusters[int(hdr[1])]
        lt = geo.local_triangles[int(cl["firstLocalTriangle"]):]
        v0 = int(r["vertexBuffer"]) // 12
        if mode == L.RT_CLUSTER_MODE_1X_SUBSET_CLUSTER:
            tris = rec[8:8 + ntri]
            assert (np.diff(tris.astype(int)) > 0).all() and ntri > 1
            assert (ib[:3 * ntri].reshape(-1, 3) == lt.reshape(-1, 3)[tris]).all() and not ib[3 * ntri:].any()
            continue
        m16 = rec[8:8 + 2 * 32].view(np.uint16)[:ntri]
        assert not rec[8 + 2 * ntri:].any() and not ib[3 * ntri:].any()
        rels = {}
        for e in m16:
            rels.setdefault(int(e) & 0xFF, len(rels))
        for tri, rel in rels.items():
            want = part_verts[(int(inst), int(hdr[1]), tri)]
            got = gv[v0 + 6 * rel:v0 + 6 * rel + len(want)]
            assert got.tobytes() == want.tobytes()
            checked += 1
    assert checked > 100 and ppos == len(raw) and ipos == len(idx)
    # BLAS lists: the transient builds follow the instance's template instantiations
    bi, lists = out["blasBuildInfos"], out["blasClusterAddresses"]
    for i in np.unique(out["transInstanceIDs"])[:8]:
        start = int(bi[i]["clusterReferences"]) // 8
        n = int(bi[i]["clusterReferencesCount"])
        mine = out["transClusterAddresses"][out["transInstanceIDs"] == i]
        assert (lists[start + n - len(mine):start + n] == mine).all()


def test_raster_batches_restatement(oracle):
    """Raster batching (render_raster_clusters_batched.task.glsl:115-215,
    .mesh.glsl:141-435): per group of 32 parts the batches are consecutive,
    within 96 vertices and 121 triangles, and maximal (the next part would not
    fit); vertex and triangle arrays follow part order; indices stay inside
    their batch; world positions are the instantiation's vertices taken to
    world space and clip positions those taken through viewProjMatrix."""
    sc = S.scene_batched(num_instances=8, map_size=64)
    cam = S.camera_orbit(7)
    caps = L.default_caps(visible_bits=14, part_bits=15, split_bits=12, vertex_bits=20, megs=64)
    st, _ = oracle.frame(sc, cam, caps, L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS)
    out = st.outputs(oracle.entries)
    r = oracle.raster_batches(st)
    parts = out["partTriangles"]
    n = len(parts)
    assert n > 100
    cfg = (parts["triangleID_config"] >> 16) & 0x7FFF
    nv = oracle.entries[cfg]["numVertices"].astype(np.int64)
    nt = oracle.entries[cfg]["numTriangles"].astype(np.int64)
    nb, tv, tt = r["counts"]
    assert tv == nv.sum() and tt == nt.sum() and nb == len(r["batches"])
    b = r["batches"]
    assert (b["numVertices"] <= 96).all() and (b["numTriangles"] <= 121).all()
    assert b["firstPart"][0] == 0 and (np.diff(b["firstPart"].astype(np.int64)) == b["partCount"][:-1]).all()
    assert int(b["firstPart"][-1]) + int(b["partCount"][-1]) == n
    cv, ct = np.concatenate([[0], np.cumsum(nv)]), np.concatenate([[0], np.cumsum(nt)])
    for rec in b:
        p0, pc = int(rec["firstPart"]), int(rec["partCount"])
        assert p0 // 32 == (p0 + pc - 1) // 32  # within one group of 32
        assert rec["firstVertex"] == cv[p0] and rec["numVertices"] == cv[p0 + pc] - cv[p0]
        assert rec["firstTriangle"] == ct[p0] and rec["numTriangles"] == ct[p0 + pc] - ct[p0]
        nxt = p0 + pc
        if nxt < n and nxt % 32:  # maximal: the next part of the group does not fit
            assert cv[nxt + 1] - cv[p0] > 96 or ct[nxt + 1] - ct[p0] > 121
        tri = r["indices"][int(rec["firstTriangle"]):int(rec["firstTriangle"]) + int(rec["numTriangles"])]
        assert (tri < rec["numVertices"]).all()
    # positions: the part instantiations' vertices (object space) taken to world and clip space
    ti = out["tempInstantiations"]
    sel = np.flatnonzero((ti["clusterIdOffset"] >> 30) == L.RT_CLUSTER_MODE_SINGLE_TESSELLATED)[:50]
    for j in sel:
        p = int(ti[j]["clusterIdOffset"]) & 0x3FFFFFFF
        v0 = int(ti[j]["vertexBufferAddress"]) // 12
        obj = out["genVertices"][v0:v0 + nv[p]].astype(np.float64)
        inst = sc.instances[int(out["tempInstanceIDs"][j])]
        m = np.asarray(inst.world, np.float64)  # row-major: p' = m @ (p, 1)
        w = r["worldPositions"][cv[p]:cv[p + 1]].astype(np.float64)
        np.testing.assert_allclose(w, obj @ m[:3, :3].T + m[:3, 3], rtol=0, atol=1e-4)
        fc = S.frame_constants(cam)
        vp = np.asarray(fc["viewProjMatrix"]["m"] if fc["viewProjMatrix"].dtype.names else fc["viewProjMatrix"],
                        np.float64).reshape(4, 4).T
        c = r["clipPositions"][cv[p]:cv[p + 1]].astype(np.float64)
        np.testing.assert_allclose(c, np.c_[w, np.ones(len(w))] @ vp.T, rtol=1e-5, atol=1e-4)


def test_factor_one_shortcut_never_changes_a_factor():
    """The classify kernel skips an edge's square root when
    (|d|^2 * spl^2) * (viewportH * tessRate)^2 < 2.25 * (1 - 1e-5) in single
    precision and takes the factor as 1 (tc_device.cuh, edge_factor). Restated
    here in float32 (each operation rounded like the GPU's) on seeded edges
    spread over [0, 3] and packed around the 1.5 threshold: wherever the
    shortcut answers, the full evaluation rint(((sqrt(s) * spl) * vh) * rate)
    clamped to [1, 32768] is 1 as well."""
    f32 = np.float32
    rng = np.random.default_rng(7)
    bound = f32(2.2499775)
    n, claims = 500_000, 0
    for it, (vh, rate) in enumerate([(1080.0, 0.25), (2160.0, 0.25), (1080.0, 0.125), (720.0, 1.0)]):
        vh, rate = f32(vh), f32(rate)
        x_target = 1.5 + rng.uniform(-3e-5, 3e-5, n) if it % 2 else rng.uniform(0.0, 3.0, n)
        spl = rng.uniform(1e-4, 1.0, n).astype(f32)
        e = (x_target / (spl.astype(np.float64) * float(vh) * float(rate))).astype(f32)
        s = (e.astype(np.float64) ** 2 * rng.uniform(0.999, 1.001, n)).astype(f32)
        k = f32(vh * rate)
        t = (s * (spl * spl)) * f32(k * k)
        claim = t < bound
        x = ((np.sqrt(s) * spl) * vh) * rate
        f = np.minimum(np.maximum(np.rint(x), f32(1)), f32(32768))
        assert not np.any(claim & (f != 1))
        claims += int(claim.sum())
    assert claims > n  # the shortcut answers for a good share of the edges


def test_cluster_factor_one_shortcut_never_changes_a_factor():
    """The classify kernel skips a cluster's distances, their reciprocals and
    every edge's square root when each edge passes
    |d|^2 * (viewportH * tessRate)^2 < 2.25 * (1 - 1e-5) * max(near^2, min(da^2, db^2))
    in single precision (tc_device.cuh, edge_factor_one_sq) and takes all its
    factors as 1. Restated in float32 on seeded edges packed around the
    threshold: wherever the test passes, the full evaluation (the distances'
    roots, the reciprocal of the clamped nearer one, the edge's root, rint of the
    product, clamp) gives 1 as well."""
    f32 = np.float32
    rng = np.random.default_rng(11)
    bound = f32(2.2499775)
    n, claims = 500_000, 0
    for it, (vh, rate, near) in enumerate([(1080.0, 0.25, 0.01), (2160.0, 0.25, 0.1), (1080.0, 0.125, 0.01),
                                           (720.0, 1.0, 2.0)]):
        vh, rate, near = f32(vh), f32(rate), f32(near)
        da2 = (rng.uniform(0.0, 4.0, n) ** 4).astype(f32)  # squared distances of the two ends
        db2 = (da2.astype(np.float64) * rng.uniform(0.9, 1.1, n)).astype(f32)
        da, db = np.sqrt(da2), np.sqrt(db2)
        m = np.minimum(da, db)
        q = np.where(near > m, near, np.where(da <= db, da, db))
        spl = f32(1) / q
        x_target = 1.5 + rng.uniform(-3e-5, 3e-5, n) if it % 2 else rng.uniform(0.0, 3.0, n)
        e = (x_target / (spl.astype(np.float64) * float(vh) * float(rate))).astype(f32)
        s2 = (e.astype(np.float64) ** 2 * rng.uniform(0.999, 1.001, n)).astype(f32)
        k = f32(vh * rate)
        claim = s2 * f32(k * k) < bound * np.maximum(f32(near * near), np.minimum(da2, db2))
        x = ((np.sqrt(s2) * spl) * vh) * rate
        f = np.minimum(np.maximum(np.rint(x), f32(1)), f32(32768))
        assert not np.any(claim & (f != 1))
        claims += int(claim.sum())
    assert claims > n
