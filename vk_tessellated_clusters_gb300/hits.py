"""Seeded ray-tracing hits on a built frame (hit-decode tests and bench): hits on
accepted instantiations (full clusters and part triangles) and transient
builds (1X subsets, 2X batches), as a cluster ray tracer reports them, plus
malformed ones."""
import numpy as np

from . import layouts as L


def sample_hits(out: dict, scene, entries: np.ndarray, n: int, seed: int = 0, bad: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ti, ids = out["tempInstantiations"], out["tempInstanceIDs"]
    full = out["fullClusters"]
    mode = ti["clusterIdOffset"] >> 30
    full_slot = np.cumsum(mode == 0) - 1  # rank of each full instantiation among the full ones
    tb = out.get("transBuilds")
    ntrans = 0 if tb is None else len(tb)
    hits = np.zeros(n + bad, L.Hit)
    slots = rng.integers(0, len(ti) + ntrans, n)
    for k, s in enumerate(slots):
        if s >= len(ti):  # a transient build: its clusterID and triangle count
            r = tb[s - len(ti)]
            u, v = rng.random(2, dtype=np.float32)
            if u + v > 1:
                u, v = np.float32(1) - u, np.float32(1) - v
            hits[k] = (int(out["transInstanceIDs"][s - len(ti)]), int(r["clusterID"]),
                       int(rng.integers(0, int(r["packed"]) & 0x1FF)), (u, v), 0)
            continue
        inst = int(ids[s])
        if mode[s] == L.RT_CLUSTER_MODE_FULL_CLUSTER:
            cid = int(full[full_slot[s]]["clusterID"])
            geo = scene.geometries[scene.instances[inst].geometry]
            ntri = int(geo.clusters[cid]["numTriangles"])
            hit_cid = cid
        else:
            part = out["partTriangles"][int(ti["clusterIdOffset"][s]) & 0x3FFFFFFF]
            cfg = int(part["triangleID_config"]) >> 16
            ntri = int(entries[cfg & 0x7FFF]["numTriangles"])
            hit_cid = int(ti["clusterIdOffset"][s])
        u, v = rng.random(2, dtype=np.float32)
        if u + v > 1:
            u, v = np.float32(1) - u, np.float32(1) - v
        hits[k] = (inst, hit_cid, int(rng.integers(0, ntri)), (u, v), 0)
    for k in range(n, n + bad):  # transient-build modes, foreign indices
        kind = k % 4
        h = hits[rng.integers(0, n)].copy()
        if kind == 0:
            h["clusterID"] = (L.RT_CLUSTER_MODE_1X_SUBSET_CLUSTER << 30) | 1
        elif kind == 1:
            h["clusterID"] = (L.RT_CLUSTER_MODE_SINGLE_TESSELLATED << 30) | 0x3FFFFFFF
        elif kind == 2:
            h["triangleID"] = 4096
        else:
            h["instanceID"] = len(scene.instances) + 7
        hits[k] = h
    return hits
