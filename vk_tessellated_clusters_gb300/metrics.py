"""Algorithmic byte counts per stage launch (the roofline numerators).

Bytes a stage must move at minimum for a given frame, counted from the frame's
outputs (compulsory reads of its inputs plus its writes), excluding the ~93 KB
tessellation table and per-item atomics:

  triangle_tess_template_instantiate, per accepted part triangle:
      24 (TessTriangleInfo read) + 32 (TemplateInstantiateInfo) + 4 (instance id)
      + 8 (CLAS address) + 12 * V_cfg (generated vertices)
    + 115 per distinct base triangle touched (3 x (12 pos + 12 normal + 8 uv)
      + 3 index bytes + 16 cluster header)
    + texel bytes: bytes_per_texel * min(4 * displaced vertices, texels) per map
  cluster_classify, per visible cluster:
      8 (ClusterInfo) + 16 (Cluster) + 12 * nv (positions) + 3 * nt (indices)
    + 24 per part/split triangle written
    + per accepted full cluster 44 (instantiation args) + 12 * nv (vertices)
      + 20 * nv (normal + uv reads)
  triangle_split (one pass): 24 per item read + 24 per child written
      + 48 per distinct base triangle (positions + indices + cluster header)
  clusters_cull: 8 per visible cluster written + 192 per instance read
  blas_setup_insertion: 32 per instance; blas_clusters_insert: 20 per CLAS
"""
from __future__ import annotations

import numpy as np

from . import layouts as L


def _cfg_index(part_tc: np.ndarray) -> np.ndarray:
    return (part_tc >> 16) & 0x7FFF


def instantiate_bytes(out: dict, entries: np.ndarray, scene) -> int:
    ti = out["tempInstantiations"]
    is_part = (ti["clusterIdOffset"] >> 30) == L.RT_CLUSTER_MODE_SINGLE_TESSELLATED
    pidx = (ti["clusterIdOffset"][is_part] & 0x3FFFFFFF).astype(np.int64)
    parts = out["partTriangles"][pidx]
    nv = entries["numVertices"][_cfg_index(parts["triangleID_config"])].astype(np.int64)
    b = int(len(parts)) * (24 + 32 + 4 + 8) + 12 * int(nv.sum())
    key = (parts["instanceID"].astype(np.uint64) << np.uint64(40)) | (parts["clusterID"].astype(np.uint64) << np.uint64(16)) \
        | (parts["triangleID_config"] & 0xFFFF).astype(np.uint64)
    b += 115 * int(np.unique(key).size)
    # texels per map
    inst_tex = np.array([i.displacement_index for i in scene.instances], np.int64)
    tex_of_part = inst_tex[parts["instanceID"].astype(np.int64)]
    for t, tx in enumerate(scene.textures):
        v = int(nv[tex_of_part == t].sum())
        b += tx.texels.dtype.itemsize * min(4 * v, tx.texels.size)
    return b


def _geometry_of_instances(scene) -> np.ndarray:
    return np.array([i.geometry for i in scene.instances], np.int64)


def classify_parts_written(out: dict) -> int:
    """Part triangles emitted by cluster_classify: they cover the whole base
    triangle, i.e. their three encoded corners are a permutation of
    (0,0), (1,0), (0,1)."""
    v = np.sort(out["partTriangles"]["vtxEncoded"], axis=1)
    corners = np.array([0, TC_ONE_U, TC_ONE_V], np.uint32)
    return int(np.count_nonzero((v == corners).all(axis=1)))


TC_ONE_U = L.TESSTABLE_COORD_MAX
TC_ONE_V = L.TESSTABLE_COORD_MAX << 16


def classify_bytes(out: dict, scene) -> int:
    vis = out["visibleClusters"]
    geo = _geometry_of_instances(scene)
    vg = geo[vis["instanceID"].astype(np.int64)]
    cid = vis["clusterID"].astype(np.int64)
    b = 24 * len(vis)
    for gi, g in enumerate(scene.geometries):
        cl = g.clusters[cid[vg == gi]]
        b += 12 * int(cl["numVertices"].astype(np.int64).sum()) + 3 * int(cl["numTriangles"].astype(np.int64).sum())
    ti = out["tempInstantiations"]
    full = (ti["clusterIdOffset"] >> 30) == 0
    nfull = int(np.count_nonzero(full))
    if nfull:
        ids = out["tempInstanceIDs"][full].astype(np.int64)
        addrs = ti["clusterTemplateAddress"][full]
        full_nv = 0
        for gi, g in enumerate(scene.geometries):
            sel = geo[ids] == gi
            if not sel.any():
                continue
            order = np.argsort(g.template_addresses)
            pos = np.minimum(np.searchsorted(g.template_addresses[order], addrs[sel]), len(order) - 1)
            full_nv += int(g.clusters["numVertices"][order[pos]].astype(np.int64).sum())
        b += nfull * 44 + (12 + 20) * full_nv
    b += 24 * (classify_parts_written(out) + max(int(out["build"]["splitTriangleCounter"]), 0))
    return b


def frame_tessellated_triangles(out: dict) -> int:
    return int(out["readback"]["numTotalTriangles"])
