"""Small seeded frames whose oracle outputs are pinned by digest."""
import hashlib

import numpy as np

from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import scene as S

FLAGS = L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS


def _caps(**kw):
    c = L.default_caps(visible_bits=14, part_bits=17, split_bits=14, vertex_bits=20, megs=64)
    c.update(kw)
    return c


CASES = {
    "icosphere3_far": (lambda: S.scene_icosphere(subdivisions=3, map_size=128),
                       lambda: S.Camera(eye=(0.0, 0.0, 3.0), center=(0.0, 0.0, 0.0), tess_rate_pixels=8.0), _caps()),
    "icosphere2_split": (lambda: S.scene_icosphere(subdivisions=2, map_size=64),
                         lambda: S.Camera(eye=(0.0, 0.0, 1.1), center=(0.0, 0.0, 0.0), tess_rate_pixels=8.0), _caps()),
    "batched8": (lambda: S.scene_batched(num_instances=8, map_size=64),
                 lambda: S.camera_orbit(7), _caps()),
}

FIELDS = ("instanceStates", "visibleClusters", "partTriangles", "tempInstantiations", "tempInstanceIDs",
          "tempClusterAddresses", "blasBuildInfos", "blasClusterAddresses", "fullClusters", "genVertices")


def outputs_digest(out: dict) -> dict:
    d = {f: hashlib.sha256(np.ascontiguousarray(out[f]).tobytes()).hexdigest() for f in FIELDS}
    d["readback"] = hashlib.sha256(out["readback"].tobytes()).hexdigest()
    d["counts"] = {k: int(out["readback"][k]) for k in ("numVisibleClusters", "numFullClusters", "numPartTriangles",
                                                         "numSplitTriangles", "numTotalTriangles", "numGenVertices")}
    return d


def run_case(name, oracle=None):
    from oracle.binding import Oracle
    mk_scene, mk_cam, caps = CASES[name]
    ora = oracle or Oracle()
    sc = mk_scene()
    st, runs = ora.frame(sc, mk_cam(), caps, FLAGS)
    return sc, st, st.outputs(ora.entries)


def run_case_digest(name, oracle=None):
    return outputs_digest(run_case(name, oracle)[2])


def _ripple(cam):
    fc = S.frame_constants(cam)
    fc["animationRippleAmplitude"], fc["animationRippleFrequency"] = 0.02, 8.0
    fc["animationRippleSpeed"], fc["animationState"] = 1.5, 0.7
    return fc


# the reference's optional shader paths: PN + ripple, 1X / 2X transient builds,
# and the raster batching of the frame's parts
VARIANTS = {
    "batched8_transient": (lambda: S.scene_batched(num_instances=8, map_size=64), lambda: S.camera_orbit(0),
                           _caps(), FLAGS | L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X),
    "icosphere_transient_pn_ripple": (lambda: S.scene_icosphere(), lambda: _ripple(S.camera_icosphere()),
                                      _caps(), FLAGS | L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X | L.FLAG_PN
                                      | L.FLAG_RIPPLE),
    "icosphere2_pn_ripple_near": (lambda: S.scene_icosphere(subdivisions=2, map_size=64),
                                  lambda: _ripple(S.Camera(eye=(0.0, 0.0, 1.3), center=(0.0, 0.0, 0.0),
                                                           tess_rate_pixels=2.0)), _caps(),
                                  FLAGS | L.FLAG_PN | L.FLAG_RIPPLE),
}

VARIANT_FIELDS = ("transBuilds", "transInstanceIDs", "transClusterAddresses", "transParts", "transIndices")
RASTER_FIELDS = ("batches", "clipPositions", "worldPositions", "indices", "primitiveIDs")


def run_variant_digest(name, oracle=None):
    from oracle.binding import Oracle
    mk_scene, mk_cam, caps, flags = VARIANTS[name]
    ora = oracle or Oracle()
    st, _ = ora.frame(mk_scene(), mk_cam(), caps, flags)
    out = st.outputs(ora.entries)
    d = outputs_digest(out)
    for f in VARIANT_FIELDS:
        if f in out:
            d[f] = hashlib.sha256(np.ascontiguousarray(out[f]).tobytes()).hexdigest()
    r = ora.raster_batches(st)
    for f in RASTER_FIELDS:
        d["raster_" + f] = hashlib.sha256(np.ascontiguousarray(r[f]).tobytes()).hexdigest()
    d["raster_counts"] = list(r["counts"])
    return d
