"""Comparison of two frames' outputs (GPU vs oracle, or GPU vs GPU).

Integer/index outputs (counters, cluster lists, part and split records with
their encoded barycentrics and configs, instantiation arguments, BLAS lists)
must be bit-exact. Generated vertex positions: GPU vs GPU bit-exact (same
kernels); GPU vs oracle within |dp| <= 1e-5 x the smallest mesh bounding-box
diagonal (`vertex_tolerance`), because the GPU evaluates the part-triangle
vertices in per-part affine form with fused multiply-adds while the oracle
restates the reference's two-level interpolation without contraction.
"""
from __future__ import annotations

import numpy as np

COUNTER_FIELDS = ("numRenderInstances", "visibleClusterCounter", "fullClusterCounter", "partTriangleCounter",
                  "dualPartTriangleCounter", "splitTriangleCounter", "splitReadCounter", "splitWriteCounter",
                  "splitPass", "splitPassStart", "splitPassEnd", "genVertexCounter", "genClusterCounter",
                  "genClusterDataCounter", "dispatchClassify", "dispatchTriangleSplit", "drawFullClusters",
                  "drawPartTriangles", "dispatchClusterInstantiate", "dispatchTriangleInstantiate",
                  "dispatchBlasTempInsert", "dispatchBlasTransInsert", "positionTruncateBitCount",
                  "blasClusterCounter", "tempInstantiateCounter", "transBuildCounter", "numBlasReservedSizes",
                  "viewPos")

ARRAY_FIELDS = ("instanceStates", "visibleClusters", "splitTriangles", "partTriangles", "tempInstantiations",
                "tempInstanceIDs", "tempClusterAddresses", "blasBuildInfos", "blasClusterAddresses", "fullClusters",
                "transBuilds", "transInstanceIDs", "transClusterAddresses", "transParts", "transIndices")


def _first_diff(a: np.ndarray, b: np.ndarray):
    ra = a.view(np.uint8).reshape(len(a), -1) if len(a) else a.view(np.uint8)
    rb = b.view(np.uint8).reshape(len(b), -1) if len(b) else b.view(np.uint8)
    rows = np.flatnonzero((ra != rb).any(axis=1)) if ra.ndim == 2 else np.array([], int)
    return (int(rows[0]), a[rows[0]], b[rows[0]], len(rows)) if rows.size else None


def diff_outputs(got: dict, want: dict, fields=ARRAY_FIELDS, vertex_tol: float | None = None) -> list[str]:
    errs = []
    gb, wb = got["build"], want["build"]
    for f in COUNTER_FIELDS:
        if gb[f].tobytes() != wb[f].tobytes():
            errs.append(f"SceneBuilding.{f}: got {gb[f]} want {wb[f]}")
    if got["readback"].tobytes() != want["readback"].tobytes():
        for f in got["readback"].dtype.names:
            if got["readback"][f].tobytes() != want["readback"][f].tobytes():
                errs.append(f"Readback.{f}: got {got['readback'][f]} want {want['readback'][f]}")
    for f in fields:
        if f not in want:
            continue
        a, b = got[f], want[f]
        if a.shape != b.shape:
            errs.append(f"{f}: shape {a.shape} vs {b.shape}")
            continue
        d = _first_diff(a, b)
        if d:
            errs.append(f"{f}: {d[3]} rows differ, first at {d[0]}: got {d[1]} want {d[2]}")
    gv, wv = got["genVertices"], want["genVertices"]
    if gv.shape != wv.shape:
        errs.append(f"genVertices: shape {gv.shape} vs {wv.shape}")
    elif vertex_tol is not None:
        d = np.abs(gv.astype(np.float64) - wv.astype(np.float64)).max(axis=1) if len(gv) else np.zeros(0)
        if not np.isfinite(gv).all():
            errs.append("genVertices: non-finite values")
        elif d.size and d.max() > vertex_tol:
            bad = int(np.argmax(d))
            errs.append(f"genVertices: max |d| {d.max():.3e} > {vertex_tol:.3e} at {bad}: got {gv[bad]} want {wv[bad]}")
    elif gv.tobytes() != wv.tobytes():
        bad = np.flatnonzero((gv != wv).any(axis=1))
        errs.append(f"genVertices: {bad.size} vertices differ bitwise, first {bad[0]}: got {gv[bad[0]]} want {wv[bad[0]]}, "
                    f"max |d| {np.abs(gv.astype(np.float64) - wv).max():.3e}")
    return errs


def assert_same(got: dict, want: dict, what: str = "", fields=ARRAY_FIELDS, vertex_tol: float | None = None) -> None:
    errs = diff_outputs(got, want, fields, vertex_tol)
    assert not errs, (what + "\n" if what else "") + "\n".join(errs[:20])


def max_position_error(got: np.ndarray, ref64: np.ndarray) -> float:
    return float(np.abs(got.astype(np.float64) - ref64).max()) if len(got) else 0.0


def scene_diagonal(scene) -> float:
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    for g in scene.geometries:
        lo = np.minimum(lo, g.lo)
        hi = np.maximum(hi, g.hi)
    return float(np.linalg.norm(hi - lo))


def vertex_tolerance(scene) -> float:
    """1e-5 x the smallest mesh bounding-box diagonal of the scene (positions
    are in each mesh's object space)."""
    return 1e-5 * min(float(np.linalg.norm(g.hi - g.lo)) for g in scene.geometries)
