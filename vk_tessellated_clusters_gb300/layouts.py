"""numpy / ctypes mirrors of the C ABI layouts in include/tc_tessellation.h.

The structured dtypes describe the device buffers of the reference's buffer
protocol (shaders/shaderio_scene.h, shaders/shaderio_building.h,
shaders/shaderio.h); their item sizes are asserted against the C header's
static_asserts so a layout drift fails at import time.
"""
from __future__ import annotations

import ctypes

import numpy as np

# ---------------------------------------------------------------------------
# constants (shaderio*.h)
# ---------------------------------------------------------------------------

TESSTABLE_COORD_MAX = 1 << 15
TESSTABLE_SIZE = 11
TESSTABLE_LOOKUP_SIZE = 16
TESSTABLE_LOOKUP_ENTRIES = 16 ** 3

INSTANCE_FRUSTUM_BIT = 1
INSTANCE_VISIBLE_BIT = 2

BUILD_SETUP_CLASSIFY = 0
BUILD_SETUP_INSTANTIATE_TESS = 1
BUILD_SETUP_DRAW_TESS = 2
BUILD_SETUP_SPLIT = 3
BUILD_SETUP_SPLIT_PASS = 4
BUILD_SETUP_BUILD_BLAS = 5

RT_CLUSTER_MODE_FULL_CLUSTER = 0
RT_CLUSTER_MODE_SINGLE_TESSELLATED = 1
RT_CLUSTER_MODE_1X_SUBSET_CLUSTER = 2
RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED = 3
VISUALIZE_TRIANGLES = 4
HIT_OK, HIT_UNSUPPORTED_MODE, HIT_OUT_OF_RANGE = 0, 1, 2

TEXEL_F32 = 0
TEXEL_F16 = 1
TEXEL_UNORM16 = 2

FLAG_CULLING = 1
FLAG_FREEZE_VIEWPOS = 2
FLAG_RASTER_CULL = 4
FLAG_WRITE_FULLCLUSTERS = 8
FLAG_PN = 16
FLAG_RIPPLE = 32
FLAG_TRANSIENT_1X = 64
FLAG_TRANSIENT_2X = 128
MINI_BATCHSIZE, MINI_TRIANGLES, MINI_VERTICES = 8, 4, 6

DEVERR_LOOKBACK_TIMEOUT = 1
DEVERR_BAD_CLUSTER = 2
DEVERR_BAD_CONFIG = 4
DEVERR_CAPACITY = 8

TC_OK = 0
TC_ERR_INVALID_ARG = 1
TC_ERR_CAPACITY = 2
TC_ERR_QUEUE_TIMEOUT = 3
TC_ERR_CUDA = 4
TC_ERR_NOT_INITIALIZED = 5

# ---------------------------------------------------------------------------
# structured dtypes (C alignment)
# ---------------------------------------------------------------------------


def _struct(fields, size):
    dt = np.dtype(fields, align=True)
    assert dt.itemsize == size, (fields[0][0], dt.itemsize, size)
    return dt


TessTableEntry = _struct([("firstTriangle", "<u2"), ("firstVertex", "<u2"), ("numTriangles", "<u2"),
                          ("numVertices", "<u2")], 8)

TessellationTable = _struct([("vertices", "<u8"), ("triangles", "<u8"), ("entries", "<u8"),
                             ("templateAddresses", "<u8"), ("templateInstantiationSizes", "<u8")], 40)

BBox = _struct([("lo", "<f4", 3), ("hi", "<f4", 3), ("shortestEdge", "<f4"), ("longestEdge", "<f4")], 32)

Cluster = _struct([("numVertices", "<u2"), ("numTriangles", "<u2"), ("firstTriangle", "<u4"),
                   ("firstLocalVertex", "<u4"), ("firstLocalTriangle", "<u4")], 16)

RenderInstance = _struct([
    ("worldMatrix", "<f4", 16),
    ("geometryID", "<u4"), ("numTriangles", "<u4"), ("numVertices", "<u4"), ("numClusters", "<u4"),
    ("displacementIndex", "<i4"), ("displacementScale", "<f4"), ("displacementOffset", "<f4"), ("_pad", "<f4"),
    ("geoLo", "<f4", 4), ("geoHi", "<f4", 4),
    ("positions", "<u8"), ("normals", "<u8"), ("texcoords", "<u8"), ("clusters", "<u8"),
    ("clusterLocalTriangles", "<u8"), ("clusterBboxes", "<u8"), ("clusterTemplateAdresses", "<u8"),
    ("clusterTemplateInstantiatonSizes", "<u8"),
], 192)

ClusterInfo = _struct([("instanceID", "<u4"), ("clusterID", "<u4")], 8)

TessTriangleInfo = _struct([("instanceID", "<u4"), ("clusterID", "<u4"), ("vtxEncoded", "<u4", 3),
                            ("triangleID_config", "<u4")], 24)

TemplateInstantiateInfo = _struct([("clusterIdOffset", "<u4"), ("geometryIndexOffset", "<u4"),
                                   ("clusterTemplateAddress", "<u8"), ("vertexBufferAddress", "<u8"),
                                   ("vertexBufferStride", "<u8")], 32)

ClasBuildInfo = _struct([("clusterID", "<u4"), ("clusterFlags", "<u4"), ("packed", "<u4"),
                         ("baseGeometryIndexAndFlags", "<u4"), ("indexBufferStride", "<u2"),
                         ("vertexBufferStride", "<u2"), ("geometryIndexAndFlagsBufferStride", "<u2"),
                         ("opacityMicromapIndexBufferStride", "<u2"), ("indexBuffer", "<u8"), ("vertexBuffer", "<u8"),
                         ("geometryIndexAndFlagsBuffer", "<u8"), ("opacityMicromapArray", "<u8"),
                         ("opacityMicromapIndexBuffer", "<u8")], 64)

BlasBuildInfo = _struct([("clusterReferencesCount", "<u4"), ("clusterReferencesStride", "<u4"),
                         ("clusterReferences", "<u8")], 16)

DispatchIndirectCommand = np.dtype([("gridX", "<u4"), ("gridY", "<u4"), ("gridZ", "<u4")])
DrawMeshTasksIndirectCommandNV = np.dtype([("count", "<u4"), ("first", "<u4")])

SceneBuilding = _struct([
    ("viewPos", "<f4", 3), ("_pad", "<u4"),
    ("numRenderInstances", "<u4"), ("visibleClusterCounter", "<u4"),
    ("fullClusterCounter", "<u4"), ("partTriangleCounter", "<u4"),
    ("dualPartTriangleCounter", "<u8"),
    ("splitTriangleCounter", "<i4"), ("splitReadCounter", "<u4"), ("splitWriteCounter", "<u4"),
    ("splitPass", "<u4"), ("splitPassStart", "<u4"), ("splitPassEnd", "<u4"),
    ("genVertexCounter", "<u4"), ("genClusterCounter", "<u4"), ("genClusterDataCounter", "<u8"),
    ("dispatchClassify", DispatchIndirectCommand), ("dispatchTriangleSplit", DispatchIndirectCommand),
    ("instanceStates", "<u8"), ("visibleClusters", "<u8"), ("fullClusters", "<u8"), ("splitTriangles", "<u8"),
    ("partTriangles", "<u8"),
    ("drawFullClusters", DrawMeshTasksIndirectCommandNV), ("drawPartTriangles", DrawMeshTasksIndirectCommandNV),
    ("dispatchClusterInstantiate", DispatchIndirectCommand), ("dispatchTriangleInstantiate", DispatchIndirectCommand),
    ("dispatchBlasTempInsert", DispatchIndirectCommand), ("dispatchBlasTransInsert", DispatchIndirectCommand),
    ("positionTruncateBitCount", "<u4"),
    ("blasClusterCounter", "<u4"), ("tempInstantiateCounter", "<u4"), ("transBuildCounter", "<u4"),
    ("basicClusterSizes", "<u8"),
    ("genClusterData", "<u8"), ("genVertices", "<u8"),
    ("tempInstanceIDs", "<u8"), ("tempInstantiations", "<u8"), ("tempClusterAddresses", "<u8"),
    ("tempClusterSizes", "<u8"),
    ("transInstanceIDs", "<u8"), ("transBuilds", "<u8"), ("transClusterAddresses", "<u8"),
    ("transClusterSizes", "<u8"),
    ("transTriMappings", "<u8"), ("transTriIndices", "<u8"),
    ("blasBuildInfos", "<u8"), ("blasBuildSizes", "<u8"), ("blasClusterAddresses", "<u8"), ("blasBuildData", "<u8"),
    ("numBlasReservedSizes", "<u4"),
], 368)

FrameConstants = _struct([
    ("projMatrix", "<f4", 16), ("projMatrixI", "<f4", 16), ("viewProjMatrix", "<f4", 16),
    ("viewProjMatrixI", "<f4", 16), ("viewMatrix", "<f4", 16), ("viewMatrixI", "<f4", 16),
    ("viewPos", "<f4", 4), ("viewDir", "<f4", 4), ("viewPlane", "<f4", 4), ("skyProjMatrixI", "<f4", 16),
    ("viewport", "<i4", 2), ("viewportf", "<f4", 2), ("viewPixelSize", "<f4", 2), ("viewClipSize", "<f4", 2),
    ("wLightPos", "<f4", 3), ("tessRate", "<f4"),
    ("displacementScale", "<f4"), ("displacementOffset", "<f4"), ("lightMixer", "<f4"), ("doShadow", "<u4"),
    ("wUpDir", "<f4", 3), ("sceneSize", "<f4"), ("bgColor", "<f4", 4),
    ("lodScale", "<f4"), ("animationState", "<f4"), ("ambientOcclusionRadius", "<f4"),
    ("ambientOcclusionSamples", "<i4"),
    ("animationRippleEnabled", "<i4"), ("animationRippleFrequency", "<f4"), ("animationRippleAmplitude", "<f4"),
    ("animationRippleSpeed", "<f4"),
    ("_pad", "<u4", 3), ("visualize", "<u4"),
    ("doAnimation", "<u4"), ("flipWinding", "<u4"), ("nearPlane", "<f4"), ("farPlane", "<f4"),
    ("hizSizeFactors", "<f4", 4), ("nearSizeFactors", "<f4", 4),
    ("hizSizeMax", "<f4"), ("facetShading", "<i4"), ("supersample", "<i4"), ("colorXor", "<u4"),
    ("dbgUint", "<u4"), ("dbgFloat", "<f4"), ("time", "<f4"), ("frame", "<u4"),
    ("mousePosition", "<u4", 2), ("wireThickness", "<f4"), ("wireSmoothing", "<f4"),
    ("wireColor", "<f4", 3), ("wireStipple", "<u4"),
    ("wireBackfaceColor", "<f4", 3), ("wireStippleRepeats", "<f4"),
    ("wireStippleLength", "<f4"), ("doWireframe", "<u4"), ("visFilterInstanceID", "<u4"),
    ("visFilterClusterID", "<u4"),
], 784)

Readback = _struct([
    ("numVisibleClusters", "<u4"), ("numFullClusters", "<u4"), ("numSplitTriangles", "<u4"),
    ("numPartTriangles", "<u4"), ("numTotalTriangles", "<u4"), ("numTempInstantiations", "<u4"),
    ("numGenVertices", "<u4"), ("numBlasClusters", "<u4"), ("numTransBuilds", "<u4"),
    ("numTransPartTriangles", "<u4"), ("numActualTransBuilds", "<u4"), ("numActualTempInstantiations", "<u4"),
    ("numGenDatas", "<u8"), ("numGenActualDatas", "<u8"),
    ("numBlasReservedSizes", "<u4"), ("numBlasActualSizes", "<u4"),
    ("debugU64", "<u8"),
    ("clusterTriangleId", "<u4"), ("_packedDepth0", "<u4"), ("instanceId", "<u4"), ("_packedDepth1", "<u4"),
    ("debugI", "<i4"), ("debugUI", "<u4"), ("debugF", "<u4"),
    ("debugA", "<u4", 64), ("debugB", "<u4", 64), ("debugC", "<u4", 64),
], 880)

DisplacementTexture = _struct([("texels", "<u8"), ("width", "<u4"), ("height", "<u4"), ("format", "<u4"),
                               ("_pad", "<u4")], 24)

GradTargets = _struct([("dPositions", "<u8"), ("dNormals", "<u8")], 16)

# hit-time decode (tc_hit / tc_base_hit)
Hit = _struct([("instanceID", "<u4"), ("clusterID", "<u4"), ("triangleID", "<u4"), ("barycentrics", "<f4", 2),
               ("_pad", "<u4")], 24)
BaseHit = _struct([("clusterID", "<u4"), ("triangleID", "<u4"), ("vertexIndices", "<u4", 3), ("barycentrics", "<f4", 3),
                   ("partID", "<u4"), ("status", "<u4")], 40)

# ---------------------------------------------------------------------------
# ctypes structs passed by pointer to the C ABI
# ---------------------------------------------------------------------------


class Caps(ctypes.Structure):
    _fields_ = [("maxVisibleClusters", ctypes.c_uint32), ("maxPartTriangles", ctypes.c_uint32),
                ("maxSplitTriangles", ctypes.c_uint32), ("maxGeneratedClusters", ctypes.c_uint32),
                ("maxGeneratedClusterMegs", ctypes.c_uint32), ("maxGeneratedVertices", ctypes.c_uint32),
                ("splitFactor", ctypes.c_uint32), ("_pad", ctypes.c_uint32)]


class FrameArgs(ctypes.Structure):
    _fields_ = [("view", ctypes.c_uint64), ("viewLast", ctypes.c_uint64), ("instances", ctypes.c_uint64),
                ("build", ctypes.c_uint64), ("readback", ctypes.c_uint64), ("textures", ctypes.c_uint64),
                ("numInstances", ctypes.c_uint32), ("numTextures", ctypes.c_uint32),
                ("totalClusters", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("caps", Caps)]


class Schedule(ctypes.Structure):
    _fields_ = [("classifyBlocksPerSM", ctypes.c_uint32), ("splitBlockSize", ctypes.c_uint32),
                ("vertexBlocksPerSM", ctypes.c_uint32), ("scanBlocksPerSM", ctypes.c_uint32),
                ("blocksPerSM", ctypes.c_uint32), ("fullVertexBlocksPerSM", ctypes.c_uint32),
                ("vertexGridPerSM", ctypes.c_uint32), ("lookbackSpinLimit", ctypes.c_uint32),
                ("frameShape", ctypes.c_uint32), ("splitPerPass", ctypes.c_uint32)]


SCHEDULE_FIELDS = ("classifyBlocksPerSM", "splitBlockSize", "vertexBlocksPerSM", "scanBlocksPerSM", "blocksPerSM",
                   "fullVertexBlocksPerSM", "vertexGridPerSM", "lookbackSpinLimit", "frameShape",
                   "splitPerPass")


RASTER_BATCH_VERTICES, RASTER_BATCH_TRIANGLES = 96, 121
RasterBatch = _struct([("firstPart", "<u4"), ("partCount", "<u4"), ("firstVertex", "<u4"), ("numVertices", "<u4"),
                       ("firstTriangle", "<u4"), ("numTriangles", "<u4")], 24)


class RasterOutputs(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_uint64), ("counts", ctypes.c_uint64), ("clipPositions", ctypes.c_uint64),
                ("worldPositions", ctypes.c_uint64), ("indices", ctypes.c_uint64), ("primitiveIDs", ctypes.c_uint64),
                ("maxBatches", ctypes.c_uint32), ("maxVertices", ctypes.c_uint32), ("maxTriangles", ctypes.c_uint32),
                ("_pad", ctypes.c_uint32)]


class ContextDesc(ctypes.Structure):
    _fields_ = [("maxInstances", ctypes.c_uint32), ("maxTotalClusters", ctypes.c_uint32), ("caps", Caps),
                ("device", ctypes.c_int32), ("_pad", ctypes.c_uint32)]


class TableInfoC(ctypes.Structure):
    _fields_ = [("maxSize", ctypes.c_uint32), ("maxSizeConfigs", ctypes.c_uint32), ("numConfigs", ctypes.c_uint32),
                ("maxVertices", ctypes.c_uint32), ("maxTriangles", ctypes.c_uint32),
                ("numRawConfigs", ctypes.c_uint32), ("deviceTable", ctypes.c_uint64),
                ("table", ctypes.c_uint64 * 5)]


assert ctypes.sizeof(Caps) == 32
assert ctypes.sizeof(FrameArgs) == 96
assert ctypes.sizeof(Schedule) == 40


def caps_from(cfg: dict) -> Caps:
    return Caps(cfg["maxVisibleClusters"], cfg["maxPartTriangles"], cfg["maxSplitTriangles"],
                cfg["maxGeneratedClusters"], cfg["maxGeneratedClusterMegs"], cfg["maxGeneratedVertices"],
                cfg["splitFactor"], 0)


def default_caps(visible_bits=20, part_bits=20, split_bits=16, vertex_bits=24, megs=1024, split_factor=8) -> dict:
    """RendererConfig defaults (src/renderer.hpp:54-61); MAX_GENERATED_CLUSTERS as
    in src/renderer_raytrace_clusters_tess.cpp:170."""
    return dict(maxVisibleClusters=1 << visible_bits, maxPartTriangles=1 << part_bits,
                maxSplitTriangles=1 << split_bits,
                maxGeneratedClusters=(1 << visible_bits) + (1 << part_bits),
                maxGeneratedClusterMegs=megs, maxGeneratedVertices=1 << vertex_bits, splitFactor=split_factor)
