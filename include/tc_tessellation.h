/*
 * tc_tessellation.h — C ABI of the GB300 (sm_103a) tessellated-cluster build pipeline.
 *
 * This library re-implements, as CUDA kernels, the per-frame compute chain of
 * nvpro-samples/vk_tessellated_clusters that turns clustered meshes into
 * cluster-acceleration-structure build inputs:
 *
 *   instances_classify -> clusters_cull -> build_setup -> cluster_classify
 *   -> triangle_split (multi-pass) -> triangle_tess_template_instantiate
 *   -> blas_setup_insertion -> blas_clusters_insert
 *
 * The boundary is the reference's buffer protocol (shaders/shaderio_*.h): every
 * array is a 64-bit device address inside tc_SceneBuilding / tc_RenderInstance,
 * counters live in tc_SceneBuilding, statistics in tc_Readback, and the layouts
 * below are byte-identical to the reference's C++ view of those structs, so the
 * buffers this library fills are what the cluster AS build consumes
 * (src/renderer_raytrace_clusters_tess.cpp:592-733).
 *
 * Ownership follows the reference (src/renderer_raytrace_clusters_tess.cpp:200-310):
 * the caller allocates every buffer referenced by tc_SceneBuilding and
 * tc_RenderInstance. The context owns only the uploaded tessellation table and a
 * scratch block sized at creation. No call below allocates device memory except
 * tc_context_create and tc_table_init.
 *
 * All entry points are asynchronous on the given stream and return a tc_status
 * describing argument validation and launch errors. Faults detected by kernels
 * (a look-back wait that ran out, inconsistent input) are recorded in a device
 * error word read by tc_read_device_errors.
 *
 * Arithmetic: IEEE single precision without contraction (no FMA), IEEE division
 * and square root, round-half-to-even for the GLSL round() of tess factors.
 */
#ifndef TC_TESSELLATION_H_
#define TC_TESSELLATION_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TC_API_VERSION 1

/* ------------------------------------------------------------------------- */
/* constants mirroring shaders/shaderio*.h                                    */
/* ------------------------------------------------------------------------- */

#define TC_TESSTABLE_COORD_MAX (1u << 15) /* shaderio_scene.h:24 */
#define TC_TESSTABLE_SIZE 11u             /* shaderio_scene.h:25 */
#define TC_TESSTABLE_LOOKUP_SIZE 16u      /* shaderio_scene.h:40 (next pow2 of 11) */
#define TC_TESSTABLE_LOOKUP_ENTRIES (TC_TESSTABLE_LOOKUP_SIZE * TC_TESSTABLE_LOOKUP_SIZE * TC_TESSTABLE_LOOKUP_SIZE)
#define TC_MAX_CLUSTER_TRIANGLES 64u
#define TC_MAX_CLUSTER_VERTICES 64u

#define TC_INSTANCE_FRUSTUM_BIT 1u /* shaderio_building.h:54 */
#define TC_INSTANCE_VISIBLE_BIT 2u /* shaderio_building.h:55 */

/* build_setup modes, shaderio.h:67-72 */
#define TC_BUILD_SETUP_CLASSIFY 0u
#define TC_BUILD_SETUP_INSTANTIATE_TESS 1u
#define TC_BUILD_SETUP_DRAW_TESS 2u
#define TC_BUILD_SETUP_SPLIT 3u
#define TC_BUILD_SETUP_SPLIT_PASS 4u
#define TC_BUILD_SETUP_BUILD_BLAS 5u

/* clusterID mode bits in TemplateInstantiateInfo.clusterIdOffset, shaderio.h:101-108 */
#define TC_RT_CLUSTER_MODE_FULL_CLUSTER 0u
#define TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED 1u
#define TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER 2u    /* transient build of a cluster's untessellated triangles */
#define TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED 3u
#define TC_VISUALIZE_TRIANGLES 4u /* FrameConstants.visualize, shaderio.h:39 */

/* ------------------------------------------------------------------------- */
/* layouts (byte-identical to the reference's C++ structs)                    */
/* ------------------------------------------------------------------------- */

typedef struct tc_vec2 { float x, y; } tc_vec2;
typedef struct tc_vec3 { float x, y, z; } tc_vec3;
typedef struct tc_vec4 { float x, y, z, w; } tc_vec4;
/* column-major like glm::mat4: m[col*4 + row] */
typedef struct tc_mat4 { float m[16]; } tc_mat4;

/* shaderio_scene.h:65-72 */
typedef struct tc_TessTableEntry {
  uint16_t firstTriangle;
  uint16_t firstVertex;
  uint16_t numTriangles;
  uint16_t numVertices;
} tc_TessTableEntry;

/* shaderio_scene.h:75-87 */
typedef struct tc_TessellationTable {
  uint64_t vertices;                   /* u32[]: (v << 16) | u, 1<<15 == 1.0 */
  uint64_t triangles;                  /* u32[]: 3 x u8 indices */
  uint64_t entries;                    /* tc_TessTableEntry[4096] lookup */
  uint64_t templateAddresses;          /* u64[4096] per config CLAS template */
  uint64_t templateInstantiationSizes; /* u32[4096] worst-case CLAS size */
} tc_TessellationTable;

/* shaderio_scene.h:89-95 */
typedef struct tc_BBox {
  tc_vec3 lo;
  tc_vec3 hi;
  float   shortestEdge;
  float   longestEdge;
} tc_BBox;

/* shaderio_scene.h:101-111 */
typedef struct tc_Cluster {
  uint16_t numVertices;
  uint16_t numTriangles;
  uint32_t firstTriangle;
  uint32_t firstLocalVertex;
  uint32_t firstLocalTriangle;
} tc_Cluster;

/* shaderio_scene.h:116-156 */
typedef struct tc_RenderInstance {
  tc_mat4  worldMatrix;
  uint32_t geometryID;
  uint32_t numTriangles;
  uint32_t numVertices;
  uint32_t numClusters;
  int32_t  displacementIndex;
  float    displacementScale;
  float    displacementOffset;
  float    _pad;
  tc_vec4  geoLo;
  tc_vec4  geoHi;
  uint64_t positions;                        /* tc_vec3[] */
  uint64_t normals;                          /* tc_vec3[] */
  uint64_t texcoords;                        /* tc_vec2[] */
  uint64_t clusters;                         /* tc_Cluster[] */
  uint64_t clusterLocalTriangles;            /* u8[] */
  uint64_t clusterBboxes;                    /* tc_BBox[] */
  uint64_t clusterTemplateAdresses;          /* u64[] (spelling as in the reference) */
  uint64_t clusterTemplateInstantiatonSizes; /* u32[] (spelling as in the reference) */
} tc_RenderInstance;

/* shaderio_building.h:62-68 */
typedef struct tc_ClusterInfo {
  uint32_t instanceID;
  uint32_t clusterID;
} tc_ClusterInfo;

/* shaderio_building.h:71-92 */
typedef struct tc_SubTriangleInfo {
  uint32_t vtxEncoded[3];
  uint32_t triangleID_config; /* triangleID | (config << 16), config bit 15 = flipped */
} tc_SubTriangleInfo;

typedef struct tc_TessTriangleInfo {
  tc_ClusterInfo     cluster;
  tc_SubTriangleInfo subTriangle;
} tc_TessTriangleInfo;

/* shaderio_building.h:95-127 */
typedef struct tc_ClasBuildInfo {
  uint32_t clusterID;
  uint32_t clusterFlags;
  uint32_t packed;
  uint32_t baseGeometryIndexAndFlags;
  uint16_t indexBufferStride;
  uint16_t vertexBufferStride;
  uint16_t geometryIndexAndFlagsBufferStride;
  uint16_t opacityMicromapIndexBufferStride;
  uint64_t indexBuffer;
  uint64_t vertexBuffer;
  uint64_t geometryIndexAndFlagsBuffer;
  uint64_t opacityMicromapArray;
  uint64_t opacityMicromapIndexBuffer;
} tc_ClasBuildInfo;

/* shaderio_building.h:130-138 */
typedef struct tc_TemplateInstantiateInfo {
  uint32_t clusterIdOffset;
  uint32_t geometryIndexOffset;
  uint64_t clusterTemplateAddress;
  uint64_t vertexBufferAddress;
  uint64_t vertexBufferStride;
} tc_TemplateInstantiateInfo;

/* shaderio_building.h:141-150 */
typedef struct tc_BlasBuildInfo {
  uint32_t clusterReferencesCount;
  uint32_t clusterReferencesStride;
  uint64_t clusterReferences;
} tc_BlasBuildInfo;

/* shaderio_core.h:99-111 */
typedef struct tc_DispatchIndirectCommand {
  uint32_t gridX, gridY, gridZ;
} tc_DispatchIndirectCommand;

typedef struct tc_DrawMeshTasksIndirectCommandNV {
  uint32_t count, first;
} tc_DrawMeshTasksIndirectCommandNV;

/* shaderio_building.h:156-263 */
typedef struct tc_SceneBuilding {
  tc_vec3  viewPos;
  uint32_t _pad;

  uint32_t numRenderInstances;
  uint32_t visibleClusterCounter;

  uint32_t fullClusterCounter;
  uint32_t partTriangleCounter;

  uint64_t dualPartTriangleCounter;

  int32_t  splitTriangleCounter;
  uint32_t splitReadCounter;
  uint32_t splitWriteCounter;
  uint32_t splitPass;
  uint32_t splitPassStart;
  uint32_t splitPassEnd;

  uint32_t genVertexCounter;
  uint32_t genClusterCounter;
  uint64_t genClusterDataCounter;

  tc_DispatchIndirectCommand dispatchClassify;
  tc_DispatchIndirectCommand dispatchTriangleSplit;

  uint64_t instanceStates;  /* u32[numRenderInstances] */
  uint64_t visibleClusters; /* tc_ClusterInfo[maxVisibleClusters] */
  uint64_t fullClusters;    /* tc_ClusterInfo[] (optional here, see tc_frame_args) */
  uint64_t splitTriangles;  /* tc_TessTriangleInfo[maxSplitTriangles] */
  uint64_t partTriangles;   /* tc_TessTriangleInfo[maxPartTriangles] */

  tc_DrawMeshTasksIndirectCommandNV drawFullClusters;
  tc_DrawMeshTasksIndirectCommandNV drawPartTriangles;

  tc_DispatchIndirectCommand dispatchClusterInstantiate;
  tc_DispatchIndirectCommand dispatchTriangleInstantiate;
  tc_DispatchIndirectCommand dispatchBlasTempInsert;
  tc_DispatchIndirectCommand dispatchBlasTransInsert;

  uint32_t positionTruncateBitCount;

  uint32_t blasClusterCounter;
  uint32_t tempInstantiateCounter;
  uint32_t transBuildCounter;

  uint64_t basicClusterSizes;

  uint64_t genClusterData; /* base address of CLAS destination memory */
  uint64_t genVertices;    /* tc_vec3[maxGeneratedVertices] */

  uint64_t tempInstanceIDs;      /* u32[maxGeneratedClusters] */
  uint64_t tempInstantiations;   /* tc_TemplateInstantiateInfo[maxGeneratedClusters] */
  uint64_t tempClusterAddresses; /* u64[maxGeneratedClusters] */
  uint64_t tempClusterSizes;     /* u32[maxGeneratedClusters] (written by the CLAS build) */

  uint64_t transInstanceIDs;
  uint64_t transBuilds;
  uint64_t transClusterAddresses;
  uint64_t transClusterSizes;

  uint64_t transTriMappings;
  uint64_t transTriIndices;

  uint64_t blasBuildInfos;       /* tc_BlasBuildInfo[numRenderInstances] */
  uint64_t blasBuildSizes;       /* u32[numRenderInstances] */
  uint64_t blasClusterAddresses; /* u64[maxGeneratedClusters] */
  uint64_t blasBuildData;

  uint32_t numBlasReservedSizes;
} tc_SceneBuilding;

/*
 * shaderio.h:180-261 up to and including visFilterClusterID. The reference's
 * trailing `SkySimpleParameters skyParams` (declared in a header of a
 * dependency that is not part of the reference) is only used by shading and is
 * not part of this boundary, which is why the two frame constant blocks are
 * passed as separate pointers (tc_frame_args.view / viewLast) instead of an
 * array of two.
 */
typedef struct tc_FrameConstants {
  tc_mat4  projMatrix;
  tc_mat4  projMatrixI;
  tc_mat4  viewProjMatrix;
  tc_mat4  viewProjMatrixI;
  tc_mat4  viewMatrix;
  tc_mat4  viewMatrixI;
  tc_vec4  viewPos;
  tc_vec4  viewDir;
  tc_vec4  viewPlane;
  tc_mat4  skyProjMatrixI;
  int32_t  viewport[2];
  tc_vec2  viewportf;
  tc_vec2  viewPixelSize;
  tc_vec2  viewClipSize;
  tc_vec3  wLightPos;
  float    tessRate;
  float    displacementScale;
  float    displacementOffset;
  float    lightMixer;
  uint32_t doShadow;
  tc_vec3  wUpDir;
  float    sceneSize;
  tc_vec4  bgColor;
  float    lodScale;
  float    animationState;
  float    ambientOcclusionRadius;
  int32_t  ambientOcclusionSamples;
  int32_t  animationRippleEnabled;
  float    animationRippleFrequency;
  float    animationRippleAmplitude;
  float    animationRippleSpeed;
  uint32_t _pad[3];
  uint32_t visualize;
  uint32_t doAnimation;
  uint32_t flipWinding;
  float    nearPlane;
  float    farPlane;
  tc_vec4  hizSizeFactors;
  tc_vec4  nearSizeFactors;
  float    hizSizeMax;
  int32_t  facetShading;
  int32_t  supersample;
  uint32_t colorXor;
  uint32_t dbgUint;
  float    dbgFloat;
  float    time;
  uint32_t frame;
  uint32_t mousePosition[2];
  float    wireThickness;
  float    wireSmoothing;
  tc_vec3  wireColor;
  uint32_t wireStipple;
  tc_vec3  wireBackfaceColor;
  float    wireStippleRepeats;
  float    wireStippleLength;
  uint32_t doWireframe;
  uint32_t visFilterInstanceID;
  uint32_t visFilterClusterID;
} tc_FrameConstants;

/* shaderio.h:263-309 (C++ view) */
typedef struct tc_Readback {
  uint32_t numVisibleClusters;
  uint32_t numFullClusters;
  uint32_t numSplitTriangles;
  uint32_t numPartTriangles;
  uint32_t numTotalTriangles;
  uint32_t numTempInstantiations;
  uint32_t numGenVertices;
  uint32_t numBlasClusters;
  uint32_t numTransBuilds;
  uint32_t numTransPartTriangles;
  uint32_t numActualTransBuilds;
  uint32_t numActualTempInstantiations;
  uint64_t numGenDatas;
  uint64_t numGenActualDatas;
  uint32_t numBlasReservedSizes;
  uint32_t numBlasActualSizes;
  uint64_t debugU64;
  uint32_t clusterTriangleId;
  uint32_t _packedDepth0;
  uint32_t instanceId;
  uint32_t _packedDepth1;
  int32_t  debugI;
  uint32_t debugUI;
  uint32_t debugF;
  uint32_t debugA[64];
  uint32_t debugB[64];
  uint32_t debugC[64];
} tc_Readback;

/* Displacement texture: replaces the reference's `sampler2D displacementTextures[]`
 * (cluster_classify.comp.glsl:105-107). Sampled bilinearly at mip 0 with REPEAT
 * addressing and texel centres at (i + 0.5) / width. */
#define TC_TEXEL_F32 0u
#define TC_TEXEL_F16 1u
#define TC_TEXEL_UNORM16 2u
typedef struct tc_DisplacementTexture {
  uint64_t texels; /* row-major, width * height texels */
  uint32_t width;
  uint32_t height;
  uint32_t format; /* TC_TEXEL_* */
  uint32_t _pad;
} tc_DisplacementTexture;

/* ------------------------------------------------------------------------- */
/* runtime configuration                                                      */
/* ------------------------------------------------------------------------- */

/* Buffer capacities. The reference bakes these into the shaders as macros
 * (src/renderer_raytrace_clusters_tess.cpp:126-131); here they are runtime values. */
typedef struct tc_caps {
  uint32_t maxVisibleClusters;      /* MAX_VISIBLE_CLUSTERS */
  uint32_t maxPartTriangles;        /* MAX_PART_TRIANGLES */
  uint32_t maxSplitTriangles;       /* MAX_SPLIT_TRIANGLES */
  uint32_t maxGeneratedClusters;    /* MAX_GENERATED_CLUSTERS */
  uint32_t maxGeneratedClusterMegs; /* MAX_GENERATED_CLUSTER_MEGS */
  uint32_t maxGeneratedVertices;    /* MAX_GENERATED_VERTICES */
  uint32_t splitFactor;             /* TESS_MAX_SPLIT_FACTOR, clamped to [2, 11] */
  uint32_t _pad;
} tc_caps;

/* tc_frame_args.flags */
#define TC_FLAG_CULLING 1u          /* DO_CULLING: invisible instances are not tessellated */
#define TC_FLAG_FREEZE_VIEWPOS 2u   /* take SceneBuilding.viewPos from viewLast */
#define TC_FLAG_RASTER_CULL 4u      /* clusters_cull drops clusters (raster semantics) */
#define TC_FLAG_WRITE_FULLCLUSTERS 8u /* also record accepted full clusters in SceneBuilding.fullClusters */
#define TC_FLAG_PN 16u     /* TESS_USE_PN: part-triangle vertices on the base triangle's PN (curved point-normal) patch */
#define TC_FLAG_RIPPLE 32u /* DO_ANIMATION: the FrameConstants ripple deformation on every generated vertex */
/* TESS_USE_1X_TRANSIENTBUILDS (cluster_classify.comp.glsl:254-343, 394-437, 489-535): a cluster with more
 * than one untessellated triangle (but not all) gets a transient CLAS build of those triangles over its own
 * vertices (ClasBuildInfo in SceneBuilding.transBuilds, u8 indices after the vertices, u8 triangle map
 * after a ClusterInfo header at the back of partTriangles) */
#define TC_FLAG_TRANSIENT_1X 64u
/* TESS_USE_2X_TRANSIENTBUILDS (cluster_classify.comp.glsl:675-905): triangles with edge factors <= 2 are
 * tessellated in place and packed, TC_2X_MINI_BATCHSIZE at a time, into transient builds (u16 map) */
#define TC_FLAG_TRANSIENT_2X 128u
/* The transient flags need SceneBuilding.basicClusterSizes (TC_MAX_CLUSTER_TRIANGLES + 1 entries) and the
 * trans* arrays; they are ray-tracing semantics (TC_ERR_INVALID_ARG with TC_FLAG_RASTER_CULL).
 * tc_generate_vertices and tc_instantiate_backward cover none of PN, ripple or transient builds: they
 * return TC_ERR_INVALID_ARG. */
#define TC_2X_MINI_BATCHSIZE 8u /* shaderio.h:149-158 */
#define TC_2X_MINI_TRIANGLES 4u
#define TC_2X_MINI_VERTICES 6u

typedef struct tc_frame_args {
  uint64_t view;      /* const tc_FrameConstants* (device): this frame */
  uint64_t viewLast;  /* const tc_FrameConstants* (device): last frame, used for culling */
  uint64_t instances; /* const tc_RenderInstance* (device) */
  uint64_t build;     /* tc_SceneBuilding* (device), pointers filled by the caller */
  uint64_t readback;  /* tc_Readback* (device) */
  uint64_t textures;  /* const tc_DisplacementTexture* (device), may be 0 */
  uint32_t numInstances;
  uint32_t numTextures;
  uint32_t totalClusters; /* sum of numClusters over all instances (host known) */
  uint32_t flags;         /* TC_FLAG_* */
  tc_caps  caps;
} tc_frame_args;

typedef enum tc_status {
  TC_OK = 0,
  TC_ERR_INVALID_ARG = 1,
  TC_ERR_CAPACITY = 2,      /* a request exceeds what the context was created for */
  TC_ERR_QUEUE_TIMEOUT = 3, /* a device-side wait gave up (see tc_read_device_errors) */
  TC_ERR_CUDA = 4,
  TC_ERR_NOT_INITIALIZED = 5
} tc_status;

/* device error word bits (tc_read_device_errors) */
#define TC_DEVERR_LOOKBACK_TIMEOUT 1u   /* a tile waited too long for its predecessor */
#define TC_DEVERR_BAD_CLUSTER 2u        /* cluster with more than 64 triangles/vertices */
#define TC_DEVERR_BAD_CONFIG 4u         /* a tess config outside the table */
#define TC_DEVERR_CAPACITY 8u           /* work beyond the context's scratch sizing was dropped */

/* Launch schedule: grid shapes per stage, picked by the autotuner
 * (vk_tessellated_clusters_gb300/autotune.py) or left at the defaults. */
typedef struct tc_schedule {
  uint32_t classifyBlocksPerSM; /* grid of the per-cluster classify kernels = SMs x this (256 threads); 4 or less:
                                 * 64 registers per thread, 5-7: 40, 8 and more: 32 */
  uint32_t splitBlockSize;      /* split tile: 128 (16 items), 256 or 512 (32 items) threads */
  uint32_t vertexBlocksPerSM;   /* register budget of the vertex-generation kernel (one 32-part chunk per warp):
                                 * 4 or less: 64 registers per thread, 5: 48, 6 and more: 40 */
  uint32_t scanBlocksPerSM;     /* grid of the instantiate allocation kernels (tile sums, arguments) = SMs x this */
  uint32_t blocksPerSM;         /* persistent grid of the split kernel = SMs x this x (512 / splitBlockSize) */
  uint32_t fullVertexBlocksPerSM; /* grid of the full-cluster vertex kernel = SMs x this (at most 4 resident);
                                   * it runs beside the rest of the frame (fewer blocks leave room for it);
                                   * 0: the default (4) */
  uint32_t vertexGridPerSM;     /* grid of the part vertex kernel = SMs x this (grid-stride over 32-part chunks);
                                 * 0: one resident wave (the blocks vertexBlocksPerSM allows) */
  uint32_t lookbackSpinLimit;   /* polls a bounded look-back wait makes before it gives up, sets
                                 * TC_DEVERR_LOOKBACK_TIMEOUT and goes on with what it has (the frame's offsets are
                                 * then unreliable); 0: the default, 2^22 polls (seconds, with back-off) */
  uint32_t frameShape;          /* the batched frame's graph: 0 allocates the first part run (classify's parts) on a
                                 * side stream while the split passes run, the later runs after them; 1 allocates
                                 * every run once after the split passes (fewer launches when splits are rare).
                                 * Outputs are identical. */
  uint32_t splitPerPass;        /* the batched frame's split passes: 0 in one launch (k_triangle_split_levels, cheap
                                 * when they have little to do), 1 one launch per pass with the set-ups between
                                 * (pays off when the passes are long). Outputs are identical. */
} tc_schedule;

typedef struct tc_context_desc {
  uint32_t maxInstances;     /* largest numInstances a frame may use */
  uint32_t maxTotalClusters; /* largest totalClusters a frame may use */
  tc_caps  caps;             /* largest capacities a frame may use */
  int32_t  device;           /* CUDA device ordinal */
  uint32_t _pad;
} tc_context_desc;

typedef struct tc_context tc_context;

typedef struct tc_table_info {
  uint32_t maxSize;        /* 11 */
  uint32_t maxSizeConfigs; /* 16 */
  uint32_t numConfigs;     /* 4096 */
  uint32_t maxVertices;    /* largest config vertex count (78) */
  uint32_t maxTriangles;   /* largest config triangle count (121) */
  uint32_t numRawConfigs;  /* 286 */
  uint64_t deviceTable;    /* address of a device tc_TessellationTable */
  tc_TessellationTable table; /* host copy of the same struct */
} tc_table_info;

const char* tc_version(void);
const char* tc_status_string(tc_status status);

/* Create/destroy a context: uploads nothing yet, allocates the scratch block
 * sized by desc. Replaces the renderer init step
 * (src/renderer_raytrace_clusters_tess.cpp:166-310, scratch part only). */
tc_status tc_context_create(const tc_context_desc* desc, tc_context** outCtx);
tc_status tc_context_destroy(tc_context* ctx);

/* Expand the raw tessellation table into the 16^3 lookup (including the
 * permuted, flipped configs) and upload it.
 * Replaces TessellationTable::init (src/tessellation_table.cpp:36-100). */
tc_status tc_table_init(tc_context* ctx, const uint32_t* vertices, uint32_t numVertices, const uint32_t* triangles,
                        uint32_t numTriangles, const uint16_t* configs, uint32_t numConfigs, uint32_t maxEdgeSegments,
                        tc_table_info* outInfo);
/* Per lookup-entry CLAS template addresses/sizes (4096 entries each), as produced
 * by TessellationTable::initTemplates (src/tessellation_table.cpp:102-404). */
tc_status tc_table_set_templates(tc_context* ctx, const uint64_t* templateAddresses, const uint32_t* instantiationSizes,
                                 void* stream);

/* Launch schedule used by the calls below. Per-SM multipliers must lie in
 * [1, 64] and splitBlockSize in {128, 256, 512} (else TC_ERR_INVALID_ARG).
 * The schedule changes launch shapes only: outputs are identical for every
 * valid schedule. */
tc_status tc_set_schedule(tc_context* ctx, const tc_schedule* schedule);
tc_status tc_get_schedule(const tc_context* ctx, tc_schedule* schedule);

/* ---- whole frame ---------------------------------------------------------- */

/* One frame of the build chain, batched over all instances: one persistent
 * launch per stage, build_setup fused into the producing kernels.
 * Replaces RendererRayTraceClustersTess::render's compute part
 * (src/renderer_raytrace_clusters_tess.cpp:410-692 minus the CLAS/BLAS builds). */
tc_status tc_frame_build(tc_context* ctx, const tc_frame_args* args, void* stream);

/* Same frame, recorded once into a CUDA graph and replayed. The graph is keyed by
 * the args; a change of args re-records. */
tc_status tc_frame_build_graph(tc_context* ctx, const tc_frame_args* args, void* stream);

/* The graph frame of tc_frame_build_graph with the frame's host traffic inside
 * the graph: its first kernel copies inputBytes from the pinned host block
 * hostInputs to the device block deviceInputs (which args->view, viewLast and
 * instances may point into), and once the frame's counters are final a kernel
 * of the graph copies its tc_Readback to the pinned host buffer hostReadback,
 * which holds it once the stream has passed the call. Replaces the reference's per-frame upload of the frame
 * constants (src/renderer_raytrace_clusters_tess.cpp:415, vkCmdUpdateBuffer)
 * and its Readback copy to a host-visible buffer (src/resources.cpp:83-90,
 * read in src/resources.cpp:497-501) without copy-engine round trips.
 * Host buffers: pinned and mapped (cudaHostAlloc, or cudaHostRegister with
 * cudaHostRegisterMapped); hostInputs and deviceInputs 16-byte aligned,
 * hostReadback 8-byte aligned (else TC_ERR_INVALID_ARG). inputBytes 0 skips
 * the upload, hostReadback NULL the Readback copy. The graph is keyed by the
 * args and the three buffers' addresses; a change re-records. */
tc_status tc_frame_build_graph_host(tc_context* ctx, const tc_frame_args* args, const void* hostInputs,
                                    uint64_t deviceInputs, uint64_t inputBytes, void* hostReadback, void* stream);

/* Same frame, with every stage launched once per instance (and per split pass)
 * from the host: the reference's per-instance dispatch pattern of clusters_cull
 * (src/renderer_raytrace_clusters_tess.cpp:454-460) applied to all stages.
 * Output is byte-identical to tc_frame_build. */
tc_status tc_frame_build_plain(tc_context* ctx, const tc_frame_args* args, void* stream);

/* ---- per stage (same semantics as the reference shader of the same name) --- */

/* Per-frame reset: counters of SceneBuilding zeroed, viewPos set, Readback zeroed,
 * splitTriangles filled with ~0 (src/renderer_raytrace_clusters_tess.cpp:412-419). */
tc_status tc_frame_begin(tc_context* ctx, const tc_frame_args* args, void* stream);
/* shaders/instances_classify.comp.glsl:102-128 */
tc_status tc_instances_classify(tc_context* ctx, const tc_frame_args* args, void* stream);
/* shaders/clusters_cull.comp.glsl:112-161 over instances [instanceBegin, instanceEnd) */
tc_status tc_clusters_cull(tc_context* ctx, const tc_frame_args* args, uint32_t instanceBegin, uint32_t instanceEnd,
                           void* stream);
/* shaders/build_setup.comp.glsl:102-265 */
tc_status tc_build_setup(tc_context* ctx, const tc_frame_args* args, uint32_t mode, void* stream);
/* shaders/cluster_classify.comp.glsl:150-666 for the visible clusters of
 * instances [instanceBegin, instanceEnd) */
tc_status tc_cluster_classify(tc_context* ctx, const tc_frame_args* args, uint32_t instanceBegin, uint32_t instanceEnd,
                              void* stream);
/* shaders/triangle_split.comp.glsl:598-632: one pass over the current split level
 * (SceneBuilding.splitPassStart/End) restricted to instances [instanceBegin, instanceEnd).
 * The split items must come from this context's tc_cluster_classify / earlier passes of
 * the same frame: they keep their base triangle's world positions in context scratch. */
tc_status tc_triangle_split(tc_context* ctx, const tc_frame_args* args, uint32_t instanceBegin, uint32_t instanceEnd,
                            void* stream);
/* shaders/triangle_tess_template_instantiate.comp.glsl:126-373 over all part
 * triangles (the reference's single indirect dispatch). partBegin must be 0 and
 * partEnd ~0u; the per-run form below covers sub-ranges. */
tc_status tc_triangle_instantiate(tc_context* ctx, const tc_frame_args* args, uint32_t partBegin, uint32_t partEnd,
                                  void* stream);
/* Same, restricted to one part run (run 0: parts from cluster_classify, run r:
 * parts from split pass r) and to instances [instanceBegin, instanceEnd).
 * run = ~0u with the full instance range is the whole list. Launching the runs
 * in order, and within a run the instances in order, reproduces the batched
 * output exactly. */
tc_status tc_triangle_instantiate_run(tc_context* ctx, const tc_frame_args* args, uint32_t run, uint32_t instanceBegin,
                                      uint32_t instanceEnd, void* stream);
/* Every pass of triangle_split in one launch (triangle_split.comp.glsl:146-331,
 * whose main_persistent :476-594 is the reference's single-dispatch form): the
 * same output as tc_triangle_split for each pass with
 * tc_build_setup(TC_BUILD_SETUP_SPLIT_PASS) between passes, for the whole
 * instance range; call it after tc_build_setup(TC_BUILD_SETUP_SPLIT) and follow
 * it with tc_build_setup(TC_BUILD_SETUP_INSTANTIATE_TESS). */
tc_status tc_triangle_split_all(tc_context* ctx, const tc_frame_args* args, void* stream);
/* shaders/blas_setup_insertion.comp.glsl:100-116 */
tc_status tc_blas_setup_insertion(tc_context* ctx, const tc_frame_args* args, void* stream);
/* shaders/blas_clusters_insert.comp.glsl:97-136 (template instantiations) */
tc_status tc_blas_clusters_insert(tc_context* ctx, const tc_frame_args* args, void* stream);

/* Largest instance count tc_blas_setup_insertion_noalloc accepts. */
#define TC_NOALLOC_MAX_INSTANCES (1u << 20)

/* No counterpart in the reference (whose Vulkan renderer allocates all its
 * buffers up front): tc_blas_setup_insertion for callers that cannot allocate
 * device memory, such as an application that owns every device byte through
 * its own pool or imported allocations, or a real-time frame loop that cannot
 * take cudaMalloc's implicit synchronisation; creating a tc_context allocates,
 * so this entry point takes none. It reads args->build and args->readback only
 * (the other pointers may be 0), with the same results as
 * tc_blas_setup_insertion. It calls no cudaMalloc, cudaFree or allocating
 * library routine: its look-back scratch is a fixed 33,024-byte __device__
 * array of the library, held on every GPU that loads the library until the
 * process exits.
 *   - args->numInstances (which must equal SceneBuilding.numRenderInstances)
 *     above TC_NOALLOC_MAX_INSTANCES: TC_ERR_CAPACITY, nothing launched.
 *     The kernel sizes its work from SceneBuilding.numRenderInstances on the
 *     device; if that count exceeds TC_NOALLOC_MAX_INSTANCES the instances
 *     beyond it get no list offsets, and only deviceErrors
 *     (TC_DEVERR_CAPACITY) tells: pass a deviceErrors word to see it.
 *   - Every call looks the array's address up (cudaGetSymbolAddress) in the
 *     current context, so it follows cudaDeviceReset and caller-owned
 *     contexts; the first call in a context may load the library's device
 *     code: make it before any stream capture.
 *   - Every call shares the array and clears it (cudaMemsetAsync on `stream`)
 *     before its launch; calls that overlap on the GPU race on it.
 *   - deviceErrors: optional device word that receives TC_DEVERR_* bits
 *     (atomic OR; 0 = not reported: the bits then land in the shared array
 *     and the next call clears them). */
tc_status tc_blas_setup_insertion_noalloc(const tc_frame_args* args, uint32_t* deviceErrors, void* stream);

/* Number of split passes the host issues for a split factor
 * (src/renderer_raytrace_clusters_tess.cpp:516-543). */
uint32_t tc_split_pass_count(uint32_t splitFactor);

/* ---- backward --------------------------------------------------------------- */

/* Gradient targets for one instance: float3 arrays parallel to the instance's
 * positions / normals (0 = not wanted). */
typedef struct tc_GradTargets {
  uint64_t dPositions;
  uint64_t dNormals;
} tc_GradTargets;

/* Forward of the vertex generation of the last frame built in `args` with its
 * tessellation decisions held fixed: regenerates genVertices of every accepted
 * instantiation from the current positions / normals / texels (the forward of
 * the differentiable path; bit-identical to the build's vertices for unchanged
 * inputs). Requires TC_FLAG_WRITE_FULLCLUSTERS. */
tc_status tc_generate_vertices(tc_context* ctx, const tc_frame_args* args, void* stream);

/* Adjoint of the vertex generation of the last frame built in `args` (full
 * clusters and part triangles, tessellation decisions held fixed): scatters
 * dL/d(genVertices) into base positions, base normals and displacement texels.
 * gradTargets: device tc_GradTargets[numInstances]; gradTexels: device
 * uint64_t[numTextures] of float arrays (width*height) or 0 entries.
 * Requires the frame to have been built with TC_FLAG_WRITE_FULLCLUSTERS. */
tc_status tc_instantiate_backward(tc_context* ctx, const tc_frame_args* args, uint64_t gradVertices,
                                  uint64_t gradTargets, uint64_t gradTexels, void* stream);

/* ---- hit-time decode ------------------------------------------------------------ */

/* A ray hit on the frame's cluster geometry as a cluster ray tracer reports it
 * (render_raytrace_clusters.rchit.glsl:131-235): the instance, the hit CLAS's
 * cluster ID with the RT_CLUSTER_MODE in its top two bits (the instantiation's
 * clusterIdOffset), the triangle within the CLAS and the two hit barycentrics. */
typedef struct tc_hit {
  uint32_t instanceID;
  uint32_t clusterID;
  uint32_t triangleID;
  float    barycentrics[2];
  uint32_t _pad;
} tc_hit;

#define TC_HIT_OK 0u
#define TC_HIT_UNSUPPORTED_MODE 1u /* a transient-build mode the frame was not built with */
#define TC_HIT_OUT_OF_RANGE 2u     /* instance, part, cluster or triangle index outside the frame's data */

/* The hit on the base mesh: base cluster and triangle, the triangle's vertex
 * indices into the instance's vertex arrays, their weights, and the
 * reference's per-hit part id (rchit.glsl:203-214; depends on
 * FrameConstants.visualize). */
typedef struct tc_base_hit {
  uint32_t clusterID;
  uint32_t triangleID;
  uint32_t vertexIndices[3];
  float    barycentrics[3];
  uint32_t partID;
  uint32_t status; /* TC_HIT_* */
} tc_base_hit;

/* Decode `count` hits (device arrays) against the frame last built in `args`
 * (render_raytrace_clusters.rchit.glsl:131-214): part-triangle and 2X batch
 * hits go through the table triangle and the sub-triangle corners to base
 * barycentrics, 1X subset hits through the triangle map, full-cluster hits map
 * directly. The transient modes decode when args->flags has the matching
 * TC_FLAG_TRANSIENT_* bit, else they report TC_HIT_UNSUPPORTED_MODE. */
tc_status tc_decode_hits(tc_context* ctx, const tc_frame_args* args, const tc_hit* hits, uint32_t count,
                         tc_base_hit* out, void* stream);

/* ---- raster batching --------------------------------------------------------- */

/* render_raster_clusters_batched.task.glsl:115-215 and .mesh.glsl:141-435 as
 * compute: the frame's part triangles, 32 at a time (one task workgroup), are
 * packed into batches of consecutive parts of at most TC_RASTER_BATCH_VERTICES
 * vertices and TC_RASTER_BATCH_TRIANGLES triangles (the task shader's linear
 * fill); every part's tessellated vertices are displaced, taken to world and
 * clip space and written with its triangles' batch-local indices and
 * primitive IDs, like the mesh shader's outputs. Vertex and triangle arrays are
 * in part order (a batch's are contiguous). */
#define TC_RASTER_BATCH_VERTICES 96u  /* shaderio_scene.h:57-58 */
#define TC_RASTER_BATCH_TRIANGLES 121u

typedef struct tc_raster_batch {
  uint32_t firstPart;     /* index into SceneBuilding.partTriangles */
  uint32_t partCount;
  uint32_t firstVertex;   /* into clipPositions / worldPositions */
  uint32_t numVertices;
  uint32_t firstTriangle; /* into indices / primitiveIDs */
  uint32_t numTriangles;
} tc_raster_batch;

typedef struct tc_raster_outputs {
  uint64_t batches;        /* tc_raster_batch[maxBatches] (device) */
  uint64_t counts;         /* uint32_t[3] (device): batches, vertices, triangles written */
  uint64_t clipPositions;  /* float[4 * maxVertices]: viewProjMatrix * world position (gl_Position) */
  uint64_t worldPositions; /* float[3 * maxVertices] (the mesh shader's wPos) */
  uint64_t indices;        /* uint8_t[3 * maxTriangles]: vertex indices local to the batch */
  uint64_t primitiveIDs;   /* uint32_t[maxTriangles]: gl_PrimitiveID ((triangleID & 0xFF) | (partID | 1) << 8) */
  uint32_t maxBatches;
  uint32_t maxVertices;
  uint32_t maxTriangles;
  uint32_t _pad;
} tc_raster_outputs;

/* Batches of the parts of the frame last built in `args` (ray-tracing or
 * raster frames alike). Totals beyond the output capacities are counted but
 * not written (TC_DEVERR_CAPACITY in the device error word). The readback is
 * not touched (the raster path's statistics would count the frame twice). */
tc_status tc_raster_batches(tc_context* ctx, const tc_frame_args* args, const tc_raster_outputs* out, void* stream);

/* ---- diagnostics ------------------------------------------------------------- */

/* Synchronously read (and clear) the device error word. */
tc_status tc_read_device_errors(tc_context* ctx, uint32_t* outBits, void* stream);
/* Number of kernel launches issued by this context since creation. */
uint64_t tc_launch_count(const tc_context* ctx);

/* No counterpart in the reference (whose look-back-free atomics never wait):
 * a check of the bounded device-side wait every look-back of this library
 * uses. One warp waits, as tile 1, for tile 0's state word in the context's
 * frame scratch. With predecessorPublished != 0 tile 0 holds an inclusive
 * prefix of 7 and *outPrefix = 7. With 0 nothing ever publishes it: the wait
 * gives up after the schedule's lookbackSpinLimit polls, sets
 * TC_DEVERR_LOOKBACK_TIMEOUT in the error word (tc_read_device_errors) and
 * returns, *outPrefix = 0. Synchronises `stream`; must not overlap a frame of
 * the same context (it reuses the frame scratch). */
tc_status tc_lookback_probe(tc_context* ctx, uint32_t predecessorPublished, uint64_t* outPrefix, void* stream);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
static_assert(sizeof(tc_TessTableEntry) == 8, "TessTableEntry");
static_assert(sizeof(tc_hit) == 24, "tc_hit");
static_assert(sizeof(tc_base_hit) == 40, "tc_base_hit");
static_assert(sizeof(tc_TessellationTable) == 40, "TessellationTable");
static_assert(sizeof(tc_BBox) == 32, "BBox");
static_assert(sizeof(tc_Cluster) == 16, "Cluster");
static_assert(sizeof(tc_RenderInstance) == 192, "RenderInstance");
static_assert(sizeof(tc_ClusterInfo) == 8, "ClusterInfo_size (shaderio_building.h:68)");
static_assert(sizeof(tc_TessTriangleInfo) == 24, "TessTriangleInfo_size (shaderio_building.h:92)");
static_assert(sizeof(tc_ClasBuildInfo) == 64, "ClasBuildInfo");
static_assert(sizeof(tc_raster_batch) == 24, "raster batch");
static_assert(sizeof(tc_raster_outputs) == 64, "raster outputs");
static_assert(sizeof(tc_TemplateInstantiateInfo) == 32, "TemplateInstantiateInfo");
static_assert(sizeof(tc_BlasBuildInfo) == 16, "BlasBuildInfo");
static_assert(sizeof(tc_SceneBuilding) == 368, "SceneBuilding");
static_assert(offsetof(tc_SceneBuilding, genClusterDataCounter) == 72, "SceneBuilding layout");
static_assert(offsetof(tc_SceneBuilding, instanceStates) == 104, "SceneBuilding layout");
static_assert(offsetof(tc_SceneBuilding, positionTruncateBitCount) == 208, "SceneBuilding layout");
static_assert(offsetof(tc_SceneBuilding, blasBuildInfos) == 328, "SceneBuilding layout");
static_assert(offsetof(tc_FrameConstants, viewport) == 496, "FrameConstants layout");
static_assert(offsetof(tc_FrameConstants, tessRate) == 540, "FrameConstants layout");
static_assert(offsetof(tc_FrameConstants, nearPlane) == 648, "FrameConstants layout");
static_assert(offsetof(tc_FrameConstants, hizSizeFactors) == 656, "FrameConstants layout");
static_assert(sizeof(tc_FrameConstants) == 784, "FrameConstants prefix");
static_assert(sizeof(tc_Readback) == 880, "Readback");
static_assert(sizeof(tc_DisplacementTexture) == 24, "DisplacementTexture");
static_assert(sizeof(tc_frame_args) == 96, "frame args");
static_assert(sizeof(tc_schedule) == 40, "schedule");
#endif

#endif /* TC_TESSELLATION_H_ */
