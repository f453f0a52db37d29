/*
 * tc_oracle.h — CPU oracle of the tessellated-cluster build chain.
 *
 * TEST INFRASTRUCTURE. This is a restatement, in plain C++, of the reference's
 * GLSL compute shaders (vk_tessellated_clusters shaders/<name>.comp.glsl and
 * shaders/tessellation.glsl) used only by tests/, by __graft_entry__.smoke()
 * and by bench.py's CPU-baseline leg, always as the checker. The shipped
 * library (libtc_gb300.so) never links or calls it.
 *
 * Parity pinning (oracle/Makefile target `ref`, checked by tests/test_ref_pin.py):
 * the tessellation table is pinned to the reference's own generated header
 * compiled here; the struct layouts of include/tc_tessellation.h to the
 * reference's shaderio headers compiled as C++ (every field's offset and size);
 * the shader functions of tessellation.glsl:28-201, culling.glsl:27-92 and
 * displacement.glsl:27-120 to the reference's own GLSL text compiled as C++
 * through a mechanical rewrite and a GLSL built-in shim (oracle/ref_shim/),
 * function by function, on exhaustive and seeded samples.
 *
 * Every "address" inside the tc_* structs handed to the oracle is a HOST
 * pointer. Output order is the canonical serial order (instance, cluster,
 * triangle, then split level by level, parent then child), which the CUDA
 * kernels reproduce exactly.
 */
#ifndef TC_ORACLE_H_
#define TC_ORACLE_H_

#include "tc_tessellation.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tco_table {
  tc_TessTableEntry entries[TC_TESSTABLE_LOOKUP_ENTRIES];
  uint64_t          templateAddresses[TC_TESSTABLE_LOOKUP_ENTRIES];
  uint32_t          templateInstantiationSizes[TC_TESSTABLE_LOOKUP_ENTRIES];
  const uint32_t*   vertices;
  const uint32_t*   triangles;
  uint32_t          numVertices;
  uint32_t          numTriangles;
  uint32_t          maxVertices;
  uint32_t          maxTriangles;
} tco_table;

/* src/tessellation_table.cpp:36-83 */
int tco_table_init(tco_table* t, const uint32_t* vertices, uint32_t numVertices, const uint32_t* triangles,
                   uint32_t numTriangles, const uint16_t* configs, uint32_t numConfigs, uint32_t maxEdgeSegments);

/* shaders/tessellation.glsl pieces, exposed for unit tests */
uint32_t tco_encode_barycentrics(float w, float u, float v);
void     tco_decode_barycentrics(uint32_t enc, float* out3);
void     tco_tess_factors(const float* a, const float* b, const float* c, const float* viewPos, float nearPlane,
                          float viewportH, float tessRate, uint32_t* out3);
uint32_t tco_get_config(const uint32_t* factors3, uint32_t* triangleVertices3);
uint32_t tco_split_factor(uint32_t factor, uint32_t splitFactor);
uint32_t tco_split_pass_count(uint32_t splitFactor);
/* tessellation.glsl:165-189 (flip-aware config triangle / vertex), :191-195 */
void     tco_config_triangle(const tco_table* t, uint32_t cfg, uint32_t tri, uint32_t* out3);
void     tco_config_vertex(const tco_table* t, uint32_t cfg, uint32_t vert, float* out3);
void     tco_interpolate3(const float* base9, const float* wuv, float* out3);
/* displacement.glsl:47-104 (deform_setupPN + deform_getPN), :106-120 rippleDeform */
void     tco_pn_position(const float* verts9, const float* normals9, const float* bary3, float* out3);
void     tco_ripple(const float* p3, uint32_t seed, float geometrySize, const tc_FrameConstants* view, float* out3);
/* culling.glsl:50-90 intersectFrustum, :30-35 intersectSize */
int      tco_intersect_frustum(const float* lo3, const float* hi3, const float* world16, const tc_FrameConstants* viewLast,
                               float* clipMin4, float* clipMax4, int* clipValid);
int      tco_intersect_size(const float* clipMin4, const float* clipMax4, const tc_FrameConstants* viewLast);

/* One frame of the chain (frame_begin .. blas_clusters_insert).
 * args: host addresses everywhere. partRunStarts (may be NULL) receives the raw
 * part counter at the start of each part run (classify, pass 1..P), P+2 entries
 * (last = final raw counter). Returns 0 on success. */
int tco_frame_build(const tco_table* t, const tc_frame_args* args, int numThreads, uint32_t* partRunStarts);

/* Individual stages (same semantics as the frame build's steps). */
void tco_frame_begin(const tc_frame_args* args);
void tco_instances_classify(const tc_frame_args* args);
void tco_clusters_cull(const tc_frame_args* args);
void tco_build_setup(const tc_frame_args* args, uint32_t mode);
void tco_cluster_classify(const tco_table* t, const tc_frame_args* args, int numThreads);
void tco_triangle_split_pass(const tco_table* t, const tc_frame_args* args, int numThreads);
void tco_triangle_instantiate(const tco_table* t, const tc_frame_args* args, int numThreads);
void tco_blas_setup_insertion(const tc_frame_args* args);
void tco_blas_clusters_insert(const tc_frame_args* args);
/* hit-time decode of the frame in `args` (see tc_decode_hits) */
/* render_raster_clusters_batched.task.glsl:115-215 + .mesh.glsl:141-435 (tc_raster_batches) */
void tco_raster_batches(const tco_table* t, const tc_frame_args* args, const tc_raster_outputs* out);
void tco_decode_hits(const tco_table* t, const tc_frame_args* args, const tc_hit* hits, uint32_t count,
                     tc_base_hit* out);

/* FP64 twin of the vertex generation for the accepted instantiations of the
 * frame in `args` (after tco_frame_build or the CUDA build): writes
 * out[3 * genVertexIndex + k] for every generated vertex. fullClusters must have
 * been recorded (TC_FLAG_WRITE_FULLCLUSTERS). Returns number of vertices. */
uint64_t tco_generate_vertices_f64(const tco_table* t, const tc_frame_args* args, double* out, int numThreads);

/* FP64 adjoint of the same vertex generation: given dL/dv per generated vertex
 * (double, 3 per vertex), accumulate into per-instance gradient arrays
 * (host double arrays, parallel to positions/normals; NULL entries skipped) and
 * per-texture texel gradients (double, width*height). */
void tco_backward_f64(const tco_table* t, const tc_frame_args* args, const double* gradVertices,
                      double* const* dPositions, double* const* dNormals, double* const* dTexels);

/* FP64 forward with overridden parameters (for finite differences): like
 * tco_generate_vertices_f64 but positions/normals/texels read from the given
 * double arrays (per instance / per texture) instead of the float inputs. */
uint64_t tco_generate_vertices_f64_params(const tco_table* t, const tc_frame_args* args,
                                          const double* const* positions, const double* const* normals,
                                          const double* const* texels, double* out);

#ifdef __cplusplus
}
#endif

#endif
