// tc_kernels.h — host-side launchers of the stage kernels (implemented in the
// tc_*.cu files). Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include "tc_tessellation.h"

namespace tc {

struct StageCtx;
typedef uint32_t u32;

// exclusive offsets of one visible cluster's appends
struct ClusterOffsets
{
  u32                part, split, gen, vert;
  unsigned long long data;
};
static_assert(sizeof(ClusterOffsets) == 24, "ClusterOffsets: three 8-byte words");

// with transient builds, the bases of the counters only they use (stored
// right after the ClusterOffsets bases): the back of the two-sided part
// counter, the transient builds and the template instantiations so far
struct TransBases
{
  u32 back, trans, temp, _pad;
};

// per range of visible clusters: the sums of the clusters' counts, packed
// (parts | splits << 32, full clusters | their vertices << 32, CLAS bytes;
// with transient builds: generated clusters | vertices << 32, and back slots |
// transient builds << 32 in backTrans)
struct RangeSums
{
  unsigned long long partsSplits, fullVerts, data, backTrans;
};

// cluster_classify scratch: per visible cluster of a launch's window, and per
// block of the classify grid (each write block owns a contiguous range of clusters)
struct ClassifyBuffers
{
  uint2*          counts;     // 8 bytes per cluster (16 with transient builds)
  u32*            triWords;   // 64 per cluster
  RangeSums*      rangeSums;  // per block: the sums of its range's counts (zero before the launch)
  ClusterOffsets* bases;      // one: the counters before the launch (then one TransBases)
  uint2*          fullRecs;   // per full cluster of the window: visible index, first generated vertex
  u32*            fullRange;  // [2]: the window's generated-cluster slots
};

cudaError_t launch_frame_begin(const StageCtx& c, u32 grid, cudaStream_t s);
cudaError_t launch_decode_hits(const StageCtx& c, const tc_hit* hits, u32 count, tc_base_hit* out, cudaStream_t s);
cudaError_t launch_instances_classify(const StageCtx& c, u32 grid, u32 block, cudaStream_t s);
// frame_begin and instances_classify in one launch (block = kInstanceTile)
cudaError_t launch_frame_begin_instances(const StageCtx& c, u32 grid, cudaStream_t s);
// side: launched on a side stream beside classify (an ordinary launch, see
// launch_side); otherwise programmatically after the kernel before it
cudaError_t launch_clusters_cull(const StageCtx& c, u32 grid, u32 block, cudaStream_t s, bool side = false);
cudaError_t launch_build_setup(const StageCtx& c, u32 mode, cudaStream_t s);
// a frame's host traffic: `bytes` from mapped pinned host memory (src, its
// device alias) to device memory, both 16-byte aligned; the Readback to
// mapped pinned host memory (dst, its device alias, 4-byte aligned)
struct HostUpload
{
  const void*        src;
  void*              dst;
  unsigned long long bytes;
};
// on its own (at most maxGrid blocks), or inside the batched frame's first
// kernel (launch_frame_begin_instances with the upload; c's frame constants
// and instance records point into the host block)
cudaError_t launch_host_upload(const HostUpload& u, u32 maxGrid, cudaStream_t s);
cudaError_t launch_frame_begin_instances_upload(const StageCtx& c, const HostUpload& u, u32 grid, cudaStream_t s);
cudaError_t launch_host_readback(const tc_Readback* src, void* dst, cudaStream_t s);
// the bounded look-back wait on its own (state: 3 words, zeroed here)
cudaError_t launch_lookback_probe(unsigned long long* state, u32 published, u32* errorWord, u32 spinLimit,
                                  cudaStream_t s);
cudaError_t launch_cluster_classify(const StageCtx& c, const ClassifyBuffers& buf, u32 maxClusters, u32 numSMs,
                                    u32 warpBlocksPerSM, cudaStream_t s);
// the full clusters' displaced vertices of the last launch_cluster_classify
cudaError_t launch_classify_full_vertices(const StageCtx& c, const ClassifyBuffers& buf, u32 maxClusters, u32 numSMs,
                                          u32 blocksPerSM, cudaStream_t s);
u32         classify_max_blocks(u32 maxClusters);
cudaError_t launch_triangle_split(const StageCtx& c, u32 blockSize, u32 grid, cudaStream_t s);
// every split pass in one launch: per level its look-back rows and control
// words (a scratch slot each; the ticket of level 0's slot is the launch's)
constexpr u32 kMaxSplitLevels = 16;
struct SplitLevels
{
  unsigned long long* lbState[kMaxSplitLevels];  // [2][stride] per level
  u32*                ctrl[kMaxSplitLevels];     // 16 words per level (see tc_split.cu)
  u32                 stride;                    // tiles per level the rows hold
  u32                 levels;                    // split passes
};
cudaError_t launch_triangle_split_levels(const StageCtx& c, const SplitLevels& lv, u32 blockSize, u32 grid,
                                         cudaStream_t s);
// triangle_tess_template_instantiate scratch, per part triangle
struct InstantiateBuffers
{
  u32*                vertexOffset;  // first generated vertex of each accepted part, ~0 otherwise
  unsigned long long* chunkSums;     // per 32 parts: packed (CLAS bytes << 20 | vertices)
};

// four launches (tile sums, tile scan, args, vertices); the slot needs 3 state rows of
// instantiate_alloc_tiles(maxParts)
cudaError_t launch_triangle_instantiate(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                        u32 scanBlocksPerSM, u32 vertexBlocksPerSM, u32 vertexGridPerSM,
                                        cudaStream_t s);
// the two halves of launch_triangle_instantiate: allocation and arguments
// (tile sums, tile scan, args), then the displaced vertices, which depend on
// the allocation alone
cudaError_t launch_instantiate_alloc(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                     u32 scanBlocksPerSM, cudaStream_t s);
// its two parts: the offsets (tile sums and scan; they advance the counters,
// the instantiation counter by the run's accepted parts), then the arguments
cudaError_t launch_instantiate_prefix(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                      u32 scanBlocksPerSM, cudaStream_t s);
cudaError_t launch_instantiate_args(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                    u32 scanBlocksPerSM, cudaStream_t s);
cudaError_t launch_instantiate_vertices(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                        u32 vertexBlocksPerSM, u32 vertexGridPerSM, cudaStream_t s);
u32         instantiate_alloc_tiles(u32 maxParts);
// the stage entry point's form: tile sums, tile scan, then arguments and
// vertices in one kernel (PN / ripple: launch_triangle_instantiate)
cudaError_t launch_instantiate_fused(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                     u32 scanBlocksPerSM, u32 vertexBlocksPerSM, u32 vertexGridPerSM, cudaStream_t s);
cudaError_t launch_blas_setup_insertion(const StageCtx& c, u32 grid, u32 block, cudaStream_t s);
cudaError_t launch_blas_clusters_insert(const StageCtx& c, u32* segStart, u32* segEnd, u32 stride, u32 grid,
                                        cudaStream_t s);
// raster batching of the frame's parts; `groups`: one uint4 per 32 parts
cudaError_t launch_raster_batches(const StageCtx& c, uint4* groups, const tc_raster_outputs& o, u32 maxParts,
                                  u32 numSMs, cudaStream_t s);
cudaError_t launch_generate_vertices(const StageCtx& c, u32 grid, cudaStream_t s);
cudaError_t launch_instantiate_backward(const StageCtx& c, const float* gradVertices, const tc_GradTargets* targets,
                                        float* const* gradTexels, u32 grid, cudaStream_t s);

// tiles per launch for each stage (used to size the look-back scratch)
constexpr u32 kInstanceTile     = 256;  // instances per tile (instances_classify, blas_setup)
constexpr u32 kCullTile         = 256;  // clusters per tile
constexpr u32 kSplitMinItems    = 16;   // smallest split items-per-tile variant
constexpr u32 kInstantiateTile  = 1024; // part triangles per instantiate tile

}  // namespace tc
