// tc_kernels.h — host-side launchers of the stage kernels (implemented in the
// tc_*.cu files). Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include "tc_tessellation.h"

namespace tc {

struct StageCtx;
typedef uint32_t u32;

cudaError_t launch_frame_begin(const StageCtx& c, u32 grid, cudaStream_t s);
cudaError_t launch_instances_classify(const StageCtx& c, u32 grid, u32 block, cudaStream_t s);
cudaError_t launch_clusters_cull(const StageCtx& c, u32 grid, u32 block, cudaStream_t s);
cudaError_t launch_build_setup(const StageCtx& c, u32 mode, cudaStream_t s);
cudaError_t launch_cluster_classify(const StageCtx& c, u32 warpsPerBlock, u32 grid, cudaStream_t s);
cudaError_t launch_triangle_split(const StageCtx& c, u32 blockSize, u32 grid, cudaStream_t s);
cudaError_t launch_triangle_instantiate(const StageCtx& c, u32 blockSize, u32 grid, cudaStream_t s);
cudaError_t launch_blas_setup_insertion(const StageCtx& c, u32 grid, u32 block, cudaStream_t s);
cudaError_t launch_blas_clusters_insert(const StageCtx& c, u32* segStart, u32* segEnd, u32 stride, u32 grid,
                                        cudaStream_t s);
cudaError_t launch_instantiate_backward(const StageCtx& c, const float* gradVertices, const tc_GradTargets* targets,
                                        float* const* gradTexels, u32 grid, cudaStream_t s);

// tiles per launch for each stage (used to size the look-back scratch)
constexpr u32 kInstanceTile     = 256;  // instances per tile (instances_classify, blas_setup)
constexpr u32 kCullTile         = 256;  // clusters per tile
constexpr u32 kClassifyMinWarps = 2;    // smallest clusters-per-tile variant
constexpr u32 kSplitMinItems    = 16;   // smallest split items-per-tile variant
constexpr u32 kInstantiateTile  = 32;   // part triangles per tile

}  // namespace tc
