// tc_stage.cuh — launch context shared by the stage kernels, the build_setup
// logic (used both by the standalone build_setup kernel and fused into the last
// block of the producing kernel), and the per-launch scratch layout.
#pragma once

#include "tc_device.cuh"

namespace tc {

// Host side of the programmatic dependent launch (see stage_prologue): a
// kernel launch on `s` that may overlap the tail of the previous kernel
// (pdl), with a launch priority (0: the default).
template <typename... Params, typename... Args>
inline cudaError_t launch_kernel(void (*kernel)(Params...), u32 grid, u32 block, int priority, bool pdl,
                                 cudaStream_t s, Args... args)
{
  cudaLaunchConfig_t  cfg = {};
  cudaLaunchAttribute attr[2];
  u32                 n = 0;
  if(pdl)
  {
    attr[n].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[n].val.programmaticStreamSerializationAllowed = 1;
    n++;
  }
  if(priority != 0)
  {
    attr[n].id           = cudaLaunchAttributePriority;
    attr[n].val.priority = priority;
    n++;
  }
  cfg.gridDim          = dim3(grid);
  cfg.blockDim         = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream           = s;
  cfg.attrs            = n ? attr : nullptr;
  cfg.numAttrs         = n;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

template <typename... Params, typename... Args>
inline cudaError_t launch_pdl_prio(void (*kernel)(Params...), u32 grid, u32 block, int priority, cudaStream_t s,
                                   Args... args)
{
  return launch_kernel(kernel, grid, block, priority, true, s, args...);
}

template <typename... Params, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(Params...), u32 grid, u32 block, cudaStream_t s, Args... args)
{
  return launch_pdl_prio(kernel, grid, block, 0, s, args...);
}

// The device's highest launch priority (latency-critical kernels that share
// the GPU with a concurrent branch of the frame).
inline int high_launch_priority()
{
  int least = 0, greatest = 0;
  if(cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
    return 0;
  return greatest;
}

// A kernel on the frame's critical path (classify, the allocations, the BLAS
// lists): highest launch priority, so that its blocks are dispatched before
// pending blocks of the vertex kernels that run beside it on other streams.
template <typename... Params, typename... Args>
inline cudaError_t launch_pdl_critical(void (*kernel)(Params...), u32 grid, u32 block, cudaStream_t s, Args... args)
{
  return launch_pdl_prio(kernel, grid, block, high_launch_priority(), s, args...);
}

// A kernel on a side stream beside the critical path's next kernel: an
// ordinary launch. Launched programmatically, its blocks would be placed on
// the SMs as soon as the kernel before it starts and wait there, holding
// registers the critical path's next kernel needs (measured on the batched
// frame: clusters_cull launched programmatically beside classify delays
// classify by about 4 us; the vertex kernels, which have more work, are
// better placed early: the terrain frame is 12 % slower without it).
template <typename... Params, typename... Args>
inline cudaError_t launch_side(void (*kernel)(Params...), u32 grid, u32 block, cudaStream_t s, Args... args)
{
  return launch_kernel(kernel, grid, block, 0, false, s, args...);
}

// Per-launch scratch: look-back tile states, the tile ticket, the "blocks done"
// counter and the totals the last tile publishes. Zeroed before every launch.
struct LaunchScratch
{
  u64* lbState;       // [numCounters][lbStride]
  u32  lbStride;      // max tiles per launch
  u32  selfClean;     // 1: the last block re-zeroes what the launch used (repeated launches on one slot)
  u32  itemCapacity;  // capacity of the stage's per-item scratch arrays (items per launch)
  u32  _pad;
  u32* ticket;
  u32* done;
  u64* totals;  // [numCounters] inclusive totals (base included) of the last tile
};

struct StageCtx
{
  const tc_FrameConstants*      view;
  const tc_FrameConstants*      viewLast;
  const tc_RenderInstance*      instances;
  tc_SceneBuilding*             build;
  tc_Readback*                  readback;
  const tc_DisplacementTexture* textures;
  u32                           numInstances;
  u32                           numTextures;
  u32                           flags;
  u32                           spinLimit;  // polls before a look-back wait gives up
  Table                         table;
  tc_caps                       caps;
  u32*                          errorWord;
  u32*                          runStarts;         // [kRunStartsSize]: part counter at each run start, the full-cluster count, full attempts
  u32*                          instClusterStart;  // [numInstances + 1] exclusive prefix of numClusters
  float*                        splitBase;         // [maxSplitTriangles][9]: world positions of each split item's base triangle
  LaunchScratch                 scratch;
  u32                           instBegin;  // instance window [instBegin, instEnd)
  u32                           instEnd;
  u32                           fuseSetup;  // build_setup mode run by the last block, or kNoSetup
  u32                           run;        // instantiate: part run index or kAllRuns
  u32                           fuseBlasSetup;  // instantiate: the last block also runs blas_setup_insertion
  u32                           flatVisible;    // classify: the visible list is every cluster in instance order
                                                // (RT semantics, whole window), read from instClusterStart
                                                // instead of waiting for clusters_cull
  uint4*                        zeroBase;  // frame_begin: scratch it zeroes (the batched frame's later slots), or null
  u64                           zeroN16;   // its size in 16-byte words
};

constexpr u32 kNoSetup        = 0xFFFFFFFFu;
constexpr u32 kAllRuns        = 0xFFFFFFFFu;
constexpr u32 kRunsAfterFirst = 0xFFFFFFFEu;  // instantiate: every run but the first (the split passes' parts)
constexpr u32 kMaxRuns  = 16;
// runStarts[kFullAttemptsSlot]: full-cluster attempts of the frame's classify
// launches (with transient builds, generated clusters are not all full ones)
constexpr u32 kFullAttemptsSlot = kMaxRuns + 2;
constexpr u32 kRunStartsSize    = kMaxRuns + 3;

__device__ __forceinline__ u32 clamp_split_factor(u32 sf) { return max(2u, min(sf, TC_TESSTABLE_SIZE)); }

__device__ __forceinline__ bool whole_window(const StageCtx& c) { return c.instBegin == 0 && c.instEnd >= c.numInstances; }

// shaders/build_setup.comp.glsl:102-265 (RT target, non-persistent split; the
// transient-build branches with TC_FLAG_TRANSIENT_*), plus bookkeeping of the part-run boundaries that the
// per-instance launch path and the backward pass use.
__device__ inline void build_setup_apply(const StageCtx& c, u32 mode)
{
  tc_SceneBuilding* b  = c.build;
  tc_Readback*      rb = c.readback;
  const tc_caps&    k  = c.caps;
  switch(mode)
  {
    case TC_BUILD_SETUP_CLASSIFY:
    {
      u32 counter              = b->visibleClusterCounter;
      rb->numVisibleClusters   = counter;
      counter                  = min(counter, k.maxVisibleClusters);
      b->visibleClusterCounter = counter;
      b->dispatchClassify      = {counter, 1, 1};
      break;
    }
    case TC_BUILD_SETUP_DRAW_TESS:
    {
      u32 full              = b->fullClusterCounter;
      u32 part              = b->partTriangleCounter;
      rb->numFullClusters   = full;
      rb->numPartTriangles  = part;
      rb->numSplitTriangles = b->splitWriteCounter;
      full                  = min(full, k.maxVisibleClusters);
      part                  = min(part, k.maxPartTriangles);
      b->drawFullClusters   = {full, 0};
      b->drawPartTriangles  = {(part + 31) / 32, 0};
      rb->numBlasClusters   = full;
      break;
    }
    case TC_BUILD_SETUP_SPLIT:
    {
      int32_t s                = b->splitTriangleCounter;
      u32     count            = s < 0 ? 0u : min((u32)s, k.maxSplitTriangles);
      b->splitWriteCounter     = count;
      b->splitTriangleCounter  = (int32_t)count;
      b->splitPassStart        = 0;
      b->splitPassEnd          = count;
      b->dispatchTriangleSplit = {(count + 63) / 64, 1, 1};
      c.runStarts[0] = 0;
      if(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
      {
        // classify's part requests from the front (its blocks may still be
        // raising the written end, partTriangleCounter, which the
        // instantiation clamps this run to)
        c.runStarts[1]            = (u32)b->dualPartTriangleCounter;
        c.runStarts[kMaxRuns + 1] = c.runStarts[kFullAttemptsSlot];
      }
      else
      {
        c.runStarts[1]            = b->partTriangleCounter;
        c.runStarts[kMaxRuns + 1] = b->genClusterCounter;  // full-cluster instantiation attempts
      }
      break;
    }
    case TC_BUILD_SETUP_SPLIT_PASS:
    {
      u32 pass                 = b->splitPass + 1;
      b->splitPass             = pass;
      u32 start                = min(b->splitPassEnd, k.maxSplitTriangles);
      u32 end                  = min(b->splitWriteCounter, k.maxSplitTriangles);
      b->splitPassStart        = start;
      b->splitPassEnd          = end;
      b->dispatchTriangleSplit = {(end - start + 63) / 64, 1, 1};
      if(pass + 1 <= kMaxRuns)
        c.runStarts[pass + 1] = b->partTriangleCounter;
      break;
    }
    case TC_BUILD_SETUP_BUILD_BLAS:
    {
      const bool trans                = (c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)) != 0;
      u32        temp                 = b->tempInstantiateCounter;
      u32        tr                   = trans ? b->transBuildCounter : 0u;
      rb->numBlasClusters             = temp + tr;
      rb->numTransBuilds              = tr;
      rb->numTempInstantiations       = temp;
      rb->numGenDatas                 = b->genClusterDataCounter;
      rb->numGenVertices              = b->genVertexCounter;
      rb->numBlasReservedSizes        = b->numBlasReservedSizes;
      temp                            = min(k.maxGeneratedClusters, temp);
      b->tempInstantiateCounter       = temp;
      rb->numActualTempInstantiations = temp;
      b->dispatchBlasTempInsert       = {(temp + 63) / 64, 1, 1};
      if(trans)  // :211-233
      {
        tr                          = min(k.maxGeneratedClusters, temp + tr) - temp;
        b->transBuildCounter        = tr;
        rb->numActualTransBuilds    = tr;
        b->dispatchBlasTransInsert  = {(tr + 63) / 64, 1, 1};
      }
      break;
    }
    case TC_BUILD_SETUP_INSTANTIATE_TESS:
    {
      u32 part              = b->partTriangleCounter;
      rb->numSplitTriangles = b->splitWriteCounter;
      if(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
      {
        // :242-265: requests from both ends; partTriangleCounter is the end
        // of the written front
        const u32 lo              = (u32)b->dualPartTriangleCounter;
        const u32 hi              = (u32)(b->dualPartTriangleCounter >> 32);
        rb->numPartTriangles      = lo + hi;
        rb->numTransPartTriangles = hi;
      }
      else
        rb->numPartTriangles = part;
      if(b->splitPass + 2 <= kMaxRuns)
        c.runStarts[b->splitPass + 2] = part;
      part                           = min(part, k.maxPartTriangles);
      b->partTriangleCounter         = part;
      b->dispatchTriangleInstantiate = {(part + 31) / 32, 1, 1};
      break;
    }
    default:
      break;
  }
}

// A launch never uses more look-back tiles than its scratch slot holds; a
// request beyond that (inconsistent host-side sizes) is recorded and truncated.
__device__ __forceinline__ u32 clamp_tiles(const StageCtx& c, u32 numTiles)
{
  if(numTiles > c.scratch.lbStride)
  {
    if(threadIdx.x == 0 && blockIdx.x == 0)
      atomicOr(c.errorWord, TC_DEVERR_CAPACITY);
    return c.scratch.lbStride;
  }
  return numTiles;
}

// Tile handout: one ticket per tile, broadcast through shared memory.
__device__ __forceinline__ u32 next_tile(const StageCtx& c, u32* s_tile)
{
  if(threadIdx.x == 0)
    *s_tile = atomicAdd(c.scratch.ticket, 1u);
  __syncthreads();
  u32 t = *s_tile;
  __syncthreads();
  return t;
}

// "Last block" detection: returns true in exactly one block, after every block
// of the launch has finished its work (classic threadfence reduction pattern).
__device__ __forceinline__ bool last_block_done(const StageCtx& c, u32* s_flag)
{
  __syncthreads();
  if(threadIdx.x == 0)
  {
    __threadfence();
    u32 prev = atomicAdd(c.scratch.done, 1u);
    *s_flag  = (prev == gridDim.x - 1) ? 1u : 0u;
  }
  __syncthreads();
  bool last = *s_flag != 0;
  if(last)
    __threadfence();
  return last;
}

// Run by every thread of the last block after its finalisation: when the slot
// is reused by the next launch without a memset, put it back to zero.
__device__ inline void scratch_release(const StageCtx& c, u32 numTiles, u32 numCounters)
{
  if(!c.scratch.selfClean)
    return;
  __syncthreads();
  const u32 n = min(numTiles, c.scratch.lbStride);
  for(u32 q = 0; q < numCounters; q++)
    for(u32 t = threadIdx.x; t < n; t += blockDim.x)
      c.scratch.lbState[(u64)q * c.scratch.lbStride + t] = 0;
  if(threadIdx.x == 0)
  {
    for(u32 q = 0; q < numCounters; q++)
      c.scratch.totals[q] = 0;
    *c.scratch.ticket = 0;
    *c.scratch.done   = 0;
  }
}

}  // namespace tc

namespace tc {

// Block-wide exclusive scan of one u32 per thread. `s_warp` needs 33
// entries (one per warp plus the total). Returns the exclusive prefix; *total
// receives the block sum.
__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32* s_warp, u32* total)
{
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  u32       x    = v;
#pragma unroll
  for(int d = 1; d < 32; d <<= 1)
  {
    u32 y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if(lane >= (u32)d)
      x += y;
  }
  if(lane == 31)
    s_warp[warp] = x;
  __syncthreads();
  if(warp == 0)
  {
    u32 w = lane < nwarps ? s_warp[lane] : 0;
    u32 s = w;
#pragma unroll
    for(int d = 1; d < 32; d <<= 1)
    {
      u32 y = __shfl_up_sync(0xFFFFFFFFu, s, d);
      if(lane >= (u32)d)
        s += y;
    }
    if(lane < nwarps)
      s_warp[lane] = s - w;  // exclusive warp offsets
    if(lane == 31)
      s_warp[32] = s;  // block total
  }
  __syncthreads();
  u32 r  = s_warp[warp] + x - v;
  *total = s_warp[32];
  __syncthreads();
  return r;
}

// shaders/blas_setup_insertion.comp.glsl:100-116 run by one block of 256
// threads (fused into the last block of the launch before it): the
// per-instance CLAS counts become list offsets, the exclusive scan in instance
// order that the multi-block k_blas_setup_insertion computes. Each thread takes
// up to kBlasSetupPerThread consecutive instances.
constexpr u32 kBlasSetupPerThread = 16;
constexpr u32 kBlasSetupFusedMax  = 256 * kBlasSetupPerThread;  // instances the fused form handles

__device__ inline void blas_setup_block(const StageCtx& c)
{
  __shared__ u32    s_scan[33];
  tc_SceneBuilding* b     = c.build;
  tc_BlasBuildInfo* infos = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  const u32*        sizes = reinterpret_cast<const u32*>(b->blasBuildSizes);
  const u32         n     = min(b->numRenderInstances, kBlasSetupFusedMax);
  const u32         per   = (n + blockDim.x - 1) / blockDim.x;
  const u32         i0 = min(n, threadIdx.x * per), i1 = min(n, i0 + per);
  const u64         base = b->blasClusterCounter;
  u32               sum = 0, statSizes = 0;
  for(u32 i = i0; i < i1; i++)
    sum += __ldcg(&infos[i].clusterReferencesCount);
  u32       total;
  const u32 excl   = block_exclusive_scan(sum, s_scan, &total);  // its barriers also order `base` before the write below
  u64       offset = base + excl;
  for(u32 i = i0; i < i1; i++)
  {
    const u32 cnt                    = __ldcg(&infos[i].clusterReferencesCount);
    infos[i].clusterReferencesCount  = 0;
    infos[i].clusterReferencesStride = 8;
    infos[i].clusterReferences       = b->blasClusterAddresses + offset * 8ull;
    offset += cnt;
    if(sizes)
      statSizes += sizes[i];  // last frame's result, statistics only
  }
  for(int o = 16; o > 0; o >>= 1)
    statSizes += __shfl_xor_sync(0xFFFFFFFFu, statSizes, o);
  if((threadIdx.x & 31) == 0 && statSizes)
    atomicAdd(&c.readback->numBlasActualSizes, statSizes);
  if(threadIdx.x == 0 && n)
    b->blasClusterCounter = (u32)(base + total);
}

}  // namespace tc
