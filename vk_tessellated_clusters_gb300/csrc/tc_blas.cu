// tc_blas.cu — per-BLAS cluster reference lists.
//
// blas_setup_insertion (shaders/blas_setup_insertion.comp.glsl:100-116): the
// per-instance CLAS counts become list offsets. The reference takes them with
// an atomicAdd per instance (arbitrary order); here they are the exclusive scan
// in instance order (block scan + look-back), as a serial loop would assign.
//
// blas_clusters_insert (shaders/blas_clusters_insert.comp.glsl:97-136): every
// template instantiation (then every transient build) appends its CLAS
// address to its instance's list. The
// reference's atomicAdd per insertion gives an arbitrary order within a list;
// here the order is the instantiation order (a stable scatter). The
// instantiation list is a concatenation of runs (full clusters, then the part
// triangles of classify and of each split pass), each sorted by instance
// because every producer appends in instance order; a first kernel marks the
// start and end of every (run, instance) segment, the scatter kernel then
// places element j at
//   list(inst) + sum_{r' < r} count(r', inst) + (j - segStart(r, inst)).
#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

namespace {

__global__ void k_blas_setup_insertion(StageCtx c)
{
  stage_prologue();
  __shared__ u32 s_tile, s_flag, s_warp[33];
  __shared__ u64 s_excl;
  tc_SceneBuilding* b        = c.build;
  tc_BlasBuildInfo* infos    = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  const u32*        sizes    = reinterpret_cast<const u32*>(b->blasBuildSizes);
  const u32         n        = b->numRenderInstances;
  u32         numTiles = (n + blockDim.x - 1) / blockDim.x;
  numTiles = clamp_tiles(c, numTiles);
  u32               statSizes = 0;
  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;
    const u32  i     = tile * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const u32  count = valid ? infos[i].clusterReferencesCount : 0u;
    u32        total;
    const u32  excl = block_exclusive_scan(count, s_warp, &total);
    if(threadIdx.x < 32)
    {
      const u64 ex =
          warp_lookback_exclusive(c.scratch.lbState, tile, total, tile == 0 ? b->blasClusterCounter : 0, c.errorWord,
                                  c.spinLimit);
      if(threadIdx.x == 0)
      {
        s_excl = ex;
        if(tile == numTiles - 1)
          c.scratch.totals[0] = ex + total;
      }
    }
    __syncthreads();
    if(valid)
    {
      const u64 offset                 = s_excl + excl;
      infos[i].clusterReferencesCount  = 0;
      infos[i].clusterReferencesStride = 8;
      infos[i].clusterReferences       = b->blasClusterAddresses + offset * 8ull;
      if(sizes)
        statSizes += sizes[i];  // last frame's result, statistics only
    }
    __syncthreads();
  }
  for(int o = 16; o > 0; o >>= 1)
    statSizes += __shfl_xor_sync(0xFFFFFFFFu, statSizes, o);
  if((threadIdx.x & 31) == 0 && statSizes)
    atomicAdd(&c.readback->numBlasActualSizes, statSizes);
  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0 && numTiles)
      b->blasClusterCounter = (u32)c.scratch.totals[0];
    scratch_release(c, numTiles, 1);
  }
}

// Run boundaries over the insertion list: template instantiations [0, F)
// full clusters, then part runs; with transient builds one more run, the
// transient builds (list positions temps + j), inserted after every template
// instantiation like the reference's second dispatch
// (blas_clusters_insert.comp.glsl:99-121).
struct Runs
{
  u32 bound[kMaxRuns + 4];
  u32 count;
  u32 temps;  // list positions below hold template instantiations
  u32 total;
};

__device__ inline void load_runs(const StageCtx& c, Runs& r)
{
  const tc_SceneBuilding* b      = c.build;
  const u32               temps  = b->tempInstantiateCounter;
  const u32               full   = c.runStarts[kMaxRuns + 1];
  const u32               nparts = min(b->splitPass + 2, kMaxRuns);
  r.bound[0]                     = 0;
  r.bound[1]                     = min(full, temps);
  for(u32 q = 0; q < nparts; q++)
    r.bound[q + 2] = min(full + c.runStarts[q + 1], temps);
  r.count = nparts + 1;
  // the last run always ends at the instantiation count
  r.bound[r.count] = temps;
  r.temps          = temps;
  r.total          = temps;
  if(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
  {
    r.total = temps + b->transBuildCounter;
    r.count += 1;
    r.bound[r.count] = r.total;
  }
}

// list position j: its instance, CLAS address and size
__device__ __forceinline__ u32 entry_instance(const tc_SceneBuilding* b, const Runs& r, u32 j)
{
  return j < r.temps ? reinterpret_cast<const u32*>(b->tempInstanceIDs)[j]
                     : reinterpret_cast<const u32*>(b->transInstanceIDs)[j - r.temps];
}

__device__ __forceinline__ u32 run_of(const Runs& r, u32 j)
{
  u32 q = 0;
  while(q + 1 < r.count && j >= r.bound[q + 1])
    q++;
  return q;
}

// Both insert kernels walk the instantiations in tiles of kInsertTile: thread t
// of a block takes elements t, t + 256, t + 512 and t + 768 of the tile, so each
// load instruction stays coalesced and a thread has four independent load
// chains in flight.
constexpr u32 kInsertBlock = 256;
constexpr u32 kInsertItems = 4;
constexpr u32 kInsertTile  = kInsertBlock * kInsertItems;

// segment tables: segStart/segEnd[run * stride + instance], zeroed beforehand
__global__ void __launch_bounds__(kInsertBlock) k_blas_segments(StageCtx c, u32* segStart, u32* segEnd, u32 stride)
{
  stage_prologue();
  __shared__ Runs s_runs;
  if(threadIdx.x == 0)
    load_runs(c, s_runs);
  __syncthreads();
  const tc_SceneBuilding* b     = c.build;
  const u32               temps = s_runs.total;
  for(u32 t0 = blockIdx.x * kInsertTile; t0 < temps; t0 += gridDim.x * kInsertTile)
  {
    u32 prev[kInsertItems], cur[kInsertItems], next[kInsertItems];
#pragma unroll
    for(u32 k = 0; k < kInsertItems; k++)
    {
      const u32 j = t0 + threadIdx.x + k * kInsertBlock;
      cur[k]      = j < temps ? entry_instance(b, s_runs, j) : 0u;
      prev[k]     = j < temps && j > 0 ? entry_instance(b, s_runs, j - 1) : 0u;
      next[k]     = j + 1 < temps ? entry_instance(b, s_runs, j + 1) : 0u;
    }
#pragma unroll
    for(u32 k = 0; k < kInsertItems; k++)
    {
      const u32 j = t0 + threadIdx.x + k * kInsertBlock;
      if(j >= temps)
        continue;
      const u32 inst = cur[k];
      if(inst >= c.numInstances)
      {
        atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
        continue;
      }
      const u32  r     = run_of(s_runs, j);
      const bool first = j == s_runs.bound[r] || prev[k] != inst;
      const bool last  = j + 1 == s_runs.bound[r + 1] || next[k] != inst;
      if(first)
        segStart[r * stride + inst] = j;
      if(last)
        segEnd[r * stride + inst] = j + 1;
    }
  }
}

__global__ void __launch_bounds__(kInsertBlock) k_blas_scatter(StageCtx c, const u32* segStart, const u32* segEnd,
                                                               u32 stride)
{
  stage_prologue();
  __shared__ Runs s_runs;
  if(threadIdx.x == 0)
    load_runs(c, s_runs);
  __syncthreads();
  const tc_SceneBuilding* b     = c.build;
  tc_BlasBuildInfo*       infos = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  const u32*              tcsz  = reinterpret_cast<const u32*>(b->tempClusterSizes);
  const u32*              rcsz  = reinterpret_cast<const u32*>(b->transClusterSizes);
  const u32               temps = s_runs.total;
  u64                     statData = 0;
  for(u32 t0 = blockIdx.x * kInsertTile; t0 < temps; t0 += gridDim.x * kInsertTile)
  {
    u32 inst[kInsertItems], size[kInsertItems];
    u64 addr[kInsertItems];
#pragma unroll
    for(u32 k = 0; k < kInsertItems; k++)
    {
      const u32  j     = t0 + threadIdx.x + k * kInsertBlock;
      const bool tmp   = j < s_runs.temps;
      const u32  jj    = tmp ? j : j - s_runs.temps;
      const u64* addrs = reinterpret_cast<const u64*>(tmp ? b->tempClusterAddresses : b->transClusterAddresses);
      const u32* csz   = tmp ? tcsz : rcsz;
      inst[k]          = j < temps ? entry_instance(b, s_runs, j) : ~0u;
      addr[k]          = j < temps ? addrs[jj] : 0ull;
      size[k]          = csz && j < temps ? csz[jj] : 0u;
    }
#pragma unroll
    for(u32 k = 0; k < kInsertItems; k++)
    {
      const u32 j = t0 + threadIdx.x + k * kInsertBlock;
      if(j >= temps || inst[k] >= c.numInstances)
        continue;
      const u32 r    = run_of(s_runs, j);
      u32       rank = j - segStart[r * stride + inst[k]];
      for(u32 q = 0; q < r; q++)
        rank += segEnd[q * stride + inst[k]] - segStart[q * stride + inst[k]];
      reinterpret_cast<u64*>(infos[inst[k]].clusterReferences)[rank] = addr[k];
      statData += size[k];
    }
  }
  // final list lengths (blas_clusters_insert.comp.glsl:131 increments them one by one)
  for(u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < c.numInstances; i += gridDim.x * blockDim.x)
  {
    u32 total = 0;
    for(u32 q = 0; q < s_runs.count; q++)
      total += segEnd[q * stride + i] - segStart[q * stride + i];
    infos[i].clusterReferencesCount = total;
  }
  for(int o = 16; o > 0; o >>= 1)
    statData += __shfl_xor_sync(0xFFFFFFFFu, statData, o);
  if((threadIdx.x & 31) == 0 && statData)
    atomicAdd(reinterpret_cast<unsigned long long*>(&c.readback->numGenActualDatas), (unsigned long long)statData);
}

}  // namespace

cudaError_t launch_blas_setup_insertion(const StageCtx& c, u32 grid, u32 block, cudaStream_t s)
{
  return launch_pdl_critical(k_blas_setup_insertion, grid, block, s, c);
}

cudaError_t launch_blas_clusters_insert(const StageCtx& c, u32* segStart, u32* segEnd, u32 stride, u32 grid,
                                        cudaStream_t s)
{
  cudaError_t e = launch_pdl_critical(k_blas_segments, grid, kInsertBlock, s, c, segStart, segEnd, stride);
  if(e != cudaSuccess)
    return e;
  return launch_pdl_critical(k_blas_scatter, grid, kInsertBlock, s, c, segStart, segEnd, stride);
}

}  // namespace tc
