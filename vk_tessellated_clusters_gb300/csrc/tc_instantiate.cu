// tc_instantiate.cu — triangle_tess_template_instantiate: template
// instantiation arguments and displaced vertices for every part triangle.
//
// shaders/triangle_tess_template_instantiate.comp.glsl:126-373.
//
// GB300 mapping, four launches; the first three work on tiles of 1024 part
// triangles (striped: item i of thread t is part tile * 1024 + i * 256 + t,
// so every load and store instruction of a warp touches 32 consecutive parts):
//   tile_sums : per tile, the CLAS bytes and vertex counts of its parts
//               (reads the config word of each part only).
//   tile_scan : one block turns the tile sums into each tile's exclusive
//               offsets (plus the counters' values before the launch) and
//               advances the counters: the serial order of the reference's
//               allocation without any cross-block waiting.
//   args      : per tile, the parts' offsets (block scan + tile offset), the
//               capacity test, the 44 B of instantiation arguments per part,
//               the first generated vertex of each part (scratch), CLAS
//               reference counts and statistics.
//   vertices  : 12 B written per generated vertex. A warp takes chunks of 32
//               consecutive parts (its first by index, the rest from a
//               ticket): every part's affine vertex form (tc_vertex.cuh) is
//               set up once in shared memory, one part per lane, then the
//               lanes walk the chunk's contiguous vertex range on consecutive
//               vertices.
#include <algorithm>

#include "tc_kernels.h"
#include "tc_stage.cuh"
#include "tc_vertex.cuh"

namespace tc {

namespace {

constexpr u32 kBlock        = 256;
constexpr u32 kItems        = 4;
constexpr u32 kTile         = kBlock * kItems;
constexpr u32 kWarps        = kBlock / 32;
constexpr u32 kPartsPerWarp = 32;  // parts staged per warp and chunk: one per lane
constexpr u32 kScanBlock    = 1024;
constexpr u32 kChunksPerTile = kTile / kPartsPerWarp;  // 32-part chunks per allocation tile
static_assert(kChunksPerTile == 32, "one warp reads a tile's chunk sums");

static_assert(kTile == kInstantiateTile, "allocation tile size");

// CLAS bytes and vertex counts travel packed as (bytes << 20) | vertices: a
// tile holds at most 1024 x 78 < 2^20 vertices and 1024 x 2^32 bytes.
constexpr u32 kPackShift = 20;
constexpr u64 kPackMask  = (1ull << kPackShift) - 1;

// parts of this launch: [0, part counter), every run after the first, or one
// run, narrowed to the instance window. A single run is bounded by the run
// table alone: the first run's instantiation may run while the split passes
// still append to the part counter.
__device__ inline void part_range(const StageCtx& c, u32& lo, u32& hi)
{
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(c.build->partTriangles);
  const u32                  cap   = c.caps.maxPartTriangles;
  lo                               = 0;
  if(c.run == kAllRuns || c.run == kRunsAfterFirst)
  {
    hi = min(c.build->partTriangleCounter, cap);
    if(c.run == kRunsAfterFirst)
      lo = min(c.runStarts[1], hi);
  }
  else
  {
    const u32 rs = c.runStarts[c.run], re = c.runStarts[c.run + 1];
    lo           = min(rs, cap);
    hi           = min(max(re, rs), cap);
    if(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
    {
      // classify's run ends at its part requests; only the written front holds parts
      hi = min(hi, c.build->partTriangleCounter);
      lo = min(lo, hi);
    }
  }
  if(!whole_window(c))
  {
    auto get = [&](u32 i) { return parts[i].cluster.instanceID; };
    u32  e   = lower_bound_instance(lo, hi, c.instEnd, get);
    lo       = lower_bound_instance(lo, e, c.instBegin, get);
    hi       = e;
  }
}

template <class T>
__device__ __forceinline__ T warp_inclusive(T x, u32 lane)
{
#pragma unroll
  for(int d = 1; d < 32; d <<= 1)
  {
    T y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if(lane >= (u32)d)
      x += y;
  }
  return x;
}

__device__ __forceinline__ u32 part_cfg(const tc_TessTriangleInfo* parts, u32 p)
{
  return __ldg(&parts[p].subTriangle.triangleID_config) >> 16;
}

__device__ __forceinline__ u64 part_packed(const StageCtx& c, u32 cfg)
{
  return ((u64)__ldg(c.table.templateSizes + cfg_index(cfg)) << kPackShift) | table_entry(c.table, cfg).numVertices;
}

// Scratch of the instantiate slot: lbState[tile] = packed tile sum,
// lbState[stride + tile] / lbState[2 * stride + tile] = the tile's exclusive
// CLAS-byte / vertex offset, totals[0] = generated-cluster counter before the
// launch.

// ---------------------------------------------------------------------------
// tile sums
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kBlock) k_instantiate_tile_sums(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ u64 s_warp[kWarps];
  __shared__ u32 s_range[2];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32                  begin    = s_range[0], n = s_range[1] - s_range[0];
  const u32                  numTiles = clamp_tiles(c, (n + kTile - 1) / kTile);
  const tc_TessTriangleInfo* parts    = reinterpret_cast<const tc_TessTriangleInfo*>(c.build->partTriangles);
  for(u32 tile = blockIdx.x; tile < numTiles; tile += gridDim.x)
  {
    // row i of warp w is the 32 consecutive parts of chunk tile * 32 + i * 8 + w
    u64 row[kItems];
#pragma unroll
    for(u32 i = 0; i < kItems; i++)
    {
      const u32 q = tile * kTile + i * kBlock + threadIdx.x;
      row[i]      = q < n ? part_packed(c, part_cfg(parts, begin + q)) : 0ull;
    }
    u64 sum = 0;
#pragma unroll
    for(u32 i = 0; i < kItems; i++)
    {
      const u64 v = warp_sum_u64(row[i]);
      if(lane == 0 && ib.chunkSums)
        ib.chunkSums[tile * kChunksPerTile + i * kWarps + warp] = v;
      sum += v;
    }
    if(lane == 0)
      s_warp[warp] = sum;
    __syncthreads();
    if(threadIdx.x == 0)
    {
      u64 t = 0;
      for(u32 w = 0; w < kWarps; w++)
        t += s_warp[w];
      c.scratch.lbState[tile] = t;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// tile scan (one block)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kScanBlock) k_instantiate_tile_scan(StageCtx c)
{
  stage_prologue();
  __shared__ u64 s_warpData[32], s_warpVerts[32];
  __shared__ u32 s_range[2], s_first, s_tile;
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  tc_SceneBuilding* b = c.build;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32 n        = s_range[1] - s_range[0];
  const u32 numTiles = clamp_tiles(c, (n + kTile - 1) / kTile);
  const u32 stride   = c.scratch.lbStride;
  u64       carryData = b->genClusterDataCounter, carryVerts = b->genVertexCounter;
  const u32 genBase = b->genClusterCounter;
  for(u32 t0 = 0; t0 < numTiles; t0 += kScanBlock)
  {
    const u32 t = t0 + threadIdx.x;
    const u64 v = t < numTiles ? c.scratch.lbState[t] : 0ull;
    u64       d = v >> kPackShift, vx = v & kPackMask;
    u64       id = warp_inclusive<u64>(d, lane), iv = warp_inclusive<u64>(vx, lane);
    if(lane == 31)
    {
      s_warpData[warp]  = id;
      s_warpVerts[warp] = iv;
    }
    __syncthreads();
    if(warp == 0)
    {
      const u64 wd = s_warpData[lane], wv = s_warpVerts[lane];
      const u64 sd = warp_inclusive<u64>(wd, lane), sv = warp_inclusive<u64>(wv, lane);
      s_warpData[lane]  = sd - wd;
      s_warpVerts[lane] = sv - wv;
    }
    __syncthreads();
    const u64 exData  = carryData + s_warpData[warp] + id - d;
    const u64 exVerts = carryVerts + s_warpVerts[warp] + iv - vx;
    if(t < numTiles)
    {
      c.scratch.lbState[stride + t]     = exData;
      c.scratch.lbState[2 * stride + t] = exVerts;
    }
    // the last thread holds the inclusive total of this round
    const u64 lastData  = __shfl_sync(0xFFFFFFFFu, exData + d, 31);
    const u64 lastVerts = __shfl_sync(0xFFFFFFFFu, exVerts + vx, 31);
    __syncthreads();
    if(threadIdx.x == kScanBlock - 1)
    {
      s_warpData[0]  = lastData;
      s_warpVerts[0] = lastVerts;
    }
    __syncthreads();
    carryData  = s_warpData[0];
    carryVerts = s_warpVerts[0];
    __syncthreads();
  }
  // Accepted instantiations: the run's parts before the first one that fails
  // the capacity test (triangle_tess_template_instantiate.comp.glsl:160-167).
  // The offsets count every attempt, so every later part fails too: the
  // accepted parts are a prefix, counted here rather than by the argument
  // launch, so that the next run's allocation need not wait for it.
  const tc_caps& k        = c.caps;
  const u64      maxData  = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  const u32      attempts = min(n, numTiles * kTile);
  u32            accepted = attempts;
  if(carryVerts > k.maxGeneratedVertices || carryData > maxData || (u64)genBase + attempts > k.maxGeneratedClusters)
  {
    // the first tile whose inclusive end exceeds a cap, then its first part that does
    if(threadIdx.x == 0)
    {
      s_first = (u64)genBase < k.maxGeneratedClusters ? k.maxGeneratedClusters - genBase : 0u;
      s_tile  = 0xFFFFFFFFu;
    }
    __syncthreads();
    for(u32 t = threadIdx.x; t < numTiles; t += kScanBlock)
    {
      const u64 v = c.scratch.lbState[t];
      if(c.scratch.lbState[stride + t] + (v >> kPackShift) > maxData
         || c.scratch.lbState[2 * stride + t] + (v & kPackMask) > k.maxGeneratedVertices)
        atomicMin(&s_tile, t);
    }
    __syncthreads();
    const u32 tf = s_tile;
    if(tf < numTiles)
    {
      const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
      const u32                  q     = tf * kTile + threadIdx.x;
      const u64                  own   = q < n ? part_packed(c, part_cfg(parts, s_range[0] + q)) : 0ull;
      const u64                  d = own >> kPackShift, vx = own & kPackMask;
      const u64                  id = warp_inclusive<u64>(d, lane), iv = warp_inclusive<u64>(vx, lane);
      if(lane == 31)
      {
        s_warpData[warp]  = id;
        s_warpVerts[warp] = iv;
      }
      __syncthreads();
      if(warp == 0)
      {
        const u64 wd = s_warpData[lane], wv = s_warpVerts[lane];
        const u64 sd = warp_inclusive<u64>(wd, lane), sv = warp_inclusive<u64>(wv, lane);
        s_warpData[lane]  = sd - wd;
        s_warpVerts[lane] = sv - wv;
      }
      __syncthreads();
      const u64 inData  = c.scratch.lbState[stride + tf] + s_warpData[warp] + id;
      const u64 inVerts = c.scratch.lbState[2 * stride + tf] + s_warpVerts[warp] + iv;
      if(q < n && (inData > maxData || inVerts > k.maxGeneratedVertices))
        atomicMin(&s_first, q);
    }
    __syncthreads();
    accepted = min(attempts, s_first);
  }
  if(threadIdx.x == 0)
  {
    *c.scratch.ticket   = 0;  // the chunk ticket of the vertex launch that follows
    c.scratch.totals[0] = genBase;
    // instantiation slots continue after the accepted ones (transient builds
    // take generated-cluster slots but no instantiation slot)
    const u32 temp         = b->tempInstantiateCounter;
    c.scratch.totals[1]    = temp;
    b->tempInstantiateCounter = temp + accepted;
    if(numTiles)
    {
      // the reference's counters count every attempt, accepted or not
      b->genClusterCounter     = genBase + attempts;
      b->genClusterDataCounter = carryData;
      b->genVertexCounter      = (u32)carryVerts;
    }
  }
}

// ---------------------------------------------------------------------------
// write: arguments, counts, vertices
// ---------------------------------------------------------------------------

// Uniform: every part of the chunk has the map, scale and offset in `m`,
// `scale`, `offset` (held in registers; the records' q6-q8 are not read).
// `tvBase`: per owner lane, its part's first table vertex minus its first
// vertex within the chunk (table index of chunk vertex jj = tvBase + jj).
template <u32 Kind, bool Uniform>
__device__ __forceinline__ void chunk_vertices(const StageCtx& c, const PartAffine* sp, u32 owner, u32 start, u32 tvBase,
                                               u32 total, float* dst, const MapDesc& m, float scale, float offset)
{
  const u32 lane  = threadIdx.x & 31;
  const u32 below = (2u << lane) - 2u;  // bits 1..lane
  #pragma unroll 2  // two steps in flight: their loads overlap
  for(u32 base = 0; base < total; base += 32)
  {
    // lane's part: those starting at or before the step's first vertex, plus
    // those starting inside the step up to the lane (one bit each)
    const u32         before = __popc(__ballot_sync(0xFFFFFFFFu, owner && start <= base));
    const u32         inside = __reduce_or_sync(0xFFFFFFFFu,
                                                (owner && start > base && start < base + 32) ? 1u << (start - base) : 0u);
    const u32         pi     = before - 1 + __popc(inside & below);
    const u32         tvIdx  = __shfl_sync(0xFFFFFFFFu, tvBase, pi & 31);
    const u32         jj     = base + lane;
    const PartAffine& r      = sp[pi];
    if(jj < total)
    {
      const u32 tv = __ldg(c.table.vertices + (tvIdx + jj));
      const f3  q  = Uniform ? affine_vertex_u<Kind>(r, tv, m, scale, offset) : affine_vertex_k<Kind>(r, tv);
      float*   d = dst + 3 * (u64)jj;
      d[0] = q.x, d[1] = q.y, d[2] = q.z;
    }
  }
}

__global__ void __launch_bounds__(kBlock, 4) k_instantiate_args(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ u64        s_rowWarp[kItems][kWarps];  // per row and warp: packed warp totals
  __shared__ u32        s_flag, s_range[2];
  __shared__ u32        s_blasKey[kWarps][2], s_blasCnt[kWarps][2], s_stat[kWarps];
  const u32         lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  tc_SceneBuilding* b    = c.build;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32 begin    = s_range[0], n = s_range[1] - s_range[0];
  const u32 numTiles = clamp_tiles(c, (n + kTile - 1) / kTile);
  const u32 stride   = c.scratch.lbStride;
  const u64 genBase  = c.scratch.totals[0];
  const u64 tempBase = c.scratch.totals[1];

  const tc_caps&             k            = c.caps;
  const tc_TessTriangleInfo* parts        = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  const u64                  maxData      = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  tc_BlasBuildInfo*          blas         = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  u32                        statTris = 0;

  for(u32 tile = blockIdx.x; tile < numTiles; tile += gridDim.x)
  {
    // ---- offsets: block scan of the packed counts, row by row ----------------
    u32 inst[kItems], cfg[kItems];
    u64 own[kItems], incl[kItems];
#pragma unroll
    for(u32 i = 0; i < kItems; i++)
    {
      const u32 q = tile * kTile + i * kBlock + threadIdx.x;
      inst[i] = ~0u, cfg[i] = 0, own[i] = 0;
      if(q < n)
      {
        const uint2* raw = reinterpret_cast<const uint2*>(parts + begin + q);
        inst[i]          = raw[0].x;
        cfg[i]           = raw[2].y >> 16;
        own[i]           = part_packed(c, cfg[i]);
      }
      incl[i] = warp_inclusive<u64>(own[i], lane);
      if(lane == 31)
        s_rowWarp[i][warp] = incl[i];
    }
    __syncthreads();
    const u64 tileData = c.scratch.lbState[stride + tile], tileVerts = c.scratch.lbState[2 * stride + tile];
    u64       rowBase = 0;
    u32       runInst = ~0u, runCount = 0;
#pragma unroll
    for(u32 i = 0; i < kItems; i++)
    {
      u64 before = 0, total = 0;
      for(u32 w = 0; w < kWarps; w++)
      {
        const u64 v = s_rowWarp[i][w];
        before += w < warp ? v : 0ull;
        total += v;
      }
      const u64 within = rowBase + before + incl[i] - own[i];
      rowBase += total;
      const u32 q = tile * kTile + i * kBlock + threadIdx.x;
      if(q >= n)
        continue;
      const u32  p            = begin + q;
      const u32  nv           = (u32)(own[i] & kPackMask);
      const u32  ds           = (u32)(own[i] >> kPackShift);
      const u64  genOffset    = genBase + q;
      const u64  dataOffset   = tileData + (within >> kPackShift);
      const u64  vertexOffset = tileVerts + (within & kPackMask);
      // triangle_tess_template_instantiate.comp.glsl:160-167 capacity test
      const bool accept = !(vertexOffset + nv > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
                            || dataOffset + ds > maxData);
      ib.vertexOffset[p] = accept ? (u32)vertexOffset : ~0u;
      if(!accept)
        continue;
      // accepted instantiations form a prefix of the serial order: consecutive slots
      const u32                   tempOffset = (u32)(tempBase + q);
      tc_TemplateInstantiateInfo* dst = reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations) + tempOffset;
      const u64   tmpl  = __ldg(c.table.templateAddresses + cfg_index(cfg[i]));
      const u64   vaddr = b->genVertices + vertexOffset * 12ull;
      const uint4 lo4   = make_uint4(p | (TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED << 30), 0u, (u32)tmpl, (u32)(tmpl >> 32));
      const uint4 hi4   = make_uint4((u32)vaddr, (u32)(vaddr >> 32), 12u, 0u);
      if((reinterpret_cast<uintptr_t>(dst) & 15) == 0)
      {
        reinterpret_cast<uint4*>(dst)[0] = lo4;
        reinterpret_cast<uint4*>(dst)[1] = hi4;
      }
      else
      {
        uint2* d2 = reinterpret_cast<uint2*>(dst);
        d2[0]     = make_uint2(lo4.x, lo4.y);
        d2[1]     = make_uint2(lo4.z, lo4.w);
        d2[2]     = make_uint2(hi4.x, hi4.y);
        d2[3]     = make_uint2(hi4.z, hi4.w);
      }
      reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]      = inst[i];
      reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset] = b->genClusterData + dataOffset;
      statTris += table_entry(c.table, cfg[i]).numTriangles;
      if(inst[i] != runInst)
      {
        if(runCount)
          atomicAdd(&blas[runInst].clusterReferencesCount, runCount);
        runInst  = inst[i];
        runCount = 0;
      }
      runCount++;
    }
    // Per-instance CLAS reference counts. Parts are instance-sorted within a
    // run, so an instance's parts in this tile are (almost always) contiguous:
    // a warp sums its threads' last runs per distinct instance; its first and
    // last instances go to shared memory and are merged across the block's
    // warps, every other instance is added directly. About one atomic per
    // instance and tile.
    {
      const u32 key      = runCount ? runInst : 0xFFFFFFFFu;
      const u32 holders  = __ballot_sync(0xFFFFFFFFu, runCount != 0);
      const u32 firstKey = holders ? __shfl_sync(0xFFFFFFFFu, key, __ffs(holders) - 1) : 0xFFFFFFFFu;
      const u32 lastKey  = holders ? __shfl_sync(0xFFFFFFFFu, key, 31 - __clz(holders)) : 0xFFFFFFFFu;
      if(lane == 0)
      {
        s_blasKey[warp][0] = firstKey;
        s_blasKey[warp][1] = lastKey;
        s_blasCnt[warp][0] = 0;
        s_blasCnt[warp][1] = 0;
      }
      __syncwarp();
      for(u32 remaining = holders; remaining;)
      {
        const int src = __ffs(remaining) - 1;
        const u32 gk  = __shfl_sync(0xFFFFFFFFu, key, src);
        const u32 sum = __reduce_add_sync(0xFFFFFFFFu, key == gk ? runCount : 0u);
        remaining &= ~__ballot_sync(0xFFFFFFFFu, key == gk);
        if((int)lane == src)
        {
          if(gk == firstKey)
            s_blasCnt[warp][0] = sum;
          else if(gk == lastKey)
            s_blasCnt[warp][1] = sum;
          else
            atomicAdd(&blas[gk].clusterReferencesCount, sum);
        }
      }
    }
    __syncthreads();
    if(threadIdx.x == 0)
    {
      u32 curKey = 0xFFFFFFFFu, curCnt = 0;
      for(u32 w = 0; w < kWarps; w++)
        for(u32 e = 0; e < 2; e++)
        {
          const u32 kk = s_blasKey[w][e], cnt = s_blasCnt[w][e];
          if(cnt == 0)
            continue;
          if(kk != curKey)
          {
            if(curCnt)
              atomicAdd(&blas[curKey].clusterReferencesCount, curCnt);
            curKey = kk;
            curCnt = 0;
          }
          curCnt += cnt;
        }
      if(curCnt)
        atomicAdd(&blas[curKey].clusterReferencesCount, curCnt);
    }

    __syncthreads();  // s_rowWarp and the count merge are rewritten by the next tile
  }

  // statistics: one atomic each per block
#pragma unroll
  for(int o = 16; o > 0; o >>= 1)
  {
    statTris += __shfl_xor_sync(0xFFFFFFFFu, statTris, o);
  }
  if(lane == 0)
  {
    s_stat[warp] = statTris;
  }
  __syncthreads();
  if(threadIdx.x == 0)
  {
    u32 t = 0;
    for(u32 w = 0; w < kWarps; w++)
      t += s_stat[w];
    if(t)
      atomicAdd(&c.readback->numTotalTriangles, t);
  }

  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0 && c.fuseSetup != kNoSetup)
      build_setup_apply(c, c.fuseSetup);
    if(c.fuseBlasSetup)
      blas_setup_block(c);
    // done counter back to zero for a reused slot (nothing else needs clearing)
    if(threadIdx.x == 0 && c.scratch.selfClean)
      *c.scratch.done = 0;
    // the vertex launch that follows hands out chunks from this ticket
    if(threadIdx.x == 0)
      *c.scratch.ticket = 0;
  }
}

// ---------------------------------------------------------------------------
// vertices
// ---------------------------------------------------------------------------

// One lane's part (records r0..r2 of its TessTriangleInfo): its affine
// record in `rec` (tc_vertex.cuh), vertex count, map kind and description,
// first table vertex, displacement scale and offset.
__device__ __forceinline__ void lane_part(const StageCtx& c, uint2 r0, uint2 r1, uint2 r2, PartAffine& rec, u32& nv,
                                          u32& kind, u32& tvBase, float& scale, float& offset, MapDesc& map)
{
  const u32                cfg = r2.y >> 16;
  const u32                tri = r2.y & 0xFFFFu;
  const tc_TessTableEntry  e   = table_entry(c.table, cfg);
  const tc_RenderInstance& in  = c.instances[r0.x];
  const tc_Cluster         cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[r0.y];
  const uint8_t*           lt  = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
  const u32                corner[3] = {r1.x, r1.y, r2.x};
  tc_DisplacementTexture   tx = {};
  if(c.numTextures > 0 && c.textures != nullptr && in.displacementIndex >= 0)
  {
    if((u32)in.displacementIndex < c.numTextures)
      tx = c.textures[in.displacementIndex];
    else
      atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
  }
  scale  = in.displacementScale * c.view->displacementScale;
  offset = in.displacementOffset + c.view->displacementOffset;
  part_affine(rec, corner, cfg_flipped(cfg), reinterpret_cast<const float*>(in.positions),
              reinterpret_cast<const float*>(in.normals), reinterpret_cast<const float*>(in.texcoords),
              cl.firstLocalVertex, lt + tri * 3, e.firstVertex, tx, scale, offset);
  map    = make_map_desc(tx);
  nv     = e.numVertices;
  kind   = map.kind;
  tvBase = e.firstVertex;
}

// The vertices of one chunk, after every lane set up its part's record in
// `sp[lane]` (nv = 0: no part): lanes walk the chunk's contiguous vertex
// range (first generated vertex: lane 0's `vo`) on consecutive vertices, with
// one specialisation for the whole chunk when its parts share a map kind, and
// the map, scale and offset in registers when they share those too.
__device__ __forceinline__ void chunk_generate(const StageCtx& c, const PartAffine* sp, float* gv, u32 vo, u32 nv,
                                             u32 kind, u32 tvBase, const MapDesc& map, float scale, float offset)
{
  const u32 lane = threadIdx.x & 31;
  const u32  inc   = warp_inclusive<u32>(nv, lane);
  const u32  start = inc - nv;  // first vertex of this lane's part within the chunk
  const u32  total = __shfl_sync(0xFFFFFFFFu, inc, kPartsPerWarp - 1);
  const u32  v0    = __shfl_sync(0xFFFFFFFFu, vo, 0);
  const bool owner = lane < kPartsPerWarp && nv > 0;
  tvBase -= start;  // table index of chunk vertex jj: tvBase + jj
  // one specialisation for the whole chunk when its parts share a map kind
  const u32 kind0 = __shfl_sync(0xFFFFFFFFu, kind, 0);
  const u32 kw    = __all_sync(0xFFFFFFFFu, !owner || kind == kind0) ? kind0 : ~0u;
  // the usual chunk: every part displaced from one map with one scale and
  // offset (lane 0 always owns a part: accepted parts form a prefix)
  MapDesc um;
  um.q7 = make_float4(__shfl_sync(0xFFFFFFFFu, map.q7.x, 0), __shfl_sync(0xFFFFFFFFu, map.q7.y, 0),
                      __shfl_sync(0xFFFFFFFFu, map.q7.z, 0), __shfl_sync(0xFFFFFFFFu, map.q7.w, 0));
  um.q8 = make_float4(__shfl_sync(0xFFFFFFFFu, map.q8.x, 0), __shfl_sync(0xFFFFFFFFu, map.q8.y, 0),
                      __shfl_sync(0xFFFFFFFFu, map.q8.z, 0), __shfl_sync(0xFFFFFFFFu, map.q8.w, 0));
  um.kind            = kind0;
  const float uScale = __shfl_sync(0xFFFFFFFFu, scale, 0), uOffset = __shfl_sync(0xFFFFFFFFu, offset, 0);
  const bool  same   = !owner
                    || (__float_as_uint(map.q7.x) == __float_as_uint(um.q7.x)
                        && __float_as_uint(map.q7.y) == __float_as_uint(um.q7.y)
                        && __float_as_uint(map.q7.z) == __float_as_uint(um.q7.z)
                        && __float_as_uint(map.q7.w) == __float_as_uint(um.q7.w)
                        && __float_as_uint(scale) == __float_as_uint(uScale)
                        && __float_as_uint(offset) == __float_as_uint(uOffset) && kind == kind0);
  const bool  uni    = __all_sync(0xFFFFFFFFu, same);
  __syncwarp();
  float* dst = gv + 3 * (u64)v0;
#define TC_CHUNK(K)                                                                                                    \
  (uni ? chunk_vertices<K, true>(c, sp, owner, start, tvBase, total, dst, um, uScale, uOffset)                       \
       : chunk_vertices<K, false>(c, sp, owner, start, tvBase, total, dst, um, uScale, uOffset))
  switch(kw)
  {
    case affine_kind(TC_TEXEL_F16, true): TC_CHUNK(affine_kind(TC_TEXEL_F16, true)); break;
    case affine_kind(TC_TEXEL_F32, true): TC_CHUNK(affine_kind(TC_TEXEL_F32, true)); break;
    case kAffineFlat:
      chunk_vertices<kAffineFlat, false>(c, sp, owner, start, tvBase, total, dst, um, uScale, uOffset);
      break;
    default: chunk_vertices<~0u, false>(c, sp, owner, start, tvBase, total, dst, um, uScale, uOffset); break;
  }
#undef TC_CHUNK
}

// cp.async: 4- and 8-byte global -> shared copies (the next chunk's part
// records and vertex offsets, fetched while the current chunk is generated)
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, int bytes)
{
  const u32 s = (u32)__cvta_generic_to_shared(smem);
  if(bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// A warp's staged part records: per lane its part's three 8-byte words and
// its first generated vertex (~0: not accepted / no part).
struct ChunkStage
{
  uint2 rec[3][32];
  u32   vo[32];
};

// MinBlocks: resident blocks per SM the register allocation is sized for
// (4: 64 registers, 5: 48, 6: 40); picked from the schedule's vertexBlocksPerSM.
template <int MinBlocks>
__global__ void __launch_bounds__(kBlock, MinBlocks) k_instantiate_vertices(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ PartAffine s_part[kWarps][kPartsPerWarp];
  __shared__ ChunkStage s_stage[kWarps];
  __shared__ u32        s_range[2];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32 begin = s_range[0], n = s_range[1] - s_range[0];

  const tc_SceneBuilding*    b         = c.build;
  const tc_TessTriangleInfo* parts     = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  float*                     gv        = reinterpret_cast<float*>(b->genVertices);
  const u32                  nwarps    = (gridDim.x * blockDim.x) >> 5;
  const u32                  numChunks = (n + kPartsPerWarp - 1) / kPartsPerWarp;
  PartAffine*                sp        = s_part[warp];
  ChunkStage&                stage     = s_stage[warp];

  // stage chunk `ck`'s records (each lane its own part; no other lane reads them)
  auto prefetch = [&](u32 ck) {
    const u32 q = ck * kPartsPerWarp + lane;
    if(ck < numChunks && q < n)
    {
      const uint2* raw = reinterpret_cast<const uint2*>(parts + begin + q);
      cp_async(&stage.rec[0][lane], raw, 8);
      cp_async(&stage.rec[1][lane], raw + 1, 8);
      cp_async(&stage.rec[2][lane], raw + 2, 8);
      cp_async(&stage.vo[lane], ib.vertexOffset + begin + q, 4);
    }
    else
      stage.vo[lane] = ~0u;
    cp_async_commit();
  };

  // chunks: the first nwarps one per warp, the rest handed out by a ticket
  // (parts differ in vertex count, so warps finish at different times); the
  // next chunk's ticket is taken, and its records staged, while the current
  // one is processed
  u32 chunk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  prefetch(chunk);
  while(chunk < numChunks)
  {
    u32 following = 0;
    if(lane == 0)
      following = nwarps + atomicAdd(c.scratch.ticket, 1u);
    cp_async_wait_all();
    const u32   vo       = stage.vo[lane];
    const bool  accepted = vo != ~0u;
    // accepted parts form a prefix of the part order: nothing further to do
    if(!__any_sync(0xFFFFFFFFu, accepted))
      break;
    u32     nv = 0, kind = 0, tvBase = 0;
    float   scale = 0.0f, offset = 0.0f;
    MapDesc map   = {};
    if(accepted)
      lane_part(c, stage.rec[0][lane], stage.rec[1][lane], stage.rec[2][lane], sp[lane], nv, kind, tvBase, scale,
                offset, map);
    const u32  next  = __shfl_sync(0xFFFFFFFFu, following, 0);
    prefetch(next);  // this lane's staged record is in registers now
    chunk_generate(c, sp, gv, vo, nv, kind, tvBase, map, scale, offset);
    __syncwarp();  // the warp's part records are rewritten by its next chunk
    chunk = next;
  }
  cp_async_wait_all();  // no copy in flight at exit
}

// Arguments and vertices in one launch (the stage entry point without PN or
// the ripple): a warp takes 32 consecutive parts (a chunk) at a time; its
// offsets are the tile's (tile scan) plus the chunk's prefix within the tile
// (the tile-sum pass left every chunk's packed sum) plus the lanes' warp
// prefix, so no per-part offset goes through memory. Each lane writes its
// part's 44 bytes of arguments (the capacity test and slots of
// k_instantiate_args), then sets up its affine record, and the warp writes the
// chunk's vertices. CLAS reference counts: a warp carries its last instance's
// count across chunks (one atomic per instance change); statistics once per
// block.
template <int MinBlocks>
__global__ void __launch_bounds__(kBlock, MinBlocks) k_instantiate_parts(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ PartAffine s_part[kWarps][kPartsPerWarp];
  __shared__ ChunkStage s_stage[kWarps];
  __shared__ u32        s_range[2], s_flag, s_stat[kWarps];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32 begin = s_range[0], n = s_range[1] - s_range[0];

  tc_SceneBuilding*          b         = c.build;
  const tc_TessTriangleInfo* parts     = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  float*                     gv        = reinterpret_cast<float*>(b->genVertices);
  tc_BlasBuildInfo*          blas      = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  const tc_caps&             k         = c.caps;
  const u64                  maxData   = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  const u32                  nwarps    = (gridDim.x * blockDim.x) >> 5;
  const u32                  numChunks = (n + kPartsPerWarp - 1) / kPartsPerWarp;
  const u32                  numTiles  = clamp_tiles(c, (n + kTile - 1) / kTile);
  const u32                  stride    = c.scratch.lbStride;
  const u64                  genBase   = c.scratch.totals[0];
  const u64                  tempBase  = c.scratch.totals[1];
  PartAffine*                sp        = s_part[warp];
  ChunkStage&                stage     = s_stage[warp];
  u32                        statTris = 0;
  u32                        carryKey = 0xFFFFFFFFu, carryCnt = 0;  // warp-uniform

  // stage chunk `ck`'s records; vo marks the lanes with a part (0) or none (~0)
  auto prefetch = [&](u32 ck) {
    const u32 q = ck * kPartsPerWarp + lane;
    if(ck < numChunks && q < n && (ck / kChunksPerTile) < numTiles)
    {
      const uint2* raw = reinterpret_cast<const uint2*>(parts + begin + q);
      cp_async(&stage.rec[0][lane], raw, 8);
      cp_async(&stage.rec[1][lane], raw + 1, 8);
      cp_async(&stage.rec[2][lane], raw + 2, 8);
      stage.vo[lane] = 0u;
    }
    else
      stage.vo[lane] = ~0u;
    cp_async_commit();
  };

  u32 chunk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  prefetch(chunk);
  while(chunk < numChunks)
  {
    u32 following = 0;
    if(lane == 0)
      following = nwarps + atomicAdd(c.scratch.ticket, 1u);
    cp_async_wait_all();
    const bool valid = stage.vo[lane] == 0u;
    if(!__any_sync(0xFFFFFFFFu, valid))
      break;
    const uint2 r0 = stage.rec[0][lane], r1 = stage.rec[1][lane], r2 = stage.rec[2][lane];
    const u32   cfg = r2.y >> 16;
    const u64   own = valid ? part_packed(c, cfg) : 0ull;

    // ---- offsets: tile + chunk within the tile + lane within the chunk ------
    const u32 tile = chunk / kChunksPerTile, w = chunk % kChunksPerTile;
    const u64 cs   = ib.chunkSums[tile * kChunksPerTile + lane];
    const u64 csi  = warp_inclusive<u64>(cs, lane);
    const u64 pre  = __shfl_sync(0xFFFFFFFFu, csi - cs, w);
    const u64 inc  = warp_inclusive<u64>(own, lane);
    const u64 within       = pre + inc - own;
    const u32 q            = chunk * kPartsPerWarp + lane;
    const u32 nvPart       = (u32)(own & kPackMask);
    const u32 ds           = (u32)(own >> kPackShift);
    const u64 genOffset    = genBase + q;
    const u64 dataOffset   = c.scratch.lbState[stride + tile] + (within >> kPackShift);
    const u64 vertexOffset = c.scratch.lbState[2 * stride + tile] + (within & kPackMask);
    // triangle_tess_template_instantiate.comp.glsl:160-167 capacity test
    const bool accept = valid && !(vertexOffset + nvPart > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
                                   || dataOffset + ds > maxData);
    if(accept)
    {
      // accepted instantiations form a prefix of the serial order: consecutive slots
      const u32                   tempOffset = (u32)(tempBase + q);
      tc_TemplateInstantiateInfo* dst  = reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations) + tempOffset;
      const u64                   tmpl = __ldg(c.table.templateAddresses + cfg_index(cfg));
      const u64                   vaddr = b->genVertices + vertexOffset * 12ull;
      const uint4 lo4 = make_uint4((begin + q) | (TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED << 30), 0u, (u32)tmpl, (u32)(tmpl >> 32));
      const uint4 hi4 = make_uint4((u32)vaddr, (u32)(vaddr >> 32), 12u, 0u);
      if((reinterpret_cast<uintptr_t>(dst) & 15) == 0)
      {
        reinterpret_cast<uint4*>(dst)[0] = lo4;
        reinterpret_cast<uint4*>(dst)[1] = hi4;
      }
      else
      {
        uint2* d2 = reinterpret_cast<uint2*>(dst);
        d2[0]     = make_uint2(lo4.x, lo4.y);
        d2[1]     = make_uint2(lo4.z, lo4.w);
        d2[2]     = make_uint2(hi4.x, hi4.y);
        d2[3]     = make_uint2(hi4.z, hi4.w);
      }
      reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]      = r0.x;
      reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset] = b->genClusterData + dataOffset;
      statTris += table_entry(c.table, cfg).numTriangles;
    }
    // CLAS reference counts per instance (the chunk's parts are instance-sorted):
    // groups of equal instance, the first continuing the warp's carried count
    {
      const u32 key     = accept ? r0.x : 0xFFFFFFFFu;
      const u32 grp     = __match_any_sync(0xFFFFFFFFu, key);
      const u32 leaders = __ballot_sync(0xFFFFFFFFu, accept && (u32)(__ffs(grp) - 1) == lane);
      if(leaders)
      {
        const int  fl = __ffs(leaders) - 1, ll = 31 - __clz(leaders);
        const u32  firstKey = __shfl_sync(0xFFFFFFFFu, key, fl), lastKey = __shfl_sync(0xFFFFFFFFu, key, ll);
        const u32  firstCnt = __popc(__shfl_sync(0xFFFFFFFFu, grp, fl));
        const u32  lastCnt  = __popc(__shfl_sync(0xFFFFFFFFu, grp, ll));
        if(((leaders >> lane) & 1u) && (int)lane != fl && (int)lane != ll)
          atomicAdd(&blas[key].clusterReferencesCount, (u32)__popc(grp));
        if(firstKey == carryKey)
          carryCnt += firstCnt;
        else
        {
          if(lane == 0 && carryCnt)
            atomicAdd(&blas[carryKey].clusterReferencesCount, carryCnt);
          carryKey = firstKey;
          carryCnt = firstCnt;
        }
        if(ll != fl)
        {
          if(lane == 0)
            atomicAdd(&blas[carryKey].clusterReferencesCount, carryCnt);
          carryKey = lastKey;
          carryCnt = lastCnt;
        }
      }
    }
    // accepted parts form a prefix: a chunk with none ends the warp's work
    if(!__any_sync(0xFFFFFFFFu, accept))
      break;

    // ---- vertices -----------------------------------------------------------
    u32     nv = 0, kind = 0, tvBase = 0;
    float   scale = 0.0f, offset = 0.0f;
    MapDesc map   = {};
    if(accept)
      lane_part(c, r0, r1, r2, sp[lane], nv, kind, tvBase, scale, offset, map);
    const u32 next = __shfl_sync(0xFFFFFFFFu, following, 0);
    prefetch(next);
    chunk_generate(c, sp, gv, (u32)vertexOffset, nv, kind, tvBase, map, scale, offset);
    __syncwarp();  // the warp's part records are rewritten by its next chunk
    chunk = next;
  }
  cp_async_wait_all();
  if(lane == 0 && carryCnt)
    atomicAdd(&blas[carryKey].clusterReferencesCount, carryCnt);

  // statistics: one atomic each per block
#pragma unroll
  for(int o = 16; o > 0; o >>= 1)
  {
    statTris += __shfl_xor_sync(0xFFFFFFFFu, statTris, o);
  }
  if(lane == 0)
  {
    s_stat[warp] = statTris;
  }
  __syncthreads();
  if(threadIdx.x == 0)
  {
    u32 t = 0;
    for(u32 wi = 0; wi < kWarps; wi++)
      t += s_stat[wi];
    if(t)
      atomicAdd(&c.readback->numTotalTriangles, t);
  }

  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0 && c.fuseSetup != kNoSetup)
      build_setup_apply(c, c.fuseSetup);
    if(c.fuseBlasSetup)
      blas_setup_block(c);
    if(threadIdx.x == 0 && c.scratch.selfClean)
      *c.scratch.done = 0;
  }
}

// triangle_tess_template_instantiate.comp.glsl:295-371 with TESS_USE_PN and /
// or DO_ANIMATION: eight lanes per part triangle over its vertices; the
// PN basis and the base attributes stay in registers. Written like the CPU
// restatement (tess_interpolate of the base barycentrics, the reference-order
// sampling and displacement) rather than in the affine form of the fast path.
__global__ void __launch_bounds__(kBlock) k_instantiate_vertices_deform(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ u32 s_range[2];
  const u32 lane = threadIdx.x & 31;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32                  begin = s_range[0], end = s_range[1];
  const tc_SceneBuilding*    b     = c.build;
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  float*                     gv    = reinterpret_cast<float*>(b->genVertices);
  const bool                 pn    = (c.flags & TC_FLAG_PN) != 0;
  const RippleParams         rp    = ripple_params(*c.view, (c.flags & TC_FLAG_RIPPLE) != 0);
  // eight lanes per part (parts average a handful of vertices), four parts per warp
  const u32                  subLane = lane & 7;
  const u32                  nsubs  = (gridDim.x * blockDim.x) >> 3;
  for(u32 p = begin + ((blockIdx.x * blockDim.x + threadIdx.x) >> 3); p < end; p += nsubs)
  {
    const u32 vo = ib.vertexOffset[p];
    if(vo == ~0u)
      break;  // accepted parts form a prefix of the part order
    const tc_TessTriangleInfo pt  = parts[p];
    const u32                 cfg = pt.subTriangle.triangleID_config >> 16;
    const u32                 tri = pt.subTriangle.triangleID_config & 0xFFFFu;
    const tc_TessTableEntry   e   = table_entry(c.table, cfg);
    const tc_RenderInstance&  in  = c.instances[pt.cluster.instanceID];
    const tc_Cluster          cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[pt.cluster.clusterID];
    const uint8_t*            lt  = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
    f3                        bp[3], bn[3], bb[3];
    f2                        bt[3];
    for(int v = 0; v < 3; v++)
    {
      const u32 vi = cl.firstLocalVertex + lt[tri * 3 + v];
      bp[v]        = ldg3(reinterpret_cast<const float*>(in.positions), vi);
      bn[v]        = normalize3(ldg3(reinterpret_cast<const float*>(in.normals), vi));  // :329
      bt[v]        = ldg2(reinterpret_cast<const float*>(in.texcoords), vi);
      bb[v]        = decode_bary(pt.subTriangle.vtxEncoded[v]);
    }
    tc_DisplacementTexture tx    = {};
    bool                   hasTx = false;
    if(c.numTextures > 0 && c.textures != nullptr && in.displacementIndex >= 0)
    {
      if((u32)in.displacementIndex < c.numTextures)
      {
        tx    = c.textures[in.displacementIndex];
        hasTx = true;
      }
      else if(subLane == 0)
        atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
    }
    BasePN basis = {};
    if(pn)
      basis = setup_pn(bp[0], bp[1], bp[2], bn[0], bn[1], bn[2]);
    for(u32 vert = subLane; vert < e.numVertices; vert += 8)
    {
      const f3 w   = interp3(bb[0], bb[1], bb[2], cfg_vertex(c.table, e, cfg, vert));
      f3       pos = pn ? get_pn(basis, w) : interp3(bp[0], bp[1], bp[2], w);
      if(hasTx)
        pos = displace(pos, interp3(bn[0], bn[1], bn[2], w), sample_bilinear(tx, interp2(bt[0], bt[1], bt[2], w)),
                       in.displacementScale, c.view->displacementScale, in.displacementOffset,
                       c.view->displacementOffset);
      if(rp.enabled)
        pos = ripple(pos, pt.cluster.instanceID, in.geoHi.w, rp);
      float* d = gv + 3 * ((u64)vo + vert);
      d[0] = pos.x, d[1] = pos.y, d[2] = pos.z;
    }
  }
}

}  // namespace

u32 instantiate_alloc_tiles(u32 maxParts) { return (maxParts + kTile - 1) / kTile; }

cudaError_t launch_instantiate_prefix(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                      u32 scanBlocksPerSM, cudaStream_t s)
{
  const u32         tiles    = std::max(1u, instantiate_alloc_tiles(maxParts));
  const u32         tileGrid = std::max(1u, std::min(tiles, numSMs * std::max(1u, scanBlocksPerSM)));
  const cudaError_t e        = launch_pdl_critical(k_instantiate_tile_sums, tileGrid, kBlock, s, c, buf);
  if(e != cudaSuccess)
    return e;
  return launch_pdl_critical(k_instantiate_tile_scan, 1u, kScanBlock, s, c);
}

cudaError_t launch_instantiate_args(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                    u32 scanBlocksPerSM, cudaStream_t s)
{
  const u32 tiles    = std::max(1u, instantiate_alloc_tiles(maxParts));
  const u32 tileGrid = std::max(1u, std::min(tiles, numSMs * std::max(1u, scanBlocksPerSM)));
  return launch_pdl_critical(k_instantiate_args, tileGrid, kBlock, s, c, buf);
}

cudaError_t launch_instantiate_alloc(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                     u32 scanBlocksPerSM, cudaStream_t s)
{
  const cudaError_t e = launch_instantiate_prefix(c, buf, maxParts, numSMs, scanBlocksPerSM, s);
  if(e != cudaSuccess)
    return e;
  return launch_instantiate_args(c, buf, maxParts, numSMs, scanBlocksPerSM, s);
}

cudaError_t launch_triangle_instantiate(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                        u32 scanBlocksPerSM, u32 vertexBlocksPerSM, u32 vertexGridPerSM,
                                        cudaStream_t s)
{
  const cudaError_t e = launch_instantiate_alloc(c, buf, maxParts, numSMs, scanBlocksPerSM, s);
  if(e != cudaSuccess)
    return e;
  return launch_instantiate_vertices(c, buf, maxParts, numSMs, vertexBlocksPerSM, vertexGridPerSM, s);
}

cudaError_t launch_instantiate_fused(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                     u32 scanBlocksPerSM, u32 vertexBlocksPerSM, u32 vertexGridPerSM, cudaStream_t s)
{
  if(c.flags & (TC_FLAG_PN | TC_FLAG_RIPPLE))  // the deformation path keeps its own vertex kernel
    return launch_triangle_instantiate(c, buf, maxParts, numSMs, scanBlocksPerSM, vertexBlocksPerSM, vertexGridPerSM, s);
  const u32   tiles    = std::max(1u, instantiate_alloc_tiles(maxParts));
  const u32   tileGrid = std::max(1u, std::min(tiles, numSMs * std::max(1u, scanBlocksPerSM)));
  cudaError_t e        = launch_pdl(k_instantiate_tile_sums, tileGrid, kBlock, s, c, buf);
  if(e != cudaSuccess)
    return e;
  if((e = launch_pdl(k_instantiate_tile_scan, 1u, kScanBlock, s, c)) != cudaSuccess)
    return e;
  const u32 chunks   = (maxParts + kPartsPerWarp - 1) / kPartsPerWarp;
  const u32 resident = vertexBlocksPerSM >= 6 ? 6u : (vertexBlocksPerSM == 5 ? 5u : 4u);
  const u32 perSM    = vertexGridPerSM ? vertexGridPerSM : resident;
  const u32 grid     = std::max(1u, std::min((chunks + kWarps - 1) / kWarps, numSMs * perSM));
  if(vertexBlocksPerSM >= 6)
    return launch_pdl(k_instantiate_parts<6>, grid, kBlock, s, c, buf);
  if(vertexBlocksPerSM == 5)
    return launch_pdl(k_instantiate_parts<5>, grid, kBlock, s, c, buf);
  return launch_pdl(k_instantiate_parts<4>, grid, kBlock, s, c, buf);
}

cudaError_t launch_instantiate_vertices(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                        u32 vertexBlocksPerSM, u32 vertexGridPerSM, cudaStream_t s)
{
  const u32 chunks = (maxParts + kPartsPerWarp - 1) / kPartsPerWarp;
  if(c.flags & (TC_FLAG_PN | TC_FLAG_RIPPLE))  // the deformation path: one warp per part
    return launch_pdl(k_instantiate_vertices_deform, std::max(1u, std::min((maxParts + 4 * kWarps - 1) / (4 * kWarps), numSMs * 8)),
                      kBlock, s, c, buf);
  // warps stride over the 32-part chunks; the grid is sized to the machine,
  // not to the capacity (blocks with no chunk would only add a tail), by
  // default one resident wave; vertexBlocksPerSM picks the register budget
  const u32 resident   = vertexBlocksPerSM >= 6 ? 6u : (vertexBlocksPerSM == 5 ? 5u : 4u);
  const u32 perSM      = vertexGridPerSM ? vertexGridPerSM : resident;
  const u32 vertexGrid = std::max(1u, std::min((chunks + kWarps - 1) / kWarps, numSMs * perSM));
  if(vertexBlocksPerSM >= 6)
    return launch_pdl(k_instantiate_vertices<6>, vertexGrid, kBlock, s, c, buf);
  if(vertexBlocksPerSM == 5)
    return launch_pdl(k_instantiate_vertices<5>, vertexGrid, kBlock, s, c, buf);
  return launch_pdl(k_instantiate_vertices<4>, vertexGrid, kBlock, s, c, buf);
}

}  // namespace tc
