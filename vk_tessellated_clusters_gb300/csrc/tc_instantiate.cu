// tc_instantiate.cu — triangle_tess_template_instantiate: template
// instantiation arguments and displaced vertices for every part triangle.
//
// shaders/triangle_tess_template_instantiate.comp.glsl:126-373.
//
// GB300 mapping, two launches:
//   alloc    : a scan over the part triangles (1024 per tile, decoupled
//              look-back between tiles) assigns generated-cluster slots, CLAS
//              bytes and vertex ranges in part order, applies the capacity test
//              and writes the 44 B of instantiation arguments per part; the
//              first vertex of each accepted part goes to scratch
//   vertices : HBM-write bound (12 B per generated vertex dominates). One warp
//              per 16 consecutive parts, whose vertices form one contiguous
//              range: each part's affine vertex form (tc_vertex.cuh, 128 B) is
//              set up once in shared memory, then the lanes walk the range
//              on consecutive vertices. No block barriers, no cross-block
//              waits.
#include <algorithm>

#include "tc_kernels.h"
#include "tc_stage.cuh"
#include "tc_vertex.cuh"

namespace tc {

namespace {

enum : int
{
  kCntGen = 0,
  kCntData,
  kCntVerts,
  kNumCounters
};

constexpr u32 kAllocBlock   = 256;
constexpr u32 kAllocItems   = 4;
constexpr u32 kAllocTile    = kAllocBlock * kAllocItems;
constexpr u32 kVertexWarps  = 8;  // warps per block of the vertex kernel
constexpr u32 kPartsPerWarp = 16;  // parts staged per warp and chunk (shared memory budget)

static_assert(kAllocTile == kInstantiateTile, "allocation tile size");

// parts of this launch: [0, part counter) or one run, narrowed to the instance window
__device__ inline void part_range(const StageCtx& c, u32& lo, u32& hi)
{
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(c.build->partTriangles);
  lo                               = 0;
  hi                               = min(c.build->partTriangleCounter, c.caps.maxPartTriangles);
  if(c.run != kAllRuns)
  {
    const u32 rs = c.runStarts[c.run], re = c.runStarts[c.run + 1];
    lo           = min(rs, hi);
    hi           = min(max(re, rs), hi);
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

// ---------------------------------------------------------------------------
// alloc
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kAllocBlock) k_instantiate_alloc(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ u64 s_warp[33][kNumCounters];
  __shared__ u64 s_excl[kNumCounters];
  __shared__ u32 s_tile, s_flag, s_range[2];
  __shared__ u32 s_blasKey[kAllocBlock / 32][2], s_blasCnt[kAllocBlock / 32][2], s_stat[kAllocBlock / 32][2];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32 begin    = s_range[0], n = s_range[1] - s_range[0];
  const u32 numTiles = clamp_tiles(c, (n + kAllocTile - 1) / kAllocTile);

  tc_SceneBuilding*          b        = c.build;
  const tc_caps&             k        = c.caps;
  const tc_TessTriangleInfo* parts    = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  const u64                  maxData  = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  tc_BlasBuildInfo*          blas     = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  u32                        statTris = 0, statTemp = 0;

  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;
    const u32 first = tile * kAllocTile + threadIdx.x * kAllocItems;
    u32       inst[kAllocItems], cfg[kAllocItems], nv[kAllocItems], nt[kAllocItems], ds[kAllocItems];
    u64       sum[kNumCounters] = {0, 0, 0};
#pragma unroll
    for(u32 i = 0; i < kAllocItems; i++)
    {
      inst[i] = ~0u;
      cfg[i] = nv[i] = nt[i] = ds[i] = 0;
      if(first + i < n)
      {
        const uint2* raw          = reinterpret_cast<const uint2*>(parts + begin + first + i);
        inst[i]                   = raw[0].x;
        cfg[i]                    = raw[2].y >> 16;
        const tc_TessTableEntry e = table_entry(c.table, cfg[i]);
        nv[i]                     = e.numVertices;
        nt[i]                     = e.numTriangles;
        ds[i]                     = __ldg(c.table.templateSizes + cfg_index(cfg[i]));
        sum[kCntGen] += 1;
        sum[kCntData] += ds[i];
        sum[kCntVerts] += nv[i];
      }
    }
    // block exclusive scan of the three counters
    u64 inc[kNumCounters];
#pragma unroll
    for(int q = 0; q < kNumCounters; q++)
    {
      inc[q] = warp_inclusive<u64>(sum[q], lane);
      if(lane == 31)
        s_warp[warp][q] = inc[q];
    }
    __syncthreads();
    if(warp == 0)
    {
#pragma unroll
      for(int q = 0; q < kNumCounters; q++)
      {
        u64 w = lane < nw ? s_warp[lane][q] : 0;
        u64 s = warp_inclusive<u64>(w, lane);
        __syncwarp();
        if(lane < nw)
          s_warp[lane][q] = s - w;
        if(lane == 31)
          s_warp[32][q] = s;
      }
    }
    __syncthreads();
    // look-back: warps 0..2, one counter each
    if(warp < kNumCounters)
    {
      const u32 q    = warp;
      u64       base = 0;
      if(tile == 0)
        base = q == kCntGen ? b->genClusterCounter : (q == kCntData ? b->genClusterDataCounter : b->genVertexCounter);
      const u64 agg = s_warp[32][q];
      const u64 ex = warp_lookback_exclusive(c.scratch.lbState + (u64)q * c.scratch.lbStride, tile, agg, base, c.errorWord);
      if(lane == 0)
      {
        s_excl[q] = ex;
        if(tile == numTiles - 1)
          c.scratch.totals[q] = ex + agg;
      }
    }
    __syncthreads();
    u64 genOffset    = s_excl[kCntGen] + s_warp[warp][kCntGen] + inc[kCntGen] - sum[kCntGen];
    u64 dataOffset   = s_excl[kCntData] + s_warp[warp][kCntData] + inc[kCntData] - sum[kCntData];
    u64 vertexOffset = s_excl[kCntVerts] + s_warp[warp][kCntVerts] + inc[kCntVerts] - sum[kCntVerts];
    u32 runInst = ~0u, runCount = 0;
#pragma unroll
    for(u32 i = 0; i < kAllocItems; i++)
    {
      if(first + i < n)
      {
        const u32 p = begin + first + i;
        // triangle_tess_template_instantiate.comp.glsl:160-167 capacity test
        const bool accept = !(vertexOffset + nv[i] > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
                              || dataOffset + ds[i] > maxData);
        if(accept)
        {
          // accepted instantiations form a prefix of the serial order: slot == generated cluster index
          const u32 tempOffset = (u32)genOffset;
          tc_TemplateInstantiateInfo* dst =
              reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations) + tempOffset;
          const u64   tmpl  = __ldg(c.table.templateAddresses + cfg_index(cfg[i]));
          const u64   vaddr = b->genVertices + vertexOffset * 12ull;
          const uint4 lo4 = make_uint4(p | (TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED << 30), 0u, (u32)tmpl, (u32)(tmpl >> 32));
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
          reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]      = inst[i];
          reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset] = b->genClusterData + dataOffset;
          ib.vertexOffset[p]                                          = (u32)vertexOffset;
          statTris += nt[i];
          statTemp += 1;
          if(inst[i] != runInst)
          {
            if(runCount)
              atomicAdd(&blas[runInst].clusterReferencesCount, runCount);
            runInst  = inst[i];
            runCount = 0;
          }
          runCount++;
        }
        else
          ib.vertexOffset[p] = ~0u;
      }
      genOffset += 1;
      dataOffset += ds[i];
      vertexOffset += nv[i];
    }
    // Per-instance CLAS reference counts. Parts are instance-sorted within a
    // run, so an instance's parts in this tile are (almost always) contiguous:
    // threads of a warp holding the same instance combine their last runs;
    // the warp's first and last instances go to shared memory and are merged
    // across the block's warps, every other instance is added directly. One
    // atomic per instance and tile instead of one per warp.
    {
      const u32  key     = runCount ? runInst : 0xFFFFFFFFu;
      const u32  peers   = __match_any_sync(0xFFFFFFFFu, key);
      u32        peerSum = 0;
      for(u32 m = peers; m; m &= m - 1)
        peerSum += __shfl_sync(peers, runCount, __ffs(m) - 1);
      const bool leader  = runCount && (__ffs(peers) - 1) == (int)lane;
      const u32  holders = __ballot_sync(0xFFFFFFFFu, runCount != 0);
      const u32  firstKey = holders ? __shfl_sync(0xFFFFFFFFu, key, __ffs(holders) - 1) : 0xFFFFFFFFu;
      const u32  lastKey  = holders ? __shfl_sync(0xFFFFFFFFu, key, 31 - __clz(holders)) : 0xFFFFFFFFu;
      if(lane == 0)
      {
        s_blasKey[warp][0] = firstKey;
        s_blasKey[warp][1] = lastKey;
        s_blasCnt[warp][0] = 0;
        s_blasCnt[warp][1] = 0;
      }
      __syncwarp();
      if(leader)
      {
        if(key == firstKey)
          s_blasCnt[warp][0] = peerSum;
        else if(key == lastKey)
          s_blasCnt[warp][1] = peerSum;
        else
          atomicAdd(&blas[runInst].clusterReferencesCount, peerSum);
      }
    }
    __syncthreads();
    if(threadIdx.x == 0)
    {
      u32 curKey = 0xFFFFFFFFu, curCnt = 0;
      for(u32 w = 0; w < nw; w++)
        for(u32 e = 0; e < 2; e++)
        {
          const u32 k = s_blasKey[w][e], n = s_blasCnt[w][e];
          if(n == 0)
            continue;
          if(k != curKey)
          {
            if(curCnt)
              atomicAdd(&blas[curKey].clusterReferencesCount, curCnt);
            curKey = k;
            curCnt = 0;
          }
          curCnt += n;
        }
      if(curCnt)
        atomicAdd(&blas[curKey].clusterReferencesCount, curCnt);
    }
    __syncthreads();
  }

  // statistics: one atomic each per block
  for(int o = 16; o > 0; o >>= 1)
  {
    statTris += __shfl_xor_sync(0xFFFFFFFFu, statTris, o);
    statTemp += __shfl_xor_sync(0xFFFFFFFFu, statTemp, o);
  }
  if(lane == 0)
  {
    s_stat[warp][0] = statTris;
    s_stat[warp][1] = statTemp;
  }
  __syncthreads();
  if(threadIdx.x == 0)
  {
    u32 t = 0, q = 0;
    for(u32 w = 0; w < nw; w++)
      t += s_stat[w][0], q += s_stat[w][1];
    if(t)
      atomicAdd(&c.readback->numTotalTriangles, t);
    if(q)
      atomicAdd(&b->tempInstantiateCounter, q);
  }

  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0)
    {
      if(numTiles)
      {
        b->genClusterCounter     = (u32)c.scratch.totals[kCntGen];
        b->genClusterDataCounter = c.scratch.totals[kCntData];
        b->genVertexCounter      = (u32)c.scratch.totals[kCntVerts];
      }
      if(c.fuseSetup != kNoSetup)
        build_setup_apply(c, c.fuseSetup);
    }
    scratch_release(c, numTiles, kNumCounters);
  }
}

// ---------------------------------------------------------------------------
// vertices
// ---------------------------------------------------------------------------

// MinBlocks: resident blocks per SM the register allocation is sized for
// (4: 64 registers, 5: 48, 6: 40); picked from the schedule's vertexBlocksPerSM.
template <int MinBlocks>
__global__ void __launch_bounds__(kVertexWarps * 32, MinBlocks) k_instantiate_vertices(StageCtx c, InstantiateBuffers ib)
{
  stage_prologue();
  __shared__ PartAffine s_part[kVertexWarps][kPartsPerWarp];
  __shared__ u32        s_range[2];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    part_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32 begin = s_range[0], n = s_range[1] - s_range[0];

  const tc_SceneBuilding*    b            = c.build;
  const tc_TessTriangleInfo* parts        = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  const bool                 haveTextures = c.numTextures > 0 && c.textures != nullptr;
  float*                     gv           = reinterpret_cast<float*>(b->genVertices);
  const float                viewScale    = c.view->displacementScale;
  const float                viewOffset   = c.view->displacementOffset;
  const u32                  nwarps       = (gridDim.x * blockDim.x) >> 5;
  const u32                  numChunks    = (n + kPartsPerWarp - 1) / kPartsPerWarp;
  PartAffine*                sp           = s_part[warp];

  for(u32 chunk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; chunk < numChunks; chunk += nwarps)
  {
    const u32  p        = begin + chunk * kPartsPerWarp + lane;
    const u32  vo       = (lane < kPartsPerWarp && p < begin + n) ? ib.vertexOffset[p] : ~0u;
    const bool accepted = vo != ~0u;
    // accepted parts form a prefix of the part order: nothing further to do
    if(!__any_sync(0xFFFFFFFFu, accepted))
      break;
    u32 nv = 0;
    if(accepted)
    {
      const uint2*             raw = reinterpret_cast<const uint2*>(parts + p);
      const uint2              r0 = raw[0], r1 = raw[1], r2 = raw[2];
      const u32                cfg = r2.y >> 16;
      const u32                tri = r2.y & 0xFFFFu;
      const tc_TessTableEntry  e   = table_entry(c.table, cfg);
      const tc_RenderInstance& in  = c.instances[r0.x];
      const tc_Cluster         cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[r0.y];
      const uint8_t*           lt  = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      const float*             pos = reinterpret_cast<const float*>(in.positions);
      const float*             nrm = reinterpret_cast<const float*>(in.normals);
      const float*             uvs = reinterpret_cast<const float*>(in.texcoords);
      const u32                corner[3] = {r1.x, r1.y, r2.x};
      f3                       bp[3], bn[3];
      f2                       bt[3];
#pragma unroll
      for(int v = 0; v < 3; v++)
      {
        const u32 vi = cl.firstLocalVertex + lt[tri * 3 + v];
        bp[v]        = ldg3(pos, vi);
        bn[v]        = normalize3(ldg3(nrm, vi));  // :329
        bt[v]        = ldg2(uvs, vi);
      }
      tc_DisplacementTexture tx = {};
      if(haveTextures && in.displacementIndex >= 0)
      {
        if((u32)in.displacementIndex < c.numTextures)
          tx = c.textures[in.displacementIndex];
        else
          atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
      }
      write_part_affine(sp[lane], corner, cfg_flipped(cfg), bp, bn, bt, e.firstVertex, tx,
                        in.displacementScale * viewScale, in.displacementOffset + viewOffset);
      nv       = e.numVertices;
    }
    const u32 inc   = warp_inclusive<u32>(nv, lane);
    const u32 start = inc - nv;  // first vertex of this lane's part within the chunk
    const u32 total = __shfl_sync(0xFFFFFFFFu, inc, kPartsPerWarp - 1);
    const u64 v0    = __shfl_sync(0xFFFFFFFFu, vo, 0);
    __syncwarp();
    if(total == 0)
      continue;

    // Lanes take consecutive vertices (lanes of one step share one to three
    // part records: broadcast reads); each vertex is three 4-byte stores. A
    // lane's part: the parts starting at or before the step's first vertex,
    // plus those starting inside the step up to the lane (one bit each).
    const bool owner = lane < kPartsPerWarp && nv > 0;
    for(u32 base = 0; base < total; base += 32)
    {
      const u32 before = __popc(__ballot_sync(0xFFFFFFFFu, owner && start <= base));
      const u32 inside = __reduce_or_sync(0xFFFFFFFFu, (owner && start > base && start < base + 32) ? 1u << (start - base) : 0u);
      const u32 pi     = before - 1 + __popc(inside & ((2u << lane) - 2u));
      const u32 pstart = __shfl_sync(0xFFFFFFFFu, start, pi & 31);
      const u32 jj     = base + lane;
      const PartAffine& r = sp[pi];
      // the step's records usually share one kind: then a branch-free specialisation
      const u32 kind  = affine_kind_of(r);
      const u32 kind0 = __shfl_sync(0xFFFFFFFFu, kind, 0);
      const u32 kw    = __all_sync(0xFFFFFFFFu, kind == kind0) ? kind0 : ~0u;
      if(jj < total)
      {
        const u32 tv = __ldg(c.table.vertices + affine_first_vertex(r) + (jj - pstart));
        f3        q;
        switch(kw)
        {
          case affine_kind(TC_TEXEL_F16, true): q = affine_vertex_k<affine_kind(TC_TEXEL_F16, true)>(r, tv); break;
          case affine_kind(TC_TEXEL_F32, true): q = affine_vertex_k<affine_kind(TC_TEXEL_F32, true)>(r, tv); break;
          case kAffineFlat: q = affine_vertex_k<kAffineFlat>(r, tv); break;
          default: q = affine_vertex_k<~0u>(r, tv); break;
        }
        float* d = gv + 3 * (v0 + jj);
        d[0] = q.x, d[1] = q.y, d[2] = q.z;
      }
    }
    __syncwarp();  // the warp's part records are rewritten by its next chunk
  }
}

}  // namespace

u32 instantiate_alloc_tiles(u32 maxParts) { return (maxParts + kAllocTile - 1) / kAllocTile; }

cudaError_t launch_triangle_instantiate(const StageCtx& c, const InstantiateBuffers& buf, u32 maxParts, u32 numSMs,
                                        u32 allocBlocksPerSM, u32 vertexBlocksPerSM, cudaStream_t s)
{
  const u32 allocGrid = std::max(1u, std::min(instantiate_alloc_tiles(maxParts), numSMs * std::max(1u, allocBlocksPerSM)));
  cudaError_t e = launch_pdl(k_instantiate_alloc, allocGrid, kAllocBlock, s, c, buf);
  if(e != cudaSuccess)
    return e;
  const u32 chunks     = (maxParts + kPartsPerWarp - 1) / kPartsPerWarp;
  const u32 vertexGrid = std::max(1u, std::min((chunks + kVertexWarps - 1) / kVertexWarps,
                                               numSMs * std::max(1u, vertexBlocksPerSM)));
  if(vertexBlocksPerSM >= 6)
    return launch_pdl(k_instantiate_vertices<6>, vertexGrid, kVertexWarps * 32, s, c, buf);
  if(vertexBlocksPerSM == 5)
    return launch_pdl(k_instantiate_vertices<5>, vertexGrid, kVertexWarps * 32, s, c, buf);
  return launch_pdl(k_instantiate_vertices<4>, vertexGrid, kVertexWarps * 32, s, c, buf);
}

}  // namespace tc
