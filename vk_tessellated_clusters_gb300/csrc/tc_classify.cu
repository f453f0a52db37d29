// tc_classify.cu — cluster_classify: per-triangle edge segment counts and the
// full / part / split classification of every visible cluster.
//
// shaders/cluster_classify.comp.glsl:150-666 (RT target, plain path).
//
// GB300 mapping: one warp per cluster (<= 64 triangles: two per lane), W
// clusters per block, the cluster's vertices staged in shared memory. Appends
// (part triangles, split triangles, full-cluster instantiations, generated
// vertices, CLAS bytes) are ordered by a block scan plus a decoupled look-back
// across tiles, so every offset equals the one a serial loop over the visible
// clusters would produce. Persistent grid: blocks pull tiles from a ticket.
#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

namespace {

enum : int
{
  kCntParts = 0,
  kCntSplits,
  kCntGen,
  kCntData,
  kCntVerts,
  kNumCounters
};

__device__ __forceinline__ void store_tess_info(tc_TessTriangleInfo* dst, const tc_ClusterInfo& ci, u32 v0, u32 v1, u32 v2,
                                                u32 tc)
{
  uint2* p = reinterpret_cast<uint2*>(dst);
  p[0]     = make_uint2(ci.instanceID, ci.clusterID);
  p[1]     = make_uint2(v0, v1);
  p[2]     = make_uint2(v2, tc);
}

template <int W>
__global__ void __launch_bounds__(W * 32) k_cluster_classify(StageCtx c)
{
  __shared__ f3  s_vert[W][TC_MAX_CLUSTER_VERTICES];
  __shared__ u32 s_cnt[W][kNumCounters];
  __shared__ u64 s_data[W];
  __shared__ u32 s_fullInst[W];  // instance of an accepted full cluster, ~0 otherwise
  __shared__ u64 s_excl[kNumCounters];
  __shared__ u32 s_tile, s_flag, s_range[2];

  const u32         lane = threadIdx.x & 31;
  const u32         warp = threadIdx.x >> 5;
  tc_SceneBuilding* b    = c.build;
  const tc_caps&    k    = c.caps;

  // visible clusters of the instance window (visibleClusters is sorted by instance)
  const tc_ClusterInfo* vis = reinterpret_cast<const tc_ClusterInfo*>(b->visibleClusters);
  if(threadIdx.x == 0)
  {
    u32 lo = 0, hi = min(b->visibleClusterCounter, c.caps.maxVisibleClusters);
    if(!whole_window(c))
    {
      auto get = [&](u32 i) { return vis[i].instanceID; };
      u32  e   = lower_bound_instance(lo, hi, c.instEnd, get);
      lo       = lower_bound_instance(lo, e, c.instBegin, get);
      hi       = e;
    }
    s_range[0] = lo;
    s_range[1] = hi;
  }
  __syncthreads();
  const u32 begin = s_range[0], end = s_range[1];
  u32 numTiles = (end - begin + W - 1) / W;
  numTiles = clamp_tiles(c, numTiles);

  FactorParams fp;
  fp.viewPos   = {b->viewPos.x, b->viewPos.y, b->viewPos.z};
  fp.nearPlane = c.view->nearPlane;
  fp.viewportH = c.view->viewportf.y;
  fp.tessRate  = c.view->tessRate;

  const bool culling      = (c.flags & TC_FLAG_CULLING) != 0;
  const bool haveTextures = c.numTextures > 0 && c.textures != nullptr;
  const u64  maxData      = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  const u32  sf           = clamp_split_factor(k.splitFactor);

  u32 statFull = 0, statTotalTris = 0, statTemp = 0;

  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;

    const u32  v     = begin + tile * W + warp;
    const bool valid = v < end;

    tc_ClusterInfo           ci = {0, 0};
    const tc_RenderInstance* in = nullptr;
    tc_Cluster               cl = {};
    uint3                    f0 = {1, 1, 1}, f1 = {1, 1, 1};
    u32                      m0 = 0, m1 = 0;
    u32                      nt = 0, nv = 0, simple = 0;
    bool                     isFull = false;
    if(valid)
    {
      ci = vis[v];
      in = c.instances + ci.instanceID;
      cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[ci.clusterID];
      nt = cl.numTriangles;
      nv = cl.numVertices;
      if(nt > TC_MAX_CLUSTER_TRIANGLES || nv > TC_MAX_CLUSTER_VERTICES)
      {
        if(lane == 0)
          atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
        nt = min(nt, TC_MAX_CLUSTER_TRIANGLES);
        nv = min(nv, TC_MAX_CLUSTER_VERTICES);
      }
      const float* pos = reinterpret_cast<const float*>(in->positions);
      // cluster_classify.comp.glsl:180-198: stage object-space vertices
      for(u32 i = lane; i < nv; i += 32)
        s_vert[warp][i] = ldg3(pos, cl.firstLocalVertex + i);
      __syncwarp();

      const bool culled = culling && (reinterpret_cast<const u32*>(b->instanceStates)[ci.instanceID] & TC_INSTANCE_VISIBLE_BIT) == 0;
      if(culled)
      {
        // cluster_classify.comp.glsl:203-211: invisible instance, no tessellation
        simple = nt;
      }
      else
      {
        // cluster_classify.comp.glsl:217-246
        const uint8_t* lt = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
        const float*   wm = in->worldMatrix.m;
        float          m[16];
#pragma unroll
        for(int j = 0; j < 16; j++)
          m[j] = __ldg(wm + j);
        // vertex indices are masked to the staged range (a malformed index reads
        // a wrong vertex of the same cluster, never outside shared memory)
        if(lane < nt)
        {
          f0 = tess_factors(xform_point(m, s_vert[warp][lt[lane * 3 + 0] & 63u]),
                            xform_point(m, s_vert[warp][lt[lane * 3 + 1] & 63u]),
                            xform_point(m, s_vert[warp][lt[lane * 3 + 2] & 63u]), fp);
          m0 = max(max(f0.x, f0.y), f0.z);
        }
        if(lane + 32 < nt)
        {
          const u32 t = lane + 32;
          f1 = tess_factors(xform_point(m, s_vert[warp][lt[t * 3 + 0] & 63u]), xform_point(m, s_vert[warp][lt[t * 3 + 1] & 63u]),
                            xform_point(m, s_vert[warp][lt[t * 3 + 2] & 63u]), fp);
          m1 = max(max(f1.x, f1.y), f1.z);
        }
        simple = __popc(__ballot_sync(0xFFFFFFFFu, lane < nt && m0 == 1))
                 + __popc(__ballot_sync(0xFFFFFFFFu, lane + 32 < nt && m1 == 1));
      }
      isFull = simple == nt;
    }

    // per-cluster counts
    if(lane == 0)
    {
      s_data[warp] = (valid && isFull) ? __ldg(reinterpret_cast<const u32*>(in->clusterTemplateInstantiatonSizes) + ci.clusterID) : 0u;
      s_cnt[warp][kCntGen]    = (valid && isFull) ? 1u : 0u;
      s_cnt[warp][kCntVerts]  = (valid && isFull) ? nv : 0u;
      s_cnt[warp][kCntParts]  = 0;
      s_cnt[warp][kCntSplits] = 0;
    }
    if(valid && !isFull)
    {
      u32 p = __popc(__ballot_sync(0xFFFFFFFFu, lane < nt && m0 <= TC_TESSTABLE_SIZE))
              + __popc(__ballot_sync(0xFFFFFFFFu, lane + 32 < nt && m1 <= TC_TESSTABLE_SIZE));
      if(lane == 0)
      {
        s_cnt[warp][kCntParts]  = p;
        s_cnt[warp][kCntSplits] = nt - p;
      }
    }
    __syncthreads();

    // tile aggregates and look-back (one warp per counter)
    for(u32 q = warp; q < kNumCounters; q += W)
    {
      u64 agg = 0;
#pragma unroll
      for(int w = 0; w < W; w++)
        agg += q == kCntData ? s_data[w] : (u64)s_cnt[w][q];
      u64 base = 0;
      if(tile == 0)
      {
        switch(q)
        {
          case kCntParts:
            base = b->partTriangleCounter;
            break;
          case kCntSplits:
            base = (u64)(u32)b->splitTriangleCounter;
            break;
          case kCntGen:
            base = b->genClusterCounter;
            break;
          case kCntData:
            base = b->genClusterDataCounter;
            break;
          default:
            base = b->genVertexCounter;
            break;
        }
      }
      const u64 ex = warp_lookback_exclusive(c.scratch.lbState + (u64)q * c.scratch.lbStride, tile, agg, base, c.errorWord);
      if(lane == 0)
      {
        s_excl[q] = ex;
        if(tile == numTiles - 1)
          c.scratch.totals[q] = ex + agg;
      }
    }
    __syncthreads();

    if(valid)
    {
      // this warp's exclusive offsets
      u64 off[kNumCounters];
#pragma unroll
      for(int q = 0; q < kNumCounters; q++)
        off[q] = s_excl[q];
      for(u32 w = 0; w < warp; w++)
      {
        off[kCntParts] += s_cnt[w][kCntParts];
        off[kCntSplits] += s_cnt[w][kCntSplits];
        off[kCntGen] += s_cnt[w][kCntGen];
        off[kCntData] += s_data[w];
        off[kCntVerts] += s_cnt[w][kCntVerts];
      }

      if(isFull)
      {
        // cluster_classify.comp.glsl:271-488: template instantiation of the full cluster
        const u64 genOffset    = off[kCntGen];
        const u64 dataOffset   = off[kCntData];
        const u64 dataSize     = s_data[warp];
        const u64 vertexOffset = off[kCntVerts];
        const bool accept      = !(vertexOffset + nv > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
                                   || dataOffset + dataSize > maxData);
        if(lane == 0)
        {
          statFull += 1;
          s_fullInst[warp] = accept ? ci.instanceID : ~0u;
        }
        if(accept)
        {
          if(lane == 0)
          {
            // accepted instantiations form a prefix of the serial order, so
            // the instantiation slot equals the generated-cluster slot
            const u32                  tempOffset = (u32)genOffset;
            tc_TemplateInstantiateInfo ti;
            ti.clusterIdOffset        = 0;
            ti.geometryIndexOffset    = 0;
            ti.clusterTemplateAddress = __ldg(reinterpret_cast<const u64*>(in->clusterTemplateAdresses) + ci.clusterID);
            ti.vertexBufferAddress    = b->genVertices + vertexOffset * 12ull;
            ti.vertexBufferStride     = 12;
            reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations)[tempOffset] = ti;
            reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]                          = ci.instanceID;
            reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset]                     = b->genClusterData + dataOffset;
            if((c.flags & TC_FLAG_WRITE_FULLCLUSTERS) && b->fullClusters)
              reinterpret_cast<tc_ClusterInfo*>(b->fullClusters)[tempOffset] = ci;
            statTemp += 1;
            statTotalTris += simple;
          }
          // cluster_classify.comp.glsl:457-482: displaced cluster vertices
          float*                        gv = reinterpret_cast<float*>(b->genVertices);
          const tc_DisplacementTexture* tx = nullptr;
          if(haveTextures && in->displacementIndex >= 0)
          {
            if((u32)in->displacementIndex < c.numTextures)
              tx = c.textures + in->displacementIndex;
            else if(lane == 0)
              atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
          }
          const float* nrm = reinterpret_cast<const float*>(in->normals);
          const float* uvs = reinterpret_cast<const float*>(in->texcoords);
          for(u32 i = lane; i < nv; i += 32)
          {
            f3 p = s_vert[warp][i];
            if(tx)
            {
              const u32 vi = cl.firstLocalVertex + i;
              float     h  = sample_bilinear(*tx, ldg2(uvs, vi));
              p = displace(p, ldg3(nrm, vi), h, in->displacementScale, c.view->displacementScale, in->displacementOffset,
                           c.view->displacementOffset);
            }
            float* dst = gv + (vertexOffset + i) * 3;
            dst[0]     = p.x;
            dst[1]     = p.y;
            dst[2]     = p.z;
          }
        }
      }
      else
      {
        // cluster_classify.comp.glsl:543-666: part and split triangles
        const bool split0 = lane < nt && m0 > TC_TESSTABLE_SIZE;
        const bool part0  = lane < nt && m0 <= TC_TESSTABLE_SIZE;
        const bool split1 = lane + 32 < nt && m1 > TC_TESSTABLE_SIZE;
        const bool part1  = lane + 32 < nt && m1 <= TC_TESSTABLE_SIZE;
        const u32  bs0 = __ballot_sync(0xFFFFFFFFu, split0), bp0 = __ballot_sync(0xFFFFFFFFu, part0);
        const u32  bs1 = __ballot_sync(0xFFFFFFFFu, split1), bp1 = __ballot_sync(0xFFFFFFFFu, part1);
        const u32  lt_mask = (1u << lane) - 1u;
        tc_TessTriangleInfo* splits = reinterpret_cast<tc_TessTriangleInfo*>(b->splitTriangles);
        tc_TessTriangleInfo* parts  = reinterpret_cast<tc_TessTriangleInfo*>(b->partTriangles);
#pragma unroll
        for(int h = 0; h < 2; h++)
        {
          const bool isSplit = h == 0 ? split0 : split1;
          const bool isPart  = h == 0 ? part0 : part1;
          if(!isSplit && !isPart)
            continue;
          const u32 tri = lane + 32 * h;
          uint3     f   = h == 0 ? f0 : f1;
          u32       v0 = 0, v1 = TC_TESSTABLE_COORD_MAX, v2 = TC_TESSTABLE_COORD_MAX << 16;
          if(isSplit)
          {
            const u64 o = off[kCntSplits] + (h == 0 ? __popc(bs0 & lt_mask) : __popc(bs0) + __popc(bs1 & lt_mask));
            if(o < k.maxSplitTriangles)
            {
              f           = make_uint3(split_factor1(f.x, sf), split_factor1(f.y, sf), split_factor1(f.z, sf));
              const u32 cfg = get_config(f, v0, v1, v2);
              store_tess_info(splits + o, ci, v0, v1, v2, tri | (cfg << 16));
            }
          }
          else
          {
            const u64 o = off[kCntParts] + (h == 0 ? __popc(bp0 & lt_mask) : __popc(bp0) + __popc(bp1 & lt_mask));
            if(o < k.maxPartTriangles)
            {
              const u32 cfg = get_config(f, v0, v1, v2);
              store_tess_info(parts + o, ci, v0, v1, v2, tri | (cfg << 16));
            }
          }
        }
        if(lane == 0)
          s_fullInst[warp] = ~0u;
      }
    }
    else if(lane == 0)
    {
      s_fullInst[warp] = ~0u;
    }
    __syncthreads();
    // per-instance CLAS reference counts, one atomic per run of equal instances
    if(threadIdx.x == 0)
    {
      u32 runInst = ~0u, runCount = 0;
      for(int w = 0; w < W; w++)
      {
        u32 i = s_fullInst[w];
        if(i == ~0u)
          continue;
        if(i != runInst)
        {
          if(runCount)
            atomicAdd(&reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos)[runInst].clusterReferencesCount, runCount);
          runInst  = i;
          runCount = 0;
        }
        runCount++;
      }
      if(runCount)
        atomicAdd(&reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos)[runInst].clusterReferencesCount, runCount);
    }
  }

  // block-level statistics: one atomic each
  for(int o = 16; o > 0; o >>= 1)
  {
    statFull += __shfl_xor_sync(0xFFFFFFFFu, statFull, o);
    statTemp += __shfl_xor_sync(0xFFFFFFFFu, statTemp, o);
    statTotalTris += __shfl_xor_sync(0xFFFFFFFFu, statTotalTris, o);
  }
  if(lane == 0)
  {
    if(statFull)
      atomicAdd(&c.readback->numFullClusters, statFull);
    if(statTemp)
      atomicAdd(&b->tempInstantiateCounter, statTemp);
    if(statTotalTris)
      atomicAdd(&c.readback->numTotalTriangles, statTotalTris);
  }

  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0)
    {
      if(numTiles)
      {
        b->partTriangleCounter   = (u32)c.scratch.totals[kCntParts];
        b->splitTriangleCounter  = (int32_t)(u32)c.scratch.totals[kCntSplits];
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

}  // namespace

u32 classify_num_counters() { return kNumCounters; }

cudaError_t launch_cluster_classify(const StageCtx& c, u32 warpsPerBlock, u32 grid, cudaStream_t s)
{
  switch(warpsPerBlock)
  {
    case 2:
      k_cluster_classify<2><<<grid, 64, 0, s>>>(c);
      break;
    case 4:
      k_cluster_classify<4><<<grid, 128, 0, s>>>(c);
      break;
    case 16:
      k_cluster_classify<16><<<grid, 512, 0, s>>>(c);
      break;
    default:
      k_cluster_classify<8><<<grid, 256, 0, s>>>(c);
      break;
  }
  return cudaGetLastError();
}

}  // namespace tc
