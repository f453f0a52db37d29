// tc_instantiate.cu — triangle_tess_template_instantiate: template
// instantiation arguments and displaced vertices for every part triangle.
//
// shaders/triangle_tess_template_instantiate.comp.glsl:126-373.
//
// GB300 mapping (HBM-write bound: 12 B per generated vertex dominates):
//  * a tile is 32 part triangles; warp 0 reads them, computes the counts
//    (generated clusters, CLAS bytes, vertices), orders them after all earlier
//    tiles with a decoupled look-back and writes the 44 B of instantiation
//    arguments per part;
//  * per-part base data (positions, normalised normals, uvs, decoded
//    barycentrics, table offsets) is staged once in shared memory;
//  * all threads then generate the tile's vertices (flat index -> part by
//    binary search), stage them in shared memory and write the tile's
//    contiguous vertex range with aligned 16-byte stores (scalar stores only at
//    the two unaligned ends).
#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

namespace {

enum : int
{
  kCntGen = 0,
  kCntData,
  kCntVerts,
  kNumCounters
};

constexpr int kPartsPerTile = 32;
constexpr int kMaxTileVerts = kPartsPerTile * 78;  // 78 = largest config vertex count of an 11-segment table

struct PartRecord
{
  f3  p[3];
  f3  n[3];
  f2  uv[3];
  f3  bb[3];
  u32 firstVertex;
  u32 cfg;
  u32 texIndex;  // ~0 = no displacement
  float scale, offset;
};

template <int B>
__global__ void __launch_bounds__(B) k_triangle_instantiate(StageCtx c)
{
  __shared__ PartRecord s_part[kPartsPerTile];
  __shared__ u32        s_vpre[kPartsPerTile + 1];  // vertex prefix within tile (accepted parts only)
  __shared__ __align__(16) float s_stage[kMaxTileVerts * 3 + 4];
  __shared__ u64 s_excl[kNumCounters];
  __shared__ u64 s_agg[kNumCounters];
  __shared__ u64 s_vbase;
  __shared__ u32 s_tile, s_flag, s_range[2];

  const u32         lane = threadIdx.x & 31;
  const u32         warp = threadIdx.x >> 5;
  tc_SceneBuilding* b    = c.build;
  const tc_caps&    k    = c.caps;
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);

  if(threadIdx.x == 0)
  {
    u32 lo = 0, hi = min(b->partTriangleCounter, c.caps.maxPartTriangles);
    if(c.run != kAllRuns)
    {
      u32 rs = c.runStarts[c.run], re = c.runStarts[c.run + 1];
      lo     = min(rs, hi);
      hi     = min(max(re, rs), hi);
    }
    if(!whole_window(c))
    {
      auto get = [&](u32 i) { return parts[i].cluster.instanceID; };
      u32  e   = lower_bound_instance(lo, hi, c.instEnd, get);
      lo       = lower_bound_instance(lo, e, c.instBegin, get);
      hi       = e;
    }
    s_range[0] = lo;
    s_range[1] = hi;
  }
  __syncthreads();
  const u32 begin = s_range[0], end = s_range[1];
  u32 numTiles = (end - begin + kPartsPerTile - 1) / kPartsPerTile;
  numTiles = clamp_tiles(c, numTiles);

  const bool haveTextures = c.numTextures > 0 && c.textures != nullptr;
  const u64  maxData      = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  const float viewScale   = c.view->displacementScale;
  const float viewOffset  = c.view->displacementOffset;
  float*      gv          = reinterpret_cast<float*>(b->genVertices);
  const bool  aligned16   = (reinterpret_cast<uintptr_t>(gv) & 15) == 0;

  u32 statTris = 0, statTemp = 0;

  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;

    // ---- warp 0: read the tile's parts, per-part counts and their scans -----------
    const u32           p     = begin + tile * kPartsPerTile + lane;
    const bool          valid = warp == 0 && p < end;
    tc_TessTriangleInfo info  = {};
    u32                 cfg = 0, nv = 0, nt = 0;
    u64                 ds = 0;
    u32                 xv = 0;
    u64                 xd = 0;
    if(warp == 0)
    {
      if(valid)
      {
        const uint2* raw                   = reinterpret_cast<const uint2*>(parts + p);
        uint2        r0 = raw[0], r1 = raw[1], r2 = raw[2];
        info.cluster                       = {r0.x, r0.y};
        info.subTriangle.vtxEncoded[0]     = r1.x;
        info.subTriangle.vtxEncoded[1]     = r1.y;
        info.subTriangle.vtxEncoded[2]     = r2.x;
        info.subTriangle.triangleID_config = r2.y;
        cfg                                = r2.y >> 16;
        const tc_TessTableEntry e          = table_entry(c.table, cfg);
        nv                                 = e.numVertices;
        nt                                 = e.numTriangles;
        ds                                 = __ldg(c.table.templateSizes + cfg_index(cfg));
      }
      // warp scans (inclusive) of vertices (u32) and CLAS bytes (u64)
      xv = nv;
      xd = ds;
#pragma unroll
      for(int d = 1; d < 32; d <<= 1)
      {
        u32 yv = __shfl_up_sync(0xFFFFFFFFu, xv, d);
        u64 yd = __shfl_up_sync(0xFFFFFFFFu, xd, d);
        if(lane >= (u32)d)
        {
          xv += yv;
          xd += yd;
        }
      }
      if(lane == 31)
      {
        s_agg[kCntGen]   = min((u32)kPartsPerTile, end - (begin + tile * kPartsPerTile));
        s_agg[kCntData]  = xd;
        s_agg[kCntVerts] = xv;
      }
    }
    __syncthreads();

    // ---- look-back: warps 0..2, one counter each ------------------------------------
    if(warp < kNumCounters)
    {
      u64 base = 0;
      if(tile == 0)
        base = warp == kCntGen ? b->genClusterCounter : (warp == kCntData ? b->genClusterDataCounter : b->genVertexCounter);
      const u64 ex = warp_lookback_exclusive(c.scratch.lbState + (u64)warp * c.scratch.lbStride, tile, s_agg[warp], base,
                                             c.errorWord);
      if(lane == 0)
      {
        s_excl[warp] = ex;
        if(tile == numTiles - 1)
          c.scratch.totals[warp] = ex + s_agg[warp];
      }
    }
    __syncthreads();

    // ---- warp 0: acceptance, instantiation arguments, per-part staging ---------------
    if(warp == 0)
    {
      const u64 genOffset    = s_excl[kCntGen] + lane;
      const u64 dataOffset   = s_excl[kCntData] + (xd - ds);
      const u64 vertexOffset = s_excl[kCntVerts] + (xv - nv);
      // triangle_tess_template_instantiate.comp.glsl:160-167 capacity test
      const bool accept = valid
                          && !(vertexOffset + nv > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
                               || dataOffset + ds > maxData);
      const u32 acceptMask = __ballot_sync(0xFFFFFFFFu, accept);
      if(accept)
      {
        // accepted instantiations form a prefix of the serial order: slot == generated cluster index
        const u32 tempOffset = (u32)genOffset;
        tc_TemplateInstantiateInfo* dst = reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations) + tempOffset;
        const u64 tmpl  = __ldg(c.table.templateAddresses + cfg_index(cfg));
        const u64 vaddr = b->genVertices + vertexOffset * 12ull;
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
        reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]      = info.cluster.instanceID;
        reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset] = b->genClusterData + dataOffset;
        statTris += nt;
      }
      if(lane == 0)
        statTemp += __popc(acceptMask);
      // per-instance CLAS reference counts: one atomic per distinct instance in the warp
      {
        const u32 inst  = accept ? info.cluster.instanceID : 0xFFFFFFFFu;
        const u32 peers = __match_any_sync(0xFFFFFFFFu, inst);
        if(accept && (__ffs(peers) - 1) == (int)lane)
          atomicAdd(&reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos)[inst].clusterReferencesCount, (u32)__popc(peers));
      }
      // staging of per-part vertex-generation inputs
      const u32 nvAcc = accept ? nv : 0u;
      u32       xa    = nvAcc;
#pragma unroll
      for(int d = 1; d < 32; d <<= 1)
      {
        u32 y = __shfl_up_sync(0xFFFFFFFFu, xa, d);
        if(lane >= (u32)d)
          xa += y;
      }
      if(lane == 0)
      {
        s_vpre[0] = 0;
        s_vbase   = s_excl[kCntVerts];
      }
      s_vpre[lane + 1] = xa;
      if(accept)
      {
        const tc_RenderInstance& in  = c.instances[info.cluster.instanceID];
        const tc_Cluster         cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[info.cluster.clusterID];
        const uint8_t*           lt  = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
        const u32                tri = info.subTriangle.triangleID_config & 0xFFFFu;
        const float*             pos = reinterpret_cast<const float*>(in.positions);
        const float*             nrm = reinterpret_cast<const float*>(in.normals);
        const float*             uvs = reinterpret_cast<const float*>(in.texcoords);
        PartRecord&              r   = s_part[lane];
#pragma unroll
        for(int v = 0; v < 3; v++)
        {
          const u32 vi = cl.firstLocalVertex + lt[tri * 3 + v];
          r.bb[v]      = decode_bary(info.subTriangle.vtxEncoded[v]);
          r.p[v]       = ldg3(pos, vi);
          r.n[v]       = normalize3(ldg3(nrm, vi));  // :329
          r.uv[v]      = ldg2(uvs, vi);
        }
        r.firstVertex = table_entry(c.table, cfg).firstVertex;
        r.cfg         = cfg;
        r.texIndex    = ~0u;
        if(haveTextures && in.displacementIndex >= 0)
        {
          if((u32)in.displacementIndex < c.numTextures)
            r.texIndex = (u32)in.displacementIndex;
          else
            atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
        }
        r.scale  = in.displacementScale;
        r.offset = in.displacementOffset;
      }
    }
    __syncthreads();

    // ---- all threads: vertex generation into shared staging -----------------------
    const u32 tileVerts = s_vpre[kPartsPerTile];
    const u64 vbase     = s_vbase;
    const u32 shift     = aligned16 ? (u32)((vbase * 3) & 3) : 0u;
    for(u32 j = threadIdx.x; j < tileVerts; j += B)
    {
      u32 lo = 0, hi = kPartsPerTile;  // last part with s_vpre[part] <= j
      while(hi - lo > 1)
      {
        u32 mid = (lo + hi) >> 1;
        if(s_vpre[mid] <= j)
          lo = mid;
        else
          hi = mid;
      }
      const PartRecord& r    = s_part[lo];
      const u32         vert = j - s_vpre[lo];
      // triangle_tess_template_instantiate.comp.glsl:343-371
      f3 w = decode_bary(__ldg(c.table.vertices + r.firstVertex + vert));
      if(cfg_flipped(r.cfg))
      {
        float s = w.x;
        w.x     = w.y;
        w.y     = s;
      }
      w        = interp3(r.bb[0], r.bb[1], r.bb[2], w);
      f3 p     = interp3(r.p[0], r.p[1], r.p[2], w);
      if(r.texIndex != ~0u)
      {
        const f3 n  = interp3(r.n[0], r.n[1], r.n[2], w);
        const f2 uv = interp2(r.uv[0], r.uv[1], r.uv[2], w);
        const float h = sample_bilinear(c.textures[r.texIndex], uv);
        p = displace(p, n, h, r.scale, viewScale, r.offset, viewOffset);
      }
      if(aligned16)
      {
        float* d = s_stage + shift + 3 * j;
        d[0]     = p.x;
        d[1]     = p.y;
        d[2]     = p.z;
      }
      else
      {
        float* d = gv + (vbase + j) * 3;
        d[0]     = p.x;
        d[1]     = p.y;
        d[2]     = p.z;
      }
    }
    __syncthreads();

    // ---- write-out: the tile's vertices are one contiguous range ----------------------
    if(aligned16 && tileVerts)
    {
      const u32 nf     = tileVerts * 3;
      const u64 g0     = vbase * 3 - shift;  // float index of the 16-B aligned start
      const u32 groups = (shift + nf + 3) / 4;
      float4*   dst4   = reinterpret_cast<float4*>(gv + g0);
      const float4* src4 = reinterpret_cast<const float4*>(s_stage);
      for(u32 g = threadIdx.x; g < groups; g += B)
      {
        const u32 lo = g * 4, hi = lo + 4;
        if(lo >= shift && hi <= shift + nf)
          dst4[g] = src4[g];
        else
          for(u32 q = max(lo, shift); q < min(hi, shift + nf); q++)
            gv[g0 + q] = s_stage[q];
      }
    }
    __syncthreads();
  }

  for(int o = 16; o > 0; o >>= 1)
  {
    statTris += __shfl_xor_sync(0xFFFFFFFFu, statTris, o);
    statTemp += __shfl_xor_sync(0xFFFFFFFFu, statTemp, o);
  }
  if(lane == 0)
  {
    if(statTris)
      atomicAdd(&c.readback->numTotalTriangles, statTris);
    if(statTemp)
      atomicAdd(&b->tempInstantiateCounter, statTemp);
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

}  // namespace

cudaError_t launch_triangle_instantiate(const StageCtx& c, u32 blockSize, u32 grid, cudaStream_t s)
{
  switch(blockSize)
  {
    case 128:
      k_triangle_instantiate<128><<<grid, 128, 0, s>>>(c);
      break;
    case 512:
      k_triangle_instantiate<512><<<grid, 512, 0, s>>>(c);
      break;
    default:
      k_triangle_instantiate<256><<<grid, 256, 0, s>>>(c);
      break;
  }
  return cudaGetLastError();
}

}  // namespace tc
