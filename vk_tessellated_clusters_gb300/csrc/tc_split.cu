// tc_split.cu — one pass of the recursive triangle split.
//
// shaders/triangle_split.comp.glsl:146-331 (processSubTask) and 598-632
// (main_multipass): every split item of the current level spawns the
// triangles of its tessellation config as children; each child's barycentrics
// are composed with the parent's, re-encoded, its segment counts re-evaluated
// on the interpolated world positions, and it is appended either to the split
// queue (next level) or to the part triangles.
//
// GB300 mapping: a tile is T parent items; their children are laid out flat
// across the block (block scan of child counts, binary search child -> parent,
// the same packing the reference does per subgroup, triangle_split.comp.glsl:350-472).
// Pass 1 classifies every child and counts; a decoupled look-back orders the
// tile's appends after all earlier tiles; pass 2 recomputes the children (pure
// ALU on L1-resident table and parent data) and writes them in (parent, child)
// order. Persistent grid, tiles from a ticket.
#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

namespace {

enum : int
{
  kCntSplit = 0,
  kCntPart,
  kNumCounters
};

constexpr u32 kMaxChildrenPerItem = TC_TESSTABLE_SIZE * TC_TESSTABLE_SIZE;  // 121

struct SplitItem
{
  tc_ClusterInfo ci;
  u32            vtx[3];
  u32            tc;
  f3             bp[3];  // world positions of the base triangle
  u32            firstTriangle;
  u32            firstVertex;
};

struct Child
{
  u32  vtx[3];
  u32  tc;
  bool split;
};

__device__ __forceinline__ Child make_child(const Table& table, const SplitItem& it, u32 sub, const FactorParams& fp, u32 sf)
{
  const u32 cfg = it.tc >> 16;
  // tessellation.glsl:165-176 triangle of the pattern, flip-aware
  u32   p  = __ldg(table.triangles + it.firstTriangle + sub);
  uint3 tv = make_uint3(p & 0xFF, (p >> 8) & 0xFF, (p >> 16) & 0xFF);
  if(cfg_flipped(cfg))
  {
    u32 s = tv.y;
    tv.y  = tv.z;
    tv.z  = s;
  }
  const f3 bb0 = decode_bary(it.vtx[0]);
  const f3 bb1 = decode_bary(it.vtx[1]);
  const f3 bb2 = decode_bary(it.vtx[2]);
  Child    ch;
  const u32 tvs[3] = {tv.x, tv.y, tv.z};
#pragma unroll
  for(int v = 0; v < 3; v++)
  {
    f3 w = decode_bary(__ldg(table.vertices + it.firstVertex + tvs[v]));
    if(cfg_flipped(cfg))
    {
      float s = w.x;
      w.x     = w.y;
      w.y     = s;
    }
    ch.vtx[v] = encode_bary(interp3(bb0, bb1, bb2, w));  // triangle_split.comp.glsl:236-243
  }
  const f3 w0 = interp3(it.bp[0], it.bp[1], it.bp[2], decode_bary(ch.vtx[0]));
  const f3 w1 = interp3(it.bp[0], it.bp[1], it.bp[2], decode_bary(ch.vtx[1]));
  const f3 w2 = interp3(it.bp[0], it.bp[1], it.bp[2], decode_bary(ch.vtx[2]));
  uint3    f  = tess_factors(w0, w1, w2, fp);
  u32      m  = max(max(f.x, f.y), f.z);
  ch.split    = m > TC_TESSTABLE_SIZE;
  if(ch.split)
    f = make_uint3(split_factor1(f.x, sf), split_factor1(f.y, sf), split_factor1(f.z, sf));
  const u32 ncfg = get_config(f, ch.vtx[0], ch.vtx[1], ch.vtx[2]);
  ch.tc          = (it.tc & 0xFFFFu) | (ncfg << 16);
  return ch;
}

template <int T, int B>
__global__ void __launch_bounds__(B) k_triangle_split(StageCtx c)
{
  stage_prologue();
  static_assert(T <= B && T <= 32, "tile items are set up by warp 0");
  constexpr u32 kMaxChildren = T * kMaxChildrenPerItem;
  constexpr u32 kMaxChunks   = (kMaxChildren + B - 1) / B;

  __shared__ SplitItem s_item[T];
  __shared__ u32       s_pre[T + 1];
  __shared__ u32       s_chunkCnt[kMaxChunks][kNumCounters];  // exclusive per chunk after the scan
  __shared__ u32       s_warpCnt[B / 32][kNumCounters];
  __shared__ u64       s_excl[kNumCounters];
  __shared__ u32       s_tile, s_flag, s_range[2];

  const u32         lane = threadIdx.x & 31;
  const u32         warp = threadIdx.x >> 5;
  tc_SceneBuilding* b    = c.build;
  const tc_caps&    k    = c.caps;
  tc_TessTriangleInfo* queue = reinterpret_cast<tc_TessTriangleInfo*>(b->splitTriangles);

  if(threadIdx.x == 0)
  {
    u32 hi = min(b->splitPassEnd, c.caps.maxSplitTriangles);
    u32 lo = min(b->splitPassStart, hi);
    if(!whole_window(c))
    {
      auto get = [&](u32 i) { return queue[i].cluster.instanceID; };
      u32  e   = lower_bound_instance(lo, hi, c.instEnd, get);
      lo       = lower_bound_instance(lo, e, c.instBegin, get);
      hi       = e;
    }
    s_range[0] = lo;
    s_range[1] = hi;
  }
  __syncthreads();
  const u32 begin = s_range[0], end = s_range[1];
  u32 numTiles = (end - begin + T - 1) / T;
  numTiles = clamp_tiles(c, numTiles);

  FactorParams fp;
  fp.viewPos   = {b->viewPos.x, b->viewPos.y, b->viewPos.z};
  fp.nearPlane = c.view->nearPlane;
  fp.viewportH = c.view->viewportf.y;
  fp.tessRate  = c.view->tessRate;
  const u32 sf = clamp_split_factor(k.splitFactor);

  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;

    // ---- tile setup: parents (warp 0) --------------------------------------
    if(warp == 0)
    {
      const u32 item  = begin + tile * T + lane;
      const bool valid = lane < T && item < end;
      u32        n     = 0;
      if(valid)
      {
        // triangle_split.comp.glsl:146-180 fillBaseVertices
        const uint2* raw = reinterpret_cast<const uint2*>(queue + item);
        uint2        r0 = raw[0], r1 = raw[1], r2 = raw[2];
        SplitItem    it;
        it.ci     = {r0.x, r0.y};
        it.vtx[0] = r1.x;
        it.vtx[1] = r1.y;
        it.vtx[2] = r2.x;
        it.tc     = r2.y;
        const tc_TessTableEntry  e  = table_entry(c.table, it.tc >> 16);
        const tc_RenderInstance& in = c.instances[it.ci.instanceID];
        const tc_Cluster         cl = reinterpret_cast<const tc_Cluster*>(in.clusters)[it.ci.clusterID];
        const uint8_t*           lt = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
        const u32                tri = it.tc & 0xFFFFu;
        const float*             pos = reinterpret_cast<const float*>(in.positions);
        float                    m[16];
#pragma unroll
        for(int j = 0; j < 16; j++)
          m[j] = __ldg(in.worldMatrix.m + j);
#pragma unroll
        for(int v = 0; v < 3; v++)
          it.bp[v] = xform_point(m, ldg3(pos, cl.firstLocalVertex + lt[tri * 3 + v]));
        it.firstTriangle = e.firstTriangle;
        it.firstVertex   = e.firstVertex;
        n                = min((u32)e.numTriangles, kMaxChildrenPerItem);
        s_item[lane]     = it;
      }
      // warp inclusive scan of child counts
      u32 x = n;
#pragma unroll
      for(int d = 1; d < 32; d <<= 1)
      {
        u32 y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if(lane >= (u32)d)
          x += y;
      }
      if(lane < T)
        s_pre[lane + 1] = x;
      if(lane == 0)
        s_pre[0] = 0;
    }
    __syncthreads();
    const u32 numChildren = s_pre[T];
    const u32 numChunks   = (numChildren + B - 1) / B;

    // ---- pass 1: classify children, count per chunk -------------------------
    for(u32 ch = 0; ch < numChunks; ch++)
    {
      const u32 j     = ch * B + threadIdx.x;
      const bool valid = j < numChildren;
      bool       split = false, part = false;
      if(valid)
      {
        u32 lo = 0, hi = T;  // last item with s_pre[item] <= j
        while(hi - lo > 1)
        {
          u32 mid = (lo + hi) >> 1;
          if(s_pre[mid] <= j)
            lo = mid;
          else
            hi = mid;
        }
        const Child child = make_child(c.table, s_item[lo], j - s_pre[lo], fp, sf);
        split             = child.split;
        part              = !child.split;
      }
      const u32 bs = __ballot_sync(0xFFFFFFFFu, split), bp = __ballot_sync(0xFFFFFFFFu, part);
      if(lane == 0)
      {
        s_warpCnt[warp][kCntSplit] = __popc(bs);
        s_warpCnt[warp][kCntPart]  = __popc(bp);
      }
      __syncthreads();
      if(threadIdx.x < kNumCounters)
      {
        u32 s = 0;
        for(u32 w = 0; w < B / 32; w++)
          s += s_warpCnt[w][threadIdx.x];
        s_chunkCnt[ch][threadIdx.x] = s;
      }
      __syncthreads();
    }

    // ---- tile totals, look-back ------------------------------------------------
    if(warp < kNumCounters)
    {
      const u32 q   = warp;
      u32       agg = 0;
      for(u32 ch = 0; ch < numChunks; ch++)
        agg += s_chunkCnt[ch][q];
      u64 base = 0;
      if(tile == 0)
        base = q == kCntSplit ? b->splitWriteCounter : b->partTriangleCounter;
      const u64 ex = warp_lookback_exclusive(c.scratch.lbState + (u64)q * c.scratch.lbStride, tile, agg, base, c.errorWord);
      if(lane == 0)
      {
        u32 run = 0;
        for(u32 ch = 0; ch < numChunks; ch++)
        {
          u32 v              = s_chunkCnt[ch][q];
          s_chunkCnt[ch][q]  = run;  // exclusive within tile
          run += v;
        }
        s_excl[q] = ex;
        if(tile == numTiles - 1)
          c.scratch.totals[q] = ex + agg;
      }
    }
    __syncthreads();

    // ---- pass 2: recompute and write ---------------------------------------------
    for(u32 ch = 0; ch < numChunks; ch++)
    {
      const u32 j     = ch * B + threadIdx.x;
      const bool valid = j < numChildren;
      Child      child;
      u32        item = 0;
      child.split     = false;
      if(valid)
      {
        u32 lo = 0, hi = T;
        while(hi - lo > 1)
        {
          u32 mid = (lo + hi) >> 1;
          if(s_pre[mid] <= j)
            lo = mid;
          else
            hi = mid;
        }
        item  = lo;
        child = make_child(c.table, s_item[lo], j - s_pre[lo], fp, sf);
      }
      const bool split = valid && child.split, part = valid && !child.split;
      const u32  bs = __ballot_sync(0xFFFFFFFFu, split), bp = __ballot_sync(0xFFFFFFFFu, part);
      if(lane == 0)
      {
        s_warpCnt[warp][kCntSplit] = __popc(bs);
        s_warpCnt[warp][kCntPart]  = __popc(bp);
      }
      __syncthreads();
      u32 wsplit = 0, wpart = 0;
      for(u32 w = 0; w < warp; w++)
      {
        wsplit += s_warpCnt[w][kCntSplit];
        wpart += s_warpCnt[w][kCntPart];
      }
      const u32 ltm = (1u << lane) - 1u;
      if(split)
      {
        const u64 o = s_excl[kCntSplit] + s_chunkCnt[ch][kCntSplit] + wsplit + __popc(bs & ltm);
        if(o < k.maxSplitTriangles)
        {
          uint2* dst = reinterpret_cast<uint2*>(queue + o);
          dst[0]     = make_uint2(s_item[item].ci.instanceID, s_item[item].ci.clusterID);
          dst[1]     = make_uint2(child.vtx[0], child.vtx[1]);
          dst[2]     = make_uint2(child.vtx[2], child.tc);
        }
      }
      else if(part)
      {
        const u64 o = s_excl[kCntPart] + s_chunkCnt[ch][kCntPart] + wpart + __popc(bp & ltm);
        if(o < k.maxPartTriangles)
        {
          uint2* dst = reinterpret_cast<uint2*>(reinterpret_cast<tc_TessTriangleInfo*>(b->partTriangles) + o);
          dst[0]     = make_uint2(s_item[item].ci.instanceID, s_item[item].ci.clusterID);
          dst[1]     = make_uint2(child.vtx[0], child.vtx[1]);
          dst[2]     = make_uint2(child.vtx[2], child.tc);
        }
      }
      __syncthreads();
    }
  }

  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0)
    {
      if(numTiles)
      {
        b->splitWriteCounter   = (u32)c.scratch.totals[kCntSplit];
        b->partTriangleCounter = (u32)c.scratch.totals[kCntPart];
      }
      if(c.fuseSetup != kNoSetup)
        build_setup_apply(c, c.fuseSetup);
    }
    scratch_release(c, numTiles, kNumCounters);
  }
}

}  // namespace

cudaError_t launch_triangle_split(const StageCtx& c, u32 blockSize, u32 grid, cudaStream_t s)
{
  switch(blockSize)
  {
    case 128:
      return launch_pdl(k_triangle_split<16, 128>, grid, 128, s, c);
    case 512:
      return launch_pdl(k_triangle_split<32, 512>, grid, 512, s, c);
    default:
      return launch_pdl(k_triangle_split<32, 256>, grid, 256, s, c);
  }
}

}  // namespace tc
