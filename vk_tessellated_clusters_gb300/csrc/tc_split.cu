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
// Pass 1 classifies every child, keeps it in shared memory and counts per
// (chunk, warp); one warp turns the counts into offsets and a decoupled
// look-back orders the tile's appends after all earlier tiles; pass 2 writes
// the children in (parent, child) order (recomputing them only when a tile
// has more than 64 children per item, i.e. split factors above 8), with no
// block barrier inside either pass. Split items carry their base
// triangle's world positions in a side array, so a tile's set-up is one load
// level instead of the instance / cluster / index / vertex chain. Persistent
// grid, tiles from a ticket.
//
// Two kernels share the tile body (split_tile):
//   k_triangle_split        one pass per launch (the reference's
//                           main_multipass dispatch; per-stage and
//                           per-instance entry points);
//   k_triangle_split_levels every pass in one launch (the batched frame and
//                           its graph): the persistent blocks take tiles of
//                           all levels from one ticket, level by level; the
//                           block that completes a level's last tile applies
//                           that pass's build_setup (what the multipass
//                           kernel's last block does) and publishes the next
//                           level's item range, for which the blocks holding
//                           later tickets wait (bounded). An empty first
//                           level leaves every level empty: one block then
//                           runs the passes' set-ups and the others return.
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

// the part counter a split pass continues from: the front of the two-sided
// counter with transient builds
__device__ __forceinline__ u32 part_base(const StageCtx& c)
{
  return (c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)) ? (u32)__ldcg(&c.build->dualPartTriangleCounter)
                                                                    : __ldcg(&c.build->partTriangleCounter);
}
__device__ __forceinline__ u32 part_cap(const StageCtx& c)
{
  const u32 m = c.caps.maxPartTriangles;
  if(!(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)))
    return m;
  const u32 y = (u32)(c.build->dualPartTriangleCounter >> 32);
  return (u64)y + 1 < m ? m - y - 1 : 0u;
}

// Shared memory of one split tile (kernel-scope; one per block).
template <int T, int B>
struct SplitShared
{
  static constexpr u32 kMaxChildren   = T * kMaxChildrenPerItem;
  static constexpr u32 kMaxChunks     = (kMaxChildren + B - 1) / B;
  static constexpr u32 kW             = B / 32;
  static constexpr u32 kSlots         = kMaxChunks * kW;  // (chunk, warp) count slots, in serial order
  static constexpr u32 kCacheChildren = T * 64;  // pass 1 keeps its children for pass 2 when they fit
  static_assert(T <= B && T <= 32, "tile items are set up by warp 0");
  static_assert(kSlots <= 128, "one warp scans the count slots, four per lane");

  uint4     child[kCacheChildren];      // vtx[3], tc
  u32       splitMask[kSlots];          // per (chunk, warp): which lanes' children are split items
  SplitItem item[T];
  u32       pre[T + 1];
  u32       cnt[kNumCounters][kSlots];  // per (chunk, warp): count, then exclusive offset within the tile
  u64       excl[kNumCounters];
  u32       tile, flag, range[2];
};

// One tile: T items of the level [begin, end) starting at begin + tile * T,
// their children classified, ordered after every earlier tile of the level
// (look-back on `lbState` rows of `lbStride`, tile 0 from the counters'
// current values) and written. The last tile publishes the level's totals.
template <int T, int B>
__device__ void split_tile(const StageCtx& c, SplitShared<T, B>& sm, u32 tile, u32 begin, u32 end, u32 numTiles,
                           u64* lbState, u32 lbStride, u64* totals, const FactorParams& fp, u32 sf, u32 partCap)
{
  using S                  = SplitShared<T, B>;
  constexpr u32 kW         = S::kW;
  const u32     lane       = threadIdx.x & 31;
  const u32     warp       = threadIdx.x >> 5;
  const u32     ltm        = (1u << lane) - 1u;
  tc_SceneBuilding*    b     = c.build;
  const tc_caps&       k     = c.caps;
  tc_TessTriangleInfo* queue = reinterpret_cast<tc_TessTriangleInfo*>(b->splitTriangles);

  // parent of child j: last item with pre[item] <= j
  auto parent_of = [&](u32 j) {
    u32 lo = 0, hi = T;
    while(hi - lo > 1)
    {
      const u32 mid = (lo + hi) >> 1;
      if(sm.pre[mid] <= j)
        lo = mid;
      else
        hi = mid;
    }
    return lo;
  };

  // ---- tile setup: parents (warp 0) --------------------------------------
  if(warp == 0)
  {
    const u32  item  = begin + tile * T + lane;
    const bool valid = lane < T && item < end;
    u32        n     = 0;
    if(valid)
    {
      // triangle_split.comp.glsl:146-180 fillBaseVertices; the base
      // triangle's world positions travel with the item (splitBase)
      // through L2: with every pass in one launch, other blocks wrote these items
      const uint2* raw = reinterpret_cast<const uint2*>(queue + item);
      uint2        r0 = __ldcg(raw), r1 = __ldcg(raw + 1), r2 = __ldcg(raw + 2);
      SplitItem    it;
      it.ci     = {r0.x, r0.y};
      it.vtx[0] = r1.x;
      it.vtx[1] = r1.y;
      it.vtx[2] = r2.x;
      it.tc     = r2.y;
      const tc_TessTableEntry e = table_entry(c.table, it.tc >> 16);
      if(c.splitBase)
      {
        const float* sb = c.splitBase + 9 * (u64)item;
#pragma unroll
        for(int v = 0; v < 3; v++)
          it.bp[v] = {__ldcg(sb + 3 * v), __ldcg(sb + 3 * v + 1), __ldcg(sb + 3 * v + 2)};
      }
      else
      {
        const tc_RenderInstance& in  = c.instances[it.ci.instanceID];
        const tc_Cluster         cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[it.ci.clusterID];
        const uint8_t*           lt  = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
        const u32                tri = it.tc & 0xFFFFu;
        const float*             pos = reinterpret_cast<const float*>(in.positions);
        float                    m[16];
#pragma unroll
        for(int j = 0; j < 16; j++)
          m[j] = __ldg(in.worldMatrix.m + j);
#pragma unroll
        for(int v = 0; v < 3; v++)
          it.bp[v] = xform_point(m, ldg3(pos, cl.firstLocalVertex + lt[tri * 3 + v]));
      }
      it.firstTriangle = e.firstTriangle;
      it.firstVertex   = e.firstVertex;
      n                = min((u32)e.numTriangles, kMaxChildrenPerItem);
      sm.item[lane]    = it;
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
      sm.pre[lane + 1] = x;
    if(lane == 0)
      sm.pre[0] = 0;
  }
  __syncthreads();
  const u32  numChildren = sm.pre[T];
  const u32  numChunks   = (numChildren + B - 1) / B;
  const bool cached      = numChildren <= S::kCacheChildren;

  // ---- pass 1: classify children; every warp counts its own slots ---------
  for(u32 ch = 0; ch < numChunks; ch++)
  {
    const u32  j     = ch * B + threadIdx.x;
    const bool valid = j < numChildren;
    bool       split = false;
    if(valid)
    {
      const u32   it    = parent_of(j);
      const Child child = make_child(c.table, sm.item[it], j - sm.pre[it], fp, sf);
      split             = child.split;
      if(cached)
        sm.child[j] = make_uint4(child.vtx[0], child.vtx[1], child.vtx[2], child.tc);
    }
    const u32 bs = __ballot_sync(0xFFFFFFFFu, valid && split), bp = __ballot_sync(0xFFFFFFFFu, valid && !split);
    if(lane == 0)
    {
      sm.cnt[kCntSplit][ch * kW + warp] = __popc(bs);
      sm.cnt[kCntPart][ch * kW + warp]  = __popc(bp);
      sm.splitMask[ch * kW + warp]      = bs;
    }
  }
  __syncthreads();

  // ---- slot offsets within the tile, tile totals, look-back ------------------
  if(warp < kNumCounters)
  {
    const u32 q     = warp;
    const u32 slots = numChunks * kW;
    u32       v[4], sum = 0;
#pragma unroll
    for(int r = 0; r < 4; r++)
    {
      const u32 i = lane * 4 + r;
      v[r]        = i < slots ? sm.cnt[q][i] : 0u;
      sum += v[r];
    }
    u32 incl = sum;
#pragma unroll
    for(int d = 1; d < 32; d <<= 1)
    {
      const u32 y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
      if(lane >= (u32)d)
        incl += y;
    }
    u32 run = incl - sum;
#pragma unroll
    for(int r = 0; r < 4; r++)
    {
      const u32 i = lane * 4 + r;
      if(i < slots)
        sm.cnt[q][i] = run;
      run += v[r];
    }
    const u32 agg  = __shfl_sync(0xFFFFFFFFu, incl, 31);
    u64       base = 0;
    if(tile == 0)  // the counters as the previous pass left them (through L2: see above)
      base = q == kCntSplit ? __ldcg(&b->splitWriteCounter) : part_base(c);
    const u64 ex = warp_lookback_exclusive(lbState + (u64)q * lbStride, tile, agg, base, c.errorWord, c.spinLimit);
    if(lane == 0)
    {
      sm.excl[q] = ex;
      if(tile == numTiles - 1)
        totals[q] = ex + agg;
    }
  }
  __syncthreads();

  // ---- pass 2: write, from pass 1's children or recomputed (no block barriers)
  for(u32 ch = 0; ch < numChunks; ch++)
  {
    const u32  j     = ch * B + threadIdx.x;
    const bool valid = j < numChildren;
    Child      child;
    u32        item = 0;
    child.split     = false;
    if(valid)
    {
      item = parent_of(j);
      if(cached)
      {
        const uint4 cc = sm.child[j];
        child.vtx[0] = cc.x, child.vtx[1] = cc.y, child.vtx[2] = cc.z, child.tc = cc.w;
        child.split  = (sm.splitMask[ch * kW + warp] >> lane) & 1u;
      }
      else
        child = make_child(c.table, sm.item[item], j - sm.pre[item], fp, sf);
    }
    const bool split = valid && child.split, part = valid && !child.split;
    const u32  bs = __ballot_sync(0xFFFFFFFFu, split), bp = __ballot_sync(0xFFFFFFFFu, part);
    if(split)
    {
      const u64 o = sm.excl[kCntSplit] + sm.cnt[kCntSplit][ch * kW + warp] + __popc(bs & ltm);
      if(o < k.maxSplitTriangles)
      {
        uint2* dst = reinterpret_cast<uint2*>(queue + o);
        dst[0]     = make_uint2(sm.item[item].ci.instanceID, sm.item[item].ci.clusterID);
        dst[1]     = make_uint2(child.vtx[0], child.vtx[1]);
        dst[2]     = make_uint2(child.vtx[2], child.tc);
        if(c.splitBase)
        {
          float* d = c.splitBase + 9 * o;
#pragma unroll
          for(int v = 0; v < 3; v++)
            d[3 * v] = sm.item[item].bp[v].x, d[3 * v + 1] = sm.item[item].bp[v].y, d[3 * v + 2] = sm.item[item].bp[v].z;
        }
      }
    }
    else if(part)
    {
      const u64 o = sm.excl[kCntPart] + sm.cnt[kCntPart][ch * kW + warp] + __popc(bp & ltm);
      if(o < partCap)
      {
        uint2* dst = reinterpret_cast<uint2*>(reinterpret_cast<tc_TessTriangleInfo*>(b->partTriangles) + o);
        dst[0]     = make_uint2(sm.item[item].ci.instanceID, sm.item[item].ci.clusterID);
        dst[1]     = make_uint2(child.vtx[0], child.vtx[1]);
        dst[2]     = make_uint2(child.vtx[2], child.tc);
      }
    }
  }
  __syncthreads();  // the item, prefix and count arrays are rewritten by the next tile
}

// The counters after a pass (triangle_split.comp.glsl:321-328 and the
// multipass dispatch's bookkeeping): run by one thread once every tile of the
// pass is done; `totals` are the last tile's inclusive totals.
__device__ inline void split_pass_counters(const StageCtx& c, u32 numTiles, const u64* totals, u32 partCap)
{
  tc_SceneBuilding* b = c.build;
  if(!numTiles)
    return;
  // another block's last tile wrote the totals: read them through L2
  b->splitWriteCounter = (u32)__ldcg(totals + kCntSplit);
  const u32 total      = (u32)__ldcg(totals + kCntPart);
  if(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
  {
    // requests to the counter's front half; partTriangleCounter is the
    // end of the written front (triangle_split.comp.glsl:321-328)
    const u32 start = (u32)b->dualPartTriangleCounter, written = min(total, partCap);
    b->dualPartTriangleCounter = (b->dualPartTriangleCounter & 0xFFFFFFFF00000000ull) | total;
    if(written > start)
      b->partTriangleCounter = max(b->partTriangleCounter, written);
  }
  else
    b->partTriangleCounter = total;
}

__device__ inline FactorParams split_factor_params(const StageCtx& c)
{
  FactorParams fp;
  fp.viewPos   = {c.build->viewPos.x, c.build->viewPos.y, c.build->viewPos.z};
  fp.nearPlane = c.view->nearPlane;
  fp.viewportH = c.view->viewportf.y;
  fp.tessRate  = c.view->tessRate;
  return fp;
}

template <int T, int B>
__global__ void __launch_bounds__(B) k_triangle_split(StageCtx c)
{
  stage_prologue();
  __shared__ SplitShared<T, B> sm;
  tc_SceneBuilding* b = c.build;
  // with transient builds a child part fits when it leaves the back's slots
  // and one more free (build.glsl:68-82, one child at a time)
  const u32            partCap = part_cap(c);
  tc_TessTriangleInfo* queue   = reinterpret_cast<tc_TessTriangleInfo*>(b->splitTriangles);

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
    sm.range[0] = lo;
    sm.range[1] = hi;
  }
  __syncthreads();
  const u32 begin    = sm.range[0], end = sm.range[1];
  const u32 numTiles = clamp_tiles(c, (end - begin + T - 1) / T);
  const FactorParams fp = split_factor_params(c);
  const u32          sf = clamp_split_factor(c.caps.splitFactor);

  for(;;)
  {
    const u32 tile = next_tile(c, &sm.tile);
    if(tile >= numTiles)
      break;
    split_tile<T, B>(c, sm, tile, begin, end, numTiles, c.scratch.lbState, c.scratch.lbStride, c.scratch.totals, fp,
                     sf, partCap);
  }

  if(last_block_done(c, &sm.flag))
  {
    if(threadIdx.x == 0)
    {
      split_pass_counters(c, numTiles, c.scratch.totals, partCap);
      if(c.fuseSetup != kNoSetup)
        build_setup_apply(c, c.fuseSetup);
    }
    scratch_release(c, numTiles, kNumCounters);
  }
}

// ---------------------------------------------------------------------------
// every pass in one launch
// ---------------------------------------------------------------------------

// Per-level control words, in the level's scratch slot (zeroed with the
// frame): [1] tiles done, [2..] u64 totals (split, part), [12] next level's
// range published, [13] finalised, [14] start, [15] end. Level 0's [0] is
// the ticket all levels share; the last level's [12] marks the end.
__device__ __forceinline__ u32* lv_done(const SplitLevels& lv, u32 L) { return lv.ctrl[L] + 1; }
__device__ __forceinline__ u64* lv_totals(const SplitLevels& lv, u32 L) { return reinterpret_cast<u64*>(lv.ctrl[L] + 2); }
__device__ __forceinline__ u32* lv_ready(const SplitLevels& lv, u32 L) { return lv.ctrl[L] + 12; }
__device__ __forceinline__ u32* lv_final(const SplitLevels& lv, u32 L) { return lv.ctrl[L] + 13; }

__device__ __forceinline__ void st_release_u32(u32* p, u32 v)
{
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Level L is complete (every tile done, or none): the pass's counters and
// set-up, then the next level's item range, published with release
// semantics. Run by one thread.
__device__ void finalize_level(const StageCtx& c, const SplitLevels& lv, u32 L, u32 numTiles, u32 partCap)
{
  tc_SceneBuilding* b = c.build;
  split_pass_counters(c, numTiles, lv_totals(lv, L), partCap);
  const bool last = L + 1 >= lv.levels;
  const u32  mode = last ? c.fuseSetup : (u32)TC_BUILD_SETUP_SPLIT_PASS;
  if(mode != kNoSetup)
    build_setup_apply(c, mode);
  if(!last)
  {
    lv.ctrl[L + 1][14] = min(b->splitPassStart, c.caps.maxSplitTriangles);
    lv.ctrl[L + 1][15] = min(b->splitPassEnd, c.caps.maxSplitTriangles);
  }
  __threadfence();
  st_release_u32(lv_ready(lv, L), 1u);
}

template <int T, int B>
__global__ void __launch_bounds__(B) k_triangle_split_levels(StageCtx c, SplitLevels lv)
{
  stage_prologue();
  __shared__ SplitShared<T, B> sm;
  __shared__ u32               s_level[4];  // level, its first ticket, its tiles, status (1: stop)
  tc_SceneBuilding* b        = c.build;
  const u32         partCap  = part_cap(c);
  const FactorParams fp      = split_factor_params(c);
  const u32          sf      = clamp_split_factor(c.caps.splitFactor);
  const u32          levels  = lv.levels;
  auto tiles_of = [&](u32 lo, u32 hi) { return min((hi - min(lo, hi) + T - 1) / T, lv.stride); };

  // level 0: the range the classify set-up (BUILD_SETUP_SPLIT) left
  u32 begin = min(min(b->splitPassStart, c.caps.maxSplitTriangles), min(b->splitPassEnd, c.caps.maxSplitTriangles));
  u32 end   = min(b->splitPassEnd, c.caps.maxSplitTriangles);
  u32 level = 0, first = 0, numTiles = tiles_of(begin, end);
  if(numTiles == 0)
  {
    // no split item: every level is empty; one block runs the passes' set-ups
    if(blockIdx.x == 0 && threadIdx.x == 0)
      for(u32 L = 0; L < levels; L++)
        finalize_level(c, lv, L, 0, partCap);
    return;
  }
  if(threadIdx.x == 0 && (end - begin + T - 1) / T > lv.stride)
    atomicOr(c.errorWord, TC_DEVERR_CAPACITY);

  for(;;)
  {
    const u32 g = next_tile(c, &sm.tile);  // one ticket over all levels
    // the level of ticket g (later levels wait for the earlier ones' completion)
    if(threadIdx.x == 0)
    {
      u32 stop = 0;
      while(g >= first + numTiles)
      {
        // level `level` has no tile for this ticket: move on to the next one
        if(numTiles == 0 && atomicCAS(lv_final(lv, level), 0u, 1u) == 0u)
        {
          __threadfence();
          finalize_level(c, lv, level, 0, partCap);
        }
        first += numTiles;
        if(++level >= levels)
        {
          stop = 1;
          break;
        }
        u32 spins = 0;
        while(ld_acquire_u32(lv_ready(lv, level - 1)) == 0u)
        {
          if(++spins > c.spinLimit)
          {
            atomicOr(c.errorWord, TC_DEVERR_LOOKBACK_TIMEOUT);
            stop = 1;
            break;
          }
          __nanosleep(spins > 64 ? 256 : 32);
        }
        if(stop)
          break;
        begin    = __ldcg(lv.ctrl[level] + 14);
        end      = __ldcg(lv.ctrl[level] + 15);
        numTiles = tiles_of(begin, end);
        if((end - min(begin, end) + T - 1) / T > lv.stride)
          atomicOr(c.errorWord, TC_DEVERR_CAPACITY);
      }
      s_level[0] = level, s_level[1] = first, s_level[2] = numTiles, s_level[3] = stop;
      sm.range[0] = begin, sm.range[1] = end;
    }
    __syncthreads();
    if(s_level[3])
      break;
    level    = s_level[0];
    first    = s_level[1];
    numTiles = s_level[2];
    begin    = sm.range[0];
    end      = sm.range[1];
    const u32 tile = g - first;
    split_tile<T, B>(c, sm, tile, begin, end, numTiles, lv.lbState[level], lv.stride, lv_totals(lv, level), fp, sf,
                     partCap);
    // the block completing the level's last tile finalises it
    if(threadIdx.x == 0)
    {
      __threadfence();
      if(atomicAdd(lv_done(lv, level), 1u) == numTiles - 1)
      {
        __threadfence();
        finalize_level(c, lv, level, numTiles, partCap);
      }
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_triangle_split_levels(const StageCtx& c, const SplitLevels& lv, u32 blockSize, u32 grid, cudaStream_t s)
{
  const int prio = high_launch_priority();
  switch(blockSize)
  {
    case 128:
      return launch_pdl_prio(k_triangle_split_levels<16, 128>, grid, 128, prio, s, c, lv);
    case 512:
      return launch_pdl_prio(k_triangle_split_levels<32, 512>, grid, 512, prio, s, c, lv);
    default:
      return launch_pdl_prio(k_triangle_split_levels<32, 256>, grid, 256, prio, s, c, lv);
  }
}

cudaError_t launch_triangle_split(const StageCtx& c, u32 blockSize, u32 grid, cudaStream_t s)
{
  // the split passes are the latency-critical branch of the frame: their
  // blocks take precedence over the concurrent instantiation's
  const int prio = high_launch_priority();
  switch(blockSize)
  {
    case 128:
      return launch_pdl_prio(k_triangle_split<16, 128>, grid, 128, prio, s, c);
    case 512:
      return launch_pdl_prio(k_triangle_split<32, 512>, grid, 512, prio, s, c);
    default:
      return launch_pdl_prio(k_triangle_split<32, 256>, grid, 256, prio, s, c);
  }
}

}  // namespace tc
