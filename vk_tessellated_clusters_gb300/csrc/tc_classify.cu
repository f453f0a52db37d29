// tc_classify.cu — cluster_classify: per-triangle edge segment counts and the
// full / part / split classification of every visible cluster.
//
// shaders/cluster_classify.comp.glsl:150-666 (RT target, plain path), and with
// TC_FLAG_TRANSIENT_1X / _2X :254-905 (transient CLAS builds of untessellated
// triangles and of 2X batches) through a count variant and a write kernel of
// their own.
//
// GB300 mapping, three launches per stage, none with a cross-block wait. Block
// b of the write grid owns the contiguous range of visible clusters
// [b * per, (b + 1) * per):
//   count : warps stride over the whole list, one cluster at a time per warp
//           (<= 64 triangles, two per lane), vertices staged in shared
//           memory; segment counts, configs and the cluster's counts (part /
//           split triangles, full-cluster vertices, CLAS bytes) go to
//           scratch, and 64-bit atomics add them to the sums of the cluster's
//           range
//   write : every block adds up the sums of the ranges before its own (the
//           counters' values before the launch included), then scans its own
//           clusters' counts in shared memory, so every offset equals what a
//           serial loop over the clusters gives; part / split triangles and
//           instantiation arguments go to those offsets, and the grid's last
//           block writes the counters' new totals
//   full vertices : the displaced vertices of the accepted full clusters, from
//           the records write leaves (a launch of its own, beside later work)
#include <algorithm>

#include "tc_kernels.h"
#include "tc_stage.cuh"
#include "tc_vertex.cuh"

namespace tc {

namespace {

constexpr u32 kBlock = 256;  // threads of the count and write blocks
constexpr u32 kWarps = kBlock / 32;

enum : int
{
  kCntParts = 0,
  kCntSplits,
  kCntGen,
  kCntVerts,
  kCntData,
  kNumCounters
};

// per-cluster counts: x = parts | splits << 7 | full << 14 | fullVertices << 15 | fullTriangles << 22,
// y = CLAS bytes
__device__ __forceinline__ uint2 pack_counts(u32 parts, u32 splits, bool full, u32 nv, u32 nt, u32 data)
{
  return make_uint2(parts | (splits << 7) | ((full ? 1u : 0u) << 14) | ((full ? nv : 0u) << 15) | ((full ? nt : 0u) << 22),
                    full ? data : 0u);
}
__device__ __forceinline__ u32 cnt_parts(uint2 r) { return r.x & 0x7F; }
__device__ __forceinline__ u32 cnt_splits(uint2 r) { return (r.x >> 7) & 0x7F; }
__device__ __forceinline__ u32 cnt_full(uint2 r) { return (r.x >> 14) & 1; }
__device__ __forceinline__ u32 cnt_verts(uint2 r) { return (r.x >> 15) & 0x7F; }
__device__ __forceinline__ u32 cnt_tris(uint2 r) { return (r.x >> 22) & 0x7F; }

// tessellation.glsl:119-144 tess_getConfig, also reporting how the three
// sub-triangle corners were rotated (0: none, 1: .yzx, 2: .zxy)
__device__ __forceinline__ u32 get_config_rot(uint3 f, u32& rot)
{
  u32 m = max(max(f.x, f.y), f.z);
  rot   = 0;
  if(m == f.y)
  {
    f   = make_uint3(f.y, f.z, f.x);
    rot = 1;
  }
  else if(m == f.z)
  {
    f   = make_uint3(f.z, f.x, f.y);
    rot = 2;
  }
  const u32 L   = TC_TESSTABLE_LOOKUP_SIZE;
  u32       idx = f.x + f.y * L + f.z * L * L - (1 + L + L * L);
  if(f.z > f.y)
    idx |= 1u << 15;
  return idx;
}

// per-triangle word: config | rotation << 16 | split << 18
__device__ __forceinline__ u32 classify_triangle(uint3 f, u32 sf)
{
  const u32  m     = max(max(f.x, f.y), f.z);
  const bool split = m > TC_TESSTABLE_SIZE;
  if(split)
    f = make_uint3(split_factor1(f.x, sf), split_factor1(f.y, sf), split_factor1(f.z, sf));
  u32       rot;
  const u32 cfg = get_config_rot(f, rot);
  return cfg | (rot << 16) | ((split ? 1u : 0u) << 18);
}

struct ClassifyScratch
{
  uint2*          counts;     // per visible cluster of the window
  u32*            triWords;   // 64 per visible cluster
  RangeSums*      rangeSums;  // per write block's range: the counts' sums, zero before count
  ClusterOffsets* bases;      // the counters before the launch
  u32             writeBlocks;  // the write launch's grid (its blocks' ranges)
  u32             _pad;
  uint2*          fullRecs;   // per full cluster (generated-cluster slot - first slot): visible index, first vertex
  u32*            fullRange;  // [2]: the launch's generated-cluster slots [begin, end)
};

constexpr u32 kRejected = 0xFFFFFFFFu;  // fullRecs: a full cluster that did not fit the capacities

// the contiguous range of visible clusters block `blk` of `nb` owns
__device__ __forceinline__ void block_range(u32 n, u32 blk, u32 nb, u32& v0, u32& v1)
{
  const u32 per = (n + nb - 1) / nb;
  v0            = min(n, blk * per);
  v1            = min(n, v0 + per);
}

// Visible cluster v when the list is every cluster in instance order (RT
// semantics: clusters_cull keeps them all): the instance whose first flat
// index is the last one <= v.
// `starts`: the instances' first flat indices (instClusterStart, or the
// block's shared copy of it)
__device__ __forceinline__ tc_ClusterInfo flat_cluster(const u32* starts, u32 numInstances, u32 v)
{
  u32 lo = 0, hi = numInstances;
  while(hi - lo > 1)
  {
    const u32 mid = (lo + hi) >> 1;
    if(starts[mid] <= v)
      lo = mid;
    else
      hi = mid;
  }
  return {lo, v - starts[lo]};
}

// Instance counts up to kFlatShared keep the prefix in shared memory, where
// the binary search of every cluster lookup runs.
constexpr u32 kFlatShared = 1024;

struct FlatStarts
{
  u32 v[kFlatShared];
};

// Called by every thread of the block (contains a barrier); returns the
// prefix the block's lookups use.
__device__ __forceinline__ const u32* stage_flat_starts(const StageCtx& c, FlatStarts& sh)
{
  if(!c.flatVisible || c.numInstances > kFlatShared)
    return c.instClusterStart;
  for(u32 i = threadIdx.x; i < c.numInstances; i += blockDim.x)
    sh.v[i] = c.instClusterStart[i];
  __syncthreads();
  return sh.v;
}

__device__ __forceinline__ tc_ClusterInfo visible_cluster(const StageCtx& c, const u32* starts,
                                                          const tc_ClusterInfo* vis, u32 v)
{
  return c.flatVisible ? flat_cluster(starts, c.numInstances, v) : vis[v];
}

// visible clusters of the instance window (visibleClusters is sorted by instance)
__device__ inline void window_range(const StageCtx& c, u32& lo, u32& hi)
{
  if(c.flatVisible)  // whole window, every cluster listed (clusters_cull runs beside classify)
  {
    lo = 0;
    hi = min(c.instClusterStart[c.numInstances], c.caps.maxVisibleClusters);
    return;
  }
  const tc_ClusterInfo* vis = reinterpret_cast<const tc_ClusterInfo*>(c.build->visibleClusters);
  lo                        = 0;
  hi                        = min(c.build->visibleClusterCounter, c.caps.maxVisibleClusters);
  if(!whole_window(c))
  {
    auto get = [&](u32 i) { return vis[i].instanceID; };
    u32  e   = lower_bound_instance(lo, hi, c.instEnd, get);
    lo       = lower_bound_instance(lo, e, c.instBegin, get);
    hi       = e;
  }
}

__device__ __forceinline__ FactorParams factor_params(const StageCtx& c)
{
  FactorParams fp;
  fp.viewPos   = {c.build->viewPos.x, c.build->viewPos.y, c.build->viewPos.z};
  fp.nearPlane = c.view->nearPlane;
  fp.viewportH = c.view->viewportf.y;
  fp.tessRate  = c.view->tessRate;
  return fp;
}

// ---------------------------------------------------------------------------
// scans
// ---------------------------------------------------------------------------

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

// block-wide exclusive scan of kNumCounters values per thread
__device__ inline void block_scan5(u64 (&v)[kNumCounters], u64 (&tot)[kNumCounters], u64 (*s_warp)[kNumCounters])
{
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  u64       inc[kNumCounters];
#pragma unroll
  for(int q = 0; q < kNumCounters; q++)
  {
    inc[q] = warp_inclusive<u64>(v[q], lane);
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
#pragma unroll
  for(int q = 0; q < kNumCounters; q++)
  {
    tot[q] = s_warp[32][q];
    v[q]   = s_warp[warp][q] + inc[q] - v[q];
  }
  __syncthreads();
}

// block-wide exclusive scan of N values per thread (totals in tot)
template <int N>
__device__ inline void block_scan_n(u64 (&v)[N], u64 (&tot)[N], u64 (*s_warp)[N])
{
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  u64       inc[N];
#pragma unroll
  for(int q = 0; q < N; q++)
  {
    inc[q] = warp_inclusive<u64>(v[q], lane);
    if(lane == 31)
      s_warp[warp][q] = inc[q];
  }
  __syncthreads();
  if(warp == 0)
  {
#pragma unroll
    for(int q = 0; q < N; q++)
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
#pragma unroll
  for(int q = 0; q < N; q++)
  {
    tot[q] = s_warp[32][q];
    v[q]   = s_warp[warp][q] + inc[q] - v[q];
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// count
// ---------------------------------------------------------------------------

// The offsets at which block `blockIdx.x` of the write launch starts: the
// counters' values before the launch plus the sums of all blocks before it.
__device__ inline void block_prefix(const ClassifyScratch& cs, u64 (&pre)[kNumCounters],
                                    u64 (*s_warp)[kNumCounters])
{
  u64 x[kNumCounters] = {0, 0, 0, 0, 0};
  for(u32 i = threadIdx.x; i < blockIdx.x; i += blockDim.x)
  {
    const RangeSums o = cs.rangeSums[i];
    x[kCntParts] += (u32)o.partsSplits;
    x[kCntSplits] += (u32)(o.partsSplits >> 32);
    x[kCntGen] += (u32)o.fullVerts;
    x[kCntVerts] += (u32)(o.fullVerts >> 32);
    x[kCntData] += o.data;
  }
  u64 tot[kNumCounters];
  block_scan5(x, tot, s_warp);
  const ClusterOffsets b0 = *cs.bases;
  pre[kCntParts]          = b0.part + tot[kCntParts];
  pre[kCntSplits]         = b0.split + tot[kCntSplits];
  pre[kCntGen]            = b0.gen + tot[kCntGen];
  pre[kCntVerts]          = b0.vert + tot[kCntVerts];
  pre[kCntData]           = b0.data + tot[kCntData];
}

// ---------------------------------------------------------------------------
// transient builds (TC_FLAG_TRANSIENT_1X / _2X)
// ---------------------------------------------------------------------------

// per-triangle word bits beyond config | rotation << 16 | split << 18
constexpr u32 kWordMini        = 1u << 19;  // packed into a 2X batch
constexpr u32 kWordSubset      = 1u << 20;  // in the cluster's 1X subset
constexpr u32 kWordFactorShift = 21;        // edge factors - 1 (3 bits) of a triangle with factors <= 2

constexpr u32 kClusterInfoBytes = 8, kTessInfoBytes = 24;
constexpr u32 kMiniBatch        = TC_2X_MINI_BATCHSIZE;
constexpr u32 kMiniBatchTris    = TC_2X_MINI_BATCHSIZE * TC_2X_MINI_TRIANGLES;
constexpr u32 kMiniBatchVerts   = TC_2X_MINI_BATCHSIZE * TC_2X_MINI_VERTICES;
constexpr u32 kMiniVertexSize   = kMiniBatchVerts + (kMiniBatchTris * 3 + 11) / 12;  // vertices, then index bytes
constexpr u32 kMiniPartSlots    = (kClusterInfoBytes + kMiniBatchTris * 2 + kTessInfoBytes - 1) / kTessInfoBytes;
__device__ __forceinline__ u32 subset_vertex_size(u32 nv, u32 simple) { return nv + (simple * 3 + 11) / 12; }
__device__ __forceinline__ u32 subset_part_slots(u32 simple)
{
  return (kClusterInfoBytes + simple + kTessInfoBytes - 1) / kTessInfoBytes;
}

// per-cluster counts with transient builds (16 bytes):
// x = parts | splits << 7 | generated clusters << 14 | transient builds << 19 | back slots << 23 | full << 28 | 1X << 29
// y = vertices | simple triangles << 10 | numVertices << 17 | numTriangles << 24, z = CLAS bytes
__device__ __forceinline__ u32 t_parts(uint4 r) { return r.x & 0x7F; }
__device__ __forceinline__ u32 t_splits(uint4 r) { return (r.x >> 7) & 0x7F; }
__device__ __forceinline__ u32 t_gen(uint4 r) { return (r.x >> 14) & 0x1F; }
__device__ __forceinline__ u32 t_trans(uint4 r) { return (r.x >> 19) & 0xF; }
__device__ __forceinline__ u32 t_back(uint4 r) { return (r.x >> 23) & 0x1F; }
__device__ __forceinline__ bool t_full(uint4 r) { return (r.x >> 28) & 1; }
__device__ __forceinline__ bool t_subset(uint4 r) { return (r.x >> 29) & 1; }
__device__ __forceinline__ u32 t_verts(uint4 r) { return r.y & 0x3FF; }
__device__ __forceinline__ u32 t_simple(uint4 r) { return (r.y >> 10) & 0x7F; }
__device__ __forceinline__ u32 t_nv(uint4 r) { return (r.y >> 17) & 0x7F; }
__device__ __forceinline__ u32 t_nt(uint4 r) { return (r.y >> 24) & 0x7F; }

// cluster_classify.comp.glsl:254-343 and 543-790, counting only: which
// triangles go to the 1X subset, to parts, to splits and to 2X batches, and
// what the cluster takes from every counter (each allocation counts whether or
// not it will fit, like the reference's atomics). m0/m1, w0/w1: the max factor
// and word of triangles lane and lane + 32.
__device__ __forceinline__ void count_transient(const StageCtx& c, const ClassifyScratch& cs, u32 v, u32 perRange, u32 nv,
                                             u32 nt, u32 simple, u32 m0, u32 m1, u32 w0, u32 w1, u32 templateSize)
{
  const u32  lane   = threadIdx.x & 31;
  const bool full   = simple == nt;
  const bool subset = (c.flags & TC_FLAG_TRANSIENT_1X) && !full && simple > 1;
  const bool mini2x = (c.flags & TC_FLAG_TRANSIENT_2X) != 0;
  const u32* basic  = reinterpret_cast<const u32*>(c.build->basicClusterSizes);
  u32        parts = 0, splits = 0, batches = 0;
  if(!full)
  {
    auto mark = [&](u32 m, u32& w) {  // :573-590
      if(subset && m == 1)
        w |= kWordSubset;
      else if(m <= TC_TESSTABLE_SIZE && mini2x && m <= 2)
        w |= kWordMini;
    };
    if(lane < nt)
      mark(m0, w0);
    if(lane + 32 < nt)
      mark(m1, w1);
    const bool v0 = lane < nt, v1 = lane + 32 < nt;
    parts  = __popc(__ballot_sync(0xFFFFFFFFu, v0 && (w0 & (kWordMini | kWordSubset | (1u << 18))) == 0))
             + __popc(__ballot_sync(0xFFFFFFFFu, v1 && (w1 & (kWordMini | kWordSubset | (1u << 18))) == 0));
    splits = __popc(__ballot_sync(0xFFFFFFFFu, v0 && (w0 & (1u << 18)))) + __popc(__ballot_sync(0xFFFFFFFFu, v1 && (w1 & (1u << 18))));
    const u32 mini0 = __popc(__ballot_sync(0xFFFFFFFFu, v0 && (w0 & kWordMini)));
    const u32 mini1 = __popc(__ballot_sync(0xFFFFFFFFu, v1 && (w1 & kWordMini)));
    batches         = (mini0 + kMiniBatch - 1) / kMiniBatch + (mini1 + kMiniBatch - 1) / kMiniBatch;
    u32* tw         = cs.triWords + (u64)v * TC_MAX_CLUSTER_TRIANGLES;
    if(v0)
      tw[lane] = w0;
    if(v1)
      tw[lane + 32] = w1;
  }
  if(lane != 0)
    return;
  const u32 one   = (full || subset) ? 1u : 0u;
  const u32 gen   = one + batches, trans = (subset ? 1u : 0u) + batches;
  const u32 verts = (full ? nv : (subset ? subset_vertex_size(nv, simple) : 0u)) + kMiniVertexSize * batches;
  const u32 back  = (subset ? subset_part_slots(simple) : 0u) + kMiniPartSlots * batches;
  u64       data  = full ? (u64)templateSize : (subset ? (u64)basic[simple] : 0ull);
  if(batches)
    data += (u64)basic[kMiniBatchTris] * batches;
  reinterpret_cast<uint4*>(cs.counts)[v] =
      make_uint4(parts | (splits << 7) | (gen << 14) | (trans << 19) | (back << 23) | ((full ? 1u : 0u) << 28)
                     | ((subset ? 1u : 0u) << 29),
                 verts | (simple << 10) | (nv << 17) | (nt << 24), (u32)data, 0u);
  RangeSums& rs = cs.rangeSums[v / perRange];
  if(parts | splits)
    atomicAdd(&rs.partsSplits, (unsigned long long)parts | ((unsigned long long)splits << 32));
  if(gen)
  {
    atomicAdd(&rs.fullVerts, (unsigned long long)gen | ((unsigned long long)verts << 32));
    if(data)
      atomicAdd(&rs.data, (unsigned long long)data);
  }
  if(trans)
    atomicAdd(&rs.backTrans, (unsigned long long)back | ((unsigned long long)trans << 32));
}

// MinBlocks: resident 256-thread blocks per SM the registers are sized for
// (4: 64 registers, 6: 40, 8: 32); more resident warps hide more of the
// dependent-load latency per cluster at the cost of some spills.
template <int MinBlocks, bool Trans = false>
__global__ void __launch_bounds__(kBlock, MinBlocks) k_classify_count(StageCtx c, ClassifyScratch cs)
{
  stage_prologue();
  __shared__ f3  s_vert[kWarps][TC_MAX_CLUSTER_VERTICES];
  __shared__ f2  s_dist[kWarps][TC_MAX_CLUSTER_VERTICES];  // per vertex: distance to the view position, its reciprocal
  __shared__ u32 s_range[2];
  __shared__ FlatStarts s_starts;
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    window_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32* starts = stage_flat_starts(c, s_starts);
  const u32 begin = s_range[0];
  const u32 n     = min(s_range[1] - s_range[0], c.scratch.itemCapacity);

  const tc_SceneBuilding* b       = c.build;
  const tc_ClusterInfo*   vis     = reinterpret_cast<const tc_ClusterInfo*>(b->visibleClusters);
  const FactorParams      fp      = factor_params(c);
  const float             rNear   = __fdiv_rn(1.0f, fp.nearPlane);
  const float             kRate   = fp.viewportH * fp.tessRate;
  const float             k2      = kRate * kRate;
  const float             near2   = fp.nearPlane * fp.nearPlane;
  const bool              culling = (c.flags & TC_FLAG_CULLING) != 0;
  const u32               sf      = clamp_split_factor(c.caps.splitFactor);
  const u32               wordOnes = classify_triangle(make_uint3(1u, 1u, 1u), sf);  // a triangle of factors 1
  if(blockIdx.x == 0 && threadIdx.x == 0)  // the offsets continue from the counters' current values
  {
    if constexpr(Trans)
    {
      // parts from the front of the two-sided counter (build.glsl:52-82)
      *cs.bases = {(u32)b->dualPartTriangleCounter, (u32)b->splitTriangleCounter, b->genClusterCounter,
                   b->genVertexCounter, b->genClusterDataCounter};
      *reinterpret_cast<TransBases*>(cs.bases + 1) = {(u32)(b->dualPartTriangleCounter >> 32), b->transBuildCounter,
                                                      b->tempInstantiateCounter, 0u};
    }
    else
      *cs.bases = {b->partTriangleCounter, (u32)b->splitTriangleCounter, b->genClusterCounter, b->genVertexCounter,
                   b->genClusterDataCounter};
  }
  // the write launch's block ranges, which collect the counts' sums
  const u32 perRange = (n + cs.writeBlocks - 1) / cs.writeBlocks;

  // the warp's clusters are v = gw + nwarps * j, j < cntW (spread over the
  // whole list, which evens out instances of uneven cost); their cluster
  // records load one lane per cluster, 32 at a time, so that only the vertex
  // and index loads remain on each cluster's dependent path
  const u32  gw     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32  nwarps = (gridDim.x * blockDim.x) >> 5;
  const u32  cntW   = gw < n ? (n - gw + nwarps - 1) / nwarps : 0u;
  const u32* states = reinterpret_cast<const u32*>(b->instanceStates);
  for(u32 j0 = 0; j0 < cntW; j0 += 32)
  {
    const u32 jn = min(32u, cntW - j0);
    u32       hInst = 0, hMeta = 0, hFirstV = 0, hFirstT = 0, hData = 0;
    if(lane < jn)
    {
      const tc_ClusterInfo     ci = visible_cluster(c, starts, vis, begin + gw + nwarps * (j0 + lane));
      const tc_RenderInstance* in = c.instances + ci.instanceID;
      const tc_Cluster         cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[ci.clusterID];
      u32                      nt = cl.numTriangles, nv = cl.numVertices;
      if(nt > TC_MAX_CLUSTER_TRIANGLES || nv > TC_MAX_CLUSTER_VERTICES)
      {
        atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
        nt = min(nt, TC_MAX_CLUSTER_TRIANGLES);
        nv = min(nv, TC_MAX_CLUSTER_VERTICES);
      }
      // cluster_classify.comp.glsl:203-211: invisible instance, no tessellation
      const bool culled = culling && (states[ci.instanceID] & TC_INSTANCE_VISIBLE_BIT) == 0;
      hInst             = ci.instanceID;
      hMeta             = nv | (nt << 8) | ((culled ? 1u : 0u) << 16);
      hFirstV           = cl.firstLocalVertex;
      hFirstT           = cl.firstLocalTriangle;
      hData             = __ldg(reinterpret_cast<const u32*>(in->clusterTemplateInstantiatonSizes) + ci.clusterID);
    }
    for(u32 jj = 0; jj < jn; jj++)
    {
      const u32                v      = gw + nwarps * (j0 + jj);
      const u32                meta   = __shfl_sync(0xFFFFFFFFu, hMeta, jj);
      const u32                nv     = meta & 0xFF, nt = (meta >> 8) & 0xFF;
      const bool               culled = (meta >> 16) != 0;
      const tc_RenderInstance* in     = c.instances + __shfl_sync(0xFFFFFFFFu, hInst, jj);
      const u32                firstV = __shfl_sync(0xFFFFFFFFu, hFirstV, jj);
      const u32                firstT = __shfl_sync(0xFFFFFFFFu, hFirstT, jj);
      u32                      m0 = 0, m1 = 0, w0 = 0, w1 = 0;
      u32                      simple = nt;
      if(!culled)
      {
        // indices first (their loads overlap the vertex loads); masked to the
        // staged range: a malformed index reads a wrong vertex of the same
        // cluster, never outside shared memory
        const uint8_t* lt = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + firstT;
        u32            ia = 0, ib = 0;
        if(lane < nt)
          ia = (lt[lane * 3 + 0] & 63u) | ((lt[lane * 3 + 1] & 63u) << 8) | ((lt[lane * 3 + 2] & 63u) << 16);
        if(lane + 32 < nt)
          ib = (lt[lane * 3 + 96] & 63u) | ((lt[lane * 3 + 97] & 63u) << 8) | ((lt[lane * 3 + 98] & 63u) << 16);
        // cluster_classify.comp.glsl:180-198 vertices, then 217-246 factors; each
        // vertex is taken to world space once here (the same operations the
        // shader applies per triangle corner, so the same bits)
        const float* pos = reinterpret_cast<const float*>(in->positions);
        float        m[16];
#pragma unroll
        for(int q = 0; q < 16; q++)
          m[q] = __ldg(in->worldMatrix.m + q);
        for(u32 i = lane; i < nv; i += 32)
        {
          const f3 w  = xform_point(m, ldg3(pos, firstV + i));
          const f3 dv = sub3(w, fp.viewPos);
          s_vert[warp][i]   = w;
          s_dist[warp][i].x = dot3(dv, dv);  // squared: the distance and its reciprocal only when needed
        }
        __syncwarp();
        // A cluster whose every edge provably has factor 1 (edge_factor_one_sq:
        // squared lengths and distances, no roots or divisions) is classified
        // without the distances; the word is that of factors (1, 1, 1).
        auto allOne = [&](u32 idx) {
          const u32   i0 = idx & 0xFF, i1 = (idx >> 8) & 0xFF, i2 = idx >> 16;
          const f3    v0 = s_vert[warp][i0], v1 = s_vert[warp][i1], v2 = s_vert[warp][i2];
          const float q0 = s_dist[warp][i0].x, q1 = s_dist[warp][i1].x, q2 = s_dist[warp][i2].x;
          return edge_factor_one_sq(v0, v1, q0, q1, k2, near2) && edge_factor_one_sq(v1, v2, q1, q2, k2, near2)
                 && edge_factor_one_sq(v2, v0, q2, q0, k2, near2);
        };
        if(__all_sync(0xFFFFFFFFu, (lane >= nt || allOne(ia)) && (lane + 32 >= nt || allOne(ib))))
        {
          if(lane < nt)
            m0 = 1, w0 = wordOnes;
          if(lane + 32 < nt)
            m1 = 1, w1 = wordOnes;
          simple = nt;
        }
        else
        {
          for(u32 i = lane; i < nv; i += 32)
          {
            const float d     = __fsqrt_rn(s_dist[warp][i].x);  // dist3(w, viewPos)
            s_dist[warp][i].y = __fdiv_rn(1.0f, d);
            s_dist[warp][i].x = d;
          }
          __syncwarp();
          auto classify = [&](u32 idx, u32& mOut, u32& wOut) {
            const u32   i0 = idx & 0xFF, i1 = (idx >> 8) & 0xFF, i2 = idx >> 16;
            const f2    d0 = s_dist[warp][i0], d1 = s_dist[warp][i1], d2 = s_dist[warp][i2];
            const uint3 f  = tess_factors_hoisted(s_vert[warp][i0], s_vert[warp][i1], s_vert[warp][i2], d0.x, d1.x,
                                                  d2.x, d0.y, d1.y, d2.y, rNear, fp);
            mOut           = max(max(f.x, f.y), f.z);
            wOut           = classify_triangle(f, sf);
            if constexpr(Trans)  // factors of a 2X candidate, for its triangle map (cluster_classify.comp.glsl:817)
              if(mOut <= 2)
                wOut |= ((f.x - 1) | ((f.y - 1) << 1) | ((f.z - 1) << 2)) << kWordFactorShift;
          };
          if(lane < nt)
            classify(ia, m0, w0);
          if(lane + 32 < nt)
            classify(ib, m1, w1);
          simple = __popc(__ballot_sync(0xFFFFFFFFu, lane < nt && m0 == 1))
                   + __popc(__ballot_sync(0xFFFFFFFFu, lane + 32 < nt && m1 == 1));
        }
        __syncwarp();  // s_vert is reused by the next cluster
      }
      const bool full  = simple == nt;
      if constexpr(Trans)
      {
        count_transient(c, cs, v, perRange, nv, nt, simple, m0, m1, w0, w1, __shfl_sync(0xFFFFFFFFu, hData, jj));
        continue;
      }
      u32        parts = 0, splits = 0;
      if(!full)
      {
        parts  = __popc(__ballot_sync(0xFFFFFFFFu, lane < nt && m0 <= TC_TESSTABLE_SIZE))
                 + __popc(__ballot_sync(0xFFFFFFFFu, lane + 32 < nt && m1 <= TC_TESSTABLE_SIZE));
        splits = nt - parts;
        u32* tw = cs.triWords + (u64)v * TC_MAX_CLUSTER_TRIANGLES;
        if(lane < nt)
          tw[lane] = w0;
        if(lane + 32 < nt)
          tw[lane + 32] = w1;
      }
      const u32 data = __shfl_sync(0xFFFFFFFFu, hData, jj);
      if(lane == 0)
      {
        cs.counts[v] = pack_counts(parts, splits, full, nv, nt, data);
        RangeSums& rs = cs.rangeSums[v / perRange];
        if(full)
        {
          atomicAdd(&rs.fullVerts, 1ull | ((unsigned long long)nv << 32));
          if(data)
            atomicAdd(&rs.data, (unsigned long long)data);
        }
        else
          atomicAdd(&rs.partsSplits, (unsigned long long)parts | ((unsigned long long)splits << 32));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// write
// ---------------------------------------------------------------------------

__device__ __forceinline__ void store_tess_info(tc_TessTriangleInfo* dst, const tc_ClusterInfo& ci, u32 v0, u32 v1,
                                                u32 v2, u32 tc)
{
  uint2* p = reinterpret_cast<uint2*>(dst);
  p[0]     = make_uint2(ci.instanceID, ci.clusterID);
  p[1]     = make_uint2(v0, v1);
  p[2]     = make_uint2(v2, tc);
}

// part / split triangle from its per-triangle word (cluster_classify.comp.glsl:608-666)
__device__ __forceinline__ void emit_triangle(tc_TessTriangleInfo* dst, const tc_ClusterInfo& ci, u32 tri, u32 word)
{
  u32       v0 = 0, v1 = TC_TESSTABLE_COORD_MAX, v2 = TC_TESSTABLE_COORD_MAX << 16;
  const u32 rot = (word >> 16) & 3;
  if(rot == 1)
  {
    u32 t = v0;
    v0 = v1, v1 = v2, v2 = t;
  }
  else if(rot == 2)
  {
    u32 t = v2;
    v2 = v1, v1 = v0, v0 = t;
  }
  store_tess_info(dst, ci, v0, v1, v2, tri | ((word & 0xFFFFu) << 16));
}

// what the vertex walk of a full cluster needs (phase 2 of k_classify_write)
struct FullRecord
{
  MapDesc      map;
  const float* pos;
  const float* nrm;
  const float* uvs;
  u32          first;  // firstLocalVertex
  float        scale;  // instance x view displacement scale
  float        offset; // instance + view displacement offset
  u32          vo;     // first generated vertex
  u32          nv;     // vertex count
  u32          inst;   // instance (the ripple's seed)
  float        size;   // its geometry size (RenderInstance.geoHi.w)
};

// the vertex walk over a batch of full clusters (records in `rec`), for
// records of map kind Kind (~0u: any)
template <u32 Kind>
__device__ __forceinline__ void full_steps(const FullRecord* rec, bool owner, u32 rStart, u32 rEnd, float* dst,
                                           const RippleParams& rp)
{
  const u32 lane = threadIdx.x & 31;
#pragma unroll 2  // two steps in flight: their loads overlap
  for(u32 base = 0; base < rEnd; base += 32)
  {
    const u32 before = __popc(__ballot_sync(0xFFFFFFFFu, owner && rStart <= base));
    const u32 inside = __reduce_or_sync(0xFFFFFFFFu,
                                        (owner && rStart > base && rStart < base + 32) ? 1u << (rStart - base) : 0u);
    const u32 ri     = before - 1 + __popc(inside & ((2u << lane) - 2u));
    const u32 rs     = __shfl_sync(0xFFFFFFFFu, rStart, ri & 31);
    const u32 jj     = base + lane;
    const FullRecord& fr = rec[ri];
    // (transient builds leave index bytes and 2X batches between the ranges)
    if(jj < rEnd && jj - rs < fr.nv)
    {
      const u32 vi = fr.first + (jj - rs);
      f3                p  = ldg3(fr.pos, vi);
      if(Kind != kAffineFlat)
        p = full_vertex_k<Kind>(p, ldg3(fr.nrm, vi), ldg2(fr.uvs, vi), fr.map, fr.scale, fr.offset);
      if(rp.enabled)  // cluster_classify.comp.glsl:483-485
        p = ripple(p, fr.inst, fr.size, rp);
      float* d = dst + (u64)jj * 3;
      d[0]     = p.x;
      d[1]     = p.y;
      d[2]     = p.z;
    }
  }
}

// full_steps for a batch whose records share the attribute arrays, map,
// displacement scale and offset (and, with the ripple, the instance): those
// stay in registers (`u`, read once per batch), and each step takes only its
// record's vertex-index offset and range end from the record's lane (two
// shuffles) instead of the record from shared memory. Same operations, so the
// same bits.
template <u32 Kind>
__device__ __forceinline__ void full_steps_uniform(const FullRecord& u, bool owner, u32 rStart, u32 rOff, u32 rStop,
                                                   u32 rEnd, float* dst, const RippleParams& rp)
{
  const u32 lane  = threadIdx.x & 31;
  const u32 below = (2u << lane) - 2u;
#pragma unroll 2  // two steps in flight: their loads overlap
  for(u32 base = 0; base < rEnd; base += 32)
  {
    const u32 before = __popc(__ballot_sync(0xFFFFFFFFu, owner && rStart <= base));
    const u32 inside = __reduce_or_sync(0xFFFFFFFFu,
                                        (owner && rStart > base && rStart < base + 32) ? 1u << (rStart - base) : 0u);
    const u32 ri     = (before - 1 + __popc(inside & below)) & 31;
    const u32 off    = __shfl_sync(0xFFFFFFFFu, rOff, ri);
    const u32 stop   = __shfl_sync(0xFFFFFFFFu, rStop, ri);
    const u32 jj     = base + lane;
    // (transient builds leave index bytes and 2X batches between the ranges)
    if(jj < stop)
    {
      const u32 vi = off + jj;
      f3        p  = ldg3(u.pos, vi);
      if(Kind != kAffineFlat)
        p = full_vertex_k<Kind>(p, ldg3(u.nrm, vi), ldg2(u.uvs, vi), u.map, u.scale, u.offset);
      if(rp.enabled)  // cluster_classify.comp.glsl:483-485
        p = ripple(p, u.inst, u.size, rp);
      float* d = dst + (u64)jj * 3;
      d[0]     = p.x;
      d[1]     = p.y;
      d[2]     = p.z;
    }
  }
}

template <int MinBlocks>
__global__ void __launch_bounds__(kBlock, MinBlocks) k_classify_write(StageCtx c, ClassifyScratch cs)
{
  stage_prologue();
  __shared__ u32            s_range[2];
  __shared__ u64            s_warp[33][kNumCounters];
  __shared__ ClusterOffsets s_off[kBlock];  // offsets of the chunk's clusters
  __shared__ uint2          s_cnt[kBlock];  // counts of the chunk's clusters
  __shared__ tc_ClusterInfo s_ci[kBlock];   // the chunk's clusters
  __shared__ FlatStarts     s_starts;
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    window_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32* starts = stage_flat_starts(c, s_starts);
  const u32 begin = s_range[0];
  const u32 n     = min(s_range[1] - s_range[0], c.scratch.itemCapacity);

  tc_SceneBuilding*     b            = c.build;
  const tc_caps&        k            = c.caps;
  const tc_ClusterInfo* vis          = reinterpret_cast<const tc_ClusterInfo*>(b->visibleClusters);
  const u64             maxData      = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  tc_TessTriangleInfo*  splits       = reinterpret_cast<tc_TessTriangleInfo*>(b->splitTriangles);
  tc_TessTriangleInfo*  parts        = reinterpret_cast<tc_TessTriangleInfo*>(b->partTriangles);
  tc_BlasBuildInfo*     blas         = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  const u32             ltm          = (1u << lane) - 1u;
  u32                   statTris = 0, statTemp = 0;

  u64 pre[kNumCounters];  // offsets of the next chunk's first cluster
  block_prefix(cs, pre, s_warp);
  const u32 genBase = cs.bases->gen;
  u32       vBegin, vEnd;
  block_range(n, blockIdx.x, gridDim.x, vBegin, vEnd);
  for(u32 c0 = vBegin; c0 < vEnd; c0 += kBlock)
  {
    // exclusive scan of the chunk's counts, in cluster order
    const u32 len = min(kBlock, vEnd - c0);
    {
      const uint2 r = threadIdx.x < len ? cs.counts[c0 + threadIdx.x] : make_uint2(0, 0);
      if(threadIdx.x < len)  // looked up once per cluster, in parallel
        s_ci[threadIdx.x] = visible_cluster(c, starts, vis, begin + c0 + threadIdx.x);
      u64 x[kNumCounters] = {cnt_parts(r), cnt_splits(r), cnt_full(r), cnt_verts(r), r.y};
      u64 tot[kNumCounters];
      block_scan5(x, tot, s_warp);
      s_cnt[threadIdx.x] = r;
      s_off[threadIdx.x] = {(u32)(pre[kCntParts] + x[kCntParts]), (u32)(pre[kCntSplits] + x[kCntSplits]),
                            (u32)(pre[kCntGen] + x[kCntGen]), (u32)(pre[kCntVerts] + x[kCntVerts]),
                            pre[kCntData] + x[kCntData]};
#pragma unroll
      for(int q = 0; q < kNumCounters; q++)
        pre[q] += tot[q];
    }
    __syncthreads();
    // each warp takes a contiguous part of the chunk (instance-sorted), so its
    // full-cluster BLAS reference counts collapse into one atomic per instance
    // it touches and its full clusters' vertices are contiguous
    const u32 perW = (len + kWarps - 1) / kWarps;
    const u32 lo = min(len, warp * perW), hi = min(len, lo + perW);

    // ---- phase 1: part and split triangles, one cluster at a time -------------
    for(u32 i = lo; i < hi; i++)
    {
      const uint2 cnt = s_cnt[i];
      if(cnt_full(cnt))
        continue;  // phase 2 (no part or split triangles)
      const u32 v = c0 + i, offPart = s_off[i].part, offSplit = s_off[i].split;
      const tc_ClusterInfo ci = s_ci[i];
      {
        // cluster_classify.comp.glsl:543-666: part and split triangles
        const u32  nt  = cnt_parts(cnt) + cnt_splits(cnt);
        const u32* tw  = cs.triWords + (u64)v * TC_MAX_CLUSTER_TRIANGLES;
        const u32  w0  = lane < nt ? tw[lane] : 0u;
        const u32  w1  = lane + 32 < nt ? tw[lane + 32] : 0u;
        const bool s0  = lane < nt && (w0 >> 18) != 0, p0 = lane < nt && (w0 >> 18) == 0;
        const bool s1  = lane + 32 < nt && (w1 >> 18) != 0, p1 = lane + 32 < nt && (w1 >> 18) == 0;
        const u32  bs0 = __ballot_sync(0xFFFFFFFFu, s0), bp0 = __ballot_sync(0xFFFFFFFFu, p0);
        const u32  bs1 = __ballot_sync(0xFFFFFFFFu, s1), bp1 = __ballot_sync(0xFFFFFFFFu, p1);
        // split items also carry their base triangle's world positions (read by
        // every split pass instead of the instance / cluster / vertex chain)
        const tc_RenderInstance* in  = nullptr;
        tc_Cluster               cl  = {};
        float                    m[16];
        if(bs0 | bs1)
        {
          in = c.instances + ci.instanceID;
          cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[ci.clusterID];
#pragma unroll
          for(int j = 0; j < 16; j++)
            m[j] = __ldg(in->worldMatrix.m + j);
        }
        auto split_base = [&](u64 o, u32 tri) {
          if(!c.splitBase)
            return;
          const uint8_t* lt  = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
          const float*   pos = reinterpret_cast<const float*>(in->positions);
          float*         d   = c.splitBase + 9 * o;
#pragma unroll
          for(int vv = 0; vv < 3; vv++)
          {
            const f3 wp = xform_point(m, ldg3(pos, cl.firstLocalVertex + lt[tri * 3 + vv]));
            d[3 * vv + 0] = wp.x, d[3 * vv + 1] = wp.y, d[3 * vv + 2] = wp.z;
          }
        };
        if(s0)
        {
          const u64 o = (u64)offSplit + __popc(bs0 & ltm);
          if(o < k.maxSplitTriangles)
          {
            emit_triangle(splits + o, ci, lane, w0);
            split_base(o, lane);
          }
        }
        else if(p0)
        {
          const u64 o = (u64)offPart + __popc(bp0 & ltm);
          if(o < k.maxPartTriangles)
            emit_triangle(parts + o, ci, lane, w0);
        }
        if(s1)
        {
          const u64 o = (u64)offSplit + __popc(bs0) + __popc(bs1 & ltm);
          if(o < k.maxSplitTriangles)
          {
            emit_triangle(splits + o, ci, lane + 32, w1);
            split_base(o, lane + 32);
          }
        }
        else if(p1)
        {
          const u64 o = (u64)offPart + __popc(bp0) + __popc(bp1 & ltm);
          if(o < k.maxPartTriangles)
            emit_triangle(parts + o, ci, lane + 32, w1);
        }
      }
    }

    // ---- phase 2: full clusters of the warp's part, 32 at a time ---------------
    // cluster_classify.comp.glsl:271-488: instantiation arguments, one lane per
    // cluster (the instance loads of 32 clusters overlap). The displaced
    // vertices (:457-482) are written by k_classify_full_vertices from the
    // records left here.
    for(u32 i0 = lo; i0 < hi; i0 += 32)
    {
      const u32 i    = i0 + lane;
      bool      full = false;
      u32       inst = 0xFFFFFFFFu;
      if(i < hi)
      {
        const uint2 r = s_cnt[i];
        if(cnt_full(r))
        {
          const ClusterOffsets off = s_off[i];
          const u32            v   = c0 + i;
          full = !((u64)off.vert + cnt_verts(r) > k.maxGeneratedVertices || (u64)off.gen + 1 > k.maxGeneratedClusters
                   || off.data + r.y > maxData);
          cs.fullRecs[off.gen - genBase] = full ? make_uint2(begin + v, off.vert) : make_uint2(kRejected, 0u);
          if(full)
          {
            const tc_ClusterInfo     ci = s_ci[i];
            const tc_RenderInstance* in = c.instances + ci.instanceID;
            // accepted instantiations form a prefix of the serial order, so the
            // instantiation slot equals the generated-cluster slot
            const u32                  tempOffset = off.gen;
            tc_TemplateInstantiateInfo ti;
            ti.clusterIdOffset        = 0;
            ti.geometryIndexOffset    = 0;
            ti.clusterTemplateAddress = __ldg(reinterpret_cast<const u64*>(in->clusterTemplateAdresses) + ci.clusterID);
            ti.vertexBufferAddress    = b->genVertices + (u64)off.vert * 12ull;
            ti.vertexBufferStride     = 12;
            reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations)[tempOffset] = ti;
            reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]                          = ci.instanceID;
            reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset]                     = b->genClusterData + off.data;
            if((c.flags & TC_FLAG_WRITE_FULLCLUSTERS) && b->fullClusters)
              reinterpret_cast<tc_ClusterInfo*>(b->fullClusters)[tempOffset] = ci;
            statTemp += 1;
            statTris += cnt_tris(r);
            inst = ci.instanceID;
          }
        }
      }
      const u32 fm = __ballot_sync(0xFFFFFFFFu, full);
      // CLAS reference counts: one atomic per distinct instance of the batch
      for(u32 remaining = fm; remaining;)
      {
        const int src = __ffs(remaining) - 1;
        const u32 gk  = __shfl_sync(0xFFFFFFFFu, inst, src);
        const u32 sel = __ballot_sync(0xFFFFFFFFu, full && inst == gk);
        remaining &= ~sel;
        if((int)lane == src)
          atomicAdd(&blas[gk].clusterReferencesCount, __popc(sel));
      }
    }
    __syncthreads();  // s_off / s_cnt are rewritten by the next chunk
  }

  // statistics: one atomic each per warp
#pragma unroll
  for(int o = 16; o > 0; o >>= 1)
  {
    statTemp += __shfl_xor_sync(0xFFFFFFFFu, statTemp, o);
    statTris += __shfl_xor_sync(0xFFFFFFFFu, statTris, o);
  }
  if(lane == 0)
  {
    if(statTemp)
      atomicAdd(&b->tempInstantiateCounter, statTemp);
    if(statTris)
      atomicAdd(&c.readback->numTotalTriangles, statTris);
  }

  // the last block's running offsets are the totals; no block reads the
  // counters after count took their values
  if(blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
  {
    cs.fullRange[0] = genBase;
    cs.fullRange[1] = (u32)pre[kCntGen];
    if(n)
    {
      const ClusterOffsets b0  = *cs.bases;
      b->partTriangleCounter   = (u32)pre[kCntParts];
      b->splitTriangleCounter  = (int32_t)(u32)pre[kCntSplits];
      b->genClusterCounter     = (u32)pre[kCntGen];
      b->genVertexCounter      = (u32)pre[kCntVerts];
      b->genClusterDataCounter = pre[kCntData];
      // cluster_classify.comp.glsl:299 counts every full cluster, accepted or not
      c.readback->numFullClusters += (u32)pre[kCntGen] - b0.gen;
    }
    if(c.fuseSetup != kNoSetup)
      build_setup_apply(c, c.fuseSetup);
  }
}

// ---------------------------------------------------------------------------
// write, with transient builds
// ---------------------------------------------------------------------------

enum : int
{
  kTFront = 0,
  kTSplit,
  kTGen,
  kTVert,
  kTData,
  kTBack,
  kTTrans,
  kTNum
};

// a cluster's offsets into every counter (exclusive, in the canonical order)
struct TransOffsets
{
  u32 front, split, gen, vert, back, trans;
  u64 data;
};

// build.glsl:52-66: slots from the back of partTriangles; maxPartTriangles
// when the two ends would meet (the counter advances either way)
__device__ __forceinline__ u32 back_alloc(u32 x, u32& y, u32 m, u32 maxParts)
{
  const u32 off = ((u64)x + y + m + 1 > maxParts) ? maxParts : maxParts - y - m;
  y += m;
  return off;
}

// cluster_classify.comp.glsl:401-431 / 751-786
__device__ __forceinline__ void store_clas_build(tc_ClasBuildInfo* dst, u32 mode, u32 partOffset, u32 numTriangles,
                                                 u32 numVertices, u32 truncateBits, u64 vertexBuffer)
{
  uint4* d = reinterpret_cast<uint4*>(dst);
  d[0]     = make_uint4((mode << 30) | partOffset, 0u, numTriangles | (numVertices << 9) | (truncateBits << 18) | (1u << 24),
                        4u << 29);
  d[1]     = make_uint4(1u | (12u << 16), 0u, (u32)(vertexBuffer + (u64)numVertices * 12), (u32)((vertexBuffer + (u64)numVertices * 12) >> 32));
  d[2]     = make_uint4((u32)vertexBuffer, (u32)(vertexBuffer >> 32), 0u, 0u);
  d[3]     = make_uint4(0u, 0u, 0u, 0u);
}

// cluster_classify.comp.glsl:810-878: one base triangle of a 2X batch (its
// word's config and corner rotation): its 3 to 6 vertices at its batch slot
__device__ inline void mini_vertices(const StageCtx& c, const tc_RenderInstance* in, const tc_Cluster& cl, u32 inst,
                                     u32 tri, u32 word, u32 rel, u32 vertexOffset, const RippleParams& rp)
{
  tc_SceneBuilding* b   = c.build;
  const u32         cfg = word & 0xFFFFu;
  const tc_TessTableEntry e = table_entry(c.table, cfg);
  u32               enc[3] = {0u, TC_TESSTABLE_COORD_MAX, TC_TESSTABLE_COORD_MAX << 16};
  const u32         rot    = (word >> 16) & 3;
  if(rot == 1)
  {
    const u32 t0 = enc[0];
    enc[0] = enc[1], enc[1] = enc[2], enc[2] = t0;
  }
  else if(rot == 2)
  {
    const u32 t2 = enc[2];
    enc[2] = enc[1], enc[1] = enc[0], enc[0] = t2;
  }
  const uint8_t* lt = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
  f3             bp[3], bn[3], bb[3];
  f2             bt[3];
  for(int q = 0; q < 3; q++)
  {
    const u32 vi = cl.firstLocalVertex + lt[tri * 3 + q];
    bp[q]        = ldg3(reinterpret_cast<const float*>(in->positions), vi);
    bn[q]        = normalize3(ldg3(reinterpret_cast<const float*>(in->normals), vi));
    bt[q]        = ldg2(reinterpret_cast<const float*>(in->texcoords), vi);
    bb[q]        = decode_bary(enc[q]);
  }
  tc_DisplacementTexture tx    = {};
  bool                   hasTx = false;
  if(c.numTextures > 0 && c.textures != nullptr && in->displacementIndex >= 0)
  {
    if((u32)in->displacementIndex < c.numTextures)
    {
      tx    = c.textures[in->displacementIndex];
      hasTx = true;
    }
    else
      atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
  }
  const bool pn    = (c.flags & TC_FLAG_PN) != 0;
  BasePN     basis = {};
  if(pn)
    basis = setup_pn(bp[0], bp[1], bp[2], bn[0], bn[1], bn[2]);
  float* gv = reinterpret_cast<float*>(b->genVertices);
  for(u32 vert = 0; vert < e.numVertices; vert++)
  {
    const f3 w   = interp3(bb[0], bb[1], bb[2], cfg_vertex(c.table, e, cfg, vert));
    f3       pos = pn ? get_pn(basis, w) : interp3(bp[0], bp[1], bp[2], w);
    if(hasTx)
      pos = displace(pos, interp3(bn[0], bn[1], bn[2], w), sample_bilinear(tx, interp2(bt[0], bt[1], bt[2], w)),
                     in->displacementScale, c.view->displacementScale, in->displacementOffset, c.view->displacementOffset);
    if(rp.enabled)
      pos = ripple(pos, inst, in->geoHi.w, rp);
    float* d = gv + 3 * ((u64)vertexOffset + rel * TC_2X_MINI_VERTICES + vert);
    d[0] = pos.x, d[1] = pos.y, d[2] = pos.z;
  }
}

// the same base triangle's u16 map entries and u8 indices (:880-903)
__device__ inline void mini_indices(const StageCtx& c, u32 tri, u32 word, u32 rel, u32 baseTris, u32 vertexOffset,
                                    u32 partOffset)
{
  tc_SceneBuilding*       b   = c.build;
  const u32               cfg = word & 0xFFFFu;
  const tc_TessTableEntry e   = table_entry(c.table, cfg);
  const u32 pf  = (word >> kWordFactorShift) & 7;
  uint8_t*  idx = reinterpret_cast<uint8_t*>(b->genVertices) + ((u64)vertexOffset + kMiniBatchVerts) * 12;
  uint16_t* map = reinterpret_cast<uint16_t*>(reinterpret_cast<uint8_t*>(b->partTriangles) + (u64)partOffset * kTessInfoBytes
                                              + kClusterInfoBytes);
  for(u32 i = 0; i < e.numTriangles; i++)
  {
    const uint3 ct        = cfg_triangle(c.table, e, cfg, i);
    const u32   triOffset = baseTris + i;
    map[triOffset]        = (uint16_t)(tri | (i << 8) | (pf << 12));
    idx[triOffset * 3 + 0] = (uint8_t)(ct.x + rel * TC_2X_MINI_VERTICES);
    idx[triOffset * 3 + 1] = (uint8_t)(ct.y + rel * TC_2X_MINI_VERTICES);
    idx[triOffset * 3 + 2] = (uint8_t)(ct.z + rel * TC_2X_MINI_VERTICES);
  }
}

// the warp zeroes `words` 32-bit words at p (4-byte aligned)
__device__ __forceinline__ void warp_zero(void* p, u32 words)
{
  u32* w = reinterpret_cast<u32*>(p);
  for(u32 i = threadIdx.x & 31; i < words; i += 32)
    w[i] = 0u;
}

// cluster_classify.comp.glsl:254-905 with transient builds, for one cluster,
// by one warp, in the canonical order: the full-cluster or 1X allocation, then
// per 32-triangle chunk its parts and splits followed by its 2X batches.
// Offsets come from the block scan; every allocation is tested like the
// reference's (the counters advance whether or not it fits). Bytes the
// reference leaves unwritten inside an allocation are written as zeros.
__device__ inline void write_cluster_transient(const StageCtx& c, const ClassifyScratch& cs, u32 visIndex, u32 v,
                                               const tc_ClusterInfo& ci, uint4 r, TransOffsets o, u32 genBase,
                                               const TransBases& tb, u32& statTemp, u32& statTrans, u32& statTris)
{
  const u32         lane = threadIdx.x & 31, ltm = (1u << lane) - 1u;
  tc_SceneBuilding* b    = c.build;
  const tc_caps&    k    = c.caps;
  const u64         maxData = (u64)k.maxGeneratedClusterMegs * 1024ull * 1024ull;
  const u32*        basic   = reinterpret_cast<const u32*>(b->basicClusterSizes);
  tc_BlasBuildInfo* blas    = reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos);
  const u32         nt = t_nt(r), nv = t_nv(r), simple = t_simple(r);
  const bool        full = t_full(r), subset = t_subset(r);
  const tc_RenderInstance* in = c.instances + ci.instanceID;
  const tc_Cluster         cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[ci.clusterID];
  u32 x = o.front, y = o.back, s = o.split, g = o.gen, vo = o.vert, tr = o.trans;
  u64 d = o.data;
  auto fits = [&](u32 vertexSize, u64 dataSize, u32 partOffset, u32 partSize) {
    return !((u64)vo + vertexSize > k.maxGeneratedVertices || (u64)g + 1 > k.maxGeneratedClusters
             || d + dataSize > maxData || (u64)partOffset + partSize > k.maxPartTriangles);
  };
  uint8_t* gvb = reinterpret_cast<uint8_t*>(b->genVertices);
  uint8_t* ptb = reinterpret_cast<uint8_t*>(b->partTriangles);

  // ---- :254-437 full cluster or 1X subset ----------------------------------------
  if(full || subset)
  {
    const u32 vertexSize = full ? nv : subset_vertex_size(nv, simple);
    const u64 dataSize   = full ? (u64)__ldg(reinterpret_cast<const u32*>(in->clusterTemplateInstantiatonSizes) + ci.clusterID)
                                : (u64)basic[simple];
    const u32 partSize   = full ? 0u : subset_part_slots(simple);
    const u32 partOffset = full ? 0u : back_alloc(x, y, partSize, k.maxPartTriangles);
    const bool ok        = fits(vertexSize, dataSize, partOffset, partSize);
    if(lane == 0)  // the vertex walk's record, per visible cluster with transient builds
      cs.fullRecs[v] = ok ? make_uint2(visIndex, vo) : make_uint2(kRejected, 0u);
    if(ok)
    {
      if(lane == 0)
      {
        if(full)
        {
          const u32                  tempOffset = tb.temp + (g - genBase) - (tr - tb.trans);
          tc_TemplateInstantiateInfo ti;
          ti.clusterIdOffset        = 0;
          ti.geometryIndexOffset    = 0;
          ti.clusterTemplateAddress = __ldg(reinterpret_cast<const u64*>(in->clusterTemplateAdresses) + ci.clusterID);
          ti.vertexBufferAddress    = b->genVertices + (u64)vo * 12ull;
          ti.vertexBufferStride     = 12;
          reinterpret_cast<tc_TemplateInstantiateInfo*>(b->tempInstantiations)[tempOffset] = ti;
          reinterpret_cast<u32*>(b->tempInstanceIDs)[tempOffset]                          = ci.instanceID;
          reinterpret_cast<u64*>(b->tempClusterAddresses)[tempOffset]                     = b->genClusterData + d;
          if((c.flags & TC_FLAG_WRITE_FULLCLUSTERS) && b->fullClusters)
            reinterpret_cast<tc_ClusterInfo*>(b->fullClusters)[tempOffset] = ci;
          statTemp += 1;
        }
        else
        {
          store_clas_build(reinterpret_cast<tc_ClasBuildInfo*>(b->transBuilds) + tr, TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER,
                           partOffset, simple, nv, b->positionTruncateBitCount, b->genVertices + (u64)vo * 12ull);
          reinterpret_cast<u32*>(b->transInstanceIDs)[tr]      = ci.instanceID;
          reinterpret_cast<u64*>(b->transClusterAddresses)[tr] = b->genClusterData + d;
          statTrans += 1;
        }
        statTris += simple;
        atomicAdd(&blas[ci.instanceID].clusterReferencesCount, 1u);
      }
      if(subset)
      {
        // :489-535 indices after the vertices, triangle map after the header
        uint8_t* idx = gvb + ((u64)vo + nv) * 12;
        uint8_t* map = ptb + (u64)partOffset * kTessInfoBytes;
        warp_zero(idx, (simple * 3 + 11) / 12 * 3);
        warp_zero(map, partSize * kTessInfoBytes / 4);
        __syncwarp();
        if(lane == 0)
          *reinterpret_cast<uint2*>(map) = make_uint2(ci.instanceID, ci.clusterID);
        const u32* tw = cs.triWords + (u64)v * TC_MAX_CLUSTER_TRIANGLES;
        const uint8_t* lt = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
        u32 out = 0;
        for(u32 t0 = 0; t0 < nt; t0 += 32)
        {
          const u32  tri = t0 + lane;
          const bool sub = tri < nt && (tw[tri] & kWordSubset);
          const u32  bm  = __ballot_sync(0xFFFFFFFFu, sub);
          if(sub)
          {
            const u32 q = out + __popc(bm & ltm);
            map[kClusterInfoBytes + q] = (uint8_t)tri;
            idx[q * 3 + 0]            = lt[tri * 3 + 0];
            idx[q * 3 + 1]            = lt[tri * 3 + 1];
            idx[q * 3 + 2]            = lt[tri * 3 + 2];
          }
          out += __popc(bm);
        }
      }
    }
    g += 1, vo += vertexSize, d += dataSize;
    if(subset)
      tr += 1;
  }
  else if(lane == 0)
    cs.fullRecs[v] = make_uint2(kRejected, 0u);
  u32 miniChunk[4] = {0u, 0u, 0u, 0u};  // per chunk: first batch vertex, accepted batches
  if(full)
  {
    if(lane == 0)
      reinterpret_cast<uint4*>(cs.counts)[v] = make_uint4(0u, 0u, 0u, 0u);
    return;
  }

  // ---- :543-905 the other triangles, one 32-triangle chunk at a time -------------
  const u32*   tw  = cs.triWords + (u64)v * TC_MAX_CLUSTER_TRIANGLES;
  tc_TessTriangleInfo* splits = reinterpret_cast<tc_TessTriangleInfo*>(b->splitTriangles);
  tc_TessTriangleInfo* parts  = reinterpret_cast<tc_TessTriangleInfo*>(b->partTriangles);
  for(u32 t0 = 0; t0 < nt; t0 += 32)
  {
    const u32  tri   = t0 + lane;
    const bool valid = tri < nt;
    const u32  word  = valid ? tw[tri] : 0u;
    const bool split = valid && (word & (1u << 18));
    const bool mini  = valid && (word & kWordMini);
    const bool part  = valid && !split && !mini && !(word & kWordSubset);
    const u32  bp = __ballot_sync(0xFFFFFFFFu, part), bs = __ballot_sync(0xFFFFFFFFu, split);
    const u32  bm = __ballot_sync(0xFFFFFFFFu, mini);
    // parts from the front of the two-sided counter: the chunk fits as a whole or not at all
    const u32  nPart   = __popc(bp);
    const bool frontOk = nPart != 0 && (u64)x + y + nPart + 1 <= k.maxPartTriangles;
    if(part && frontOk)
      emit_triangle(parts + x + __popc(bp & ltm), ci, tri, word);
    if(frontOk && lane == 0)  // the written front's end
      atomicMax(&b->partTriangleCounter, x + nPart);
    x += nPart;
    if(split)
    {
      const u64 so = (u64)s + __popc(bs & ltm);
      if(so < k.maxSplitTriangles)
      {
        emit_triangle(splits + so, ci, tri, word);
        if(c.splitBase)
        {
          const uint8_t* lt  = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
          const float*   pos = reinterpret_cast<const float*>(in->positions);
          float          m[16];
#pragma unroll
          for(int j = 0; j < 16; j++)
            m[j] = __ldg(in->worldMatrix.m + j);
          float* dd = c.splitBase + 9 * so;
#pragma unroll
          for(int vv = 0; vv < 3; vv++)
          {
            const f3 wp = xform_point(m, ldg3(pos, cl.firstLocalVertex + lt[tri * 3 + vv]));
            dd[3 * vv + 0] = wp.x, dd[3 * vv + 1] = wp.y, dd[3 * vv + 2] = wp.z;
          }
        }
      }
    }
    s += __popc(bs);
    // :675-790 the chunk's 2X batches, kMiniBatch triangles each, in triangle
    // order. Batch q's offsets follow from the chunk's (every batch takes the
    // same amounts), so all of them are set up and written at once: lane by
    // lane for the base triangles, the batch's first triangle for the build.
    const u32 nMini = __popc(bm);
    if(nMini)
    {
      const u32  nb       = (nMini + kMiniBatch - 1) / kMiniBatch;
      const u64  dataSize = (u64)basic[kMiniBatchTris];
      const u32  rank = __popc(bm & ltm), q = rank / kMiniBatch, rel = rank % kMiniBatch;
      // the lanes of this lane's batch, the sum of their table triangles and this one's start
      const u32  group   = __match_any_sync(0xFFFFFFFFu, mini ? q : 0xFFFFFFFFu);
      const u32  ntris   = mini ? (u32)table_entry(c.table, word & 0xFFFFu).numTriangles : 0u;
      const u32  incl    = warp_inclusive<u32>(ntris, lane);
      const u32  first   = __shfl_sync(0xFFFFFFFFu, incl - ntris, __ffs(group) - 1);
      const u32  last    = __shfl_sync(0xFFFFFFFFu, incl, 31 - __clz(group));
      auto       back_of = [&](u32 qq) {  // build.glsl:52-66 for batch qq of the chunk
        const u32 yq = y + kMiniPartSlots * qq;
        return ((u64)x + yq + kMiniPartSlots + 1 > k.maxPartTriangles) ? k.maxPartTriangles
                                                                        : k.maxPartTriangles - yq - kMiniPartSlots;
      };
      auto fits_q = [&](u32 qq) {
        const u32 po = back_of(qq);
        return !((u64)vo + kMiniVertexSize * (qq + 1) > k.maxGeneratedVertices
                 || (u64)g + qq + 1 > k.maxGeneratedClusters || d + dataSize * (qq + 1) > maxData
                 || (u64)po + kMiniPartSlots > k.maxPartTriangles);
      };
      for(u32 qq = 0; qq < nb; qq++)  // zero the accepted batches' regions
        if(fits_q(qq))
        {
          warp_zero(gvb + ((u64)vo + kMiniVertexSize * qq) * 12, kMiniVertexSize * 3);
          warp_zero(ptb + (u64)back_of(qq) * kTessInfoBytes, kMiniPartSlots * kTessInfoBytes / 4);
        }
      __syncwarp();
      if(mini && fits_q(q))
      {
        const u32 vq = vo + kMiniVertexSize * q, po = back_of(q);
        if(rel == 0)
        {
          const u32 trq = tr + q;
          store_clas_build(reinterpret_cast<tc_ClasBuildInfo*>(b->transBuilds) + trq,
                           TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED, po, last - first, kMiniBatchVerts,
                           b->positionTruncateBitCount, b->genVertices + (u64)vq * 12ull);
          reinterpret_cast<u32*>(b->transInstanceIDs)[trq]      = ci.instanceID;
          reinterpret_cast<u64*>(b->transClusterAddresses)[trq] = b->genClusterData + d + dataSize * q;
          *reinterpret_cast<uint2*>(ptb + (u64)po * kTessInfoBytes) = make_uint2(ci.instanceID, ci.clusterID);
          atomicAdd(&blas[ci.instanceID].clusterReferencesCount, 1u);
          statTrans += 1;
          statTris += last - first;
        }
        mini_indices(c, tri, word, rel, incl - ntris - first, vq, po);
      }
      // for k_classify_mini_vertices: the chunk's first batch vertex and its accepted batches
      u32 okMask = 0;
      for(u32 qq = 0; qq < nb; qq++)
        okMask |= fits_q(qq) ? 1u << qq : 0u;
      if(lane == 0)
      {
        miniChunk[2 * (t0 >> 5)]     = vo;
        miniChunk[2 * (t0 >> 5) + 1] = okMask;
      }
      __syncwarp();
      g += nb, vo += kMiniVertexSize * nb, d += dataSize * nb, tr += nb, y += kMiniPartSlots * nb;
    }
  }
  if(lane == 0)  // (counts of this cluster were read into shared memory before)
    reinterpret_cast<uint4*>(cs.counts)[v] = make_uint4(miniChunk[0], miniChunk[1], miniChunk[2], miniChunk[3]);
}

// The offsets at which block `blockIdx.x` of the write launch starts, with
// transient builds (the seven counters of TransOffsets).
__device__ inline void block_prefix_transient(const ClassifyScratch& cs, u64 (&pre)[kTNum], u64 (*s_warp)[kTNum])
{
  u64 x[kTNum] = {0, 0, 0, 0, 0, 0, 0};
  for(u32 i = threadIdx.x; i < blockIdx.x; i += blockDim.x)
  {
    const RangeSums o = cs.rangeSums[i];
    x[kTFront] += (u32)o.partsSplits;
    x[kTSplit] += (u32)(o.partsSplits >> 32);
    x[kTGen] += (u32)o.fullVerts;
    x[kTVert] += (u32)(o.fullVerts >> 32);
    x[kTData] += o.data;
    x[kTBack] += (u32)o.backTrans;
    x[kTTrans] += (u32)(o.backTrans >> 32);
  }
  u64 tot[kTNum];
  block_scan_n<kTNum>(x, tot, s_warp);
  const ClusterOffsets b0 = *cs.bases;
  const TransBases     t0 = *reinterpret_cast<const TransBases*>(cs.bases + 1);
  pre[kTFront] = b0.part + tot[kTFront];
  pre[kTSplit] = b0.split + tot[kTSplit];
  pre[kTGen]   = b0.gen + tot[kTGen];
  pre[kTVert]  = b0.vert + tot[kTVert];
  pre[kTData]  = b0.data + tot[kTData];
  pre[kTBack]  = t0.back + tot[kTBack];
  pre[kTTrans] = t0.trans + tot[kTTrans];
}

__global__ void __launch_bounds__(kBlock, 6) k_classify_write_transient(StageCtx c, ClassifyScratch cs)
{
  stage_prologue();
  __shared__ u32            s_range[2];
  __shared__ u64            s_warp[33][kTNum];
  __shared__ TransOffsets   s_off[kBlock];
  __shared__ uint4          s_cnt[kBlock];
  __shared__ tc_ClusterInfo s_ci[kBlock];
  __shared__ FlatStarts     s_starts;
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0)
    window_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32* starts = stage_flat_starts(c, s_starts);
  const u32  begin  = s_range[0];
  const u32  n      = min(s_range[1] - s_range[0], c.scratch.itemCapacity);
  tc_SceneBuilding*     b   = c.build;
  const tc_ClusterInfo* vis = reinterpret_cast<const tc_ClusterInfo*>(b->visibleClusters);
  const uint4*          counts = reinterpret_cast<const uint4*>(cs.counts);
  u32                   statTemp = 0, statTrans = 0, statTris = 0;

  u64 pre[kTNum];
  block_prefix_transient(cs, pre, s_warp);
  const u32        genBase = cs.bases->gen;
  const TransBases tb      = *reinterpret_cast<const TransBases*>(cs.bases + 1);
  u32              vBegin, vEnd;
  block_range(n, blockIdx.x, gridDim.x, vBegin, vEnd);
  for(u32 c0 = vBegin; c0 < vEnd; c0 += kBlock)
  {
    const u32 len = min(kBlock, vEnd - c0);
    {
      const uint4 r = threadIdx.x < len ? counts[c0 + threadIdx.x] : make_uint4(0, 0, 0, 0);
      if(threadIdx.x < len)
        s_ci[threadIdx.x] = visible_cluster(c, starts, vis, begin + c0 + threadIdx.x);
      u64 x[kTNum] = {t_parts(r), t_splits(r), t_gen(r), t_verts(r), r.z, t_back(r), t_trans(r)};
      u64 tot[kTNum];
      block_scan_n<kTNum>(x, tot, s_warp);
      s_cnt[threadIdx.x] = r;
      s_off[threadIdx.x] = {(u32)(pre[kTFront] + x[kTFront]), (u32)(pre[kTSplit] + x[kTSplit]),
                            (u32)(pre[kTGen] + x[kTGen]),     (u32)(pre[kTVert] + x[kTVert]),
                            (u32)(pre[kTBack] + x[kTBack]),   (u32)(pre[kTTrans] + x[kTTrans]),
                            pre[kTData] + x[kTData]};
#pragma unroll
      for(int q = 0; q < kTNum; q++)
        pre[q] += tot[q];
    }
    __syncthreads();
    const u32 perW = (len + kWarps - 1) / kWarps;
    const u32 lo = min(len, warp * perW), hi = min(len, lo + perW);
    for(u32 i = lo; i < hi; i++)
      write_cluster_transient(c, cs, begin + c0 + i, c0 + i, s_ci[i], s_cnt[i], s_off[i], genBase, tb, statTemp,
                              statTrans, statTris);
    __syncthreads();
  }
  statTemp  = __reduce_add_sync(0xFFFFFFFFu, statTemp);
  statTrans = __reduce_add_sync(0xFFFFFFFFu, statTrans);
  statTris  = __reduce_add_sync(0xFFFFFFFFu, statTris);
  if(lane == 0)
  {
    if(statTemp)
      atomicAdd(&b->tempInstantiateCounter, statTemp);
    if(statTrans)
      atomicAdd(&b->transBuildCounter, statTrans);
    if(statTris)
      atomicAdd(&c.readback->numTotalTriangles, statTris);
  }
  if(blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
  {
    cs.fullRange[0] = 0;  // the walk's records are per visible cluster here
    cs.fullRange[1] = n;
    if(n)
    {
      const ClusterOffsets b0 = *cs.bases;
      b->dualPartTriangleCounter = (u64)(u32)pre[kTFront] | ((u64)(u32)pre[kTBack] << 32);
      b->splitTriangleCounter    = (int32_t)(u32)pre[kTSplit];
      b->genClusterCounter       = (u32)pre[kTGen];
      b->genVertexCounter        = (u32)pre[kTVert];
      b->genClusterDataCounter   = pre[kTData];
      // :299 counts every full-cluster attempt; the full attempts also bound
      // the full clusters' run of the instantiation list
      const u32 fullAttempts = ((u32)pre[kTGen] - b0.gen) - ((u32)pre[kTTrans] - tb.trans);
      c.readback->numFullClusters += fullAttempts;
      c.runStarts[kFullAttemptsSlot] += fullAttempts;
    }
    if(c.fuseSetup != kNoSetup)
      build_setup_apply(c, c.fuseSetup);
  }
}

// cluster_classify.comp.glsl:810-878: the vertices of the accepted 2X
// batches, from what k_classify_write_transient left per cluster (each
// chunk's first batch vertex and accepted batches, in place of its counts).
// One warp per cluster, one lane per base triangle.
__global__ void __launch_bounds__(kBlock, 2) k_classify_mini_vertices(StageCtx c, ClassifyScratch cs)
{
  stage_prologue();
  __shared__ u32        s_range[2];
  __shared__ FlatStarts s_starts;
  if(threadIdx.x == 0)
    window_range(c, s_range[0], s_range[1]);
  __syncthreads();
  const u32*            starts = stage_flat_starts(c, s_starts);
  const u32             lane = threadIdx.x & 31, ltm = (1u << lane) - 1u;
  const u32             begin = s_range[0];
  const u32             n     = min(s_range[1] - s_range[0], c.scratch.itemCapacity);
  const tc_ClusterInfo* vis   = reinterpret_cast<const tc_ClusterInfo*>(c.build->visibleClusters);
  const RippleParams    rp    = ripple_params(*c.view, (c.flags & TC_FLAG_RIPPLE) != 0);
  const u32             nwarps = (gridDim.x * blockDim.x) >> 5;
  for(u32 v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nwarps)
  {
    const uint4 m = reinterpret_cast<const uint4*>(cs.counts)[v];
    if((m.y | m.w) == 0)
      continue;
    const tc_ClusterInfo     ci = visible_cluster(c, starts, vis, begin + v);
    const tc_RenderInstance* in = c.instances + ci.instanceID;
    const tc_Cluster         cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[ci.clusterID];
    const u32                nt = min((u32)cl.numTriangles, TC_MAX_CLUSTER_TRIANGLES);
    const u32*               tw = cs.triWords + (u64)v * TC_MAX_CLUSTER_TRIANGLES;
    for(u32 q = 0; q < 2; q++)
    {
      const u32 ok = q ? m.w : m.y, vo = q ? m.z : m.x;
      if(ok == 0)
        continue;
      const u32  tri  = 32 * q + lane;
      const u32  word = tri < nt ? tw[tri] : 0u;
      const bool mini = tri < nt && (word & kWordMini);
      const u32  rank = __popc(__ballot_sync(0xFFFFFFFFu, mini) & ltm);
      const u32  qb   = rank / kMiniBatch;
      if(mini && ((ok >> qb) & 1u))
        mini_vertices(c, in, cl, ci.instanceID, tri, word, rank % kMiniBatch, vo + kMiniVertexSize * qb, rp);
    }
  }
}

// cluster_classify.comp.glsl:457-482: the displaced vertices of the full
// clusters the write launch accepted. A warp takes `per` <= 32 consecutive
// generated-cluster slots (per: the slots spread over all of the grid's
// warps): one lane per cluster sets up its record, then the clusters' vertex
// ranges, contiguous in genVertices, are walked on consecutive lanes. Its own
// launch so that it can overlap other work.
template <int MinBlocks>
__global__ void __launch_bounds__(kBlock, MinBlocks) k_classify_full_vertices(StageCtx c, ClassifyScratch cs)
{
  stage_prologue();
  __shared__ FullRecord s_full[kWarps][32];
  __shared__ FlatStarts s_starts;
  const u32*            starts = stage_flat_starts(c, s_starts);
  const u32             lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32             ltm  = (1u << lane) - 1u;
  const u32             count        = cs.fullRange[1] - cs.fullRange[0];
  const u32             totalWarps   = gridDim.x * kWarps;
  const u32             per          = min(32u, max(1u, (count + totalWarps - 1) / totalWarps));
  const u32             numChunks    = (count + per - 1) / per;
  const tc_SceneBuilding* b          = c.build;
  const tc_ClusterInfo* vis          = reinterpret_cast<const tc_ClusterInfo*>(b->visibleClusters);
  const bool            haveTextures = c.numTextures > 0 && c.textures != nullptr;
  float*                gv           = reinterpret_cast<float*>(b->genVertices);
  FullRecord*           rec          = s_full[warp];
  const RippleParams    rp           = ripple_params(*c.view, (c.flags & TC_FLAG_RIPPLE) != 0);

  for(u32 chunk = blockIdx.x * kWarps + warp; chunk < numChunks; chunk += totalWarps)
  {
    const u32  slot  = chunk * per + lane;
    bool       owner = false;
    FullRecord fr;
    if(lane < per && slot < count)
    {
      const uint2 fs = cs.fullRecs[slot];
      if(fs.x != kRejected)
      {
        const tc_ClusterInfo     ci = visible_cluster(c, starts, vis, fs.x);
        const tc_RenderInstance* in = c.instances + ci.instanceID;
        const tc_Cluster         cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[ci.clusterID];
        owner                       = true;
        fr.vo                       = fs.y;
        fr.nv                       = min((u32)cl.numVertices, TC_MAX_CLUSTER_VERTICES);
        fr.pos                      = reinterpret_cast<const float*>(in->positions);
        fr.nrm                      = reinterpret_cast<const float*>(in->normals);
        fr.uvs                      = reinterpret_cast<const float*>(in->texcoords);
        fr.first                    = cl.firstLocalVertex;
        tc_DisplacementTexture tx   = {};
        if(haveTextures && in->displacementIndex >= 0)
        {
          if((u32)in->displacementIndex < c.numTextures)
            tx = c.textures[in->displacementIndex];
          else
            atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
        }
        fr.map    = make_map_desc(tx);
        fr.scale  = in->displacementScale * c.view->displacementScale;
        fr.offset = in->displacementOffset + c.view->displacementOffset;
        fr.inst   = ci.instanceID;
        fr.size   = in->geoHi.w;
      }
    }
    // the owners' records in slot order (their vertex ranges follow each
    // other, with gaps only where transient builds placed other data)
    const u32 fm = __ballot_sync(0xFFFFFFFFu, owner);
    if(fm == 0)
      continue;
    if(owner)
      rec[__popc(fm & ltm)] = fr;
    __syncwarp();
    // per record (lane r < nrec): first vertex within the batch and vertex count
    const u32  nrec   = __popc(fm);
    const u32  vBase  = rec[0].vo;
    const u32  rStart = lane < nrec ? rec[lane].vo - vBase : 0u;
    const u32  rCount = lane < nrec ? rec[lane].nv : 0u;
    const u32  rEnd   = __shfl_sync(0xFFFFFFFFu, rStart + rCount, nrec - 1);
    const bool own    = lane < nrec;
    // one specialisation when the batch's clusters share a map kind
    const u32 kind  = own ? rec[lane].map.kind : 0u;
    const u32 kind0 = rec[0].map.kind;
    const u32 kw    = __all_sync(0xFFFFFFFFu, !own || kind == kind0) ? kind0 : ~0u;
    float*    dst   = gv + (u64)vBase * 3;
    // the usual batch: consecutive clusters of instances of one mesh and map
    const FullRecord u    = rec[0];
    const bool       same = !own
                      || (rec[lane].pos == u.pos && rec[lane].nrm == u.nrm && rec[lane].uvs == u.uvs
                          && rec[lane].map.kind == u.map.kind
                          && __float_as_uint(rec[lane].map.q7.x) == __float_as_uint(u.map.q7.x)
                          && __float_as_uint(rec[lane].map.q7.y) == __float_as_uint(u.map.q7.y)
                          && __float_as_uint(rec[lane].map.q7.z) == __float_as_uint(u.map.q7.z)
                          && __float_as_uint(rec[lane].map.q7.w) == __float_as_uint(u.map.q7.w)
                          && __float_as_uint(rec[lane].scale) == __float_as_uint(u.scale)
                          && __float_as_uint(rec[lane].offset) == __float_as_uint(u.offset)
                          && (!rp.enabled || (rec[lane].inst == u.inst && __float_as_uint(rec[lane].size) == __float_as_uint(u.size))));
    if(__all_sync(0xFFFFFFFFu, same))
    {
      // per record (lane r): vertex index of batch vertex jj is rOff + jj, for jj < rStop
      const u32 rOff  = own ? rec[lane].first - rStart : 0u;
      const u32 rStop = own ? rStart + rCount : 0u;
      switch(u.map.kind)
      {
        case affine_kind(TC_TEXEL_F32, true):
          full_steps_uniform<affine_kind(TC_TEXEL_F32, true)>(u, own, rStart, rOff, rStop, rEnd, dst, rp);
          break;
        case affine_kind(TC_TEXEL_F16, true):
          full_steps_uniform<affine_kind(TC_TEXEL_F16, true)>(u, own, rStart, rOff, rStop, rEnd, dst, rp);
          break;
        case kAffineFlat: full_steps_uniform<kAffineFlat>(u, own, rStart, rOff, rStop, rEnd, dst, rp); break;
        default: full_steps_uniform<~0u>(u, own, rStart, rOff, rStop, rEnd, dst, rp); break;
      }
    }
    else
      switch(kw)
      {
        case affine_kind(TC_TEXEL_F32, true):
          full_steps<affine_kind(TC_TEXEL_F32, true)>(rec, own, rStart, rEnd, dst, rp);
          break;
        case affine_kind(TC_TEXEL_F16, true):
          full_steps<affine_kind(TC_TEXEL_F16, true)>(rec, own, rStart, rEnd, dst, rp);
          break;
        case kAffineFlat: full_steps<kAffineFlat>(rec, own, rStart, rEnd, dst, rp); break;
        default: full_steps<~0u>(rec, own, rStart, rEnd, dst, rp); break;
      }
    __syncwarp();  // records are rewritten by the next batch
  }
}

}  // namespace

cudaError_t launch_cluster_classify(const StageCtx& c, const ClassifyBuffers& buf, u32 maxClusters, u32 numSMs,
                                    u32 warpBlocksPerSM, cudaStream_t s)
{
  // the write launch's blocks own contiguous ranges of clusters, whose count
  // sums the count launch accumulates (its warps stride over the whole list)
  const u32 grid = std::max(1u, std::min(classify_max_blocks(maxClusters), numSMs * std::max(1u, warpBlocksPerSM)));
  ClassifyScratch cs{buf.counts, buf.triWords, buf.rangeSums, buf.bases, grid, 0, buf.fullRecs, buf.fullRange};
  // register budget from the requested residency: 4 or less -> 64, 5-7 -> 40, 8 and more -> 32
  if(c.flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
  {
    // the transient write is latency-bound per cluster: a full wave of its
    // six resident blocks per SM (the count uses the same ranges)
    const u32 tgrid = std::max(1u, std::min(classify_max_blocks(maxClusters), numSMs * std::max(6u, warpBlocksPerSM)));
    ClassifyScratch ts = cs;
    ts.writeBlocks     = tgrid;
    cudaError_t e      = launch_pdl_critical(k_classify_count<4, true>, tgrid, kBlock, s, c, ts);
    if(e != cudaSuccess)
      return e;
    return launch_pdl_critical(k_classify_write_transient, tgrid, kBlock, s, c, ts);
  }
  const int   occ = warpBlocksPerSM >= 8 ? 8 : (warpBlocksPerSM >= 5 ? 6 : 4);
  cudaError_t e   = occ == 8   ? launch_pdl_critical(k_classify_count<8>, grid, kBlock, s, c, cs)
                    : occ == 6 ? launch_pdl_critical(k_classify_count<6>, grid, kBlock, s, c, cs)
                               : launch_pdl_critical(k_classify_count<4>, grid, kBlock, s, c, cs);
  if(e != cudaSuccess)
    return e;
  return occ == 8   ? launch_pdl_critical(k_classify_write<8>, grid, kBlock, s, c, cs)
         : occ == 6 ? launch_pdl_critical(k_classify_write<6>, grid, kBlock, s, c, cs)
                    : launch_pdl_critical(k_classify_write<4>, grid, kBlock, s, c, cs);
}

cudaError_t launch_classify_full_vertices(const StageCtx& c, const ClassifyBuffers& buf, u32 maxClusters, u32 numSMs,
                                          u32 blocksPerSM, cudaStream_t s)
{
  ClassifyScratch cs{buf.counts, buf.triWords, buf.rangeSums, buf.bases, 0, 0, buf.fullRecs, buf.fullRange};
  // every warp of the grid takes a share of the slots
  const u32 grid = std::max(1u, std::min((maxClusters + kWarps - 1) / kWarps, numSMs * std::max(1u, blocksPerSM)));
  // register budget from the requested residency: 4 or less -> 64, 5-6 -> 40, 7 and more -> 32
  cudaError_t e = blocksPerSM >= 7   ? launch_pdl(k_classify_full_vertices<8>, grid, kBlock, s, c, cs)
                  : blocksPerSM >= 5 ? launch_pdl(k_classify_full_vertices<6>, grid, kBlock, s, c, cs)
                                     : launch_pdl(k_classify_full_vertices<4>, grid, kBlock, s, c, cs);
  if(e != cudaSuccess || !(c.flags & TC_FLAG_TRANSIENT_2X))
    return e;
  // the 2X batches' vertices (one warp per visible cluster of the window)
  const u32 miniGrid = std::max(1u, std::min((maxClusters + kWarps - 1) / kWarps, numSMs * 8));
  return launch_pdl(k_classify_mini_vertices, miniGrid, kBlock, s, c, cs);
}

u32 classify_max_blocks(u32 maxClusters) { return std::max(1u, (maxClusters + kWarps - 1) / kWarps); }

}  // namespace tc
