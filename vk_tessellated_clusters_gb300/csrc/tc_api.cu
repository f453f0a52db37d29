// tc_api.cu — the C ABI (include/tc_tessellation.h): context and scratch
// management, tessellation table upload, and the frame orchestrations
// (batched, CUDA-graph replay, per-instance launches).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "tc_kernels.h"
#include "tc_stage.cuh"

using namespace tc;

namespace {

constexpr u32 kMaxCounters = 5;

// One look-back slot: state rows for up to kMaxCounters counters, plus the
// ticket / done / totals words.
struct SlotPlan
{
  size_t stateOffset;  // bytes into the scratch block
  u32    stride;       // tiles
  u32    counters;
  size_t ctrlOffset;  // ticket, done (u32 x2) + totals (u64 x kMaxCounters)
};

constexpr size_t kCtrlBytes = 64;  // ticket, done, totals (u64 x kMaxCounters), then the split levels' words
static_assert(8 + 8 * kMaxCounters <= 48, "the split levels' control words start at byte 48");

// kernels of a batched frame besides the split launch (every pass in one): frame_begin,
// frame_begin + instances_classify (one launch), clusters_cull, classify (3),
// instantiate (4, twice: the first part run overlapped with the split passes,
// then the others), blas setup, blas insert (2)
constexpr uint64_t kFrameFixedLaunches = 16;

constexpr u32 kDefaultFullVertexBlocksPerSM = 4;

struct Plan
{
  // slot indices
  u32 slotInstances, slotCull, slotClassify, slotSplit0, slotInstantiate, slotInstantiate0, slotBlas;
  u32 numSlots;
  std::vector<SlotPlan> slots;
  size_t frameBytes;  // zeroed once per batched frame (all slots + segment tables)
  size_t segOffset;   // segment tables (segStart then segEnd)
  u32    segStride;   // instances
  u32    segRows;     // runs
  size_t runOffset;   // run starts (u32 x kMaxRuns+2)
  u32    classifyCap; // clusters the classify scratch holds
  size_t clsCountsOffset, clsTriWordsOffset, clsBlockSumsOffset, clsFullRecsOffset;
  size_t rasterOffset;
  size_t partVertexOffset;  // u32 per part triangle
  size_t chunkSumsOffset;   // u64 per 32 part triangles
  size_t splitBaseOffset;   // 9 floats per split item: its base triangle's world positions
  size_t instOffset;  // instance cluster prefix (u32 x maxInstances+1)
  size_t errOffset;   // device error word
  size_t totalBytes;
};

// A frame's host traffic inside its graph (tc_frame_build_graph_host): the
// device aliases of the pinned host buffers, the device input block.
struct HostIo
{
  const void* hostIn   = nullptr;  // device alias of the caller's input block
  void*       devIn    = nullptr;
  uint64_t    bytes    = 0;
  void*       hostRb   = nullptr;  // device alias of the caller's Readback buffer
  const void* callerIn = nullptr;  // the caller's addresses
  const void* callerRb = nullptr;
  bool        fused    = false;    // the upload runs inside the frame's first kernel (inputs_in_block)
  bool same_buffers(const HostIo& o) const
  {
    return callerIn == o.callerIn && devIn == o.devIn && bytes == o.bytes && callerRb == o.callerRb;
  }
  bool operator==(const HostIo& o) const
  {
    return same_buffers(o) && hostIn == o.hostIn && hostRb == o.hostRb && fused == o.fused;
  }
  uint64_t launches() const { return (bytes && !fused ? 1 : 0) + (hostRb ? 1 : 0); }
};

u32 ceil_div(u64 a, u64 b) { return (u32)((a + b - 1) / b); }

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct tc_context
{
  int             device   = 0;
  u32             numSMs   = 0;
  tc_context_desc desc     = {};
  tc_schedule     schedule = {};
  uint64_t        launches = 0;

  // tessellation table
  bool                  tableReady = false;
  u32*                  dVertices  = nullptr;
  u32*                  dTriangles = nullptr;
  tc_TessTableEntry*    dEntries   = nullptr;
  u64*                  dTemplateAddresses = nullptr;
  u32*                  dTemplateSizes     = nullptr;
  tc_TessellationTable* dTable             = nullptr;
  tc_TessellationTable  hTable             = {};

  // scratch
  Plan     plan;
  uint8_t* dScratch = nullptr;

  // second stream of the batched frame: the first part run's instantiation
  // overlaps the split passes (fork / join through the two events)
  cudaStream_t side    = nullptr;  // the first part run's instantiation
  cudaStream_t side2   = nullptr;  // the full clusters' vertices
  cudaEvent_t  evFork  = nullptr;
  cudaEvent_t  evJoin  = nullptr;  // first part run allocated
  cudaEvent_t  evJoin2 = nullptr;  // full clusters' vertices written
  cudaEvent_t  evArgs1 = nullptr;  // later part runs allocated
  cudaEvent_t  evVerts = nullptr;  // all part vertices written
  cudaEvent_t  evInst  = nullptr;  // instances classified
  cudaEvent_t  evScan0 = nullptr;  // first part run's offsets (and the counters after it)
  cudaEvent_t  evCull  = nullptr;  // clusters_cull done (on the second side stream)

  // graph cache
  cudaGraphExec_t graphExec = nullptr;
  cudaGraph_t     graph     = nullptr;
  tc_frame_args   graphArgs = {};
  tc_schedule     graphSchedule = {};
  HostIo          graphIo       = {};
  bool            graphValid = false;

  std::mutex mutex;
};

namespace {

#define TC_CHECK_CUDA(expr)                                                                                            \
  do                                                                                                                   \
  {                                                                                                                    \
    cudaError_t _e = (expr);                                                                                           \
    if(_e != cudaSuccess)                                                                                              \
      return TC_ERR_CUDA;                                                                                              \
  } while(0)

u32 clamp_sf(u32 sf) { return std::max(2u, std::min(sf, TC_TESSTABLE_SIZE)); }

u32 split_passes(u32 splitFactor)
{
  u32 sf = clamp_sf(splitFactor), n = 0, coord = TC_TESSTABLE_COORD_MAX;
  while(coord > sf)
  {
    coord /= sf;
    n++;
  }
  return n;
}

Plan make_plan(const tc_context_desc& d)
{
  Plan p;
  const tc_caps& k     = d.caps;
  const u32      passes = split_passes(2);  // worst case number of split passes
  auto add = [&](u32 stride, u32 counters) {
    SlotPlan s;
    s.stride   = std::max(1u, stride);
    s.counters = counters;
    p.slots.push_back(s);
    return (u32)p.slots.size() - 1;
  };
  p.slotInstances   = add(ceil_div(d.maxInstances, kInstanceTile), 1);
  p.slotCull        = add(ceil_div(d.maxTotalClusters, kCullTile), 1);
  p.classifyCap     = (u32)std::max<u64>(1, std::min<u64>(k.maxVisibleClusters, d.maxTotalClusters));
  p.slotClassify    = add(classify_max_blocks(p.classifyCap), 4);  // the range sums (zeroed with the frame)
  p.slotSplit0      = add(ceil_div(k.maxSplitTriangles, kSplitMinItems), 2);
  for(u32 i = 1; i < passes; i++)
    add(ceil_div(k.maxSplitTriangles, kSplitMinItems), 2);
  p.slotInstantiate = add(instantiate_alloc_tiles(k.maxPartTriangles), 3);
  p.slotInstantiate0 = add(instantiate_alloc_tiles(k.maxPartTriangles), 3);
  p.slotBlas        = add(ceil_div(d.maxInstances, kInstanceTile), 1);
  p.numSlots        = (u32)p.slots.size();
  size_t off        = 0;
  for(SlotPlan& s : p.slots)
  {
    s.stateOffset = off;
    off           = align_up(off + (size_t)s.stride * s.counters * 8, 256);
    s.ctrlOffset  = off;
    off           = align_up(off + kCtrlBytes, 256);
  }
  p.segStride = std::max(1u, d.maxInstances);
  p.segRows   = kMaxRuns + 2;  // the instantiation runs, then the transient builds
  p.segOffset = off;
  off         = align_up(off + (size_t)p.segStride * p.segRows * 4 * 2, 256);
  p.frameBytes = off;
  p.runOffset  = off;
  off          = align_up(off + 4 * kRunStartsSize, 256);
  p.instOffset = off;
  off          = align_up(off + 4 * ((size_t)d.maxInstances + 1), 256);
  p.errOffset  = off;
  off          = align_up(off + 4, 256);
  // per-item scratch (written before it is read every launch; never zeroed)
  p.clsCountsOffset   = off;
  off                 = align_up(off + (size_t)p.classifyCap * 16, 256);  // uint2, or uint4 with transient builds
  p.clsTriWordsOffset = off;
  off                 = align_up(off + (size_t)p.classifyCap * TC_MAX_CLUSTER_TRIANGLES * 4, 256);
  p.clsBlockSumsOffset = off;  // the counter bases
  off = align_up(off + sizeof(ClusterOffsets) + sizeof(TransBases), 256);
  p.clsFullRecsOffset = off;  // per full cluster, then the slot range
  off = align_up(off + (size_t)p.classifyCap * 8 + 8, 256);
  p.partVertexOffset  = off;
  off                 = align_up(off + (size_t)std::max(1u, k.maxPartTriangles) * 4, 256);
  p.chunkSumsOffset   = off;
  off                 = align_up(off + (size_t)ceil_div(std::max(1u, k.maxPartTriangles), 1024) * 32 * 8, 256);
  p.splitBaseOffset   = off;
  off                 = align_up(off + (size_t)std::max(1u, k.maxSplitTriangles) * 36, 256);
  p.rasterOffset      = off;  // raster batching: per group of 32 parts its counts, then offsets
  off                 = align_up(off + (size_t)ceil_div(std::max(1u, k.maxPartTriangles), 32) * 16, 256);
  p.totalBytes        = off;
  return p;
}

bool caps_fit(const tc_caps& want, const tc_caps& have)
{
  return want.maxVisibleClusters <= have.maxVisibleClusters && want.maxPartTriangles <= have.maxPartTriangles
         && want.maxSplitTriangles <= have.maxSplitTriangles;
}

tc_status validate(const tc_context* ctx, const tc_frame_args* a)
{
  if(!ctx || !a)
    return TC_ERR_INVALID_ARG;
  if(!ctx->tableReady)
    return TC_ERR_NOT_INITIALIZED;
  if(!a->view || !a->viewLast || !a->instances || !a->build || !a->readback)
    return TC_ERR_INVALID_ARG;
  if(a->numTextures && !a->textures)
    return TC_ERR_INVALID_ARG;
  if(a->numInstances > ctx->desc.maxInstances || a->totalClusters > ctx->desc.maxTotalClusters)
    return TC_ERR_CAPACITY;
  if(!caps_fit(a->caps, ctx->desc.caps))
    return TC_ERR_CAPACITY;
  if(a->caps.splitFactor < 2 || a->caps.splitFactor > TC_TESSTABLE_SIZE)
    return TC_ERR_INVALID_ARG;
  // transient builds are ray-tracing semantics (shaderio.h:140-141)
  if((a->flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)) && (a->flags & TC_FLAG_RASTER_CULL))
    return TC_ERR_INVALID_ARG;
  return TC_OK;
}

StageCtx base_ctx(tc_context* ctx, const tc_frame_args* a)
{
  StageCtx c;
  std::memset(&c, 0, sizeof(c));
  c.view                    = reinterpret_cast<const tc_FrameConstants*>(a->view);
  c.viewLast                = reinterpret_cast<const tc_FrameConstants*>(a->viewLast);
  c.instances               = reinterpret_cast<const tc_RenderInstance*>(a->instances);
  c.build                   = reinterpret_cast<tc_SceneBuilding*>(a->build);
  c.readback                = reinterpret_cast<tc_Readback*>(a->readback);
  c.textures                = reinterpret_cast<const tc_DisplacementTexture*>(a->textures);
  c.numInstances            = a->numInstances;
  c.numTextures             = a->numTextures;
  c.flags                   = a->flags;
  c.table.entries           = ctx->dEntries;
  c.table.vertices          = ctx->dVertices;
  c.table.triangles         = ctx->dTriangles;
  c.table.templateAddresses = ctx->dTemplateAddresses;
  c.table.templateSizes     = ctx->dTemplateSizes;
  c.caps                    = a->caps;
  c.errorWord               = reinterpret_cast<u32*>(ctx->dScratch + ctx->plan.errOffset);
  c.runStarts               = reinterpret_cast<u32*>(ctx->dScratch + ctx->plan.runOffset);
  c.instClusterStart        = reinterpret_cast<u32*>(ctx->dScratch + ctx->plan.instOffset);
  c.splitBase               = reinterpret_cast<float*>(ctx->dScratch + ctx->plan.splitBaseOffset);
  c.instBegin               = 0;
  c.instEnd                 = a->numInstances;
  c.fuseSetup               = kNoSetup;
  c.run                     = kAllRuns;
  c.spinLimit               = ctx->schedule.lookbackSpinLimit ? ctx->schedule.lookbackSpinLimit : kSpinLimit;
  return c;
}

void bind_slot(tc_context* ctx, StageCtx& c, u32 slot, bool selfClean)
{
  const SlotPlan& s   = ctx->plan.slots[slot];
  c.scratch.lbState   = reinterpret_cast<u64*>(ctx->dScratch + s.stateOffset);
  c.scratch.lbStride  = s.stride;
  c.scratch.selfClean = selfClean ? 1u : 0u;
  c.scratch.itemCapacity = slot == ctx->plan.slotClassify ? ctx->plan.classifyCap : 0xFFFFFFFFu;
  c.scratch.ticket    = reinterpret_cast<u32*>(ctx->dScratch + s.ctrlOffset);
  c.scratch.done      = reinterpret_cast<u32*>(ctx->dScratch + s.ctrlOffset + 4);
  c.scratch.totals    = reinterpret_cast<u64*>(ctx->dScratch + s.ctrlOffset + 8);
}

ClassifyBuffers classify_buffers(tc_context* ctx)
{
  const Plan& p = ctx->plan;
  return {reinterpret_cast<uint2*>(ctx->dScratch + p.clsCountsOffset),
          reinterpret_cast<u32*>(ctx->dScratch + p.clsTriWordsOffset),
          reinterpret_cast<RangeSums*>(ctx->dScratch + p.slots[p.slotClassify].stateOffset),
          reinterpret_cast<ClusterOffsets*>(ctx->dScratch + p.clsBlockSumsOffset),
          reinterpret_cast<uint2*>(ctx->dScratch + p.clsFullRecsOffset),
          reinterpret_cast<u32*>(ctx->dScratch + p.clsFullRecsOffset + (size_t)p.classifyCap * 8)};
}

InstantiateBuffers instantiate_buffers(tc_context* ctx)
{
  return {reinterpret_cast<u32*>(ctx->dScratch + ctx->plan.partVertexOffset),
          reinterpret_cast<unsigned long long*>(ctx->dScratch + ctx->plan.chunkSumsOffset)};
}

u32 persistent_grid(const tc_context* ctx, u32 maxTiles, u32 blocksPerSM)
{
  u32 g = ctx->numSMs * std::max(1u, blocksPerSM);
  return std::max(1u, std::min(g, std::max(1u, maxTiles)));
}

u32 frame_begin_grid(const tc_context* ctx, const tc_frame_args* a)
{
  return std::max(1u, std::min(ctx->numSMs * 2, ceil_div((u64)a->caps.maxSplitTriangles * 6, 256)));
}

// kernels one batched frame launches (the BLAS set-up is fused for up to
// kBlasSetupFusedMax instances)
uint64_t frame_launches(const tc_context* ctx, const tc_frame_args* a)
{
  return kFrameFixedLaunches + (ctx->schedule.splitPerPass ? split_passes(a->caps.splitFactor) : 1)
         - (a->numInstances <= kBlasSetupFusedMax ? 1 : 0)
         - (ctx->schedule.frameShape == 1 ? 4 : 0)  // one allocation + vertex launch instead of two
         + ((a->flags & TC_FLAG_TRANSIENT_2X) ? 1 : 0);  // the 2X batches' vertices
}

u32 insert_grid(const tc_context* ctx, const tc_frame_args* a)
{
  // tiles of 1024 instantiations, at most one resident wave of blocks that
  // stride over them (blocks past the frame's instantiations only read the run
  // table, but each costs a dispatch)
  return std::max(1u, std::min(ceil_div(a->caps.maxGeneratedClusters, 1024), ctx->numSMs * 4));
}

SplitLevels split_levels(const tc_context* ctx, u32 passes)
{
  SplitLevels lv = {};
  const Plan& p  = ctx->plan;
  lv.levels      = std::min(passes, kMaxSplitLevels);
  lv.stride      = p.slots[p.slotSplit0].stride;
  for(u32 L = 0; L < lv.levels; L++)
  {
    const SlotPlan& s = p.slots[p.slotSplit0 + L];
    lv.lbState[L]     = reinterpret_cast<unsigned long long*>(ctx->dScratch + s.stateOffset);
    lv.ctrl[L]        = reinterpret_cast<u32*>(ctx->dScratch + s.ctrlOffset);
  }
  return lv;
}

u32 split_block(const tc_schedule& s)
{
  u32 b = s.splitBlockSize;
  return (b == 128 || b == 256 || b == 512) ? b : 256;
}
u32 split_items_per_tile(u32 block) { return block == 128 ? 16 : 32; }

// The batched frame: one persistent launch per stage, build_setup fused into the
// producers' last block. Graph-capturable (no host synchronisation, no allocation).
tc_status record_batched_frame(tc_context* ctx, const tc_frame_args* a, cudaStream_t s, const HostIo& io = HostIo())
{
  const Plan&        p     = ctx->plan;
  const tc_schedule& sched = ctx->schedule;
  const u32          bpsm  = std::max(1u, sched.blocksPerSM);

  // No memset before the frame: the instance classification's slot (the
  // first) puts itself back to zero after each use, and the frame's first
  // kernel zeroes the rest of the frame's scratch, which only later kernels use.
  StageCtx c = base_ctx(ctx, a);
  bind_slot(ctx, c, p.slotInstances, true);
  const size_t zeroOff = align_up(p.slots[p.slotInstances].ctrlOffset + kCtrlBytes, 256);
  c.zeroBase           = reinterpret_cast<uint4*>(ctx->dScratch + zeroOff);
  c.zeroN16            = (p.frameBytes - zeroOff) / 16;
  const u32 beginGrid = std::max(frame_begin_grid(ctx, a), ceil_div(a->numInstances, kInstanceTile));
  if(io.bytes)
  {
    const HostUpload up = {io.hostIn, io.devIn, io.bytes};
    if(io.fused)
    {
      // the first kernel copies the block and reads its own inputs from the host block
      StageCtx  ch   = c;
      const u64 d0   = reinterpret_cast<u64>(io.devIn);
      auto      host = [&](uint64_t ptr) { return static_cast<const char*>(io.hostIn) + (ptr - d0); };
      ch.view        = reinterpret_cast<const tc_FrameConstants*>(host(a->view));
      ch.viewLast    = reinterpret_cast<const tc_FrameConstants*>(host(a->viewLast));
      ch.instances   = reinterpret_cast<const tc_RenderInstance*>(host(a->instances));
      TC_CHECK_CUDA(launch_frame_begin_instances_upload(ch, up, beginGrid, s));
    }
    else
    {
      TC_CHECK_CUDA(launch_host_upload(up, ctx->numSMs, s));
      TC_CHECK_CUDA(launch_frame_begin_instances(c, beginGrid, s));
    }
  }
  else
    TC_CHECK_CUDA(launch_frame_begin_instances(c, beginGrid, s));
  c.zeroBase = nullptr;
  c.zeroN16  = 0;

  // With RT semantics every cluster of every instance is visible, in instance
  // order: classify reads that list from the instances' cluster prefix and
  // clusters_cull (which writes it out, with its counter and set-up) runs on
  // the second side stream, joined at the frame's end.
  const bool flat = (a->flags & TC_FLAG_RASTER_CULL) == 0;
  {
    StageCtx cc = c;
    bind_slot(ctx, cc, p.slotCull, false);
    cc.fuseSetup         = TC_BUILD_SETUP_CLASSIFY;
    cudaStream_t cs      = s;
    if(flat)
    {
      TC_CHECK_CUDA(cudaEventRecord(ctx->evInst, s));
      TC_CHECK_CUDA(cudaStreamWaitEvent(ctx->side2, ctx->evInst, 0));
      cs = ctx->side2;
    }
    TC_CHECK_CUDA(
        launch_clusters_cull(cc, persistent_grid(ctx, ceil_div(a->totalClusters, kCullTile), 4), kCullTile, cs, flat));
    if(flat && io.hostRb)
      TC_CHECK_CUDA(cudaEventRecord(ctx->evCull, cs));
  }
  c.flatVisible = flat ? 1u : 0u;

  bind_slot(ctx, c, p.slotClassify, false);
  c.fuseSetup = TC_BUILD_SETUP_SPLIT;
  TC_CHECK_CUDA(launch_cluster_classify(c, classify_buffers(ctx), std::min(a->totalClusters, a->caps.maxVisibleClusters),
                                        ctx->numSMs, sched.classifyBlocksPerSM, s));

  // The parts classify produced (run 0) come first in the instantiation order
  // and their offsets depend on nothing the split passes do: they are
  // allocated on the side stream while the (latency-bound) split passes run,
  // the other runs after both. Nothing later in the frame reads generated
  // vertices, so each run's vertex kernel stays on the side stream, beside
  // the next allocation and the BLAS lists, and joins at the frame's end.
  TC_CHECK_CUDA(cudaEventRecord(ctx->evFork, s));
  TC_CHECK_CUDA(cudaStreamWaitEvent(ctx->side, ctx->evFork, 0));
  // The full clusters' vertices depend on classify alone and nothing later in
  // the frame reads them: they run on a second side stream, joined at the end.
  TC_CHECK_CUDA(cudaStreamWaitEvent(ctx->side2, ctx->evFork, 0));
  TC_CHECK_CUDA(launch_classify_full_vertices(c, classify_buffers(ctx),
                                              std::min(a->totalClusters, a->caps.maxVisibleClusters), ctx->numSMs,
                                              sched.fullVertexBlocksPerSM, ctx->side2));
  TC_CHECK_CUDA(cudaEventRecord(ctx->evJoin2, ctx->side2));
  const bool earlyRun0 = sched.frameShape == 0;
  if(earlyRun0)
  {
    StageCtx c0 = c;
    bind_slot(ctx, c0, p.slotInstantiate0, false);
    c0.fuseSetup = kNoSetup;
    c0.run       = 0;
    TC_CHECK_CUDA(launch_instantiate_prefix(c0, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                            sched.scanBlocksPerSM, ctx->side));
    TC_CHECK_CUDA(cudaEventRecord(ctx->evScan0, ctx->side));
    TC_CHECK_CUDA(launch_instantiate_args(c0, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                          sched.scanBlocksPerSM, ctx->side));
    TC_CHECK_CUDA(cudaEventRecord(ctx->evJoin, ctx->side));
    TC_CHECK_CUDA(launch_instantiate_vertices(c0, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                              sched.vertexBlocksPerSM, sched.vertexGridPerSM, ctx->side));
  }

  const u32 sb     = split_block(sched);
  const u32 passes = split_passes(a->caps.splitFactor);
  const u32 sgrid  = persistent_grid(ctx, ceil_div(a->caps.maxSplitTriangles, split_items_per_tile(sb)), bpsm * (512 / sb));
  if(sched.splitPerPass)
  {
    // one launch per pass, the pass set-up fused into its last block
    for(u32 q = 0; q < passes; q++)
    {
      bind_slot(ctx, c, p.slotSplit0 + q, false);
      c.fuseSetup = (q + 1 < passes) ? TC_BUILD_SETUP_SPLIT_PASS : TC_BUILD_SETUP_INSTANTIATE_TESS;
      TC_CHECK_CUDA(launch_triangle_split(c, sb, sgrid, s));
    }
  }
  else
  {
    // every split pass in one persistent launch (level by level inside)
    SplitLevels lv = split_levels(ctx, passes);
    bind_slot(ctx, c, p.slotSplit0, false);
    c.fuseSetup = TC_BUILD_SETUP_INSTANTIATE_TESS;
    TC_CHECK_CUDA(launch_triangle_split_levels(c, lv, sb, sgrid, s));
  }
  // the later runs' offsets continue from the counters the first run's scan
  // left; their arguments wait for the first run's (whose CLAS counts the
  // BLAS set-up in their last block sums)
  if(earlyRun0)
    TC_CHECK_CUDA(cudaStreamWaitEvent(s, ctx->evScan0, 0));
  bind_slot(ctx, c, p.slotInstantiate, false);
  c.fuseSetup = TC_BUILD_SETUP_BUILD_BLAS;
  c.run       = earlyRun0 ? kRunsAfterFirst : kAllRuns;
  // up to kBlasSetupFusedMax instances the BLAS list offsets are computed by
  // the argument kernel's last block instead of a launch of their own
  const bool fuseBlas = a->numInstances <= kBlasSetupFusedMax;
  c.fuseBlasSetup     = fuseBlas ? 1u : 0u;
  TC_CHECK_CUDA(launch_instantiate_prefix(c, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                          sched.scanBlocksPerSM, s));
  if(earlyRun0)
    TC_CHECK_CUDA(cudaStreamWaitEvent(s, ctx->evJoin, 0));
  TC_CHECK_CUDA(launch_instantiate_args(c, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                        sched.scanBlocksPerSM, s));
  c.fuseBlasSetup = 0;
  TC_CHECK_CUDA(cudaEventRecord(ctx->evArgs1, s));
  TC_CHECK_CUDA(cudaStreamWaitEvent(ctx->side, ctx->evArgs1, 0));
  TC_CHECK_CUDA(launch_instantiate_vertices(c, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                            sched.vertexBlocksPerSM, sched.vertexGridPerSM, ctx->side));
  TC_CHECK_CUDA(cudaEventRecord(ctx->evVerts, ctx->side));

  bind_slot(ctx, c, p.slotBlas, false);
  c.fuseSetup = kNoSetup;
  c.run       = kAllRuns;
  if(!fuseBlas)
    TC_CHECK_CUDA(
        launch_blas_setup_insertion(c, std::max(1u, ceil_div(a->numInstances, kInstanceTile)), kInstanceTile, s));

  u32* seg = reinterpret_cast<u32*>(ctx->dScratch + p.segOffset);
  TC_CHECK_CUDA(launch_blas_clusters_insert(c, seg, seg + (size_t)p.segStride * p.segRows, p.segStride, insert_grid(ctx, a), s));
  if(io.hostRb)
  {
    // Every Readback writer is behind this point on this stream (the first
    // part run's argument kernel joined at evJoin) except clusters_cull on the
    // second side stream, whose fused set-up writes numVisibleClusters; the
    // vertex kernels still running beside write none. So the copy to the host
    // waits for the cull alone and overlaps the vertex kernels' tails.
    if(flat)
      TC_CHECK_CUDA(cudaStreamWaitEvent(s, ctx->evCull, 0));
    TC_CHECK_CUDA(launch_host_readback(c.readback, io.hostRb, s));
  }
  TC_CHECK_CUDA(cudaStreamWaitEvent(s, ctx->evVerts, 0));
  TC_CHECK_CUDA(cudaStreamWaitEvent(s, ctx->evJoin2, 0));

  ctx->launches += frame_launches(ctx, a) + io.launches();
  return TC_OK;
}

// Replays the batched frame's graph (recorded again when the args, the
// schedule or the host buffers changed).
tc_status graph_frame(tc_context* ctx, const tc_frame_args* args, const HostIo& io, cudaStream_t s)
{
  if(!ctx->graphValid || std::memcmp(&ctx->graphArgs, args, sizeof(tc_frame_args)) != 0
     || std::memcmp(&ctx->graphSchedule, &ctx->schedule, sizeof(tc_schedule)) != 0 || !(ctx->graphIo == io))
  {
    if(ctx->graphExec)
      cudaGraphExecDestroy(ctx->graphExec);
    if(ctx->graph)
      cudaGraphDestroy(ctx->graph);
    ctx->graphExec  = nullptr;
    ctx->graph      = nullptr;
    ctx->graphValid = false;
    // capture on a private stream so the caller's stream may be the legacy default stream
    cudaStream_t cap;
    TC_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    uint64_t launchesBefore = ctx->launches;
    if(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    {
      cudaStreamDestroy(cap);
      return TC_ERR_CUDA;
    }
    tc_status rst = record_batched_frame(ctx, args, cap, io);
    cudaGraph_t g  = nullptr;
    cudaError_t ce = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    ctx->launches = launchesBefore;
    if(rst != TC_OK)
    {
      if(g)
        cudaGraphDestroy(g);
      return rst;
    }
    if(ce != cudaSuccess)
      return TC_ERR_CUDA;
    ctx->graph = g;
    TC_CHECK_CUDA(cudaGraphInstantiate(&ctx->graphExec, g, 0));
    ctx->graphArgs     = *args;
    ctx->graphSchedule = ctx->schedule;
    ctx->graphIo       = io;
    ctx->graphValid    = true;
  }
  TC_CHECK_CUDA(cudaGraphLaunch(ctx->graphExec, s));
  ctx->launches += frame_launches(ctx, args) + io.launches();
  return TC_OK;
}

// The device alias of [p, p + bytes) in pinned, mapped host memory, or null
// when either end is not pinned host memory or the two ends are not one
// contiguous mapping.
void* host_alias(const void* p, uint64_t bytes)
{
  cudaPointerAttributes a0, a1;
  const char* last = static_cast<const char*>(p) + bytes - 1;
  if(cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess)
  {
    cudaGetLastError();  // not sticky: clear it for the caller
    return nullptr;
  }
  if(a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  if(static_cast<char*>(a1.devicePointer) - static_cast<char*>(a0.devicePointer) != (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a0.devicePointer;
}

// Whether the frame constants (this frame's and last frame's) and the
// instance records all lie in the uploaded block [d0, d0 + bytes): then the
// frame's first kernel can read them from the host block while it uploads it.
bool inputs_in_block(const tc_frame_args* a, uint64_t d0, uint64_t bytes)
{
  auto inside = [&](uint64_t p, uint64_t size) { return p >= d0 && p - d0 <= bytes && size <= bytes - (p - d0); };
  return inside(a->view, sizeof(tc_FrameConstants)) && inside(a->viewLast, sizeof(tc_FrameConstants))
         && inside(a->instances, (uint64_t)a->numInstances * sizeof(tc_RenderInstance));
}

// Whether both ends of [p, p + bytes) are device (or managed) memory.
bool device_range(const void* p, uint64_t bytes)
{
  cudaPointerAttributes a0, a1;
  const char* last = static_cast<const char*>(p) + bytes - 1;
  if(cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess)
  {
    cudaGetLastError();
    return false;
  }
  auto dev = [](const cudaPointerAttributes& a) {
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
  };
  return dev(a0) && dev(a1);
}

}  // namespace

extern "C" {

const char* tc_version(void) { return "vk_tessellated_clusters_gb300 1.0 (sm_103a)"; }

const char* tc_status_string(tc_status s)
{
  switch(s)
  {
    case TC_OK:
      return "ok";
    case TC_ERR_INVALID_ARG:
      return "invalid argument";
    case TC_ERR_CAPACITY:
      return "request exceeds the context's capacity";
    case TC_ERR_QUEUE_TIMEOUT:
      return "device-side wait timed out";
    case TC_ERR_CUDA:
      return "CUDA error";
    case TC_ERR_NOT_INITIALIZED:
      return "tessellation table not initialised";
  }
  return "unknown";
}

uint32_t tc_split_pass_count(uint32_t splitFactor) { return split_passes(splitFactor); }

namespace {

void destroy_streams(tc_context* ctx)
{
  for(cudaEvent_t* e : {&ctx->evFork, &ctx->evJoin, &ctx->evJoin2, &ctx->evArgs1, &ctx->evVerts, &ctx->evInst,
                        &ctx->evScan0, &ctx->evCull})
    if(*e)
      cudaEventDestroy(*e), *e = nullptr;
  for(cudaStream_t* st : {&ctx->side, &ctx->side2})
    if(*st)
      cudaStreamDestroy(*st), *st = nullptr;
}

}  // namespace

tc_status tc_context_create(const tc_context_desc* desc, tc_context** outCtx)
{
  if(!desc || !outCtx)
    return TC_ERR_INVALID_ARG;
  *outCtx = nullptr;
  if(desc->caps.maxPartTriangles == 0 || desc->caps.maxSplitTriangles == 0 || desc->caps.maxVisibleClusters == 0)
    return TC_ERR_INVALID_ARG;
  tc_context* ctx = new(std::nothrow) tc_context();
  if(!ctx)
    return TC_ERR_INVALID_ARG;
  ctx->device = desc->device;
  ctx->desc   = *desc;
  if(cudaSetDevice(desc->device) != cudaSuccess)
  {
    delete ctx;
    return TC_ERR_CUDA;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, desc->device);
  ctx->numSMs   = (u32)std::max(1, sms);
  if(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess
     || cudaStreamCreateWithFlags(&ctx->side2, cudaStreamNonBlocking) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evFork, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evJoin, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evJoin2, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evArgs1, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evVerts, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evInst, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evScan0, cudaEventDisableTiming) != cudaSuccess
     || cudaEventCreateWithFlags(&ctx->evCull, cudaEventDisableTiming) != cudaSuccess)
  {
    destroy_streams(ctx);
    delete ctx;
    return TC_ERR_CUDA;
  }
  ctx->schedule = {4, 256, 4, 4, 1, kDefaultFullVertexBlocksPerSM, 0, 0, 0, 0};  // the batched scene's tuned shape
  ctx->plan     = make_plan(*desc);
  if(cudaMalloc(&ctx->dScratch, ctx->plan.totalBytes) != cudaSuccess
     || cudaMemset(ctx->dScratch, 0, ctx->plan.totalBytes) != cudaSuccess)
  {
    cudaFree(ctx->dScratch);
    destroy_streams(ctx);
    delete ctx;
    return TC_ERR_CUDA;
  }
  *outCtx = ctx;
  return TC_OK;
}

tc_status tc_context_destroy(tc_context* ctx)
{
  if(!ctx)
    return TC_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  if(ctx->graphExec)
    cudaGraphExecDestroy(ctx->graphExec);
  if(ctx->graph)
    cudaGraphDestroy(ctx->graph);
  cudaFree(ctx->dVertices);
  cudaFree(ctx->dTriangles);
  cudaFree(ctx->dEntries);
  cudaFree(ctx->dTemplateAddresses);
  cudaFree(ctx->dTemplateSizes);
  cudaFree(ctx->dTable);
  cudaFree(ctx->dScratch);
  destroy_streams(ctx);
  delete ctx;
  return TC_OK;
}

// src/tessellation_table.cpp:36-100
tc_status tc_table_init(tc_context* ctx, const uint32_t* vertices, uint32_t numVertices, const uint32_t* triangles,
                        uint32_t numTriangles, const uint16_t* configs, uint32_t numConfigs, uint32_t maxEdgeSegments,
                        tc_table_info* outInfo)
{
  if(!ctx || !vertices || !triangles || !configs)
    return TC_ERR_INVALID_ARG;
  if(maxEdgeSegments != TC_TESSTABLE_SIZE)
    return TC_ERR_INVALID_ARG;
  const u32 L = TC_TESSTABLE_LOOKUP_SIZE;
  std::vector<tc_TessTableEntry> lookup(TC_TESSTABLE_LOOKUP_ENTRIES);
  std::memset(lookup.data(), 0, lookup.size() * sizeof(tc_TessTableEntry));
  auto idx = [&](u32 x, u32 y, u32 z) { return x + y * L + z * L * L - (1 + L + L * L); };
  u32 ci = 0, maxV = 0, maxT = 0;
  for(u32 x = 1; x <= maxEdgeSegments; x++)
    for(u32 y = 1; y <= x; y++)
      for(u32 z = 1; z <= y; z++, ci++)
      {
        if(ci >= numConfigs)
          return TC_ERR_INVALID_ARG;
        tc_TessTableEntry e = {configs[ci * 4 + 0], configs[ci * 4 + 1], configs[ci * 4 + 2], configs[ci * 4 + 3]};
        // every config must stay inside the raw arrays and the per-config limits
        // (TESSTABLE_MAX_TRIANGLES / TESSTABLE_MAX_VERTICES, shaderio_scene.h:43-49)
        if((u32)e.firstTriangle + e.numTriangles > numTriangles || (u32)e.firstVertex + e.numVertices > numVertices
           || e.numTriangles > TC_TESSTABLE_SIZE * TC_TESSTABLE_SIZE
           || e.numVertices > ((TC_TESSTABLE_SIZE + 1) * (TC_TESSTABLE_SIZE + 2)) / 2)
          return TC_ERR_INVALID_ARG;
        lookup[idx(x, y, z)] = e;
        if(z != y && x > 1)
          lookup[idx(x, z, y)] = e;
        maxT = std::max(maxT, (u32)e.numTriangles);
        maxV = std::max(maxV, (u32)e.numVertices);
      }
  if(ci != numConfigs)
    return TC_ERR_INVALID_ARG;
  for(u32 t = 0; t < numTriangles; t++)
  {
    const u32 p = triangles[t];
    // indices are relative to a config's first vertex; a config has at most 78 vertices
    if((p & 0xFF) >= 78 || ((p >> 8) & 0xFF) >= 78 || ((p >> 16) & 0xFF) >= 78)
      return TC_ERR_INVALID_ARG;
  }

  std::lock_guard<std::mutex> lock(ctx->mutex);
  TC_CHECK_CUDA(cudaSetDevice(ctx->device));
  cudaFree(ctx->dVertices);
  cudaFree(ctx->dTriangles);
  cudaFree(ctx->dEntries);
  cudaFree(ctx->dTemplateAddresses);
  cudaFree(ctx->dTemplateSizes);
  cudaFree(ctx->dTable);
  ctx->dVertices = nullptr;
  ctx->dTriangles = nullptr;
  ctx->dEntries = nullptr;
  ctx->dTemplateAddresses = nullptr;
  ctx->dTemplateSizes = nullptr;
  ctx->dTable = nullptr;
  TC_CHECK_CUDA(cudaMalloc(&ctx->dVertices, sizeof(u32) * numVertices));
  TC_CHECK_CUDA(cudaMalloc(&ctx->dTriangles, sizeof(u32) * numTriangles));
  TC_CHECK_CUDA(cudaMalloc(&ctx->dEntries, sizeof(tc_TessTableEntry) * TC_TESSTABLE_LOOKUP_ENTRIES));
  TC_CHECK_CUDA(cudaMalloc(&ctx->dTemplateAddresses, sizeof(u64) * TC_TESSTABLE_LOOKUP_ENTRIES));
  TC_CHECK_CUDA(cudaMalloc(&ctx->dTemplateSizes, sizeof(u32) * TC_TESSTABLE_LOOKUP_ENTRIES));
  TC_CHECK_CUDA(cudaMalloc(&ctx->dTable, sizeof(tc_TessellationTable)));
  TC_CHECK_CUDA(cudaMemcpy(ctx->dVertices, vertices, sizeof(u32) * numVertices, cudaMemcpyHostToDevice));
  TC_CHECK_CUDA(cudaMemcpy(ctx->dTriangles, triangles, sizeof(u32) * numTriangles, cudaMemcpyHostToDevice));
  TC_CHECK_CUDA(cudaMemcpy(ctx->dEntries, lookup.data(), sizeof(tc_TessTableEntry) * TC_TESSTABLE_LOOKUP_ENTRIES,
                           cudaMemcpyHostToDevice));
  TC_CHECK_CUDA(cudaMemset(ctx->dTemplateAddresses, 0, sizeof(u64) * TC_TESSTABLE_LOOKUP_ENTRIES));
  TC_CHECK_CUDA(cudaMemset(ctx->dTemplateSizes, 0, sizeof(u32) * TC_TESSTABLE_LOOKUP_ENTRIES));
  ctx->hTable.vertices                   = (uint64_t)(uintptr_t)ctx->dVertices;
  ctx->hTable.triangles                  = (uint64_t)(uintptr_t)ctx->dTriangles;
  ctx->hTable.entries                    = (uint64_t)(uintptr_t)ctx->dEntries;
  ctx->hTable.templateAddresses          = (uint64_t)(uintptr_t)ctx->dTemplateAddresses;
  ctx->hTable.templateInstantiationSizes = (uint64_t)(uintptr_t)ctx->dTemplateSizes;
  TC_CHECK_CUDA(cudaMemcpy(ctx->dTable, &ctx->hTable, sizeof(tc_TessellationTable), cudaMemcpyHostToDevice));
  ctx->tableReady = true;
  ctx->graphValid = false;
  if(outInfo)
  {
    outInfo->maxSize        = maxEdgeSegments;
    outInfo->maxSizeConfigs = L;
    outInfo->numConfigs     = TC_TESSTABLE_LOOKUP_ENTRIES;
    outInfo->maxVertices    = maxV;
    outInfo->maxTriangles   = maxT;
    outInfo->numRawConfigs  = numConfigs;
    outInfo->deviceTable    = (uint64_t)(uintptr_t)ctx->dTable;
    outInfo->table          = ctx->hTable;
  }
  return TC_OK;
}

tc_status tc_table_set_templates(tc_context* ctx, const uint64_t* templateAddresses, const uint32_t* instantiationSizes,
                                 void* stream)
{
  if(!ctx)
    return TC_ERR_INVALID_ARG;
  if(!ctx->tableReady)
    return TC_ERR_NOT_INITIALIZED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if(templateAddresses)
    TC_CHECK_CUDA(cudaMemcpyAsync(ctx->dTemplateAddresses, templateAddresses, sizeof(u64) * TC_TESSTABLE_LOOKUP_ENTRIES,
                                  cudaMemcpyHostToDevice, s));
  if(instantiationSizes)
    TC_CHECK_CUDA(cudaMemcpyAsync(ctx->dTemplateSizes, instantiationSizes, sizeof(u32) * TC_TESSTABLE_LOOKUP_ENTRIES,
                                  cudaMemcpyHostToDevice, s));
  TC_CHECK_CUDA(cudaStreamSynchronize(s));
  return TC_OK;
}

tc_status tc_set_schedule(tc_context* ctx, const tc_schedule* schedule)
{
  if(!ctx || !schedule)
    return TC_ERR_INVALID_ARG;
  const tc_schedule& q = *schedule;
  const u32 perSM[] = {q.classifyBlocksPerSM, q.vertexBlocksPerSM, q.scanBlocksPerSM, q.blocksPerSM};
  for(u32 v : perSM)
    if(v < 1 || v > 64)
      return TC_ERR_INVALID_ARG;
  if(q.splitBlockSize != 128 && q.splitBlockSize != 256 && q.splitBlockSize != 512)
    return TC_ERR_INVALID_ARG;
  if(q.fullVertexBlocksPerSM > 64 || q.vertexGridPerSM > 64 || q.frameShape > 1 || q.splitPerPass > 1)
    return TC_ERR_INVALID_ARG;
  ctx->schedule   = *schedule;
  if(ctx->schedule.fullVertexBlocksPerSM == 0)
    ctx->schedule.fullVertexBlocksPerSM = kDefaultFullVertexBlocksPerSM;
  ctx->graphValid = false;
  return TC_OK;
}

tc_status tc_get_schedule(const tc_context* ctx, tc_schedule* schedule)
{
  if(!ctx || !schedule)
    return TC_ERR_INVALID_ARG;
  *schedule = ctx->schedule;
  return TC_OK;
}

tc_status tc_frame_build(tc_context* ctx, const tc_frame_args* args, void* stream)
{
  tc_status st = validate(ctx, args);
  if(st != TC_OK)
    return st;
  return record_batched_frame(ctx, args, reinterpret_cast<cudaStream_t>(stream));
}

tc_status tc_frame_build_graph(tc_context* ctx, const tc_frame_args* args, void* stream)
{
  tc_status st = validate(ctx, args);
  if(st != TC_OK)
    return st;
  return graph_frame(ctx, args, HostIo(), reinterpret_cast<cudaStream_t>(stream));
}

tc_status tc_frame_build_graph_host(tc_context* ctx, const tc_frame_args* args, const void* hostInputs,
                                    uint64_t deviceInputs, uint64_t inputBytes, void* hostReadback, void* stream)
{
  tc_status st = validate(ctx, args);
  if(st != TC_OK)
    return st;
  if(inputBytes && (!hostInputs || !deviceInputs || (reinterpret_cast<uintptr_t>(hostInputs) & 15) || (deviceInputs & 15)))
    return TC_ERR_INVALID_ARG;
  if(hostReadback && (reinterpret_cast<uintptr_t>(hostReadback) & 7))
    return TC_ERR_INVALID_ARG;
  HostIo io;
  io.bytes    = inputBytes;
  io.devIn    = inputBytes ? reinterpret_cast<void*>(deviceInputs) : nullptr;
  io.callerIn = inputBytes ? hostInputs : nullptr;
  io.callerRb = hostReadback;
  io.fused    = inputBytes && inputs_in_block(args, deviceInputs, inputBytes);
  if(ctx->graphValid && io.same_buffers(ctx->graphIo))
  {
    // checked when the graph was recorded
    io.hostIn = ctx->graphIo.hostIn;
    io.hostRb = ctx->graphIo.hostRb;
  }
  else
  {
    if(inputBytes)
    {
      io.hostIn = host_alias(hostInputs, inputBytes);
      if(!io.hostIn || !device_range(io.devIn, inputBytes))
        return TC_ERR_INVALID_ARG;
    }
    if(hostReadback)
    {
      io.hostRb = host_alias(hostReadback, sizeof(tc_Readback));
      if(!io.hostRb)
        return TC_ERR_INVALID_ARG;
    }
  }
  return graph_frame(ctx, args, io, reinterpret_cast<cudaStream_t>(stream));
}

tc_status tc_frame_begin(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TC_CHECK_CUDA(cudaMemsetAsync(ctx->dScratch, 0, ctx->plan.frameBytes, s));
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_frame_begin(c, frame_begin_grid(ctx, a), s));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_instances_classify(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  StageCtx c = base_ctx(ctx, a);
  bind_slot(ctx, c, ctx->plan.slotInstances, true);
  TC_CHECK_CUDA(launch_instances_classify(c, std::max(1u, ceil_div(a->numInstances, kInstanceTile)), kInstanceTile,
                                          reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_clusters_cull(tc_context* ctx, const tc_frame_args* a, uint32_t instanceBegin, uint32_t instanceEnd,
                           void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(instanceBegin > instanceEnd || instanceEnd > a->numInstances)
    return TC_ERR_INVALID_ARG;
  StageCtx c  = base_ctx(ctx, a);
  c.instBegin = instanceBegin;
  c.instEnd   = instanceEnd;
  bind_slot(ctx, c, ctx->plan.slotCull, true);
  TC_CHECK_CUDA(launch_clusters_cull(c, persistent_grid(ctx, ceil_div(a->totalClusters, kCullTile), 2), kCullTile,
                                     reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_build_setup(tc_context* ctx, const tc_frame_args* a, uint32_t mode, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(mode > TC_BUILD_SETUP_BUILD_BLAS)
    return TC_ERR_INVALID_ARG;
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_build_setup(c, mode, reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_cluster_classify(tc_context* ctx, const tc_frame_args* a, uint32_t instanceBegin, uint32_t instanceEnd,
                              void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(instanceBegin > instanceEnd || instanceEnd > a->numInstances)
    return TC_ERR_INVALID_ARG;
  StageCtx c  = base_ctx(ctx, a);
  c.instBegin = instanceBegin;
  c.instEnd   = instanceEnd;
  bind_slot(ctx, c, ctx->plan.slotClassify, true);
  {
    // the range sums the count kernel accumulates start at zero
    const SlotPlan& sl = ctx->plan.slots[ctx->plan.slotClassify];
    TC_CHECK_CUDA(cudaMemsetAsync(ctx->dScratch + sl.stateOffset, 0, (size_t)sl.stride * sl.counters * 8,
                                  reinterpret_cast<cudaStream_t>(stream)));
  }
  TC_CHECK_CUDA(launch_cluster_classify(c, classify_buffers(ctx), std::min(a->totalClusters, a->caps.maxVisibleClusters),
                                        ctx->numSMs, ctx->schedule.classifyBlocksPerSM,
                                        reinterpret_cast<cudaStream_t>(stream)));
  TC_CHECK_CUDA(launch_classify_full_vertices(c, classify_buffers(ctx),
                                              std::min(a->totalClusters, a->caps.maxVisibleClusters), ctx->numSMs,
                                              4, reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += (a->flags & TC_FLAG_TRANSIENT_2X) ? 4 : 3;
  return TC_OK;
}

tc_status tc_triangle_split(tc_context* ctx, const tc_frame_args* a, uint32_t instanceBegin, uint32_t instanceEnd,
                            void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(instanceBegin > instanceEnd || instanceEnd > a->numInstances)
    return TC_ERR_INVALID_ARG;
  StageCtx c  = base_ctx(ctx, a);
  c.instBegin = instanceBegin;
  c.instEnd   = instanceEnd;
  bind_slot(ctx, c, ctx->plan.slotSplit0, true);
  const u32 sb = split_block(ctx->schedule);
  TC_CHECK_CUDA(launch_triangle_split(c, sb,
                                      persistent_grid(ctx, ceil_div(a->caps.maxSplitTriangles, split_items_per_tile(sb)),
                                                      std::max(1u, ctx->schedule.blocksPerSM) * (512 / sb)),
                                      reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_triangle_split_all(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  cudaStream_t s      = reinterpret_cast<cudaStream_t>(stream);
  const Plan&  p      = ctx->plan;
  const u32    passes = split_passes(a->caps.splitFactor);
  // the levels' look-back rows and control words start at zero
  const SlotPlan& first = p.slots[p.slotSplit0];
  const SlotPlan& last  = p.slots[p.slotSplit0 + passes - 1];
  TC_CHECK_CUDA(cudaMemsetAsync(ctx->dScratch + first.stateOffset, 0, last.ctrlOffset + kCtrlBytes - first.stateOffset, s));
  StageCtx c = base_ctx(ctx, a);
  bind_slot(ctx, c, p.slotSplit0, false);
  c.fuseSetup          = kNoSetup;  // the caller's BUILD_SETUP_INSTANTIATE_TESS follows, as after the last pass
  const u32 sb         = split_block(ctx->schedule);
  const SplitLevels lv = split_levels(ctx, passes);
  TC_CHECK_CUDA(launch_triangle_split_levels(
      c, lv, sb,
      persistent_grid(ctx, ceil_div(a->caps.maxSplitTriangles, split_items_per_tile(sb)),
                      std::max(1u, ctx->schedule.blocksPerSM) * (512 / sb)),
      s));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_triangle_instantiate_run(tc_context* ctx, const tc_frame_args* a, uint32_t run, uint32_t instanceBegin,
                                      uint32_t instanceEnd, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(instanceBegin > instanceEnd || instanceEnd > a->numInstances || (run != kAllRuns && run >= kMaxRuns))
    return TC_ERR_INVALID_ARG;
  if(run == kAllRuns && !(instanceBegin == 0 && instanceEnd == a->numInstances))
    return TC_ERR_INVALID_ARG;  // part triangles are only instance-sorted within a run
  StageCtx c  = base_ctx(ctx, a);
  c.instBegin = instanceBegin;
  c.instEnd   = instanceEnd;
  c.run       = run;
  bind_slot(ctx, c, ctx->plan.slotInstantiate, true);
  // one kernel for arguments and vertices (the frame graph keeps them apart:
  // its BLAS lists need the arguments only)
  TC_CHECK_CUDA(launch_instantiate_fused(c, instantiate_buffers(ctx), a->caps.maxPartTriangles, ctx->numSMs,
                                         ctx->schedule.scanBlocksPerSM, ctx->schedule.vertexBlocksPerSM,
                                         ctx->schedule.vertexGridPerSM, reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += (a->flags & (TC_FLAG_PN | TC_FLAG_RIPPLE)) ? 4 : 3;
  return TC_OK;
}

tc_status tc_triangle_instantiate(tc_context* ctx, const tc_frame_args* a, uint32_t partBegin, uint32_t partEnd,
                                  void* stream)
{
  // whole part list only (the per-run form is tc_triangle_instantiate_run)
  if(partBegin != 0 || partEnd != 0xFFFFFFFFu)
    return TC_ERR_INVALID_ARG;
  return tc_triangle_instantiate_run(ctx, a, kAllRuns, 0, a ? a->numInstances : 0, stream);
}

tc_status tc_blas_setup_insertion(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  StageCtx c = base_ctx(ctx, a);
  bind_slot(ctx, c, ctx->plan.slotBlas, true);
  TC_CHECK_CUDA(launch_blas_setup_insertion(c, std::max(1u, ceil_div(a->numInstances, kInstanceTile)), kInstanceTile,
                                            reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_blas_clusters_insert(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const Plan&  p = ctx->plan;
  u32*         seg = reinterpret_cast<u32*>(ctx->dScratch + p.segOffset);
  TC_CHECK_CUDA(cudaMemsetAsync(seg, 0, (size_t)p.segStride * p.segRows * 4 * 2, s));
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_blas_clusters_insert(c, seg, seg + (size_t)p.segStride * p.segRows, p.segStride, insert_grid(ctx, a), s));
  ctx->launches += 2;
  return TC_OK;
}

// Per-instance launches of every stage, level by level, separate build_setup
// launches in between (the reference's per-instance clusters_cull dispatch,
// src/renderer_raytrace_clusters_tess.cpp:454-460, applied to every stage).
tc_status tc_frame_build_plain(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
#define TC_TRY(x)                                                                                                      \
  do                                                                                                                   \
  {                                                                                                                    \
    tc_status _s = (x);                                                                                                \
    if(_s != TC_OK)                                                                                                    \
      return _s;                                                                                                       \
  } while(0)
  const u32 n = a->numInstances;
  TC_TRY(tc_frame_begin(ctx, a, stream));
  TC_TRY(tc_instances_classify(ctx, a, stream));
  for(u32 i = 0; i < n; i++)
    TC_TRY(tc_clusters_cull(ctx, a, i, i + 1, stream));
  TC_TRY(tc_build_setup(ctx, a, TC_BUILD_SETUP_CLASSIFY, stream));
  for(u32 i = 0; i < n; i++)
    TC_TRY(tc_cluster_classify(ctx, a, i, i + 1, stream));
  TC_TRY(tc_build_setup(ctx, a, TC_BUILD_SETUP_SPLIT, stream));
  const u32 passes = split_passes(a->caps.splitFactor);
  for(u32 q = 0; q < passes; q++)
  {
    for(u32 i = 0; i < n; i++)
      TC_TRY(tc_triangle_split(ctx, a, i, i + 1, stream));
    if(q + 1 < passes)
      TC_TRY(tc_build_setup(ctx, a, TC_BUILD_SETUP_SPLIT_PASS, stream));
  }
  TC_TRY(tc_build_setup(ctx, a, TC_BUILD_SETUP_INSTANTIATE_TESS, stream));
  for(u32 r = 0; r <= passes && r < kMaxRuns; r++)
    for(u32 i = 0; i < n; i++)
      TC_TRY(tc_triangle_instantiate_run(ctx, a, r, i, i + 1, stream));
  TC_TRY(tc_build_setup(ctx, a, TC_BUILD_SETUP_BUILD_BLAS, stream));
  TC_TRY(tc_blas_setup_insertion(ctx, a, stream));
  TC_TRY(tc_blas_clusters_insert(ctx, a, stream));
#undef TC_TRY
  return TC_OK;
}

tc_status tc_instantiate_backward(tc_context* ctx, const tc_frame_args* a, uint64_t gradVertices, uint64_t gradTargets,
                                  uint64_t gradTexels, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(!gradVertices || !gradTargets || (a->numTextures && !gradTexels))
    return TC_ERR_INVALID_ARG;
  // the adjoint covers the linear, displaced path of template instantiations only
  if(a->flags & (TC_FLAG_PN | TC_FLAG_RIPPLE | TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
    return TC_ERR_INVALID_ARG;
  if(!(a->flags & TC_FLAG_WRITE_FULLCLUSTERS))
    return TC_ERR_INVALID_ARG;
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_instantiate_backward(c, reinterpret_cast<const float*>(gradVertices),
                                            reinterpret_cast<const tc_GradTargets*>(gradTargets),
                                            reinterpret_cast<float* const*>(gradTexels), ctx->numSMs * 8,
                                            reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_generate_vertices(tc_context* ctx, const tc_frame_args* a, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(!(a->flags & TC_FLAG_WRITE_FULLCLUSTERS)
     || (a->flags & (TC_FLAG_PN | TC_FLAG_RIPPLE | TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)))
    return TC_ERR_INVALID_ARG;
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_generate_vertices(c, ctx->numSMs * 8, reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 1;
  return TC_OK;
}

tc_status tc_decode_hits(tc_context* ctx, const tc_frame_args* a, const tc_hit* hits, uint32_t count,
                         tc_base_hit* out, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(count && (!hits || !out))
    return TC_ERR_INVALID_ARG;
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_decode_hits(c, hits, count, out, reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += count ? 1 : 0;
  return TC_OK;
}

tc_status tc_raster_batches(tc_context* ctx, const tc_frame_args* a, const tc_raster_outputs* out, void* stream)
{
  tc_status st = validate(ctx, a);
  if(st != TC_OK)
    return st;
  if(!out || !out->batches || !out->counts || !out->clipPositions || !out->worldPositions || !out->indices
     || !out->primitiveIDs)
    return TC_ERR_INVALID_ARG;
  StageCtx c = base_ctx(ctx, a);
  TC_CHECK_CUDA(launch_raster_batches(c, reinterpret_cast<uint4*>(ctx->dScratch + ctx->plan.rasterOffset), *out,
                                      a->caps.maxPartTriangles, ctx->numSMs, reinterpret_cast<cudaStream_t>(stream)));
  ctx->launches += 3;
  return TC_OK;
}

tc_status tc_read_device_errors(tc_context* ctx, uint32_t* outBits, void* stream)
{
  if(!ctx || !outBits)
    return TC_ERR_INVALID_ARG;
  cudaStream_t s   = reinterpret_cast<cudaStream_t>(stream);
  u32*         err = reinterpret_cast<u32*>(ctx->dScratch + ctx->plan.errOffset);
  TC_CHECK_CUDA(cudaMemcpyAsync(outBits, err, 4, cudaMemcpyDeviceToHost, s));
  TC_CHECK_CUDA(cudaMemsetAsync(err, 0, 4, s));
  TC_CHECK_CUDA(cudaStreamSynchronize(s));
  return TC_OK;
}

tc_status tc_lookback_probe(tc_context* ctx, uint32_t predecessorPublished, uint64_t* outPrefix, void* stream)
{
  if(!ctx || !outPrefix)
    return TC_ERR_INVALID_ARG;
  cudaStream_t s     = reinterpret_cast<cudaStream_t>(stream);
  u64*         state = reinterpret_cast<u64*>(ctx->dScratch + ctx->plan.segOffset);  // frame scratch, >= 3 words
  u32*         err   = reinterpret_cast<u32*>(ctx->dScratch + ctx->plan.errOffset);
  const u32    limit = ctx->schedule.lookbackSpinLimit ? ctx->schedule.lookbackSpinLimit : kSpinLimit;
  TC_CHECK_CUDA(launch_lookback_probe(reinterpret_cast<unsigned long long*>(state), predecessorPublished ? 1u : 0u,
                                      err, limit, s));
  ctx->launches += 1;
  TC_CHECK_CUDA(cudaMemcpyAsync(outPrefix, state + 2, sizeof(u64), cudaMemcpyDeviceToHost, s));
  TC_CHECK_CUDA(cudaStreamSynchronize(s));
  return TC_OK;
}

uint64_t tc_launch_count(const tc_context* ctx) { return ctx ? ctx->launches : 0; }

}  // extern "C"
