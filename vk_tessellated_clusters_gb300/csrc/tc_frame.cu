// tc_frame.cu — per-frame reset, instance classification, cluster culling and
// the standalone build_setup kernel.
#include <algorithm>

#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

// ---------------------------------------------------------------------------
// culling.glsl:30-113
// ---------------------------------------------------------------------------

struct Clip
{
  float x, y, z, w;
};

__device__ inline void mat_mul(const float* A, const float* B, float* C)
{
#pragma unroll
  for(int col = 0; col < 4; col++)
#pragma unroll
    for(int r = 0; r < 4; r++)
      C[col * 4 + r] = ((A[0 * 4 + r] * B[col * 4 + 0] + A[1 * 4 + r] * B[col * 4 + 1]) + A[2 * 4 + r] * B[col * 4 + 2])
                       + A[3 * 4 + r] * B[col * 4 + 3];
}

// culling.glsl:50-90
__device__ inline bool intersect_frustum(f3 lo, f3 hi, const float* world, const tc_FrameConstants& vl, Clip& omin,
                                         Clip& omax, bool& ovalid)
{
  float wvp[16];
  mat_mul(vl.viewProjMatrix.m, world, wvp);
  const float eps   = 1.2e-07f;
  u32         bits  = 0;
  bool        valid = true;
  Clip        cmin = {0, 0, 0, 0}, cmax = {0, 0, 0, 0};
#pragma unroll 1
  for(int n = 0; n < 8; n++)
  {
    float p[3] = {(n & 1) ? hi.x : lo.x, (n & 2) ? hi.y : lo.y, (n & 4) ? hi.z : lo.z};
    float h[4];
#pragma unroll
    for(int r = 0; r < 4; r++)
      h[r] = ((wvp[r] * p[0] + wvp[4 + r] * p[1]) + wvp[8 + r] * p[2]) + wvp[12 + r] * 1.0f;
    bool  v  = !(-eps < h[3] && h[3] < eps);
    float aw = fabsf(h[3]);
    Clip  cl = {__fdiv_rn(h[0], aw), __fdiv_rn(h[1], aw), __fdiv_rn(h[2], aw), h[3]};
    u32   cb = 0;
    cb |= h[0] < -h[3] ? 1 : 0;
    cb |= h[0] > h[3] ? 2 : 0;
    cb |= h[1] < -h[3] ? 4 : 0;
    cb |= h[1] > h[3] ? 8 : 0;
    cb |= h[2] < 0 ? 16 : 0;
    cb |= h[2] > h[3] ? 32 : 0;
    cb |= h[3] <= 0 ? 64 : 0;
    if(n == 0)
    {
      bits  = cb;
      cmin  = cl;
      cmax  = cl;
      valid = v;
    }
    else
    {
      bits &= cb;
      cmin  = {fminf(cmin.x, cl.x), fminf(cmin.y, cl.y), fminf(cmin.z, cl.z), fminf(cmin.w, cl.w)};
      cmax  = {fmaxf(cmax.x, cl.x), fmaxf(cmax.y, cl.y), fmaxf(cmax.z, cl.z), fmaxf(cmax.w, cl.w)};
      valid = valid && v;
    }
  }
  ovalid = valid;
  omin   = {fminf(fmaxf(cmin.x, -1.0f), 1.0f), fminf(fmaxf(cmin.y, -1.0f), 1.0f), cmin.z, cmin.w};
  omax   = {fminf(fmaxf(cmax.x, -1.0f), 1.0f), fminf(fmaxf(cmax.y, -1.0f), 1.0f), cmax.z, cmax.w};
  return bits == 0;
}

// culling.glsl:30-35
__device__ inline bool intersect_size(const Clip& cmin, const Clip& cmax, const tc_FrameConstants& vl)
{
  float rx = cmax.x - cmin.x, ry = cmax.y - cmin.y;
  return rx > __fdiv_rn(2.0f, vl.viewportf.x) || ry > __fdiv_rn(2.0f, vl.viewportf.y);
}

// culling.glsl:94-113 needs last frame's HiZ pyramid; headless builds have none
// and the test passes.
__device__ inline bool intersect_hiz(const Clip&, const Clip&) { return true; }

// ---------------------------------------------------------------------------
// per-frame reset (src/renderer_raytrace_clusters_tess.cpp:412-419)
// ---------------------------------------------------------------------------

__device__ inline void frame_begin_body(const StageCtx& c)
{
  tc_SceneBuilding* b = c.build;
  if(blockIdx.x == 0)
  {
    u32* rb = reinterpret_cast<u32*>(c.readback);
    for(u32 i = threadIdx.x; i < sizeof(tc_Readback) / 4; i += blockDim.x)
      rb[i] = 0;
    if(threadIdx.x == 0)
    {
      const tc_FrameConstants* vp = (c.flags & TC_FLAG_FREEZE_VIEWPOS) ? c.viewLast : c.view;
      b->viewPos                     = {vp->viewPos.x, vp->viewPos.y, vp->viewPos.z};
      b->numRenderInstances          = c.numInstances;
      b->visibleClusterCounter       = 0;
      b->fullClusterCounter          = 0;
      b->partTriangleCounter         = 0;
      b->dualPartTriangleCounter     = 0;
      b->splitTriangleCounter        = 0;
      b->splitReadCounter            = 0;
      b->splitWriteCounter           = 0;
      b->splitPass                   = 0;
      b->splitPassStart              = 0;
      b->splitPassEnd                = 0;
      b->genVertexCounter            = 0;
      b->genClusterCounter           = 0;
      b->genClusterDataCounter       = 0;
      b->dispatchClassify            = {0, 0, 0};
      b->dispatchTriangleSplit       = {0, 0, 0};
      b->drawFullClusters            = {0, 0};
      b->drawPartTriangles           = {0, 0};
      b->dispatchClusterInstantiate  = {0, 0, 0};
      b->dispatchTriangleInstantiate = {0, 0, 0};
      b->dispatchBlasTempInsert      = {0, 0, 0};
      b->dispatchBlasTransInsert     = {0, 0, 0};
      b->blasClusterCounter          = 0;
      b->tempInstantiateCounter      = 0;
      b->transBuildCounter           = 0;
    }
    for(u32 i = threadIdx.x; i < kRunStartsSize; i += blockDim.x)
      c.runStarts[i] = 0;
  }
  // the batched frame's scratch for the stages after this one (their
  // look-back states and counters), in place of a memset before the frame
  for(u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < c.zeroN16; i += (u64)gridDim.x * blockDim.x)
    c.zeroBase[i] = make_uint4(0u, 0u, 0u, 0u);
  // the split queue is filled with ~0 every frame
  u32* split = reinterpret_cast<u32*>(b->splitTriangles);
  if(split)
  {
    const u64 n = (u64)c.caps.maxSplitTriangles * (sizeof(tc_TessTriangleInfo) / 4);
    for(u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
      split[i] = 0xFFFFFFFFu;
  }
}

__global__ void k_frame_begin(StageCtx c)
{
  stage_prologue();
  frame_begin_body(c);
}

// ---------------------------------------------------------------------------
// instances_classify.comp.glsl:102-128, plus the exclusive prefix of
// numClusters over instances that the batched cull uses to flatten
// (instance, cluster) pairs.
// ---------------------------------------------------------------------------

__device__ inline void instances_classify_body(const StageCtx& c)
{
  __shared__ u32 s_tile, s_flag, s_warp[33];
  __shared__ u64 s_excl;
  const u32      n        = c.numInstances;
  u32      numTiles = (n + blockDim.x - 1) / blockDim.x;
  numTiles = clamp_tiles(c, numTiles);
  tc_SceneBuilding* b     = c.build;
  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;
    const u32 i     = tile * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    u32        nc    = 0;
    if(valid)
    {
      const tc_RenderInstance& in = c.instances[i];
      nc                          = in.numClusters;
      Clip cmin, cmax;
      bool cvalid;
      bool inFrustum = intersect_frustum({in.geoLo.x, in.geoLo.y, in.geoLo.z}, {in.geoHi.x, in.geoHi.y, in.geoHi.z},
                                         in.worldMatrix.m, *c.viewLast, cmin, cmax, cvalid);
      bool visible = inFrustum && (!cvalid || (intersect_size(cmin, cmax, *c.viewLast) && intersect_hiz(cmin, cmax)));
      reinterpret_cast<u32*>(b->instanceStates)[i] =
          (inFrustum ? TC_INSTANCE_FRUSTUM_BIT : 0u) | (visible ? TC_INSTANCE_VISIBLE_BIT : 0u);
      reinterpret_cast<tc_BlasBuildInfo*>(b->blasBuildInfos)[i].clusterReferencesCount = 0;
    }
    u32 total;
    u32 excl = block_exclusive_scan(nc, s_warp, &total);
    if(threadIdx.x < 32)
    {
      const u64 ex = warp_lookback_exclusive(c.scratch.lbState, tile, total, 0, c.errorWord,
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
      c.instClusterStart[i] = (u32)s_excl + excl;
    __syncthreads();
  }
  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0)
      c.instClusterStart[n] = numTiles ? (u32)c.scratch.totals[0] : 0u;
    scratch_release(c, numTiles, 1);
  }
}

__global__ void k_instances_classify(StageCtx c)
{
  stage_prologue();
  instances_classify_body(c);
}

// Both in one launch (the batched frame): instances_classify reads nothing the
// per-frame reset writes, so every block does its share of the reset and then
// takes instance tiles.
__global__ void k_frame_begin_instances(StageCtx c)
{
  stage_prologue();
  frame_begin_body(c);
  instances_classify_body(c);
}

// ---------------------------------------------------------------------------
// clusters_cull.comp.glsl:112-161 over the clusters of instances
// [instBegin, instEnd): one tile = blockDim consecutive (instance, cluster)
// pairs, compaction by block scan + look-back (instance, then cluster order).
// RT semantics: nothing is culled; TC_FLAG_RASTER_CULL enables the raster
// path's cluster tests (clusters_cull.comp.glsl:136-143).
// ---------------------------------------------------------------------------

__global__ void k_clusters_cull(StageCtx c)
{
  stage_prologue();
  __shared__ u32 s_tile, s_flag, s_warp[33];
  __shared__ u64 s_excl;
  tc_SceneBuilding* b          = c.build;
  const u32         flatBegin  = c.instClusterStart[c.instBegin];
  const u32         flatEnd    = c.instClusterStart[c.instEnd];
  const u32         n          = flatEnd - flatBegin;
  u32         numTiles   = (n + blockDim.x - 1) / blockDim.x;
  numTiles = clamp_tiles(c, numTiles);
  const bool        rasterCull = (c.flags & TC_FLAG_RASTER_CULL) && (c.flags & TC_FLAG_CULLING);
  tc_ClusterInfo*   vis        = reinterpret_cast<tc_ClusterInfo*>(b->visibleClusters);
  const u32*        states     = reinterpret_cast<const u32*>(b->instanceStates);
  for(;;)
  {
    const u32 tile = next_tile(c, &s_tile);
    if(tile >= numTiles)
      break;
    const u32  g     = flatBegin + tile * blockDim.x + threadIdx.x;
    const bool valid = g < flatEnd;
    u32        inst = 0, cluster = 0;
    bool       visible = false;
    if(valid)
    {
      // last instance whose first flat index is <= g
      u32 lo = c.instBegin, hi = c.instEnd;
      while(hi - lo > 1)
      {
        u32 mid = (lo + hi) >> 1;
        if(c.instClusterStart[mid] <= g)
          lo = mid;
        else
          hi = mid;
      }
      inst    = lo;
      cluster = g - c.instClusterStart[inst];
      visible = true;
      if(rasterCull)
      {
        const tc_RenderInstance& in = c.instances[inst];
        const tc_BBox&           bb = reinterpret_cast<const tc_BBox*>(in.clusterBboxes)[cluster];
        Clip                     cmin, cmax;
        bool                     cvalid;
        if((states[inst] & TC_INSTANCE_VISIBLE_BIT) == 0)
          visible = false;
        visible = visible
                  && intersect_frustum({bb.lo.x, bb.lo.y, bb.lo.z}, {bb.hi.x, bb.hi.y, bb.hi.z}, in.worldMatrix.m,
                                       *c.viewLast, cmin, cmax, cvalid);
        visible = visible && (!cvalid || (intersect_size(cmin, cmax, *c.viewLast) && intersect_hiz(cmin, cmax)));
      }
    }
    u32 total;
    u32 rank = block_exclusive_scan(visible ? 1u : 0u, s_warp, &total);
    if(threadIdx.x < 32)
    {
      const u64 ex =
          warp_lookback_exclusive(c.scratch.lbState, tile, total, tile == 0 ? b->visibleClusterCounter : 0, c.errorWord,
                                  c.spinLimit);
      if(threadIdx.x == 0)
      {
        s_excl = ex;
        if(tile == numTiles - 1)
          c.scratch.totals[0] = ex + total;
      }
    }
    __syncthreads();
    const u64 off = s_excl + rank;
    if(visible && off < c.caps.maxVisibleClusters)
      vis[off] = {inst, cluster};
    __syncthreads();
  }
  if(last_block_done(c, &s_flag))
  {
    if(threadIdx.x == 0)
    {
      if(numTiles)
        b->visibleClusterCounter = (u32)c.scratch.totals[0];
      if(c.fuseSetup != kNoSetup)
        build_setup_apply(c, c.fuseSetup);
    }
    scratch_release(c, numTiles, 1);
  }
}

__global__ void k_build_setup(StageCtx c, u32 mode)
{
  stage_prologue();
  if(blockIdx.x == 0 && threadIdx.x == 0)
    build_setup_apply(c, mode);
}

// One warp runs the look-back wait of tile 1 against tile 0's state word,
// which holds an inclusive prefix of 7 when `published`, and otherwise stays
// at zero (pending): nothing ever publishes it, so the wait has to run out,
// set TC_DEVERR_LOOKBACK_TIMEOUT and return. out[0] = the prefix tile 1 got.
__global__ void k_lookback_probe(u64* state, u32 published, u32* errorWord, u32 spinLimit, u64* out)
{
  if(threadIdx.x == 0 && published)
    st_relaxed_u64(state, kLbPrefix | 7ull);
  __syncwarp();
  const u64 ex = warp_lookback_exclusive(state, 1, 5, 0, errorWord, spinLimit);
  if(threadIdx.x == 0)
    out[0] = ex;
}

// ---------------------------------------------------------------------------
// A frame's host traffic inside its graph (tc_frame_build_graph_host): the
// input block (frame constants, instance records) read from mapped pinned host
// memory at the frame's start, the Readback written back to it once the
// frame's counters are final.
// Plain loads and stores through the mapping replace the copy-engine round
// trips of cudaMemcpyAsync (the reference: vkCmdUpdateBuffer of the frame
// constants, src/renderer_raytrace_clusters_tess.cpp:415, and the Readback copy
// to a host-visible buffer, src/resources.cpp:83-90). The kernel boundary
// makes the stores visible to the host once the stream has passed the frame.
// ---------------------------------------------------------------------------

constexpr u32 kUploadPerThread = 4;  // 16-byte loads in flight per thread before its stores

// the grid's share of a host upload (16-byte words, then the tail bytes)
__device__ __forceinline__ void host_upload_body(const HostUpload& u)
{
  const uint4* __restrict__ src = static_cast<const uint4*>(u.src);
  uint4* __restrict__ dst       = static_cast<uint4*>(u.dst);
  const u64 n16    = u.bytes / 16;
  const u64 stride = (u64)gridDim.x * blockDim.x;
  for(u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride * kUploadPerThread)
  {
    uint4 v[kUploadPerThread];
#pragma unroll
    for(u32 k = 0; k < kUploadPerThread; k++)
      if(i + k * stride < n16)
        v[k] = src[i + k * stride];
#pragma unroll
    for(u32 k = 0; k < kUploadPerThread; k++)
      if(i + k * stride < n16)
        dst[i + k * stride] = v[k];
  }
  const u32 tail = (u32)(u.bytes % 16);
  if(blockIdx.x == 0 && threadIdx.x < tail)
    static_cast<unsigned char*>(u.dst)[n16 * 16 + threadIdx.x] = static_cast<const unsigned char*>(u.src)[n16 * 16 + threadIdx.x];
}

__global__ void k_host_upload(HostUpload u)
{
  stage_prologue();
  host_upload_body(u);
}

// The batched frame's first kernel with the upload in it: every block copies
// its share of the input block, and the frame's own reads of the frame
// constants and instance records (c points them into the host block) go to
// the host memory directly. Kernels after it read the device copy.
__global__ void k_frame_begin_instances_upload(StageCtx c, HostUpload u)
{
  stage_prologue();
  host_upload_body(u);
  frame_begin_body(c);
  instances_classify_body(c);
}

__global__ void k_host_readback(const u32* __restrict__ src, u32* __restrict__ dst, u32 words)
{
  stage_prologue();
  for(u32 i = threadIdx.x; i < words; i += blockDim.x)
    dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

cudaError_t launch_host_upload(const HostUpload& u, u32 maxGrid, cudaStream_t s)
{
  const u64 per  = 256ull * kUploadPerThread;
  const u32 grid = (u32)std::max<u64>(1, std::min<u64>((u.bytes / 16 + per - 1) / per, maxGrid));
  return launch_side(k_host_upload, grid, 256, s, u);
}

cudaError_t launch_frame_begin_instances_upload(const StageCtx& c, const HostUpload& u, u32 grid, cudaStream_t s)
{
  return launch_pdl(k_frame_begin_instances_upload, grid, kInstanceTile, s, c, u);
}

cudaError_t launch_host_readback(const tc_Readback* src, void* dst, cudaStream_t s)
{
  static_assert(sizeof(tc_Readback) % 4 == 0, "the Readback is copied in 32-bit words");
  return launch_side(k_host_readback, 1, 256, s, reinterpret_cast<const u32*>(src), static_cast<u32*>(dst),
                     (u32)(sizeof(tc_Readback) / 4));
}

cudaError_t launch_lookback_probe(u64* state, u32 published, u32* errorWord, u32 spinLimit, cudaStream_t s)
{
  // state[0..1]: tile states, state[2]: the result
  const cudaError_t e = cudaMemsetAsync(state, 0, 3 * sizeof(u64), s);
  if(e != cudaSuccess)
    return e;
  k_lookback_probe<<<1, 32, 0, s>>>(state, published, errorWord, spinLimit, state + 2);
  return cudaGetLastError();
}

cudaError_t launch_frame_begin(const StageCtx& c, u32 grid, cudaStream_t s)
{
  return launch_pdl(k_frame_begin, grid, 256, s, c);
}

cudaError_t launch_instances_classify(const StageCtx& c, u32 grid, u32 block, cudaStream_t s)
{
  return launch_pdl(k_instances_classify, grid, block, s, c);
}

cudaError_t launch_frame_begin_instances(const StageCtx& c, u32 grid, cudaStream_t s)
{
  return launch_pdl(k_frame_begin_instances, grid, kInstanceTile, s, c);
}

cudaError_t launch_clusters_cull(const StageCtx& c, u32 grid, u32 block, cudaStream_t s, bool side)
{
  return side ? launch_side(k_clusters_cull, grid, block, s, c) : launch_pdl(k_clusters_cull, grid, block, s, c);
}

cudaError_t launch_build_setup(const StageCtx& c, u32 mode, cudaStream_t s)
{
  return launch_pdl(k_build_setup, 1, 32, s, c, mode);
}

}  // namespace tc
