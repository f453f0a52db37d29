// tc_raster.cu — raster-style batching of the frame's part triangles:
// render_raster_clusters_batched.task.glsl:115-215 (the linear fill of 32
// parts into batches of <= 96 vertices and <= 121 triangles) and
// render_raster_clusters_batched.mesh.glsl:141-435 (the batch's displaced
// vertices in world and clip space, its triangles' local indices and
// primitive IDs) as compute kernels writing plain vertex and index arrays.
//
// Three launches: per group of 32 parts (one warp) its batch, vertex and
// triangle counts; one block scans the groups' counts into offsets; per group
// again (four warps, a quarter of the parts each) the batch records, then part
// by part the vertices (lanes over the part's vertices) and triangles.
#include "tc_kernels.h"
#include "tc_stage.cuh"
#include "tc_vertex.cuh"

namespace tc {

namespace {

constexpr u32 kRasterBlock   = 256;
constexpr u32 kWarpsPerGroup = 4;  // k_raster_write: warps per group of 32 parts
constexpr u32 kPartsPerWarp  = 32 / kWarpsPerGroup;

// what the vertex and triangle loops of one part need
struct RasterPart
{
  f3                     bp[3], bn[3], bb[3];
  f2                     bt[3];
  tc_DisplacementTexture tx;
  const float*           world;
  float                  scale, offset, size;
  u32                    cfg, triID, inst, partID, v0, t0, vs;
  bool                   hasTx;
};

// the group's parts: per lane (part g0 + lane) its inclusive vertex and
// triangle sums; lanes past the parts count as a full batch (they never fit)
struct GroupSums
{
  u32 v, t;        // this lane's part
  u32 sumV, sumT;  // inclusive
};

__device__ __forceinline__ GroupSums group_sums(const StageCtx& c, u32 g0, u32 local)
{
  const u32                  lane  = threadIdx.x & 31;
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(c.build->partTriangles);
  GroupSums                  s;
  s.v = TC_RASTER_BATCH_VERTICES, s.t = TC_RASTER_BATCH_TRIANGLES;
  if(lane < local)
  {
    const tc_TessTableEntry e = table_entry(c.table, parts[g0 + lane].subTriangle.triangleID_config >> 16);
    s.v = e.numVertices, s.t = e.numTriangles;
  }
  s.sumV = s.v, s.sumT = s.t;
#pragma unroll
  for(int d = 1; d < 32; d <<= 1)
  {
    const u32 a = __shfl_up_sync(0xFFFFFFFFu, s.sumV, d), b = __shfl_up_sync(0xFFFFFFFFu, s.sumT, d);
    if(lane >= (u32)d)
      s.sumV += a, s.sumT += b;
  }
  return s;
}

// task.glsl:150-205: batch q's last part (its end) for every batch, calling
// fn(q, start, end, vertices before start, triangles before start)
template <class F>
__device__ __forceinline__ u32 group_batches(const GroupSums& s, u32 local, F&& fn)
{
  u32 start = 0, lastV = 0, lastT = 0, left = local, q = 0;
  while(left != 0 && q < 32)
  {
    // unsigned differences: parts before the batch do not fit
    const u32 fit = __ballot_sync(0xFFFFFFFFu, s.sumV - lastV <= TC_RASTER_BATCH_VERTICES
                                                   && s.sumT - lastT <= TC_RASTER_BATCH_TRIANGLES);
    const u32 end = 31 - __clz(fit);
    fn(q, start, end, lastV, lastT);
    const u32 count = 1 + end - start;
    lastV           = __shfl_sync(0xFFFFFFFFu, s.sumV, end);
    lastT           = __shfl_sync(0xFFFFFFFFu, s.sumT, end);
    start           = end + 1;
    left -= min(count, left);
    q++;
  }
  return q;
}

__device__ __forceinline__ u32 num_parts(const StageCtx& c)
{
  return min(c.build->partTriangleCounter, c.caps.maxPartTriangles);
}

__global__ void __launch_bounds__(kRasterBlock) k_raster_counts(StageCtx c, uint4* groups)
{
  stage_prologue();
  const u32 lane = threadIdx.x & 31, n = num_parts(c), ngroups = (n + 31) / 32;
  for(u32 g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += (gridDim.x * blockDim.x) >> 5)
  {
    const u32       g0 = g * 32, local = min(32u, n - g0);
    const GroupSums s  = group_sums(c, g0, local);
    const u32       nb = group_batches(s, local, [](u32, u32, u32, u32, u32) {});
    const u32       vTot = __shfl_sync(0xFFFFFFFFu, s.sumV, local - 1), tTot = __shfl_sync(0xFFFFFFFFu, s.sumT, local - 1);
    if(lane == 0)
      groups[g] = make_uint4(nb, vTot, tTot, 0u);
  }
}

// one block: exclusive scan of the groups' counts, in place; totals to counts[3]
__global__ void __launch_bounds__(1024) k_raster_scan(StageCtx c, uint4* groups, u32* counts)
{
  stage_prologue();
  __shared__ uint4 s_warp[32];
  __shared__ uint4 s_carry;
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32 ngroups = (num_parts(c) + 31) / 32;
  if(threadIdx.x == 0)
    s_carry = make_uint4(0, 0, 0, 0);
  __syncthreads();
  for(u32 base = 0; base < ngroups; base += blockDim.x)
  {
    const u32 i = base + threadIdx.x;
    uint4     v = i < ngroups ? groups[i] : make_uint4(0, 0, 0, 0);
    uint4     inc = v;
#pragma unroll
    for(int d = 1; d < 32; d <<= 1)
    {
      const u32 a = __shfl_up_sync(0xFFFFFFFFu, inc.x, d), b = __shfl_up_sync(0xFFFFFFFFu, inc.y, d),
                e = __shfl_up_sync(0xFFFFFFFFu, inc.z, d);
      if(lane >= (u32)d)
        inc.x += a, inc.y += b, inc.z += e;
    }
    if(lane == 31)
      s_warp[warp] = inc;
    __syncthreads();
    if(warp == 0)
    {
      uint4 w = s_warp[lane], wi = w;
#pragma unroll
      for(int d = 1; d < 32; d <<= 1)
      {
        const u32 a = __shfl_up_sync(0xFFFFFFFFu, wi.x, d), b = __shfl_up_sync(0xFFFFFFFFu, wi.y, d),
                  e = __shfl_up_sync(0xFFFFFFFFu, wi.z, d);
        if(lane >= (u32)d)
          wi.x += a, wi.y += b, wi.z += e;
      }
      s_warp[lane] = make_uint4(wi.x - w.x, wi.y - w.y, wi.z - w.z, 0u);
    }
    __syncthreads();
    const uint4 cw = s_carry, ww = s_warp[warp];
    if(i < ngroups)
      groups[i] = make_uint4(cw.x + ww.x + inc.x - v.x, cw.y + ww.y + inc.y - v.y, cw.z + ww.z + inc.z - v.z, 0u);
    __syncthreads();
    if(threadIdx.x == blockDim.x - 1)
      s_carry = make_uint4(cw.x + ww.x + inc.x, cw.y + ww.y + inc.y, cw.z + ww.z + inc.z, 0u);
    __syncthreads();
  }
  if(threadIdx.x == 0)
  {
    counts[0] = s_carry.x, counts[1] = s_carry.y, counts[2] = s_carry.z;
  }
}

__global__ void __launch_bounds__(kRasterBlock) k_raster_write(StageCtx c, const uint4* groups, tc_raster_outputs o)
{
  stage_prologue();
  __shared__ RasterPart      s_parts[kRasterBlock / 32][kPartsPerWarp];
  const u32                  lane = threadIdx.x & 31, n = num_parts(c), ngroups = (n + 31) / 32;
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(c.build->partTriangles);
  tc_raster_batch*           batches = reinterpret_cast<tc_raster_batch*>(o.batches);
  float*                     clip    = reinterpret_cast<float*>(o.clipPositions);
  float*                     world   = reinterpret_cast<float*>(o.worldPositions);
  uint8_t*                   idx     = reinterpret_cast<uint8_t*>(o.indices);
  u32*                       prim    = reinterpret_cast<u32*>(o.primitiveIDs);
  const bool                 visTriangles = c.view->visualize == TC_VISUALIZE_TRIANGLES;
  const bool                 pn = (c.flags & TC_FLAG_PN) != 0;
  const RippleParams         rp = ripple_params(*c.view, (c.flags & TC_FLAG_RIPPLE) != 0);
  float                      vp[16];
#pragma unroll
  for(int q = 0; q < 16; q++)
    vp[q] = c.view->viewProjMatrix.m[q];
  bool overflow = false;
  // kWarpsPerGroup warps share a group, each taking a quarter of its parts
  // (the batch layout is recomputed by each, the first writes the records)
  for(u32 gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; gw < ngroups * kWarpsPerGroup;
      gw += (gridDim.x * blockDim.x) >> 5)
  {
    const u32       g = gw / kWarpsPerGroup, sub = gw % kWarpsPerGroup;
    const u32       g0 = g * 32, local = min(32u, n - g0);
    const uint4     off = groups[g];  // batches, vertices, triangles before this group
    const GroupSums s   = group_sums(c, g0, local);
    // per part: the vertex count before its batch (its batch-local vertex start)
    u32 batchStartV = 0;
    group_batches(s, local, [&](u32 q, u32 start, u32 end, u32 lastV, u32 lastT) {
      const u32 ev = __shfl_sync(0xFFFFFFFFu, s.sumV, end), et = __shfl_sync(0xFFFFFFFFu, s.sumT, end);
      if(lane >= start && lane <= end)
        batchStartV = lastV;
      if(lane == 0 && sub == 0)
      {
        const u32 slot = off.x + q;
        if(slot < o.maxBatches)
        {
          tc_raster_batch r;
          r.firstPart     = g0 + start;
          r.partCount     = 1 + end - start;
          r.firstVertex   = off.y + lastV;
          r.numVertices   = ev - lastV;
          r.firstTriangle = off.z + lastT;
          r.numTriangles  = et - lastT;
          batches[slot]   = r;
        }
        else
          overflow = true;
      }
    });
    // mesh.glsl:190-435: lanes 0..7 set up the warp's parts at once (their
    // dependent loads overlap), then part by part lanes take its vertices
    // and triangles
    const u32 pBegin = sub * kPartsPerWarp, pEnd = min(local, pBegin + kPartsPerWarp);
    RasterPart* rec = s_parts[threadIdx.x >> 5];
    // lane l < kPartsPerWarp sets up part pBegin + l: its exclusive sums and
    // its first vertex within its batch, from that part's lane
    const u32 src = pBegin + (lane & (kPartsPerWarp - 1));
    const u32 exV = __shfl_sync(0xFFFFFFFFu, s.sumV - s.v, src), exT = __shfl_sync(0xFFFFFFFFu, s.sumT - s.t, src);
    const u32 vsP = __shfl_sync(0xFFFFFFFFu, s.sumV - s.v - batchStartV, src);
    if(pBegin + lane < pEnd && lane < kPartsPerWarp)
    {
      const u32                 i   = pBegin + lane;
      const tc_TessTriangleInfo pt  = parts[g0 + i];
      RasterPart&               r   = rec[lane];
      r.cfg                         = pt.subTriangle.triangleID_config >> 16;
      r.triID                       = pt.subTriangle.triangleID_config & 0xFFFFu;
      r.inst                        = pt.cluster.instanceID;
      r.v0                          = off.y + exV;
      r.t0                          = off.z + exT;
      r.vs                          = vsP;
      const tc_RenderInstance& in   = c.instances[pt.cluster.instanceID];
      const tc_Cluster         cl   = reinterpret_cast<const tc_Cluster*>(in.clusters)[pt.cluster.clusterID];
      const uint8_t* lt = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      u32            partID = 0;
      for(int v = 0; v < 3; v++)
      {
        const u32 vi = cl.firstLocalVertex + lt[r.triID * 3 + v];
        r.bp[v]      = ldg3(reinterpret_cast<const float*>(in.positions), vi);
        r.bn[v]      = normalize3(ldg3(reinterpret_cast<const float*>(in.normals), vi));
        r.bt[v]      = ldg2(reinterpret_cast<const float*>(in.texcoords), vi);
        r.bb[v]      = decode_bary(pt.subTriangle.vtxEncoded[v]);
        partID ^= (pt.subTriangle.vtxEncoded[v] >> 20) | ((pt.subTriangle.vtxEncoded[v] >> 4) & 0xFFFu);
      }
      r.partID = partID;
      r.hasTx  = false;
      if(c.numTextures > 0 && c.textures != nullptr && in.displacementIndex >= 0)
      {
        if((u32)in.displacementIndex < c.numTextures)
        {
          r.tx    = c.textures[in.displacementIndex];
          r.hasTx = true;
        }
        else
          atomicOr(c.errorWord, TC_DEVERR_BAD_CLUSTER);
      }
      r.scale  = in.displacementScale;
      r.offset = in.displacementOffset;
      r.size   = in.geoHi.w;
      r.world  = in.worldMatrix.m;
    }
    __syncwarp();
    for(u32 i = pBegin; i < pEnd; i++)
    {
      const RasterPart&       r = rec[i - pBegin];
      const tc_TessTableEntry e = table_entry(c.table, r.cfg);
      BasePN                  basis = {};
      if(pn)
        basis = setup_pn(r.bp[0], r.bp[1], r.bp[2], r.bn[0], r.bn[1], r.bn[2]);
      for(u32 vert = lane; vert < e.numVertices; vert += 32)
      {
        if(r.v0 + vert >= o.maxVertices)
        {
          overflow = true;
          break;
        }
        const f3 w   = interp3(r.bb[0], r.bb[1], r.bb[2], cfg_vertex(c.table, e, r.cfg, vert));
        f3       pos = pn ? get_pn(basis, w) : interp3(r.bp[0], r.bp[1], r.bp[2], w);
        if(r.hasTx)
          pos = displace(pos, interp3(r.bn[0], r.bn[1], r.bn[2], w),
                         sample_bilinear(r.tx, interp2(r.bt[0], r.bt[1], r.bt[2], w)), r.scale,
                         c.view->displacementScale, r.offset, c.view->displacementOffset);
        if(rp.enabled)
          pos = ripple(pos, r.inst, r.size, rp);
        float m[16];
#pragma unroll
        for(int q = 0; q < 16; q++)
          m[q] = __ldg(r.world + q);
        const f3 wp = xform_point(m, pos);
        const f3 cp = xform_point(vp, wp);
        float*   wo = world + 3 * (u64)(r.v0 + vert);
        float*   co = clip + 4 * (u64)(r.v0 + vert);
        wo[0] = wp.x, wo[1] = wp.y, wo[2] = wp.z;
        co[0] = cp.x, co[1] = cp.y, co[2] = cp.z;
        co[3] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(vp[3], wp.x), __fmul_rn(vp[7], wp.y)), __fmul_rn(vp[11], wp.z)), vp[15]);
      }
      for(u32 tri = lane; tri < e.numTriangles; tri += 32)
      {
        if(r.t0 + tri >= o.maxTriangles)
        {
          overflow = true;
          break;
        }
        const uint3 ct = cfg_triangle(c.table, e, r.cfg, tri);
        uint8_t*    d  = idx + 3 * (u64)(r.t0 + tri);
        d[0] = (uint8_t)(ct.x + r.vs), d[1] = (uint8_t)(ct.y + r.vs), d[2] = (uint8_t)(ct.z + r.vs);
        prim[r.t0 + tri] = (r.triID & 0xFFu) | (((visTriangles ? tri * 3 : r.partID) | 1u) << 8);
      }
    }
    __syncwarp();  // the records are rewritten by the warp's next group
  }
  if(overflow)
    atomicOr(c.errorWord, TC_DEVERR_CAPACITY);
}

}  // namespace

cudaError_t launch_raster_batches(const StageCtx& c, uint4* groups, const tc_raster_outputs& o, u32 maxParts,
                                  u32 numSMs, cudaStream_t s)
{
  const u32   ngroups = std::max(1u, (maxParts + 31) / 32);
  const u32   grid    = std::max(1u, std::min((ngroups + 7) / 8, numSMs * 8));
  const u32   wgrid   = std::max(1u, std::min((ngroups * kWarpsPerGroup + 7) / 8, numSMs * 8));
  cudaError_t e       = launch_pdl(k_raster_counts, grid, kRasterBlock, s, c, groups);
  if(e != cudaSuccess)
    return e;
  e = launch_pdl(k_raster_scan, 1u, 1024u, s, c, groups, reinterpret_cast<u32*>(o.counts));
  if(e != cudaSuccess)
    return e;
  return launch_pdl(k_raster_write, wgrid, kRasterBlock, s, c, const_cast<const uint4*>(groups), o);
}

}  // namespace tc
