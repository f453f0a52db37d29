// tc_decode.cu — hit-time decode of cluster ray-tracing hits into base-mesh
// hits: render_raytrace_clusters.rchit.glsl:131-214 (RT target; 1X subset and
// 2X batch hits when the frame was built with those transient builds), as a
// kernel any CUDA ray tracer can run over its hit records.
//
// One thread per hit; every index is checked against the frame's data (a hit
// from another frame reports TC_HIT_OUT_OF_RANGE instead of reading past a
// buffer). Barycentric compositions are separate multiplies and adds in the
// shader's order, so the results equal the CPU restatement's bit for bit.
#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

namespace {

__device__ __forceinline__ f3 scale_add(f3 acc, f3 v, float w)
{
  return {__fadd_rn(acc.x, __fmul_rn(v.x, w)), __fadd_rn(acc.y, __fmul_rn(v.y, w)), __fadd_rn(acc.z, __fmul_rn(v.z, w))};
}

// a * w.x + b * w.y + c * w.z, left to right
__device__ __forceinline__ f3 compose(f3 a, f3 b, f3 c, f3 w)
{
  f3 r = {__fmul_rn(a.x, w.x), __fmul_rn(a.y, w.x), __fmul_rn(a.z, w.x)};
  r    = scale_add(r, b, w.y);
  return scale_add(r, c, w.z);
}

__global__ void k_decode_hits(StageCtx c, const tc_hit* hits, u32 count, tc_base_hit* out)
{
  stage_prologue();
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= count)
    return;
  const tc_hit h = hits[i];
  tc_base_hit  r = {};
  u32          mode = h.clusterID >> 30, clusterID = h.clusterID & 0x3FFFFFFFu;
  u32          triangleID = h.triangleID, subTriangleID = h.triangleID, cfg = 0;
  const bool   visTriangles = c.view->visualize == TC_VISUALIZE_TRIANGLES;
  u32          partID       = visTriangles ? triangleID + 1 : 0u;
  uint4        enc          = {0, 0, 0, 0};
  bool         tess         = mode == TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED;
  r.status                  = TC_HIT_OK;
  if((mode == TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER && !(c.flags & TC_FLAG_TRANSIENT_1X))
     || (mode == TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED && !(c.flags & TC_FLAG_TRANSIENT_2X)))
    r.status = TC_HIT_UNSUPPORTED_MODE;
  else if(h.instanceID >= c.numInstances)
    r.status = TC_HIT_OUT_OF_RANGE;
  else if(mode == TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER || mode == TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED)
  {
    // rchit.glsl:150-180: a transient build's ClusterInfo header and triangle
    // map at the back of partTriangles
    const bool mini = mode == TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED;
    const u64  need = mini ? 10ull + 2ull * triangleID : 9ull + triangleID;  // header + map entry, in bytes
    if(clusterID >= c.caps.maxPartTriangles || need > (u64)(c.caps.maxPartTriangles - clusterID) * 24
       || triangleID >= (mini ? 32u : 64u))
      r.status = TC_HIT_OUT_OF_RANGE;
    else
    {
      const uint8_t* rec = reinterpret_cast<const uint8_t*>(c.build->partTriangles) + (u64)clusterID * 24;
      const uint2    hdr = *reinterpret_cast<const uint2*>(rec);
      if(mini)
      {
        const u32 packed = reinterpret_cast<const uint16_t*>(rec + 8)[triangleID];
        triangleID       = packed & 0xFFu;
        subTriangleID    = (packed >> 8) & 4u;  // the shader's mask (rchit.glsl:161), kept as written
        u32 e3[3]        = {0u, TC_TESSTABLE_COORD_MAX, TC_TESSTABLE_COORD_MAX << 16};
        const uint3 f    = make_uint3(1u + ((packed >> 12) & 1u), 1u + ((packed >> 13) & 1u), 1u + (packed >> 14));
        cfg              = get_config(f, e3[0], e3[1], e3[2]);
        enc              = {e3[0], e3[1], e3[2], 0};
        tess             = true;
      }
      else
        triangleID = rec[8 + triangleID];
      clusterID = hdr.y;
      if(hdr.x != h.instanceID || (tess && subTriangleID >= table_entry(c.table, cfg).numTriangles))
        r.status = TC_HIT_OUT_OF_RANGE;
    }
  }
  else if(mode == TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED)
  {
    // rchit.glsl:146, 183-186: the part triangle names its base cluster and triangle
    if(clusterID >= min(c.build->partTriangleCounter, c.caps.maxPartTriangles))
      r.status = TC_HIT_OUT_OF_RANGE;
    else
    {
      const tc_TessTriangleInfo pt = reinterpret_cast<const tc_TessTriangleInfo*>(c.build->partTriangles)[clusterID];
      triangleID                   = pt.subTriangle.triangleID_config & 0xFFFFu;
      cfg                          = pt.subTriangle.triangleID_config >> 16;
      clusterID                    = pt.cluster.clusterID;
      enc = {pt.subTriangle.vtxEncoded[0], pt.subTriangle.vtxEncoded[1], pt.subTriangle.vtxEncoded[2], 0};
      if(pt.cluster.instanceID != h.instanceID || subTriangleID >= table_entry(c.table, cfg).numTriangles)
        r.status = TC_HIT_OUT_OF_RANGE;
    }
  }
  const tc_RenderInstance* in = c.instances + min(h.instanceID, c.numInstances - 1);
  if(r.status == TC_HIT_OK && clusterID >= in->numClusters)
    r.status = TC_HIT_OUT_OF_RANGE;
  tc_Cluster cl = {};
  if(r.status == TC_HIT_OK)
  {
    cl = reinterpret_cast<const tc_Cluster*>(in->clusters)[clusterID];
    if(triangleID >= cl.numTriangles)
      r.status = TC_HIT_OUT_OF_RANGE;
  }
  if(r.status != TC_HIT_OK)
  {
    out[i] = r;
    return;
  }
  // rchit.glsl:191-200: the base triangle's vertices
  const uint8_t* lt = reinterpret_cast<const uint8_t*>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
  for(int v = 0; v < 3; v++)
    r.vertexIndices[v] = lt[triangleID * 3 + v] + cl.firstLocalVertex;
  // rchit.glsl:202-203: (1 - u - v, u, v)
  const f3 w = {__fsub_rn(__fsub_rn(1.0f, h.barycentrics[0]), h.barycentrics[1]), h.barycentrics[0],
                h.barycentrics[1]};
  f3       base = w;
  if(tess)
  {
    // rchit.glsl:207-235: micro-triangle -> sub-triangle -> base triangle
    const u32 e[3] = {enc.x, enc.y, enc.z};
    partID         = 0;
    for(int v = 0; v < 3; v++)
      partID ^= (e[v] >> 20) | ((e[v] >> 4) & 0xFFFu);
    const tc_TessTableEntry te = table_entry(c.table, cfg);
    const uint3             t  = cfg_triangle(c.table, te, cfg, subTriangleID);
    const f3                sub =
        compose(cfg_vertex(c.table, te, cfg, t.x), cfg_vertex(c.table, te, cfg, t.y), cfg_vertex(c.table, te, cfg, t.z), w);
    base   = compose(decode_bary(e[0]), decode_bary(e[1]), decode_bary(e[2]), sub);
    partID = visTriangles ? subTriangleID * 3 : partID;
    partID = triangleID | ((partID | 1u) << 8);
  }
  r.clusterID       = clusterID;
  r.triangleID      = triangleID;
  r.barycentrics[0] = base.x;
  r.barycentrics[1] = base.y;
  r.barycentrics[2] = base.z;
  r.partID          = partID;
  out[i]            = r;
}

}  // namespace

cudaError_t launch_decode_hits(const StageCtx& c, const tc_hit* hits, u32 count, tc_base_hit* out, cudaStream_t s)
{
  if(count == 0)
    return cudaSuccess;
  return launch_pdl(k_decode_hits, (count + 255) / 256, 256u, s, c, hits, count, out);
}

}  // namespace tc
