// tc_backward.cu — adjoint of the vertex generation with the tessellation
// decisions (factors, configs, split tree, allocation) of the forward frame
// held fixed: they are piecewise constant in the inputs.
//
// Forward being differentiated (per generated vertex):
//   part triangle   (triangle_tess_template_instantiate.comp.glsl:343-371)
//     w = interp(bb, tableVertex);  P = sum_k w_k p_k
//     N = sum_k w_k normalize(n_k);  uv = sum_k w_k uv_k
//     h = bilinear(tex, uv) * s + o;  v = P + normalize(N) * h
//   full cluster    (cluster_classify.comp.glsl:457-482)
//     v = p + normalize(n) * (bilinear(tex, uv) * s + o)
// with s = instance.displacementScale * view.displacementScale.
//
// Gradients scattered: dL/dp, dL/dn (per base vertex) and dL/dtexel (the four
// bilinear taps). Full clusters: one warp per instantiation, one lane per
// vertex, direct atomics. Part triangles: one lane per instantiation; it sums
// the per-base-vertex terms of its vertices in registers and adds them with
// one atomic per component; texel taps use global atomics.
#include "tc_kernels.h"
#include "tc_stage.cuh"
#include "tc_vertex.cuh"

namespace tc {

namespace {

__device__ __forceinline__ void scatter_texels(float* grad, const tc_DisplacementTexture& tx, const Taps& t, float dB)
{
  const float gx = 1.0f - t.fx, gy = 1.0f - t.fy;
  atomicAdd(grad + (u64)t.y0 * tx.width + t.x0, (gy * gx) * dB);
  atomicAdd(grad + (u64)t.y0 * tx.width + t.x1, (gy * t.fx) * dB);
  atomicAdd(grad + (u64)t.y1 * tx.width + t.x0, (t.fy * gx) * dB);
  atomicAdd(grad + (u64)t.y1 * tx.width + t.x1, (t.fy * t.fx) * dB);
}

__device__ __forceinline__ void atomic_add3(float* base, u64 index, f3 v)
{
  atomicAdd(base + 3 * index + 0, v.x);
  atomicAdd(base + 3 * index + 1, v.y);
  atomicAdd(base + 3 * index + 2, v.z);
}

constexpr u32 kWarps = 8;

// number of leading full-cluster instantiations (they precede all parts)
__device__ __forceinline__ u32 full_count(const StageCtx& c, u32 temps)
{
  return min(c.runStarts[kMaxRuns + 1], temps);
}

__global__ void __launch_bounds__(kWarps * 32, 2) k_instantiate_backward(StageCtx c, const float* gradVertices,
                                                                      const tc_GradTargets* targets,
                                                                      float* const* gradTexels)
{
  stage_prologue();
  const u32         lane  = threadIdx.x & 31;
  const u32         gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32         nwarp = (gridDim.x * blockDim.x) >> 5;
  tc_SceneBuilding* b     = c.build;
  const u32         temps = min(b->tempInstantiateCounter, c.caps.maxGeneratedClusters);
  const u32         nfull = full_count(c, temps);
  const tc_TemplateInstantiateInfo* ti    = reinterpret_cast<const tc_TemplateInstantiateInfo*>(b->tempInstantiations);
  const tc_ClusterInfo*             fulls = reinterpret_cast<const tc_ClusterInfo*>(b->fullClusters);
  const bool  haveTextures = c.numTextures > 0 && c.textures != nullptr;
  const float viewScale    = c.view->displacementScale, viewOffset = c.view->displacementOffset;

  // full clusters: every generated vertex is one base vertex (cluster_classify.comp.glsl:457-482)
  for(u32 j = gwarp; fulls && j < nfull; j += nwarp)
  {
    const tc_TemplateInstantiateInfo info  = ti[j];
    const u64                        vbase = (info.vertexBufferAddress - b->genVertices) / 12;
    const tc_ClusterInfo             ci    = fulls[j];
    const tc_RenderInstance&         in    = c.instances[ci.instanceID];
    const tc_Cluster                 cl    = reinterpret_cast<const tc_Cluster*>(in.clusters)[ci.clusterID];
    const tc_GradTargets             gt    = targets[ci.instanceID];
    tc_DisplacementTexture           tx    = {};
    if(haveTextures && in.displacementIndex >= 0 && (u32)in.displacementIndex < c.numTextures)
      tx = c.textures[in.displacementIndex];
    float*      gtex = tx.width ? gradTexels[in.displacementIndex] : nullptr;
    const float s    = in.displacementScale * viewScale;
    const u32   nv   = min((u32)cl.numVertices, TC_MAX_CLUSTER_VERTICES);
    for(u32 v = lane; v < nv; v += 32)
    {
      const u32 vi = cl.firstLocalVertex + v;
      const f3  g  = ldg3(gradVertices, vbase + v);
      if(gt.dPositions)
        atomic_add3(reinterpret_cast<float*>(gt.dPositions), vi, g);
      if(!tx.width)
        continue;
      const f3    n    = ldg3(reinterpret_cast<const float*>(in.normals), vi);
      const f2    uv   = ldg2(reinterpret_cast<const float*>(in.texcoords), vi);
      const float nl   = len3(n);
      const f3    nh   = normalize3(n);
      const float hraw = sample_bilinear(tx, uv);
      const float h    = ((hraw * in.displacementScale) * viewScale + in.displacementOffset) + viewOffset;
      const float dh   = dot3(nh, g);
      if(gt.dNormals)
      {
        // d normalize(n) / dn = (I - nh nh^T) / |n|
        const float k  = h / nl;
        const f3    dn = {k * (g.x - nh.x * dh), k * (g.y - nh.y * dh), k * (g.z - nh.z * dh)};
        atomic_add3(reinterpret_cast<float*>(gt.dNormals), vi, dn);
      }
      if(gtex)
        scatter_texels(gtex, tx, bilinear_taps(tx, uv), dh * s);
    }
  }

  // part triangles (triangle_tess_template_instantiate.comp.glsl:343-371): one
  // lane per part instantiation walks its vertices (3-78) and sums the
  // per-base-vertex terms in registers; one atomic per component and base
  // vertex at the end, no shared-memory traffic
  const tc_TessTriangleInfo* parts = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  const u32                  gtid  = blockIdx.x * blockDim.x + threadIdx.x;
  const u32                  nthr  = gridDim.x * blockDim.x;
  for(u32 j = nfull + gtid; j < temps; j += nthr)
  {
    const tc_TemplateInstantiateInfo info = ti[j];
    const u64                 vbase = (info.vertexBufferAddress - b->genVertices) / 12;
    const tc_TessTriangleInfo pi    = parts[info.clusterIdOffset & 0x3FFFFFFFu];
    const u32                 cfg   = pi.subTriangle.triangleID_config >> 16;
    const u32                 tri   = pi.subTriangle.triangleID_config & 0xFFFFu;
    const tc_RenderInstance&  in    = c.instances[pi.cluster.instanceID];
    const tc_Cluster          cl    = reinterpret_cast<const tc_Cluster*>(in.clusters)[pi.cluster.clusterID];
    const uint8_t*            lt    = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
    const tc_TessTableEntry   e     = table_entry(c.table, cfg);
    const tc_GradTargets      gt    = targets[pi.cluster.instanceID];
    tc_DisplacementTexture    tx    = {};
    if(haveTextures && in.displacementIndex >= 0 && (u32)in.displacementIndex < c.numTextures)
      tx = c.textures[in.displacementIndex];
    float* const gtex = tx.width ? gradTexels[in.displacementIndex] : nullptr;
    const float  s    = in.displacementScale * viewScale;
    u32          vi[3];
    f3           bb[3], nh[3];
    f2           uvb[3];
    float        nl[3];
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      vi[k]      = cl.firstLocalVertex + lt[tri * 3 + k];
      bb[k]      = decode_bary(pi.subTriangle.vtxEncoded[k]);
      const f3 n = ldg3(reinterpret_cast<const float*>(in.normals), vi[k]);
      nl[k]      = len3(n);
      nh[k]      = normalize3(n);
      uvb[k]     = ldg2(reinterpret_cast<const float*>(in.texcoords), vi[k]);
    }
    f3 dP[3]  = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    f3 dNh[3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for(u32 v = 0; v < e.numVertices; v++)
    {
      f3 w = decode_bary(__ldg(c.table.vertices + e.firstVertex + v));
      if(cfg_flipped(cfg))
      {
        const float x = w.x;
        w.x           = w.y;
        w.y           = x;
      }
      w                 = interp3(bb[0], bb[1], bb[2], w);
      const f3    g     = ldg3(gradVertices, vbase + v);
      const float wk[3] = {w.x, w.y, w.z};
#pragma unroll
      for(int k = 0; k < 3; k++)
        dP[k] = {dP[k].x + wk[k] * g.x, dP[k].y + wk[k] * g.y, dP[k].z + wk[k] * g.z};
      if(tx.width == 0)
        continue;
      const f3    N    = interp3(nh[0], nh[1], nh[2], w);
      const f2    uv   = interp2(uvb[0], uvb[1], uvb[2], w);
      const float Nl   = len3(N);
      const f3    m    = normalize3(N);
      const float hraw = sample_bilinear(tx, uv);
      const float h    = ((hraw * in.displacementScale) * viewScale + in.displacementOffset) + viewOffset;
      const float dh   = dot3(m, g);
      // d normalize(N) / dN = (I - m m^T) / |N|
      const float kN = h / Nl;
      const f3    gN = {kN * (g.x - m.x * dh), kN * (g.y - m.y * dh), kN * (g.z - m.z * dh)};
#pragma unroll
      for(int k = 0; k < 3; k++)
        dNh[k] = {dNh[k].x + wk[k] * gN.x, dNh[k].y + wk[k] * gN.y, dNh[k].z + wk[k] * gN.z};
      if(gtex)
        scatter_texels(gtex, tx, bilinear_taps(tx, uv), dh * s);
    }
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      if(gt.dPositions)
        atomic_add3(reinterpret_cast<float*>(gt.dPositions), vi[k], dP[k]);
      if(tx.width && gt.dNormals)
      {
        // d normalize(n_k) / dn_k = (I - nh nh^T) / |n_k|
        const float d  = dot3(nh[k], dNh[k]);
        const float rr = 1.0f / nl[k];
        const f3    dn = {rr * (dNh[k].x - nh[k].x * d), rr * (dNh[k].y - nh[k].y * d), rr * (dNh[k].z - nh[k].z * d)};
        atomic_add3(reinterpret_cast<float*>(gt.dNormals), vi[k], dn);
      }
    }
  }
}

// Forward of the same frozen frame: regenerates every accepted instantiation's
// vertices with the arithmetic of the build kernels (bit-identical output).
__global__ void __launch_bounds__(256) k_generate_vertices(StageCtx c)
{
  stage_prologue();
  __shared__ PartAffine s_aff[8];
  const u32         lane  = threadIdx.x & 31;
  const u32         gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32         nwarp = (gridDim.x * blockDim.x) >> 5;
  tc_SceneBuilding* b     = c.build;
  const u32         temps = min(b->tempInstantiateCounter, c.caps.maxGeneratedClusters);
  const tc_TemplateInstantiateInfo* ti    = reinterpret_cast<const tc_TemplateInstantiateInfo*>(b->tempInstantiations);
  const tc_TessTriangleInfo*        parts = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  const tc_ClusterInfo*             fulls = reinterpret_cast<const tc_ClusterInfo*>(b->fullClusters);
  const bool  haveTextures = c.numTextures > 0 && c.textures != nullptr;
  const float vscale       = c.view->displacementScale, voffset = c.view->displacementOffset;
  float*      gv           = reinterpret_cast<float*>(b->genVertices);

  for(u32 j = gwarp; j < temps; j += nwarp)
  {
    const tc_TemplateInstantiateInfo info  = ti[j];
    const u32                        mode  = info.clusterIdOffset >> 30;
    const u64                        vbase = (info.vertexBufferAddress - b->genVertices) / 12;
    if(mode == TC_RT_CLUSTER_MODE_FULL_CLUSTER)
    {
      if(!fulls)
        continue;
      const tc_ClusterInfo     ci = fulls[j];
      const tc_RenderInstance& in = c.instances[ci.instanceID];
      const tc_Cluster         cl = reinterpret_cast<const tc_Cluster*>(in.clusters)[ci.clusterID];
      tc_DisplacementTexture   tx = {};
      if(haveTextures && in.displacementIndex >= 0 && (u32)in.displacementIndex < c.numTextures)
        tx = c.textures[in.displacementIndex];
      // the build's full-cluster vertex function (tc_vertex.cuh): identical bits
      const MapDesc map    = make_map_desc(tx);
      const float   scale  = in.displacementScale * vscale;
      const float   offset = in.displacementOffset + voffset;
      const u32     nv     = min((u32)cl.numVertices, TC_MAX_CLUSTER_VERTICES);
      for(u32 v = lane; v < nv; v += 32)
      {
        const u32 vi = cl.firstLocalVertex + v;
        f3        p  = ldg3(reinterpret_cast<const float*>(in.positions), vi);
        if(map.kind != kAffineFlat)
          p = full_vertex_k<~0u>(p, ldg3(reinterpret_cast<const float*>(in.normals), vi),
                                 ldg2(reinterpret_cast<const float*>(in.texcoords), vi), map, scale, offset);
        float* d = gv + (vbase + v) * 3;
        d[0] = p.x, d[1] = p.y, d[2] = p.z;
      }
    }
    else
    {
      // the affine vertex form of the build kernel (tc_vertex.cuh): identical bits
      const tc_TessTriangleInfo pi  = parts[info.clusterIdOffset & 0x3FFFFFFFu];
      const u32                 cfg = pi.subTriangle.triangleID_config >> 16;
      const tc_TessTableEntry   e   = table_entry(c.table, cfg);
      PartAffine&               r   = s_aff[threadIdx.x >> 5];
      if(lane == 0)
      {
        const u32                tri = pi.subTriangle.triangleID_config & 0xFFFFu;
        const tc_RenderInstance& in  = c.instances[pi.cluster.instanceID];
        const tc_Cluster         cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[pi.cluster.clusterID];
        const uint8_t* lt = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
        tc_DisplacementTexture tx = {};
        if(haveTextures && in.displacementIndex >= 0 && (u32)in.displacementIndex < c.numTextures)
          tx = c.textures[in.displacementIndex];
        part_affine(r, pi.subTriangle.vtxEncoded, cfg_flipped(cfg), reinterpret_cast<const float*>(in.positions),
                    reinterpret_cast<const float*>(in.normals), reinterpret_cast<const float*>(in.texcoords),
                    cl.firstLocalVertex, lt + tri * 3, e.firstVertex, tx, in.displacementScale * vscale,
                    in.displacementOffset + voffset);
      }
      __syncwarp();
      for(u32 v = lane; v < e.numVertices; v += 32)
      {
        const f3 q = affine_vertex(r, __ldg(c.table.vertices + e.firstVertex + v));
        float*   d = gv + (vbase + v) * 3;
        d[0] = q.x, d[1] = q.y, d[2] = q.z;
      }
      __syncwarp();  // the record is rewritten by the warp's next part
    }
  }
}

}  // namespace

cudaError_t launch_generate_vertices(const StageCtx& c, u32 grid, cudaStream_t s)
{
  return launch_pdl(k_generate_vertices, grid, 256, s, c);
}

cudaError_t launch_instantiate_backward(const StageCtx& c, const float* gradVertices, const tc_GradTargets* targets,
                                        float* const* gradTexels, u32 grid, cudaStream_t s)
{
  return launch_pdl(k_instantiate_backward, grid, 256, s, c, gradVertices, targets, gradTexels);
}

}  // namespace tc
